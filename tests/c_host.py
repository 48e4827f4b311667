"""Build helper of the plain C host in tests/c (gcc against include/ and the
in-tree library)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "abi_host.c")
LIBDIR = os.path.join(ROOT, "droplet_gb300")


def build(out_dir):
    exe = os.path.join(str(out_dir), "abi_host")
    cmd = ["gcc", "-O2", "-std=c99", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-ldroplet_gb300", "-Wl,-rpath," + LIBDIR, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return exe
