"""The C-ABI is usable from plain C: the host program in tests/c compiles
against include/droplet_gb300.h alone and links to the in-tree library (no
GPU needed to build it)."""
import os

import pytest

from droplet_gb300 import build as libbuild

from c_host import build


def test_c_host_compiles_and_links(tmp_path):
    if not os.path.exists(libbuild.LIB):
        pytest.skip("library not built")
    exe = build(tmp_path)
    assert os.path.exists(exe)
