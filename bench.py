#!/usr/bin/env python
"""Benchmark of the GB300 droplet step: prints ONE JSON line.

A "step" is one time step of the D3Q15 two-phase droplet update over the
whole resident domain. The default workload is the forced-turbulence case
(128^3, LES, constant-injection band forcing, one droplet R = 16), run in the
FP32 form; --form and --workload select others.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU implementation of the same step on the host
cores (the oracle's OpenMP restatement of the reference, which cannot itself
be built here: it is Fortran + MPI + 2decomp_fft). Under torchrun only rank 0
runs it. The path has no exchange step between independent droplet domains,
so N > 1 runs N independent replicas ("replicas only"), weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MLUPS and % HBM roofline, chosen vs plain FP64 form at stated φ error; adjoint/fwd"
UNIT = "MLUPS"
# algorithmic bytes per lattice update: 2 distributions x 15 x (read + write) x bytes per population
BYTES_PER_SITE = {64: 480, 32: 240, 16: 120}  # two distributions; the single-phase step moves half


def bytes_per_site(form: int, single: bool) -> int:
    return BYTES_PER_SITE[form] // (2 if single else 1)
EVENT_STRIDE = 10  # timed region: CUDA events around every 10th launch ...


def event_stride(steps: int) -> int:
    """... or more often, so that at least 10 launches of the timed region are sampled."""
    return max(1, min(EVENT_STRIDE, steps // 10))
FORMS = {"fp64": 64, "fp32": 32, "fp16": 16}
DTYPE = {64: "f64", 32: "f32", 16: "f32 (f16 storage)"}
MAIN_KERNEL = {64: "collide_fp64", 32: "step_fused", 16: "step_fused"}


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(p) as fh:
            for line in fh:
                line = line.split("#", 1)[0].strip()
                if "=" not in line:
                    continue
                key, val = (t.strip() for t in line.split("=", 1))
                if key == f"{kernel}:{workload}":
                    return int(val)
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = os.path.join("/tmp", f"dl_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value: float, dist=None, device: str = "cuda") -> float:
    """The slowest rank's time: every rank of a replicas run processes its
    own domain, so the whole job takes as long as its slowest member."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(sites_per_rank: int, steps: int, world: int, seconds: float) -> float:
    """Whole-job MLUPS of N independent replicas (weak scaling)."""
    return sites_per_rank * steps * world / seconds / 1e6


def make_workload(name: str, form: int):
    from droplet_gb300 import configs

    if name == "config1":
        w = configs.config1()
        w.form = form
    elif name == "config2":
        w = configs.config2(form=form)
    elif name == "config3":
        w = configs.config3()
        w.form = form
    elif name == "precursor":
        w = configs.precursor(form=form)
    else:
        raise SystemExit(f"unknown workload {name}")
    return w


def new_sim(w, rank: int = 0):
    from droplet_gb300.solver import Droplet

    sim = Droplet(w.params, w.shape, w.form, single_phase=w.single_phase)
    sim.set_fields(**w.fields)
    sim.init_equilibrium()
    sim.set_force(w.force_mode)
    return sim


def checkpoints_for(steps: int):
    """Steps at which the accuracy leg compares the forms: 500, 1000, 2000,
    5000, ... up to and including ``steps``."""
    out = [c for c in (100, 250, 500, 1000, 2000, 3000, 5000) if c < steps]
    return out + [steps]


def spectrum_errors(e_form, e_ref):
    """Relative errors of a kinetic-energy spectrum (shells k = 1 ..) against
    the FP64 form's: L2 over all shells, and the largest over the shells that
    hold at least 1e-3 of the peak shell's energy."""
    import numpy as np

    a = np.asarray(e_form[1:], dtype=np.float64)
    b = np.asarray(e_ref[1:], dtype=np.float64)
    l2 = float(np.sqrt(((a - b) ** 2).sum() / max((b * b).sum(), 1e-300)))
    sig = b >= 1e-3 * b.max()
    mx = float((np.abs(a - b)[sig] / b[sig]).max()) if sig.any() else 0.0
    return l2, mx, int(sig.sum())


def accuracy_run(w, forms, steps: int, stream_ptr: int):
    """The stated error of the reduced-precision forms: the same workload (full
    size, same seed) stepped in the plain FP64 form and in each chosen form on
    this GPU, compared at checkpoints up to ``steps``: max |phi~| difference
    (phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1), max |u| and |p| difference,
    droplet-volume drift (sum of w against the FP64 form's), the kinetic-energy
    spectrum by shell (dl_energy, enesupe_cal of
    program/turbulence_hit_xy.f90:588-645) and the dissipation rate in both
    conventions, 2 nu <S:S> (program/energy_budget.f90:1494) and
    0.5 nu <S:S> (program/turbulence_hit_xy.f90:449), from dl_reduce.
    The FP64 form's own speed is timed over its first chunk with CUDA events
    (its collide kernel with per-launch events)."""
    import numpy as np
    import torch
    from droplet_gb300.solver import Droplet

    nx, ny, nz = w.shape
    N = nx * ny * nz
    nb = nx // 2 + 1
    sims = {}
    for form in (64,) + tuple(forms):
        d = Droplet(w.params, w.shape, form, single_phase=w.single_phase)
        d.set_stream(stream_ptr)
        d.set_fields(**w.fields)
        d.init_equilibrium()
        d.set_force(w.force_mode)
        sims[form] = d
    # control: the FP64 form started from the fields as the FP32 forms store them
    # (phi - phi1, u, p - 1/3 rounded to FP32): how far rounding of the start
    # alone carries the chaotic flow in the same number of steps
    P = w.params
    rounded = {"phi": P.phi1 + (w.fields["phi"] - P.phi1).astype(np.float32).astype(np.float64),
               "u1": w.fields["u1"].astype(np.float32).astype(np.float64),
               "u2": w.fields["u2"].astype(np.float32).astype(np.float64),
               "u3": w.fields["u3"].astype(np.float32).astype(np.float64),
               "p": 1.0 / 3.0 + (w.fields["p"] - 1.0 / 3.0).astype(np.float32).astype(np.float64)}
    ctl = Droplet(w.params, w.shape, 64, single_phase=w.single_phase)
    ctl.set_stream(stream_ptr)
    ctl.set_fields(**rounded)
    ctl.init_equilibrium()
    ctl.set_force(w.force_mode)
    sims["ctl"] = ctl
    stream = torch.cuda.ExternalStream(stream_ptr)
    span = w.params.phi2 - w.params.phi1
    curves = {f: [] for f in forms}
    fp64_timing = None
    done = 0
    for c in checkpoints_for(steps):
        n = c - done
        for form, d in sims.items():
            if form == 64 and fp64_timing is None:
                d.profile(True, every=1)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                d.step(n)
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                pr = d.profile_read()
                d.profile(False)
                fp64_timing = {"steps": n, "ms_per_step": ms / n, "mlups": N * n / (ms / 1e3) / 1e6,
                               "collide_ms": pr["main_ms"] / max(pr["main_launches"], 1),
                               "launches_per_step": pr["launches"] / n}
            else:
                d.step(n)
        done = c
        ref_f = sims[64].get_fields()
        ref_d = sims[64].reduce()
        ref_e = sims[64].energy(nb)
        for form in forms:
            a = sims[form].get_fields()
            dd = sims[form].reduce()
            ee = sims[form].energy(nb)
            row = {"step": c,
                   "u_max": float(max(np.abs(a[k] - ref_f[k]).max() for k in ("u1", "u2", "u3"))),
                   "p_max": float(np.abs(a["p"] - ref_f["p"]).max())}
            if not w.single_phase:
                row["phi_tilde_max"] = float(2.0 * np.abs(a["phi"] - ref_f["phi"]).max() / span)
                row["volume_drift_rel"] = float((dd["vol_smooth"] - ref_d["vol_smooth"]) / ref_d["vol_smooth"])
            l2, mx, nsig = spectrum_errors(ee["spectrum"], ref_e["spectrum"])
            row["spectrum_rel_l2"] = l2
            row["spectrum_rel_max"] = mx
            row["ke_rel"] = float((dd["ke"] - ref_d["ke"]) / ref_d["ke"])
            row["dissipation_2nu"] = dd["diss"] / N
            row["dissipation_rel"] = float((dd["diss"] - ref_d["diss"]) / ref_d["diss"])
            curves[form].append(row)
        cf, cd, ce = sims["ctl"].get_fields(), sims["ctl"].reduce(), sims["ctl"].energy(nb)
        l2c, mxc, _ = spectrum_errors(ce["spectrum"], ref_e["spectrum"])
        crow = {"step": c, "u_max": float(max(np.abs(cf[k] - ref_f[k]).max() for k in ("u1", "u2", "u3"))),
                "spectrum_rel_l2": l2c, "spectrum_rel_max": mxc,
                "dissipation_rel": float((cd["diss"] - ref_d["diss"]) / ref_d["diss"])}
        if not w.single_phase:
            crow["phi_tilde_max"] = float(2.0 * np.abs(cf["phi"] - ref_f["phi"]).max() / span)
            crow["volume_drift_rel"] = float((cd["vol_smooth"] - ref_d["vol_smooth"]) / ref_d["vol_smooth"])
        curves.setdefault("fp64_rounded_start", []).append(crow)
        curves.setdefault("fp64_reference", []).append(
            {"step": c, "ke_mean": ref_d["ke"] / N, "dissipation_2nu": ref_d["diss"] / N,
             "dissipation_half_nu": 0.25 * ref_d["diss"] / N, "vol_smooth": ref_d["vol_smooth"]})
    for d in sims.values():
        d.close()
    out = {}
    for form in forms:
        last = dict(curves[form][-1])
        name = {32: "fp32", 16: "fp16"}[form]
        out[name] = {"vs": "plain FP64 form on the GPU", "steps": steps, **{k: v for k, v in last.items() if k != "step"},
                     "curve": curves[form]}
    out["fp64_reference"] = curves["fp64_reference"]
    out["fp64_rounded_start"] = {
        "what": "the FP64 form started from the FP32-rounded fields, against the FP64 form: the divergence that "
                "rounding the start alone causes in this flow (a floor for any reduced-precision form)",
        "curve": curves["fp64_rounded_start"]}
    out["spectrum_shells"] = f"k = 1..{nb - 1}; max over shells holding >= 1e-3 of the peak shell"
    out["dissipation_conventions"] = "dissipation_2nu = 2 nu <S:S> per site; 0.5 nu <S:S> = dissipation_2nu / 4"
    return out, fp64_timing


def time_form(w, form: int, steps: int, stream, tune: bool = True):
    """MLUPS of ``steps`` steps of workload ``w`` in ``form`` (device-timed,
    inputs resident) and the dominant kernel's time from per-launch events in
    a second pass of at least 20 launches."""
    import torch

    nx, ny, nz = w.shape
    N = nx * ny * nz
    sim = new_sim(w)
    sim.set_stream(stream.cuda_stream)
    tuned = None
    if tune and form != 64:
        from droplet_gb300 import autotune

        tuned = autotune.tune_droplet(sim)
    sim.step(3)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    kern = kernel_sample(sim, max(20, min(steps, 50)))
    sim.sync()
    sim.close()
    return {"mlups": round(N * steps / (ms / 1e3) / 1e6, 3), "ms_per_step": round(ms / steps, 5),
            "steps": steps, **kern, "tune": None if tuned is None else tuned.get("lz")}


def kernel_sample(sim, launches: int):
    """The dominant kernel's mean duration from CUDA events around each of
    ``launches`` consecutive steps (run after the timed region, untimed)."""
    import torch

    sim.profile(True, every=1)
    sim.step(launches)
    torch.cuda.synchronize()
    pr = sim.profile_read()
    sim.profile(False)
    return {"kernel_ms": round(pr["main_ms"] / max(pr["main_launches"], 1), 5),
            "kernel_samples": int(pr["main_launches"]),
            "kernel_share": round(pr["main_ms"] / max(pr["total_ms"], 1e-12), 4)}


def physical_cores():
    """Physical cores of this host from lscpu (unique core, socket pairs);
    falls back to the logical CPU count."""
    try:
        r = subprocess.run(["lscpu", "-p=CORE,SOCKET"], capture_output=True, text=True, timeout=10)
        pairs = {tuple(l.split(",")[:2]) for l in r.stdout.splitlines() if l and not l.startswith("#")}
        if pairs:
            return len(pairs), "lscpu physical cores"
    except Exception:
        pass
    return os.cpu_count() or 1, "os.cpu_count (lscpu unavailable)"


def cpu_protocol_env():
    """OpenMP placement of the CPU baseline: one thread per physical core,
    OMP_PROC_BIND=close, set before the oracle's OpenMP runtime starts."""
    cores, source = physical_cores()
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    return cores, source


E2E_MIN_STEPS = 1000  # steps of the end-to-end run (at least; more when --steps is larger)
OUTPUT_EVERY = 1000   # field output interval of the end-to-end run
CPU_WARMUP, CPU_REPS, CPU_STEPS = 20, 5, 200  # CPU timing protocol: 20 warm-up + 5 x 200 timed steps, median


def cpu_protocol(w, budget_s: float, warmup: int = CPU_WARMUP, reps: int = CPU_REPS, steps: int = CPU_STEPS):
    """Oracle (OpenMP restatement of the reference loops) MLUPS by the stated
    protocol: ``warmup`` steps, then ``reps`` timed runs of ``steps`` steps,
    median; on the full domain if that fits ``budget_s`` of CPU time, else on a
    slab of the domain (all x, y; the first nz_s planes) with the same physics."""
    import numpy as np

    cores, source = cpu_protocol_env()
    from oracle import pyoracle

    pyoracle.set_threads(cores)
    nx, ny, nz = w.shape
    # per-site rate on one step of a thin slab
    nz_p = min(nz, 8)
    sub = {k: np.ascontiguousarray(v[:nz_p]) for k, v in w.fields.items()}
    o = pyoracle.OracleDroplet(w.params, (nx, ny, nz_p), single_phase=w.single_phase)
    o.set_fields(**sub)
    o.init_equilibrium()
    o.set_force(w.force_mode)
    o.step(1)
    t0 = time.perf_counter()
    o.step(2)
    rate = nx * ny * nz_p * 2 / (time.perf_counter() - t0)
    o.close()
    total = warmup + reps * steps
    nz_s = int(max(4, min(nz, budget_s * rate / (nx * ny * total))))
    sub = {k: np.ascontiguousarray(v[:nz_s]) for k, v in w.fields.items()}
    o = pyoracle.OracleDroplet(w.params, (nx, ny, nz_s), single_phase=w.single_phase)
    o.set_fields(**sub)
    o.init_equilibrium()
    o.set_force(w.force_mode)
    o.step(warmup)
    runs = []
    for _ in range(reps):
        t0 = time.perf_counter()
        o.step(steps)
        runs.append(nx * ny * nz_s * steps / (time.perf_counter() - t0) / 1e6)
    o.close()
    value = statistics.median(runs)
    sample = (f"{warmup} warm-up + {reps} x {steps} timed steps, median, on a {nx}x{ny}x{nz_s} "
              f"{'domain' if nz_s == nz else 'slab'} of the {w.name} workload (same physics); FP64 C/OpenMP "
              f"restatement of the reference loops; {cores} threads = {source}, OMP_PROC_BIND="
              f"{os.environ.get('OMP_PROC_BIND')}, OMP_PLACES={os.environ.get('OMP_PLACES')}")
    return ({"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
             "runs": [round(r, 3) for r in runs]}, nx * ny * nz_s)


def run_reference(args):
    """--impl reference: the CPU restatement on the host's physical cores
    (OMP_PROC_BIND=close): ``--warmup`` (at least 20) warm-up steps, then the
    ``--steps`` timed steps in 5 runs, median MLUPS, on a slab of the workload
    sized to keep the run within a few minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from droplet_gb300 import configs  # noqa: F401  (workload generation)

    form = FORMS[args.form]
    w = make_workload(args.workload, form)
    reps = CPU_REPS if args.steps >= CPU_REPS else 1
    per = max(1, args.steps // reps)
    warm = max(args.warmup, CPU_WARMUP)
    cpu, sites = cpu_protocol(w, budget_s=120.0, warmup=warm, reps=reps, steps=per)
    value = cpu["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": w.name, "form": "fp64 (CPU)", "sites": w.n_sites, "seed": w.seed},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["ms_per_step"] = round(sites / (value * 1e6) * 1e3, 4)
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    form = FORMS[args.form]
    w = make_workload(args.workload, form)
    nx, ny, nz = w.shape
    N = nx * ny * nz
    stream = torch.cuda.Stream()
    sim = new_sim(w, rank)
    sim.set_stream(stream.cuda_stream)
    tune = None
    if form != 64 and not args.no_tune:
        from droplet_gb300 import autotune

        tune = autotune.tune_droplet(sim)
    sim.step(args.warmup)
    sim.sync()

    # ---- timed region: K steps, events on the library's stream -------------------
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    # events around every stride-th launch: the kernel's duration is sampled live
    # inside the timed region, at least 10 launches whatever --steps is, without
    # the events' own cost on every step
    stride = event_stride(args.steps)
    sim.profile(True, every=stride)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    prof = sim.profile_read()
    sim.profile(False)
    clk = clocks.stop()
    sim.sync()  # raises if the NaN watchdog tripped
    ms = max_over_ranks(ms, dist)
    value = N * args.steps * world / (ms / 1e3) / 1e6

    # roofline of the dominant kernel. When the timed region holds nothing but one
    # launch of it per step, its average launch duration is the region's time over
    # the launches (gaps between launches included, so an upper bound); otherwise
    # the launches sampled with events around them (each interval then also holds
    # the events' own cost)
    peak, peak_kind = measured_peak_gbs()
    sampled_ms = prof["main_ms"] / max(prof["main_launches"], 1)  # main_launches: the sampled ones
    one_launch_per_step = int(prof["launches"]) == args.steps and prof["main_ms"] >= 0.999 * prof["total_ms"]
    avg_main_ms = ms / args.steps if one_launch_per_step else sampled_ms
    bytes_per_launch = bytes_per_site(form, w.single_phase) * N
    achieved = bytes_per_launch / (avg_main_ms / 1e3) / 1e9
    # the FP32 form steps in the push form where eligible (its own kernel)
    kname = "step_push" if (form != 64 and sim.get_option("pushed")) else MAIN_KERNEL[form]
    traffic = committed_traffic(f"{kname}_{args.form}", w.name)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": kname, "kernel_ms": round(avg_main_ms, 5),
                "kernel_ms_source": ("timed region / launches (one launch of the kernel per step)"
                                     if one_launch_per_step else "event-sampled launches"),
                "kernel_ms_event_sampled": round(sampled_ms, 5),
                "kernel_share": round(prof["main_ms"] / max(prof["total_ms"], 1e-12), 4),
                "timed_launches": int(prof["timed_launches"]), "event_stride": stride,
                "algorithmic_bytes_per_launch": bytes_per_launch}
    # cross-check: events around every launch of a separate untimed pass
    kp = kernel_sample(sim, 30)
    roofline["kernel_ms_every_launch_pass"] = kp["kernel_ms"]
    roofline["every_launch_pass_samples"] = kp["kernel_samples"]
    if form != 64:
        # the same pull pattern with no arithmetic, on this GPU, after the timed region
        ceil_gbps = sim.pull_ceiling(20)
        roofline["pull_pattern_ceiling"] = round(ceil_gbps, 1)
        roofline["achieved_over_pull_pattern_ceiling"] = round(achieved / ceil_gbps, 4)
    else:
        # the plain form is bound by the FP64 pipe: flops from the committed SASS counts,
        # peak = this GPU's measured FP64 FMA throughput
        flops = committed_traffic(f"flops:{MAIN_KERNEL[form]}_{args.form}", w.name)
        peak64 = sim.fp64_ceiling()
        hbm = dict(roofline)
        roofline = {"bound": "fp64", "achieved": None, "peak": round(peak64, 4), "unit": "TFLOP/s", "frac": None,
                    "traffic": None, "peak_source": "measured (dl_fp64_ceiling)", "kernel": MAIN_KERNEL[form],
                    "kernel_ms": hbm["kernel_ms"], "kernel_share": hbm["kernel_share"],
                    "flops_per_launch": flops, "hbm": hbm}
        if flops:
            tf = flops / (avg_main_ms / 1e3) / 1e12
            roofline["achieved"] = round(tf, 4)
            roofline["frac"] = round(tf / peak64, 4)

    # ---- e2e through the C-ABI with host buffers ------------------------------------
    e2e = None
    if not args.no_e2e:
        # a run as the reference's main loop makes one: at least E2E_MIN_STEPS steps, the
        # fields written out every OUTPUT_EVERY steps (step_output, program/lbm_drop_xy.f90:28,842)
        k_e2e = max(args.steps, E2E_MIN_STEPS)
        pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in w.fields.items()}
        out = {k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy() for k, v in w.fields.items()}
        from droplet_gb300.solver import Droplet

        sim2 = Droplet(w.params, w.shape, w.form, single_phase=w.single_phase)
        sim2.set_stream(stream.cuda_stream)
        if tune is not None:
            for k in ("lz", "prefetch", "pipeline", "stage"):
                if k in tune:
                    sim2.set_option(k, tune[k])
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        sim2.set_fields(**pinned)
        sim2.init_equilibrium()
        sim2.set_force(w.force_mode)
        n_full = n_out = 0
        # every step's phi range (the viscosity interpolation's input) reaches the host:
        # the step that takes the counter to n writes it into pinned slot n % 2 itself
        # (dl_set_minmax_mirror), read on the host one step behind while step n+1 runs
        slots = torch.zeros((2, 2), dtype=torch.float64).pin_memory()
        sim2.set_minmax_mirror(slots.data_ptr(), 2)
        done = [torch.cuda.Event(), torch.cuda.Event()]
        seen = []
        # the push form's launch n writes step n-1's range (the state it loads) into slot n-1
        lag = 1 if sim2.get_option("push_eligible") else 0
        for k in range(k_e2e):
            sim2.step(1)
            done[k % 2].record(stream)
            if k > 0:
                done[(k - 1) % 2].synchronize()
                seen.append(float(slots[(k - lag) % 2, 1]))
            if (k + 1) % args.diag_every == 0 or k + 1 == k_e2e:
                sim2.reduce()  # device -> host read of the whole-domain diagnostics
                n_full += 1
            if (k + 1) % OUTPUT_EVERY == 0 and k + 1 < k_e2e:
                sim2.get_fields_into(out)  # the periodic field output (D2H)
                n_out += 1
        done[(k_e2e - 1) % 2].synchronize()
        seen.append(float(slots[(k_e2e - lag) % 2, 1]))
        assert len(seen) == k_e2e
        sim2.get_fields_into(out)
        n_out += 1
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        dt = max_over_ranks(dt, dist)
        sim2.close()
        from droplet_gb300 import _abi
        import ctypes

        h2d = 5 * N * 8
        d2h = n_out * 5 * N * 8 + k_e2e * 16 + n_full * ctypes.sizeof(_abi.DLDiag)
        e2e = {"value": round(N * k_e2e * world / dt / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(round(h2d / k_e2e)), "d2h_bytes_per_step": int(round(d2h / k_e2e)),
               "steps": k_e2e,
               "note": "set_fields(host) + init_equilibrium + per step: dl_step(1), whose last block writes "
                       "the step's phi range into pinned host memory (dl_set_minmax_mirror), read on the host "
                       "one step behind; "
                       f"dl_reduce (D2H of the diagnostics) every {args.diag_every} steps; dl_get_fields(host) "
                       f"every {OUTPUT_EVERY} steps and at the end; all timed"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, _ = cpu_protocol(w, budget_s=args.cpu_budget)

    # ---- the rest of the metric, same invocation ----------------------------------------
    accuracy, forms = None, {}
    acc_steps = w.steps if args.accuracy_steps < 0 else args.accuracy_steps
    if rank == 0 and form != 64 and acc_steps > 0:
        chosen = (32, 16) if not w.single_phase else (form,)
        accuracy, fp64_t = accuracy_run(w, chosen, acc_steps, stream.cuda_stream)
        peak64 = sim.fp64_ceiling()
        flops = committed_traffic(f"flops:{MAIN_KERNEL[64]}_fp64", w.name)
        forms["fp64"] = {"mlups": round(fp64_t["mlups"], 3), "ms_per_step": round(fp64_t["ms_per_step"], 5),
                         "steps": fp64_t["steps"], "collide_ms": round(fp64_t["collide_ms"], 5),
                         "launches_per_step": fp64_t["launches_per_step"],
                         "hbm_frac": round(bytes_per_site(64, w.single_phase) * N / (fp64_t["ms_per_step"] / 1e3)
                                           / 1e9 / peak, 4),
                         "fp64_ceiling_tflops": round(peak64, 4), "bound": "fp64"}
        if flops:
            tf = flops / (fp64_t["collide_ms"] / 1e3) / 1e12
            forms["fp64"]["collide_tflops"] = round(tf, 4)
            forms["fp64"]["fp64_ceiling_frac"] = round(tf / peak64, 4)
        forms["fp64"]["note"] = "timed in the accuracy leg's first chunk (CUDA events on the stream)"
    if rank == 0 and form != 64 and not w.single_phase and not args.no_extras:
        other = 16 if form == 32 else 32
        w2 = make_workload(args.workload, other)
        t2 = time_form(w2, other, max(args.steps, 100), stream, tune=not args.no_tune)
        t2["hbm_frac"] = round(bytes_per_site(other, False) * N / (t2["kernel_ms"] / 1e3) / 1e9 / peak, 4)
        t2["achieved_gbs"] = round(bytes_per_site(other, False) * N / (t2["kernel_ms"] / 1e3) / 1e9, 1)
        forms[{16: "fp16", 32: "fp32"}[other]] = t2
    extras = {}
    if rank == 0 and world == 1 and args.workload == "config2" and not args.no_extras:
        sim.close()
        sim = None
        torch.cuda.synchronize()
        extras["ensemble_config4"] = measure_ensemble(args.members, 100, 32, stream)
        extras["adjoint_config5"] = measure_adjoint(500)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[form], "data": "synthetic (seeded)",
            "config": {"workload": w.name, "form": args.form, "sites": N, "shape": list(w.shape),
                       "seed": w.seed, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (populations {:.0f} MB)".format(
                           bytes_per_site(form, w.single_phase) * N / 2 / 1e6),
                       "notes": w.notes,
                       "tune": None if tune is None else {k: v for k, v in tune.items() if k != "timings"}},
            "roofline": roofline,
            "accuracy": accuracy,
            "forms": forms or None,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": int(prof["launches"]),
        }
        if extras:
            line["adjoint_over_forward"] = extras["adjoint_config5"]["adjoint_over_forward"]
            line["ensemble"] = extras["ensemble_config4"]
            line["adjoint"] = extras["adjoint_config5"]
        print(json.dumps(line), flush=True)
    if sim is not None:
        sim.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def measure_ensemble(n_members: int, steps: int, form: int, stream, tune: bool = True):
    """config4: ``n_members`` members of uneven size stepped together (the
    members' own one-launch steps on concurrent streams; option "persistent":
    one launch per step over all members), against the same members one
    launch at a time. Returns MLUPS of both and the batched launch's HBM rate."""
    import torch
    from droplet_gb300 import autotune, configs
    from droplet_gb300.ensemble import Ensemble
    from droplet_gb300.solver import Droplet

    ws = configs.ensemble_members(n_members=n_members, form=form)
    sites = sum(w.n_sites for w in ws)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(persistent):
        ens = Ensemble([w.params for w in ws], [w.shape for w in ws], form)
        ens.set_stream(stream.cuda_stream)
        for mem, w in zip(ens.members, ws):
            mem.set_fields(**w.fields)
            mem.init_equilibrium()
            mem.set_force(w.force_mode)
        ens.set_option("persistent", persistent)
        tuned = autotune.tune_ensemble(ens) if tune else {"lz": int(ens.get_option("lz"))}
        ens.step(4)
        ens.sync()
        ens.profile(True, every=EVENT_STRIDE)
        torch.cuda.synchronize()
        e0.record(stream)
        ens.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        prof = ens.profile_read()
        ens.profile(False)
        ens.sync()
        ens.close()
        return ms, tuned, prof

    # the default mode (members' own steps on concurrent streams), then one
    # persistent launch per step over all members (push form, CUDA graph)
    ms, tuned, prof = timed(0)
    persistent = 0
    value = sites * steps / (ms / 1e3) / 1e6
    ms_p, tuned_p, prof_p = timed(1)
    value_p = sites * steps / (ms_p / 1e3) / 1e6
    # the same members, one launch per member per step
    k_seq = min(steps, 40)
    solos = []
    for w in ws:
        d = Droplet(w.params, w.shape, form)
        d.set_stream(stream.cuda_stream)
        d.set_fields(**w.fields)
        d.init_equilibrium()
        d.set_force(w.force_mode)
        d.set_option("lz", min(tuned["lz"], w.shape[2]))
        d.step(2)
        solos.append(d)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(k_seq):
        for d in solos:
            d.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_seq = e0.elapsed_time(e1)
    seq = sites * k_seq / (ms_seq / 1e3) / 1e6
    for d in solos:
        d.close()
    peak, _ = measured_peak_gbs()
    achieved = BYTES_PER_SITE[form] * sites / (ms / steps / 1e3) / 1e9
    achieved_p = BYTES_PER_SITE[form] * sites / (ms_p / steps / 1e3) / 1e9
    return {"workload": f"ensemble_{len(ws)}_members", "members": len(ws), "sites": sites,
            "member_sizes": sorted({w.shape[0] for w in ws}), "seed": 4, "steps": steps,
            "mlups": round(value, 3), "ms_per_step": round(ms / steps, 5),
            "sequential_mlups": round(seq, 3), "batched_over_sequential": round(value / seq, 3),
            "mode": "persistent launch + graph" if persistent else "members' one-launch steps on concurrent streams",
            "hbm_frac": round(achieved / peak, 4), "achieved_gbs": round(achieved, 1),
            "tune": {k: v for k, v in tuned.items() if k != "timings"}, "gpu_launches": int(prof["launches"]),
            "persistent": {"mode": "one persistent launch per step over all members' tiles (push form, work items "
                                   "taken from a counter), two steps per CUDA graph replay",
                           "mlups": round(value_p, 3), "ms_per_step": round(ms_p / steps, 5),
                           "hbm_frac": round(achieved_p / peak, 4), "achieved_gbs": round(achieved_p, 1),
                           "batched_over_sequential": round(value_p / seq, 3),
                           "tune": {k: v for k, v in tuned_p.items() if k != "timings"},
                           "gpu_launches": int(prof_p["launches"])}}


def run_ensemble(args):
    """--workload config4 as a bench line of its own."""
    import torch

    torch.cuda.set_device(0)
    form = FORMS[args.form]
    stream = torch.cuda.Stream()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    r = measure_ensemble(args.members, args.steps, form, stream, tune=not args.no_tune)
    clk = clocks.stop()
    peak, peak_kind = measured_peak_gbs()
    line = {
        "metric": METRIC, "value": r["mlups"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[form], "data": "synthetic (seeded)",
        "config": {"workload": r["workload"], "form": args.form, "sites": r["sites"],
                   "member_sizes": r["member_sizes"], "seed": r["seed"],
                   "sequential_mlups": r["sequential_mlups"], "batched_over_sequential": r["batched_over_sequential"],
                   "mode": r["mode"], "tune": r["tune"], "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": r["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": r["hbm_frac"], "traffic": None, "peak_source": peak_kind,
                     "kernel": "step_batched" if "persistent" in r["mode"] else "step_fused (members concurrent)",
                     "kernel_ms": r["ms_per_step"]},
        "cpu_baseline": None, "e2e": None, "clocks": clk, "gpu_launches": r["gpu_launches"],
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_adjoint(nsteps: int):
    """config5: forward and reverse (hand-written adjoint) of the 96^3 shear
    droplet over ``nsteps``; the adjoint/forward time ratio with every step's
    state kept in HBM (the default when it fits) and with sqrt(n) checkpoints."""
    import math
    import torch
    from droplet_gb300 import configs
    from droplet_gb300.adjoint import CheckpointedRun

    w = configs.config5()
    f = w.fields
    res = {}
    for label, seg in (("stored", None), ("sqrt_checkpoints", max(1, math.ceil(math.sqrt(nsteps))))):
        run = CheckpointedRun(w.params, w.shape, (f["u1"], f["u2"], f["u3"]), f["p"], nsteps, segment=seg)
        run.forward(f["phi"])  # warm-up pass (builds, allocates)
        run.backward(download=False)
        D = run.forward(f["phi"])
        g = run.backward(download=False)
        res[label] = (run.timing.forward_s, run.timing.backward_s, run.S, D, g)
        run.close()
        torch.cuda.synchronize()
    N = w.n_sites
    fwd, bwd, S, D, g = res["stored"]
    fwd2, bwd2, S2, _, _ = res["sqrt_checkpoints"]
    return {"workload": w.name + " adjoint", "form": "fp32", "sites": N, "steps": nsteps,
            "forward_mlups": round(N * nsteps / fwd / 1e6, 3),
            "adjoint_over_forward": round(bwd / fwd, 3), "forward_s": round(fwd, 4), "backward_s": round(bwd, 4),
            "states_kept": S, "adjoint_over_forward_sqrt_checkpoints": round(bwd2 / fwd2, 3),
            "sqrt_checkpoints": {"every": S2, "forward_s": round(fwd2, 4), "backward_s": round(bwd2, 4)},
            "loss_D": D, "grads": {k: v for k, v in g.items() if k != "dphi0"},
            "note": "forward = n steps with state saves and the device loss; backward = device loss gradient + "
                    "reverse steps (+ segment recomputation with sqrt(n) checkpoints) + reverse of the initial "
                    "equilibrium; dD/dphi0 stays on the device"}


def run_adjoint(args):
    """--workload config5 as a bench line of its own."""
    import torch

    torch.cuda.set_device(0)
    nsteps = args.steps if args.steps else 500
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    r = measure_adjoint(nsteps)
    clk = clocks.stop()
    line = {
        "metric": METRIC, "value": r["forward_mlups"], "unit": UNIT, "n_gpus": 1, "steps": nsteps, "warmup": 1,
        "ms_per_step": round(r["forward_s"] * 1e3 / nsteps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": r, "roofline": None, "cpu_baseline": None, "e2e": None, "clocks": clk, "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=sorted(FORMS), default="fp32")
    ap.add_argument("--workload", default="config2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU work of the CPU baseline (sets the slab size)")
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--accuracy-steps", type=int, default=-1,
                    help="steps of the FP64-form comparison that states the phi error "
                         "(-1: the workload's own run length, 5000 for config2; 0: skip)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the other forms, the ensemble and the adjoint in the default line")
    ap.add_argument("--diag-every", type=int, default=100, help="steps between whole-domain diagnostics in e2e")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "config4":
        return run_ensemble(args)
    if args.workload == "config5":
        return run_adjoint(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
