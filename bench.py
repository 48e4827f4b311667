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
EVENT_STRIDE = 10  # timed region: CUDA events around every 10th launch
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


def phi_error(w, steps: int, stream_ptr: int):
    """The stated error of the reduced-precision form: the same workload (full
    size, same seed) run `steps` steps in the plain FP64 form and in the chosen
    form on this GPU; max |phi~ difference| (phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1)
    and max |u| difference."""
    import numpy as np
    from droplet_gb300.solver import Droplet

    out, diag = {}, {}
    for form in (64, w.form):
        d = Droplet(w.params, w.shape, form, single_phase=w.single_phase)
        d.set_stream(stream_ptr)
        d.set_fields(**w.fields)
        d.init_equilibrium()
        d.set_force(w.force_mode)
        d.step(steps)
        out[form] = d.get_fields()
        diag[form] = d.reduce()
        d.close()
    a, b = out[w.form], out[64]
    span = w.params.phi2 - w.params.phi1
    res = {"vs": "plain FP64 form on the GPU", "steps": steps,
           "u_max": float(max(np.abs(a[k] - b[k]).max() for k in ("u1", "u2", "u3"))),
           "p_max": float(np.abs(a["p"] - b["p"]).max())}
    if not w.single_phase:
        res["phi_tilde_max"] = float(2.0 * np.abs(a["phi"] - b["phi"]).max() / span)
        v64 = diag[64]["vol_smooth"]
        res["volume_drift_rel"] = float((diag[w.form]["vol_smooth"] - v64) / v64)
    return res


def cpu_baseline(w, budget_s: float = 15.0, threads: int | None = None):
    """Oracle (OpenMP restatement) MLUPS on this host on a bounded sample of
    the workload: the full domain when a step fits the budget, else a slab."""
    from oracle import pyoracle

    threads = threads or os.cpu_count() or 1
    pyoracle.set_threads(threads)
    nx, ny, nz = w.shape
    o = pyoracle.OracleDroplet(w.params, w.shape, single_phase=w.single_phase)
    o.set_fields(**w.fields)
    o.init_equilibrium()
    o.set_force(w.force_mode)
    t0 = time.perf_counter()
    o.step(1)
    t1 = time.perf_counter()
    per = t1 - t0
    steps = max(1, min(200, int(budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": round(nx * ny * nz * steps / dt / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the full {nx}x{ny}x{nz} workload after 1 warm-up step, "
                      f"FP64 C/OpenMP restatement of the reference loops ({threads} threads)"}


def run_reference(args):
    """--impl reference: the CPU restatement on all host cores, K timed steps
    on a slab of the workload sized to keep the run within a few minutes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np
    from oracle import pyoracle
    from droplet_gb300 import configs

    form = FORMS[args.form]
    w = make_workload(args.workload, form)
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    nx, ny, nz = w.shape
    # probe the per-site rate on one step of the full domain
    o = pyoracle.OracleDroplet(w.params, w.shape, single_phase=w.single_phase)
    o.set_fields(**w.fields)
    o.init_equilibrium()
    o.set_force(w.force_mode)
    t0 = time.perf_counter()
    o.step(1)
    rate = nx * ny * nz / (time.perf_counter() - t0)
    o.close()
    budget = 120.0
    total_steps = args.steps + args.warmup
    nz_s = int(max(8, min(nz, budget * rate / (nx * ny * max(total_steps, 1)))))
    sub = dict((k, np.ascontiguousarray(v[:nz_s])) for k, v in w.fields.items())
    P = w.params
    o = pyoracle.OracleDroplet(P, (nx, ny, nz_s), single_phase=w.single_phase)
    o.set_fields(**sub)
    o.init_equilibrium()
    o.set_force(w.force_mode)
    o.step(args.warmup)
    t0 = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t0
    sites = nx * ny * nz_s
    value = sites * args.steps / dt / 1e6
    sample = (f"{args.steps} timed steps (after {args.warmup} warm-up) of a {nx}x{ny}x{nz_s} slab of the "
              f"{w.name} workload, same physics; FP64 C/OpenMP restatement of the reference loops")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / max(args.steps, 1), 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": w.name, "form": "fp64 (CPU)", "sites": sites, "seed": w.seed},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
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
    # events around every EVENT_STRIDE-th launch: the kernel's duration is sampled live
    # inside the timed region without the events' own cost on every step
    sim.profile(True, every=EVENT_STRIDE)
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

    # roofline of the dominant kernel (live per-launch events, sampled, over the timed region)
    peak, peak_kind = measured_peak_gbs()
    avg_main_ms = prof["main_ms"] / max(prof["main_launches"], 1)
    bytes_per_launch = bytes_per_site(form, w.single_phase) * N
    achieved = bytes_per_launch / (avg_main_ms / 1e3) / 1e9
    traffic = committed_traffic(f"{MAIN_KERNEL[form]}_{args.form}", w.name)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": MAIN_KERNEL[form], "kernel_ms": round(avg_main_ms, 5),
                "kernel_share": round(prof["main_ms"] / max(prof["total_ms"], 1e-12), 4),
                "timed_launches": int(prof["timed_launches"]), "event_stride": EVENT_STRIDE,
                "algorithmic_bytes_per_launch": bytes_per_launch}
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
        k_e2e = min(args.steps, 500)
        pinned = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in w.fields.items()}
        out = {k: torch.empty(v.shape, dtype=torch.float64).pin_memory().numpy() for k, v in w.fields.items()}
        from droplet_gb300.solver import Droplet

        sim2 = Droplet(w.params, w.shape, w.form, single_phase=w.single_phase)
        sim2.set_stream(stream.cuda_stream)
        if tune is not None:
            for k in ("lz", "prefetch", "pipeline"):
                if k in tune:
                    sim2.set_option(k, tune[k])
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        sim2.set_fields(**pinned)
        sim2.init_equilibrium()
        sim2.set_force(w.force_mode)
        n_full = 0
        # every step's phi range (the viscosity interpolation's input) reaches the host:
        # the step that takes the counter to n writes it into pinned slot n % 2 itself
        # (dl_set_minmax_mirror), read on the host one step behind while step n+1 runs
        slots = torch.zeros((2, 2), dtype=torch.float64).pin_memory()
        sim2.set_minmax_mirror(slots.data_ptr(), 2)
        done = [torch.cuda.Event(), torch.cuda.Event()]
        seen = []
        for k in range(k_e2e):
            sim2.step(1)
            done[k % 2].record(stream)
            if k > 0:
                done[(k - 1) % 2].synchronize()
                seen.append(float(slots[k % 2, 1]))
            if (k + 1) % args.diag_every == 0 or k + 1 == k_e2e:
                sim2.reduce()  # device -> host read of the whole-domain diagnostics
                n_full += 1
        done[(k_e2e - 1) % 2].synchronize()
        seen.append(float(slots[k_e2e % 2, 1]))
        assert len(seen) == k_e2e
        sim2.get_fields_into(out)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        dt = max_over_ranks(dt, dist)
        sim2.close()
        from droplet_gb300 import _abi
        import ctypes

        h2d = 5 * N * 8
        d2h = 5 * N * 8 + k_e2e * 16 + n_full * ctypes.sizeof(_abi.DLDiag)
        e2e = {"value": round(N * k_e2e * world / dt / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(round(h2d / k_e2e)), "d2h_bytes_per_step": int(round(d2h / k_e2e)),
               "steps": k_e2e,
               "note": "set_fields(host) + init_equilibrium + per step: dl_step(1), whose last block writes "
                       "the step's phi range into pinned host memory (dl_set_minmax_mirror), read on the host "
                       "one step behind; "
                       f"dl_reduce (D2H of the diagnostics) every {args.diag_every} steps; final "
                       "dl_get_fields(host); all timed"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, budget_s=args.cpu_budget)

    accuracy = None
    if rank == 0 and form != 64 and args.accuracy_steps > 0:
        accuracy = phi_error(w, args.accuracy_steps, stream.cuda_stream)

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
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": int(prof["launches"]),
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_ensemble(args):
    """config4: 64 members of uneven size stepped together (the members' own
    one-launch steps on concurrent streams; option "persistent": one launch
    per step over all members), against the same members one at a time."""
    import torch
    from droplet_gb300 import autotune, configs
    from droplet_gb300.ensemble import Ensemble
    from droplet_gb300.solver import Droplet

    torch.cuda.set_device(0)
    form = FORMS[args.form]
    ws = configs.ensemble_members(n_members=args.members, form=form)
    sites = sum(w.n_sites for w in ws)
    stream = torch.cuda.Stream()
    ens = Ensemble([w.params for w in ws], [w.shape for w in ws], form)
    ens.set_stream(stream.cuda_stream)
    for mem, w in zip(ens.members, ws):
        mem.set_fields(**w.fields)
        mem.init_equilibrium()
        mem.set_force(w.force_mode)
    ens_persistent = int(ens.get_option("persistent"))
    tune = autotune.tune_ensemble(ens)
    ens.step(args.warmup + (args.warmup % 2))
    ens.sync()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.3)
    ens.profile(True, every=EVENT_STRIDE)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ens.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    prof = ens.profile_read()
    ens.profile(False)
    clk = clocks.stop()
    ens.sync()
    value = sites * args.steps / (ms / 1e3) / 1e6
    ens.close()
    # the same members, one launch per member per step
    k_seq = min(args.steps, 40)
    solos = []
    for w in ws:
        d = Droplet(w.params, w.shape, form)
        d.set_stream(stream.cuda_stream)
        d.set_fields(**w.fields)
        d.init_equilibrium()
        d.set_force(w.force_mode)
        d.set_option("lz", tune["lz"])
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
    peak, peak_kind = measured_peak_gbs()
    achieved = BYTES_PER_SITE[form] * sites / (ms / args.steps / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE[form], "data": "synthetic (seeded)",
        "config": {"workload": f"ensemble_{len(ws)}_members", "form": args.form, "sites": sites,
                   "member_sizes": sorted({w.shape[0] for w in ws}), "seed": 4,
                   "sequential_mlups": round(seq, 3), "batched_over_sequential": round(value / seq, 3),
                   "tune": {k: v for k, v in tune.items() if k != "timings"},
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "kernel": "step_batched" if ens_persistent else "step_fused (members concurrent)",
                     "kernel_ms": round(ms / args.steps, 5)},
        "cpu_baseline": None, "e2e": None, "clocks": clk, "gpu_launches": int(prof["launches"]),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_adjoint(args):
    """config5: forward and reverse (hand-written adjoint) of the 96^3 shear
    droplet; reports the adjoint/forward time ratio with every step's state
    kept in HBM (the default when it fits) and with sqrt(n) checkpoints."""
    import math
    import torch
    from droplet_gb300 import configs
    from droplet_gb300.adjoint import CheckpointedRun

    torch.cuda.set_device(0)
    w = configs.config5()
    nsteps = args.steps if args.steps else w.steps
    f = w.fields
    res = {}
    clk = None
    for label, seg in (("stored", None), ("sqrt_checkpoints", max(1, math.ceil(math.sqrt(nsteps))))):
        run = CheckpointedRun(w.params, w.shape, (f["u1"], f["u2"], f["u3"]), f["p"], nsteps, segment=seg)
        run.forward(f["phi"])  # warm-up pass (builds, allocates)
        run.backward(download=False)
        clocks = ClockSampler(torch.cuda.current_device())
        if label == "stored":
            clocks.start()
            time.sleep(0.3)
        D = run.forward(f["phi"])
        g = run.backward(download=False)
        if label == "stored":
            clk = clocks.stop()
        res[label] = (run.timing.forward_s, run.timing.backward_s, run.S, D, g)
        run.close()
    N = w.n_sites
    fwd, bwd, S, D, g = res["stored"]
    fwd2, bwd2, S2, _, _ = res["sqrt_checkpoints"]
    value = N * nsteps / fwd / 1e6
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": 1, "steps": nsteps, "warmup": 1,
        "ms_per_step": round(fwd * 1e3 / nsteps, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": w.name + " adjoint", "form": "fp32", "sites": N,
                   "adjoint_over_forward": round(bwd / fwd, 3), "forward_s": round(fwd, 4),
                   "backward_s": round(bwd, 4), "states_kept": S,
                   "adjoint_over_forward_sqrt_checkpoints": round(bwd2 / fwd2, 3),
                   "sqrt_checkpoints": {"every": S2, "forward_s": round(fwd2, 4), "backward_s": round(bwd2, 4)},
                   "loss_D": D, "grads": {k: v for k, v in g.items() if k != "dphi0"},
                   "note": "forward = n steps with state saves and the device loss; backward = device loss "
                           "gradient + reverse steps (+ segment recomputation with sqrt(n) checkpoints) + "
                           "reverse of the initial equilibrium; dD/dphi0 stays on the device"},
        "roofline": None, "cpu_baseline": None, "e2e": None, "clocks": clk, "gpu_launches": None,
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
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--members", type=int, default=64)
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--accuracy-steps", type=int, default=500,
                    help="steps of the FP64-form comparison that states the phi error (0: skip)")
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
