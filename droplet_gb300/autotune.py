"""Autotuner for the launch shape of the fused step.

The tunable knobs are those of the C-ABI: for one domain the number of z
planes a block marches ("lz", ``dl_set_option``) and, in the push form, the
staging of the next plane ("stage" 0, 1, and 2 on full 32 x 8 tiles), in the
pull form the bulk L2 prefetch ("prefetch") and, for the single-phase step,
"pipeline"; for an ensemble "lz"
and, with its persistent launch, the number of blocks per SM
("blocks_per_sm", ``dl_batch_set_option``). Each candidate is timed after a
few warm-up steps, with the library's own per-launch CUDA events (one domain,
persistent ensemble) or by wall clock (members launched concurrently, whose
kernels overlap); the fastest is applied and cached in a JSON file keyed by
the GPU, the form and the member shapes, so later runs reuse it without
timing. The cache lives at $DROPLET_GB300_TUNE_CACHE or
~/.cache/droplet_gb300/tune.json.
"""
from __future__ import annotations

import itertools
import json
import os
import threading

LZ_CANDIDATES = (4, 8, 16, 32, 64)
BPS_CANDIDATES = (1, 2)
_lock = threading.Lock()


def cache_path() -> str:
    p = os.environ.get("DROPLET_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "droplet_gb300", "tune.json")


def _load() -> dict:
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _store(key: str, value: dict) -> None:
    with _lock:
        d = _load()
        d[key] = value
        p = cache_path()
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
        os.replace(tmp, p)


def gpu_name() -> str:
    try:
        import torch

        return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        return "unknown-gpu"


def _time_steps(obj, steps: int) -> float:
    obj.step(3)
    obj.profile(True)
    obj.step(steps)
    s = obj.profile_read()
    obj.profile(False)
    return s["main_ms"] / steps


def _key(kind: str, form: int, shapes, extra: str) -> str:
    sig = ",".join("x".join(str(v) for v in s) for s in sorted(tuple(s) for s in shapes))
    return f"{kind}|{gpu_name()}|form{form}|{extra}|{sig}"


def tune_droplet(sim, steps: int = 20, use_cache: bool = True) -> dict:
    """Pick "lz" and, for the push form, "stage", else "prefetch" (and, for
    the single-phase pull step, "pipeline") for one Droplet (fast forms).
    Returns the chosen settings."""
    p = sim.params
    single = bool(getattr(sim, "single_phase", False))
    # the push form (FP32 where eligible) has its own knob, the staging of the
    # next plane in shared memory; the pull form the L2 prefetch (and, single
    # phase, the register pipeline)
    push = bool(sim.get_option("push_eligible"))
    key = _key("single", sim.form, [(sim.nx, sim.ny, sim.nz)],
               f"les{int(bool(p.les))}" + ("_1phase" if single else "") + ("_push" if push else "_pf"))
    values = {"prefetch": (0, 1), "pipeline": (0, 1), "stage": (0, 1)}
    if push:
        knobs = ["stage"]
        # stage 2 (tensor copies) needs full 32 x 8 tiles
        if sim.nx % 32 == 0 and sim.ny % 8 == 0:
            values["stage"] = (0, 1, 2)
    else:
        knobs = ["prefetch"] + (["pipeline"] if single else [])
    if use_cache:
        hit = _load().get(key)
        if hit:
            sim.set_option("lz", hit["lz"])
            for k in knobs:
                sim.set_option(k, hit[k])
            return dict(hit, cached=True)
    best = None
    timings = {}
    combos = [dict(zip(knobs, v)) for v in itertools.product(*(values[k] for k in knobs))]
    for combo in combos:
        for k, v in combo.items():
            sim.set_option(k, v)
        for lz in LZ_CANDIDATES:
            if lz > sim.nz:
                continue
            sim.set_option("lz", lz)
            ms = _time_steps(sim, steps)
            timings["lz%d_" % lz + "_".join(f"{k}{v}" for k, v in combo.items())] = ms
            if best is None or ms < best[2]:
                best = (lz, combo, ms)
    sim.set_option("lz", best[0])
    for k, v in best[1].items():
        sim.set_option(k, v)
    res = dict({"lz": best[0], "ms_per_step": best[2], "timings": timings}, **best[1])
    _store(key, res)
    return dict(res, cached=False)


def _wall_steps(obj, steps: int) -> float:
    """Wall-clock ms per step of obj.step(steps) between two syncs (the members'
    launches overlap, so summed kernel times would not rank the shapes)."""
    import time

    obj.step(2)
    obj.sync()
    t0 = time.perf_counter()
    obj.step(steps)
    obj.sync()
    return (time.perf_counter() - t0) * 1e3 / steps


def tune_ensemble(ens, steps: int = 10, use_cache: bool = True) -> dict:
    """Pick "lz" (and, for the persistent launch, "blocks_per_sm") for an
    Ensemble in its current mode."""
    shapes = [(m.nx, m.ny, m.nz) for m in ens.members]
    persistent = int(ens.get_option("persistent"))
    key = _key("batch", ens.form, shapes, f"les{int(bool(ens.members[0].params.les))}_p{persistent}")
    if use_cache:
        hit = _load().get(key)
        if hit:
            ens.set_option("lz", hit["lz"])
            ens.set_option("blocks_per_sm", hit["blocks_per_sm"])
            return dict(hit, cached=True)
    best = None
    timings = {}
    for bps in (BPS_CANDIDATES if persistent else (2,)):
        for lz in LZ_CANDIDATES:
            ens.set_option("lz", lz)
            ens.set_option("blocks_per_sm", bps)
            ms = _time_steps(ens, steps) if persistent else _wall_steps(ens, steps)
            timings[f"lz{lz}_bps{bps}"] = ms
            if best is None or ms < best[2]:
                best = (lz, bps, ms)
    ens.set_option("lz", best[0])
    ens.set_option("blocks_per_sm", best[1])
    res = {"lz": best[0], "blocks_per_sm": best[1], "ms_per_step": best[2], "timings": timings}
    _store(key, res)
    return dict(res, cached=False)
