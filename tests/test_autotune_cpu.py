"""The autotuner's search and cache, driven by a fake timing source (no GPU)."""
import json

from droplet_gb300 import autotune


class FakeSim:
    """Looks like a Droplet to the tuner; lz = 8 with the prefetch on is fastest."""

    def __init__(self):
        self.nx = self.ny = self.nz = 64
        self.form = 32
        self.lz = 16
        self.prefetch = 0
        self.steps = 0

        class P:
            les = True

        self.params = P()

    def set_option(self, k, v):
        assert k in ("lz", "prefetch")
        setattr(self, k, v)

    def get_option(self, k):
        assert k == "push_eligible"
        return 0

    def step(self, n):
        self.steps += n

    def profile(self, on):
        self.steps = 0

    def profile_read(self):
        return {"main_ms": self.steps * (1.0 + abs(self.lz - 8) / 8.0 - 0.1 * self.prefetch)}


def test_tuner_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("DROPLET_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "gpu_name", lambda: "fake-gpu")
    sim = FakeSim()
    r = autotune.tune_droplet(sim, steps=5)
    assert r["lz"] == 8 and sim.lz == 8 and r["prefetch"] == 1 and sim.prefetch == 1 and not r["cached"]
    data = json.load(open(tmp_path / "tune.json"))
    assert len(data) == 1 and "fake-gpu" in next(iter(data))
    sim2 = FakeSim()
    r2 = autotune.tune_droplet(sim2, steps=5)
    assert r2["cached"] and sim2.lz == 8 and sim2.prefetch == 1 and sim2.steps == 0


class FakePushSim(FakeSim):
    """A handle that steps in the push form: its knob is "stage" (lz = 16 with
    staging fastest); "prefetch" is never set."""

    def __init__(self):
        super().__init__()
        self.stage = 0

    def set_option(self, k, v):
        assert k in ("lz", "stage")
        setattr(self, k, v)

    def get_option(self, k):
        assert k == "push_eligible"
        return 1

    def profile_read(self):
        return {"main_ms": self.steps * (1.0 + abs(self.lz - 16) / 16.0 - 0.1 * self.stage)}


def test_tuner_push_form_tunes_staging(tmp_path, monkeypatch):
    monkeypatch.setenv("DROPLET_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "gpu_name", lambda: "fake-gpu")
    sim = FakePushSim()
    r = autotune.tune_droplet(sim, steps=5)
    # full 32 x 8 tiles: the tensor-copy staging (2) is a candidate
    assert r["lz"] == 16 and r["stage"] == 2 and "prefetch" not in r and sim.stage == 2
    # a partial tile in x: stages 0 and 1 only
    sim2 = FakePushSim()
    sim2.nx = 40
    r2 = autotune.tune_droplet(sim2, steps=5)
    assert r2["stage"] == 1 and sim2.stage == 1 and not r2["cached"]


class FakeEnsemble:
    """Looks like an Ensemble to the tuner: lz = 16 is fastest by wall clock in the
    concurrent mode; lz = 8 with 2 blocks per SM by launch time in the persistent one."""

    def __init__(self, persistent):
        class M:
            nx = ny = nz = 48

            class params:
                les = True

        self.members = [M(), M()]
        self.form = 32
        self.opts = {"lz": 32, "blocks_per_sm": 2, "persistent": persistent}
        self.steps = 0
        self.clock = 0.0

    def get_option(self, k):
        return self.opts[k]

    def set_option(self, k, v):
        assert k in ("lz", "blocks_per_sm")
        self.opts[k] = v

    def step(self, n):
        lz, bps = self.opts["lz"], self.opts["blocks_per_sm"]
        cost = 1.0 + abs(lz - 16) / 16.0 if not self.opts["persistent"] else 1.0 + abs(lz - 8) / 8.0 + (bps != 2)
        self.clock += n * cost * 1e-3
        self.steps += n

    def sync(self):
        pass

    def profile(self, on):
        self.steps = 0

    def profile_read(self):
        lz, bps = self.opts["lz"], self.opts["blocks_per_sm"]
        return {"main_ms": self.steps * (1.0 + abs(lz - 8) / 8.0 + (bps != 2))}


def test_ensemble_tuner_times_concurrent_members_by_wall_clock(tmp_path, monkeypatch):
    monkeypatch.setenv("DROPLET_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "gpu_name", lambda: "fake-gpu")
    ens = FakeEnsemble(persistent=0)
    monkeypatch.setattr("time.perf_counter", lambda: ens.clock)
    r = autotune.tune_ensemble(ens, steps=4)
    assert r["lz"] == 16 and ens.opts["lz"] == 16 and ens.opts["blocks_per_sm"] == 2
    assert set(r["timings"]) == {f"lz{lz}_bps2" for lz in autotune.LZ_CANDIDATES}
    pers = FakeEnsemble(persistent=1)
    r2 = autotune.tune_ensemble(pers, steps=4)
    assert r2["lz"] == 8 and r2["blocks_per_sm"] == 2 and not r2["cached"]
    assert len(json.load(open(tmp_path / "tune.json"))) == 2  # one cache entry per mode
