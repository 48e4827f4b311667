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
