"""Autotuner search and cache logic (CPU: a fake tracker and timer), and on
the GPU the tuned tracker's results against the default tuning."""
import json

import numpy as np
import pytest

import xtrack_gb300 as xt
from xtrack_gb300 import tuning as at


class FakeTracker:
    arith = "fast"
    device = None

    def __init__(self):
        self._records = np.arange(10, dtype=np.float64)
        self._cfg = b"cfg"
        self.tuning = {"block_size": 256, "compact_every": 0, "chunk_bytes": 49152, "use_graph": 0}
        self.applied = []

    def get_tuning(self):
        return dict(self.tuning)

    def set_tuning(self, **kw):
        self.tuning.update(kw)
        self.applied.append(dict(self.tuning))
        return dict(self.tuning)


class FakeParticles:
    _capacity = 3000


def cost(t):
    # minimum at block 128, chunk 16384, compact 8, graph 1
    return (abs(t["block_size"] - 128) / 64 + abs(t["chunk_bytes"] - 16384) / 16384
            + abs(t["compact_every"] - 8) / 8 + (1 - t["use_graph"]) * 0.1 + 1.0)


def test_coordinate_descent_finds_separable_minimum(tmp_path):
    tr = FakeTracker()
    calls = []
    timer = lambda t: (calls.append(t), cost(t))[1]
    best, rep = at.autotune(tr, FakeParticles(), 100, cache_path=str(tmp_path / "c.json"),
                            timer=timer, device_name="dev")
    assert best == {"block_size": 128, "compact_every": 8, "chunk_bytes": 16384, "use_graph": 1}
    assert rep["source"] == "search"
    assert tr.tuning == best
    # every distinct candidate timed once
    keys = [tuple(sorted(c.items())) for c in calls]
    assert len(keys) == len(set(keys))


def test_cache_hit_applies_stored_tuning_without_timing(tmp_path):
    path = str(tmp_path / "c.json")
    best, _ = at.autotune(FakeTracker(), FakeParticles(), 100, cache_path=path, timer=cost,
                          device_name="dev")
    tr = FakeTracker()

    def no_timer(t):
        raise AssertionError("timed on a cache hit")
    got, rep = at.autotune(tr, FakeParticles(), 100, cache_path=path, timer=no_timer,
                           device_name="dev")
    assert rep["source"] == "cache" and got == best and tr.tuning == best
    data = json.load(open(path))
    assert list(data) == [rep["key"]]
    # a different size bucket or device is a different key
    got2, rep2 = at.autotune(FakeTracker(), type("P", (), {"_capacity": 10**6})(), 100,
                             cache_path=path, timer=cost, device_name="dev")
    assert rep2["source"] == "search" and rep2["key"] != rep["key"]
    got3, rep3 = at.autotune(FakeTracker(), FakeParticles(), 100, cache_path=path, timer=cost,
                             device_name="other")
    assert rep3["source"] == "search"


def test_refresh_searches_again(tmp_path):
    path = str(tmp_path / "c.json")
    at.autotune(FakeTracker(), FakeParticles(), 100, cache_path=path, timer=cost, device_name="d")
    n = []
    at.autotune(FakeTracker(), FakeParticles(), 100, cache_path=path, refresh=True,
                timer=lambda t: (n.append(1), cost(t))[1], device_name="d")
    assert len(n) > 1


def test_key_buckets():
    assert at._pow2_bucket(1) == 1 and at._pow2_bucket(3000) == 4096 and at._pow2_bucket(4096) == 4096


@pytest.mark.gpu
def test_autotuned_tracker_matches_default(tmp_path):
    import torch
    from xtrack_gb300 import workloads
    line = workloads.toy_ring()
    p0c = 450e9
    beam = workloads.gaussian_beam(4000, p0c, seed=3, device="cuda", sigma_x=8e-3, sigma_px=8e-5)
    ref = beam.copy()
    t_def = line.build_tracker(device="cuda", arith="fast")
    t_def._track(ref, num_turns=30)
    tr = line.build_tracker(device="cuda", arith="fast")
    path = str(tmp_path / "tune.json")
    best, rep = at.autotune(tr, beam, 30, cache_path=path, probe_turns=4, repeats=1)
    assert rep["source"] == "search" and tr.get_tuning() == best
    got = beam.copy()
    tr._track(got, num_turns=30)
    tr.device_status()
    for f in ("x", "px", "y", "py", "zeta", "delta", "state", "at_turn", "at_element"):
        assert torch.equal(getattr(got, f), getattr(ref, f)), f
    tr2 = line.build_tracker(device="cuda", arith="fast")
    best2, rep2 = at.autotune(tr2, beam, 30, cache_path=path)
    assert rep2["source"] == "cache" and best2 == best


@pytest.mark.gpu
def test_autotuned_batch_matches_default(tmp_path):
    """The tuner drives a BatchTracker through its lattice index; the tuned
    batch tracks every particle as the default one does."""
    import math

    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300 import workloads
    lines = [workloads.thick_ring(seed=s, n_arcs=1, n_cells=3, bend_angle=2 * math.pi / 1104)
             for s in range(3)]
    n = 2000
    lat = np.random.default_rng(4).integers(0, 3, size=n).astype(np.int32)
    beam = workloads.gaussian_beam(n, 7e12, seed=5, device="cuda", sigma_x=2e-3, sigma_px=2e-5)
    ref = beam.copy()
    xt.BatchTracker(lines, device="cuda", arith="fast").track(ref, lattice_index=lat, num_turns=12)
    bt = xt.BatchTracker(lines, device="cuda", arith="fast")
    best, rep = at.autotune(bt, beam, 12, cache_path=str(tmp_path / "t.json"), probe_turns=2,
                            repeats=1, lattice_index=lat,
                            space={"block_size": (32, 256), "chunk_bytes": (0, 12288)})
    assert rep["source"] == "search" and bt.get_tuning() == best
    assert len(rep["timings"]) >= 3
    got = beam.copy()
    bt.track(got, lattice_index=lat, num_turns=12)
    bt.device_status()
    for f in ("x", "px", "y", "py", "zeta", "delta", "state", "at_turn", "at_element"):
        assert torch.equal(getattr(got, f), getattr(ref, f)), f
