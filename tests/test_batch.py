"""BatchTracker: error seeds of one ring in one persistent launch against
each seed tracked on its own (same kernels: bit-identical) and against the
oracle."""
import math

import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import workloads
from xtg_testutil import compare

pytestmark = pytest.mark.gpu

FIELDS = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s",
          "state", "at_turn", "at_element")


def _seeds(n):
    return [workloads.thick_ring(seed=s, n_arcs=1, n_cells=3, bend_angle=2 * math.pi / 1104)
            for s in range(1, n + 1)]


def _same(a, b):
    """Bitwise equality (NaN-aware) of two tensors."""
    import torch
    if a.dtype == torch.float64:
        return torch.equal(a.view(torch.int64), b.view(torch.int64))
    return torch.equal(a, b)


def _beam(n, seed, scale):
    rng = np.random.default_rng(seed)
    return dict(p0c=7e12, x=rng.normal(0, 1e-3 * scale, n), px=rng.normal(0, 1e-5 * scale, n),
                y=rng.normal(0, 1e-3 * scale, n), py=rng.normal(0, 1e-5 * scale, n),
                zeta=rng.normal(0, 0.05, n), delta=rng.normal(0, 1e-4, n))


@pytest.mark.parametrize("arith", ["exact", "fast"])
@pytest.mark.parametrize("tuning", [{}, {"compact_every": 3, "chunk_bytes": 4096, "use_graph": 1},
                                    {"chunk_bytes": 0, "block_size": 64},
                                    {"compact_every": 2, "chunk_bytes": 8192, "block_size": 32}])
def test_batch_equals_per_seed_trackers(arith, tuning):
    import torch
    lines = _seeds(4)
    n = 3000
    rng = np.random.default_rng(9)
    lat = rng.integers(0, 4, size=n).astype(np.int32)
    beam = xt.Particles(device="cuda", **_beam(n, 17, 6.0))
    bt = xt.BatchTracker(lines, device="cuda", arith=arith)
    if tuning:
        bt.set_tuning(**tuning)
    got = beam.copy()
    bt.track(got, lattice_index=lat, num_turns=10)
    bt.device_status()
    assert int((got.state <= 0).sum()) > 50        # losses in the window
    for s, line in enumerate(lines):
        sel = torch.from_numpy(np.nonzero(lat == s)[0]).cuda()
        one = xt.Particles(device="cuda", **{k: (v[lat == s] if np.ndim(v) else v)
                                             for k, v in _beam(n, 17, 6.0).items()})
        tr = line.build_tracker(device="cuda", arith=arith)
        tr._track(one, num_turns=10)
        for f in FIELDS:
            a = getattr(got, f).index_select(0, sel)
            b = getattr(one, f)
            assert _same(a, b), (s, f)


def test_batch_matches_oracle_with_partial_turns():
    lines = _seeds(3)
    n = 900
    lat = (np.arange(n) % 3).astype(np.int32)
    kw = _beam(n, 5, 6.0)
    beam = xt.Particles(device="cuda", **kw)
    bt = xt.BatchTracker(lines, device="cuda", arith="exact")
    ele_start = 11
    bt.track(beam, lattice_index=lat, ele_start=ele_start, num_turns=4, ele_stop=30)
    got = pyoracle.host_arrays(beam.to_numpy())
    L = lines[0].get_length()
    for s in range(3):
        sel = lat == s
        p = xt.Particles(device="cpu", **{k: (v[sel] if np.ndim(v) else v) for k, v in kw.items()})
        ref = pyoracle.host_arrays(p.to_numpy())
        recs = lines[s]._element_records()
        nel = len(recs)
        # the same three calls as Tracker._track (tracker.py:1270-1333): with
        # ele_stop > ele_start, num_turns=4 is a first partial turn, 2 middle
        # turns and a last partial turn
        pyoracle.track(recs, ref, line_length=L, num_turns=1, ele_start=ele_start,
                       num_ele_track=nel - ele_start)
        pyoracle.track(recs, ref, line_length=L, num_turns=2, ele_start=0, num_ele_track=nel)
        pyoracle.track(recs, ref, line_length=L, num_turns=1, ele_start=0, num_ele_track=30,
                       flag_end_turn_actions=0)
        ref["particle_id"] = np.nonzero(sel)[0]      # ids of the batched beam
        compare({k: v[sel] for k, v in got.items()}, ref, 5e-14)


def test_batch_rejects_bad_inputs():
    lines = _seeds(2)
    bt = xt.BatchTracker(lines, device="cuda")
    beam = xt.Particles(device="cuda", **_beam(10, 1, 1.0))
    with pytest.raises(ValueError):
        bt.track(beam, lattice_index=np.zeros(9, dtype=np.int32))
    with pytest.raises(ValueError):
        bt.track(beam, lattice_index=np.full(10, 2, dtype=np.int32))
    short = workloads.thick_ring(seed=1, n_arcs=1, n_cells=2, bend_angle=2 * math.pi / 1104)
    with pytest.raises(ValueError):
        xt.BatchTracker([lines[0], short], device="cuda")
