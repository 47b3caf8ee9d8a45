"""GPU parity: the CUDA push against the CPU oracle, through the C-ABI,
on the same seeded inputs.

Tolerances (scale-relative: max|gpu - oracle| / max|oracle| per field):
  * exact arithmetic, 1 turn        <= 1e-14 (the bar of the specification);
    in practice only the last-ulp behaviour of sin/cos/atan2/asin/sinh/cosh
    separates the two, and most values are bit-identical;
  * exact arithmetic, many turns    <= 1e-9 for particles in the regular
    region (no loss in either run);
  * fast arithmetic, 1 turn         <= 1e-11 (merged kicks with fused
    multiply-adds round differently from the reference, as the reference's
    own FMA-contracted builds do);
  * fast arithmetic, 1000 turns     <= 1e-9 in the regular region.
state, at_turn and at_element are compared bit for bit.
"""
import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import workloads
from lattice_cases import element_zoo, sliced_line, small_beam
from xtg_testutil import compare, gpu_track, make_monitor

pytestmark = pytest.mark.gpu


def _setup(line, beam_kw):
    recs = line._element_records()
    p = xt.Particles(device="cpu", **beam_kw)
    arrs = pyoracle.host_arrays(p.to_numpy())
    return recs, arrs, line.get_length()


def _run_both(recs, arrs, L, arith="exact", **kw):
    ref = {k: v.copy() for k, v in arrs.items()}
    pyoracle.track(recs, ref, line_length=L, **kw)
    got, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, arith=arith, line_length=L, **kw)
    return got, ref


BEFORE_CAVITY = ("x", "px", "y", "py", "zeta", "s")


def test_toy_ring_one_turn_exact():
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(10000, p0c=450e9, seed=11))
    got, ref = _run_both(recs, arrs, L, num_turns=1)
    compare(got, ref, 1e-14)
    # the cavity is the last element: everything computed before its sin()
    # is bit-identical to the reference arithmetic
    for f in BEFORE_CAVITY:
        assert np.array_equal(got[f], ref[f]), f


def test_thick_ring_one_turn_exact():
    recs, arrs, L = _setup(workloads.thick_ring(), small_beam(512, seed=12))
    got, ref = _run_both(recs, arrs, L, num_turns=1)
    compare(got, ref, 1e-14)
    assert np.all(got["at_turn"] == 1)
    for f in BEFORE_CAVITY:
        assert np.array_equal(got[f], ref[f]), f


def test_thick_ring_one_turn_fast():
    recs, arrs, L = _setup(workloads.thick_ring(), small_beam(512, seed=13))
    got, ref = _run_both(recs, arrs, L, arith="fast", num_turns=1)
    compare(got, ref, 1e-11)


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_toy_ring_1000_turns(arith):
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(1000, p0c=450e9, seed=14))
    got, ref = _run_both(recs, arrs, L, arith=arith, num_turns=1000)
    regular = (ref["state"] > 0) & (got["state"] > 0)
    assert regular.sum() > 900
    compare(got, ref, 1e-9, mask=regular)


@pytest.mark.parametrize("arith", ["exact", "fast"])
@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 2, 1 << 3, 1 << 4])
def test_element_zoo(arith, flags):
    recs, arrs, L = _setup(element_zoo(), small_beam(256, seed=15, scale=0.3))
    got, ref = _run_both(recs, arrs, L, arith=arith, num_turns=2, track_flags=flags)
    compare(got, ref, 1e-14 if arith == "exact" else 1e-10)


@pytest.mark.parametrize("cfg", [{"use_exact_drifts": True}, {"cavity_preserve_angle": True},
                                 {"global_xy_limit": None}, {"global_xy_limit": 0.005}])
def test_config_switches(cfg):
    recs, arrs, L = _setup(element_zoo(), small_beam(256, seed=16, scale=0.3))
    got, ref = _run_both(recs, arrs, L, num_turns=2, **cfg)
    compare(got, ref, 1e-14)


@pytest.mark.parametrize("thin", [True, False])
@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_sliced_lines(thin, arith):
    recs, arrs, L = _setup(sliced_line(thin), small_beam(512, seed=17))
    got, ref = _run_both(recs, arrs, L, arith=arith, num_turns=5)
    compare(got, ref, 1e-14 if arith == "exact" else 1e-11)


@pytest.mark.parametrize("start,count,turns,end", [(0, 10, 1, 0), (5, 20, 1, 1), (3, 30, 2, 1),
                                                   (7, 0, 1, 0)])
def test_partial_ranges(start, count, turns, end):
    recs, arrs, L = _setup(element_zoo(), small_beam(128, seed=18, scale=0.3))
    got, ref = _run_both(recs, arrs, L, num_turns=turns, ele_start=start, num_ele_track=count,
                         flag_end_turn_actions=end)
    compare(got, ref, 1e-14)


def test_losses_bookkeeping_toy_ring():
    """Large amplitudes: many losses on the ellipse and the global aperture;
    state / at_turn / at_element must be bit-exact."""
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(4000, p0c=450e9, seed=19, scale=12.0))
    got, ref = _run_both(recs, arrs, L, num_turns=50)
    assert (ref["state"] <= 0).sum() > 200
    compare(got, ref, 1e-9, mask=(ref["state"] > 0))
    for f in ("state", "at_turn", "at_element"):
        assert np.array_equal(got[f], ref[f])


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_monitor_turn_by_turn(arith):
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(300, p0c=450e9, seed=20, scale=10.0))
    mon = make_monitor(0, 12, (10, 250))
    ref = {k: v.copy() for k, v in arrs.items()}
    mref = make_monitor(0, 12, (10, 250))
    pyoracle.track(recs, ref, line_length=L, num_turns=12, monitor=mref, flag_monitor=1)
    got, mgot = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, arith=arith,
                          line_length=L, num_turns=12, monitor=mon, flag_monitor=1)
    tol = 1e-14 if arith == "exact" else 1e-10
    for f, v in mref["data"].items():
        if f in ("at_turn", "at_element", "state", "particle_id"):
            assert np.array_equal(mgot[f], v), f
        else:
            scale = np.max(np.abs(v)) or 1.0
            assert np.max(np.abs(mgot[f] - v)) / scale <= tol, f


def test_monitor_repetitions_and_ebe():
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(50, p0c=450e9, seed=21))
    for kw in (dict(n_repetitions=3, repetition_period=4), dict(ebe_mode=1)):
        stop = 3 if "n_repetitions" in kw else len(recs) + 1
        flag = 1 if "n_repetitions" in kw else 2
        turns = 12 if "n_repetitions" in kw else 1
        mref = make_monitor(0, stop, (0, 50), **kw)
        mon = make_monitor(0, stop, (0, 50), **kw)
        ref = {k: v.copy() for k, v in arrs.items()}
        pyoracle.track(recs, ref, line_length=L, num_turns=turns, monitor=mref, flag_monitor=flag)
        got, mgot = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, line_length=L,
                              num_turns=turns, monitor=mon, flag_monitor=flag)
        for f, v in mref["data"].items():
            scale = np.max(np.abs(v)) or 1.0
            assert np.max(np.abs(mgot[f] - v)) / scale <= 1e-14, f


@pytest.mark.parametrize("compact_every,block", [(1, 0), (7, 128), (0, 64)])
def test_launch_shapes_do_not_change_results(compact_every, block):
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(3000, p0c=450e9, seed=22, scale=8.0))
    base, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, line_length=L, num_turns=20)
    got, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, line_length=L, num_turns=20,
                       compact_every=compact_every, block_size=block)
    for f in base:
        assert np.array_equal(got[f], base[f], equal_nan=True), f


def test_edge_cases():
    recs, arrs, L = _setup(workloads.toy_ring(), small_beam(64, p0c=450e9, seed=23))
    # already-lost and unallocated particles are left untouched
    arrs["state"][:10] = 0
    arrs["state"][10:20] = -999999999
    arrs["x"][20] = np.nan
    arrs["px"][21] = 1e30
    got, ref = _run_both(recs, arrs, L, num_turns=5)
    for f in ("state", "at_turn", "at_element"):
        assert np.array_equal(got[f], ref[f]), f
    for f in ("x", "px", "y", "py", "zeta", "delta"):
        assert np.array_equal(got[f][:20], arrs[f][:20], equal_nan=True)
    # zero turns and zero elements are no-ops
    got0, _ = gpu_track(recs, {k: v.copy() for k, v in arrs.items()}, line_length=L, num_turns=0)
    for f in arrs:
        assert np.array_equal(got0[f], arrs[f], equal_nan=True)


def test_api_line_track_matches_oracle():
    """The xtrack-style API (Line.track with the turn split of
    tracker.py:1270-1436) against one oracle call over the same turns."""
    line = workloads.toy_ring()
    beam_kw = small_beam(2000, p0c=450e9, seed=24)
    p = xt.Particles(device="cuda", **beam_kw)
    host = pyoracle.host_arrays(p.to_numpy())
    line.build_tracker(device="cuda")
    line.track(p, num_turns=7, turn_by_turn_monitor=True)
    pyoracle.track(line._element_records(), host, num_turns=7, line_length=line.get_length())
    got = p.to_numpy()
    compare(got, host, 1e-14)
    mon = line.record_last_track
    assert mon.x.shape == (2000, 7)
    assert np.array_equal(mon.at_turn[0], np.arange(7))
    # ele_start / ele_stop split: first partial turn, middle turns, last partial turn
    p2 = xt.Particles(device="cuda", **beam_kw)
    h2 = pyoracle.host_arrays(p2.to_numpy())
    line.track(p2, ele_start=100, ele_stop=50, num_turns=3)
    recs = line._element_records()
    n = len(recs)
    pyoracle.track(recs, h2, num_turns=1, ele_start=100, num_ele_track=n - 100,
                   line_length=line.get_length())
    pyoracle.track(recs, h2, num_turns=2, ele_start=0, num_ele_track=n,
                   line_length=line.get_length())
    pyoracle.track(recs, h2, num_turns=1, ele_start=0, num_ele_track=50, flag_end_turn_actions=0,
                   line_length=line.get_length())
    compare(p2.to_numpy(), h2, 1e-14)


def test_backtrack_returns_to_start():
    """tests/test_magnet.py:62-110 of the reference: tracking forward then
    backward through a line gives back the initial coordinates."""
    line = sliced_line(thin=False)
    line.config.XTRACK_GLOBAL_XY_LIMIT = None
    p = xt.Particles(device="cuda", **small_beam(256, seed=25))
    x0 = p.to_numpy()
    line.build_tracker(device="cuda")
    n = len(line.element_names)
    line.track(p, num_elements=n)
    line.track(p, num_elements=n, backtrack=True)
    x1 = p.to_numpy()
    for f in ("x", "px", "y", "py"):
        scale = np.max(np.abs(x0[f]))
        assert np.max(np.abs(x1[f] - x0[f])) / scale < 5e-12, f
