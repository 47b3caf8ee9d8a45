"""Pins the C restatement (oracle/xtg_oracle.c) to the reference's own
element C code compiled in this tree (oracle/_ref): every field must be bit
for bit identical. Runs where the reference sources were available to build
oracle/_ref; elsewhere the committed golden vectors (test_golden.py) pin the
oracle instead."""
import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300 import workloads
from lattice_cases import (element_zoo, fringe_zoo, shifted_apertures, shifted_thin_elements,
                           sliced_line, small_beam)

pyoracle.ensure_built(with_ref=True)
pytestmark = pytest.mark.skipif(not pyoracle.ref_available(),
                                reason="reference-compiled oracle not built here")

FIELDS = pyoracle.DOUBLE_FIELDS + pyoracle.INT_FIELDS


def _both(line, beam_kw, **kw):
    recs = line._element_records()
    p = xt.Particles(device="cpu", **beam_kw)
    a = pyoracle.host_arrays(p.to_numpy())
    b = pyoracle.host_arrays(p.to_numpy())
    L = line.get_length()
    pyoracle.track(recs, a, line_length=L, which="oracle", **kw)
    pyoracle.track(recs, b, line_length=L, which="ref", **kw)
    return a, b


def _assert_identical(a, b):
    for f in FIELDS:
        assert np.array_equal(a[f], b[f], equal_nan=True), f"{f} differs"


def test_toy_ring_20_turns():
    line = workloads.toy_ring()
    a, b = _both(line, small_beam(300, p0c=450e9, seed=1), num_turns=20)
    _assert_identical(a, b)
    assert (a["state"] > 0).sum() > 250


def test_thick_ring_one_turn():
    line = workloads.thick_ring()
    a, b = _both(line, small_beam(40, seed=2), num_turns=1)
    _assert_identical(a, b)
    assert np.all(a["at_turn"] == 1)


@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 2, 1 << 3, 1 << 4])
@pytest.mark.parametrize("cfg", [{}, {"use_exact_drifts": True}, {"cavity_preserve_angle": True},
                                 {"global_xy_limit": None}])
def test_element_zoo(flags, cfg):
    line = element_zoo()
    a, b = _both(line, small_beam(64, seed=3, scale=0.3), num_turns=2, track_flags=flags, **cfg)
    _assert_identical(a, b)


@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 3])
def test_fringe_zoo(flags):
    """Full and dipole-only edge models (and the kill of backtracked
    particles at such edges) bit for bit against the reference's code."""
    line = fringe_zoo()
    a, b = _both(line, small_beam(64, seed=9, scale=0.5), num_turns=2, track_flags=flags)
    _assert_identical(a, b)
    if flags & 1:
        assert np.all(a["state"] == -32)
    else:
        assert (a["state"] > 0).sum() > 50


@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 2])
@pytest.mark.parametrize("case", ["zoo", "fringe", "toy"])
def test_freeze_longitudinal(case, flags):
    """freeze_longitudinal: the restatement with its freeze flag equals the
    reference's code compiled with the FREEZE_VAR set of freeze_longitudinal
    bit for bit (cavities, curved and exact drifts, edges, kills), and
    zeta, ptau, delta, rpp and rvv keep their initial values."""
    line, beam = {"zoo": (element_zoo, small_beam(64, seed=3, scale=0.3)),
                  "fringe": (fringe_zoo, small_beam(64, seed=9, scale=0.5)),
                  "toy": (workloads.toy_ring, small_beam(300, p0c=450e9, seed=1))}[case]
    line = line()
    a, b = _both(line, beam, num_turns=3, track_flags=flags, freeze_longitudinal=True)
    _assert_identical(a, b)
    p0 = pyoracle.host_arrays(xt.Particles(device="cpu", **beam).to_numpy())
    for f in ("zeta", "ptau", "delta", "rpp", "rvv"):
        assert np.array_equal(a[f], p0[f]), f
    moved = np.any(a["x"] != p0["x"])
    assert moved
    # without the freeze the same call changes the longitudinal coordinates
    c, _ = _both(line, beam, num_turns=3, track_flags=flags)
    assert np.any(c["zeta"] != p0["zeta"])


@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 4])
def test_shifted_apertures(flags):
    """Apertures with shift_x / shift_y through the reference's own
    transformation wrapper: survivors are shifted back, particles lost
    there keep the shifted frame, and with local apertures ignored the
    shifts still apply; bit for bit."""
    a, b = _both(shifted_apertures(), small_beam(400, seed=13, scale=8.0), num_turns=2,
                 track_flags=flags)
    _assert_identical(a, b)
    if flags == 0:
        assert 50 < np.sum(a["state"] == 0) < 350


@pytest.mark.parametrize("flags", [0, 1 << 0, 1 << 4])
def test_shifted_thin_elements(flags):
    """Thin multipoles (one of zero strength, one with a curvature kick) and
    dipole edges (linear, full, suppressed) with transverse shifts and
    tilts, through the reference's own transformation wrapper for
    Multipole and DipoleEdge; forward, backtracking (the full edge kills)
    and with local apertures ignored; bit for bit."""
    a, b = _both(shifted_thin_elements(), small_beam(400, seed=17, scale=6.0), num_turns=3,
                 track_flags=flags)
    _assert_identical(a, b)
    if flags == 0:
        assert 0 < np.sum(a["state"] <= 0) < 400
    plain = shifted_thin_elements()
    for e in plain.elements:
        for f in ("shift_x", "shift_y", "rot_s_rad", "rot_s_rad_no_frame"):
            if hasattr(e, f):
                setattr(e, f, 0.0)
    c, _ = _both(plain, small_beam(400, seed=17, scale=6.0), num_turns=3, track_flags=flags)
    assert not np.array_equal(a["x"], c["x"])   # the transforms act


@pytest.mark.parametrize("thin", [True, False])
@pytest.mark.parametrize("flags", [0, 1])
def test_sliced_lines(thin, flags):
    line = sliced_line(thin)
    a, b = _both(line, small_beam(64, seed=4), num_turns=3, track_flags=flags)
    _assert_identical(a, b)


@pytest.mark.parametrize("start,count,turns,end", [(0, 10, 1, 0), (5, 20, 1, 1), (3, 30, 2, 1)])
def test_partial_element_ranges(start, count, turns, end):
    line = element_zoo()
    a, b = _both(line, small_beam(32, seed=5, scale=0.3), num_turns=turns, ele_start=start,
                 num_ele_track=count, flag_end_turn_actions=end)
    _assert_identical(a, b)


def test_openmp_structure_matches_per_particle():
    """The reference's CPU OpenMP driver (chunks, element-outer loop, swap
    compaction, reorganize) gives per-particle results equal to the
    one-particle-at-a-time driver; only the order of the slots changes."""
    line = workloads.toy_ring()
    p = xt.Particles(device="cpu", **small_beam(500, p0c=450e9, seed=6, scale=8.0))
    a = pyoracle.host_arrays(p.to_numpy())
    b = pyoracle.host_arrays(p.to_numpy())
    recs = line._element_records()
    L = line.get_length()
    pyoracle.track(recs, a, num_turns=30, line_length=L, mode=pyoracle.MODE_PER_PARTICLE)
    pyoracle.track(recs, b, num_turns=30, line_length=L, mode=pyoracle.MODE_OPENMP, num_threads=4)
    assert (a["state"] <= 0).sum() > 10, "want some losses to exercise the swaps"
    order = np.argsort(b["particle_id"])
    for f in FIELDS:
        assert np.array_equal(a[f], b[f][order], equal_nan=True), f
    # active particles first after the final reorganize
    st = b["state"]
    n_act = (st > 0).sum()
    assert np.all(st[:n_act] > 0) and np.all(st[n_act:] <= 0)
