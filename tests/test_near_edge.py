"""The near-edge listing used by the parity tests (CPU, oracle only).

Integer fields (state, at_turn, at_element) must match the reference bit
for bit, except for particles that pass within 1e-9 m of an aperture edge:
a last-ulp difference in their coordinates may flip the aperture compare.
near_edge_mask lists them from the oracle's own run (oracle.
xto_set_edge_distance), and compare() exempts them only where the integer
fields actually differ."""
import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtg_testutil import compare, near_edge_mask


def _line():
    return xt.Line(elements=[xt.Drift(length=1.0),
                             xt.LimitRect(min_x=-0.01, max_x=0.01, min_y=-0.02, max_y=0.02),
                             xt.Drift(length=1.0),
                             xt.LimitEllipse(a=0.03, b=0.015)])


def _beam():
    # particle 0 ends 0.4 nm inside the rectangle's edge, particle 1 0.4 nm
    # outside, particle 2 is 5 um inside, particle 3 crosses the ellipse's
    # edge in y by 0.2 nm, particle 4 is far from every edge
    x = np.array([0.01 - 4e-10, 0.01 + 4e-10, 0.01 - 5e-6, 0.0, 0.001])
    y = np.array([0.0, 0.0, 0.0, 0.015 + 2e-10, 0.001])
    return xt.Particles(device="cpu", p0c=7e12, x=x, y=y)


def test_edge_distance_lists_the_particles_near_an_edge():
    line = _line()
    arrs = pyoracle.host_arrays(_beam().to_numpy())
    d = pyoracle.edge_distance(line._element_records(), arrs, line_length=line.get_length())
    assert d[0] == pytest.approx(4e-10, rel=1e-3)
    assert d[1] == pytest.approx(4e-10, rel=1e-3)
    assert d[2] == pytest.approx(5e-6, rel=1e-6)
    assert d[3] < 1e-9
    assert d[4] > 1e-3
    mask = near_edge_mask(line._element_records(), arrs, line_length=line.get_length())
    assert mask.tolist() == [True, True, False, True, False]


def test_compare_exempts_only_near_edge_particles_whose_integers_differ():
    line = _line()
    recs = line._element_records()
    arrs = pyoracle.host_arrays(_beam().to_numpy())
    ref = {k: v.copy() for k, v in arrs.items()}
    pyoracle.track(recs, ref, line_length=line.get_length())
    assert ref["state"].tolist() == [1, 0, 1, 0, 1]
    near = near_edge_mask(recs, arrs, line_length=line.get_length())
    # a planted survival flip of a near-edge particle: exempt, listed
    got = {k: v.copy() for k, v in ref.items()}
    got["state"][0] = 0
    got["x"][0] += 1.0
    compare(got, ref, 1e-14, near_edge=near)
    # the same flip on a particle far from every edge fails
    got = {k: v.copy() for k, v in ref.items()}
    got["state"][2] = 0
    with pytest.raises(AssertionError, match="farther than the near-edge tolerance"):
        compare(got, ref, 1e-14, near_edge=near)
    # without the listing, integer fields stay bit-exact for every particle
    got = {k: v.copy() for k, v in ref.items()}
    got["at_element"][0] += 1
    with pytest.raises(AssertionError, match="at_element differs"):
        compare(got, ref, 1e-14)
