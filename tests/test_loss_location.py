"""Loss-location refinement: the short line's construction (CPU) and, on
the GPU, refined loss positions against the analytic crossing of a
straight track with the aperture edge (the reference's own check,
tests/test_loss_location_refinement.py) and against a fine oracle scan."""
import numpy as np
import pytest

import xtrack_gb300 as xt
from xtrack_gb300 import loss_location as ll


def _line(with_quad=False, thin_multipole=False):
    ap = dict(min_x=-0.01, max_x=0.01, min_y=-0.01, max_y=0.01)
    els = [xt.Marker(), xt.LimitRect(**ap), xt.Drift(length=2.0)]
    names = ["start", "ap0", "d0"]
    if with_quad:
        els += [xt.Quadrupole(length=3.0, k1=0.02, num_multipole_kicks=4,
                              model="drift-kick-drift-expanded", integrator="uniform")]
        names += ["q"]
    if thin_multipole:
        els += [xt.Multipole(knl=[0.0, 1e-3])]
        names += ["mp"]
    els += [xt.Drift(length=5.0), xt.Marker(), xt.LimitRect(**ap), xt.Drift(length=1.0)]
    names += ["d1", "m1", "ap1", "dend"]
    return xt.Line(elements=els, element_names=names)


def test_interp_locations_and_line_structure():
    line = _line(with_quad=True)
    s = line.get_s_elements()
    s0, s1, sv = ll.interp_aperture_locations(s, 1, 6, 0.5)
    assert (s0, s1) == (0.0, 10.0) and len(sv) == 19
    assert ll.find_adjacent_thick(line, 6, "upstream") == 4
    assert ll.find_adjacent_thick(line, 1, "downstream") == 2
    interp = ll.build_interp_line(line, 1, 5, s0, sv, line["ap1"])
    es = interp.elements
    assert isinstance(es[0], xt.LimitRect) and isinstance(es[-1], xt.LimitRect)
    # apertures at every s_vect position, total length preserved
    assert abs(interp.get_length() - 10.0) < 1e-12
    s_int = interp.get_s_elements()
    ap_s = [si for si, e in zip(s_int, es) if isinstance(e, xt.LimitRect)][1:-1]
    assert np.allclose(ap_s, sv, atol=1e-12)
    # the quadrupole is cut into an entry edge, thick slices and an exit edge
    kinds = [type(e).__name__ for e in es]
    assert "ThinSliceQuadrupoleEntry" in kinds and "ThinSliceQuadrupoleExit" in kinds
    w = sum(e.weight for e in es if type(e).__name__ == "ThickSliceQuadrupole")
    assert abs(w - 1.0) < 1e-12


def test_identical_apertures():
    a = xt.LimitRect(min_x=-1, max_x=1)
    assert ll.apertures_are_identical(a, xt.LimitRect(min_x=-1, max_x=1))
    assert not ll.apertures_are_identical(a, xt.LimitRect(min_x=-1, max_x=2))
    assert not ll.apertures_are_identical(a, xt.LimitEllipse(a=1, b=1))


@pytest.mark.gpu
def test_refined_location_matches_analytic_crossing():
    line = _line()
    line.build_tracker(device="cuda")
    n = 200
    px = np.linspace(1.6e-3, 4.5e-3, n)       # crossing x = 1 cm between s = 2.2 and 6.25 m
    p = xt.Particles(p0c=7e12, x=np.zeros(n), px=px, device="cuda")
    line.track(p)
    state = p.state.cpu().numpy()
    at_el = p.at_element.cpu().numpy()
    assert np.all(state == 0) and np.all(at_el == line.element_names.index("ap1"))
    ds = 0.05
    ref = ll.LossLocationRefinement(line, ds=ds)
    ref.refine_loss_location(p)
    s = p.s.cpu().numpy()
    rpp = 1.0                                  # delta = 0
    s_cross = 0.01 / (px * rpp)
    # the refined position is the first inserted aperture after the crossing
    assert np.all(s >= s_cross - 1e-9)
    assert np.all(s - s_cross <= ds + 1e-9)
    # coordinates are those at the refined position
    x = p.x.cpu().numpy()
    assert np.allclose(x, px * s, rtol=1e-12, atol=1e-15)
    assert np.all(p.state.cpu().numpy() == 0)


@pytest.mark.gpu
def test_refined_location_through_a_quadrupole_matches_oracle_scan():
    """Through a thick quadrupole: the refined s and coordinates equal
    those of the oracle tracking the original particles from the start of
    the line through the same cut line (apertures every ds from the start),
    i.e. where the particle first fails an aperture."""
    import pyoracle
    line = _line(with_quad=True)
    line.build_tracker(device="cuda")
    n = 64
    rng = np.random.default_rng(4)
    kw = dict(x=rng.uniform(-4e-3, 4e-3, n),
              px=rng.uniform(1.5e-3, 3e-3, n) * rng.choice([-1.0, 1.0], n),
              y=rng.uniform(-1e-3, 1e-3, n))
    p = xt.Particles(p0c=7e12, device="cuda", **kw)
    line.track(p)
    i_ap1 = line.element_names.index("ap1")
    lost = (p.state.cpu().numpy() == 0) & (p.at_element.cpu().numpy() == i_ap1)
    assert lost.sum() > 10
    ds = 0.1
    ref = ll.LossLocationRefinement(line, ds=ds, save_refine_lines=True)
    ref.refine_loss_location(p)
    interp = ref.refine_lines[i_ap1]
    # oracle: start + ap0 + the cut line, from the initial coordinates
    scan = xt.Line(elements=[line["start"], line["ap0"]] + interp.elements,
                   element_names=["start", "ap0"] + interp.element_names)
    p0 = xt.Particles(p0c=7e12, device="cpu", **{k: v[lost] for k, v in kw.items()})
    arrs = pyoracle.host_arrays(p0.to_numpy())
    pyoracle.track(scan._element_records(), arrs, num_turns=1, flag_end_turn_actions=0,
                   flag_reset_s=0, line_length=scan.get_length())
    assert np.all(arrs["state"] == 0)
    got_s = p.s.cpu().numpy()[lost]
    assert np.allclose(got_s, arrs["s"], rtol=0, atol=1e-9)
    for f in ("x", "px", "y", "py"):
        assert np.allclose(getattr(p, f).cpu().numpy()[lost], arrs[f], rtol=1e-9, atol=1e-15), f


def test_thin_multipole_cannot_be_backtracked():
    line = _line(thin_multipole=True)
    ref = ll.LossLocationRefinement.__new__(ll.LossLocationRefinement)
    ref.line = line
    ref.allowed_backtrack_types = ()
    # the elements between the thick neighbours of ap0 and ap1: d0, mp, d1, m1
    with pytest.raises(TypeError):
        ref._check_backtrack(2, 6)
    ref.allowed_backtrack_types = (xt.Multipole,)
    ref._check_backtrack(2, 6)


def _polygon_line():
    th = np.linspace(0, 2 * np.pi, 13)[:-1]
    poly = xt.LimitPolygon(x_vertices=0.012 * np.cos(th), y_vertices=0.009 * np.sin(th))
    return xt.Line(elements=[xt.Drift(length=1.0), poly, xt.Drift(length=0.5),
                             xt.LimitRect(min_x=-0.02, max_x=0.011, min_y=-0.01, max_y=0.01)],
                   element_names=["d0", "poly", "d1", "rect"])


def test_polygon_area_and_impacts():
    sq = xt.LimitPolygon(x_vertices=[1.0, -1.0, -1.0, 1.0], y_vertices=[1.0, 1.0, -1.0, -1.0])
    assert sq.area == 4.0 and sq.get_area(signed=True) == 4.0
    x, y, z, nx, ny, i = sq.impact_point_and_normal([0.0, 0.0], [0.0, 0.0], [0.0, 0.0],
                                                    [3.0, 0.0], [0.0, -5.0], [0.0, 0.0])
    assert np.allclose(x, [1.0, 0.0]) and np.allclose(y, [0.0, -1.0])
    # the reference's orientation: (-dy, dx) of a counter-clockwise polygon
    assert np.allclose(nx, [-1.0, 0.0]) and np.allclose(ny, [0.0, 1.0])
    with pytest.raises(ValueError):
        xt.LimitPolygon(x_vertices=[0, 1], y_vertices=[0, 1])


@pytest.mark.gpu
def test_polygon_aperture_gpu_matches_oracle():
    import pyoracle
    line = _polygon_line()
    rng = np.random.default_rng(8)
    n = 4000
    p = xt.Particles(device="cpu", p0c=7e12, x=rng.uniform(-0.02, 0.02, n),
                     y=rng.uniform(-0.015, 0.015, n), px=rng.normal(0, 1e-4, n))
    arrs = pyoracle.host_arrays(p.to_numpy())
    ref = {k: v.copy() for k, v in arrs.items()}
    pyoracle.track(line._element_records(), ref, line_length=line.get_length())
    from xtg_testutil import gpu_track
    got, _ = gpu_track(line._element_records(), {k: v.copy() for k, v in arrs.items()},
                       line_length=line.get_length())
    for f in ("state", "at_element", "at_turn"):
        assert np.array_equal(got[f], ref[f]), f
    assert 0.2 < np.mean(ref["state"] > 0) < 0.9


@pytest.mark.gpu
def test_polygon_mode_refinement_between_different_apertures():
    """A rectangle then an ellipse 10 m later: the refined s of particles
    moving along x with slope px lies where the linearly interpolated
    aperture radius at angle 0 equals px * s (within ds and dr)."""
    a0 = xt.LimitRect(min_x=-0.01, max_x=0.01, min_y=-0.01, max_y=0.01)
    a1 = xt.LimitEllipse(a=0.03, b=0.02)
    line = xt.Line(elements=[xt.Marker(), a0, xt.Drift(length=10.0), a1, xt.Drift(length=1.0)],
                   element_names=["m", "ap0", "d", "ap1", "dend"])
    line.build_tracker(device="cuda")
    n = 60
    px = np.linspace(3.05e-3, 4.5e-3, n)      # beyond the ellipse at s = 10, inside the rect at 0
    p = xt.Particles(p0c=7e12, x=np.zeros(n), px=px, device="cuda")
    line.track(p)
    assert np.all(p.state.cpu().numpy() == 0)
    assert np.all(p.at_element.cpu().numpy() == 3)
    ds, dr = 0.05, 1e-4
    ref = ll.LossLocationRefinement(line, ds=ds, n_theta=72, r_max=0.05, dr=dr)
    ref.refine_loss_location(p)
    s = p.s.cpu().numpy()
    # radius at angle 0 interpolates from 1 cm (s = 0) to 3 cm (s = 10)
    s_cross = 0.01 / (px - 0.002)
    # the crossing lies between two inserted apertures; the polygon's
    # vertex radius is known to dr
    assert np.all(np.abs(s - s_cross) <= 2 * ds + dr / (px - 0.002))
    assert np.allclose(p.x.cpu().numpy(), px * s, rtol=1e-12)
