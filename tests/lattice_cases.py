"""Small lattices that exercise every element class, model, integrator,
slice kind and edge configuration of the push (shared by the oracle-pin
tests and the GPU parity tests)."""
import math

import numpy as np

import xtrack_gb300 as xt


def _errs(rng, n, scale):
    return list(rng.normal(0, scale, n + 1))


def element_zoo(seed=3):
    """One of every in-scope configuration, strengths small enough that a
    millimetre beam survives one pass."""
    rng = np.random.default_rng(seed)
    els = []
    names = []

    def add(name, e):
        names.append(name)
        els.append(e)

    add("m0", xt.Marker())
    add("d_adapt", xt.Drift(length=0.7))
    add("d_exact", xt.Drift(length=0.9, model="exact"))
    add("mult_thin", xt.Multipole(knl=[1e-5, 2e-3, 0.05, 0.3], ksl=[-2e-6, 1e-4, 0.01],
                                  knl_rel=_errs(rng, 6, 1e-3), ksl_rel=_errs(rng, 6, 1e-3),
                                  main_order=1))
    add("mult_hxl", xt.Multipole(knl=[1e-3], hxl=1e-3, length=0.4))
    add("mult_thick", xt.Multipole(knl=[0, 1e-3, 0.02], isthick=True, length=0.5,
                                   num_multipole_kicks=3))
    angle = 2 * math.pi / 1104
    for model in ("adaptive", "drift-kick-drift-expanded", "drift-kick-drift-exact",
                  "rot-kick-rot", "mat-kick-mat", "bend-kick-bend", "rot-kick-rot-low-order",
                  "rot-kick-rot-high-order"):
        for integ in ("adaptive", "uniform", "teapot", "yoshida4"):
            add(f"b.{model}.{integ}", xt.Bend(length=2.0, angle=angle, k1=1e-3,
                                               knl_rel=_errs(rng, 10, 1e-4),
                                               ksl_rel=_errs(rng, 10, 1e-4),
                                               model=model, integrator=integ,
                                               num_multipole_kicks=(0 if integ == "adaptive" else 5),
                                               edge_entry_angle=0.01, edge_exit_angle=-0.005,
                                               edge_entry_hgap=0.02, edge_entry_fint=0.4))
    add("b_k0", xt.Bend(length=1.5, angle=1e-3, k0=1.2e-3, num_multipole_kicks=2))
    add("b_noedge", xt.Bend(length=1.0, angle=2e-3, edge_entry_active=False,
                            edge_exit_model="suppressed"))
    for model in ("adaptive", "drift-kick-drift-expanded", "drift-kick-drift-exact",
                  "mat-kick-mat"):
        for integ in ("adaptive", "uniform", "teapot", "yoshida4"):
            add(f"q.{model}.{integ}", xt.Quadrupole(length=1.1, k1=0.01, k1s=-2e-3,
                                                    knl_rel=_errs(rng, 10, 1e-4),
                                                    ksl_rel=_errs(rng, 10, 1e-4),
                                                    model=model, integrator=integ,
                                                    num_multipole_kicks=(0 if integ == "adaptive" else 4)))
    add("q_skew", xt.Quadrupole(length=0.8, k1s=0.004, main_is_skew=True,
                                knl_rel=[0, 0, 1e-3], ksl_rel=[0, 1e-3]))
    add("s", xt.Sextupole(length=0.37, k2=0.1, k2s=0.01, knl_rel=_errs(rng, 8, 1e-4),
                          num_multipole_kicks=3))
    add("o", xt.Octupole(length=0.3, k3=2.0, k3s=0.5, num_multipole_kicks=2,
                         integrator="teapot"))
    add("cav", xt.Cavity(voltage=3e6, frequency=200e6, lag=175.0))
    add("cav_h", xt.Cavity(voltage=1e6, harmonic=20, lag=10.0, phase=0.1))
    add("cav_thick", xt.Cavity(voltage=2e6, frequency=400e6, lag=170.0, length=0.5,
                               num_kicks=3))
    add("cav_abs", xt.Cavity(voltage=1e6, frequency=100e6, lag=180.0, absolute_time=1))
    add("de_in", xt.DipoleEdge(k=2e-3, e1=0.01, hgap=0.03, fint=0.5))
    add("de_out", xt.DipoleEdge(k=2e-3, e1=-0.004, e1_fd=1e-3, hgap=0.03, fint=0.4,
                                side="exit"))
    add("de_zero", xt.DipoleEdge(k=1e-3))
    add("de_off", xt.DipoleEdge(k=5e-3, e1=0.02, model="suppressed"))
    add("ell", xt.LimitEllipse(a=0.03, b=0.02))
    add("rect", xt.LimitRect(min_x=-0.03, max_x=0.028, min_y=-0.02, max_y=0.021))
    # shifted apertures (transformations of the reference with only shift_x,
    # shift_y nonzero); particles lost there keep the shifted frame
    add("rect_shift", xt.LimitRect(min_x=-0.02, max_x=0.02, min_y=-0.015, max_y=0.015,
                                   shift_x=4e-3, shift_y=-1e-3))
    add("ell_shift", xt.LimitEllipse(a=0.025, b=0.018, shift_y=2e-3))
    add("rect_ell", xt.LimitRectEllipse(max_x=0.022, max_y=0.017, a=0.026, b=0.02))
    return xt.Line(elements=els, element_names=names)


def fringe_zoo(seed=5):
    """Magnets with the nonlinear edge models: bends with the full and the
    dipole-only fringe (face angles, fringe integrals, gaps, normal and skew
    multipoles), and quadrupoles, sextupoles and octupoles with active
    edges (their edges use the full model)."""
    rng = np.random.default_rng(seed)
    els, names = [], []

    def add(name, e):
        names.append(name)
        els.append(e)

    angle = 2 * math.pi / 1104
    add("d0", xt.Drift(length=0.5))
    for k, (em, e1, e2, fint, hgap) in enumerate([
            ("full", 0.01, -0.005, 0.4, 0.02), ("full", 0.0, 0.0, 0.5, 0.03),
            ("dipole-only", 0.008, 0.004, 0.6, 0.025), ("full", -0.012, 0.02, 0.0, 0.0),
            ("dipole-only", 0.0, 0.0, 0.0, 0.0)]):
        add(f"b{k}", xt.Bend(length=2.0, angle=angle * (1 + k), k1=1e-3 * (-1) ** k,
                             knl=[0, 2e-4, 1e-3, 1e-2], ksl=[1e-6, 1e-4, 5e-4],
                             knl_rel=_errs(rng, 8, 1e-4), ksl_rel=_errs(rng, 8, 1e-4),
                             model="drift-kick-drift-expanded", integrator="uniform",
                             num_multipole_kicks=3, edge_entry_model=em, edge_exit_model=em,
                             edge_entry_angle=e1, edge_exit_angle=e2, edge_entry_fint=fint,
                             edge_exit_fint=fint * 0.8, edge_entry_hgap=hgap,
                             edge_exit_hgap=hgap * 1.1))
        add(f"db{k}", xt.Drift(length=0.3))
    add("b_mixed", xt.Bend(length=1.5, angle=angle, edge_entry_model="full",
                           edge_exit_model="linear", edge_entry_angle=0.005, edge_exit_angle=0.003,
                           edge_entry_fint=0.5, edge_entry_hgap=0.02))
    add("q_edges", xt.Quadrupole(length=1.1, k1=0.01, k1s=-2e-3, edge_entry_active=True,
                                 edge_exit_active=True, knl=[0, 0, 1e-3, 5e-3],
                                 ksl=[0, 0, 2e-4], num_multipole_kicks=4,
                                 model="drift-kick-drift-expanded", integrator="uniform"))
    add("q_entry", xt.Quadrupole(length=0.8, k1=-0.008, edge_entry_active=True,
                                 num_multipole_kicks=2))
    add("s_edges", xt.Sextupole(length=0.37, k2=0.1, k2s=0.02, edge_entry_active=True,
                                edge_exit_active=True, num_multipole_kicks=3))
    add("o_edges", xt.Octupole(length=0.3, k3=2.0, k3s=0.5, edge_exit_active=True,
                               num_multipole_kicks=2, integrator="teapot"))
    # DipoleEdge full model: entry, a face angle below 1e-9 (no rotation), exit
    add("de_full_in", xt.DipoleEdge(k=3e-3, e1=0.015, hgap=0.03, fint=0.5, model="full"))
    add("de_full_flat", xt.DipoleEdge(k=3e-3, e1=5e-10, hgap=0.03, fint=0.5, model="full"))
    add("de_full_out", xt.DipoleEdge(k=3e-3, e1=0.015, hgap=0.03, fint=0.5, model="full",
                                     side="exit"))
    add("d_end", xt.Drift(length=0.4))
    return xt.Line(elements=els, element_names=names)


def sliced_line(thin=True):
    """A short ring of thick magnets sliced thin (Teapot) or thick (Uniform)."""
    angle = 0.01
    els = [xt.Drift(length=1.0),
           xt.Bend(length=3.0, angle=angle, k1=2e-3, knl_rel=[0, 1e-4, 1e-3], ksl_rel=[0, 0, 1e-4],
                   edge_entry_angle=0.002, edge_exit_angle=0.001),
           xt.Drift(length=0.5),
           xt.Quadrupole(length=1.0, k1=0.02, knl_rel=[1e-4, 0, 0, 1e-3]),
           xt.Drift(length=0.5),
           xt.Sextupole(length=0.4, k2=0.2),
           xt.Octupole(length=0.3, k3=1.0),
           xt.Multipole(knl=[0, 5e-3, 0.02], isthick=True, length=0.6),
           xt.Cavity(voltage=1e6, frequency=400e6, lag=180.0, length=0.4),
           xt.Drift(length=2.0)]
    names = ["d0", "mb", "d1", "mq", "d2", "ms", "mo", "mm", "cav", "d3"]
    line = xt.Line(elements=els, element_names=names)
    if thin:
        line.slice_thick_elements([xt.Strategy(slicing=xt.Teapot(4)),
                                   xt.Strategy(slicing=xt.Uniform(3), element_type=xt.Bend),
                                   xt.Strategy(slicing=xt.Teapot(2), name="d3")])
    else:
        line.slice_thick_elements([xt.Strategy(slicing=xt.Uniform(3, mode="thick")),
                                   xt.Strategy(slicing=xt.Teapot(2, mode="thick"), element_type=xt.Bend)])
    return line


def small_beam(n, p0c=7e12, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    return dict(p0c=p0c, x=rng.normal(0, 1e-3 * scale, n), px=rng.normal(0, 1e-5 * scale, n),
                y=rng.normal(0, 1e-3 * scale, n), py=rng.normal(0, 1e-5 * scale, n),
                zeta=rng.normal(0, 0.05 * scale, n), delta=rng.normal(0, 1e-4 * scale, n))


def shifted_apertures():
    """Drifts and transversely shifted apertures that a wide beam hits."""
    els = [xt.Drift(length=0.5),
           xt.LimitRect(min_x=-0.01, max_x=0.012, min_y=-0.008, max_y=0.008, shift_x=3e-3,
                        shift_y=-1.5e-3),
           xt.Drift(length=0.7),
           xt.LimitEllipse(a=0.015, b=0.01, shift_x=-2e-3, shift_y=1e-3),
           xt.Drift(length=0.3),
           xt.LimitRect(min_x=-0.02, max_x=0.02, min_y=-0.02, max_y=0.02, shift_y=5e-3),
           xt.Drift(length=0.2),
           xt.LimitRectEllipse(max_x=0.016, max_y=0.013, a=0.019, b=0.016, shift_x=1e-3),
           xt.Drift(length=0.25),
           # tilted apertures: rot_s_rad, rot_s_rad_no_frame, with and without shifts
           xt.LimitRect(min_x=-0.012, max_x=0.012, min_y=-0.006, max_y=0.006, rot_s_rad=0.3),
           xt.Drift(length=0.1),
           xt.LimitEllipse(a=0.016, b=0.008, rot_s_rad_no_frame=-0.2, rot_s_rad=0.05,
                           shift_x=5e-4)]
    return xt.Line(elements=els)


def shifted_thin_elements():
    """Thin multipoles and dipole edges with transverse shifts and tilts
    (skew and shifted kicks as MAD-X thin lattices give them), among drifts
    and an aperture that a wide beam hits."""
    els = [xt.Drift(length=0.4),
           xt.Multipole(knl=[0.0, 0.08, 0.5], ksl=[0.0, 0.01], shift_x=1e-3, shift_y=-5e-4),
           xt.Drift(length=0.3),
           xt.Multipole(knl=[0.0, -0.06], rot_s_rad=0.4),                      # tilted quad
           xt.Drift(length=0.3),
           xt.Multipole(knl=[2e-3], hxl=2e-3, length=0.5, rot_s_rad=-0.1, shift_x=-2e-4),
           xt.Drift(length=0.2),
           xt.Multipole(knl=[0.0, 0.0, 0.0], shift_x=7e-4, rot_s_rad_no_frame=0.2),  # no strength
           xt.DipoleEdge(k=0.02, e1=0.1, hgap=0.03, fint=0.5, shift_x=5e-4, shift_y=3e-4),
           xt.Drift(length=0.3),
           xt.DipoleEdge(k=0.02, e1=-0.05, model="full", side="exit", rot_s_rad=0.25),
           xt.Drift(length=0.2),
           xt.DipoleEdge(k=0.02, e1=0.1, model="suppressed", shift_y=-4e-4, rot_s_rad=0.1),
           xt.Drift(length=0.3),
           xt.LimitRect(min_x=-0.015, max_x=0.015, min_y=-0.01, max_y=0.01),
           xt.Drift(length=0.2),
           xt.Multipole(knl=[0.0, 0.05, -0.3, 2.0], ksl=[0.0, 0.0, 0.1], shift_y=2e-3,
                        rot_s_rad=0.7, rot_s_rad_no_frame=-0.3)]
    return xt.Line(elements=els)


def drift_aperture_pairs():
    """Drifts followed by apertures (the pattern of MAD-X thin lattices),
    runs of markers after drifts, apertures and kicks, an aperture after a
    kick, a shifted aperture after a drift, a drift followed by a drift,
    and a drift-aperture pair and a marker at the end of the line. The
    apertures cut into a wide beam."""
    els = [xt.Marker(),
           xt.Drift(length=0.5),
           xt.LimitRect(min_x=-0.02, max_x=0.018, min_y=-0.012, max_y=0.014),
           xt.Marker(), xt.Marker(),
           xt.Drift(length=0.3),
           xt.LimitEllipse(a=0.022, b=0.015),
           xt.Multipole(knl=[0.0, 0.04, 0.3]),
           xt.Marker(),
           xt.Drift(length=0.4),
           xt.Marker(),
           xt.LimitRect(min_x=-0.021, max_x=0.021, min_y=-0.016, max_y=0.016),
           xt.Drift(length=0.2),
           xt.LimitRect(min_x=-0.017, max_x=0.019, min_y=-0.013, max_y=0.013, shift_x=1e-3),
           xt.Marker(), xt.Marker(), xt.Marker(),
           xt.Drift(length=0.6),
           xt.LimitEllipse(a=0.019, b=0.013),
           xt.Drift(length=0.1),
           xt.Drift(length=0.2),
           xt.LimitRect(min_x=-0.018, max_x=0.017, min_y=-0.0125, max_y=0.012),
           xt.Multipole(knl=[0.0, -0.04]),
           xt.Drift(length=0.35),
           xt.LimitEllipse(a=0.0185, b=0.0122),
           xt.Marker()]
    return xt.Line(elements=els)
