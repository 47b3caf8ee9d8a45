"""Synthetic lattices and beams of the benchmark configurations.

No public dataset is involved: every lattice and beam below is generated
from a fixed seed with numpy's PCG64 generator, so it is identical on every
machine.

toy_ring()       100 thin FODO cells [Drift 5 m, Multipole knl=[0,+0.02,+0.1],
                 Drift 5 m, Multipole knl=[0,-0.02,-0.1], LimitEllipse a=b=0.02]
                 plus one Cavity (6 MV, 400 MHz, lag 180 deg); protons at
                 p0c = 450 GeV. 501 elements.
thick_ring()     8 arcs x 23 FODO cells of thick magnets: per cell 6 Bends
                 (L = 14.3 m, angle = 2*pi/1104), 2 Quadrupoles (L = 3.1 m,
                 k1 = +-0.0087 m^-2), 2 Sextupoles (L = 0.37 m, k2 = +-0.1 m^-3)
                 and 2 thin octupoles (Multipole order 3), each magnet tracked
                 drift-kick-drift-expanded with 8 uniform kicks, a LimitRect
                 after every magnet, Gaussian relative multipole errors of
                 orders 0..10 (sigma 1e-4 of the main field at R = 17 mm) and
                 one Cavity (16 MV, 400 MHz, lag 180 deg); protons at 7 TeV.
                 6993 elements.
gaussian_beam()  x, y sigma 1 mm; px, py sigma 1e-5; zeta sigma 0.1 m;
                 delta sigma 1e-4.
"""
import math

import numpy as np

from . import elements as el
from .line import Line
from .particles import Particles, PROTON_MASS_EV


def toy_ring():
    elements, names = [], []
    qf = el.Multipole(knl=[0.0, 0.02, 0.1])
    qd = el.Multipole(knl=[0.0, -0.02, -0.1])
    for i in range(100):
        elements += [el.Drift(length=5.0), qf, el.Drift(length=5.0), qd,
                     el.LimitEllipse(a=0.02, b=0.02)]
        names += [f"d1.{i}", f"qf.{i}", f"d2.{i}", f"qd.{i}", f"ap.{i}"]
    elements.append(el.Cavity(voltage=6e6, frequency=400e6, lag=180.0))
    names.append("cav")
    line = Line(elements=elements, element_names=names)
    line.particle_ref = Particles(p0c=450e9, mass0=PROTON_MASS_EV, device="cpu")
    return line


def _rel_errors(rng, main_order, sigma=1e-4, r_ref=0.017, max_order=10):
    """knl_rel / ksl_rel for relative field errors b_n, a_n ~ N(0, sigma) at
    the reference radius: knl_n / knl_main = b_n * n!/m! * R^(m-n)."""
    knl_rel, ksl_rel = [], []
    for n in range(max_order + 1):
        scale = math.factorial(n) / math.factorial(main_order) * r_ref ** (main_order - n)
        knl_rel.append(rng.normal(0.0, sigma) * scale)
        ksl_rel.append(rng.normal(0.0, sigma) * scale)
    return knl_rel, ksl_rel


def thick_ring(seed=1, n_arcs=8, n_cells=23, with_errors=True, num_kicks=8,
               model="drift-kick-drift-expanded", integrator="uniform", k3l=0.5,
               aperture=(0.022, 0.0176), bend_angle=None):
    """``bend_angle`` defaults to 2 pi / (6 n_arcs n_cells) (a closed ring);
    shorter test rings pass the full ring's angle to keep its cell optics."""
    rng = np.random.default_rng(seed)
    angle = 2 * math.pi / (6 * n_arcs * n_cells) if bend_angle is None else bend_angle
    kw = dict(model=model, integrator=integrator, num_multipole_kicks=num_kicks)
    ax, ay = aperture
    elements, names = [], []

    def add(name, e):
        elements.append(e)
        names.append(name)

    def err(order):
        return _rel_errors(rng, order) if with_errors else (None, None)

    for a in range(n_arcs):
        for c in range(n_cells):
            tag = f"{a}.{c}"
            add(f"start.{tag}", el.Marker())
            for half, sign in (("f", 1.0), ("d", -1.0)):
                knl_rel, ksl_rel = err(1)
                add(f"dq{half}.{tag}", el.Drift(length=0.5))
                add(f"mq{half}.{tag}", el.Quadrupole(length=3.1, k1=sign * 0.0087,
                                                     knl_rel=knl_rel, ksl_rel=ksl_rel, **kw))
                add(f"apq{half}.{tag}", el.LimitRect(min_x=-ax, max_x=ax, min_y=-ay, max_y=ay))
                knl_rel, ksl_rel = err(2)
                add(f"ds{half}.{tag}", el.Drift(length=0.5))
                add(f"ms{half}.{tag}", el.Sextupole(length=0.37, k2=sign * 0.1,
                                                    knl_rel=knl_rel, ksl_rel=ksl_rel, **kw))
                add(f"aps{half}.{tag}", el.LimitRect(min_x=-ax, max_x=ax, min_y=-ay, max_y=ay))
                knl_rel, ksl_rel = err(3)
                add(f"do{half}.{tag}", el.Drift(length=0.3))
                add(f"mo{half}.{tag}", el.Multipole(knl=[0.0, 0.0, 0.0, sign * k3l], main_order=3,
                                                    knl_rel=knl_rel, ksl_rel=ksl_rel))
                add(f"apo{half}.{tag}", el.LimitRect(min_x=-ax, max_x=ax, min_y=-ay, max_y=ay))
                for b in range(3):
                    knl_rel, ksl_rel = err(0)
                    add(f"db{half}{b}.{tag}", el.Drift(length=0.5))
                    add(f"mb{half}{b}.{tag}", el.Bend(length=14.3, angle=angle, knl_rel=knl_rel,
                                                      ksl_rel=ksl_rel, **kw))
                    add(f"apb{half}{b}.{tag}", el.LimitRect(min_x=-ax, max_x=ax, min_y=-ay, max_y=ay))
            add(f"dend.{tag}", el.Drift(length=8.56))
    add("cav", el.Cavity(voltage=16e6, frequency=400e6, lag=180.0))
    line = Line(elements=elements, element_names=names)
    line.particle_ref = Particles(p0c=7e12, mass0=PROTON_MASS_EV, device="cpu")
    return line


def gaussian_beam(n, p0c, seed=0, device=None, sigma_x=1e-3, sigma_px=1e-5, sigma_zeta=0.1,
                  sigma_delta=1e-4):
    rng = np.random.default_rng(seed)
    x = rng.normal(0.0, sigma_x, n)
    px = rng.normal(0.0, sigma_px, n)
    y = rng.normal(0.0, sigma_x, n)
    py = rng.normal(0.0, sigma_px, n)
    zeta = rng.normal(0.0, sigma_zeta, n)
    delta = rng.normal(0.0, sigma_delta, n)
    return Particles(p0c=p0c, mass0=PROTON_MASS_EV, x=x, px=px, y=y, py=py, zeta=zeta,
                     delta=delta, device=device)
