"""Known-answer tests ported from the reference's own test-suite (their
assertions, restated on this package's API). Each runs on the CPU oracle
(checking that the oracle reproduces the reference's expected physics) and,
marked gpu, through Line.track on the GPU.

Sources (xtrack/tests): test_elements.py:496-551 (drift maps),
test_elements.py:822-846 (cavity energy gain), test_aperture_turn_ele_and_
monitor.py:14-113 (loss s / turn / element), test_apertures.py:16-44
(global aperture after thick elements only), test_magnet.py:25-110
(drift-kick-drift without kicks is a drift; backtracking returns to the
start), test_knl_rel_ksl_rel.py:21-150 (relative strengths), test_slice_
elements.py:13-130 (thin slices converge to the thick element),
test_monitor.py:71-192 (monitor layout)."""
import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt
from xtrack_gb300.particles import PROTON_MASS_EV


def _oracle(line, particles_kw, **kw):
    recs = line._element_records()
    p = xt.Particles(device="cpu", **particles_kw)
    a = pyoracle.host_arrays(p.to_numpy())
    pyoracle.track(recs, a, line_length=line.get_length(), **kw)
    return a


def _gpu(line, particles_kw, **kw):
    p = xt.Particles(device="cuda", **particles_kw)
    line.build_tracker(device="cuda")
    line.track(p, **kw)
    return p.to_numpy()


RUNNERS = [pytest.param(_oracle, id="oracle"),
           pytest.param(_gpu, id="gpu", marks=pytest.mark.gpu)]


def _track_kw(runner, n_el, num_turns=1, **extra):
    if runner is _oracle:
        return dict(num_turns=num_turns, **extra)
    return dict(num_turns=num_turns)


@pytest.mark.parametrize("run", RUNNERS)
def test_drift_maps(run):
    rng = np.random.default_rng(0)
    n = 50
    kw = dict(p0c=1e9, x=rng.normal(0, 1e-3, n), px=rng.normal(0, 1e-3, n),
              y=rng.normal(0, 1e-3, n), py=rng.normal(0, 1e-3, n), delta=rng.normal(0, 1e-3, n))
    L = 2.3
    for model in ("expanded", "exact"):
        line = xt.Line(elements=[xt.Drift(length=L, model=model)])
        line.config.XTRACK_GLOBAL_XY_LIMIT = None
        out = run(line, kw, **_track_kw(run, 1, flag_end_turn_actions=0) if run is _oracle else {})
        x0, px, py, d = kw["x"], kw["px"], kw["py"], kw["delta"]
        if model == "expanded":
            xe = x0 + px / (1 + d) * L
        else:
            xe = x0 + px / np.sqrt((1 + d) ** 2 - px ** 2 - py ** 2) * L
        np.testing.assert_allclose(out["x"], xe, rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(out["s"] if run is _oracle else L, L, rtol=1e-15)


@pytest.mark.parametrize("run", RUNNERS)
def test_cavity_energy_gain(run):
    cav = xt.Cavity(frequency=0, phase=np.pi / 2, voltage=30)
    line = xt.Line(elements=[cav])
    kw = dict(p0c=1e9, delta=[0, 1e-2], zeta=[0, 0.2])
    p0 = xt.Particles(device="cpu", **kw)
    out = run(line, kw, **({"flag_end_turn_actions": 0} if run is _oracle else {}))
    p0c = p0.p0c.numpy()
    energy0 = np.sqrt(p0c ** 2 + PROTON_MASS_EV ** 2) + p0.ptau.numpy() * p0c
    energy = np.sqrt(p0c ** 2 + PROTON_MASS_EV ** 2) + out["ptau"] * p0c
    np.testing.assert_allclose(energy, energy0 + 30, atol=5e-7, rtol=0)
    Pc = np.sqrt(energy ** 2 - PROTON_MASS_EV ** 2)
    delta = Pc / p0c - 1
    beta = Pc / energy
    beta0 = p0.beta0.numpy()
    np.testing.assert_allclose(out["delta"], delta, atol=1e-14, rtol=0)
    np.testing.assert_allclose(out["rpp"], 1 / (1 + delta), atol=1e-14, rtol=0)
    np.testing.assert_allclose(out["rvv"], beta / beta0, atol=1e-14, rtol=0)
    np.testing.assert_allclose(out["zeta"] / beta0, p0.zeta.numpy() / beta0, atol=1e-14, rtol=0)
    np.testing.assert_allclose((out["ptau"] - p0.ptau.numpy()) * p0c, 30, atol=1e-9, rtol=0)


@pytest.mark.parametrize("run", RUNNERS)
def test_aperture_turn_element_and_monitor(run):
    n_part = 100
    kw = dict(p0c=6500e9, x=np.zeros(n_part), px=np.linspace(-1, 1, n_part),
              y=np.zeros(n_part), py=np.linspace(-2, 2, n_part))
    tot_length = 2.0
    n_slices = 10000
    line = xt.Line(elements=n_slices * [xt.Drift(length=tot_length / n_slices)],
                   element_names=[f"drift{ii}" for ii in range(n_slices)])
    n_turns = 3
    if run is _oracle:
        recs = line._element_records()
        p = xt.Particles(device="cpu", **kw)
        a = pyoracle.host_arrays(p.to_numpy())
        mon = dict(start_at_turn=0, stop_at_turn=n_turns, part_id_start=0, part_id_end=n_part,
                   ebe_mode=0, n_repetitions=1, repetition_period=-1, n_records=n_turns * n_part,
                   data={f: np.zeros(n_turns * n_part, dtype=np.int64 if f in ("at_turn",) else np.float64)
                         for f in ("at_turn", "s", "x", "y", "px", "py")})
        pyoracle.track(recs, a, line_length=line.get_length(), num_turns=n_turns, monitor=mon,
                       flag_monitor=1)
        out = a
        mon_x = mon["data"]["x"].reshape(n_part, n_turns)
        mon_y = mon["data"]["y"].reshape(n_part, n_turns)
        mon_s = mon["data"]["s"].reshape(n_part, n_turns)
        mon_turn = mon["data"]["at_turn"].reshape(n_part, n_turns)
        mon_px = mon["data"]["px"].reshape(n_part, n_turns)
    else:
        p = xt.Particles(device="cuda", **kw)
        line.build_tracker(device="cuda")
        line.track(p, num_turns=n_turns, turn_by_turn_monitor=True)
        out = p.to_numpy()
        m = line.record_last_track
        mon_x, mon_y, mon_s, mon_turn, mon_px = m.x, m.y, m.s, m.at_turn, m.px

    lim = 1.0
    s_tot = tot_length * n_turns
    s_expected = []
    for ii in range(n_part):
        sx = abs(lim / out["px"][ii]) if abs(out["px"][ii]) * s_tot > lim else s_tot
        sy = abs(lim / out["py"][ii]) if abs(out["py"][ii] * s_tot) > lim else s_tot
        s_expected.append(min(sx, sy))
    s_expected = np.array(s_expected)
    at_turn_expected = np.clip(np.floor(s_expected / tot_length), 0, n_turns).astype(int)
    at_element_expected = np.clip(np.floor((s_expected - tot_length * at_turn_expected)
                                           / (tot_length / n_slices)), 0, n_slices - 1).astype(int)
    np.testing.assert_allclose(out["s"] + at_turn_expected * tot_length, s_expected, atol=1e-3)
    np.testing.assert_array_equal(out["at_turn"], at_turn_expected)
    np.testing.assert_allclose(out["at_element"], at_element_expected, atol=1.1)
    for ii in range(n_part):
        for tt in range(n_turns):
            if tt <= out["at_turn"][ii]:
                assert mon_turn[ii, tt] == tt
                assert abs(mon_s[ii, tt]) < 1e-14
                assert np.isclose(mon_x[ii, tt], tt * tot_length * out["px"][ii], atol=1e-14)
                assert np.isclose(mon_y[ii, tt], tt * tot_length * out["py"][ii], atol=1e-14)
                assert np.isclose(mon_px[ii, tt], out["px"][ii], atol=1e-14)
            else:
                assert mon_turn[ii, tt] == 0 and mon_s[ii, tt] == 0 and mon_x[ii, tt] == 0


@pytest.mark.parametrize("run", RUNNERS)
def test_global_aperture_only_after_thick(run):
    """A Multipole (dynamic isthick) is not followed by the global check; a
    Drift of zero length is."""
    kw = dict(p0c=1e9, x=[0.5, 2.0], px=[0.0, 0.0])
    line = xt.Line(elements=[xt.Multipole(knl=[0.0]), xt.Marker()])
    out = run(line, kw, **({"flag_end_turn_actions": 0} if run is _oracle else {}))
    assert np.all(out["state"] == 1)
    line = xt.Line(elements=[xt.Drift(length=0.0), xt.Marker()])
    out = run(line, kw, **({"flag_end_turn_actions": 0} if run is _oracle else {}))
    np.testing.assert_array_equal(out["state"], [1, -1])
    # the survivor passed both elements (the GPU run also ends the turn)
    np.testing.assert_array_equal(out["at_element"], [2, 0] if run is _oracle else [0, 0])


def test_dkd_without_kicks_is_a_drift():
    kw = dict(p0c=7e12, x=[1e-3, -2e-3], px=[1e-5, -3e-5], y=[2e-3, 1e-3], py=[-1e-5, 2e-5],
              delta=[1e-4, -2e-4])
    q = xt.Quadrupole(length=2.0, k1=0.0, model="drift-kick-drift-expanded", num_multipole_kicks=3)
    a = _oracle(xt.Line(elements=[q]), kw, flag_end_turn_actions=0)
    b = _oracle(xt.Line(elements=[xt.Drift(length=2.0)]), kw, flag_end_turn_actions=0)
    for f in ("x", "px", "y", "py", "zeta"):
        np.testing.assert_allclose(a[f], b[f], rtol=1e-15, atol=1e-15)


def test_knl_rel_equals_scaled_knl():
    kw = dict(p0c=7e12, x=[1e-3, -2e-3, 5e-3], y=[2e-3, 1e-3, -4e-3])
    k1, L = 0.01, 1.3
    rel = [1e-4, 2e-3, 5e-2, 1e-1]
    qa = xt.Quadrupole(length=L, k1=k1, knl_rel=rel, num_multipole_kicks=1,
                       model="drift-kick-drift-expanded")
    qb = xt.Quadrupole(length=L, k1=k1, knl=[r * k1 * L for r in rel], num_multipole_kicks=1,
                       model="drift-kick-drift-expanded")
    a = _oracle(xt.Line(elements=[qa]), kw, flag_end_turn_actions=0)
    b = _oracle(xt.Line(elements=[qb]), kw, flag_end_turn_actions=0)
    for f in ("x", "px", "y", "py"):
        np.testing.assert_allclose(a[f], b[f], rtol=1e-13, atol=1e-18)


def test_thin_slices_converge_to_thick_bend():
    kw = dict(p0c=7e12, x=[1e-3, -2e-3], px=[1e-5, 2e-5], y=[1e-3, 0.0], delta=[0.0, 1e-4])
    mk = lambda: xt.Bend(length=2.0, angle=0.01, k1=1e-3, model="drift-kick-drift-expanded",
                         num_multipole_kicks=1000, edge_entry_active=False,
                         edge_exit_active=False)
    thick = _oracle(xt.Line(elements=[mk()]), kw, flag_end_turn_actions=0)
    line = xt.Line(elements=[mk()], element_names=["b"])
    line.slice_thick_elements([xt.Strategy(slicing=xt.Teapot(1000))])
    thin = _oracle(line, kw, flag_end_turn_actions=0)
    for f in ("x", "px", "y", "py"):
        np.testing.assert_allclose(thin[f], thick[f], rtol=1e-6, atol=1e-12)


def test_backtrack_returns_to_start_oracle():
    from lattice_cases import sliced_line, small_beam
    line = sliced_line(thin=False)
    kw = small_beam(32, seed=3)
    recs = line._element_records()
    p = xt.Particles(device="cpu", **kw)
    a = pyoracle.host_arrays(p.to_numpy())
    x0 = {k: v.copy() for k, v in a.items()}
    L = line.get_length()
    pyoracle.track(recs, a, line_length=L, global_xy_limit=None)
    pyoracle.track(recs, a, line_length=L, global_xy_limit=None, track_flags=1)
    for f in ("x", "px", "y", "py"):
        np.testing.assert_allclose(a[f], x0[f], rtol=0, atol=5e-12 * np.max(np.abs(x0[f])))
    np.testing.assert_array_equal(a["at_turn"], 0)


def test_monitor_layout_multiframe():
    line = xt.Line(elements=[xt.Drift(length=1.0)])
    recs = line._element_records()
    n_part, period, nrep, n_turns_rec = 5, 4, 3, 2
    p = xt.Particles(device="cpu", p0c=1e9, x=np.zeros(n_part), px=np.linspace(0, 1e-3, n_part))
    a = pyoracle.host_arrays(p.to_numpy())
    n_rec = n_turns_rec * n_part * nrep
    mon = dict(start_at_turn=1, stop_at_turn=1 + n_turns_rec, part_id_start=0, part_id_end=n_part,
               ebe_mode=0, n_repetitions=nrep, repetition_period=period, n_records=n_rec,
               data={"at_turn": np.zeros(n_rec, dtype=np.int64), "particle_id": np.zeros(n_rec, dtype=np.int64)})
    pyoracle.track(recs, a, line_length=1.0, num_turns=14, monitor=mon, flag_monitor=1)
    at_turn = mon["data"]["at_turn"].reshape(nrep, n_part, n_turns_rec)
    pid = mon["data"]["particle_id"].reshape(nrep, n_part, n_turns_rec)
    for f in range(nrep):
        for t in range(n_turns_rec):
            assert np.all(at_turn[f, :, t] == 1 + f * period + t)
        assert np.all(pid[f] == np.arange(n_part)[:, None])
