"""Monitors placed in the line: LastTurnsMonitor and BeamPositionMonitor
with the scenarios of the reference's tests/test_monitor.py (a one-element
line, particles moved and lost between turns), run on the CPU oracle and
on the GPU push; and a ParticlesMonitor element against the turn-by-turn
monitor of the tracker."""
import numpy as np
import pytest

import pyoracle
import xtrack_gb300 as xt


def _oracle_turn(line, p):
    a = pyoracle.host_arrays(p.to_numpy())
    pyoracle.track(line._element_records(), a, num_turns=1, line_length=line.get_length())
    for k in ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "state",
              "at_turn", "at_element"):
        getattr(p, k).copy_(__import__("torch").from_numpy(a[k]))


def _gpu_turn(line, p):
    line.track(p, num_turns=1)


def _last_turns_scenario(device, turn_fn):
    p = xt.Particles(p0c=6.5e12, x=[1.0, 2, 3, 4, 5, 6], device=device)
    mon = xt.LastTurnsMonitor(n_last_turns=5, particle_id_range=(1, 5), device=device)
    line = xt.Line(elements=[mon], element_names=["mon"])
    if device != "cpu":
        line.build_tracker(device=device)
    for turn in range(10):
        turn_fn(line, p)
        d = np.array([1, -1, 2, -2, 3, -3], dtype=np.float64)
        p.x += __import__("torch").from_numpy(d).to(p.x.device)
        if turn == 2:
            p.state[1] = 0
        if turn == 4:
            p.state[2] = 0
        if turn == 6:
            p.state[3] = 0
    return mon


def _check_last_turns(mon):
    assert np.all(mon.particle_id == np.array([[0, 0, 1, 1, 1], [2] * 5, [3] * 5, [4] * 5]))
    expect_turn = np.array([np.clip(n - np.arange(4, -1, -1), 0, None) for n in (2, 4, 6, 9)])
    assert np.all(mon.at_turn == expect_turn)
    assert np.all(mon.x == np.array([[0, 0, 2, 1, 0], [3, 5, 7, 9, 11], [0, -2, -4, -6, -8],
                                     [20, 23, 26, 29, 32]]))


def _bpm_scenario(device, turn_fn):
    import torch
    npart = 512
    n = npart + 4
    p = xt.Particles(p0c=6.5e12, x=0.1 * np.arange(n), y=-0.1 * np.arange(n),
                     zeta=-2.99792458e8 * np.tile([0.0, 0.5], n // 2), device=device)
    mon = xt.BeamPositionMonitor(num_particles=npart, start_at_turn=0, stop_at_turn=10, frev=1,
                                 sampling_frequency=2, device=device)
    line = xt.Line(elements=[mon], element_names=["bpm"])
    if device != "cpu":
        line.build_tracker(device=device)
    for turn in range(11):
        p.x[0] += 0.5
        p.y[0] -= 0.5
        if turn == 8:
            p.state[256:] = 0
        if turn == 9:
            p.state[:] = 0
        turn_fn(line, p)
    return mon, npart


def _check_bpm(mon, npart):
    expected_count = np.tile([npart // 2, npart // 2], 10).astype(float)
    expected_count[16:18] = 128
    expected_count[18:20] = 0
    assert np.array_equal(mon.count, expected_count)
    expected_x_sum = np.tile([0.1 * (npart - 2) * npart / 4, 0.1 * npart * npart / 4], 10)
    expected_x_sum[0::2] += 0.5 * np.arange(1, 11)
    expected_x_sum[16:18] = [1625.6 + 4.5, 1638.4]
    expected_x_sum[18:20] = 0
    assert np.allclose(mon.x_sum, expected_x_sum, rtol=1e-12)
    assert np.allclose(mon.y_sum, -expected_x_sum, rtol=1e-12)
    cen = mon.x_cen
    assert np.allclose(cen[:18], expected_x_sum[:18] / expected_count[:18], rtol=1e-12)
    assert np.all(np.isnan(cen[18:]))


def test_last_turns_monitor_oracle():
    _check_last_turns(_last_turns_scenario("cpu", _oracle_turn))


def test_beam_position_monitor_oracle():
    _check_bpm(*_bpm_scenario("cpu", _oracle_turn))


def test_monitor_element_validation():
    m = xt.LastTurnsMonitor(n_last_turns=2, num_particles=3, device="cpu")
    with pytest.raises(ValueError):
        xt.LastTurnsMonitor(n_last_turns=2, num_particles=3, particle_id_range=(0, 3))
    with pytest.raises(ValueError):
        xt.LastTurnsMonitor(n_last_turns=0, num_particles=3)
    assert m.to_record()["cls"] == 10


@pytest.mark.gpu
def test_last_turns_monitor_gpu():
    _check_last_turns(_last_turns_scenario("cuda", _gpu_turn))


@pytest.mark.gpu
def test_beam_position_monitor_gpu():
    _check_bpm(*_bpm_scenario("cuda", _gpu_turn))


@pytest.mark.gpu
def test_particles_monitor_element_equals_turn_by_turn_monitor():
    """A ParticlesMonitor at the start of the ring records what the
    tracker's turn-by-turn monitor records, and the ring's tracking is
    unchanged by monitor elements (LastTurns and BPM inserted too)."""
    from xtrack_gb300 import workloads
    base = workloads.toy_ring()
    n = 200
    rng = np.random.default_rng(3)
    kw = dict(p0c=450e9, x=rng.normal(0, 3e-3, n), px=rng.normal(0, 3e-5, n),
              y=rng.normal(0, 3e-3, n), zeta=rng.normal(0, 0.1, n), delta=rng.normal(0, 1e-4, n))
    pm = xt.ParticlesMonitor(start_at_turn=0, stop_at_turn=20, num_particles=n, device="cuda")
    lt = xt.LastTurnsMonitor(n_last_turns=4, num_particles=n, device="cuda")
    bpm = xt.BeamPositionMonitor(start_at_turn=0, stop_at_turn=20, frev=1, sampling_frequency=1,
                                 device="cuda")
    names = ["pm", "lt", "bpm"] + list(base.element_names)
    line = xt.Line(elements=[pm, lt, bpm] + [base[nm] for nm in base.element_names],
                   element_names=names)
    line.build_tracker(device="cuda")
    p = xt.Particles(device="cuda", **kw)
    line.track(p, num_turns=20, turn_by_turn_monitor=True)
    tbt = line.record_last_track
    for f in ("x", "px", "y", "py", "zeta", "delta", "at_turn", "state"):
        assert np.array_equal(getattr(pm, f), getattr(tbt, f)), f
    ref = xt.Particles(device="cuda", **kw)
    base.build_tracker(device="cuda")
    base.track(ref, num_turns=20)
    assert np.array_equal(p.x.cpu().numpy(), ref.x.cpu().numpy())
    assert np.array_equal(p.at_element.cpu().numpy() - 3 * (p.state.cpu().numpy() <= 0),
                          ref.at_element.cpu().numpy())
    # the BPM saw every pass of every alive particle
    alive_per_turn = (tbt.state > 0).sum(axis=0)
    assert np.array_equal(bpm.count, alive_per_turn.astype(float))


def _size_scenario(device, turn_fn):
    npart = 512
    x = np.linspace(-0.1, 0.1, npart + 4) ** 2
    p = xt.Particles(p0c=6.5e12, x=x, y=10 * x,
                     zeta=-2.99792458e8 * np.tile([0.0, 0.5], (npart + 4) // 2), device=device)
    mon = xt.BeamSizeMonitor(num_particles=npart, start_at_turn=0, stop_at_turn=10, frev=1,
                             sampling_frequency=2, device=device)
    line = xt.Line(elements=[mon], element_names=["bsm"])
    if device != "cpu":
        line.build_tracker(device=device)
    for turn in range(11):
        p.x[0] += 0.005
        p.y[0] += 0.05
        if turn == 8:
            p.state[256:] = 0
        if turn == 9:
            p.state[:] = 0
        turn_fn(line, p)
    return mon, x, npart


def _check_size(mon, x, npart):
    expected_count = np.tile([npart // 2, npart // 2], 10).astype(float)
    expected_count[16:18] = 128
    expected_count[18:20] = 0
    assert np.array_equal(mon.count, expected_count)
    xr = x[:npart].reshape((-1, 2))
    ex = np.tile(np.sum(xr, axis=0), 10)
    ex[0::2] += 0.005 * np.arange(1, 11)
    ex[16:18] -= np.sum(xr[128:, :], axis=0)
    ex[18:20] = 0
    assert np.allclose(mon.x_sum, ex, rtol=1e-10, atol=1e-15)
    assert np.allclose(mon.y_sum, 10 * ex, rtol=1e-10, atol=1e-14)
    ex2 = np.tile(np.sum(xr ** 2, axis=0), 10)
    ex2[0::2] += 2 * xr[0, 0] * 0.005 * np.arange(1, 11) + (0.005 * np.arange(1, 11)) ** 2
    ex2[16:18] -= np.sum(xr[128:, :] ** 2, axis=0)
    ex2[18:20] = 0
    assert np.allclose(mon.x2_sum, ex2, rtol=1e-10, atol=1e-16)
    assert np.allclose(mon.y2_sum, 100 * ex2, rtol=1e-10, atol=1e-14)
    mean = ex[:18] / expected_count[:18]
    var = ex2[:18] / expected_count[:18] - mean ** 2
    assert np.allclose(mon.x_var[:18], var, rtol=1e-6, atol=1e-15)
    assert np.all(np.isnan(mon.x_std[18:]))


def _profile_scenario(device, turn_fn):
    gen = np.random.default_rng(seed=38715345)
    npart = 512
    x = gen.normal(size=npart + 4)
    y = gen.normal(size=npart + 4)
    p = xt.Particles(p0c=6.5e12, x=x, y=y, zeta=-2.99792458e8 * np.tile([0.0, 0.5], x.size // 2),
                     device=device)
    mon = xt.BeamProfileMonitor(num_particles=npart, start_at_turn=0, stop_at_turn=10, frev=1,
                                sampling_frequency=2, n=100, x_range=5, y_range=(-4, 2),
                                device=device)
    line = xt.Line(elements=[mon], element_names=["bpf"])
    if device != "cpu":
        line.build_tracker(device=device)
    for turn in range(11):
        p.x[0] += 0.1
        p.y[0] -= 0.1
        if turn == 8:
            p.state[256:] = 0
        if turn == 9:
            p.state[:] = 0
        turn_fn(line, p)
    return mon, x, y, npart


def _check_profile(mon, x, y, npart):
    nb = 100
    ex_x = np.zeros((20, nb))
    ex_y = np.zeros((20, nb))
    for turn in range(10):
        for sub in range(2):
            lim = {8: 256, 9: 0}.get(turn, npart)
            xs = np.copy(x[:lim][sub::2])
            ys = np.copy(y[:lim][sub::2])
            if sub == 0 and lim > 0:
                xs[0] += 0.1 * (turn + 1)
                ys[0] -= 0.1 * (turn + 1)
            hx, edges_x = np.histogram(xs, bins=nb, range=(-2.5, 2.5))
            hy, edges_y = np.histogram(ys, bins=nb, range=(-4, 2))
            ex_x[2 * turn + sub] = hx
            ex_y[2 * turn + sub] = hy
    assert np.allclose(mon.x_edges, edges_x)
    assert np.allclose(mon.y_grid, 0.5 * (edges_y[1:] + edges_y[:-1]))
    assert np.array_equal(mon.x_intensity, ex_x)
    assert np.array_equal(mon.y_intensity, ex_y)


def test_beam_size_monitor_oracle():
    _check_size(*_size_scenario("cpu", _oracle_turn))


def test_beam_profile_monitor_oracle():
    _check_profile(*_profile_scenario("cpu", _oracle_turn))


@pytest.mark.gpu
def test_beam_size_monitor_gpu():
    _check_size(*_size_scenario("cuda", _gpu_turn))


@pytest.mark.gpu
def test_beam_profile_monitor_gpu():
    _check_profile(*_profile_scenario("cuda", _gpu_turn))


def _multi_element_oracle(line, kw, names, turns):
    """The oracle's multi-element monitor over the same observation points."""
    import pyoracle as po
    recs = line._element_records()
    p = xt.Particles(device="cpu", **kw)
    arrs = po.host_arrays(p.to_numpy())
    elnames = list(line.element_names)
    obs = [elnames.index(n) for n in names]
    mapping = np.full(len(elnames) + 1, -1, dtype=np.int64)
    mapping[obs] = np.arange(len(obs))
    data = np.zeros((turns, len(arrs["x"]), 7, len(obs)))
    po.set_multi_element_monitor(mapping, data, 0, turns, 0, len(arrs["x"]))
    try:
        po.track(recs, arrs, num_turns=turns, line_length=line.get_length())
    finally:
        po.set_multi_element_monitor(None, None, 0, 0, 0, 0)
    return data


def test_multi_element_monitor_oracle_records_before_elements():
    from xtrack_gb300 import workloads
    line = workloads.toy_ring()
    n = 16
    rng = np.random.default_rng(4)
    kw = dict(p0c=450e9, x=rng.normal(0, 1e-3, n), px=rng.normal(0, 1e-5, n))
    names = [line.element_names[k] for k in (0, 3, 250, 500)]
    data = _multi_element_oracle(line, kw, names, 3)
    # before the first element of turn 0: the initial coordinates
    assert np.array_equal(data[0, :, 0, 0], kw["x"])
    assert np.all(data[:, :, 6, 0] == 0.0)       # s at the start of each turn
    assert np.all(np.diff(data[0, :, 6, :], axis=1) > 0)


@pytest.mark.gpu
def test_multi_element_monitor_gpu_matches_oracle():
    from xtrack_gb300 import workloads
    line = workloads.toy_ring()
    n = 300
    rng = np.random.default_rng(5)
    kw = dict(p0c=450e9, x=rng.normal(0, 3e-3, n), px=rng.normal(0, 3e-5, n),
              y=rng.normal(0, 3e-3, n), zeta=rng.normal(0, 0.1, n), delta=rng.normal(0, 1e-4, n))
    names = [line.element_names[k] for k in (0, 1, 3, 17, 250, 499, 500)]
    ref = _multi_element_oracle(line, kw, names, 5)
    line.build_tracker(device="cuda")
    p = xt.Particles(device="cuda", **kw)
    line.track(p, num_turns=5, multi_element_monitor_at=names)
    mem = line.record_multi_element_last_track
    got = mem.data
    assert got.shape == ref.shape
    scale = np.max(np.abs(ref), axis=(0, 1, 3), keepdims=True)
    scale[scale == 0] = 1
    assert np.max(np.abs(got - ref) / scale) <= 5e-14
    assert np.array_equal(mem.get("x", obs_name=names[0], particle_id=3, turn=0), kw["x"][3])
