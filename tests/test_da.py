"""DA tools: normal form, closed orbit and DA extraction on known maps
(CPU), and on the GPU a scaled-down batched DA scan whose per-seed result
equals the scan of each seed tracked on its own."""
import numpy as np
import pytest

from xtrack_gb300 import da


def _rot(mu):
    return np.array([[np.cos(mu), np.sin(mu)], [-np.sin(mu), np.cos(mu)]])


def _cs(beta, alpha):
    return np.array([[np.sqrt(beta), 0.0], [-alpha / np.sqrt(beta), 1 / np.sqrt(beta)]])


def _known_map():
    W = np.zeros((6, 6))
    W[0:2, 0:2] = _cs(80.0, -1.3)
    W[2:4, 2:4] = _cs(25.0, 0.7)
    W[4:6, 4:6] = _cs(900.0, 0.0)
    # a dispersion-like coupling of delta into x (symplectic shear)
    T = np.eye(6)
    T[0, 5] = 1.7
    T[1, 5] = 0.03
    T[4, 0] = -0.03
    T[4, 1] = 1.7
    W = T @ W
    Rot = np.zeros((6, 6))
    q = (0.31, 0.32, 0.002)
    for k in range(3):
        Rot[2 * k:2 * k + 2, 2 * k:2 * k + 2] = _rot(2 * np.pi * q[k])
    return W @ Rot @ np.linalg.inv(W), W, q


def test_known_map_is_symplectic():
    R, W, _ = _known_map()
    assert np.allclose(W.T @ da.S6 @ W, da.S6, atol=1e-12)
    assert np.allclose(R.T @ da.S6 @ R, da.S6, atol=1e-12)


def test_linear_normal_form_recovers_tunes_and_block_rotation():
    R, W0, q = _known_map()
    W, tunes = da.linear_normal_form(R)
    assert np.allclose(tunes, q, atol=1e-12)
    assert np.allclose(W.T @ da.S6 @ W, da.S6, atol=1e-10)
    B = np.linalg.inv(W) @ R @ W
    for k in range(3):
        assert np.allclose(B[2 * k:2 * k + 2, 2 * k:2 * k + 2], _rot(2 * np.pi * q[k]), atol=1e-10)
    off = B.copy()
    for k in range(3):
        off[2 * k:2 * k + 2, 2 * k:2 * k + 2] = 0
    assert np.max(np.abs(off)) < 1e-10
    # Courant-Snyder form of the transverse blocks: W[0,1] = W[2,3] = 0
    assert abs(W[0, 1]) < 1e-12 and abs(W[2, 3]) < 1e-12
    assert np.isclose(W[0, 0], np.sqrt(80.0), rtol=1e-9)


def test_closed_orbit_and_matrix_of_an_affine_map():
    R, _, _ = _known_map()
    co = np.array([1e-3, -2e-5, 3e-4, 1e-5, 0.02, 1e-4])
    fn = lambda c: (np.atleast_2d(c) - co) @ R.T + co
    x = da.closed_orbit(fn, guess=np.zeros(6))
    assert np.allclose(x, co, rtol=0, atol=1e-12)
    M, _ = da.one_turn_matrix(fn, x)
    assert np.allclose(M, R, atol=1e-6)


def test_polar_grid_and_dynamic_aperture():
    r, th = da.polar_grid(r_max=10.0, n_r=10, n_angles=3)
    assert r.shape == th.shape == (30,)
    assert np.all((th > 0) & (th < np.pi / 2))
    # lost above an angle-dependent radius, at a turn below the budget
    ang = np.unique(th)
    lim = {a: 3.0 + 2 * k for k, a in enumerate(ang)}
    state = np.array([0 if rr >= lim[t] else 1 for rr, t in zip(r, th)])
    at_turn = np.where(state > 0, 100, 17)
    a, d = da.dynamic_aperture(r, th, state, at_turn, 100)
    assert np.allclose(a, ang)
    assert np.allclose(d, [3.0, 5.0, 7.0])
    # a loss at the last turn boundary does not count (the turn was survived)
    a, d = da.dynamic_aperture(r, th, np.zeros_like(state), np.full_like(state, 100), 100)
    assert np.allclose(d, 10.0)


def test_normalized_to_physical_round_trip():
    R, W, _ = _known_map()
    co = np.array([1e-3, 0, 0, 0, 0, 0])
    z = da.normalized_to_physical(W, co, np.array([1.0, 2.0]), np.array([0.5, 0.0]), 2.5e-6,
                                  2.5e-6, 1.0, 7460.5)
    eps = 2.5e-6 / 7460.5
    zn = np.linalg.inv(W) @ (z - co[:, None])
    assert np.allclose(zn[0], [np.sqrt(eps), 2 * np.sqrt(eps)])
    assert np.allclose(zn[2], [0.5 * np.sqrt(eps), 0.0])


@pytest.mark.gpu
def test_batched_da_scan_equals_per_seed_scans():
    import xtrack_gb300 as xt
    from xtrack_gb300 import workloads
    # 3 cells: horizontal tune near 0.75 (4 cells would sit on the integer)
    seeds = [workloads.thick_ring(seed=s, n_arcs=1, n_cells=3, bend_angle=2 * np.pi / 1104)
             for s in (1, 2, 3)]
    ref_kw = dict(p0c=7e12, mass0=xt.PROTON_MASS_EV)
    beta0 = float(seeds[0].particle_ref.beta0[0])
    gamma0 = float(seeds[0].particle_ref.gamma0[0])
    r, th = da.polar_grid(r_max=400.0, n_r=40, n_angles=5)
    coords, lat = [], []
    for s, line in enumerate(seeds):
        tr = line.build_tracker(device="cuda")
        fn = da.line_track_fn(tr, ref_kw)
        co = da.closed_orbit(fn)
        R, _ = da.one_turn_matrix(fn, co)
        W, tunes = da.linear_normal_form(R)
        assert np.all(tunes > 0)
        z = da.normalized_to_physical(W, co, r * np.cos(th), r * np.sin(th), 2.5e-6, 2.5e-6,
                                      beta0, gamma0)
        coords.append(z)
        lat.append(np.full(len(r), s, dtype=np.int32))
    z = np.concatenate(coords, axis=1)
    lat = np.concatenate(lat)
    kw = {f: z[k] for k, f in enumerate(da.COORDS)}
    beam = xt.Particles(device="cuda", **ref_kw, **kw)
    bt = xt.BatchTracker(seeds, device="cuda")
    bt.set_tuning(compact_every=8)
    turns = 64
    bt.track(beam, lattice_index=lat, num_turns=turns)
    state = beam.state.cpu().numpy()
    at_turn = beam.at_turn.cpu().numpy()
    pid = beam.particle_id.cpu().numpy()
    assert np.array_equal(pid, np.arange(len(pid)))
    lost_any = False
    for s, line in enumerate(seeds):
        sel = lat == s
        a, d = da.dynamic_aperture(r, th, state[sel], at_turn[sel], turns)
        one = xt.Particles(device="cuda", **ref_kw, **{f: v[sel] for f, v in kw.items()})
        line.build_tracker(device="cuda")._track(one, num_turns=turns)
        a1, d1 = da.dynamic_aperture(r, th, one.state.cpu().numpy(), one.at_turn.cpu().numpy(),
                                     turns)
        assert np.array_equal(d, d1)
        lost_any |= bool(np.any(d < r.max()))
    assert lost_any


@pytest.mark.gpu
def test_scan_module_da_table_matches_plain_tracking():
    """scan.build_scan / run_scan / da_table over two seeds: the DA table
    from one batched run equals the one from tracking each seed alone, and
    the screened outcome with every particle tracked is the plain one."""
    import xtrack_gb300 as xt
    from xtrack_gb300 import scan as sc
    from xtrack_gb300 import surrogate as sg
    from xtrack_gb300 import workloads
    lines = [workloads.thick_ring(seed=s, n_arcs=1, n_cells=3, bend_angle=2 * np.pi / 1104)
             for s in (5, 6)]
    s = sc.build_scan(lines, [880, 1320], r_max=300.0, n_angles=4, features=sg.seed_features)
    assert s.seed_features.shape == (2, sg.N_SEED_FEATURES)
    bt = xt.BatchTracker(lines, device="cuda")
    st, at, ae = sc.run_scan(bt, s, 40)
    surv = sg.targets(st, at, 40)[0] > 0
    table = sc.da_table(s, surv, 2)
    assert table.shape == (2, 2, 4)
    assert np.any(table < 300.0)
    for k, line in enumerate(lines):
        sel = s.lattice_index == k
        p = sc.make_particles(s, sel)
        line.build_tracker(device="cuda")._track(p, num_turns=40)
        assert np.array_equal(p.state.cpu().numpy(), st[sel])
        assert np.array_equal(p.at_turn.cpu().numpy(), at[sel])
    p_all = np.full(s.n, 0.5)
    out = sg.screened_outcome(p_all, np.ones(s.n, dtype=bool), surv)
    assert np.array_equal(out, surv)


def test_linear_aperture_of_an_uncoupled_ring():
    """One rectangular aperture at the start of a ring with Courant-Snyder
    optics (beta_x = 80 m, beta_y = 25 m), no orbit: the linear aperture of
    a ray at angle t is min(a_x / (cos t sigma_x), a_y / (sin t sigma_y))."""
    W = np.zeros((6, 6))
    W[0:2, 0:2] = _cs(80.0, -1.3)
    W[2:4, 2:4] = _cs(25.0, 0.7)
    W[4:6, 4:6] = _cs(900.0, 0.0)
    dx = np.zeros((6, 1))
    dy = np.zeros((6, 1))
    dx[0, 0] = 1.0
    dy[2, 0] = 1.0
    ax, ay = 0.02, 0.015
    rect = np.array([[-ax, ax, -ay, ay]])
    ell = np.full((1, 2), np.inf)
    angles = np.linspace(0.1, 1.4, 7)
    beta0, gamma0 = 0.9999, 7000.0
    eps = 2.5e-6 / (beta0 * gamma0)
    got = da.linear_aperture(np.zeros(1), np.zeros(1), dx, dy, W, rect, ell, [0.0], angles,
                             2.5e-6, 2.5e-6, beta0, gamma0)
    sx, sy = np.sqrt(80.0 * eps), np.sqrt(25.0 * eps)
    want = np.minimum(ax / (np.cos(angles) * sx), ay / (np.sin(angles) * sy))
    assert np.allclose(got[0], want, rtol=1e-9)
    # an orbit offset eats into the aperture on one side
    got_co = da.linear_aperture(np.array([0.005]), np.zeros(1), dx, dy, W, rect, ell, [0.0],
                                angles, 2.5e-6, 2.5e-6, beta0, gamma0)
    want_co = np.minimum((ax - 0.005) / (np.cos(angles) * sx), ay / (np.sin(angles) * sy))
    assert np.allclose(got_co[0], want_co, rtol=1e-9)
    # an elliptical aperture of the same half axes, on the diagonal ray
    got_e = da.linear_aperture(np.zeros(1), np.zeros(1), dx, dy, W,
                               np.array([[-np.inf, np.inf, -np.inf, np.inf]]),
                               np.array([[ax, ay]]), [0.0], [np.pi / 4], 2.5e-6, 2.5e-6,
                               beta0, gamma0)
    c = np.cos(np.pi / 4)
    want_e = 1.0 / np.sqrt((c * sx / ax) ** 2 + (c * sy / ay) ** 2)
    assert np.isclose(got_e[0, 0], want_e, rtol=1e-9)
