"""Dynamic-aperture scans on top of the push.

The pieces a DA study needs around ``Line.track``:

* ``closed_orbit`` and ``one_turn_matrix``: Newton search of the 6-D closed
  orbit and the central-difference one-turn matrix around it, both from
  tracking (the quantities xtrack's twiss derives for its normalisation:
  xtrack/twiss/closed_orbit.py:24 ``find_closed_orbit_line``,
  xtrack/line.py:3324 ``compute_one_turn_matrix_finite_differences``);
* ``linear_normal_form``: the symplectic matrix W with R = W Rot W^-1 that
  maps normalised coordinates to physical ones (xtrack/linear_normal_form.py:
  61-147 ``get_linear_normal_form``);
* ``polar_grid`` and ``normalized_to_physical``: initial conditions on a
  polar grid of normalised amplitudes (in beam sigmas);
* ``dynamic_aperture``: per angle, the smallest amplitude lost within the
  turn budget, from the ``state`` / ``at_turn`` map that tracking leaves;
* ``linear_aperture``: per ray, the amplitude at which the linear motion
  around the closed orbit first reaches an aperture (a physics prior for
  the DA of an aperture-limited ring).

``track_fn(coords) -> coords`` is any one-turn map on an ``(n, 6)`` array of
(x, px, y, py, zeta, delta); ``line_track_fn`` builds one from a tracker.
"""
import itertools

import numpy as np

COORDS = ("x", "px", "y", "py", "zeta", "delta")

S6 = np.zeros((6, 6))
for _k in range(3):
    S6[2 * _k, 2 * _k + 1] = 1.0
    S6[2 * _k + 1, 2 * _k] = -1.0


def line_track_fn(tracker, particle_ref_kwargs, device="cuda"):
    """One-turn map through ``tracker`` for (n, 6) coordinate arrays."""
    from .particles import Particles

    def fn(c):
        c = np.atleast_2d(np.asarray(c, dtype=np.float64))
        p = Particles(device=device, x=c[:, 0], px=c[:, 1], y=c[:, 2], py=c[:, 3],
                      zeta=c[:, 4], delta=c[:, 5], **particle_ref_kwargs)
        tracker._track(p, num_turns=1)
        out = np.stack([getattr(p, f).cpu().numpy() for f in COORDS], axis=1)
        state = p.state.cpu().numpy()
        if np.any(state <= 0):
            raise RuntimeError("a probe particle was lost while computing the one-turn map")
        return out
    return fn


def one_turn_matrix(track_fn, co, steps=(1e-10, 1e-10, 1e-10, 1e-10, 1e-9, 1e-9)):
    """Central differences around ``co``: column j is
    (M(co + h e_j) - M(co - h e_j)) / 2h."""
    co = np.asarray(co, dtype=np.float64)
    probes = [co]
    for j in range(6):
        e = np.zeros(6)
        e[j] = steps[j]
        probes.append(co + e)
        probes.append(co - e)
    out = track_fn(np.array(probes))
    R = np.empty((6, 6))
    for j in range(6):
        R[:, j] = (out[1 + 2 * j] - out[2 + 2 * j]) / (2 * steps[j])
    return R, out[0]


def closed_orbit(track_fn, guess=None, tol=1e-14, max_iter=20,
                 steps=(1e-10, 1e-10, 1e-10, 1e-10, 1e-9, 1e-9)):
    """Newton iteration on M(x) - x = 0 with the finite-difference matrix."""
    x = np.zeros(6) if guess is None else np.asarray(guess, dtype=np.float64).copy()
    for _ in range(max_iter):
        R, mx = one_turn_matrix(track_fn, x, steps)
        res = mx - x
        if np.max(np.abs(res)) < tol:
            return x
        x = x - np.linalg.solve(R - np.eye(6), res)
    return x


def linear_normal_form(R):
    """W (6x6, symplectic) and the tunes with R = W Rot(q) W^-1.

    The eigenvectors v of R come in conjugate pairs; for each pair the one
    with Im(v^H S v) > 0 is kept, scaled to Im(v^H S v) = 2, and gives
    the columns Re v, Im v. Modes are assigned to the planes (x, y, zeta)
    by the permutation that maximises the product of each mode's amplitude
    in its plane."""
    w, v = np.linalg.eig(R)
    cols = []
    for i in range(6):
        vi = v[:, i]
        sn = np.imag(np.conj(vi) @ S6 @ vi)
        if sn > 0:
            cols.append((vi / np.sqrt(sn / 2.0), w[i]))
    if len(cols) != 3:
        raise ValueError("one-turn matrix is not stable in all three planes")
    # assign modes to planes: the permutation that maximises the product of
    # each mode's amplitude in its plane (robust when x and y are coupled)
    amp = np.array([[np.hypot(abs(vi[2 * k]), abs(vi[2 * k + 1])) for k in range(3)]
                    for vi, _ in cols])
    best, plane_of = -1.0, None
    for perm in itertools.permutations(range(3)):
        score = np.prod([amp[m, perm[m]] for m in range(3)])
        if score > best:
            best, plane_of = score, list(perm)
    W = np.zeros((6, 6))
    tunes = np.zeros(3)
    for (vi, lam), k in zip(cols, plane_of):
        # fix the phase so that the (2k, 2k+1) entries form a lower-triangular block
        phase = np.angle(vi[2 * k])
        vi = vi * np.exp(-1j * phase)
        W[:, 2 * k] = np.real(vi)
        W[:, 2 * k + 1] = np.imag(vi)
        tunes[k] = np.angle(lam) / (2 * np.pi)
    return W, np.mod(tunes, 1.0)


def polar_grid(r_max=20.0, n_r=40, n_angles=11, r_min=None, angle_range=(0.0, np.pi / 2)):
    """(r, theta) of a polar grid in sigma units: n_angles angles spread
    evenly inside angle_range with both ends excluded (so that both planes
    are excited), n_r amplitudes from r_min to r_max."""
    a0, a1 = angle_range
    theta = np.linspace(a0, a1, n_angles + 2)[1:-1]
    r_min = r_max / n_r if r_min is None else r_min
    r = np.linspace(r_min, r_max, n_r)
    rr, tt = np.meshgrid(r, theta, indexing="ij")
    return rr.ravel(), tt.ravel()


def normalized_to_physical(W, co, x_norm, y_norm, nemitt_x, nemitt_y, beta0, gamma0,
                           px_norm=0.0, py_norm=0.0, zeta_norm=0.0, pzeta_norm=0.0, delta=None):
    """Physical (x, px, y, py, zeta, delta) from normalised amplitudes in
    sigma units: z = co + W diag(sqrt(eps)) z_n, eps = nemitt / (beta0 gamma0).
    With ``delta`` given, the delta of every particle is overwritten with
    it after the transformation (off-momentum scans; no dispersive shift is
    added to x)."""
    n = np.broadcast(x_norm, y_norm).shape
    gx = np.sqrt(nemitt_x / (beta0 * gamma0))
    gy = np.sqrt(nemitt_y / (beta0 * gamma0))
    zn = np.zeros((6,) + n)
    zn[0] = np.asarray(x_norm) * gx
    zn[1] = np.asarray(px_norm) * gx
    zn[2] = np.asarray(y_norm) * gy
    zn[3] = np.asarray(py_norm) * gy
    zn[4] = zeta_norm
    zn[5] = pzeta_norm
    z = np.asarray(co).reshape((6,) + (1,) * len(n)) + np.tensordot(W, zn, axes=1)
    if delta is not None:
        z[5] = delta
    return z


def dynamic_aperture(r, theta, state, at_turn, num_turns):
    """Per angle: the smallest amplitude whose particle was lost before
    completing ``num_turns`` turns (r_max of the grid when none was lost).
    Returns (angles, da)."""
    r = np.asarray(r)
    theta = np.asarray(theta)
    lost = (np.asarray(state) <= 0) & (np.asarray(at_turn) < num_turns)
    angles = np.unique(theta)
    da = np.empty(len(angles))
    for k, a in enumerate(angles):
        sel = theta == a
        rl = r[sel & lost]
        da[k] = rl.min() if rl.size else r[sel].max()
    return angles, da


def linear_aperture(co_x, co_y, dx_dz, dy_dz, W, rect, ellipse, deltas, angles, nemitt_x, nemitt_y,
                    beta0, gamma0, r_hi=1000.0, iters=60):
    """Linear aperture in sigma for each (delta, angle) ray: the smallest
    amplitude r at which a particle started at the scan's initial condition
    (``normalized_to_physical`` with x_norm = r cos(angle), y_norm =
    r sin(angle), delta offset added) touches an aperture when its
    transverse normal modes take every phase while its longitudinal mode
    keeps its initial phase (a short scan sees a fraction of a synchrotron
    period).

    co_x, co_y: (n_ap,) closed orbit at the apertures; dx_dz, dy_dz:
    (6, n_ap) derivatives of x and y at the apertures with respect to the
    start coordinates (one turn of offset particles); rect: (n_ap, 4)
    min_x, max_x, min_y, max_y (+-inf where unlimited); ellipse: (n_ap, 2)
    semi-axes a, b (inf where the aperture is not an ellipse). Returns an
    array (len(deltas), len(angles)); r_hi where nothing is touched."""
    W = np.asarray(W, dtype=np.float64)
    Hx = W.T @ np.asarray(dx_dz)          # x at each aperture per normalised coordinate
    Hy = W.T @ np.asarray(dy_dz)
    hxx, hxy = np.hypot(Hx[0], Hx[1]), np.hypot(Hx[2], Hx[3])
    hyx, hyy = np.hypot(Hy[0], Hy[1]), np.hypot(Hy[2], Hy[3])
    rect = np.asarray(rect, dtype=np.float64)
    ell = np.asarray(ellipse, dtype=np.float64)
    gx = np.sqrt(nemitt_x / (beta0 * gamma0))
    gy = np.sqrt(nemitt_y / (beta0 * gamma0))
    Winv = np.linalg.inv(W)
    out = np.empty((len(deltas), len(angles)))

    def touches(r, u, c):
        zn = r * u + c
        ax, ay = np.hypot(zn[0], zn[1]), np.hypot(zn[2], zn[3])
        xc = co_x + Hx[4] * zn[4] + Hx[5] * zn[5]
        yc = co_y + Hy[4] * zn[4] + Hy[5] * zn[5]
        ex = ax * hxx + ay * hxy
        ey = ax * hyx + ay * hyy
        hit = ((xc + ex > rect[:, 1]) | (xc - ex < rect[:, 0]) |
               (yc + ey > rect[:, 3]) | (yc - ey < rect[:, 2]))
        with np.errstate(divide="ignore", invalid="ignore"):
            e = np.square((np.abs(xc) + ex) / ell[:, 0]) + np.square((np.abs(yc) + ey) / ell[:, 1])
        return bool(np.any(hit | (e > 1.0)))

    for d, dl in enumerate(deltas):
        c = Winv @ np.array([0.0, 0.0, 0.0, 0.0, 0.0, float(dl)])
        for a, th in enumerate(angles):
            u = np.array([np.cos(th) * gx, 0.0, np.sin(th) * gy, 0.0, 0.0, 0.0])
            if touches(0.0, u, c):
                out[d, a] = 0.0
                continue
            if not touches(r_hi, u, c):
                out[d, a] = r_hi
                continue
            lo, hi = 0.0, r_hi
            for _ in range(iters):
                mid = 0.5 * (lo + hi)
                if touches(mid, u, c):
                    hi = mid
                else:
                    lo = mid
            out[d, a] = hi
    return out
