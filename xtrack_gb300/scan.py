"""Batched dynamic-aperture scans over error seeds.

A scan places, for each seed, particles on a polar grid of normalised
amplitude (in beam sigmas) x angle x momentum offset, converts them to
physical coordinates with that seed's closed orbit and linear normal form,
and tracks all seeds at once with a ``BatchTracker`` (one persistent
launch, per-particle lattice index). The outcome per particle is its
``state``, ``at_turn`` and ``at_element``; the DA per seed, angle and
momentum offset is the smallest lost amplitude (``da.dynamic_aperture``).
"""
import numpy as np
import torch

from . import da
from .batch import BatchTracker
from .particles import Particles


class Scan:
    """Initial conditions of a multi-seed scan (host arrays)."""

    def __init__(self):
        self.coords = None        # (6, n) physical x, px, y, py, zeta, delta
        self.lattice_index = None  # (n,) int32
        self.r = None             # amplitude in sigma
        self.theta = None
        self.delta_index = None   # index into deltas
        self.deltas = None
        self.seed_features = None  # (n_seeds, k)
        self.tunes = None
        self.co_extremes = None   # (n_seeds, 4): max x, min x, max y, min y of the orbit

    @property
    def n(self):
        return len(self.r)


def seed_normal_form(tracker, particle_ref_kwargs, device="cuda"):
    fn = da.line_track_fn(tracker, particle_ref_kwargs, device=device)
    co = da.closed_orbit(fn)
    R, _ = da.one_turn_matrix(fn, co)
    W, tunes = da.linear_normal_form(R)
    return co, W, tunes


def closed_orbit_extremes(tracker, co, particle_ref_kwargs, device="cuda"):
    """Largest and smallest x and y of the closed orbit over the ring's
    elements [m], from one element-by-element turn of the closed-orbit
    particle (ONE_TURN_EBE monitor)."""
    p = Particles(device=device, x=[co[0]], px=[co[1]], y=[co[2]], py=[co[3]], zeta=[co[4]],
                  delta=[co[5]], **particle_ref_kwargs)
    tracker._track(p, num_turns=1, turn_by_turn_monitor="ONE_TURN_EBE")
    mon = tracker.record_last_track
    x = np.asarray(mon.x).ravel()
    y = np.asarray(mon.y).ravel()
    return np.array([x.max(), x.min(), y.max(), y.min()])


def build_scan(lines, counts, r_max=20.0, n_angles=11, deltas=(0.0, 2.7e-4), nemitt=2.5e-6,
               seed=0, device="cuda", arith="fast", features=None):
    """Initial conditions for ``lines`` (one per seed) with ``counts[s]``
    particles for seed s, spread over n_angles x len(deltas) rays with
    amplitudes uniform in (0, r_max] on each ray."""
    ref = lines[0].particle_ref
    ref_kw = dict(p0c=float(ref.p0c[0]), mass0=float(ref.mass0), q0=float(ref.q0))
    beta0 = float(ref.beta0[0])
    gamma0 = float(ref.gamma0[0])
    theta_rays = np.linspace(0.0, np.pi / 2, n_angles + 2)[1:-1]
    out = Scan()
    out.deltas = np.asarray(deltas, dtype=np.float64)
    parts = {k: [] for k in ("coords", "lat", "r", "theta", "di")}
    tunes = []
    co_ext = []
    for s, line in enumerate(lines):
        tr = line.build_tracker(device=device, arith=arith)
        co, W, q = seed_normal_form(tr, ref_kw, device=device)
        tunes.append(q)
        co_ext.append(closed_orbit_extremes(tr, co, ref_kw, device=device))
        n_rays = n_angles * len(deltas)
        per_ray = max(1, int(counts[s]) // n_rays)
        r = np.tile(np.linspace(r_max / per_ray, r_max, per_ray), n_rays)
        th = np.repeat(np.tile(theta_rays, len(deltas)), per_ray)
        di = np.repeat(np.repeat(np.arange(len(deltas)), n_angles), per_ray)
        z = da.normalized_to_physical(W, co, r * np.cos(th), r * np.sin(th), nemitt, nemitt,
                                      beta0, gamma0)
        z[5] = co[5] + out.deltas[di]
        parts["coords"].append(z)
        parts["lat"].append(np.full(len(r), s, dtype=np.int32))
        parts["r"].append(r)
        parts["theta"].append(th)
        parts["di"].append(di)
    out.coords = np.concatenate(parts["coords"], axis=1)
    out.lattice_index = np.concatenate(parts["lat"])
    out.r = np.concatenate(parts["r"])
    out.theta = np.concatenate(parts["theta"])
    out.delta_index = np.concatenate(parts["di"])
    out.tunes = np.array(tunes)
    out.co_extremes = np.array(co_ext)
    out.ref_kw = ref_kw
    if features is not None:
        out.seed_features = np.stack([features(line) for line in lines])
    return out


def make_particles(scan, select=None, device="cuda"):
    sel = slice(None) if select is None else select
    kw = {f: scan.coords[k][sel] for k, f in enumerate(da.COORDS)}
    return Particles(device=device, **scan.ref_kw, **kw)


def run_scan(tracker, scan, num_turns, select=None, device="cuda"):
    """Tracks the scan's particles (all, or the boolean ``select``) through
    ``tracker`` (a BatchTracker over the scan's lines). Returns host arrays
    (state, at_turn, at_element) in scan order of the selected particles."""
    p = make_particles(scan, select, device=device)
    lat = scan.lattice_index if select is None else scan.lattice_index[select]
    tracker.track(p, lattice_index=lat, num_turns=num_turns)
    return (p.state.cpu().numpy(), p.at_turn.cpu().numpy(), p.at_element.cpu().numpy())


def da_table(scan, survive, n_seeds):
    """DA (sigma) per seed, momentum offset and angle from a survival map:
    array (n_seeds, n_deltas, n_angles)."""
    angles = np.unique(scan.theta)
    out = np.zeros((n_seeds, len(scan.deltas), len(angles)))
    lost = ~np.asarray(survive, dtype=bool)
    for s in range(n_seeds):
        for d in range(len(scan.deltas)):
            sel = (scan.lattice_index == s) & (scan.delta_index == d)
            for k, a in enumerate(angles):
                m = sel & (scan.theta == a)
                rl = scan.r[m & lost]
                out[s, d, k] = rl.min() if rl.size else scan.r[m].max()
    return out
