"""Helpers shared by the tests: run the same track_line call on the GPU
(through the C-ABI) and on the CPU oracle, and compare the results."""
import ctypes

import numpy as np

import pyoracle
from xtrack_gb300 import _abi

COORDS = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s")
INTS = ("state", "at_turn", "at_element", "particle_id")


def beam_arrays(particles):
    return pyoracle.host_arrays(particles.to_numpy())


def gpu_track(records, arrs, arith="exact", q0=1.0, mass0=938272088.16, t_sim=0.0,
              num_turns=1, ele_start=0, num_ele_track=None, flag_end_turn_actions=1,
              flag_reset_s=1, line_length=0.0, track_flags=0, use_exact_drifts=False,
              cavity_preserve_angle=False, global_xy_limit=1.0, monitor=None,
              flag_monitor=0, num_ele_line=None, compact_every=None, block_size=None,
              chunk_bytes=None, use_graph=None):
    """One xtg_track call on cuda:0 over copies of the host arrays ``arrs``.
    Returns (arrays, monitor_data) as numpy."""
    import torch
    lib = _abi.load_library()
    n = len(records)
    if num_ele_track is None:
        num_ele_track = n - ele_start
    if num_ele_line is None:
        num_ele_line = n
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in arrs.items()}
    ps = _abi.particles_struct_from_ptrs(len(arrs["x"]), q0, mass0, t_sim,
                                         {k: v.data_ptr() for k, v in t.items()})
    cfg = _abi.XtgConfig()
    cfg.use_exact_drifts = int(bool(use_exact_drifts))
    cfg.cavity_preserve_angle = int(bool(cavity_preserve_angle))
    cfg.has_global_xy_limit = 0 if global_xy_limit is None else 1
    cfg.global_xy_limit = 0.0 if global_xy_limit is None else float(global_xy_limit)
    cfg.arith = _abi.ARITH_EXACT if arith == "exact" else _abi.ARITH_FAST
    h = ctypes.c_void_p()
    recs = np.ascontiguousarray(records)
    _abi.check(lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), n, ctypes.byref(cfg),
                                      ctypes.byref(h)))
    try:
        tu = _abi.XtgTuning()
        _abi.check(lib.xtg_get_tuning(h, ctypes.byref(tu)))
        for name, v in (("compact_every", compact_every), ("block_size", block_size),
                        ("chunk_bytes", chunk_bytes), ("use_graph", use_graph)):
            if v is not None:
                setattr(tu, name, int(v))
        _abi.check(lib.xtg_set_tuning(h, ctypes.byref(tu)))
        mst = None
        mdata = None
        if monitor is not None:
            mdata = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
                     for k, v in monitor["data"].items()}
            mst = _abi.XtgMonitor()
            for k in ("start_at_turn", "stop_at_turn", "part_id_start", "part_id_end",
                      "ebe_mode", "n_repetitions", "repetition_period", "n_records"):
                setattr(mst, k, int(monitor[k]))
            mst.data = _abi.particles_struct_from_ptrs(monitor["n_records"], 0., 0., 0.,
                                                       {k: v.data_ptr() for k, v in mdata.items()})
        _abi.check(lib.xtg_track(h, ctypes.byref(ps), num_turns, ele_start, num_ele_track,
                                 flag_end_turn_actions, flag_reset_s, flag_monitor, num_ele_line,
                                 line_length, ctypes.byref(mst) if mst is not None else None,
                                 int(track_flags), None))
        _abi.check(lib.xtg_sync(None))
        _abi.check(lib.xtg_device_status(h))
    finally:
        lib.xtg_lattice_destroy(h)
    out = {k: v.cpu().numpy() for k, v in t.items()}
    mon = {k: v.cpu().numpy() for k, v in mdata.items()} if mdata is not None else None
    return out, mon


def gpu_track_batch(record_sets, arrs, lattice_index, arith="exact", q0=1.0,
                    mass0=938272088.16, num_turns=1, line_length=0.0, global_xy_limit=1.0,
                    compact_every=None, chunk_bytes=None, use_graph=None, block_size=None):
    """One xtg_track_batch call on cuda:0: particle i is tracked through the
    lattice built from ``record_sets[lattice_index[i]]``."""
    import torch
    lib = _abi.load_library()
    n = len(record_sets[0])
    dev = torch.device("cuda:0")
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in arrs.items()}
    idx = torch.from_numpy(np.ascontiguousarray(lattice_index, dtype=np.int32)).to(dev)
    ps = _abi.particles_struct_from_ptrs(len(arrs["x"]), q0, mass0, 0.0,
                                         {k: v.data_ptr() for k, v in t.items()})
    cfg = _abi.XtgConfig()
    cfg.has_global_xy_limit = 0 if global_xy_limit is None else 1
    cfg.global_xy_limit = 0.0 if global_xy_limit is None else float(global_xy_limit)
    cfg.arith = _abi.ARITH_EXACT if arith == "exact" else _abi.ARITH_FAST
    handles = []
    b = ctypes.c_void_p()
    try:
        for recs in record_sets:
            h = ctypes.c_void_p()
            recs = np.ascontiguousarray(recs)
            _abi.check(lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), n,
                                              ctypes.byref(cfg), ctypes.byref(h)))
            handles.append(h)
        arr = (ctypes.c_void_p * len(handles))(*[h.value for h in handles])
        _abi.check(lib.xtg_batch_create(arr, len(handles), ctypes.byref(b)))
        tu = _abi.XtgTuning(block_size=256, compact_every=0, chunk_bytes=49152, use_graph=0)
        for name, v in (("compact_every", compact_every), ("block_size", block_size),
                        ("chunk_bytes", chunk_bytes), ("use_graph", use_graph)):
            if v is not None:
                setattr(tu, name, int(v))
        _abi.check(lib.xtg_batch_set_tuning(b, ctypes.byref(tu)))
        _abi.check(lib.xtg_track_batch(b, ctypes.byref(ps), ctypes.c_void_p(idx.data_ptr()),
                                       num_turns, 0, n, 1, 1, 0, n, line_length, None, 0, None))
        _abi.check(lib.xtg_sync(None))
        _abi.check(lib.xtg_batch_device_status(b))
    finally:
        if b.value:
            lib.xtg_batch_destroy(b)
        for h in handles:
            lib.xtg_lattice_destroy(h)
    return {k: v.cpu().numpy() for k, v in t.items()}


def make_monitor(start, stop, pid_range, fields=("x", "px", "y", "py", "zeta", "delta", "s",
                                                 "at_turn", "at_element", "state", "particle_id"),
                 n_repetitions=1, repetition_period=-1, ebe_mode=0):
    n_rec = (stop - start) * (pid_range[1] - pid_range[0]) * n_repetitions
    data = {}
    for f in fields:
        dt = np.int64 if f in pyoracle.INT_FIELDS else np.float64
        data[f] = np.zeros(n_rec, dtype=dt)
    return dict(start_at_turn=start, stop_at_turn=stop, part_id_start=pid_range[0],
                part_id_end=pid_range[1], ebe_mode=ebe_mode, n_repetitions=n_repetitions,
                repetition_period=repetition_period, n_records=n_rec, data=data)


def rel_err(a, b, field):
    """max |a-b| / max(|b|) over the array (scale-relative error). Equal
    values (infinities of a killed particle included) count as zero error,
    two NaNs as equal; the scale ignores non-finite values and the 1e30 that
    a killed particle's coordinates are set to."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not b.size:
        return 0.0
    fin = np.isfinite(b) & (np.abs(b) < 1e29)
    scale = np.max(np.abs(b[fin])) if fin.any() else 1.0
    if scale == 0:
        scale = 1.0
    same = (a == b) | (np.isnan(a) & np.isnan(b))
    if same.all():
        return 0.0
    return float(np.max(np.abs(a[~same] - b[~same])) / scale)


# Per-particle relative error: |got - ref| / max(|ref|, PP_FLOOR * scale),
# scale = max |ref| of the field over the compared particles. Values below
# a thousandth of the field's scale are measured against that floor, so
# that a coordinate that happens to pass near zero does not report an
# unbounded relative error.
PP_FLOOR = 1e-3


def per_particle_rel_err(a, b):
    """Largest per-particle relative error (see PP_FLOOR) of finite pairs."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fin = np.isfinite(a) & np.isfinite(b) & (np.abs(b) < 1e29)
    if not fin.any():
        return 0.0
    a, b = a[fin], b[fin]
    scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), PP_FLOOR * scale)))


def near_edge_mask(records, arrs, tol=1e-9, **track_kw):
    """Particles (by particle_id, as a mask over the arrays' order) that come
    within ``tol`` metres of an aperture edge in the oracle's run of the
    same call: the particles whose state, at_turn and at_element a last-ulp
    difference of the coordinates could change."""
    d = pyoracle.edge_distance(records, arrs, **track_kw)
    pid = np.asarray(arrs["particle_id"], dtype=np.int64)
    return d[pid] <= tol


def compare(got, ref, coord_tol, fields=COORDS, mask=None, near_edge=None, label=""):
    """Asserts integer fields bit-exact and coordinates within coord_tol
    (scale-relative). With ``near_edge`` (a mask from near_edge_mask), the
    particles whose integer fields differ must all be near-edge ones; they
    are listed and left out of the coordinate comparison. Prints, per
    field, the scale-relative and the per-particle relative error.
    Returns {field: (rel_err, n_bitexact, per_particle_rel_err)}."""
    report = {}
    n = len(ref["x"])
    sel = np.ones(n, dtype=bool) if mask is None else np.asarray(mask, dtype=bool).copy()
    differ = np.zeros(n, dtype=bool)
    for f in INTS:
        if f in ref:
            differ |= np.asarray(got[f]) != np.asarray(ref[f])
    differ &= sel
    if near_edge is not None:
        listed = np.nonzero(differ)[0]
        outside = listed[~near_edge[listed]]
        assert len(outside) == 0, (f"integer fields differ for particles {outside[:10]} that stay "
                                   f"farther than the near-edge tolerance from every aperture")
        print(f"{label} near-edge particles: {int(near_edge[sel].sum())} within tolerance, "
              f"integer mismatches among them: {listed.tolist()}")
        sel &= ~differ
    else:
        for f in INTS:
            if f in ref:
                assert np.array_equal(got[f][sel], ref[f][sel]), f"{f} differs"
    for f in fields:
        e = rel_err(got[f][sel], ref[f][sel], f)
        pp = per_particle_rel_err(got[f][sel], ref[f][sel])
        report[f] = (e, int(np.sum(got[f][sel] == ref[f][sel])), pp)
        assert e <= coord_tol, f"{f}: relative error {e:.3e} > {coord_tol:.1e}"
    print(f"{label} scale-relative / per-particle relative error: " +
          ", ".join(f"{f} {v[0]:.1e}/{v[2]:.1e}" for f, v in report.items()))
    return report


def fma_spread(records, arrs, fields=COORDS, **kw):
    """Per-field scale-relative distance between the oracle compiled without
    and with fused multiply-adds after the same call: the reference's own
    rounding noise for this case. Returns ({field: spread}, mask of particles
    alive in both runs)."""
    a = {k: v.copy() for k, v in arrs.items()}
    b = {k: v.copy() for k, v in arrs.items()}
    pyoracle.track(records, a, which="oracle", **kw)
    pyoracle.track(records, b, which="oracle_fma", **kw)
    ok = (a["state"] > 0) & (b["state"] > 0)
    return {f: rel_err(b[f][ok], a[f][ok], f) for f in fields}, ok


def compare_within_spread(got, ref, spread, mask, factor=3.0, floor=1e-15, fields=COORDS):
    """Coordinates of ``got`` within ``factor`` x the reference's own FMA
    spread of ``ref`` (scale-relative, per field)."""
    out = {}
    for f in fields:
        e = rel_err(got[f][mask], ref[f][mask], f)
        lim = factor * spread[f] + floor
        out[f] = (e, lim)
        assert e <= lim, f"{f}: {e:.3e} > {factor} x reference FMA spread {spread[f]:.3e}"
    return out
