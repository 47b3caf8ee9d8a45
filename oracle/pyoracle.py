"""Python bindings of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the checker / timed baseline; no
product code path imports it.

Two CPU libraries share one calling convention (raw element records of
include/xtrack_gb300.h and host particle arrays):
  * ``libxtg_oracle.so``   the C restatement of the reference (xtg_oracle.c),
                           built everywhere by ``make -C oracle``;
  * ``_ref/libxtref*.so``  the reference's own element C code compiled with
                           stand-in xobjects headers (``make -C oracle ref``),
                           available only where the reference sources are.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "libxtg_oracle.so")
ORACLE_FMA_LIB = os.path.join(HERE, "libxtg_oracle_fma.so")
REF_LIBS = {
    "default": os.path.join(HERE, "_ref", "libxtref.so"),
    "exact_drifts": os.path.join(HERE, "_ref", "libxtref_exact.so"),
    "preserve_angle": os.path.join(HERE, "_ref", "libxtref_preserve.so"),
    "frozen": os.path.join(HERE, "_ref", "libxtref_frozen.so"),
}
FLAG_FREEZE_LONGITUDINAL = 32

MODE_PER_PARTICLE = 0
MODE_OPENMP = 1

_XTG_MAX_KNL = 21
_KNL = ctypes.c_double * _XTG_MAX_KNL
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int64)

DOUBLE_FIELDS = ("p0c", "gamma0", "beta0", "s", "zeta", "x", "y", "px", "py", "ptau",
                 "delta", "rpp", "rvv", "chi", "charge_ratio", "weight", "ax", "ay")
INT_FIELDS = ("pdg_id", "particle_id", "at_element", "at_turn", "state", "parent_particle_id")


class _Particles(ctypes.Structure):
    _fields_ = ([("capacity", ctypes.c_int64), ("q0", ctypes.c_double),
                 ("mass0", ctypes.c_double), ("t_sim", ctypes.c_double)]
                + [(f, _DP) for f in DOUBLE_FIELDS] + [(f, _IP) for f in INT_FIELDS])


class _Monitor(ctypes.Structure):
    _fields_ = [("start_at_turn", ctypes.c_int64), ("stop_at_turn", ctypes.c_int64),
                ("part_id_start", ctypes.c_int64), ("part_id_end", ctypes.c_int64),
                ("ebe_mode", ctypes.c_int64), ("n_repetitions", ctypes.c_int64),
                ("repetition_period", ctypes.c_int64), ("n_records", ctypes.c_int64),
                ("data", _Particles)]


class _Config(ctypes.Structure):
    _fields_ = [("use_exact_drifts", ctypes.c_int32), ("cavity_preserve_angle", ctypes.c_int32),
                ("has_global_xy_limit", ctypes.c_int32), ("arith", ctypes.c_int32),
                ("global_xy_limit", ctypes.c_double)]


def ensure_built(with_ref=True):
    """Builds the oracle libraries if they are missing."""
    need = not os.path.exists(ORACLE_LIB) or not os.path.exists(ORACLE_FMA_LIB)
    if with_ref:
        need = need or not os.path.exists(REF_LIBS["default"])
    if need:
        targets = ["all", "ref"] if with_ref else ["all"]
        # the xtrack sources: XTG_REFERENCE_SRC, else "reference" beside the repository
        ref = os.environ.get("XTG_REFERENCE_SRC") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                  "reference")
        subprocess.run(["make", "-C", HERE] + targets + [f"REF={ref}"], check=True, capture_output=True)


def ref_available():
    return all(os.path.exists(p) for p in REF_LIBS.values())


_libs = {}


def _load(path, kind):
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    if kind == "oracle":
        lib.xto_track.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(_Config),
                                  ctypes.POINTER(_Particles), ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_double, ctypes.POINTER(_Monitor),
                                  ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32]
        lib.xto_track.restype = ctypes.c_int32
        lib.xto_validate.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64]
        lib.xto_validate.restype = ctypes.c_int32
        lib.xto_max_threads.restype = ctypes.c_int32
    else:
        lib.xtr_track.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(_Config),
                                  ctypes.POINTER(_Particles), ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_double, ctypes.c_uint64]
        lib.xtr_track.restype = ctypes.c_int32
    _libs[path] = lib
    return lib


def _pstruct(arrs, q0, mass0, t_sim, capacity=None):
    st = _Particles()
    st.capacity = len(arrs["x"]) if capacity is None else int(capacity)
    st.q0, st.mass0, st.t_sim = q0, mass0, t_sim
    for f in DOUBLE_FIELDS:
        a = arrs.get(f)
        setattr(st, f, a.ctypes.data_as(_DP) if a is not None else ctypes.cast(None, _DP))
    for f in INT_FIELDS:
        a = arrs.get(f)
        setattr(st, f, a.ctypes.data_as(_IP) if a is not None else ctypes.cast(None, _IP))
    return st


def _config(use_exact_drifts=False, cavity_preserve_angle=False, global_xy_limit=1.0):
    c = _Config()
    c.use_exact_drifts = 1 if use_exact_drifts else 0
    c.cavity_preserve_angle = 1 if cavity_preserve_angle else 0
    c.has_global_xy_limit = 0 if global_xy_limit is None else 1
    c.global_xy_limit = 0.0 if global_xy_limit is None else float(global_xy_limit)
    return c


def host_arrays(particles_dict):
    """Contiguous float64/int64 copies of the fields the oracle reads."""
    out = {}
    for f in DOUBLE_FIELDS:
        out[f] = np.ascontiguousarray(np.array(particles_dict[f], dtype=np.float64))
    for f in INT_FIELDS:
        out[f] = np.ascontiguousarray(np.array(particles_dict[f], dtype=np.int64))
    return out


def track(records, arrs, q0=1.0, mass0=938272088.16, t_sim=0.0, num_turns=1, ele_start=0,
          num_ele_track=None, flag_end_turn_actions=1, flag_reset_s=1, line_length=0.0,
          track_flags=0, use_exact_drifts=False, cavity_preserve_angle=False,
          global_xy_limit=1.0, monitor=None, flag_monitor=0, mode=MODE_PER_PARTICLE,
          num_threads=0, num_ele_line=None, which="oracle", freeze_longitudinal=False):
    """Runs one track_line call in place on host arrays ``arrs``.

    which='oracle'     -> C restatement (no contraction: the reference's CPU
                          arithmetic);
    which='oracle_fma' -> the same source compiled with fused multiply-adds
                          (the reference's arithmetic as its CUDA build
                          rounds it);
    which='ref'        -> reference-compiled code (no monitor, no OpenMP mode).

    freeze_longitudinal: the oracle sets its freeze flag; the reference
    build with the FREEZE_VAR_<name> set of freeze_longitudinal is used."""
    records = np.ascontiguousarray(records)
    n = len(records)
    if num_ele_track is None:
        num_ele_track = n - ele_start
    if num_ele_line is None:
        num_ele_line = n
    cfg = _config(use_exact_drifts, cavity_preserve_angle, global_xy_limit)
    ps = _pstruct(arrs, q0, mass0, t_sim)
    if freeze_longitudinal and which in ("oracle", "oracle_fma"):
        track_flags = int(track_flags) | (1 << FLAG_FREEZE_LONGITUDINAL)
    if which in ("oracle", "oracle_fma"):
        ensure_built(with_ref=False)
        lib = _load(ORACLE_LIB if which == "oracle" else ORACLE_FMA_LIB, "oracle")
        mst = None
        if monitor is not None:
            mst = _Monitor()
            for k in ("start_at_turn", "stop_at_turn", "part_id_start", "part_id_end", "ebe_mode",
                      "n_repetitions", "repetition_period", "n_records"):
                setattr(mst, k, int(monitor[k]))
            mst.data = _pstruct(monitor["data"], 0.0, 0.0, 0.0, capacity=monitor["n_records"])
        st = lib.xto_track(records.ctypes.data, n, ctypes.byref(cfg), ctypes.byref(ps),
                           num_turns, ele_start, num_ele_track, flag_end_turn_actions,
                           flag_reset_s, flag_monitor, num_ele_line, line_length,
                           ctypes.byref(mst) if mst is not None else None,
                           int(track_flags), mode, num_threads)
    else:
        if freeze_longitudinal:
            if use_exact_drifts or cavity_preserve_angle:
                raise ValueError("no reference build freezes with another config switch")
            path = REF_LIBS["frozen"]
        elif use_exact_drifts:
            path = REF_LIBS["exact_drifts"]
        elif cavity_preserve_angle:
            path = REF_LIBS["preserve_angle"]
        else:
            path = REF_LIBS["default"]
        if not os.path.exists(path):
            raise RuntimeError("reference-compiled oracle not built (make -C oracle ref)")
        if monitor is not None or flag_monitor:
            raise ValueError("the reference-compiled oracle has no monitor")
        lib = _load(path, "ref")
        st = lib.xtr_track(records.ctypes.data, n, ctypes.byref(cfg), ctypes.byref(ps),
                           num_turns, ele_start, num_ele_track, flag_end_turn_actions,
                           flag_reset_s, num_ele_line, line_length, int(track_flags))
    if st != 0:
        raise RuntimeError(f"oracle returned status {st}")
    return arrs


class _MultiMon(ctypes.Structure):
    _fields_ = [("start_at_turn", ctypes.c_int64), ("stop_at_turn", ctypes.c_int64),
                ("part_id_start", ctypes.c_int64), ("part_id_end", ctypes.c_int64),
                ("mapping_len", ctypes.c_int64), ("n_obs", ctypes.c_int64),
                ("at_element_mapping", ctypes.c_void_p), ("data", ctypes.c_void_p)]


def set_multi_element_monitor(mapping, data, start_at_turn, stop_at_turn, part_id_start,
                              part_id_end, which="oracle"):
    """Multi-element monitor for the following track() calls of the oracle
    (host numpy buffers: int64 mapping, float64 data of shape
    (turns, particles, 7, n_obs)); mapping=None clears it."""
    lib = _load(ORACLE_LIB if which == "oracle" else ORACLE_FMA_LIB, "oracle")
    lib.xto_set_multi_element_monitor.argtypes = [ctypes.POINTER(_MultiMon)]
    if mapping is None:
        lib.xto_set_multi_element_monitor(None)
        return
    m = _MultiMon(start_at_turn, stop_at_turn, part_id_start, part_id_end, len(mapping),
                  data.shape[-1], mapping.ctypes.data, data.ctypes.data)
    lib.xto_set_multi_element_monitor(ctypes.byref(m))


def edge_distance(records, arrs, **track_kw):
    """Tracks a copy of ``arrs`` through the oracle and returns, per
    particle_id (0 .. n-1), the smallest distance in metres to the edge of
    any aperture the particle reached (+inf: it reached none)."""
    lib = _load(ORACLE_LIB, "oracle")
    lib.xto_set_edge_distance.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    n = len(arrs["x"])
    out = np.full(n, np.inf)
    lib.xto_set_edge_distance(out.ctypes.data, n)
    try:
        track(records, {k: v.copy() for k, v in arrs.items()}, which="oracle", **track_kw)
    finally:
        lib.xto_set_edge_distance(None, 0)
    return out


def validate(records):
    ensure_built(with_ref=False)
    lib = _load(ORACLE_LIB, "oracle")
    buf = ctypes.create_string_buffer(256)
    records = np.ascontiguousarray(records)
    st = lib.xto_validate(records.ctypes.data, len(records), buf, 256)
    return st, buf.value.decode()


def max_threads():
    ensure_built(with_ref=False)
    return _load(ORACLE_LIB, "oracle").xto_max_threads()
