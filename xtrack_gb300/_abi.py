"""ctypes mirror of include/xtrack_gb300.h and the loader of the CUDA library.

The structures below follow the C declarations field by field; a numpy
dtype of the element record is derived from the ctypes structure so that a
whole lattice can be filled as one structured array and handed to the
library without per-element Python calls.

The library is built in-tree (see ``xtrack_gb300._build``). Loading it never
falls back to anything: if the shared object is missing or fails to load,
``load_library`` raises.
"""
import ctypes
import os

import numpy as np

XTG_MAX_KNL = 21
XTG_NOALLOC_MAX_PARTICLES = 1048576

XTG_OK = 0
XTG_E_NULL = -1
XTG_E_VALUE = -2
XTG_E_UNSUPPORTED = -3
XTG_E_CUDA = -4
XTG_E_CAPACITY = -5
XTG_E_TIMEOUT = -6
XTG_E_NOMEM = -7

# element classes (xtrack/beam_elements)
CLS_MARKER = 0
CLS_DRIFT = 1
CLS_MULTIPOLE = 2
CLS_BEND = 3
CLS_QUADRUPOLE = 4
CLS_SEXTUPOLE = 5
CLS_OCTUPOLE = 6
CLS_CAVITY = 7
CLS_LIMIT_ELLIPSE = 8
CLS_LIMIT_RECT = 9
CLS_MONITOR = 10
CLS_LIMIT_POLYGON = 11
CLS_DIPOLE_EDGE = 12
CLS_LIMIT_RECT_ELLIPSE = 13

SLICE_NONE = 0
SLICE_THICK = 1
SLICE_THIN = 2
SLICE_DRIFT = 3
SLICE_ENTRY = 4
SLICE_EXIT = 5

FLAG_BACKTRACK = 0
FLAG_KILL_CAVITY_KICK = 2
FLAG_IGNORE_GLOBAL_APERTURE = 3
FLAG_IGNORE_LOCAL_APERTURE = 4
FLAG_FREEZE_LONGITUDINAL = 32

ARITH_EXACT = 0
ARITH_FAST = 1

_KNL = ctypes.c_double * XTG_MAX_KNL


class XtgElement(ctypes.Structure):
    _fields_ = [
        ("cls", ctypes.c_int32),
        ("slice", ctypes.c_int32),
        ("model", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("num_multipole_kicks", ctypes.c_int64),
        ("order", ctypes.c_int64),
        ("order_rel", ctypes.c_int64),
        ("isthick", ctypes.c_int32),
        ("main_is_skew", ctypes.c_int32),
        ("main_order", ctypes.c_int32),
        ("edge_entry_active", ctypes.c_int32),
        ("edge_exit_active", ctypes.c_int32),
        ("edge_entry_model", ctypes.c_int32),
        ("edge_exit_model", ctypes.c_int32),
        ("absolute_time", ctypes.c_int32),
        ("weight", ctypes.c_double),
        ("length", ctypes.c_double),
        ("h", ctypes.c_double),
        ("hxl", ctypes.c_double),
        ("k0", ctypes.c_double), ("k1", ctypes.c_double),
        ("k2", ctypes.c_double), ("k3", ctypes.c_double),
        ("k0s", ctypes.c_double), ("k1s", ctypes.c_double),
        ("k2s", ctypes.c_double), ("k3s", ctypes.c_double),
        ("inv_factorial_order", ctypes.c_double),
        ("knl", _KNL), ("ksl", _KNL), ("knl_rel", _KNL), ("ksl_rel", _KNL),
        ("edge_entry_angle", ctypes.c_double), ("edge_exit_angle", ctypes.c_double),
        ("edge_entry_angle_fdown", ctypes.c_double), ("edge_exit_angle_fdown", ctypes.c_double),
        ("edge_entry_fint", ctypes.c_double), ("edge_exit_fint", ctypes.c_double),
        ("edge_entry_hgap", ctypes.c_double), ("edge_exit_hgap", ctypes.c_double),
        ("voltage", ctypes.c_double), ("frequency", ctypes.c_double),
        ("harmonic", ctypes.c_double), ("lag", ctypes.c_double), ("phase", ctypes.c_double),
        ("a_squ", ctypes.c_double), ("b_squ", ctypes.c_double), ("a_b_squ", ctypes.c_double),
        ("min_x", ctypes.c_double), ("max_x", ctypes.c_double),
        ("min_y", ctypes.c_double), ("max_y", ctypes.c_double),
        ("shift_x", ctypes.c_double), ("shift_y", ctypes.c_double), ("shift_s", ctypes.c_double),
        ("rot_x_rad", ctypes.c_double), ("rot_y_rad", ctypes.c_double),
        ("rot_s_rad", ctypes.c_double), ("rot_s_rad_no_frame", ctypes.c_double),
        ("aux", ctypes.c_uint64),
        ("k", ctypes.c_double), ("e1", ctypes.c_double), ("hgap", ctypes.c_double),
        ("fint", ctypes.c_double), ("r21", ctypes.c_double), ("r43", ctypes.c_double),
        ("side", ctypes.c_int32), ("reserved_dipole_edge", ctypes.c_int32),
    ]


ELEMENT_DTYPE = np.dtype(XtgElement)

_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int64)

PARTICLE_DOUBLE_FIELDS = (
    "p0c", "gamma0", "beta0", "s", "zeta", "x", "y", "px", "py",
    "ptau", "delta", "rpp", "rvv", "chi", "charge_ratio", "weight", "ax", "ay")
PARTICLE_INT_FIELDS = (
    "pdg_id", "particle_id", "at_element", "at_turn", "state", "parent_particle_id")


class XtgParticles(ctypes.Structure):
    _fields_ = [
        ("capacity", ctypes.c_int64),
        ("q0", ctypes.c_double), ("mass0", ctypes.c_double), ("t_sim", ctypes.c_double),
        ("p0c", _DP), ("gamma0", _DP), ("beta0", _DP),
        ("s", _DP), ("zeta", _DP), ("x", _DP), ("y", _DP), ("px", _DP), ("py", _DP),
        ("ptau", _DP), ("delta", _DP), ("rpp", _DP), ("rvv", _DP),
        ("chi", _DP), ("charge_ratio", _DP), ("weight", _DP),
        ("ax", _DP), ("ay", _DP),
        ("pdg_id", _IP), ("particle_id", _IP), ("at_element", _IP), ("at_turn", _IP),
        ("state", _IP), ("parent_particle_id", _IP),
    ]


class XtgMonitor(ctypes.Structure):
    _fields_ = [
        ("start_at_turn", ctypes.c_int64), ("stop_at_turn", ctypes.c_int64),
        ("part_id_start", ctypes.c_int64), ("part_id_end", ctypes.c_int64),
        ("ebe_mode", ctypes.c_int64),
        ("n_repetitions", ctypes.c_int64), ("repetition_period", ctypes.c_int64),
        ("n_records", ctypes.c_int64),
        ("data", XtgParticles),
    ]


class XtgPolygon(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_int64), ("x_vertices", ctypes.c_void_p),
                ("y_vertices", ctypes.c_void_p)]


MON_PARTICLES = 1
MON_LAST_TURNS = 2
MON_BEAM_POSITION = 3
MON_BEAM_SIZE = 4
MON_BEAM_PROFILE = 5


class XtgElementMonitor(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("particle_id_start", ctypes.c_int64), ("num_particles", ctypes.c_int64),
        ("n_last_turns", ctypes.c_int64), ("every_n_turns", ctypes.c_int64),
        ("start_at_turn", ctypes.c_int64), ("n_slots", ctypes.c_int64),
        ("frev", ctypes.c_double), ("sampling_frequency", ctypes.c_double),
        ("lost_at_offset", ctypes.c_void_p), ("lt_particle_id", ctypes.c_void_p),
        ("lt_at_turn", ctypes.c_void_p),
        ("lt_x", ctypes.c_void_p), ("lt_px", ctypes.c_void_p), ("lt_y", ctypes.c_void_p),
        ("lt_py", ctypes.c_void_p), ("lt_delta", ctypes.c_void_p), ("lt_zeta", ctypes.c_void_p),
        ("count", ctypes.c_void_p), ("x_sum", ctypes.c_void_p), ("y_sum", ctypes.c_void_p),
        ("x2_sum", ctypes.c_void_p), ("y2_sum", ctypes.c_void_p),
        ("nx", ctypes.c_int64), ("ny", ctypes.c_int64),
        ("x_min", ctypes.c_double), ("dx", ctypes.c_double),
        ("y_min", ctypes.c_double), ("dy", ctypes.c_double),
        ("counts_x", ctypes.c_void_p), ("counts_y", ctypes.c_void_p),
        ("particles", XtgMonitor),
    ]


class XtgMultiElementMonitor(ctypes.Structure):
    _fields_ = [
        ("start_at_turn", ctypes.c_int64), ("stop_at_turn", ctypes.c_int64),
        ("part_id_start", ctypes.c_int64), ("part_id_end", ctypes.c_int64),
        ("mapping_len", ctypes.c_int64), ("n_obs", ctypes.c_int64),
        ("at_element_mapping", ctypes.c_void_p), ("data", ctypes.c_void_p),
    ]


class XtgTuning(ctypes.Structure):
    _fields_ = [
        ("block_size", ctypes.c_int32),
        ("compact_every", ctypes.c_int32),
        ("chunk_bytes", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
    ]


class XtgConfig(ctypes.Structure):
    _fields_ = [
        ("use_exact_drifts", ctypes.c_int32),
        ("cavity_preserve_angle", ctypes.c_int32),
        ("has_global_xy_limit", ctypes.c_int32),
        ("arith", ctypes.c_int32),
        ("global_xy_limit", ctypes.c_double),
    ]


def particles_struct_from_ptrs(capacity, q0, mass0, t_sim, ptrs):
    """Fills an XtgParticles from a dict name -> integer address (0 = NULL)."""
    st = XtgParticles()
    st.capacity = int(capacity)
    st.q0 = float(q0)
    st.mass0 = float(mass0)
    st.t_sim = float(t_sim)
    for name in PARTICLE_DOUBLE_FIELDS:
        setattr(st, name, ctypes.cast(ctypes.c_void_p(ptrs.get(name, 0) or None), _DP))
    for name in PARTICLE_INT_FIELDS:
        setattr(st, name, ctypes.cast(ctypes.c_void_p(ptrs.get(name, 0) or None), _IP))
    return st


_PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG_DIR, "libxtrack_gb300.so")

EXPORTED_SYMBOLS = (
    "xtg_abi_version", "xtg_get_last_error", "xtg_lattice_create", "xtg_lattice_destroy",
    "xtg_lattice_info", "xtg_track", "xtg_track_noalloc", "xtg_set_multi_element_monitor",
    "xtg_get_tuning", "xtg_set_tuning", "xtg_device_status",
    "xtg_batch_create", "xtg_batch_destroy", "xtg_batch_get_tuning", "xtg_batch_set_tuning", "xtg_batch_device_status",
    "xtg_track_batch", "xtg_sync", "xtg_launch_count", "xtg_measure_fp64_peak",
    "xtg_check_bounded_wait", "xtg_f64_mul_host", "xtg_f64_mul_device", "xtg_measure_emul_rate",
    "xtg_mlp_gemm", "xtg_mlp_act_backward", "xtg_mlp_colsum", "xtg_mlp_loss", "xtg_mlp_adam",
    "xtg_mlp_to_bf16", "xtg_mlp_device_status", "xtg_mlp_check_bounded_wait",
    "xtg_mlp_get_last_error",
)

MLP_ACT_NONE = 0
MLP_ACT_GELU = 1

_lib = None


def load_library(path=None):
    """Loads the CUDA library and declares its prototypes. Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(
            f"xtrack_gb300: CUDA library not found at {path}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m xtrack_gb300._build`.")
    lib = ctypes.CDLL(path)
    c = ctypes
    lib.xtg_abi_version.restype = c.c_int32
    lib.xtg_get_last_error.argtypes = [c.c_char_p, c.c_int64]
    lib.xtg_get_last_error.restype = c.c_int32
    lib.xtg_lattice_create.argtypes = [c.c_void_p, c.c_int64, c.POINTER(XtgConfig), c.POINTER(c.c_void_p)]
    lib.xtg_lattice_create.restype = c.c_int32
    lib.xtg_lattice_destroy.argtypes = [c.c_void_p]
    lib.xtg_lattice_destroy.restype = c.c_int32
    lib.xtg_lattice_info.argtypes = [c.c_void_p, c.POINTER(c.c_int64), c.c_int64, c.c_int64,
                                     c.POINTER(c.c_double)]
    lib.xtg_lattice_info.restype = c.c_int32
    lib.xtg_track.argtypes = [c.c_void_p, c.POINTER(XtgParticles), c.c_int32, c.c_int32, c.c_int32,
                              c.c_int32, c.c_int32, c.c_int32, c.c_int32, c.c_double,
                              c.POINTER(XtgMonitor), c.c_uint64, c.c_void_p]
    lib.xtg_track.restype = c.c_int32
    lib.xtg_track_noalloc.argtypes = lib.xtg_track.argtypes
    lib.xtg_track_noalloc.restype = c.c_int32
    lib.xtg_set_multi_element_monitor.argtypes = [c.c_void_p, c.POINTER(XtgMultiElementMonitor)]
    lib.xtg_set_multi_element_monitor.restype = c.c_int32
    lib.xtg_get_tuning.argtypes = [c.c_void_p, c.POINTER(XtgTuning)]
    lib.xtg_get_tuning.restype = c.c_int32
    lib.xtg_set_tuning.argtypes = [c.c_void_p, c.POINTER(XtgTuning)]
    lib.xtg_set_tuning.restype = c.c_int32
    lib.xtg_device_status.argtypes = [c.c_void_p]
    lib.xtg_device_status.restype = c.c_int32
    lib.xtg_batch_create.argtypes = [c.POINTER(c.c_void_p), c.c_int32, c.POINTER(c.c_void_p)]
    lib.xtg_batch_create.restype = c.c_int32
    lib.xtg_batch_destroy.argtypes = [c.c_void_p]
    lib.xtg_batch_destroy.restype = c.c_int32
    lib.xtg_batch_get_tuning.argtypes = [c.c_void_p, c.POINTER(XtgTuning)]
    lib.xtg_batch_get_tuning.restype = c.c_int32
    lib.xtg_batch_set_tuning.argtypes = [c.c_void_p, c.POINTER(XtgTuning)]
    lib.xtg_batch_set_tuning.restype = c.c_int32
    lib.xtg_batch_device_status.argtypes = [c.c_void_p]
    lib.xtg_batch_device_status.restype = c.c_int32
    lib.xtg_track_batch.argtypes = [c.c_void_p, c.POINTER(XtgParticles), c.c_void_p, c.c_int32,
                                    c.c_int32, c.c_int32, c.c_int32, c.c_int32, c.c_int32, c.c_int32,
                                    c.c_double, c.POINTER(XtgMonitor), c.c_uint64, c.c_void_p]
    lib.xtg_track_batch.restype = c.c_int32
    vp, i64, i32, f32 = c.c_void_p, c.c_int64, c.c_int32, c.c_float
    lib.xtg_mlp_gemm.argtypes = [vp, i64, i64, vp, i64, i64, i32, i32, i32, vp, i32, vp, i64,
                                 vp, i64, vp, i64, i32, vp]
    lib.xtg_mlp_gemm.restype = i32
    lib.xtg_mlp_act_backward.argtypes = [vp, vp, i64, i32, vp, vp, vp]
    lib.xtg_mlp_act_backward.restype = i32
    lib.xtg_mlp_colsum.argtypes = [vp, i64, i32, i64, vp, i32, vp]
    lib.xtg_mlp_colsum.restype = i32
    lib.xtg_mlp_loss.argtypes = [vp, i64, vp, vp, i64, f32, vp, vp, vp, vp]
    lib.xtg_mlp_loss.restype = i32
    lib.xtg_mlp_adam.argtypes = [vp, vp, vp, vp, vp, i64, f32, f32, f32, f32, f32, i64, vp]
    lib.xtg_mlp_adam.restype = i32
    lib.xtg_mlp_to_bf16.argtypes = [vp, i64, vp, vp]
    lib.xtg_mlp_to_bf16.restype = i32
    lib.xtg_mlp_device_status.argtypes = []
    lib.xtg_mlp_device_status.restype = i32
    lib.xtg_mlp_check_bounded_wait.argtypes = [i64]
    lib.xtg_mlp_check_bounded_wait.restype = i32
    lib.xtg_mlp_get_last_error.argtypes = [c.c_char_p, i64]
    lib.xtg_mlp_get_last_error.restype = i32
    lib.xtg_sync.argtypes = [c.c_void_p]
    lib.xtg_sync.restype = c.c_int32
    lib.xtg_launch_count.restype = c.c_int64
    lib.xtg_measure_fp64_peak.argtypes = [c.POINTER(c.c_double)]
    lib.xtg_measure_fp64_peak.restype = c.c_int32
    lib.xtg_check_bounded_wait.argtypes = [c.c_int64]
    lib.xtg_check_bounded_wait.restype = c.c_int32
    lib.xtg_f64_mul_host.argtypes = [c.c_void_p, c.c_void_p, c.c_void_p, c.c_int64]
    lib.xtg_f64_mul_host.restype = c.c_int32
    lib.xtg_f64_mul_device.argtypes = [c.c_void_p, c.c_void_p, c.c_void_p, c.c_int64, c.c_void_p]
    lib.xtg_f64_mul_device.restype = c.c_int32
    lib.xtg_measure_emul_rate.argtypes = [c.POINTER(c.c_double)]
    lib.xtg_measure_emul_rate.restype = c.c_int32
    if lib.xtg_abi_version() != 3:
        raise RuntimeError("xtrack_gb300: ABI version mismatch")
    if path == LIB_PATH:
        _lib = lib
    return lib


def last_error(lib=None):
    lib = lib or load_library()
    buf = ctypes.create_string_buffer(1024)
    lib.xtg_get_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class XtgError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"xtrack_gb300 error {code}: {message}")
        self.code = code


def check(status, lib=None):
    if status != XTG_OK:
        raise XtgError(status, last_error(lib))
    return status


def check_mlp(status, lib=None):
    """``check`` for the xtg_mlp_* entry points (their own error slot)."""
    if status != XTG_OK:
        lib = lib or load_library()
        buf = ctypes.create_string_buffer(512)
        lib.xtg_mlp_get_last_error(buf, len(buf))
        raise XtgError(status, buf.value.decode(errors="replace"))
    return status
