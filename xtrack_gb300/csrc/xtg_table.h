// Packed element-parameter table: the device-side form of a lattice.
//
// The reference hands its kernel a table of references to per-class element
// structs (ElementRefData, xtrack/tracker.py:1771-1792) and resolves each
// magnet's model, integrator, number of kicks and strength splits per
// particle at run time (xtrack/beam_elements/elements_src/track_magnet.h:
// 518-574). Here all of that is resolved once on the host: each element
// becomes one variable-length record of plain doubles/ints that the kernel
// walks sequentially. Records are 16-byte aligned so a chunk of consecutive
// records can be copied into shared memory with one bulk copy.
//
// Shared by the host packer (xtg_lattice.cpp) and the kernels (xtg_track.cu).
#pragma once
#include <stdint.h>
#include <string.h>

#include "../../include/xtrack_gb300.h"

#ifdef __CUDACC__
#define XTG_HD_INLINE __host__ __device__ __forceinline__
#else
#define XTG_HD_INLINE static inline
#endif

namespace xtg {

enum Op : int32_t {
    OP_NOP = 0,           // Marker, suppressed edges, zero-effect elements
    OP_DRIFT = 1,         // Drift / DriftSlice*
    OP_MAGNET = 2,        // Multipole, Bend, Quadrupole, Sextupole, Octupole
                          // and their thick/thin/entry/exit slices
    OP_CAVITY = 3,        // Cavity and its slices
    OP_LIMIT_ELLIPSE = 4,
    OP_LIMIT_RECT = 5,
    OP_KICK = 6,          // a magnet that is a single kick with no edges (thin
                          // multipoles, thin slices): compact form of OP_MAGNET
    OP_MON_PARTICLES = 7, // monitors placed in the line (monitors/*.h)
    OP_MON_LAST_TURNS = 8,
    OP_MON_BPM = 9,       // beam position and beam size monitors
    OP_MON_PROFILE = 10,
    OP_LIMIT_POLYGON = 11,
    OP_DIPOLE_EDGE = 12,  // DipoleEdge (dipoleedge.h): linear or full model
    OP_LIMIT_RECT_ELLIPSE = 13,
};

// RecHeader.flags
enum : int32_t {
    F_GLOBAL_APER = 1,    // statically thick class: global aperture follows
    F_SHIFTED = 2,        // aperture, thin Multipole or DipoleEdge with a transverse
                          // shift or tilt: the record ends with its ApertureShift block
};

struct alignas(16) RecHeader {
    int32_t op;
    int32_t flags;
    int32_t nbytes;       // size of the whole record, multiple of 16
    int32_t reserved;
};

struct alignas(16) DriftRec {
    RecHeader h;
    double length;        // signed (negated for backtracking tables)
    int32_t exact;        // 1: exact drift map, 0: expanded
    int32_t reserved;
};

// LimitEllipse (limitellipse.h:12-38): the final compare of x^2 b^2 +
// y^2 a^2 against a_b_squ on ordered keys (upper_key(a_b_squ)); the sum is
// +0 or more, or NaN, so [key(-0), key_a_b_squ] decides it as the FP64
// compare does.
struct alignas(16) LimitEllipseRec {
    RecHeader h;
    double a_squ, b_squ;
    int64_t key_a_b_squ;
    int64_t reserved;
};

// Transverse shift and tilt of an aperture, a thin Multipole or a
// DipoleEdge (track_local_particle_with_transformations.h with shift_x, shift_y,
// rot_s_rad, rot_s_rad_no_frame; track_misalignments.h:38-112,
// track_xyshift.h, track_srotation.h). Entry: the XYShift adds in_x, in_y
// (-(dx - 0); -(0 - dx) in backtracking tables), then the s-rotations by
// rot_s_rad_no_frame and rot_s_rad, each when nonzero, as (sin, cos). Exit:
// the s-rotations by -rot_s_rad and -rot_s_rad_no_frame, then the XYShift
// adds out_x, out_y. The entry applies to every particle reaching the
// element, the exit only to those that survive it (the CPU per-particle
// blocks skip lost particles); both apply when local apertures are ignored.
struct ApertureShift {
    double in_x, in_y, out_x, out_y;
    double rot_in[2][2];      // (sin, cos) of the entry rotations, in order
    double rot_out[2][2];     // (sin, cos) of the exit rotations, in order
    int32_t n_rot_in, n_rot_out;
    int32_t reserved[2];
};

// LimitRect (limitrect.h:9-36): the bounds as ordered integer keys of their
// IEEE bit patterns (ord_key in xtg_table.h), so that the four compares
// run on the integer pipe instead of the narrow FP64 pipe.
struct alignas(16) LimitRectRec {
    RecHeader h;
    int64_t key_min_x, key_max_x, key_min_y, key_max_y;
};

// Ordered integer key of an IEEE double: for non-NaN a, b other than the
// pair (-0, +0), a <= b exactly when key(a) <= key(b); a NaN of either sign
// lies above key(+inf) or below key(-inf), outside every interval between
// non-NaN bounds. The bounds are normalised so that both zeros pass as they
// do in the FP64 compare: a lower bound of 0 is key(-0), an upper bound of
// 0 is key(+0); a NaN bound loses every particle, as the FP64 compare does.
XTG_HD_INLINE int64_t ord_key(double v) {
#ifdef __CUDA_ARCH__
    int64_t const b = __double_as_longlong(v);
#else
    int64_t b;
    memcpy(&b, &v, sizeof(b));
#endif
    return b ^ ((b >> 63) & (int64_t)0x7FFFFFFFFFFFFFFFLL);
}
XTG_HD_INLINE int64_t lower_key(double lo) {
    if (lo != lo) return (int64_t)0x7FFFFFFFFFFFFFFFLL;
    return ord_key(lo == 0.0 ? -0.0 : lo);
}
XTG_HD_INLINE int64_t upper_key(double hi) {
    if (hi != hi) return (int64_t)(-0x7FFFFFFFFFFFFFFFLL - 1);
    return ord_key(hi == 0.0 ? 0.0 : hi);
}

// LimitRectEllipse (limitrectellipse.h:14-44): the symmetric rectangle
// (+-max_x, +-max_y) and the ellipse, all compares on ordered keys.
struct alignas(16) LimitRectEllipseRec {
    RecHeader h;
    int64_t key_min_x, key_max_x, key_min_y, key_max_y;
    double a_squ, b_squ;
    int64_t key_a_b_squ;
    int64_t reserved;
};

// LimitPolygon (limitpolygon.h:13-90): x vertices then y vertices follow.
struct alignas(16) LimitPolygonRec {
    RecHeader h;
    int64_t n;
    double inner_radius_sq;   // points inside this circle skip the test
};

// Integrators (reference numbering, _common.py:40-47)
enum : int32_t { INT_TEAPOT = 1, INT_YOSHIDA4 = 2, INT_UNIFORM = 3 };

// One kick_simple_single_coordinates pass in the reference's arithmetic
// (track_magnet_kick.h:182-228). Coefficients live in the record's
// coefficient area at `coef` doubles from its start, highest order first:
// for each order i = top..0 the quintuple
//   A_i = round(round(knl_i*factor)*invf_i)   (value of chi*knl_i*factor*invf_i at chi = 1)
//   B_i = same with ksl_i
//   knl_i, ksl_i, invf_i                        (for particles with chi != 1)
// `top` is the highest order with a non-zero coefficient (-1: skip pass).
struct ExactPass {
    int32_t top;
    int32_t coef;
    double factor;
};

enum : int32_t { EDGE_NONE = 0, EDGE_AXAY = 1, EDGE_LINEAR = 2, EDGE_FRINGE = 3 };

// Parameters of one nonlinear edge (full or dipole-only model,
// track_magnet_edge.h:83-158): a block of doubles in the record's
// coefficient area, at MagnetRec::entry_fringe / exit_fringe.
enum : int32_t {
    FR_MODEL = 0,        // 1 full, 2 dipole-only
    FR_IS_EXIT = 1,
    FR_K0 = 2,           // dipole strength of the fringe (sign flipped at the exit)
    FR_FINT = 3,
    FR_HGAP = 4,
    FR_FACE_ANGLE = 5,
    FR_ROTATE = 6,       // |face angle| > 1e-9
    FR_SIN = 7, FR_COS = 8, FR_TAN = 9,            // of the face angle
    FR_WSIN = 10, FR_WCOS = 11, FR_WTAN = 12,      // of theta = -face angle
    FR_WSIN2 = 13,                                 // sin(2 theta)
    FR_LENGTH = 14,      // length / factor_knl_ksl (multipole fringe)
    FR_KL_ORDER = 15,
    FR_KNORM = 16,       // k0..k3
    FR_KSKEW = 20,       // k0s..k3s
    FR_KNL = 24,         // knl[0..kl_order], then ksl[0..kl_order]
};

struct alignas(16) MagnetRec {
    RecHeader h;
    // --- structure ---
    int32_t body_active;
    int32_t integrator;       // INT_*
    int32_t n_kicks;          // resolved number of kicks (>= 0)
    int32_t drift_model;      // -1 kick only, 0 expanded, 1 exact, 2 polar,
                              // 3 expanded combined, 4/5 exact bend, 7/8 yoshida
    int32_t only_drift;       // body is a single drift of the full length
    int32_t kick_rot_frame;
    int32_t edge_entry;       // EDGE_*
    int32_t edge_exit;
    int32_t n_kw;             // distinct kick weights (1, or 4 for Yoshida)
    int32_t curv_terms;       // bit0: rot-frame term, bit1: k0h term, bit2: k1h term
    int32_t fast_top;         // merged-polynomial top order for the fast path (-1: none)
    int32_t fast_coef;        // offset of merged coefficients (pairs cn_i, cs_i)
    // --- drift lengths (as the reference computes them) ---
    double length;            // core length (weight and backtrack applied)
    double d_edge;            // TEAPOT edge drift / uniform half drift
    double d_inside;          // TEAPOT inside drift
    double d_fast_inside;     // fast path: merged uniform drift (2*d_edge)
    double d_yoshida[4];      // Yoshida drifts slice_length*d_i
    double k0_drift, k1_drift, h_drift;
    // --- kick weights and curvature constants per kick weight ---
    double kw[4];
    double hl[4];             // h*L*kw + hxl*kw
    double C0[4];             // round(round(-Q0*kw)*htot)  (chi = 1)
    double C1[4];             // round(round(htot*Q1)*kw)   (chi = 1)
    double fast_scale[4];     // fast path: kick weight relative to kw[0]
    double htot, Q0, Q1;
    // --- linear edges ---
    double entry_r21, entry_r43, exit_r21, exit_r43;
    // --- nonlinear edges: FringeRec offsets (doubles) in the coefficient area ---
    int32_t entry_fringe, exit_fringe;
    int32_t backtrack;        // the record belongs to a backtracking table
    int32_t reserved_fr;
    // --- exact kick passes: knl, knl_rel, main strengths ---
    ExactPass pass[3];
    // coefficient area follows (doubles)
};

// Compact record of a thin kick (model -1, one kick, no edges). Same
// meaning as the MagnetRec fields of kick-weight slot 0.
struct alignas(16) KickRec {
    RecHeader h;
    int32_t fast_top;
    int32_t fast_coef;
    int32_t curv_terms;
    int32_t reserved;
    ExactPass pass[3];
    double kw, hl, C0, C1, htot, Q0, Q1, reserved2;
    // coefficient area follows (doubles)
};

// DipoleEdge (dipoleedge.h:14-71). model 0: the linear kick with r21, r43
// (negated in backtracking tables); model 1: a FringeRec block (dipole-only
// layout) at `fringe` doubles into the coefficient area that follows.
struct alignas(16) DipoleEdgeRec {
    RecHeader h;
    int32_t model;
    int32_t fringe;
    int32_t backtrack;
    int32_t reserved;
    double r21, r43;
    // coefficient area follows (doubles)
};

struct alignas(16) CavityRec {
    RecHeader h;
    int32_t integrator;
    int32_t n_kicks;
    int32_t drift_model;      // -1, 0, 1, 3 (see configure_tracking_model)
    int32_t absolute_time;
    double length;            // body_length * weight
    double voltage;           // voltage * weight (sign flipped when backtracking)
    double d_edge, d_inside, d_yoshida[4];
    double kw[4];
    double frequency;
    double harmonic;
    double lag_rad;           // DEG2RAD*lag
    double phase;
    double phi_const;         // DEG2RAD*lag + phase (valid when phase0 == 0)
    double w_freq;            // (2*pi/c)*frequency (valid when harmonic == 0)
};

// ParticlesMonitor as a line element (particles_monitor.h:12-77).
struct alignas(16) MonParticlesRec {
    RecHeader h;
    xtg_monitor m;
};

// LastTurnsMonitor (last_turns_monitor.h:17-55).
struct alignas(16) MonLastTurnsRec {
    RecHeader h;
    int64_t particle_id_start, particle_id_stop, n_last_turns, every_n_turns;
    uint32_t *lost_at_offset, *particle_id, *at_turn;
    float *x, *px, *y, *py, *delta, *zeta;
};

// BeamPositionMonitor (beam_position_monitor.h:16-58).
struct alignas(16) MonBpmRec {
    RecHeader h;
    int64_t particle_id_start, particle_id_stop, start_at_turn, n_slots;
    double frev, sampling_frequency;
    double *count, *x_sum, *y_sum;
    double *x2_sum, *y2_sum;      // beam size monitor (NULL for beam position)
};

// BeamProfileMonitor (beam_profile_monitor.h:16-80).
struct alignas(16) MonProfileRec {
    RecHeader h;
    int64_t particle_id_start, particle_id_stop, start_at_turn, sample_size;
    double frev, sampling_frequency;
    int64_t nx, ny;
    double x_min, dx, y_min, dy;
    double *counts_x, *counts_y;
};

// Header of an uploaded table.
struct TableInfo {
    int64_t n_elements;
    int64_t table_bytes;
};

}  // namespace xtg
