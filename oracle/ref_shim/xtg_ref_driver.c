/*
 * Driver that compiles the reference's OWN element C code (xtrack/headers,
 * xtrack/particles/local_particle_custom_api.h and
 * xtrack/beam_elements/elements_src/*.h, included from the reference tree
 * at build time, never copied) into a CPU library, oracle/_ref/libxtref*.so.
 * TEST INFRASTRUCTURE ONLY: it pins the C restatement in xtg_oracle.c to the
 * reference's own arithmetic.
 *
 * What this file supplies is what xobjects would normally generate:
 *   - the LocalParticle struct and its accessors (particles.py:86-408),
 *   - the <Class>Data getters of each in-scope element class, here all read
 *     from one xtg_element record (slice parents resolved into the record),
 *   - a per-particle restatement of the track_line driver
 *     (tracker.py:594-736, GPU semantics).
 * Build flags choose the TrackerConfig: XTRACK_USE_EXACT_DRIFTS,
 * XTRACK_CAVITY_PRESERVE_ANGLE and the FREEZE_VAR_<name> set of
 * freeze_longitudinal produce separate libraries.
 */
#define XO_CONTEXT_CPU
#define XO_CONTEXT_CPU_OPENMP
#define XTRACK_MULTIPOLE_NO_SYNRAD
/* The reference emits global_aperture_check only when this macro is
 * defined (tracker.py:681-689); its value is read at run time here. */
static double xtr_global_xy_limit = 1.0;
#define XTRACK_GLOBAL_XY_LIMIT (xtr_global_xy_limit)

#include "xobjects/headers/common.h"
#include "../../include/xtrack_gb300.h"

#include <stdlib.h>
#include <string.h>

/* ---- LocalParticle (restated from the generator, particles.py:96-112) -- */
#define XTR_DBL_FIELDS(X) X(p0c) X(gamma0) X(beta0) X(s) X(zeta) X(x) X(y) \
    X(px) X(py) X(ptau) X(delta) X(rpp) X(rvv) X(chi) X(charge_ratio) X(weight) \
    X(ax) X(ay) X(spin_x) X(spin_y) X(spin_z) X(anomalous_magnetic_moment)
#define XTR_I64_FIELDS(X) X(pdg_id) X(particle_id) X(at_element) X(at_turn) \
    X(state) X(parent_particle_id)
/* The subset that xtg_particles carries (spin fields stay local). */
#define XTR_IO_DBL_FIELDS(X) X(p0c) X(gamma0) X(beta0) X(s) X(zeta) X(x) X(y) \
    X(px) X(py) X(ptau) X(delta) X(rpp) X(rvv) X(chi) X(charge_ratio) X(weight) \
    X(ax) X(ay)

typedef struct {
    int64_t _capacity;
    int64_t _num_active_particles;
    int64_t _num_lost_particles;
    int64_t start_tracking_at_element;
    double q0;
    double mass0;
    double t_sim;
#define XTR_DECL_D(f) double* f;
#define XTR_DECL_I(f) int64_t* f;
    XTR_DBL_FIELDS(XTR_DECL_D)
    XTR_I64_FIELDS(XTR_DECL_I)
    uint32_t* _rng_s1;
    uint32_t* _rng_s2;
    uint32_t* _rng_s3;
    uint32_t* _rng_s4;
    int64_t ipart;
    int64_t endpart;
    uint64_t track_flags;
    double line_length;
    int8_t* io_buffer;
} LocalParticle;

#define XTR_ACC(T, f) \
    static inline T LocalParticle_get_##f(LocalParticle* p) { return p->f[p->ipart]; } \
    static inline void LocalParticle_set_##f(LocalParticle* p, T v) { p->f[p->ipart] = v; } \
    static inline void LocalParticle_add_to_##f(LocalParticle* p, T v) { p->f[p->ipart] += v; } \
    static inline void LocalParticle_scale_##f(LocalParticle* p, T v) { p->f[p->ipart] *= v; }
#define XTR_ACC_D(f) XTR_ACC(double, f)
#define XTR_ACC_I(f) XTR_ACC(int64_t, f)
/* FREEZE_VAR_<name>: the generator wraps the setter, adder and scaler of
 * <name> in #ifndef FREEZE_VAR_<name> (particles.py:185-225), so a frozen
 * variable keeps its value; freeze_longitudinal freezes zeta and the four
 * energy variables (line.py:4446-4469). */
#define XTR_ACC_FROZEN(T, f) \
    static inline T LocalParticle_get_##f(LocalParticle* p) { return p->f[p->ipart]; } \
    static inline void LocalParticle_set_##f(LocalParticle* p, T v) { (void)p; (void)v; } \
    static inline void LocalParticle_add_to_##f(LocalParticle* p, T v) { (void)p; (void)v; } \
    static inline void LocalParticle_scale_##f(LocalParticle* p, T v) { (void)p; (void)v; }
#define XTR_FREE_DBL_FIELDS(X) X(p0c) X(gamma0) X(beta0) X(s) X(x) X(y) \
    X(px) X(py) X(chi) X(charge_ratio) X(weight) \
    X(ax) X(ay) X(spin_x) X(spin_y) X(spin_z) X(anomalous_magnetic_moment)
XTR_FREE_DBL_FIELDS(XTR_ACC_D)
#ifdef FREEZE_VAR_zeta
XTR_ACC_FROZEN(double, zeta)
#else
XTR_ACC_D(zeta)
#endif
#ifdef FREEZE_VAR_ptau
XTR_ACC_FROZEN(double, ptau)
#else
XTR_ACC_D(ptau)
#endif
#ifdef FREEZE_VAR_delta
XTR_ACC_FROZEN(double, delta)
#else
XTR_ACC_D(delta)
#endif
#ifdef FREEZE_VAR_rpp
XTR_ACC_FROZEN(double, rpp)
#else
XTR_ACC_D(rpp)
#endif
#ifdef FREEZE_VAR_rvv
XTR_ACC_FROZEN(double, rvv)
#else
XTR_ACC_D(rvv)
#endif
XTR_I64_FIELDS(XTR_ACC_I)

static inline double LocalParticle_get_q0(LocalParticle* p) { return p->q0; }
static inline double LocalParticle_get_mass0(LocalParticle* p) { return p->mass0; }
static inline double LocalParticle_get_t_sim(LocalParticle* p) { return p->t_sim; }
static inline int64_t LocalParticle_get__num_active_particles(LocalParticle* p) { return p->_num_active_particles; }
static inline uint64_t LocalParticle_check_track_flag(LocalParticle* p, uint8_t index) {
    return (p->track_flags >> index) & 1;
}
static inline void LocalParticle_exchange(LocalParticle* p, int64_t a, int64_t b) {
#define XTR_SW_D(f) { double t = p->f[a]; p->f[a] = p->f[b]; p->f[b] = t; }
#define XTR_SW_I(f) { int64_t t = p->f[a]; p->f[a] = p->f[b]; p->f[b] = t; }
    XTR_DBL_FIELDS(XTR_SW_D)
    XTR_I64_FIELDS(XTR_SW_I)
}

/* Track flag names (track_flags.py:5-12). */
#define XS_FLAG_BACKTRACK (0)
#define XS_FLAG_KILL_CAVITY_KICK (2)
#define XS_FLAG_IGNORE_GLOBAL_APERTURE (3)
#define XS_FLAG_IGNORE_LOCAL_APERTURE (4)
#define XS_FLAG_SR_TAPER (5)
#define XS_FLAG_SR_KICK_SAME_AS_FIRST (6)

/* ---- element data getters --------------------------------------------- */
typedef void* SynchrotronRadiationRecordData;

#define XTR_GET_D(C, f, expr) \
    static inline double C##Data_get_##f(C##Data el) { return (expr); } \
    static inline double C##Data_get__parent_##f(C##Data el) { return (expr); }
#define XTR_GET_I(C, f, expr) \
    static inline int64_t C##Data_get_##f(C##Data el) { return (expr); } \
    static inline int64_t C##Data_get__parent_##f(C##Data el) { return (expr); }
#define XTR_ARR(C, f, len) \
    static inline const double* C##Data_getp1_##f(C##Data el, int64_t i) { return &el->f[i]; } \
    static inline const double* C##Data_getp1__parent_##f(C##Data el, int64_t i) { return &el->f[i]; } \
    static inline double C##Data_get_##f(C##Data el, int64_t i) { return el->f[i]; } \
    static inline double C##Data_get__parent_##f(C##Data el, int64_t i) { return el->f[i]; } \
    static inline int64_t C##Data_len_##f(C##Data el) { return (len); } \
    static inline int64_t C##Data_len__parent_##f(C##Data el) { return (len); }

#define XTR_CLASS(C) \
    typedef const xtg_element* C##Data; \
    XTR_GET_D(C, length, el->length) XTR_GET_D(C, h, el->h) XTR_GET_D(C, hxl, el->hxl) \
    XTR_GET_D(C, k0, el->k0) XTR_GET_D(C, k1, el->k1) XTR_GET_D(C, k2, el->k2) \
    XTR_GET_D(C, k3, el->k3) XTR_GET_D(C, k0s, el->k0s) XTR_GET_D(C, k1s, el->k1s) \
    XTR_GET_D(C, k2s, el->k2s) XTR_GET_D(C, k3s, el->k3s) \
    XTR_GET_D(C, inv_factorial_order, el->inv_factorial_order) \
    XTR_GET_D(C, edge_entry_angle, el->edge_entry_angle) \
    XTR_GET_D(C, edge_exit_angle, el->edge_exit_angle) \
    XTR_GET_D(C, edge_entry_angle_fdown, el->edge_entry_angle_fdown) \
    XTR_GET_D(C, edge_exit_angle_fdown, el->edge_exit_angle_fdown) \
    XTR_GET_D(C, edge_entry_fint, el->edge_entry_fint) \
    XTR_GET_D(C, edge_exit_fint, el->edge_exit_fint) \
    XTR_GET_D(C, edge_entry_hgap, el->edge_entry_hgap) \
    XTR_GET_D(C, edge_exit_hgap, el->edge_exit_hgap) \
    XTR_GET_D(C, voltage, el->voltage) XTR_GET_D(C, frequency, el->frequency) \
    XTR_GET_D(C, harmonic, el->harmonic) XTR_GET_D(C, lag, el->lag) \
    XTR_GET_D(C, phase, el->phase) XTR_GET_D(C, a_squ, el->a_squ) \
    XTR_GET_D(C, b_squ, el->b_squ) XTR_GET_D(C, a_b_squ, el->a_b_squ) \
    XTR_GET_D(C, min_x, el->min_x) XTR_GET_D(C, max_x, el->max_x) \
    XTR_GET_D(C, min_y, el->min_y) XTR_GET_D(C, max_y, el->max_y) \
    XTR_GET_D(C, weight, el->weight) XTR_GET_D(C, delta_taper, 0.) \
    XTR_GET_D(C, shift_x, el->shift_x) XTR_GET_D(C, shift_y, el->shift_y) \
    XTR_GET_D(C, shift_s, el->shift_s) XTR_GET_D(C, rot_x_rad, el->rot_x_rad) \
    XTR_GET_D(C, rot_y_rad, el->rot_y_rad) XTR_GET_D(C, rot_s_rad, el->rot_s_rad) \
    XTR_GET_D(C, rot_s_rad_no_frame, el->rot_s_rad_no_frame) XTR_GET_D(C, rot_shift_anchor, 0.) \
    XTR_GET_D(C, lag_taper, 0.) XTR_GET_D(C, phase_taper, 0.) \
    XTR_GET_I(C, order, el->order) XTR_GET_I(C, num_multipole_kicks, el->num_multipole_kicks) \
    XTR_GET_I(C, num_kicks, el->num_multipole_kicks) XTR_GET_I(C, model, el->model) \
    XTR_GET_I(C, integrator, el->integrator) XTR_GET_I(C, isthick, el->isthick) \
    XTR_GET_I(C, main_is_skew, el->main_is_skew) XTR_GET_I(C, main_order, el->main_order) \
    XTR_GET_I(C, edge_entry_active, el->edge_entry_active) \
    XTR_GET_I(C, edge_exit_active, el->edge_exit_active) \
    XTR_GET_I(C, edge_entry_model, el->edge_entry_model) \
    XTR_GET_I(C, edge_exit_model, el->edge_exit_model) \
    XTR_GET_I(C, absolute_time, el->absolute_time) XTR_GET_I(C, radiation_flag, 0) \
    XTR_ARR(C, knl, el->order + 1) XTR_ARR(C, ksl, el->order + 1) \
    XTR_ARR(C, knl_rel, el->order_rel + 1) XTR_ARR(C, ksl_rel, el->order_rel + 1) \
    static inline SynchrotronRadiationRecordData C##Data_getp_internal_record(C##Data el, LocalParticle* p) { \
        (void)el; (void)p; return NULL; }

XTR_CLASS(Drift)
XTR_CLASS(Multipole)
XTR_CLASS(Bend)
XTR_CLASS(Quadrupole)
XTR_CLASS(Sextupole)
XTR_CLASS(Octupole)
XTR_CLASS(Cavity)
XTR_CLASS(LimitEllipse)
XTR_CLASS(LimitRect)
XTR_CLASS(LimitRectEllipse)
XTR_CLASS(ThickSliceBend) XTR_CLASS(ThinSliceBend) XTR_CLASS(DriftSliceBend)
XTR_CLASS(ThinSliceBendEntry) XTR_CLASS(ThinSliceBendExit)
XTR_CLASS(ThickSliceQuadrupole) XTR_CLASS(ThinSliceQuadrupole) XTR_CLASS(DriftSliceQuadrupole)
XTR_CLASS(ThinSliceQuadrupoleEntry) XTR_CLASS(ThinSliceQuadrupoleExit)
XTR_CLASS(ThickSliceSextupole) XTR_CLASS(ThinSliceSextupole) XTR_CLASS(DriftSliceSextupole)
XTR_CLASS(ThinSliceSextupoleEntry) XTR_CLASS(ThinSliceSextupoleExit)
XTR_CLASS(ThickSliceOctupole) XTR_CLASS(ThinSliceOctupole) XTR_CLASS(DriftSliceOctupole)
XTR_CLASS(ThinSliceOctupoleEntry) XTR_CLASS(ThinSliceOctupoleExit)
XTR_CLASS(ThickSliceMultipole) XTR_CLASS(ThinSliceMultipole) XTR_CLASS(DriftSliceMultipole)
XTR_CLASS(ThickSliceCavity) XTR_CLASS(ThinSliceCavity) XTR_CLASS(DriftSliceCavity)

/* DipoleEdge (dipole_edge.py _xofields): r21, r43 as the class computes
 * them, the full model's k, e1, fint, hgap, side; model 0/1/-1. */
typedef const xtg_element* DipoleEdgeData;
XTR_GET_D(DipoleEdge, r21, el->r21) XTR_GET_D(DipoleEdge, r43, el->r43)
XTR_GET_D(DipoleEdge, k, el->k) XTR_GET_D(DipoleEdge, e1, el->e1)
XTR_GET_D(DipoleEdge, fint, el->fint) XTR_GET_D(DipoleEdge, hgap, el->hgap)
XTR_GET_D(DipoleEdge, delta_taper, 0.)
XTR_GET_I(DipoleEdge, model, el->model) XTR_GET_I(DipoleEdge, side, el->side)
XTR_GET_D(DipoleEdge, shift_x, el->shift_x) XTR_GET_D(DipoleEdge, shift_y, el->shift_y)
XTR_GET_D(DipoleEdge, shift_s, el->shift_s) XTR_GET_D(DipoleEdge, rot_x_rad, el->rot_x_rad)
XTR_GET_D(DipoleEdge, rot_y_rad, el->rot_y_rad) XTR_GET_D(DipoleEdge, rot_s_rad, el->rot_s_rad)
XTR_GET_D(DipoleEdge, rot_s_rad_no_frame, el->rot_s_rad_no_frame)
XTR_GET_D(DipoleEdge, rot_shift_anchor, 0.)

/* ---- the reference's element code, compiled as-is --------------------- */
#include "xtrack/headers/constants.h"
#include "xtrack/headers/particle_states.h"
#include "xtrack/particles/local_particle_custom_api.h"
#include "xtrack/beam_elements/elements_src/drift.h"
#include "xtrack/beam_elements/elements_src/multipole.h"
#include "xtrack/beam_elements/elements_src/bend.h"
#include "xtrack/beam_elements/elements_src/quadrupole.h"
#include "xtrack/beam_elements/elements_src/sextupole.h"
#include "xtrack/beam_elements/elements_src/octupole.h"
#include "xtrack/beam_elements/elements_src/cavity.h"
#include "xtrack/beam_elements/elements_src/limitellipse.h"
#include "xtrack/beam_elements/elements_src/limitrect.h"
#include "xtrack/beam_elements/elements_src/dipoleedge.h"
#include "xtrack/beam_elements/elements_src/limitrectellipse.h"

/* The apertures through the reference's transformation wrapper, as its
 * kernel calls every element (base_element.py:83-126): the entry and exit
 * shifts of a shifted aperture come from the reference's own code. */
#define ELEMENT_NAME LimitRect
#define ALLOW_ROT_AND_SHIFT 1
#include "xtrack/headers/track_local_particle_with_transformations.h"
#undef ALLOW_ROT_AND_SHIFT
#undef ELEMENT_NAME
#define ELEMENT_NAME LimitEllipse
#define ALLOW_ROT_AND_SHIFT 1
#include "xtrack/headers/track_local_particle_with_transformations.h"
#undef ALLOW_ROT_AND_SHIFT
#undef ELEMENT_NAME
#define ELEMENT_NAME LimitRectEllipse
#define ALLOW_ROT_AND_SHIFT 1
#include "xtrack/headers/track_local_particle_with_transformations.h"
#undef ALLOW_ROT_AND_SHIFT
#undef ELEMENT_NAME
/* Multipole: `isthick` in its fields (IS_THICK_DYNAMIC), no `h` (straight);
 * DipoleEdge: no length, no `h` (base_element.py:83-126) */
#define ELEMENT_NAME Multipole
#define ALLOW_ROT_AND_SHIFT 1
#define IS_THICK_DYNAMIC 1
#include "xtrack/headers/track_local_particle_with_transformations.h"
#undef IS_THICK_DYNAMIC
#undef ALLOW_ROT_AND_SHIFT
#undef ELEMENT_NAME
#define ELEMENT_NAME DipoleEdge
#define ALLOW_ROT_AND_SHIFT 1
#include "xtrack/headers/track_local_particle_with_transformations.h"
#undef ALLOW_ROT_AND_SHIFT
#undef ELEMENT_NAME
#include "xtrack/beam_elements/elements_src/thick_slice_bend.h"
#include "xtrack/beam_elements/elements_src/thin_slice_bend.h"
#include "xtrack/beam_elements/elements_src/drift_slice_bend.h"
#include "xtrack/beam_elements/elements_src/thin_slice_bend_entry.h"
#include "xtrack/beam_elements/elements_src/thin_slice_bend_exit.h"
#include "xtrack/beam_elements/elements_src/thick_slice_quadrupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_quadrupole.h"
#include "xtrack/beam_elements/elements_src/drift_slice_quadrupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_quadrupole_entry.h"
#include "xtrack/beam_elements/elements_src/thin_slice_quadrupole_exit.h"
#include "xtrack/beam_elements/elements_src/thick_slice_sextupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_sextupole.h"
#include "xtrack/beam_elements/elements_src/drift_slice_sextupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_sextupole_entry.h"
#include "xtrack/beam_elements/elements_src/thin_slice_sextupole_exit.h"
#include "xtrack/beam_elements/elements_src/thick_slice_octupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_octupole.h"
#include "xtrack/beam_elements/elements_src/drift_slice_octupole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_octupole_entry.h"
#include "xtrack/beam_elements/elements_src/thin_slice_octupole_exit.h"
#include "xtrack/beam_elements/elements_src/thick_slice_multipole.h"
#include "xtrack/beam_elements/elements_src/thin_slice_multipole.h"
#include "xtrack/beam_elements/elements_src/drift_slice_multipole.h"
#include "xtrack/beam_elements/elements_src/thick_slice_cavity.h"
#include "xtrack/beam_elements/elements_src/thin_slice_cavity.h"
#include "xtrack/beam_elements/elements_src/drift_slice_cavity.h"

/* ---- dispatch: the switch of tracker.py:660-697 ----------------------- */
/* Returns 1 when the class is statically thick (global aperture follows). */
static int xtr_apply(const xtg_element* e, LocalParticle* lp) {
#define XTR_SLICES(C, THICK_RET) \
    switch (e->slice) { \
    case XTG_SLICE_NONE: C##_track_local_particle(e, lp); return THICK_RET; \
    case XTG_SLICE_THICK: ThickSlice##C##_track_local_particle(e, lp); return 1; \
    case XTG_SLICE_THIN: ThinSlice##C##_track_local_particle(e, lp); return 0; \
    case XTG_SLICE_DRIFT: DriftSlice##C##_track_local_particle(e, lp); return 1; \
    default: break; }
#define XTR_EDGES(C) \
    if (e->slice == XTG_SLICE_ENTRY) { ThinSlice##C##Entry_track_local_particle(e, lp); return 0; } \
    if (e->slice == XTG_SLICE_EXIT) { ThinSlice##C##Exit_track_local_particle(e, lp); return 0; }
    switch (e->cls) {
    case XTG_CLS_MARKER: return 0;
    case XTG_CLS_DRIFT: Drift_track_local_particle(e, lp); return 1;
    case XTG_CLS_LIMIT_ELLIPSE: LimitEllipse_track_local_particle_with_transformations(e, lp); return 0;
    case XTG_CLS_LIMIT_RECT: LimitRect_track_local_particle_with_transformations(e, lp); return 0;
    case XTG_CLS_DIPOLE_EDGE: DipoleEdge_track_local_particle_with_transformations(e, lp); return 0;
    case XTG_CLS_LIMIT_RECT_ELLIPSE: LimitRectEllipse_track_local_particle_with_transformations(e, lp); return 0;
    case XTG_CLS_MULTIPOLE:
        if (e->slice == XTG_SLICE_NONE) { Multipole_track_local_particle_with_transformations(e, lp); return 0; }
        XTR_SLICES(Multipole, 0) return 0;
    case XTG_CLS_BEND: XTR_EDGES(Bend) XTR_SLICES(Bend, 1) return 0;
    case XTG_CLS_QUADRUPOLE: XTR_EDGES(Quadrupole) XTR_SLICES(Quadrupole, 1) return 0;
    case XTG_CLS_SEXTUPOLE: XTR_EDGES(Sextupole) XTR_SLICES(Sextupole, 1) return 0;
    case XTG_CLS_OCTUPOLE: XTR_EDGES(Octupole) XTR_SLICES(Octupole, 1) return 0;
    case XTG_CLS_CAVITY: XTR_SLICES(Cavity, 1) return 0;
    default: return 0;
    }
#undef XTR_SLICES
#undef XTR_EDGES
}

/* ---- per-particle track_line (tracker.py:594-736) ---------------------- */
int32_t xtr_track(const xtg_element* els, int64_t n_elements, const xtg_config* cfg,
                  xtg_particles* P, int32_t num_turns, int32_t ele_start,
                  int32_t num_ele_track, int32_t flag_end_turn_actions,
                  int32_t flag_reset_s_at_end_turn, int32_t num_ele_line,
                  double line_length, uint64_t track_flags) {
    if (!els || !cfg || !P) return XTG_E_NULL;
    if (ele_start < 0 || num_ele_track < 0 || (int64_t)ele_start + num_ele_track > n_elements)
        return XTG_E_VALUE;
    xtr_global_xy_limit = cfg->global_xy_limit;
    int const backtrack = (int)((track_flags >> XS_FLAG_BACKTRACK) & 1u);
    for (int64_t i = 0; i < P->capacity; i++) {
        /* one-particle LocalParticle over local copies of every field */
#define XTR_LOC_D(f) double f##_v = 0.;
#define XTR_LOC_I(f) int64_t f##_v = 0;
#define XTR_IN(f) if (P->f) f##_v = P->f[i];
        XTR_DBL_FIELDS(XTR_LOC_D)
        XTR_I64_FIELDS(XTR_LOC_I)
        XTR_IO_DBL_FIELDS(XTR_IN)
        XTR_I64_FIELDS(XTR_IN)
        uint32_t rng_v[4] = {0, 0, 0, 0};
        LocalParticle lp;
        memset(&lp, 0, sizeof(lp));
        lp._capacity = 1;
        lp._num_active_particles = 1;
        lp.q0 = P->q0;
        lp.mass0 = P->mass0;
        lp.t_sim = P->t_sim;
#define XTR_PTR(f) lp.f = &f##_v;
        XTR_DBL_FIELDS(XTR_PTR)
        XTR_I64_FIELDS(XTR_PTR)
        lp._rng_s1 = &rng_v[0]; lp._rng_s2 = &rng_v[1];
        lp._rng_s3 = &rng_v[2]; lp._rng_s4 = &rng_v[3];
        lp.ipart = 0;
        lp.endpart = 1;
        lp.track_flags = track_flags;
        lp.line_length = line_length;

        int64_t isactive = check_is_active(&lp);
        for (int64_t iturn = 0; iturn < num_turns; iturn++) {
            if (!isactive) break;
            int64_t const ele_stop = (int64_t)ele_start + num_ele_track;
            int64_t elem_idx, increm;
            if (backtrack) {
                elem_idx = ele_stop - 1;
                increm = -1;
                if (flag_end_turn_actions > 0)
                    increment_at_turn_backtrack(&lp, flag_reset_s_at_end_turn,
                                                line_length, num_ele_line);
            } else {
                elem_idx = ele_start;
                increm = 1;
            }
            for (; (elem_idx >= ele_start) && (elem_idx < ele_stop); elem_idx += increm) {
                if (xtr_apply(&els[elem_idx], &lp)) {
                    if (cfg->has_global_xy_limit) global_aperture_check(&lp);
                }
                isactive = check_is_active(&lp);
                if (!isactive) break;
                increment_at_element(&lp, backtrack ? -1 : 1);
            }
            if (!backtrack && flag_end_turn_actions > 0) {
                if (isactive) increment_at_turn(&lp, flag_reset_s_at_end_turn);
            }
        }
#define XTR_OUT(f) if (P->f) P->f[i] = f##_v;
        XTR_IO_DBL_FIELDS(XTR_OUT)
        XTR_I64_FIELDS(XTR_OUT)
    }
    return XTG_OK;
}
