// Host-side lattice packer: raw element records (the reference's
// `_xofields`, xtrack_gb300.h::xtg_element) -> packed device table
// (xtg_table.h).
//
// Everything the reference computes per particle but that depends only on
// the element is computed here once, with the same IEEE operations in the
// same order, so that the exact-arithmetic kernel reproduces the reference
// bit for bit. This file must be compiled without floating-point
// contraction (-ffp-contract=off): several values below are products whose
// rounding must match the reference's separate multiplications.
#include "xtg_lattice.h"

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace xtg {

namespace {

// default_magnet_config.h:9-23
constexpr int kBendDefaultModel = 3;
constexpr int kQuadDefaultModel = 4;
constexpr int kStraightDefaultModel = 6;   // sextupole, octupole, multipole
constexpr int kBendDefaultIntegrator = 2;
constexpr int kStraightDefaultIntegrator = 3;

// track_magnet.h:240-253 (Yoshida-4 coefficients from MAD-NG)
constexpr double kDYoshida[4] = {
    3.922568052387799819591407413100e-01, 5.100434119184584780271052295575e-01,
    -4.710533854097565531482416645304e-01, 6.875316825251809316199569366290e-02};
constexpr double kKYoshida[4] = {
    7.845136104775599639182814826199e-01, 2.355732133593569921359289764951e-01,
    -1.177679984178870098432412305556e+00, 1.315186320683906284756403692882e+00};

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751;
constexpr double kDeg2Rad = 0.0174532925199432957692369076848861271344287188854;
constexpr double kCLight = 299792458.0;

// xtrack/headers/factorial.h:4-35: 1/n! (correctly rounded; n! is exact in
// double for n <= 22).
double one_over_factorial(int64_t n) {
    if (n < 0) return 0.;
    double f = 1.0;
    for (int64_t i = 2; i <= n; i++) f *= (double)i;
    return 1. / f;
}

double main_strength(const xtg_element& e) {
    switch (e.cls) {
    case XTG_CLS_BEND: return e.k0 * e.length;
    case XTG_CLS_QUADRUPOLE: return e.length * (e.main_is_skew ? e.k1s : e.k1);
    case XTG_CLS_SEXTUPOLE: return e.length * (e.main_is_skew ? e.k2s : e.k2);
    case XTG_CLS_OCTUPOLE: return e.length * (e.main_is_skew ? e.k3s : e.k3);
    case XTG_CLS_MULTIPOLE:
        return e.main_is_skew ? e.ksl[e.main_order] : e.knl[e.main_order];
    default: return 0.;
    }
}

// Byte buffer of one record; grows in doubles, keeps 16-byte size.
struct RecBuf {
    std::vector<unsigned char> bytes;
    template <class T>
    T* head() { return reinterpret_cast<T*>(bytes.data()); }
    void init(size_t head_size) { bytes.assign(head_size, 0); }
    // appends n doubles; returns offset (in doubles) from `coef_base`
    int32_t append(const double* v, size_t n, size_t coef_base) {
        size_t off = bytes.size();
        bytes.resize(off + n * sizeof(double));
        std::memcpy(bytes.data() + off, v, n * sizeof(double));
        return (int32_t)((off - coef_base) / sizeof(double));
    }
    void pad16() {
        while (bytes.size() % 16) bytes.push_back(0);
    }
};

// Resolved magnet parameters (what track_magnet_particles works with).
struct MagnetIn {
    double weight = 1.0;
    double length = 0.;
    int64_t order = 0;
    double inv_factorial_order = 1.;
    const double* knl = nullptr;
    const double* ksl = nullptr;
    int64_t order_rel = -1;
    const double* knl_rel = nullptr;
    const double* ksl_rel = nullptr;
    double rel_ref_strength = 0.;
    int64_t num_multipole_kicks = 0;
    int64_t model = 0, default_model = 0, integrator = 0, default_integrator = 0;
    double h = 0, hxl = 0, k0 = 0, k1 = 0, k2 = 0, k3 = 0, k0s = 0, k1s = 0, k2s = 0, k3s = 0;
    int body_active = 1;
    int edge_entry_active = 0, edge_exit_active = 0;
    int edge_entry_model = 0, edge_exit_model = 0;
    double edge_entry_angle = 0, edge_exit_angle = 0;
    double edge_entry_angle_fdown = 0, edge_exit_angle_fdown = 0;
    double edge_entry_fint = 0, edge_exit_fint = 0;
    double edge_entry_hgap = 0, edge_exit_hgap = 0;
};

// Class-specific argument lists of the <Class>_track_local_particle
// functions (bend.h, quadrupole.h, sextupole.h, octupole.h, multipole.h and
// the slice headers).
MagnetIn magnet_inputs(const xtg_element& e) {
    MagnetIn m;
    m.length = e.length;
    m.order = e.order;
    m.inv_factorial_order = e.inv_factorial_order;
    m.knl = e.knl;
    m.ksl = e.ksl;
    m.order_rel = e.order_rel;
    m.knl_rel = e.knl_rel;
    m.ksl_rel = e.ksl_rel;
    m.rel_ref_strength = main_strength(e);
    m.num_multipole_kicks = e.num_multipole_kicks;
    m.model = e.model;
    m.integrator = e.integrator;
    switch (e.cls) {
    case XTG_CLS_BEND:
        m.default_model = kBendDefaultModel;
        m.default_integrator = kBendDefaultIntegrator;
        m.h = e.h; m.k0 = e.k0; m.k1 = e.k1; m.k2 = e.k2;
        m.edge_entry_active = e.edge_entry_active;
        m.edge_exit_active = e.edge_exit_active;
        m.edge_entry_model = e.edge_entry_model;
        m.edge_exit_model = e.edge_exit_model;
        m.edge_entry_angle = e.edge_entry_angle;
        m.edge_exit_angle = e.edge_exit_angle;
        m.edge_entry_angle_fdown = e.edge_entry_angle_fdown;
        m.edge_exit_angle_fdown = e.edge_exit_angle_fdown;
        m.edge_entry_fint = e.edge_entry_fint;
        m.edge_exit_fint = e.edge_exit_fint;
        m.edge_entry_hgap = e.edge_entry_hgap;
        m.edge_exit_hgap = e.edge_exit_hgap;
        break;
    case XTG_CLS_QUADRUPOLE:
        m.default_model = kQuadDefaultModel;
        m.default_integrator = kStraightDefaultIntegrator;
        m.k1 = e.k1; m.k1s = e.k1s;
        m.edge_entry_active = e.edge_entry_active;
        m.edge_exit_active = e.edge_exit_active;
        m.edge_entry_model = 1; m.edge_exit_model = 1;
        break;
    case XTG_CLS_SEXTUPOLE:
        m.default_model = kStraightDefaultModel;
        m.default_integrator = kStraightDefaultIntegrator;
        m.k2 = e.k2; m.k2s = e.k2s;
        m.edge_entry_active = e.edge_entry_active;
        m.edge_exit_active = e.edge_exit_active;
        m.edge_entry_model = 1; m.edge_exit_model = 1;
        break;
    case XTG_CLS_OCTUPOLE:
        m.default_model = kStraightDefaultModel;
        m.default_integrator = kStraightDefaultIntegrator;
        m.k3 = e.k3; m.k3s = e.k3s;
        m.edge_entry_active = e.edge_entry_active;
        m.edge_exit_active = e.edge_exit_active;
        m.edge_entry_model = 1; m.edge_exit_model = 1;
        break;
    case XTG_CLS_MULTIPOLE:
        m.default_model = kStraightDefaultModel;
        m.default_integrator = kStraightDefaultIntegrator;
        m.model = (e.isthick <= 0) ? -1 : e.model;
        m.hxl = e.hxl;
        break;
    default: break;
    }
    switch (e.slice) {
    case XTG_SLICE_THICK:
        m.weight = e.weight;
        m.edge_entry_active = m.edge_exit_active = 0;
        m.edge_entry_model = m.edge_exit_model = 0;
        break;
    case XTG_SLICE_THIN:
        m.weight = e.weight;
        m.num_multipole_kicks = 1;
        m.model = -1;
        m.integrator = 3;
        m.edge_entry_active = m.edge_exit_active = 0;
        break;
    case XTG_SLICE_ENTRY:
    case XTG_SLICE_EXIT: {
        bool entry = e.slice == XTG_SLICE_ENTRY;
        m.weight = 0.;
        m.num_multipole_kicks = 0;
        m.model = 0;
        m.integrator = 0;
        m.body_active = 0;
        if (entry) {
            m.edge_exit_active = 0;
            m.edge_exit_model = 0;
            m.edge_exit_angle = m.edge_exit_angle_fdown = 0;
            m.edge_exit_fint = m.edge_exit_hgap = 0;
        } else {
            m.edge_entry_active = 0;
            m.edge_entry_model = 0;
            m.edge_entry_angle = m.edge_entry_angle_fdown = 0;
            m.edge_entry_fint = m.edge_entry_hgap = 0;
        }
        break;
    }
    default: break;
    }
    return m;
}

// track_magnet_configure.h:6-194
struct Configured {
    int drift_model;
    double k0_drift, k1_drift, h_drift, k0_kick, k1_kick, h_kick;
    double k0_h_correction, k1_h_correction;
    int kick_rot_frame;
};

Configured configure(int64_t model, double k0, double k1, double h) {
    if (model == 1) model = 3;
    bool h_is_zero = std::fabs(h) < 1e-8;
    int dm;
    if (model == 2) dm = h_is_zero ? 5 : 4;
    else if (model == 3) dm = h_is_zero ? 1 : 7;
    else if (model == 4) dm = 3;
    else if (model == 5) dm = 1;
    else if (model == 6) dm = 0;
    else if (model == -1) dm = -1;
    else if (model == -2) dm = 6;
    else if (model == 7) dm = h_is_zero ? 1 : 2;
    else if (model == 8) dm = h_is_zero ? 1 : 8;
    else dm = 99999999;
    Configured c{};
    c.drift_model = dm;
    if (dm == -1 || dm == 0 || dm == 1) {
        c.k0_kick = k0; c.k1_kick = k1; c.h_kick = h;
        c.k0_h_correction = k0; c.k1_h_correction = k1; c.kick_rot_frame = 1;
    } else if (dm == 2) {
        c.h_drift = h; c.k0_kick = k0; c.k1_kick = k1; c.h_kick = h;
        c.k0_h_correction = k0; c.k1_h_correction = k1;
    } else if (dm == 3) {
        c.k0_drift = k0; c.k1_drift = k1; c.h_drift = h; c.h_kick = h;
        c.k1_h_correction = k1;
    } else if (dm == 4) {
        c.k0_drift = k0; c.h_drift = h; c.k1_kick = k1; c.h_kick = h;
        c.k1_h_correction = k1;
    } else if (dm == 5) {
        c.k0_drift = k0; c.k1_kick = k1;
    } else if (dm == 7 || dm == 8) {
        c.k0_drift = k0; c.h_drift = h; c.k1_kick = k1; c.h_kick = h;
        c.k0_h_correction = k0; c.k1_h_correction = k1;
    }
    return c;
}

// track_magnet_kick.h:149-179
bool kick_is_inactive(const MagnetIn& m) {
    if (m.h != 0 || m.k0 != 0 || m.k1 != 0 || m.k2 != 0 || m.k3 != 0) return false;
    if (m.k0s != 0 || m.k1s != 0 || m.k2s != 0 || m.k3s != 0) return false;
    for (int64_t i = m.order; i >= 0; i--) {
        if (m.knl[i] != 0 || m.ksl[i] != 0) return false;
    }
    return true;
}

// track_dipole_edge_linear.h:11-28 plus the k0 assembly of
// track_magnet_edge.h:41-50.
void edge_linear(const MagnetIn& m, bool exit, double factor_knl_ksl_edge,
                 double factor_for_backtrack, double* r21, double* r43) {
    double k0 = 0;
    k0 += m.k0;
    if (std::fabs(m.length) > 1e-10 && m.order > -1) {
        k0 += factor_knl_ksl_edge * m.knl[0] / m.length;
    }
    double const factor_rel = factor_knl_ksl_edge * m.rel_ref_strength;
    if (std::fabs(m.length) > 1e-10 && m.order_rel > -1 && m.knl_rel != nullptr) {
        k0 += factor_rel * m.knl_rel[0] / m.length;
    }
    double e1 = exit ? m.edge_exit_angle : m.edge_entry_angle;
    double e1_fd = exit ? m.edge_exit_angle_fdown : m.edge_entry_angle_fdown;
    double hgap = exit ? m.edge_exit_hgap : m.edge_entry_hgap;
    double fint = exit ? m.edge_exit_fint : m.edge_entry_fint;
    double const corr = 2.0 * k0 * hgap * fint;
    double const r21_out = k0 * std::tan(e1);
    double const e1_v = e1 + e1_fd;
    double const sin_e1_v = std::sin(e1_v);
    double const temp = corr / std::cos(e1_v) * (1.0 + sin_e1_v * sin_e1_v);
    double const r43_out = -k0 * std::tan(e1_v - temp);
    *r21 = r21_out * factor_for_backtrack;
    *r43 = r43_out * factor_for_backtrack;
}

// DipoleEdge full model (track_dipole_edge_nonlinear.h:9-44) in the
// dipole-only layout that fringe_edge runs: y-rotation by the face angle
// (skipped below 1e-9 rad, as the reference's sentinel test does), dipole
// fringe with k (-k at the exit), wedge by -e1 with k. The trigonometric
// values are evaluated here with the libm calls the reference makes.
std::vector<double> dipole_edge_fringe_block(const xtg_element& e) {
    std::vector<double> fr(FR_KNL, 0.0);
    bool const exit = e.side == 1;
    fr[FR_MODEL] = 2;
    fr[FR_IS_EXIT] = exit ? 1.0 : 0.0;
    fr[FR_K0] = exit ? -e.k : e.k;
    fr[FR_FINT] = e.fint;
    fr[FR_HGAP] = e.hgap;
    fr[FR_FACE_ANGLE] = e.e1;
    if (!(std::fabs(e.e1) < 10e-10)) {
        fr[FR_ROTATE] = 1.0;
        fr[FR_SIN] = std::sin(e.e1);
        fr[FR_COS] = std::cos(e.e1);
        fr[FR_TAN] = std::tan(e.e1);
    } else {
        fr[FR_ROTATE] = 0.0;
        fr[FR_SIN] = 0.0;
        fr[FR_COS] = 1.0;
        fr[FR_TAN] = 0.0;
    }
    double const theta = -e.e1;
    fr[FR_WSIN] = std::sin(theta);
    fr[FR_WCOS] = std::cos(theta);
    fr[FR_WTAN] = std::tan(theta);
    fr[FR_WSIN2] = std::sin(2 * theta);
    fr[FR_LENGTH] = 0.0;
    fr[FR_KL_ORDER] = -1.0;
    fr[FR_KNORM] = e.k;
    return fr;
}

// Parameter block of one nonlinear edge (track_magnet_edge.h:40-50 for the
// fringe's k0, 83-158 for the rest); layout FR_* of xtg_table.h. The
// trigonometric values of the face angle are evaluated here once, with the
// same libm calls the reference makes per particle.
std::vector<double> fringe_block(const MagnetIn& m, bool exit, int model, double factor_knl_ksl_edge) {
    std::vector<double> fr(FR_KNL, 0.0);
    double k0 = 0;
    k0 += m.k0;
    if (std::fabs(m.length) > 1e-10 && m.order > -1) {
        k0 += factor_knl_ksl_edge * m.knl[0] / m.length;
    }
    double const factor_rel = factor_knl_ksl_edge * m.rel_ref_strength;
    if (std::fabs(m.length) > 1e-10 && m.order_rel > -1 && m.knl_rel != nullptr) {
        k0 += factor_rel * m.knl_rel[0] / m.length;
    }
    if (exit) k0 = -k0;
    double const face = exit ? m.edge_exit_angle : m.edge_entry_angle;
    fr[FR_MODEL] = model;
    fr[FR_IS_EXIT] = exit ? 1.0 : 0.0;
    fr[FR_K0] = k0;
    fr[FR_FINT] = exit ? m.edge_exit_fint : m.edge_entry_fint;
    fr[FR_HGAP] = exit ? m.edge_exit_hgap : m.edge_entry_hgap;
    fr[FR_FACE_ANGLE] = face;
    if (std::fabs(face) > 10e-10) {
        fr[FR_ROTATE] = 1.0;
        fr[FR_SIN] = std::sin(face);
        fr[FR_COS] = std::cos(face);
        fr[FR_TAN] = std::tan(face);
    } else {
        fr[FR_ROTATE] = 0.0;
        fr[FR_SIN] = 0.0;
        fr[FR_COS] = 1.0;
        fr[FR_TAN] = 0.0;
    }
    double const theta = -face;
    fr[FR_WSIN] = std::sin(theta);
    fr[FR_WCOS] = std::cos(theta);
    fr[FR_WTAN] = std::tan(theta);
    fr[FR_WSIN2] = std::sin(2 * theta);
    fr[FR_LENGTH] = m.length / factor_knl_ksl_edge;
    fr[FR_KL_ORDER] = (double)m.order;
    double const kn[4] = {m.k0, m.k1, m.k2, m.k3};
    double const ks[4] = {m.k0s, m.k1s, m.k2s, m.k3s};
    for (int i = 0; i < 4; i++) {
        fr[FR_KNORM + i] = kn[i];
        fr[FR_KSKEW + i] = ks[i];
    }
    for (int64_t i = 0; i <= m.order; i++) fr.push_back(m.knl[i]);
    for (int64_t i = 0; i <= m.order; i++) fr.push_back(m.ksl[i]);
    return fr;
}

// Builds the reference-arithmetic coefficient quintuples of one
// kick_simple pass. Returns the effective top order (-1 when all zero).
int32_t exact_pass_coefs(int64_t order, double inv_factorial, const double* knl,
                         const double* ksl, double factor, std::vector<double>* out) {
    out->clear();
    if (order < 0 || knl == nullptr || ksl == nullptr) return -1;
    std::vector<double> invf(order + 1);
    invf[order] = inv_factorial;
    for (int64_t index = order; index > 0; index--) {
        invf[index - 1] = invf[index] * (double)index;   // inv_factorial *= index
    }
    int64_t top = -1;
    for (int64_t i = order; i >= 0; i--) {
        if (knl[i] != 0 || ksl[i] != 0) { top = i; break; }
    }
    for (int64_t i = top; i >= 0; i--) {
        double const a = (knl[i] * factor) * invf[i];   // (chi*knl*factor)*invf at chi = 1
        double const b = (ksl[i] * factor) * invf[i];
        out->push_back(a);
        out->push_back(b);
        out->push_back(knl[i]);
        out->push_back(ksl[i]);
        out->push_back(invf[i]);
    }
    return (int32_t)top;
}

}  // namespace

// Elements whose transverse shifts and s-tilts run through the straight
// misalignment of zero length (track_local_particle_with_transformations.h:
// 99-160, track_misalignments.h:38-130 at zero length, anchor, shift_s,
// rot_x_rad and rot_y_rad): the apertures, a thin Multipole (no `h` field,
// so not curved; `isthick` 0, so length 0) and DipoleEdge (no length).
static bool thin_straight(const xtg_element& e) {
    return e.cls == XTG_CLS_LIMIT_RECT || e.cls == XTG_CLS_LIMIT_ELLIPSE ||
           e.cls == XTG_CLS_LIMIT_POLYGON || e.cls == XTG_CLS_LIMIT_RECT_ELLIPSE ||
           e.cls == XTG_CLS_DIPOLE_EDGE ||
           (e.cls == XTG_CLS_MULTIPOLE && e.isthick <= 0 && e.slice == XTG_SLICE_NONE);
}

// --------------------------------------------------------------------------
int32_t validate_element(const xtg_element& e, int64_t idx, std::string* why) {
    auto fail = [&](const char* m) {
        *why = "element " + std::to_string(idx) + ": " + m;
        return (int32_t)XTG_E_UNSUPPORTED;
    };
    if (e.cls < 0 || e.cls >= XTG_NUM_CLS) return fail("unknown element class");
    if (e.slice < 0 || e.slice > XTG_SLICE_EXIT) return fail("unknown slice kind");
    if (e.order < 0 || e.order >= XTG_MAX_KNL) return fail("multipole order out of range");
    if (e.order_rel < -1 || e.order_rel >= 20)
        return fail("relative multipole order out of range (0..19)");
    bool const movable = thin_straight(e);
    if (!movable && (e.shift_x != 0 || e.shift_y != 0))
        return fail("misalignments (shift/rotation) are not supported (transverse shifts: apertures, "
                    "thin Multipoles and DipoleEdges only)");
    if (!movable && (e.rot_s_rad != 0 || e.rot_s_rad_no_frame != 0))
        return fail("misalignments (shift/rotation) are not supported (transverse shifts and tilts: "
                    "apertures, thin Multipoles and DipoleEdges only)");
    if (e.shift_s != 0 || e.rot_x_rad != 0 || e.rot_y_rad != 0)
        return fail("misalignments (shift/rotation) are not supported (transverse shifts and tilts: "
                    "apertures, thin Multipoles and DipoleEdges only)");
    if (e.cls >= XTG_CLS_MULTIPOLE && e.cls <= XTG_CLS_OCTUPOLE) {
        int64_t model = e.model;
        if (e.cls == XTG_CLS_MULTIPOLE && e.isthick <= 0) model = -1;
        if (model == 0) model = (e.cls == XTG_CLS_BEND) ? 3 : (e.cls == XTG_CLS_QUADRUPOLE) ? 4 : 6;
        if (model == -2) return fail("solenoid model is not supported");
        if (model < -1 || model > 8) return fail("unknown magnet model");
        if (e.integrator < 0 || e.integrator > 3) return fail("unknown integrator");
        bool entry = e.edge_entry_active && (e.slice == XTG_SLICE_NONE || e.slice == XTG_SLICE_ENTRY);
        bool exit_ = e.edge_exit_active && (e.slice == XTG_SLICE_NONE || e.slice == XTG_SLICE_EXIT);
        int em_in = (e.cls == XTG_CLS_BEND) ? e.edge_entry_model : 1;
        int em_out = (e.cls == XTG_CLS_BEND) ? e.edge_exit_model : 1;
        if (e.cls == XTG_CLS_MULTIPOLE) entry = exit_ = false;
        if ((entry && (em_in < -1 || em_in > 3)) || (exit_ && (em_out < -1 || em_out > 3)))
            return fail("unknown edge model");
        if (e.slice == XTG_SLICE_ENTRY || e.slice == XTG_SLICE_EXIT) {
            if (e.cls == XTG_CLS_MULTIPOLE) return fail("Multipole has no entry/exit slices");
        }
    } else if (e.cls == XTG_CLS_CAVITY) {
        int64_t model = e.model == 0 ? 6 : e.model;
        if (!(model == -1 || model == 4 || model == 5 || model == 6))
            return fail("unsupported cavity model");
        if (e.integrator < 0 || e.integrator > 3) return fail("unknown integrator");
        if (e.slice == XTG_SLICE_ENTRY || e.slice == XTG_SLICE_EXIT)
            return fail("Cavity has no entry/exit slices");
    } else if (e.slice != XTG_SLICE_NONE) {
        return fail("slice kind not valid for this class");
    }
    if (e.cls == XTG_CLS_DIPOLE_EDGE) {
        if (e.model < -1 || e.model > 1) return fail("unknown DipoleEdge model (linear, full, suppressed)");
        if (e.side != 0 && e.side != 1) return fail("DipoleEdge side must be 0 (entry) or 1 (exit)");
    }
    if (e.cls == XTG_CLS_LIMIT_POLYGON) {
        const xtg_polygon* pg = reinterpret_cast<const xtg_polygon*>(e.aux);
        if (!pg) return fail("LimitPolygon without its vertices");
        if (pg->n_vertices < 3 || !pg->x_vertices || !pg->y_vertices)
            return fail("LimitPolygon needs at least 3 vertices");
    }
    if (e.cls == XTG_CLS_MONITOR) {
        const xtg_element_monitor* m = reinterpret_cast<const xtg_element_monitor*>(e.aux);
        if (!m) return fail("monitor element without its descriptor");
        if (m->kind == XTG_MON_LAST_TURNS) {
            if (m->n_last_turns < 1 || m->every_n_turns < 1 || m->num_particles < 0)
                return fail("LastTurnsMonitor needs n_last_turns >= 1, every_n_turns >= 1");
            if (m->num_particles > 0 && (!m->lost_at_offset || !m->lt_particle_id || !m->lt_at_turn ||
                                         !m->lt_x || !m->lt_px || !m->lt_y || !m->lt_py ||
                                         !m->lt_delta || !m->lt_zeta))
                return fail("LastTurnsMonitor with a NULL buffer");
        } else if (m->kind == XTG_MON_BEAM_POSITION || m->kind == XTG_MON_BEAM_SIZE) {
            if (m->n_slots < 0) return fail("beam position/size monitor with a negative size");
            if (m->n_slots > 0 && (!m->count || !m->x_sum || !m->y_sum))
                return fail("beam position/size monitor with a NULL buffer");
            if (m->kind == XTG_MON_BEAM_SIZE && m->n_slots > 0 && (!m->x2_sum || !m->y2_sum))
                return fail("BeamSizeMonitor with a NULL buffer");
        } else if (m->kind == XTG_MON_BEAM_PROFILE) {
            if (m->n_slots < 0 || m->nx < 0 || m->ny < 0)
                return fail("BeamProfileMonitor with a negative size");
            if (m->n_slots > 0 && ((m->nx > 0 && !m->counts_x) || (m->ny > 0 && !m->counts_y)))
                return fail("BeamProfileMonitor with a NULL buffer");
        } else if (m->kind == XTG_MON_PARTICLES) {
            if (m->particles.n_records < 0) return fail("ParticlesMonitor with a negative size");
            if (m->particles.n_repetitions > 1 && m->particles.repetition_period <= 0)
                return fail("ParticlesMonitor repetition_period must be > 0");
        } else {
            return fail("unknown monitor kind");
        }
    }
    return XTG_OK;
}

namespace {

void pack_drift(double length, bool exact, bool global_aper, RecBuf* rb) {
    rb->init(sizeof(DriftRec));
    DriftRec* r = rb->head<DriftRec>();
    r->h.op = OP_DRIFT;
    r->h.flags = global_aper ? F_GLOBAL_APER : 0;
    r->length = length;
    r->exact = exact ? 1 : 0;
}

void pack_magnet(const xtg_element& e, bool backtrack, bool exact, RecBuf* rb) {
    MagnetIn m = magnet_inputs(e);
    const bool statically_thick =
        (e.slice == XTG_SLICE_NONE && e.cls != XTG_CLS_MULTIPOLE) || e.slice == XTG_SLICE_THICK;

    // track_magnet.h:414-442 backtracking
    double const factor_knl_ksl = 1.0;
    double core_length, factor_body, factor_edge, factor_bt_edge;
    if (backtrack) {
        core_length = -m.length * m.weight;
        factor_body = -factor_knl_ksl * m.weight;
        factor_edge = factor_knl_ksl;
        factor_bt_edge = -1.;
        m.hxl = -m.hxl;
        std::swap(m.edge_entry_active, m.edge_exit_active);
        std::swap(m.edge_entry_model, m.edge_exit_model);
        std::swap(m.edge_entry_angle, m.edge_exit_angle);
        std::swap(m.edge_entry_angle_fdown, m.edge_exit_angle_fdown);
        std::swap(m.edge_entry_fint, m.edge_exit_fint);
        std::swap(m.edge_entry_hgap, m.edge_exit_hgap);
    } else {
        core_length = m.length * m.weight;
        factor_body = factor_knl_ksl * m.weight;
        factor_edge = factor_knl_ksl;
        factor_bt_edge = 1.;
    }

    rb->init(sizeof(MagnetRec));
    size_t const coef_base = sizeof(MagnetRec);
    {
        MagnetRec* r = rb->head<MagnetRec>();
        r->h.op = OP_MAGNET;
        r->h.flags = statically_thick ? F_GLOBAL_APER : 0;
        r->fast_top = -1;
        for (int p = 0; p < 3; p++) r->pass[p].top = -1;
    }
    auto R = [&]() { return rb->head<MagnetRec>(); };

    // edges (track_magnet_edge.h:16-80)
    // A linear edge whose coefficients are both zero adds (+-0)*x to px and
    // py, which leaves them unchanged: only its ax/ay reset remains.
    if (m.edge_entry_active) {
        R()->edge_entry = EDGE_AXAY;   // suppressed / ax-ay-only models
        if (m.edge_entry_model == 0) {
            double r21, r43;
            edge_linear(m, false, factor_edge, factor_bt_edge, &r21, &r43);
            if (r21 != 0 || r43 != 0) R()->edge_entry = EDGE_LINEAR;
            R()->entry_r21 = r21;
            R()->entry_r43 = r43;
        }
    }
    if (m.edge_exit_active) {
        R()->edge_exit = EDGE_AXAY;
        if (m.edge_exit_model == 0) {
            double r21, r43;
            edge_linear(m, true, factor_edge, factor_bt_edge, &r21, &r43);
            if (r21 != 0 || r43 != 0) R()->edge_exit = EDGE_LINEAR;
            R()->exit_r21 = r21;
            R()->exit_r43 = r43;
        }
    }
    // nonlinear edges (full / dipole-only models): parameter blocks
    R()->backtrack = backtrack ? 1 : 0;
    if (m.edge_entry_active && (m.edge_entry_model == 1 || m.edge_entry_model == 2)) {
        std::vector<double> fr = fringe_block(m, false, m.edge_entry_model, factor_edge);
        rb->pad16();
        int32_t off = rb->append(fr.data(), fr.size(), coef_base);
        R()->edge_entry = EDGE_FRINGE;
        R()->entry_fringe = off;
    }
    if (m.edge_exit_active && (m.edge_exit_model == 1 || m.edge_exit_model == 2)) {
        std::vector<double> fr = fringe_block(m, true, m.edge_exit_model, factor_edge);
        rb->pad16();
        int32_t off = rb->append(fr.data(), fr.size(), coef_base);
        R()->edge_exit = EDGE_FRINGE;
        R()->exit_fringe = off;
    }

    if (m.body_active) {
        int64_t integrator = m.integrator;
        int64_t model = m.model;
        int64_t n = m.num_multipole_kicks;
        if (integrator == 0) integrator = m.default_integrator;
        if (model == 0) model = m.default_model;
        if (model == -1) {
            integrator = 3;
            n = 1;
        }
        if (m.weight != 1.0 && n > 0) n = (int64_t)std::ceil(n * m.weight);
        if (n == 0) {
            if (!kick_is_inactive(m)) {
                if (std::fabs(m.h) < 1e-8) {
                    n = 1;
                } else {
                    double b_circum = 2 * 3.14159 / std::fabs(m.h);
                    n = (int64_t)(std::fabs(core_length) / b_circum / 0.5e-3);
                    if (n < 1) n = 1;
                }
            }
        }
        Configured c = configure(model, m.k0, m.k1, m.h);
        MagnetRec* r = R();
        r->body_active = 1;
        r->integrator = (int32_t)integrator;
        r->n_kicks = (int32_t)n;
        r->drift_model = c.drift_model;
        r->kick_rot_frame = c.kick_rot_frame;
        r->length = core_length;
        r->k0_drift = c.k0_drift;
        r->k1_drift = c.k1_drift;
        r->h_drift = c.h_drift;
        r->only_drift = (n == 0 && c.k0_kick == 0 && c.k1_kick == 0 && c.h_kick == 0) ? 1 : 0;

        // kick weights and drift lengths (track_magnet.h:192-277)
        double kw[4] = {0, 0, 0, 0};
        int n_kw = 1;
        if (n > 0) {
            if (integrator == INT_TEAPOT) {
                kw[0] = 1. / n;
                double edge_w = 0.5, inside_w = 0;
                if (n > 1) {
                    edge_w = 1. / (2 * (1 + n));
                    inside_w = (((double)n) / ((double)(n * n) - 1));
                }
                r->d_edge = edge_w * core_length;
                r->d_inside = inside_w * core_length;
            } else if (integrator == INT_UNIFORM) {
                kw[0] = 1. / n;
                double const drift_weight = kw[0];
                r->d_edge = 0.5 * drift_weight * core_length;
                r->d_inside = 0;
                r->d_fast_inside = drift_weight * core_length;
            } else if (integrator == INT_YOSHIDA4) {
                int64_t const num_slices = (n / 7 + (n % 7 != 0));
                double const slice_length = core_length / (num_slices);
                double const kick_weight = 1. / num_slices;
                for (int i = 0; i < 4; i++) {
                    r->d_yoshida[i] = slice_length * kDYoshida[i];
                    kw[i] = kick_weight * kKYoshida[i];
                }
                n_kw = 4;
                r->n_kicks = (int32_t)num_slices;   // slices of 7 kicks
            }
        }
        r->n_kw = n_kw;

        // curvature constants (track_magnet_kick.h:97-139)
        double const L = core_length;
        double const h = c.h_kick;
        double htot = h;
        if (L != 0) htot += m.hxl / L;
        double k0l_mult = 0;
        if (m.order >= 0) k0l_mult = m.knl[0] * factor_body;
        if (m.order_rel >= 0 && m.knl_rel != nullptr)
            k0l_mult += m.knl_rel[0] * factor_body * m.rel_ref_strength;
        double k1l_mult = 0;
        if (m.order >= 1) k1l_mult = m.knl[1] * factor_body;
        if (m.order_rel >= 1 && m.knl_rel != nullptr)
            k1l_mult += m.knl_rel[1] * factor_body * m.rel_ref_strength;
        double const Q0 = c.k0_h_correction * L + k0l_mult;
        double const Q1 = c.k1_h_correction * L + k1l_mult;
        r->htot = htot;
        r->Q0 = Q0;
        r->Q1 = Q1;
        int curv = 0;
        for (int k = 0; k < n_kw; k++) {
            r->kw[k] = kw[k];
            r->hl[k] = h * L * kw[k] + m.hxl * kw[k];
            r->C0[k] = ((-Q0) * kw[k]) * htot;   // (-chi*Q0*kw)*htot at chi = 1
            r->C1[k] = (htot * Q1) * kw[k];      // (htot*chi*Q1)*kw at chi = 1
            r->fast_scale[k] = (kw[0] != 0) ? kw[k] / kw[0] : 0.;
            if (c.kick_rot_frame && r->hl[k] != 0) curv |= 1;
            if (htot != 0 && Q0 != 0) curv |= 2;
            if (htot != 0 && Q1 != 0) curv |= 4;
        }
        r->curv_terms = curv;

        // exact kick passes (track_magnet_kick.h:67-94)
        std::vector<double> coefs;
        int32_t top;
        // Only the arithmetic mode of the table stores its coefficients; the
        // orders are kept in both (they also drive the FLOP accounting).
        top = exact_pass_coefs(m.order, m.inv_factorial_order, m.knl, m.ksl, factor_body, &coefs);
        if (!exact) coefs.clear();
        {
            int32_t off = rb->append(coefs.data(), coefs.size(), coef_base);
            R()->pass[0].top = top;
            R()->pass[0].coef = off;
            R()->pass[0].factor = factor_body;
        }
        double const factor_rel = factor_body * m.rel_ref_strength;
        top = exact_pass_coefs(m.order_rel, one_over_factorial(m.order_rel), m.knl_rel,
                               m.ksl_rel, factor_rel, &coefs);
        if (!exact) coefs.clear();
        {
            int32_t off = rb->append(coefs.data(), coefs.size(), coef_base);
            R()->pass[1].top = top;
            R()->pass[1].coef = off;
            R()->pass[1].factor = factor_rel;
        }
        double knl_main[4] = {c.k0_kick, c.k1_kick, m.k2, m.k3};
        double ksl_main[4] = {m.k0s, m.k1s, m.k2s, m.k3s};
        for (int i = 0; i < 4; i++) {
            knl_main[i] = knl_main[i] * L;
            ksl_main[i] = ksl_main[i] * L;
        }
        top = exact_pass_coefs(3, 1. / (3 * 2), knl_main, ksl_main, 1, &coefs);
        if (!exact) coefs.clear();
        {
            int32_t off = rb->append(coefs.data(), coefs.size(), coef_base);
            R()->pass[2].top = top;
            R()->pass[2].coef = off;
            R()->pass[2].factor = 1.0;
        }

        // merged polynomial for the fast path:
        // c_i = kw0 * (knl_i*f/i! + knl_rel_i*f_rel/i! + knl_main_i/i!)
        int fmax = (int)std::max<int64_t>(std::max<int64_t>(m.order, m.order_rel), 3);
        std::vector<double> cn(fmax + 1, 0.), cs(fmax + 1, 0.);
        for (int i = 0; i <= fmax; i++) {
            double const inv = one_over_factorial(i);
            if (i <= m.order) {
                cn[i] += m.knl[i] * factor_body * inv;
                cs[i] += m.ksl[i] * factor_body * inv;
            }
            if (m.order_rel >= 0 && i <= m.order_rel) {
                cn[i] += m.knl_rel[i] * factor_rel * inv;
                cs[i] += m.ksl_rel[i] * factor_rel * inv;
            }
            if (i <= 3) {
                cn[i] += knl_main[i] * inv;
                cs[i] += ksl_main[i] * inv;
            }
        }
        int ftop = -1;
        for (int i = fmax; i >= 0; i--) {
            if (cn[i] != 0 || cs[i] != 0) { ftop = i; break; }
        }
        std::vector<double> fc;
        for (int i = ftop; i >= 0 && !exact; i--) {
            fc.push_back(cn[i] * kw[0]);
            fc.push_back(cs[i] * kw[0]);
        }
        rb->pad16();   // (cn_i, cs_i) pairs are read as 16-byte vectors
        int32_t off = rb->append(fc.data(), fc.size(), coef_base);
        R()->fast_top = ftop;
        R()->fast_coef = off;
    }
    rb->pad16();

    // A lone kick without edges gets the compact record (same coefficients).
    const MagnetRec* r = R();
    if (r->body_active && r->edge_entry == EDGE_NONE && r->edge_exit == EDGE_NONE &&
        r->drift_model == -1 && r->only_drift == 0 && r->n_kicks == 1 &&
        r->integrator == INT_UNIFORM) {
        RecBuf kb;
        kb.init(sizeof(KickRec));
        KickRec* k = kb.head<KickRec>();
        k->h = r->h;
        k->h.op = OP_KICK;
        k->fast_top = r->fast_top;
        k->fast_coef = r->fast_coef;
        k->curv_terms = r->curv_terms;
        for (int q = 0; q < 3; q++) k->pass[q] = r->pass[q];
        k->kw = r->kw[0];
        k->hl = r->hl[0];
        k->C0 = r->C0[0];
        k->C1 = r->C1[0];
        k->htot = r->htot;
        k->Q0 = r->Q0;
        k->Q1 = r->Q1;
        size_t const ncoef = (rb->bytes.size() - coef_base) / sizeof(double);
        kb.append(reinterpret_cast<const double*>(rb->bytes.data() + coef_base), ncoef,
                  sizeof(KickRec));
        kb.pad16();
        rb->bytes.swap(kb.bytes);
    }
}

void pack_cavity(const xtg_element& e, bool backtrack, RecBuf* rb) {
    // cavity.h:11-48 and slices, track_rf.h:293-453
    double weight = 1.0;
    int64_t num_kicks = e.num_multipole_kicks;
    int64_t model = e.model;
    int64_t integrator = e.integrator;
    bool thick = true;
    if (e.slice == XTG_SLICE_THICK) {
        weight = e.weight;
    } else if (e.slice == XTG_SLICE_THIN) {
        weight = e.weight;
        num_kicks = 1;
        model = -1;
        integrator = 3;
        thick = false;
    }
    double voltage = e.voltage;
    double body_length;
    if (backtrack) {
        body_length = -e.length;
        voltage = -voltage;
    } else {
        body_length = e.length;
    }
    if (integrator == 0) integrator = 3;
    if (model == 0) model = 6;
    if (model == -1) {
        integrator = 3;
        num_kicks = 1;
    }
    if (weight != 1.0 && num_kicks > 0) num_kicks = (int64_t)std::ceil(num_kicks * weight);
    if (num_kicks == 0) num_kicks = 1;
    Configured c = configure(model, 0, 0, 0);

    rb->init(sizeof(CavityRec));
    CavityRec* r = rb->head<CavityRec>();
    r->h.op = OP_CAVITY;
    r->h.flags = thick ? F_GLOBAL_APER : 0;
    r->integrator = (int32_t)integrator;
    r->n_kicks = (int32_t)num_kicks;
    r->drift_model = c.drift_model;
    r->absolute_time = (int32_t)e.absolute_time;
    double const length = body_length * weight;
    r->length = length;
    r->voltage = voltage * weight;
    int64_t const n = num_kicks;
    if (integrator == INT_TEAPOT) {
        r->kw[0] = 1. / n;
        double edge_w = 0.5, inside_w = 0;
        if (n > 1) {
            edge_w = 1. / (2 * (1 + n));
            inside_w = (((double)n) / ((double)(n * n) - 1));
        }
        r->d_edge = edge_w * length;
        r->d_inside = inside_w * length;
    } else if (integrator == INT_UNIFORM) {
        r->kw[0] = 1. / n;
        r->d_edge = 0.5 * r->kw[0] * length;
    } else if (integrator == INT_YOSHIDA4) {
        int64_t const num_slices = (n / 7 + (n % 7 != 0));
        double const slice_length = length / (num_slices);
        double const kick_weight = 1. / num_slices;
        for (int i = 0; i < 4; i++) {
            r->d_yoshida[i] = slice_length * kDYoshida[i];
            r->kw[i] = kick_weight * kKYoshida[i];
        }
        r->n_kicks = (int32_t)num_slices;
    }
    r->frequency = e.frequency;
    r->harmonic = e.harmonic;
    r->lag_rad = kDeg2Rad * e.lag;
    r->phase = e.phase;
    r->phi_const = 0 + kDeg2Rad * e.lag + e.phase;
    r->w_freq = (2.0 * kPi) / kCLight * e.frequency;
    rb->pad16();
}

}  // namespace

int32_t pack_lattice(const xtg_element* els, int64_t n, const xtg_config& cfg,
                     bool backtrack, PackedLattice* out, std::string* err) {
    out->bytes.clear();
    out->offsets.assign(n + 1, 0);
    out->flops_fast.assign(n, 0.);
    RecBuf rb;
    for (int64_t k = 0; k < n; k++) {
        // the backtracking table holds the elements in reverse order
        int64_t const i = backtrack ? (n - 1 - k) : k;
        const xtg_element& e = els[i];
        int32_t st = validate_element(e, i, err);
        if (st != XTG_OK) return st;
        switch (e.cls) {
        case XTG_CLS_MARKER:
            rb.init(sizeof(RecHeader));
            rb.head<RecHeader>()->op = OP_NOP;
            break;
        case XTG_CLS_DRIFT: {
            // drift.h:13-37
            double length = e.length;
            if (backtrack) length = -length;
            int model;
            if (cfg.use_exact_drifts) model = 2;
            else {
                model = e.model;
                if (model == 0) model = 1;
            }
            if (model == 1 || model == 2) pack_drift(length, model == 2, true, &rb);
            else {
                rb.init(sizeof(RecHeader));
                rb.head<RecHeader>()->op = OP_NOP;
                rb.head<RecHeader>()->flags = F_GLOBAL_APER;
            }
            break;
        }
        case XTG_CLS_LIMIT_ELLIPSE: {
            rb.init(sizeof(LimitEllipseRec));
            LimitEllipseRec* r = rb.head<LimitEllipseRec>();
            r->h.op = OP_LIMIT_ELLIPSE;
            r->a_squ = e.a_squ;
            r->b_squ = e.b_squ;
            r->key_a_b_squ = upper_key(e.a_b_squ);
            break;
        }
        case XTG_CLS_MONITOR: {
            // monitors are replaced by markers in backtracking tables
            // (get_backtrack_element of monitors/*.py)
            const xtg_element_monitor* m = reinterpret_cast<const xtg_element_monitor*>(e.aux);
            if (backtrack) {
                rb.init(sizeof(RecHeader));
                rb.head<RecHeader>()->op = OP_NOP;
            } else if (m->kind == XTG_MON_PARTICLES) {
                rb.init(sizeof(MonParticlesRec));
                MonParticlesRec* r = rb.head<MonParticlesRec>();
                r->h.op = OP_MON_PARTICLES;
                r->m = m->particles;
            } else if (m->kind == XTG_MON_LAST_TURNS) {
                rb.init(sizeof(MonLastTurnsRec));
                MonLastTurnsRec* r = rb.head<MonLastTurnsRec>();
                r->h.op = OP_MON_LAST_TURNS;
                r->particle_id_start = m->particle_id_start;
                r->particle_id_stop = m->particle_id_start + m->num_particles;
                r->n_last_turns = m->n_last_turns;
                r->every_n_turns = m->every_n_turns;
                r->lost_at_offset = m->lost_at_offset;
                r->particle_id = m->lt_particle_id;
                r->at_turn = m->lt_at_turn;
                r->x = m->lt_x;
                r->px = m->lt_px;
                r->y = m->lt_y;
                r->py = m->lt_py;
                r->delta = m->lt_delta;
                r->zeta = m->lt_zeta;
            } else if (m->kind == XTG_MON_BEAM_PROFILE) {
                rb.init(sizeof(MonProfileRec));
                MonProfileRec* r = rb.head<MonProfileRec>();
                r->h.op = OP_MON_PROFILE;
                r->particle_id_start = m->particle_id_start;
                r->particle_id_stop = m->particle_id_start + m->num_particles;
                r->start_at_turn = m->start_at_turn;
                r->sample_size = m->n_slots;
                r->frev = m->frev;
                r->sampling_frequency = m->sampling_frequency;
                r->nx = m->nx;
                r->ny = m->ny;
                r->x_min = m->x_min;
                r->dx = m->dx;
                r->y_min = m->y_min;
                r->dy = m->dy;
                r->counts_x = m->counts_x;
                r->counts_y = m->counts_y;
            } else {
                rb.init(sizeof(MonBpmRec));
                MonBpmRec* r = rb.head<MonBpmRec>();
                r->h.op = OP_MON_BPM;
                if (m->kind == XTG_MON_BEAM_SIZE) {
                    r->x2_sum = m->x2_sum;
                    r->y2_sum = m->y2_sum;
                }
                r->particle_id_start = m->particle_id_start;
                r->particle_id_stop = m->particle_id_start + m->num_particles;
                r->start_at_turn = m->start_at_turn;
                r->n_slots = m->n_slots;
                r->frev = m->frev;
                r->sampling_frequency = m->sampling_frequency;
                r->count = m->count;
                r->x_sum = m->x_sum;
                r->y_sum = m->y_sum;
            }
            break;
        }
        case XTG_CLS_LIMIT_POLYGON: {
            // limitpolygon.h:13-90; the inscribed-circle radius of the CPU
            // build is computed here once (limitpolygon.h:27-62)
            const xtg_polygon* pg = reinterpret_cast<const xtg_polygon*>(e.aux);
            int64_t const nv = pg->n_vertices;
            double inner_radius_sq = 0.0;
            for (int64_t ii = 0; ii < nv; ii++) {
                int64_t const jj = (ii + 1) % nv;
                double const x0 = pg->x_vertices[ii], y0 = pg->y_vertices[ii];
                double const x1 = pg->x_vertices[jj], y1 = pg->y_vertices[jj];
                double const dx = x1 - x0;
                double const dy = y1 - y0;
                double const seg_len_sq = dx * dx + dy * dy;
                double dist_sq;
                if (seg_len_sq > 0.0) {
                    double t = -(x0 * dx + y0 * dy) / seg_len_sq;
                    if (t < 0.0) t = 0.0;
                    else if (t > 1.0) t = 1.0;
                    double const xp = x0 + t * dx;
                    double const yp = y0 + t * dy;
                    dist_sq = xp * xp + yp * yp;
                } else {
                    dist_sq = x0 * x0 + y0 * y0;
                }
                if (ii == 0 || dist_sq < inner_radius_sq) inner_radius_sq = dist_sq;
            }
            rb.init(sizeof(LimitPolygonRec));
            LimitPolygonRec* r = rb.head<LimitPolygonRec>();
            r->h.op = OP_LIMIT_POLYGON;
            r->n = nv;
            r->inner_radius_sq = inner_radius_sq;
            rb.append(pg->x_vertices, (size_t)nv, sizeof(LimitPolygonRec));
            rb.append(pg->y_vertices, (size_t)nv, sizeof(LimitPolygonRec));
            rb.pad16();
            break;
        }
        case XTG_CLS_DIPOLE_EDGE: {
            // dipoleedge.h:14-71: model -1 does nothing
            if (e.model == -1) {
                rb.init(sizeof(RecHeader));
                rb.head<RecHeader>()->op = OP_NOP;
                break;
            }
            rb.init(sizeof(DipoleEdgeRec));
            rb.head<DipoleEdgeRec>()->h.op = OP_DIPOLE_EDGE;
            rb.head<DipoleEdgeRec>()->model = e.model;
            rb.head<DipoleEdgeRec>()->backtrack = backtrack ? 1 : 0;
            if (e.model == 0) {
                // the linear coefficients change sign when backtracking
                rb.head<DipoleEdgeRec>()->r21 = backtrack ? -e.r21 : e.r21;
                rb.head<DipoleEdgeRec>()->r43 = backtrack ? -e.r43 : e.r43;
            } else {
                std::vector<double> fr = dipole_edge_fringe_block(e);
                rb.pad16();
                int32_t const off = rb.append(fr.data(), fr.size(), sizeof(DipoleEdgeRec));
                rb.head<DipoleEdgeRec>()->fringe = off;
            }
            break;
        }
        case XTG_CLS_LIMIT_RECT_ELLIPSE: {
            rb.init(sizeof(LimitRectEllipseRec));
            LimitRectEllipseRec* r = rb.head<LimitRectEllipseRec>();
            r->h.op = OP_LIMIT_RECT_ELLIPSE;
            r->key_min_x = lower_key(-e.max_x);
            r->key_max_x = upper_key(e.max_x);
            r->key_min_y = lower_key(-e.max_y);
            r->key_max_y = upper_key(e.max_y);
            r->a_squ = e.a_squ;
            r->b_squ = e.b_squ;
            r->key_a_b_squ = upper_key(e.a_b_squ);
            break;
        }
        case XTG_CLS_LIMIT_RECT: {
            rb.init(sizeof(LimitRectRec));
            LimitRectRec* r = rb.head<LimitRectRec>();
            r->h.op = OP_LIMIT_RECT;
            r->key_min_x = lower_key(e.min_x);
            r->key_max_x = upper_key(e.max_x);
            r->key_min_y = lower_key(e.min_y);
            r->key_max_y = upper_key(e.max_y);
            break;
        }
        case XTG_CLS_CAVITY:
            if (e.slice == XTG_SLICE_DRIFT) {
                double length = e.weight * e.length;
                if (backtrack) length = -e.weight * e.length;
                pack_drift(length, cfg.use_exact_drifts != 0, true, &rb);
            } else {
                pack_cavity(e, backtrack, &rb);
            }
            break;
        default:   // magnets
            if (e.slice == XTG_SLICE_DRIFT) {
                double length = e.weight * e.length;
                if (backtrack) length = -e.weight * e.length;
                pack_drift(length, cfg.use_exact_drifts != 0, true, &rb);
            } else {
                pack_magnet(e, backtrack, cfg.arith == XTG_ARITH_EXACT, &rb);
            }
            break;
        }
        if (thin_straight(e) &&
            (e.shift_x != 0.0 || e.shift_y != 0.0 || e.rot_s_rad != 0.0 || e.rot_s_rad_no_frame != 0.0)) {
            // the kernel applies the block on these records only
            int32_t const op = rb.head<RecHeader>()->op;
            if (!(op == OP_KICK || op == OP_NOP || op == OP_DIPOLE_EDGE || op == OP_LIMIT_RECT ||
                  op == OP_LIMIT_ELLIPSE || op == OP_LIMIT_POLYGON || op == OP_LIMIT_RECT_ELLIPSE)) {
                *err = "element " + std::to_string(i) +
                       ": misalignments (shift/rotation) are not supported on this record kind";
                return (int32_t)XTG_E_UNSUPPORTED;
            }
            // entry and exit of track_misalignment_entry/exit_straight with
            // zero anchor, shift_s, rot_x_rad and rot_y_rad
            double const mis_in_x = e.shift_x - 0.0, mis_in_y = e.shift_y - 0.0;
            double const mis_out_x = 0.0 - e.shift_x, mis_out_y = 0.0 - e.shift_y;
            ApertureShift sh;
            std::memset(&sh, 0, sizeof(sh));
            // S_ROTATE(psi_no_frame), S_ROTATE(psi_with_frame) at the entry;
            // S_ROTATE(-psi_with_frame), S_ROTATE(-psi_no_frame) at the exit
            // (the same order in backtracking tables)
            double const psi_nf = e.rot_s_rad_no_frame, psi_wf = e.rot_s_rad;
            if (psi_nf != 0.0) {
                sh.rot_in[sh.n_rot_in][0] = std::sin(psi_nf);
                sh.rot_in[sh.n_rot_in][1] = std::cos(psi_nf);
                sh.n_rot_in++;
            }
            if (psi_wf != 0.0) {
                sh.rot_in[sh.n_rot_in][0] = std::sin(psi_wf);
                sh.rot_in[sh.n_rot_in][1] = std::cos(psi_wf);
                sh.n_rot_in++;
            }
            if (psi_wf != 0.0) {
                sh.rot_out[sh.n_rot_out][0] = std::sin(-psi_wf);
                sh.rot_out[sh.n_rot_out][1] = std::cos(-psi_wf);
                sh.n_rot_out++;
            }
            if (psi_nf != 0.0) {
                sh.rot_out[sh.n_rot_out][0] = std::sin(-psi_nf);
                sh.rot_out[sh.n_rot_out][1] = std::cos(-psi_nf);
                sh.n_rot_out++;
            }
            if (!backtrack) {
                sh.in_x = -mis_in_x;
                sh.in_y = -mis_in_y;
                sh.out_x = -mis_out_x;
                sh.out_y = -mis_out_y;
            } else {
                sh.in_x = -(-mis_out_x);
                sh.in_y = -(-mis_out_y);
                sh.out_x = -(-mis_in_x);
                sh.out_y = -(-mis_in_y);
            }
            rb.pad16();
            size_t const off = rb.bytes.size();
            rb.bytes.resize(off + sizeof(ApertureShift));
            std::memcpy(rb.bytes.data() + off, &sh, sizeof(sh));
            rb.head<RecHeader>()->flags |= F_SHIFTED;
        }
        rb.pad16();
        rb.head<RecHeader>()->nbytes = (int32_t)rb.bytes.size();
        out->offsets[k] = (int64_t)out->bytes.size();
        out->bytes.insert(out->bytes.end(), rb.bytes.begin(), rb.bytes.end());
        out->flops_fast[k] = canonical_flops(rb.bytes.data());
    }
    out->offsets[n] = (int64_t)out->bytes.size();
    return XTG_OK;
}

// Canonical minimal FP64 operation count of one element for one particle
// (FMA = 2 FLOPs; add, mul = 1; div, sqrt, sin, cos = 1):
//   expanded drift 16: xp, yp (2 mul), t = xp^2+yp^2 (mul+fma), 1+t/2 (fma),
//                      1-rv0v*w (fma), x, y, zeta (3 fma), s (add);
//   exact drift 18:    pz^2 (mul + 2 fma), sqrt, 1/pz (div), 1-rv0v*opd/pz
//                      (mul+fma), px/pz*L (mul), x, y, zeta (3 fma), s (add);
//   kick of merged order N: 4N fma (complex Horner) + 2 fma (apply, chi);
//   curvature: rot-frame 5 (fma, mul+fma), k0*h 3 (mul+fma),
//              k1*h 10 (3 mul, 2 fma for w, fma, mul+fma);
//   cavity 25 (tau, phase, sin, energy kick, ptau/delta/rpp/rvv update).
double canonical_flops(const unsigned char* rec) {
    const RecHeader* h = reinterpret_cast<const RecHeader*>(rec);
    const double drift_exp = 16.0;
    const double drift_exact = 18.0;
    switch (h->op) {
    case OP_DRIFT: {
        const DriftRec* r = reinterpret_cast<const DriftRec*>(rec);
        return r->exact ? drift_exact : drift_exp;
    }
    case OP_LIMIT_ELLIPSE:
    case OP_LIMIT_RECT_ELLIPSE:
        return 5.0;                    // 2 mul, 1 fma-free mul-add pair
    case OP_LIMIT_RECT:
        return 0.0;
    case OP_DIPOLE_EDGE: {
        // linear: two products and two fused adds; full: as a magnet's
        // dipole-only fringe
        const DipoleEdgeRec* r = reinterpret_cast<const DipoleEdgeRec*>(rec);
        return r->model == 0 ? 4.0 : 60.0;
    }
    case OP_CAVITY:
        return 25.0;
    case OP_KICK: {
        const KickRec* r = reinterpret_cast<const KickRec*>(rec);
        double kick = 8.0 * (r->fast_top > 0 ? r->fast_top : 0) + 4.0;
        if (r->curv_terms & 1) kick += 5;
        if (r->curv_terms & 2) kick += 3;
        if (r->curv_terms & 4) kick += 10;
        return kick;
    }
    case OP_MAGNET: {
        const MagnetRec* r = reinterpret_cast<const MagnetRec*>(rec);
        double f = 0;
        if (r->edge_entry == EDGE_LINEAR && (r->entry_r21 != 0 || r->entry_r43 != 0)) f += 4;
        if (r->edge_exit == EDGE_LINEAR && (r->exit_r21 != 0 || r->exit_r43 != 0)) f += 4;
        // nonlinear edge: dipole fringe ~60, multipole fringe ~40 per order
        const double* cf = reinterpret_cast<const double*>(rec + sizeof(MagnetRec));
        if (r->edge_entry == EDGE_FRINGE) f += 60.0 + 40.0 * (4 + cf[r->entry_fringe + FR_KL_ORDER]);
        if (r->edge_exit == EDGE_FRINGE) f += 60.0 + 40.0 * (4 + cf[r->exit_fringe + FR_KL_ORDER]);
        if (!r->body_active) return f;
        double const dr = (r->drift_model == 1) ? drift_exact : (r->drift_model == 0 ? drift_exp : 40.0);
        if (r->only_drift) return f + (r->drift_model < 0 ? 0 : dr);
        // kick: merged complex Horner, 4 FMA per order, plus 2 FMA to apply
        double kick = 8.0 * (r->fast_top > 0 ? r->fast_top : 0) + 4.0;
        if (r->curv_terms & 1) kick += 5;   // hl*(1+delta), rv0v*hl*x
        if (r->curv_terms & 2) kick += 3;
        if (r->curv_terms & 4) kick += 10;
        int64_t n_kicks = r->n_kicks;
        int64_t n_drifts = 0;
        if (r->integrator == INT_YOSHIDA4) {
            n_kicks = 7 * (int64_t)r->n_kicks;
            n_drifts = 8 * (int64_t)r->n_kicks;
        } else if (r->integrator == INT_UNIFORM) {
            n_drifts = n_kicks + 1;     // adjacent half drifts merged
        } else {
            n_drifts = n_kicks + 1;
        }
        if (r->drift_model < 0) n_drifts = 0;
        return f + n_kicks * kick + n_drifts * dr;
    }
    default:
        return 0.0;
    }
}

}  // namespace xtg
