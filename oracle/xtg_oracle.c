/*
 * CPU oracle for the xtrack `Line.track` push — TEST INFRASTRUCTURE ONLY.
 *
 * A C99 restatement of the reference's element arithmetic and of its
 * generated `track_line` driver. Every expression keeps the reference's
 * operation order (C left-to-right evaluation, no contraction: build with
 * -ffp-contract=off) so that results equal the reference's CPU results bit
 * for bit, libm aside. Paths below are inside the xtrack source tree.
 *
 * Used by the test-suite as the checker and by the benchmark as the timed
 * CPU baseline. Product code never calls it.
 */
#include "xtg_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* xtrack/headers/constants.h:9-27 */
#define XTO_C_LIGHT 299792458.0
#define XTO_PI 3.1415926535897932384626433832795028841971693993751
#define XTO_DEG2RAD 0.0174532925199432957692369076848861271344287188854
/* default_magnet_config.h:9-23 */
#define XTO_BEND_DEFAULT_MODEL 3
#define XTO_QUADRUPOLE_DEFAULT_MODEL 4
#define XTO_SEXTUPOLE_DEFAULT_MODEL 6
#define XTO_OCTUPOLE_DEFAULT_MODEL 6
#define XTO_MULTIPOLE_DEFAULT_MODEL 6
#define XTO_BEND_DEFAULT_INTEGRATOR 2
#define XTO_STRAIGHT_DEFAULT_INTEGRATOR 3

/* One particle, as the reference's LocalParticle sees it
 * (particles.py:86-408 generated accessors). */
typedef struct {
    double x, px, y, py, zeta, delta, ptau, rpp, rvv, s;
    double chi, charge_ratio, beta0, p0c, q0, ax, ay, t_sim;
    int64_t state, at_element, at_turn, particle_id;
    uint64_t track_flags;
    double line_length;
} xto_part;

static int flag_set(const xto_part* p, int bit) {
    /* particles.py:124-127 LocalParticle_check_track_flag */
    return (int)((p->track_flags >> bit) & 1u);
}

/* Frozen longitudinal coordinates: the generated setters, adders and
 * scalers of zeta, ptau, delta, rpp and rvv are no-ops
 * (particles.py:185-225, FREEZE_VAR_<name>; line.py:4446-4469). */
static int xto_frozen(const xto_part* p) { return flag_set(p, XTG_FLAG_FREEZE_LONGITUDINAL); }
static void xto_set_zeta(xto_part* p, double v) { if (!xto_frozen(p)) p->zeta = v; }
static void xto_add_to_zeta(xto_part* p, double v) { if (!xto_frozen(p)) p->zeta += v; }
static void xto_set_energy(xto_part* p, double delta, double rvv, double rpp, double ptau) {
    if (xto_frozen(p)) return;
    p->delta = delta;
    p->rvv = rvv;
    p->ptau = ptau;
    p->rpp = rpp;
}

/* ---------------------------------------------------------------------- */
/* Energy variables: particles/local_particle_custom_api.h                */
/* ---------------------------------------------------------------------- */

/* local_particle_custom_api.h:20-33 */
static void xto_update_ptau(xto_part* p, double new_ptau) {
    double const beta0 = p->beta0;
    double const ptau = new_ptau;
    double const irpp = sqrt(ptau * ptau + 2 * ptau / beta0 + 1);
    double const new_rpp = 1. / irpp;
    double const new_rvv = irpp / (1 + beta0 * ptau);
    xto_set_energy(p, irpp - 1, new_rvv, new_rpp, ptau);
}

/* local_particle_custom_api.h:195-217 */
static void xto_add_to_energy(xto_part* p, double delta_energy, int pz_only) {
    double ptau = p->ptau;
    double const mass_ratio = p->charge_ratio / p->chi;
    ptau += delta_energy / p->p0c / mass_ratio;
    double const old_rpp = p->rpp;
    xto_update_ptau(p, ptau);
    if (!pz_only) {
        double const f = old_rpp / p->rpp;
        p->px *= f;
        p->py *= f;
    }
}

/* ---------------------------------------------------------------------- */
/* Drift maps: track_drift.h, track_magnet_drift.h                        */
/* ---------------------------------------------------------------------- */

/* track_drift.h:10-23 (same arithmetic as track_magnet_drift.h:13-26) */
static void xto_drift_expanded(xto_part* p, double length) {
    double const rpp = p->rpp;
    double const rv0v = 1. / p->rvv;
    double const xp = p->px * rpp;
    double const yp = p->py * rpp;
    double const dzeta = 1 - rv0v * (1. + (xp * xp + yp * yp) / 2.);
    p->x += xp * length;
    p->y += yp * length;
    p->s += length;
    xto_add_to_zeta(p, length * dzeta);
}

/* track_drift.h:26-42 */
static void xto_drift_exact(xto_part* p, double length) {
    double const px = p->px;
    double const py = p->py;
    double const rv0v = 1. / p->rvv;
    double const opd = 1. + p->delta;
    double const one_over_pz = 1. / sqrt(opd * opd - px * px - py * py);
    double const dzeta = 1 - rv0v * opd * one_over_pz;
    p->x += px * one_over_pz * length;
    p->y += py * one_over_pz * length;
    xto_add_to_zeta(p, dzeta * length);
    p->s += length;
}

/* track_drift.h:45-51: expanded unless XTRACK_USE_EXACT_DRIFTS */
static void xto_drift_default(xto_part* p, double length, int use_exact) {
    if (use_exact) xto_drift_exact(p, length);
    else xto_drift_expanded(p, length);
}

/* track_magnet_drift.h:44-87 */
static void xto_drift_polar(xto_part* p, double length, double h) {
    double const rvv = p->rvv;
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    double const s = length;
    double const opd = p->delta + 1.0;
    double const pz = sqrt((opd) * (opd) - (px) * (px) - (py) * (py));
    double const rho = 1 / h;
    double const ca = cos(h * s);
    double const sa = sin(h * s);
    double const sa2 = sin(0.5 * h * s);
    double const _pz = 1 / pz;
    double const pxt = px * _pz;
    double const _ptt = 1 / (ca - sa * pxt);
    double const pst = (x + rho) * sa * _pz * _ptt;
    double const new_x = (x + rho * (2 * sa2 * sa2 + sa * pxt)) * _ptt;
    double const new_px = ca * px + sa * pz;
    double const new_y = y + pst * py;
    double const delta_ell = opd * (x + rho) * sa / ca / pz / (1 - px * sa / ca / pz);
    p->x = new_x;
    p->px = new_px;
    p->y = new_y;
    xto_add_to_zeta(p, length - delta_ell / rvv);
    p->s += s;
}

/* track_magnet_drift.h:90-213 (MAD-X trrun expanded dipole-quadrupole) */
static void xto_drift_cf_expanded(xto_part* p, double length, double k0_,
                                  double k1_, double h) {
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    double const rvv = p->rvv;
    double const dp1 = p->delta + 1;
    double const chi = p->chi;
    double const k0 = chi * k0_ / dp1;
    double const k1 = chi * k1_ / dp1;
    double const Kx = k0 * h + k1;
    double const Ky = -k1;
    double x_, px_, y_, py_, Sx, Sy, Cx, Cy;

    if (Kx > 0.0) {
        double sq = sqrt(Kx);
        Sx = sin(sq * length) / sq;
        Cx = cos(sq * length);
    } else if (Kx < 0.0) {
        double sq = sqrt(-Kx);
        Sx = sinh(sq * length) / sq;
        Cx = cosh(sq * length);
    } else {
        Sx = length;
        Cx = 1.0;
    }
    if (Ky > 0.0) {
        double sq = sqrt(Ky);
        Sy = sin(sq * length) / sq;
        Cy = cos(sq * length);
    } else if (Ky < 0.0) {
        double sq = sqrt(-Ky);
        Sy = sinh(sq * length) / sq;
        Cy = cosh(sq * length);
    } else {
        Sy = length;
        Cy = 1.0;
    }

    double const xp = px / dp1;
    double const yp = py / dp1;
    double const A = -Kx * x - k0 + h;
    double const B = xp;
    double const C = -Ky * y;
    double const D = yp;

    x_ = x * Cx + xp * Sx;
    y_ = y * Cy + yp * Sy;
    px_ = (A * Sx + B * Cx) * dp1;
    py_ = (C * Sy + D * Cy) * dp1;

    if (Kx != 0.0) x_ = x_ + (k0 - h) * (Cx - 1.0) / Kx;
    else x_ = x_ - (k0 - h) * 0.5 * ((length) * (length));

    double length_ = length;
    if (Kx != 0.0) {
        length_ -= (h * ((Cx - 1.0) * xp + Sx * A + length * (k0 - h))) / Kx;
        length_ += 0.5 * (
            - (((A) * (A)) * Cx * Sx) / (2.0 * Kx)
            + (((B) * (B)) * Cx * Sx) / 2.0
            + (((A) * (A)) * length) / (2.0 * Kx)
            + (((B) * (B)) * length) / 2.0
            - (A * B * ((Cx) * (Cx))) / Kx
            + (A * B) / Kx);
    } else {
        length_ += h * length * (3.0 * length * xp + 6.0 * x
                                 - (k0 - h) * ((length) * (length))) / 6.0;
        length_ += 0.5 * (((B) * (B))) * length;
    }
    if (Ky != 0.0) {
        length_ += 0.5 * (
            - (((C) * (C)) * Cy * Sy) / (2.0 * Ky)
            + (((D) * (D)) * Cy * Sy) / 2.0
            + (((C) * (C)) * length) / (2.0 * Ky)
            + (((D) * (D)) * length) / 2.0
            - (C * D * ((Cy) * (Cy))) / Ky
            + (C * D) / Ky);
    } else {
        length_ += 0.5 * ((D) * (D)) * length;
    }

    double const dzeta = length - length_ / rvv;
    p->x = x_;
    p->px = px_;
    p->y = y_;
    p->py = py_;
    xto_add_to_zeta(p, dzeta);
    p->s += length;
}

/* track_magnet_drift.h:271-345 */
static void xto_drift_curved_exact_bend(xto_part* p, double length, double k0,
                                        double h) {
    double const k0_chi = k0 * p->chi;
    if (fabs(k0_chi) < 1e-8) {
        xto_drift_polar(p, length, h);
        return;
    }
    double const rvv = p->rvv;
    double const x0 = p->x, y0 = p->y, px0 = p->px, py = p->py;
    double const s = length;
    double const opd = p->delta + 1.0;
    double const hs = h * s;
    double const sin_hs = sin(hs);
    double const cos_hs = cos(hs);
    double const sin_hs_2 = sin(hs / 2);
    double const pz0 = sqrt((opd) * (opd) - (px0) * (px0) - (py) * (py));
    double const C = pz0 - k0_chi * ((1.0 / h) + x0);
    double const pxs = px0 * cos_hs + C * sin_hs;
    double const pzs = sqrt((opd) * (opd) - (pxs) * (pxs) - (py) * (py));
    double const delta_pz = (px0 - pxs) * (px0 + pxs) / (pz0 + pzs);
    double const delta_D = -2 * C * ((sin_hs_2) * (sin_hs_2)) - px0 * sin_hs;
    double const delta_x = (delta_pz - delta_D) / k0_chi;
    double const delta_px = -2 * px0 * ((sin_hs_2) * (sin_hs_2)) + C * sin_hs;
    double const N_a = px0 * delta_pz - pz0 * delta_px;
    double const D_a = pz0 * pzs + px0 * pxs;
    double const delta_a = atan2(N_a, D_a);
    double const integ = (hs + delta_a) / k0_chi;
    double const new_y = y0 + py * integ;
    double const delta_ell = opd * integ;
    p->x += delta_x;
    p->px = pxs;
    p->y = new_y;
    xto_add_to_zeta(p, length - delta_ell / rvv);
    p->s += s;
}

/* track_magnet_drift.h:348-393 */
static void xto_drift_straight_exact_bend(xto_part* p, double length, double k0) {
    double const k0_chi = k0 * p->chi;
    if (fabs(k0_chi) < 1e-8) {
        xto_drift_exact(p, length);
        return;
    }
    double const rvv = p->rvv;
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    double const s = length;
    double const opd = p->delta + 1.0;
    double const A = 1.0 / sqrt((opd) * (opd) - (py) * (py));
    double const pz = sqrt((opd) * (opd) - (px) * (px) - (py) * (py));
    double const new_px = px - k0_chi * s;
    double const new_x = x + (sqrt((opd) * (opd) - (new_px) * (new_px) - (py) * (py)) - pz) / k0_chi;
    double const D = asin(A * px) - asin(A * new_px);
    double const new_y = y + (py / k0_chi) * D;
    double const delta_ell = (opd / k0_chi) * D;
    p->x = new_x;
    p->px = new_px;
    p->y = new_y;
    xto_add_to_zeta(p, length - delta_ell / rvv);
    p->s += s;
}

/* track_magnet_drift.h:469-555 (solenoid model 6 is not built) */
static void xto_magnet_drift(xto_part* p, double length, double k0, double k1,
                             double h, int drift_model) {
    if (drift_model == -1) return;
    if (length == 0.0) return;
    switch (drift_model) {
    case 0: xto_drift_expanded(p, length); break;
    case 1: xto_drift_exact(p, length); break;
    case 2: xto_drift_polar(p, length, h); break;
    case 3: xto_drift_cf_expanded(p, length, k0, k1, h); break;
    case 4: xto_drift_curved_exact_bend(p, length, k0, h); break;
    case 5: xto_drift_straight_exact_bend(p, length, k0); break;
    case 7:
        xto_drift_polar(p, 0.6756035959798289 * length, h);
        p->px = p->px - 1.3512071919596578 * k0 * p->chi * length;
        xto_drift_polar(p, -0.17560359597982889 * length, h);
        p->px = p->px - (-1.7024143839193155) * k0 * p->chi * length;
        xto_drift_polar(p, -0.17560359597982889 * length, h);
        p->px = p->px - 1.3512071919596578 * k0 * p->chi * length;
        xto_drift_polar(p, 0.6756035959798289 * length, h);
        break;
    case 8:
        xto_drift_polar(p, 3.922568052387799819591407413100e-01 * length, h);
        p->px = p->px - 7.845136104775599639182814826199e-01 * k0 * p->chi * length;
        xto_drift_polar(p, 5.100434119184584780271052295575e-01 * length, h);
        p->px = p->px - 2.355732133593569921359289764951e-01 * k0 * p->chi * length;
        xto_drift_polar(p, -4.710533854097565531482416645304e-01 * length, h);
        p->px = p->px - (-1.177679984178870098432412305556e+00) * k0 * p->chi * length;
        xto_drift_polar(p, 6.875316825251809316199569366290e-02 * length, h);
        p->px = p->px - 1.315186320683906284756403692882e+00 * k0 * p->chi * length;
        xto_drift_polar(p, 6.875316825251809316199569366290e-02 * length, h);
        p->px = p->px - (-1.177679984178870098432412305556e+00) * k0 * p->chi * length;
        xto_drift_polar(p, -4.710533854097565531482416645304e-01 * length, h);
        p->px = p->px - 2.355732133593569921359289764951e-01 * k0 * p->chi * length;
        xto_drift_polar(p, 5.100434119184584780271052295575e-01 * length, h);
        p->px = p->px - 7.845136104775599639182814826199e-01 * k0 * p->chi * length;
        xto_drift_polar(p, 3.922568052387799819591407413100e-01 * length, h);
        break;
    default: break;
    }
}

/* ---------------------------------------------------------------------- */
/* Multipole kicks: track_magnet_kick.h                                   */
/* ---------------------------------------------------------------------- */

/* track_magnet_kick.h:182-228 */
static void xto_kick_coords(double x, double y, double chi, int64_t order,
                            double inv_factorial, const double* knl,
                            const double* ksl, double factor, double kick_weight,
                            double* dpx, double* dpy) {
    if (knl == NULL || ksl == NULL) {
        *dpx = 0.;
        *dpy = 0.;
        return;
    }
    int64_t index = order;
    double dpx_mul = chi * knl[index] * factor * inv_factorial;
    double dpy_mul = chi * ksl[index] * factor * inv_factorial;
    while (index > 0) {
        double const zre = dpx_mul * x - dpy_mul * y;
        double const zim = dpx_mul * y + dpy_mul * x;
        inv_factorial *= index;
        index -= 1;
        double this_knl = chi * knl[index] * factor;
        double this_ksl = chi * ksl[index] * factor;
        dpx_mul = this_knl * inv_factorial + zre;
        dpy_mul = this_ksl * inv_factorial + zim;
    }
    dpx_mul = -dpx_mul;
    *dpx = kick_weight * dpx_mul;
    *dpy = kick_weight * dpy_mul;
}

/* track_magnet_kick.h:231-260 */
static void xto_kick_simple(xto_part* p, int64_t order, double inv_factorial,
                            const double* knl, const double* ksl, double factor,
                            double kick_weight) {
    double dpx, dpy;
    xto_kick_coords(p->x, p->y, p->chi, order, inv_factorial, knl, ksl, factor,
                    kick_weight, &dpx, &dpy);
    p->px += dpx;
    p->py += dpy;
}

/* Parameters of one magnet body, as passed down by track_magnet_particles. */
typedef struct {
    double length;            /* body (core) length                       */
    int64_t order;
    double inv_factorial_order;
    const double* knl;
    const double* ksl;
    int64_t order_rel;
    double inv_factorial_order_rel;
    const double* knl_rel;
    const double* ksl_rel;
    double rel_ref_strength;
    double factor_knl_ksl;
    int64_t num_multipole_kicks;
    int kick_rot_frame;
    int drift_model;
    int integrator;
    double k0_drift, k1_drift, h_drift;
    double k0_kick, k1_kick, h_kick, hxl;
    double k0_h_correction, k1_h_correction;
    double k2, k3, k0s, k1s, k2s, k3s;
} xto_body;

/* track_magnet_kick.h:23-144 */
static void xto_magnet_kick(xto_part* p, const xto_body* b, double kick_weight) {
    double const length = b->length;
    double const chi = p->chi;
    double const x = p->x;
    double const y = p->y;
    double knl_main[4] = {b->k0_kick, b->k1_kick, b->k2, b->k3};
    double ksl_main[4] = {b->k0s, b->k1s, b->k2s, b->k3s};
    for (int index = 0; index < 4; index++) {
        knl_main[index] = knl_main[index] * length;
        ksl_main[index] = ksl_main[index] * length;
    }
    xto_kick_simple(p, b->order, b->inv_factorial_order, b->knl, b->ksl,
                    b->factor_knl_ksl, kick_weight);
    xto_kick_simple(p, b->order_rel, b->inv_factorial_order_rel, b->knl_rel,
                    b->ksl_rel, b->factor_knl_ksl * b->rel_ref_strength,
                    kick_weight);
    xto_kick_simple(p, 3, 1. / (3 * 2), knl_main, ksl_main, 1, kick_weight);

    double dpx = 0;
    double dpy = 0;
    double dzeta = 0;
    double const h = b->h_kick;
    if (b->kick_rot_frame) {
        double const hl = h * length * kick_weight + b->hxl * kick_weight;
        dpx += hl * (1. + p->delta);
        double const rv0v = 1. / p->rvv;
        dzeta += -rv0v * hl * x;
    }
    double htot = h;
    if (length != 0) {
        htot += b->hxl / length;
    }
    double k0l_mult = 0;
    if (b->order >= 0) {
        k0l_mult = b->knl[0] * b->factor_knl_ksl;
    }
    if (b->order_rel >= 0 && b->knl_rel != NULL) {
        k0l_mult += b->knl_rel[0] * b->factor_knl_ksl * b->rel_ref_strength;
    }
    dpx += -chi * (b->k0_h_correction * length + k0l_mult) * kick_weight * htot * x;
    double k1l_mult = 0;
    if (b->order >= 1) {
        k1l_mult = b->knl[1] * b->factor_knl_ksl;
    }
    if (b->order_rel >= 1 && b->knl_rel != NULL) {
        k1l_mult += b->knl_rel[1] * b->factor_knl_ksl * b->rel_ref_strength;
    }
    dpx += htot * chi * (b->k1_h_correction * length + k1l_mult) * kick_weight
           * (-x * x + 0.5 * y * y);
    dpy += htot * chi * (b->k1_h_correction * length + k1l_mult) * kick_weight * x * y;
    p->px += dpx;
    p->py += dpy;
    xto_add_to_zeta(p, dzeta);
}

/* track_magnet_kick.h:149-179 */
static int xto_kick_is_inactive(int64_t order, const double* knl, const double* ksl,
                                double k0, double k1, double k2, double k3,
                                double k0s, double k1s, double k2s, double k3s,
                                double h) {
    if (h != 0) return 0;
    if (k0 != 0) return 0;
    if (k1 != 0) return 0;
    if (k2 != 0) return 0;
    if (k3 != 0) return 0;
    if (k0s != 0) return 0;
    if (k1s != 0) return 0;
    if (k2s != 0) return 0;
    if (k3s != 0) return 0;
    for (int64_t index = order; index >= 0; index--) {
        if (knl[index] != 0) return 0;
        if (ksl[index] != 0) return 0;
    }
    return 1;
}

/* ---------------------------------------------------------------------- */
/* Model configuration: track_magnet_configure.h:6-194                    */
/* ---------------------------------------------------------------------- */
static void xto_configure(int64_t model, double k0, double k1, double h,
                          xto_body* b) {
    if (model == 1) model = 3;
    int const h_is_zero = (fabs(h) < 1e-8);
    int drift_model = 0;
    if (model == 2) drift_model = h_is_zero ? 5 : 4;
    else if (model == 3) drift_model = h_is_zero ? 1 : 7;
    else if (model == 4) drift_model = 3;
    else if (model == 5) drift_model = 1;
    else if (model == 6) drift_model = 0;
    else if (model == -1) drift_model = -1;
    else if (model == -2) drift_model = 6;
    else if (model == 7) drift_model = h_is_zero ? 1 : 2;
    else if (model == 8) drift_model = h_is_zero ? 1 : 8;
    else drift_model = 99999999;

    if (drift_model == -1 || drift_model == 0 || drift_model == 1) {
        b->k0_drift = 0.0; b->k1_drift = 0.0; b->h_drift = 0.0;
        b->k0_kick = k0; b->k1_kick = k1; b->h_kick = h;
        b->k0_h_correction = k0; b->k1_h_correction = k1;
        b->kick_rot_frame = 1;
    } else if (drift_model == 2) {
        b->k0_drift = 0.0; b->k1_drift = 0.0; b->h_drift = h;
        b->k0_kick = k0; b->k1_kick = k1; b->h_kick = h;
        b->k0_h_correction = k0; b->k1_h_correction = k1;
        b->kick_rot_frame = 0;
    } else if (drift_model == 3) {
        b->k0_drift = k0; b->k1_drift = k1; b->h_drift = h;
        b->k0_kick = 0.0; b->k1_kick = 0.0; b->h_kick = h;
        b->k0_h_correction = 0.; b->k1_h_correction = k1;
        b->kick_rot_frame = 0;
    } else if (drift_model == 4) {
        b->k0_drift = k0; b->k1_drift = 0.0; b->h_drift = h;
        b->k0_kick = 0.0; b->k1_kick = k1; b->h_kick = h;
        b->k0_h_correction = 0.; b->k1_h_correction = k1;
        b->kick_rot_frame = 0;
    } else if (drift_model == 5) {
        b->k0_drift = k0; b->k1_drift = 0.0; b->h_drift = 0.0;
        b->k0_kick = 0.0; b->k1_kick = k1; b->h_kick = 0.0;
        b->k0_h_correction = 0.; b->k1_h_correction = 0.;
        b->kick_rot_frame = 0;
    } else if (drift_model == 7 || drift_model == 8) {
        b->k0_drift = k0; b->k1_drift = 0.0; b->h_drift = h;
        b->k0_kick = 0.0; b->k1_kick = k1; b->h_kick = h;
        b->k0_h_correction = k0; b->k1_h_correction = k1;
        b->kick_rot_frame = 0;
    } else {
        /* drift_model 6 (solenoid) and unknown models leave the outputs at
         * their zero initial values, as the reference does for the fields
         * it does not assign. */
        b->k0_drift = 0.0; b->k1_drift = 0.0; b->h_drift = 0.0;
        b->k0_kick = 0.0; b->k1_kick = 0.0; b->h_kick = 0.0;
        b->k0_h_correction = 0.0; b->k1_h_correction = 0.0;
        b->kick_rot_frame = 0;
    }
    b->drift_model = drift_model;
}

/* ---------------------------------------------------------------------- */
/* Magnet body integrators: track_magnet.h:25-285                          */
/* ---------------------------------------------------------------------- */
static const double XTO_D_YOSHIDA[4] = {
    3.922568052387799819591407413100e-01, 5.100434119184584780271052295575e-01,
    -4.710533854097565531482416645304e-01, 6.875316825251809316199569366290e-02};
static const double XTO_K_YOSHIDA[4] = {
    7.845136104775599639182814826199e-01, 2.355732133593569921359289764951e-01,
    -1.177679984178870098432412305556e+00, 1.315186320683906284756403692882e+00};

#define XTO_MDRIFT(P, L) xto_magnet_drift((P), (L), b->k0_drift, b->k1_drift, b->h_drift, b->drift_model)
#define XTO_MKICK(P, W) xto_magnet_kick((P), b, (W))

static void xto_magnet_body(xto_part* p, const xto_body* b) {
    double const length = b->length;
    int64_t const n = b->num_multipole_kicks;
    if (n == 0 && b->k0_kick == 0 && b->k1_kick == 0 && b->h_kick == 0) {
        XTO_MDRIFT(p, length);
        return;
    }
    if (b->integrator == 1) {              /* TEAPOT, track_magnet.h:192-213 */
        double const kick_weight = 1. / n;
        double edge_drift_weight = 0.5;
        double inside_drift_weight = 0;
        if (n > 1) {
            edge_drift_weight = 1. / (2 * (1 + n));
            inside_drift_weight = (((double)n) / ((double)(n * n) - 1));
        }
        XTO_MDRIFT(p, edge_drift_weight * length);
        for (int i_kick = 0; i_kick < n - 1; i_kick++) {
            XTO_MKICK(p, kick_weight);
            XTO_MDRIFT(p, inside_drift_weight * length);
        }
        XTO_MKICK(p, kick_weight);
        XTO_MDRIFT(p, edge_drift_weight * length);
    } else if (b->integrator == 3) {       /* uniform, track_magnet.h:215-228 */
        double const kick_weight = 1. / n;
        double const drift_weight = kick_weight;
        for (int i_kick = 0; i_kick < n; i_kick++) {
            XTO_MDRIFT(p, 0.5 * drift_weight * length);
            XTO_MKICK(p, kick_weight);
            XTO_MDRIFT(p, 0.5 * drift_weight * length);
        }
    } else if (b->integrator == 2) {       /* Yoshida-4, track_magnet.h:230-277 */
        int64_t const n_kicks_yoshida = 7;
        int64_t const num_slices = (n / n_kicks_yoshida + (n % n_kicks_yoshida != 0));
        double const slice_length = length / (num_slices);
        double const kick_weight = 1. / num_slices;
        for (int ii = 0; ii < num_slices; ii++) {
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[0]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[0]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[1]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[1]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[2]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[2]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[3]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[3]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[3]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[2]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[2]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[1]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[1]);
            XTO_MKICK(p, kick_weight * XTO_K_YOSHIDA[0]);
            XTO_MDRIFT(p, slice_length * XTO_D_YOSHIDA[0]);
        }
    }
}
#undef XTO_MDRIFT
#undef XTO_MKICK

/* ---------------------------------------------------------------------- */
/* Linear dipole edge: track_dipole_edge_linear.h, track_magnet_edge.h     */
/* ---------------------------------------------------------------------- */

/* track_dipole_edge_linear.h:11-28 */
static void xto_edge_linear_coefficients(double k, double e1, double e1_fd,
                                         double hgap, double fint, double* r21,
                                         double* r43) {
    double const corr = 2.0 * k * hgap * fint;
    double const r21_out = k * tan(e1);
    double const e1_v = e1 + e1_fd;
    double const sin_e1_v = sin(e1_v);
    double const temp = corr / cos(e1_v) * (1.0 + sin_e1_v * sin_e1_v);
    double const r43_out = -k * tan(e1_v - temp);
    *r21 = r21_out;
    *r43 = r43_out;
}

/* ---------------------------------------------------------------------- */
/* Nonlinear edges (full and dipole-only models)                           */
/* ---------------------------------------------------------------------- */

/* local_particle_custom_api.h:36-49 */
static void xto_update_delta(xto_part* p, double new_delta_value) {
    double const beta0 = p->beta0;
    double const delta_beta0 = new_delta_value * beta0;
    double const ptau_beta0 = sqrt(delta_beta0 * delta_beta0 + 2 * delta_beta0 * beta0 + 1) - 1;
    double const one_plus_delta = 1 + new_delta_value;
    xto_set_energy(p, new_delta_value, one_plus_delta / (1 + ptau_beta0), 1 / one_plus_delta,
                   ptau_beta0 / beta0);
}

/* local_particle_custom_api.h:248-256 */
static void xto_kill(xto_part* p, int64_t kill_state) {
    p->x = 1e30;
    p->px = 1e30;
    p->y = 1e30;
    p->py = 1e30;
    xto_set_zeta(p, 1e30);
    xto_update_delta(p, -1);
    p->state = kill_state;
}

/* track_yrotation.h:13-48 (no spin) */
static void xto_yrotation(xto_part* p, double sin_angle, double cos_angle, double tan_angle) {
    double const beta0 = p->beta0;
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    double const t = p->zeta / beta0;
    double const pt = (p->ptau / beta0) * beta0;       /* get_pzeta * beta0 */
    double const pz = sqrt(1.0 + 2.0 * pt / beta0 + pt * pt - px * px - py * py);
    double const ptt = 1.0 + tan_angle * px / pz;
    double const x_hat = x / (cos_angle * ptt);
    double const px_hat = cos_angle * px - sin_angle * pz;
    double const y_hat = y - tan_angle * x * py / (pz * ptt);
    double const t_hat = t + tan_angle * x * (1.0 / beta0 + pt) / (pz * ptt);
    p->x = x_hat;
    p->px = px_hat;
    p->y = y_hat;
    xto_set_zeta(p, t_hat * beta0);
}

/* track_dipole_fringe.h:16-82 (the MAD-NG form, the default build) */
static void xto_dipole_fringe(xto_part* p, double fint, double hgap, double k0) {
    if (fabs(k0) < 10e-10) return;
    double const beta0 = p->beta0;
    double const x = p->x, px = p->px, y = p->y, py = p->py;
    double const t = p->zeta / beta0;
    double const pt = p->ptau;
    double const delta = p->delta;
    double const fh = hgap * fint;
    double const fsad = (fh > 10e-10) ? 1. / (72 * fh) : 0;
    double const k0w = k0 * p->chi;
    double const inv_beta = 1. / beta0;
    double const b0 = k0w;
    double const dpp = (1. + delta) * (1. + delta);
    double const pz = sqrt(dpp - px * px - py * py);
    double const ipz = 1. / pz;
    double const relp = 1. / sqrt(dpp);
    double const tfac = -(inv_beta + pt);
    double const c2 = b0 * fh * 2;
    double const c3 = (b0 * b0) * fsad * relp;
    double const xp = px / pz;
    double const yp = py / pz;
    double const xyp = xp * yp;
    double const yp2 = 1. + yp * yp;
    double const xp2 = xp * xp;
    double const iyp2 = 1. / yp2;
    double const fi0 = atan((xp * iyp2)) - c2 * (1 + xp2 * (1 + yp2)) * ipz;
    double const cfi = cos(fi0);
    double const co2 = b0 / (cfi * cfi);
    double const q = xp * iyp2;
    double const co1 = co2 / (1 + q * q) * iyp2;
    double const co3 = co2 * c2;
    double const fi1 = co1 - co3 * 2 * xp * (1 + yp2) * ipz;
    double const fi2 = -2 * co1 * xyp * iyp2 - co3 * 2 * xp * xyp * ipz;
    double const fi3 = +co3 * (1 + xp2 * (1 + yp2)) * (ipz * ipz);
    double const kx = fi1 * (1 + xp2) * ipz + fi2 * xyp * ipz - fi3 * xp;
    double const ky = fi1 * xyp * ipz + fi2 * yp2 * ipz - fi3 * yp;
    double const kz = fi1 * tfac * xp * (ipz * ipz) + fi2 * tfac * yp * (ipz * ipz) - fi3 * tfac * ipz;
    double const new_y = 2 * y / (1 + sqrt(1 - 2 * ky * y));
    double const new_x = x + 0.5 * kx * (new_y * new_y);
    double const new_py = py - 4 * c3 * (new_y * new_y * new_y) - b0 * tan(fi0) * new_y;
    double const new_t = t + 0.5 * kz * (new_y * new_y) +
                         c3 * (new_y * new_y * new_y * new_y) * (relp * relp) * tfac;
    p->x = new_x;
    p->y = new_y;
    p->py = new_py;
    xto_set_zeta(p, new_t * beta0);
}

/* track_mult_fringe.h:12-128 */
static void xto_mult_fringe(xto_part* p, const double* kn, const double* ks, int64_t k_order,
                            const double* knl, const double* ksl, int64_t kl_order,
                            double length, int is_exit, uint64_t min_order) {
    if (k_order == -1 && kl_order == -1) return;
    if (flag_set(p, 0)) {            /* XS_FLAG_BACKTRACK */
        xto_kill(p, -32);
        return;
    }
    double const beta0 = p->beta0;
    double const direction = is_exit ? -1 : 1;
    double const x = p->x, px = p->px, y = p->y, py = p->py;
    double const t = p->zeta / beta0;
    double const pt = p->ptau;
    double const rpp = p->rpp;
    double const chi = p->chi;
    double rx = 1, ix = 0;
    double fx = 0, fxx = 0, fxy = 0, fy = 0, fyx = 0, fyy = 0;
    uint32_t const order = (uint32_t)((k_order > kl_order) ? k_order : kl_order);
    double inv_factorial = 1;
    for (uint32_t ii = 0; ii <= order; ii++) {
        if (ii > 1) inv_factorial /= ii;
        double const component = ii + 1;
        double const drx = rx;
        double const dix = ix;
        rx = drx * x - dix * y;
        ix = drx * y + dix * x;
        double kn_total = 0, ks_total = 0;
        if (ii >= min_order) {
            if ((int64_t)ii <= k_order) {
                kn_total += kn[ii] * inv_factorial;
                ks_total += ks[ii] * inv_factorial;
            }
            if ((int64_t)ii <= kl_order && length != 0.) {
                kn_total += knl[ii] / length * inv_factorial;
                ks_total += ksl[ii] / length * inv_factorial;
            }
        }
        double const nj = -direction / (4 * (component + 1));
        double const nf = (component + 2) / component;
        double const kj = kn_total * chi;
        double const ksj = ks_total * chi;
        double u, v, du, dv;
        if (ii == 0) {
            u = nj * (-ksj * ix);
            v = nj * (ksj * rx);
            du = nj * (-ksj * dix);
            dv = nj * (ksj * drx);
        } else {
            u = nj * (kj * rx - ksj * ix);
            v = nj * (kj * ix + ksj * rx);
            du = nj * (kj * drx - ksj * dix);
            dv = nj * (kj * dix + ksj * drx);
        }
        double const dux = component * du;
        double const dvx = component * dv;
        double const duy = -component * dv;
        double const dvy = component * du;
        fx = fx + u * x + nf * v * y;
        fy = fy + u * y - nf * v * x;
        fxx = fxx + dux * x + nf * dvx * y + u;
        fyy = fyy + duy * y - nf * dvy * x + u;
        fxy = fxy + duy * x + nf * (dvy * y + v);
        fyx = fyx + dux * y - nf * (dvx * x + v);
    }
    double const a = 1 - fxx * rpp;
    double const b = -fyx * rpp;
    double const c = -fxy * rpp;
    double const d = 1 - fyy * rpp;
    double const det = (a * d - b * c);
    double const new_px = (d * px - b * py) / det;
    double const new_py = (a * py - c * px) / det;
    double const delta_t = (1 / beta0 + pt) * (new_px * fx + new_py * fy) * (rpp * rpp * rpp);
    p->x += -fx * rpp;
    p->y += -fy * rpp;
    p->px = new_px;
    p->py = new_py;
    xto_set_zeta(p, (t + delta_t) * beta0);
}

/* track_wedge.h:14-58 (no spin) */
static void xto_wedge(xto_part* p, double theta, double k0) {
    double const b1 = k0 * p->chi;
    if (fabs(b1) < 10e-10) {
        double const sin_ = sin(theta);
        double const cos_ = cos(theta);
        double const tan_ = tan(theta);
        xto_yrotation(p, -sin_, cos_, -tan_);
        return;
    }
    double const rvv = p->rvv;
    double const x = p->x, px = p->px, py = p->py;
    double const one_plus_delta = p->delta + 1.0;
    double const A = 1.0 / sqrt(one_plus_delta * one_plus_delta - py * py);
    double const pz = sqrt(one_plus_delta * one_plus_delta - px * px - py * py);
    double const new_px = px * cos(theta) + (pz - b1 * x) * sin(theta);
    double const new_pz = sqrt(one_plus_delta * one_plus_delta - new_px * new_px - py * py);
    double const st = sin(theta);
    double const new_x = x * cos(theta) +
                         (x * px * sin(2 * theta) + (st * st) * (2 * x * pz - b1 * (x * x))) /
                             (new_pz + pz * cos(theta) - px * sin(theta));
    double const D = asin(A * px) - asin(A * new_px);
    double const delta_y = py * (theta + D) / b1;
    double const delta_ell = one_plus_delta * (theta + D) / b1;
    p->x = new_x;
    p->y += delta_y;
    p->px = new_px;
    xto_add_to_zeta(p, -delta_ell / rvv);
}

/* track_wedge.h:60-82 */
static void xto_quad_wedge(xto_part* p, double theta, double k1) {
    double const b2 = k1 * p->chi;
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    double const new_px = px - b2 * x * x * theta + b2 * y * y / 2 * theta;
    double const new_py = py + b2 * x * y * theta;
    p->px = new_px;
    p->py = new_py;
}

/* track_magnet_edge.h:16-158: linear (0), full (1), dipole-only (2),
 * ax/ay-only (3) and suppressed (-1) models. */
static void xto_magnet_edge(xto_part* p, int model, int is_exit, double half_gap,
                            const double* knorm, const double* kskew, const double* knl,
                            const double* ksl, double factor_knl_ksl, int64_t kl_order,
                            const double* knl_rel, double factor_knl_ksl_rel,
                            int64_t order_rel, double length, double face_angle,
                            double face_angle_feed_down, double fringe_integral,
                            double factor_for_backtrack) {
    double k0 = 0;
    k0 += knorm[0];                        /* k_order == 3 > -1 */
    if (fabs(length) > 1e-10 && kl_order > -1) {
        k0 += factor_knl_ksl * knl[0] / length;
    }
    if (fabs(length) > 1e-10 && order_rel > -1 && knl_rel != NULL) {
        k0 += factor_knl_ksl_rel * knl_rel[0] / length;
    }
    if (is_exit) {
        p->ax = 0.;
        p->ay = 0.;
    } else {
        double const ksol = 0.;
        p->ax = -0.5 * ksol * (p->y - 0.);
        p->ay = 0.5 * ksol * (p->x - 0.);
    }
    if (model == 0) {
        double r21, r43;
        xto_edge_linear_coefficients(k0, face_angle, face_angle_feed_down,
                                     half_gap, fringe_integral, &r21, &r43);
        r21 = r21 * factor_for_backtrack;
        r43 = r43 * factor_for_backtrack;
        /* track_dipole_edge_linear.h:30-39 */
        double const x = p->x;
        double const y = p->y;
        double const chi = p->chi;
        p->px += chi * r21 * x;
        p->py += chi * r43 * y;
        return;
    } else if (model == 1 || model == 2) {
        /* the kill runs in its own per-particle block; the blocks that
         * follow (the fringe maps, the body, the other edge) skip the
         * particle, whose state is no longer positive (headers/track.h) */
        if (factor_for_backtrack < 0) {
            xto_kill(p, -32);
            return;
        }
        int should_rotate = 0;
        double sin_ = 0, cos_ = 1, tan_ = 0;
        if (fabs(face_angle) > 10e-10) {
            should_rotate = 1;
            sin_ = sin(face_angle);
            cos_ = cos(face_angle);
            tan_ = tan(face_angle);
        }
        if (is_exit) k0 = -k0;
        int64_t const k_order = 3;
        if (is_exit == 0) {
            if (should_rotate) xto_yrotation(p, -sin_, cos_, -tan_);
            xto_dipole_fringe(p, fringe_integral, half_gap, k0);
            if (model == 1)
                xto_mult_fringe(p, knorm, kskew, k_order, knl, ksl, kl_order,
                                length / factor_knl_ksl, is_exit, 1);
            if (model == 1 && should_rotate && k_order >= 1)
                xto_quad_wedge(p, -face_angle, knorm[1]);
            if (should_rotate && k_order >= 0) xto_wedge(p, -face_angle, knorm[0]);
        } else {
            if (should_rotate && k_order >= 0) xto_wedge(p, -face_angle, knorm[0]);
            if (model == 1 && should_rotate && k_order >= 1)
                xto_quad_wedge(p, -face_angle, knorm[1]);
            if (model == 1)
                xto_mult_fringe(p, knorm, kskew, k_order, knl, ksl, kl_order,
                                length / factor_knl_ksl, is_exit, 1);
            xto_dipole_fringe(p, fringe_integral, half_gap, k0);
            if (should_rotate) xto_yrotation(p, -sin_, cos_, -tan_);
        }
    }
}

/* ---------------------------------------------------------------------- */
/* track_magnet_particles: track_magnet.h:288-648 (rbend_model = -1)       */
/* ---------------------------------------------------------------------- */
typedef struct {
    double weight;
    double length;
    int64_t order;
    double inv_factorial_order;
    const double* knl;
    const double* ksl;
    int64_t order_rel;
    double inv_factorial_order_rel;
    const double* knl_rel;
    const double* ksl_rel;
    double rel_ref_strength;
    int64_t num_multipole_kicks;
    int64_t model, default_model, integrator, default_integrator;
    double h, hxl, k0, k1, k2, k3, k0s, k1s, k2s, k3s;
    int body_active;
    int edge_entry_active, edge_exit_active;
    int edge_entry_model, edge_exit_model;
    double edge_entry_angle, edge_exit_angle;
    double edge_entry_angle_fdown, edge_exit_angle_fdown;
    double edge_entry_fint, edge_exit_fint;
    double edge_entry_hgap, edge_exit_hgap;
} xto_magnet;

#define XTO_VSWAP_D(a, b) { double t_ = a; a = b; b = t_; }
#define XTO_VSWAP_I(a, b) { int t_ = a; a = b; b = t_; }

static void xto_track_magnet(xto_part* p, xto_magnet m) {
    double const factor_knl_ksl = 1.0;
    double core_length, factor_knl_ksl_body, factor_knl_ksl_edge, factor_backtrack_edge;
    if (flag_set(p, XTG_FLAG_BACKTRACK)) {
        core_length = -m.length * m.weight;
        factor_knl_ksl_body = -factor_knl_ksl * m.weight;
        factor_knl_ksl_edge = factor_knl_ksl;
        factor_backtrack_edge = -1.;
        m.hxl = -m.hxl;
        XTO_VSWAP_I(m.edge_entry_active, m.edge_exit_active);
        XTO_VSWAP_I(m.edge_entry_model, m.edge_exit_model);
        XTO_VSWAP_D(m.edge_entry_angle, m.edge_exit_angle);
        XTO_VSWAP_D(m.edge_entry_angle_fdown, m.edge_exit_angle_fdown);
        XTO_VSWAP_D(m.edge_entry_fint, m.edge_exit_fint);
        XTO_VSWAP_D(m.edge_entry_hgap, m.edge_exit_hgap);
    } else {
        core_length = m.length * m.weight;
        factor_knl_ksl_body = factor_knl_ksl * m.weight;
        factor_knl_ksl_edge = factor_knl_ksl;
        factor_backtrack_edge = 1.;
    }
    double const knorm[4] = {m.k0, m.k1, m.k2, m.k3};
    double const kskew[4] = {m.k0s, m.k1s, m.k2s, m.k3s};

    if (m.edge_entry_active) {
        xto_magnet_edge(p, m.edge_entry_model, 0, m.edge_entry_hgap, knorm, kskew,
                        m.knl, m.ksl, factor_knl_ksl_edge, m.order, m.knl_rel,
                        factor_knl_ksl_edge * m.rel_ref_strength, m.order_rel,
                        m.length, m.edge_entry_angle, m.edge_entry_angle_fdown,
                        m.edge_entry_fint, factor_backtrack_edge);
        if (p->state <= 0) return;
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
        if (m.weight != 1.0 && n > 0) {
            n = (int64_t)ceil(n * m.weight);
        }
        if (n == 0) {
            if (!xto_kick_is_inactive(m.order, m.knl, m.ksl, m.k0, m.k1, m.k2, m.k3,
                                      m.k0s, m.k1s, m.k2s, m.k3s, m.h)) {
                if (fabs(m.h) < 1e-8) {
                    n = 1;
                } else {
                    double b_circum = 2 * 3.14159 / fabs(m.h);
                    n = fabs(core_length) / b_circum / 0.5e-3;
                    if (n < 1) n = 1;
                }
            }
        }
        xto_body b;
        memset(&b, 0, sizeof(b));
        xto_configure(model, m.k0, m.k1, m.h, &b);
        b.length = core_length;
        b.order = m.order;
        b.inv_factorial_order = m.inv_factorial_order;
        b.knl = m.knl;
        b.ksl = m.ksl;
        b.order_rel = m.order_rel;
        b.inv_factorial_order_rel = m.inv_factorial_order_rel;
        b.knl_rel = m.knl_rel;
        b.ksl_rel = m.ksl_rel;
        b.rel_ref_strength = m.rel_ref_strength;
        b.factor_knl_ksl = factor_knl_ksl_body;
        b.num_multipole_kicks = n;
        b.integrator = (int)integrator;
        b.hxl = m.hxl;
        b.k2 = m.k2; b.k3 = m.k3;
        b.k0s = m.k0s; b.k1s = m.k1s; b.k2s = m.k2s; b.k3s = m.k3s;
        xto_magnet_body(p, &b);
    }

    if (m.edge_exit_active) {
        xto_magnet_edge(p, m.edge_exit_model, 1, m.edge_exit_hgap, knorm, kskew,
                        m.knl, m.ksl, factor_knl_ksl_edge, m.order, m.knl_rel,
                        factor_knl_ksl_edge * m.rel_ref_strength, m.order_rel,
                        m.length, m.edge_exit_angle, m.edge_exit_angle_fdown,
                        m.edge_exit_fint, factor_backtrack_edge);
    }
}

/* ---------------------------------------------------------------------- */
/* RF: track_rf.h                                                          */
/* ---------------------------------------------------------------------- */

/* track_rf.h:17-167 with order = -1 and zero transverse voltage (Cavity). */
static void xto_rf_kick(xto_part* p, double voltage, double frequency,
                        double harmonic, double lag, double phase,
                        int64_t absolute_time, int kill_energy_kick,
                        int preserve_angle) {
    double phase0 = 0;
    double const beta0 = p->beta0;
    if (harmonic != 0) {
        double const line_length = p->line_length;
        double const t_rev0 = line_length / (beta0 * XTO_C_LIGHT);
        frequency += (harmonic / t_rev0);
    }
    if (absolute_time == 1) {
        double const t_sim = p->t_sim;
        int64_t const at_turn = p->at_turn;
        phase0 += 2 * XTO_PI * at_turn * frequency * t_sim;
    }
    double const zeta = p->zeta;
    double const q = fabs(p->q0) * p->charge_ratio;
    double const tau = zeta / beta0;
    double const energy_kick = q * voltage
        * sin(phase0 + XTO_DEG2RAD * lag + phase
              - (2.0 * XTO_PI) / XTO_C_LIGHT * frequency * tau);
    double const rfmultipole_energy_kick = 0;
    if (!kill_energy_kick) {
        xto_add_to_energy(p, energy_kick + rfmultipole_energy_kick,
                          preserve_angle ? 0 : 1);
    }
}

typedef struct {
    double weight, length, voltage, frequency, harmonic, lag, phase;
    int64_t absolute_time, num_kicks, model, integrator;
} xto_rf;

/* track_rf.h:170-290 (body) and 293-453 (track_rf_particles) */
static void xto_track_rf(xto_part* p, xto_rf r, int preserve_angle) {
    int const kill = flag_set(p, XTG_FLAG_KILL_CAVITY_KICK);
    double body_length;
    if (flag_set(p, XTG_FLAG_BACKTRACK)) {
        body_length = -r.length;
        r.voltage = -r.voltage;
    } else {
        body_length = r.length;
    }
    int64_t integrator = r.integrator;
    int64_t model = r.model;
    int64_t n = r.num_kicks;
    if (integrator == 0) integrator = 3;
    if (model == 0) model = 6;
    if (model == -1) {
        integrator = 3;
        n = 1;
    }
    if (r.weight != 1.0 && n > 0) n = (int64_t)ceil(n * r.weight);
    if (n == 0) n = 1;
    xto_body cfg;
    memset(&cfg, 0, sizeof(cfg));
    xto_configure(model, 0, 0, 0, &cfg);
    int const dm = cfg.drift_model;

    double const length = body_length * r.weight;
    double const voltage = r.voltage * r.weight;
#define XTO_RDRIFT(L) xto_magnet_drift(p, (L), 0., 0., 0., dm)
#define XTO_RKICK(W) xto_rf_kick(p, voltage * (W), r.frequency, r.harmonic, r.lag, \
                                 r.phase, r.absolute_time, kill, preserve_angle)
    if (integrator == 1) {
        double const kick_weight = 1. / n;
        double edge_drift_weight = 0.5;
        double inside_drift_weight = 0;
        if (n > 1) {
            edge_drift_weight = 1. / (2 * (1 + n));
            inside_drift_weight = (((double)n) / ((double)(n * n) - 1));
        }
        XTO_RDRIFT(edge_drift_weight * length);
        for (int i_kick = 0; i_kick < n - 1; i_kick++) {
            XTO_RKICK(kick_weight);
            XTO_RDRIFT(inside_drift_weight * length);
        }
        XTO_RKICK(kick_weight);
        XTO_RDRIFT(edge_drift_weight * length);
    } else if (integrator == 3) {
        double const kick_weight = 1. / n;
        double const drift_weight = kick_weight;
        for (int i_kick = 0; i_kick < n; i_kick++) {
            XTO_RDRIFT(0.5 * drift_weight * length);
            XTO_RKICK(kick_weight);
            XTO_RDRIFT(0.5 * drift_weight * length);
        }
    } else if (integrator == 2) {
        int64_t const num_slices = (n / 7 + (n % 7 != 0));
        double const slice_length = length / (num_slices);
        double const kick_weight = 1. / num_slices;
        for (int ii = 0; ii < num_slices; ii++) {
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[0]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[0]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[1]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[1]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[2]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[2]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[3]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[3]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[3]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[2]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[2]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[1]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[1]);
            XTO_RKICK(kick_weight * XTO_K_YOSHIDA[0]);
            XTO_RDRIFT(slice_length * XTO_D_YOSHIDA[0]);
        }
    }
#undef XTO_RDRIFT
#undef XTO_RKICK
}

/* ---------------------------------------------------------------------- */
/* 1/n!: xtrack/headers/factorial.h:4-35                                   */
/* ---------------------------------------------------------------------- */
static double xto_one_over_factorial(int64_t n) {
    if (n < 0) return 0.;
    double f = 1.0;
    for (int64_t i = 2; i <= n; i++) f *= (double)i;  /* exact up to 22! */
    return 1. / f;
}

/* ---------------------------------------------------------------------- */
/* Per-class dispatch: the element _track_local_particle functions         */
/* ---------------------------------------------------------------------- */

static double xto_main_strength(const xtg_element* e) {
    /* bend.h:31, quadrupole.h:31, sextupole.h:31, octupole.h:31,
     * multipole.h:30 */
    switch (e->cls) {
    case XTG_CLS_BEND: return e->k0 * e->length;
    case XTG_CLS_QUADRUPOLE: return e->length * (e->main_is_skew ? e->k1s : e->k1);
    case XTG_CLS_SEXTUPOLE: return e->length * (e->main_is_skew ? e->k2s : e->k2);
    case XTG_CLS_OCTUPOLE: return e->length * (e->main_is_skew ? e->k3s : e->k3);
    case XTG_CLS_MULTIPOLE:
        return e->main_is_skew ? e->ksl[e->main_order] : e->knl[e->main_order];
    default: return 0.;
    }
}

static void xto_fill_magnet(const xtg_element* e, xto_magnet* m) {
    memset(m, 0, sizeof(*m));
    m->weight = 1.0;
    m->length = e->length;
    m->order = e->order;
    m->inv_factorial_order = e->inv_factorial_order;
    m->knl = e->knl;
    m->ksl = e->ksl;
    m->order_rel = e->order_rel;
    m->inv_factorial_order_rel = xto_one_over_factorial(e->order_rel);
    m->knl_rel = e->knl_rel;
    m->ksl_rel = e->ksl_rel;
    m->rel_ref_strength = xto_main_strength(e);
    m->num_multipole_kicks = e->num_multipole_kicks;
    m->model = e->model;
    m->integrator = e->integrator;
    m->body_active = 1;
    switch (e->cls) {
    case XTG_CLS_BEND:
        /* bend.h:20-73 */
        m->default_model = XTO_BEND_DEFAULT_MODEL;
        m->default_integrator = XTO_BEND_DEFAULT_INTEGRATOR;
        m->h = e->h; m->k0 = e->k0; m->k1 = e->k1; m->k2 = e->k2;
        m->edge_entry_active = e->edge_entry_active;
        m->edge_exit_active = e->edge_exit_active;
        m->edge_entry_model = e->edge_entry_model;
        m->edge_exit_model = e->edge_exit_model;
        m->edge_entry_angle = e->edge_entry_angle;
        m->edge_exit_angle = e->edge_exit_angle;
        m->edge_entry_angle_fdown = e->edge_entry_angle_fdown;
        m->edge_exit_angle_fdown = e->edge_exit_angle_fdown;
        m->edge_entry_fint = e->edge_entry_fint;
        m->edge_exit_fint = e->edge_exit_fint;
        m->edge_entry_hgap = e->edge_entry_hgap;
        m->edge_exit_hgap = e->edge_exit_hgap;
        break;
    case XTG_CLS_QUADRUPOLE:
        /* quadrupole.h:20-73 */
        m->default_model = XTO_QUADRUPOLE_DEFAULT_MODEL;
        m->default_integrator = XTO_STRAIGHT_DEFAULT_INTEGRATOR;
        m->k1 = e->k1; m->k1s = e->k1s;
        m->edge_entry_active = e->edge_entry_active;
        m->edge_exit_active = e->edge_exit_active;
        m->edge_entry_model = 1; m->edge_exit_model = 1;
        break;
    case XTG_CLS_SEXTUPOLE:
        m->default_model = XTO_SEXTUPOLE_DEFAULT_MODEL;
        m->default_integrator = XTO_STRAIGHT_DEFAULT_INTEGRATOR;
        m->k2 = e->k2; m->k2s = e->k2s;
        m->edge_entry_active = e->edge_entry_active;
        m->edge_exit_active = e->edge_exit_active;
        m->edge_entry_model = 1; m->edge_exit_model = 1;
        break;
    case XTG_CLS_OCTUPOLE:
        m->default_model = XTO_OCTUPOLE_DEFAULT_MODEL;
        m->default_integrator = XTO_STRAIGHT_DEFAULT_INTEGRATOR;
        m->k3 = e->k3; m->k3s = e->k3s;
        m->edge_entry_active = e->edge_entry_active;
        m->edge_exit_active = e->edge_exit_active;
        m->edge_entry_model = 1; m->edge_exit_model = 1;
        break;
    case XTG_CLS_MULTIPOLE:
        /* multipole.h:18-73: thin unless isthick */
        m->default_model = XTO_MULTIPOLE_DEFAULT_MODEL;
        m->default_integrator = XTO_STRAIGHT_DEFAULT_INTEGRATOR;
        m->model = (e->isthick <= 0) ? -1 : e->model;
        m->hxl = e->hxl;
        break;
    default: break;
    }
}

static void xto_monitor(const xtg_monitor* m, const xto_part* p, const xtg_particles* src,
                        int64_t isrc);

/* last_turns_monitor.h:17-55 */
static void xto_last_turns(const xtg_element_monitor* m, const xto_part* p) {
    int64_t const particle_id_stop = m->particle_id_start + m->num_particles;
    int64_t const particle_id = p->particle_id;
    int64_t const at_turn = p->at_turn;
    if (at_turn >= 0 && at_turn % m->every_n_turns == 0 && m->particle_id_start <= particle_id &&
        particle_id < particle_id_stop) {
        int64_t const offset = (at_turn / m->every_n_turns) % m->n_last_turns;
        int64_t const ip = particle_id - m->particle_id_start;
        int64_t const slot = m->n_last_turns * ip + offset;
        m->lost_at_offset[ip] = (uint32_t)offset;
        m->lt_particle_id[slot] = (uint32_t)particle_id;
        m->lt_at_turn[slot] = (uint32_t)at_turn;
        m->lt_x[slot] = (float)p->x;
        m->lt_px[slot] = (float)p->px;
        m->lt_y[slot] = (float)p->y;
        m->lt_py[slot] = (float)p->py;
        m->lt_delta[slot] = (float)p->delta;
        m->lt_zeta[slot] = (float)p->zeta;
    }
}

/* beam_position_monitor.h:16-58 (atomic sums, as the reference's atomicAdd) */
static void xto_bpm(const xtg_element_monitor* m, const xto_part* p) {
    int64_t const particle_id_stop = m->particle_id_start + m->num_particles;
    int64_t const particle_id = p->particle_id;
    if (particle_id_stop < 0 || (m->particle_id_start <= particle_id && particle_id < particle_id_stop)) {
        double const zeta = p->zeta;
        double const at_turn = (double)p->at_turn;
        double const beta0 = p->beta0;
        int64_t const slot = (int64_t)round(m->sampling_frequency *
                                            ((at_turn - m->start_at_turn) / m->frev - zeta / beta0 / XTO_C_LIGHT));
        if (slot >= 0 && slot < m->n_slots) {
            double const x = p->x, y = p->y;
#ifdef _OPENMP
#pragma omp atomic
#endif
            m->count[slot] += 1.0;
#ifdef _OPENMP
#pragma omp atomic
#endif
            m->x_sum[slot] += x;
#ifdef _OPENMP
#pragma omp atomic
#endif
            m->y_sum[slot] += y;
            if (m->kind == XTG_MON_BEAM_SIZE) {
                /* beam_size_monitor.h:16-64 */
#ifdef _OPENMP
#pragma omp atomic
#endif
                m->x2_sum[slot] += x * x;
#ifdef _OPENMP
#pragma omp atomic
#endif
                m->y2_sum[slot] += y * y;
            }
        }
    }
}

/* beam_profile_monitor.h:16-80 */
static void xto_profile(const xtg_element_monitor* m, const xto_part* p) {
    int64_t const particle_id_stop = m->particle_id_start + m->num_particles;
    int64_t const particle_id = p->particle_id;
    if (particle_id_stop < 0 || (m->particle_id_start <= particle_id && particle_id < particle_id_stop)) {
        double const zeta = p->zeta;
        double const at_turn = (double)p->at_turn;
        double const beta0 = p->beta0;
        int64_t const sample = (int64_t)round(m->sampling_frequency *
                                              ((at_turn - m->start_at_turn) / m->frev - zeta / beta0 / XTO_C_LIGHT));
        if (sample >= 0 && sample < m->n_slots) {
            int64_t const bin_x = (int64_t)floor((p->x - m->x_min) / m->dx);
            int64_t const bin_y = (int64_t)floor((p->y - m->y_min) / m->dy);
            if (bin_x >= 0 && bin_x < m->nx) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                m->counts_x[sample * m->nx + bin_x] += 1.;
            }
            if (bin_y >= 0 && bin_y < m->ny) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                m->counts_y[sample * m->ny + bin_y] += 1.;
            }
        }
    }
}

/* track_srotation.h:9-37 (no spin) */
static void xto_srotation(xto_part* p, double sin_z, double cos_z) {
    double const x = p->x, y = p->y, px = p->px, py = p->py;
    p->x = cos_z * x + sin_z * y;
    p->y = -sin_z * x + cos_z * y;
    p->px = cos_z * px + sin_z * py;
    p->py = -sin_z * px + cos_z * py;
}

/* Per particle (indexed by particle_id), the smallest distance in metres
 * from the particle to the edge of any aperture it reached, inside or out
 * (set by xto_set_edge_distance; no counterpart in the reference: it lists
 * the particles whose survival a last-ulp difference could flip). The
 * distance to a rectangle is that to its nearest side line, to an ellipse
 * |sqrt(x^2/a^2 + y^2/b^2) - 1| * min(a, b), to a polygon that to its
 * nearest segment. */
static double* xto_edge = NULL;
static int64_t xto_edge_n = 0;

static void xto_record_edge(const xtg_element* e, const xto_part* p) {
    int64_t const id = p->particle_id;
    if (!xto_edge || id < 0 || id >= xto_edge_n) return;
    double const x = p->x, y = p->y;
    double d = INFINITY;
    if (e->cls == XTG_CLS_LIMIT_RECT || e->cls == XTG_CLS_LIMIT_RECT_ELLIPSE) {
        double const lo_x = e->cls == XTG_CLS_LIMIT_RECT ? e->min_x : -e->max_x;
        double const lo_y = e->cls == XTG_CLS_LIMIT_RECT ? e->min_y : -e->max_y;
        d = fmin(fmin(fabs(x - lo_x), fabs(e->max_x - x)), fmin(fabs(y - lo_y), fabs(e->max_y - y)));
    }
    if (e->cls == XTG_CLS_LIMIT_ELLIPSE || e->cls == XTG_CLS_LIMIT_RECT_ELLIPSE) {
        double const a = sqrt(e->a_squ), b = sqrt(e->b_squ);
        double const r = sqrt(x * x / e->a_squ + y * y / e->b_squ);
        d = fmin(d, fabs(r - 1.0) * fmin(a, b));
    }
    if (e->cls == XTG_CLS_LIMIT_POLYGON) {
        const xtg_polygon* pg = (const xtg_polygon*)(uintptr_t)e->aux;
        for (int64_t ii = 0; ii < pg->n_vertices; ii++) {
            int64_t const jj = (ii + 1) % pg->n_vertices;
            double const x0 = pg->x_vertices[ii], y0 = pg->y_vertices[ii];
            double const dx = pg->x_vertices[jj] - x0, dy = pg->y_vertices[jj] - y0;
            double const l2 = dx * dx + dy * dy;
            double t = l2 > 0.0 ? ((x - x0) * dx + (y - y0) * dy) / l2 : 0.0;
            if (t < 0.0) t = 0.0;
            else if (t > 1.0) t = 1.0;
            d = fmin(d, hypot(x - (x0 + t * dx), y - (y0 + t * dy)));
        }
    }
    if (d != d) d = 0.0;   /* a NaN coordinate is as close to the edge as can be */
    if (d < xto_edge[id]) xto_edge[id] = d;
}

int32_t xto_set_edge_distance(double* out, int64_t n) {
    xto_edge = out;
    xto_edge_n = out ? n : 0;
    return XTG_OK;
}

/* The aperture check of one LimitEllipse / LimitPolygon / LimitRect on the
 * particle's current x, y (limitellipse.h, limitpolygon.h, limitrect.h). */
static void xto_aperture(const xtg_element* e, xto_part* p) {
    if (xto_edge && !flag_set(p, XTG_FLAG_IGNORE_LOCAL_APERTURE)) xto_record_edge(e, p);
    switch (e->cls) {
    case XTG_CLS_LIMIT_RECT_ELLIPSE: {
        /* limitrectellipse.h:14-44 */
        if (flag_set(p, XTG_FLAG_IGNORE_LOCAL_APERTURE)) return;
        double const max_x = e->max_x, max_y = e->max_y;
        double const x = p->x, y = p->y;
        double const temp = x * x * e->b_squ + y * y * e->a_squ;
        int64_t const is_alive = (int64_t)((x <= max_x) && (x >= -max_x) && (y <= max_y) &&
                                           (y >= -max_y) && (temp <= e->a_b_squ));
        if (!is_alive) p->state = 0;
        return;
    }
    case XTG_CLS_LIMIT_ELLIPSE: {
        /* limitellipse.h:12-38 */
        if (flag_set(p, XTG_FLAG_IGNORE_LOCAL_APERTURE)) return;
        double const x = p->x, y = p->y;
        double const temp = x * x * e->b_squ + y * y * e->a_squ;
        int64_t const is_alive = (int64_t)(temp <= e->a_b_squ);
        if (!is_alive) p->state = 0;
        return;
    }
    case XTG_CLS_LIMIT_POLYGON: {
        /* limitpolygon.h:13-90 (CPU build: inscribed-circle shortcut) */
        if (flag_set(p, XTG_FLAG_IGNORE_LOCAL_APERTURE)) return;
        const xtg_polygon* pg = (const xtg_polygon*)(uintptr_t)e->aux;
        int64_t const N_edg = pg->n_vertices;
        double inner_radius_sq = 0.0;
        for (int64_t ii = 0; ii < N_edg; ii++) {
            int64_t const jj = (ii + 1) % N_edg;
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
                double const x_proj = x0 + t * dx;
                double const y_proj = y0 + t * dy;
                dist_sq = x_proj * x_proj + y_proj * y_proj;
            } else {
                dist_sq = x0 * x0 + y0 * y0;
            }
            if (ii == 0 || dist_sq < inner_radius_sq) inner_radius_sq = dist_sq;
        }
        double const x = p->x, y = p->y;
        if (x * x + y * y > inner_radius_sq) {
            int64_t ii = 0, jj = N_edg - 1;
            int64_t is_alive = 0;
            while (ii < N_edg) {
                double const Vx_ii = pg->x_vertices[ii], Vx_jj = pg->x_vertices[jj];
                double const Vy_ii = pg->y_vertices[ii], Vy_jj = pg->y_vertices[jj];
                if (((Vy_ii > y) != (Vy_jj > y)) &&
                    (x < (Vx_jj - Vx_ii) * (y - Vy_ii) / (Vy_jj - Vy_ii) + Vx_ii))
                    is_alive = !is_alive;
                jj = ii;
                ii++;
            }
            if (!is_alive) p->state = 0;
        }
        return;
    }
    case XTG_CLS_LIMIT_RECT: {
        /* limitrect.h:9-36 */
        if (flag_set(p, XTG_FLAG_IGNORE_LOCAL_APERTURE)) return;
        double const x = p->x, y = p->y;
        int64_t const is_alive = (int64_t)((x >= e->min_x) && (x <= e->max_x)
                                           && (y >= e->min_y) && (y <= e->max_y));
        if (!is_alive) p->state = 0;
        return;
    }
    default:
        return;
    }
}

/* Transverse shift and s-tilt of an element of zero length and straight
 * frame: track_misalignment_entry/exit_straight (track_misalignments.h:
 * 38-130) with zero length, anchor, shift_s, rot_x_rad and rot_y_rad. The
 * entry XYShift, then S_ROTATE by rot_s_rad_no_frame and by rot_s_rad;
 * the exit S_ROTATE by -rot_s_rad and -rot_s_rad_no_frame, then the XYShift
 * (the roles swap in backtracking). */
static int xto_shifted(const xtg_element* e) {
    return e->shift_x != 0.0 || e->shift_y != 0.0 || e->rot_s_rad_no_frame != 0.0 || e->rot_s_rad != 0.0;
}
static void xto_shift_in(const xtg_element* e, xto_part* p, int backtrack) {
    double const psi_nf = e->rot_s_rad_no_frame, psi_wf = e->rot_s_rad;
    double mx, my;
    if (!backtrack) { mx = e->shift_x - 0.0; my = e->shift_y - 0.0; }
    else { mx = -(0.0 - e->shift_x); my = -(0.0 - e->shift_y); }
    p->x += -mx;
    p->y += -my;
    if (psi_nf != 0.0) xto_srotation(p, sin(psi_nf), cos(psi_nf));
    if (psi_wf != 0.0) xto_srotation(p, sin(psi_wf), cos(psi_wf));
}
static void xto_shift_out(const xtg_element* e, xto_part* p, int backtrack) {
    double const psi_nf = e->rot_s_rad_no_frame, psi_wf = e->rot_s_rad;
    double mx, my;
    if (psi_wf != 0.0) xto_srotation(p, sin(-psi_wf), cos(-psi_wf));
    if (psi_nf != 0.0) xto_srotation(p, sin(-psi_nf), cos(-psi_nf));
    if (!backtrack) { mx = 0.0 - e->shift_x; my = 0.0 - e->shift_y; }
    else { mx = -(e->shift_x - 0.0); my = -(e->shift_y - 0.0); }
    p->x += -mx;
    p->y += -my;
}

static int xto_apply_local(const xtg_element* e, const xtg_config* cfg, xto_part* p,
                           const xtg_particles* src, int64_t isrc);

/* Applies one element to one particle. Returns whether the class is
 * statically thick (global aperture check follows, tracker.py:681-689).
 * `src`/`isrc` locate the particle in its arrays (monitors copy the fields
 * the push does not carry). A thin Multipole (no `h` field: straight;
 * `isthick` 0: zero length) or a DipoleEdge with a transverse shift or tilt
 * runs inside the transforms of track_local_particle_with_transformations.h:
 * 146-165; the exit only for a particle that survives. Apertures apply
 * theirs around the test itself. */
static int xto_apply(const xtg_element* e, const xtg_config* cfg, xto_part* p,
                     const xtg_particles* src, int64_t isrc) {
    if (((e->cls == XTG_CLS_MULTIPOLE && e->isthick <= 0 && e->slice == XTG_SLICE_NONE) ||
         e->cls == XTG_CLS_DIPOLE_EDGE) && xto_shifted(e)) {
        int const backtrack = flag_set(p, XTG_FLAG_BACKTRACK);
        xto_shift_in(e, p, backtrack);
        int const thick = xto_apply_local(e, cfg, p, src, isrc);
        if (p->state > 0) xto_shift_out(e, p, backtrack);
        return thick;
    }
    return xto_apply_local(e, cfg, p, src, isrc);
}

static int xto_apply_local(const xtg_element* e, const xtg_config* cfg, xto_part* p,
                           const xtg_particles* src, int64_t isrc) {
    int const backtrack = flag_set(p, XTG_FLAG_BACKTRACK);
    switch (e->cls) {
    case XTG_CLS_MARKER:
        return 0;
    case XTG_CLS_MONITOR: {
        /* monitors/*.py: get_backtrack_element is a Marker */
        const xtg_element_monitor* m = (const xtg_element_monitor*)(uintptr_t)e->aux;
        if (backtrack) return 0;
        if (m->kind == XTG_MON_PARTICLES) xto_monitor(&m->particles, p, src, isrc);
        else if (m->kind == XTG_MON_LAST_TURNS) xto_last_turns(m, p);
        else if (m->kind == XTG_MON_BEAM_POSITION || m->kind == XTG_MON_BEAM_SIZE) xto_bpm(m, p);
        else if (m->kind == XTG_MON_BEAM_PROFILE) xto_profile(m, p);
        return 0;
    }
    case XTG_CLS_DRIFT: {
        /* drift.h:13-37 */
        double length = e->length;
        if (backtrack) length = -length;
        int model;
        if (cfg->use_exact_drifts) model = 2;
        else {
            model = e->model;
            if (model == 0) model = 1;
        }
        if (model == 1) xto_drift_expanded(p, length);
        else if (model == 2) xto_drift_exact(p, length);
        return 1;
    }
    case XTG_CLS_LIMIT_ELLIPSE:
    case XTG_CLS_LIMIT_POLYGON:
    case XTG_CLS_LIMIT_RECT_ELLIPSE:
    case XTG_CLS_LIMIT_RECT: {
        /* track_local_particle_with_transformations.h:146-165 with only
         * shift_x / shift_y nonzero (track_misalignments.h:38-112): the entry
         * XYShift for the particle reaching the element, the exit XYShift
         * only if it survives (the CPU per-particle blocks skip lost
         * particles); both also when local apertures are ignored */
        int const shifted = xto_shifted(e);
        if (shifted) xto_shift_in(e, p, backtrack);
        xto_aperture(e, p);
        if (shifted && p->state > 0) xto_shift_out(e, p, backtrack);
        return 0;
    }
    case XTG_CLS_DIPOLE_EDGE: {
        /* dipoleedge.h:14-71 (no synchrotron-radiation taper) */
        if (e->model == 0) {
            double r21 = e->r21, r43 = e->r43;
            if (backtrack) {
                r21 = -r21;
                r43 = -r43;
            }
            /* track_dipole_edge_linear.h:29-37 */
            double const x = p->x, y = p->y, chi = p->chi;
            p->px += chi * r21 * x;
            p->py += chi * r43 * y;
        } else if (e->model == 1) {
            if (backtrack) {
                xto_kill(p, -32);
                return 0;
            }
            /* track_dipole_edge_nonlinear.h:9-44 */
            double sin_, cos_, tan_;
            if (fabs(e->e1) < 10e-10) {
                sin_ = -999.0; cos_ = -999.0; tan_ = -999.0;
            } else {
                sin_ = sin(e->e1); cos_ = cos(e->e1); tan_ = tan(e->e1);
            }
            if (e->side == 0) {
                if (sin_ > -99.) xto_yrotation(p, -sin_, cos_, -tan_);
                xto_dipole_fringe(p, e->fint, e->hgap, e->k);
                if (sin_ > -99.) xto_wedge(p, -e->e1, e->k);
            } else {
                if (sin_ > -99.) xto_wedge(p, -e->e1, e->k);
                xto_dipole_fringe(p, e->fint, e->hgap, -e->k);
                if (sin_ > -99.) xto_yrotation(p, -sin_, cos_, -tan_);
            }
        }
        return 0;
    }
    case XTG_CLS_CAVITY: {
        xto_rf r;
        r.weight = 1.0;
        r.length = e->length;
        r.voltage = e->voltage;
        r.frequency = e->frequency;
        r.harmonic = e->harmonic;
        r.lag = e->lag;
        r.phase = e->phase;
        r.absolute_time = e->absolute_time;
        r.num_kicks = e->num_multipole_kicks;
        r.model = e->model;
        r.integrator = e->integrator;
        switch (e->slice) {
        case XTG_SLICE_NONE:          /* cavity.h:11-48 */
            xto_track_rf(p, r, cfg->cavity_preserve_angle);
            return 1;
        case XTG_SLICE_THICK:         /* thick_slice_cavity.h */
            r.weight = e->weight;
            xto_track_rf(p, r, cfg->cavity_preserve_angle);
            return 1;
        case XTG_SLICE_THIN:          /* thin_slice_cavity.h */
            r.weight = e->weight;
            r.num_kicks = 1;
            r.model = -1;
            r.integrator = 3;
            xto_track_rf(p, r, cfg->cavity_preserve_angle);
            return 0;
        case XTG_SLICE_DRIFT: {       /* drift_slice_cavity.h */
            double length = e->weight * e->length;
            if (backtrack) length = -e->weight * e->length;
            xto_drift_default(p, length, cfg->use_exact_drifts);
            return 1;
        }
        default:
            return 0;
        }
    }
    case XTG_CLS_MULTIPOLE:
    case XTG_CLS_BEND:
    case XTG_CLS_QUADRUPOLE:
    case XTG_CLS_SEXTUPOLE:
    case XTG_CLS_OCTUPOLE: {
        int const statically_thick = (e->cls != XTG_CLS_MULTIPOLE);
        xto_magnet m;
        xto_fill_magnet(e, &m);
        switch (e->slice) {
        case XTG_SLICE_NONE:
            xto_track_magnet(p, m);
            return statically_thick;
        case XTG_SLICE_THICK:
            /* thick_slice_*.h: weight from the slice, edges off */
            m.weight = e->weight;
            m.edge_entry_active = 0;
            m.edge_exit_active = 0;
            m.edge_entry_model = 0;
            m.edge_exit_model = 0;
            xto_track_magnet(p, m);
            return 1;
        case XTG_SLICE_THIN:
            /* thin_slice_*.h: kick only */
            m.weight = e->weight;
            m.num_multipole_kicks = 1;
            m.model = -1;
            m.integrator = 3;
            m.edge_entry_active = 0;
            m.edge_exit_active = 0;
            xto_track_magnet(p, m);
            return 0;
        case XTG_SLICE_DRIFT: {
            /* drift_slice_*.h */
            double length = e->weight * e->length;
            if (backtrack) length = -e->weight * e->length;
            xto_drift_default(p, length, cfg->use_exact_drifts);
            return 1;
        }
        case XTG_SLICE_ENTRY:
        case XTG_SLICE_EXIT: {
            /* thin_slice_*_entry.h / _exit.h: body off, one edge */
            int const is_entry = (e->slice == XTG_SLICE_ENTRY);
            m.weight = 0.;
            m.num_multipole_kicks = 0;
            m.model = 0;
            m.integrator = 0;
            m.body_active = 0;
            m.edge_entry_active = is_entry ? m.edge_entry_active : 0;
            m.edge_exit_active = is_entry ? 0 : m.edge_exit_active;
            if (is_entry) {
                m.edge_exit_model = 0;
                m.edge_exit_angle = 0; m.edge_exit_angle_fdown = 0;
                m.edge_exit_fint = 0; m.edge_exit_hgap = 0;
            } else {
                m.edge_entry_model = 0;
                m.edge_entry_angle = 0; m.edge_entry_angle_fdown = 0;
                m.edge_entry_fint = 0; m.edge_entry_hgap = 0;
            }
            xto_track_magnet(p, m);
            return 0;
        }
        default:
            return 0;
        }
    }
    default:
        return 0;
    }
}

/* local_particle_custom_api.h:259-287 */
static void xto_global_aperture(const xtg_config* cfg, xto_part* p) {
    if (!cfg->has_global_xy_limit) return;
    if (flag_set(p, XTG_FLAG_IGNORE_GLOBAL_APERTURE)) return;
    double const lim = cfg->global_xy_limit;
    double const x = p->x, y = p->y;
    int64_t const is_within = (int64_t)((x >= -lim) && (x <= lim) && (y >= -lim) && (y <= lim));
    if (p->state > 0 && !is_within) p->state = -1;
}

/* ---------------------------------------------------------------------- */
/* Validation of the element set                                           */
/* ---------------------------------------------------------------------- */
int32_t xto_validate(const xtg_element* els, int64_t n, char* msg, int64_t msg_len) {
    for (int64_t i = 0; i < n; i++) {
        const xtg_element* e = &els[i];
        const char* why = NULL;
        if (e->cls < 0 || e->cls >= XTG_NUM_CLS) why = "unknown element class";
        else if (e->cls == XTG_CLS_MONITOR && e->aux == 0)
            why = "monitor element without its descriptor";
        else if (e->cls == XTG_CLS_LIMIT_POLYGON &&
                 (e->aux == 0 || ((const xtg_polygon*)(uintptr_t)e->aux)->n_vertices < 3))
            why = "LimitPolygon needs at least 3 vertices";
        else if (e->slice < 0 || e->slice > XTG_SLICE_EXIT) why = "unknown slice kind";
        else if (e->order < 0 || e->order >= XTG_MAX_KNL) why = "multipole order out of range";
        else if (e->order_rel < -1 || e->order_rel >= 20) why = "relative multipole order out of range (0..19)";
        else if (((e->shift_x != 0 || e->shift_y != 0 || e->rot_s_rad != 0 || e->rot_s_rad_no_frame != 0)
                  && e->cls != XTG_CLS_LIMIT_RECT && e->cls != XTG_CLS_LIMIT_ELLIPSE
                  && e->cls != XTG_CLS_LIMIT_POLYGON && e->cls != XTG_CLS_LIMIT_RECT_ELLIPSE
                  && e->cls != XTG_CLS_DIPOLE_EDGE
                  && !(e->cls == XTG_CLS_MULTIPOLE && e->isthick <= 0 && e->slice == XTG_SLICE_NONE))
                 || e->shift_s != 0 || e->rot_x_rad != 0 || e->rot_y_rad != 0)
            why = "misalignments (shift/rotation) are not supported (transverse shifts and tilts: "
                  "apertures, thin Multipoles and DipoleEdges only)";
        else if (e->cls >= XTG_CLS_MULTIPOLE && e->cls <= XTG_CLS_OCTUPOLE) {
            int64_t model = e->model;
            if (e->cls == XTG_CLS_MULTIPOLE && e->isthick <= 0) model = -1;
            if (model == 0) {
                model = (e->cls == XTG_CLS_BEND) ? 3 : (e->cls == XTG_CLS_QUADRUPOLE) ? 4 : 6;
            }
            if (model == -2) why = "solenoid model is not supported";
            else if (model < -1 || model > 8) why = "unknown magnet model";
            int const entry = e->edge_entry_active && (e->slice == XTG_SLICE_NONE || e->slice == XTG_SLICE_ENTRY);
            int const exit_ = e->edge_exit_active && (e->slice == XTG_SLICE_NONE || e->slice == XTG_SLICE_EXIT);
            int const em_in = (e->cls == XTG_CLS_BEND) ? e->edge_entry_model : 1;
            int const em_out = (e->cls == XTG_CLS_BEND) ? e->edge_exit_model : 1;
            if ((entry && (em_in < -1 || em_in > 3)) || (exit_ && (em_out < -1 || em_out > 3)))
                why = "unknown edge model";
            if (e->integrator < 0 || e->integrator > 3) why = "unknown integrator";
        } else if (e->cls == XTG_CLS_CAVITY) {
            int64_t model = e->model == 0 ? 6 : e->model;
            if (!(model == -1 || model == 4 || model == 5 || model == 6))
                why = "unsupported cavity model";
        } else if (e->cls == XTG_CLS_DIPOLE_EDGE) {
            if (e->model < -1 || e->model > 1) why = "unknown DipoleEdge model (linear, full, suppressed)";
            else if (e->side != 0 && e->side != 1) why = "DipoleEdge side must be 0 (entry) or 1 (exit)";
        }
        if (why) {
            if (msg && msg_len > 0) snprintf(msg, (size_t)msg_len, "element %lld: %s", (long long)i, why);
            return XTG_E_UNSUPPORTED;
        }
    }
    return XTG_OK;
}

/* ---------------------------------------------------------------------- */
/* Particles <-> local particle                                            */
/* ---------------------------------------------------------------------- */
static void xto_load(const xtg_particles* P, int64_t i, uint64_t flags, double line_length,
                     xto_part* p) {
    p->x = P->x[i]; p->px = P->px[i]; p->y = P->y[i]; p->py = P->py[i];
    p->zeta = P->zeta[i]; p->delta = P->delta[i]; p->ptau = P->ptau[i];
    p->rpp = P->rpp[i]; p->rvv = P->rvv[i]; p->s = P->s[i];
    p->chi = P->chi[i]; p->charge_ratio = P->charge_ratio[i];
    p->beta0 = P->beta0[i]; p->p0c = P->p0c[i]; p->q0 = P->q0;
    p->ax = P->ax ? P->ax[i] : 0.; p->ay = P->ay ? P->ay[i] : 0.;
    p->t_sim = P->t_sim;
    p->state = P->state[i]; p->at_element = P->at_element[i];
    p->at_turn = P->at_turn[i]; p->particle_id = P->particle_id[i];
    p->track_flags = flags;
    p->line_length = line_length;
}

static void xto_store(const xto_part* p, const xtg_particles* P, int64_t i) {
    P->x[i] = p->x; P->px[i] = p->px; P->y[i] = p->y; P->py[i] = p->py;
    P->zeta[i] = p->zeta; P->delta[i] = p->delta; P->ptau[i] = p->ptau;
    P->rpp[i] = p->rpp; P->rvv[i] = p->rvv; P->s[i] = p->s;
    if (P->ax) P->ax[i] = p->ax;
    if (P->ay) P->ay[i] = p->ay;
    P->state[i] = p->state; P->at_element[i] = p->at_element;
    P->at_turn[i] = p->at_turn;
}

/* One record of LocalParticle_to_Particles into the monitor data
 * (particles.py:157-180); NULL arrays are skipped. */
static void xto_monitor_store(const xto_part* p, const xtg_particles* src, int64_t isrc,
                              const xtg_particles* D, int64_t k) {
#define XTO_ST(f, v) if (D->f) D->f[k] = (v)
    XTO_ST(x, p->x); XTO_ST(px, p->px); XTO_ST(y, p->y); XTO_ST(py, p->py);
    XTO_ST(zeta, p->zeta); XTO_ST(delta, p->delta); XTO_ST(ptau, p->ptau);
    XTO_ST(rpp, p->rpp); XTO_ST(rvv, p->rvv); XTO_ST(s, p->s);
    XTO_ST(chi, p->chi); XTO_ST(charge_ratio, p->charge_ratio);
    XTO_ST(beta0, p->beta0); XTO_ST(p0c, p->p0c);
    XTO_ST(ax, p->ax); XTO_ST(ay, p->ay);
    XTO_ST(state, p->state); XTO_ST(at_element, p->at_element);
    XTO_ST(at_turn, p->at_turn); XTO_ST(particle_id, p->particle_id);
    XTO_ST(gamma0, src->gamma0 ? src->gamma0[isrc] : 0.);
    XTO_ST(weight, src->weight ? src->weight[isrc] : 0.);
    XTO_ST(pdg_id, src->pdg_id ? src->pdg_id[isrc] : 0);
    XTO_ST(parent_particle_id, src->parent_particle_id ? src->parent_particle_id[isrc] : 0);
#undef XTO_ST
}

/* particles_monitor.h:12-77 */
static void xto_monitor(const xtg_monitor* m, const xto_part* p,
                        const xtg_particles* src, int64_t isrc) {
    int64_t at_turn;
    if (m->ebe_mode) {
        at_turn = p->at_element;
    } else {
        if (flag_set(p, XTG_FLAG_BACKTRACK)) return;
        at_turn = p->at_turn;
    }
    int64_t const n_turns_record = m->stop_at_turn - m->start_at_turn;
    if (m->n_repetitions == 1) {
        if (at_turn >= m->start_at_turn && at_turn < m->stop_at_turn) {
            int64_t const pid = p->particle_id;
            if (pid < m->part_id_end && pid >= m->part_id_start) {
                int64_t const store_at = n_turns_record * (pid - m->part_id_start)
                                         + at_turn - m->start_at_turn;
                xto_monitor_store(p, src, isrc, &m->data, store_at);
            }
        }
    } else if (m->n_repetitions > 1) {
        if (at_turn < m->start_at_turn) return;
        int64_t const i_frame = (at_turn - m->start_at_turn) / m->repetition_period;
        if (i_frame < m->n_repetitions
            && at_turn >= m->start_at_turn + i_frame * m->repetition_period
            && at_turn < m->stop_at_turn + i_frame * m->repetition_period) {
            int64_t const pid = p->particle_id;
            if (pid < m->part_id_end && pid >= m->part_id_start) {
                int64_t const store_at =
                    n_turns_record * (m->part_id_end - m->part_id_start) * i_frame
                    + n_turns_record * (pid - m->part_id_start)
                    + (at_turn - i_frame * m->repetition_period) - m->start_at_turn;
                xto_monitor_store(p, src, isrc, &m->data, store_at);
            }
        }
    }
}

/* multi_element_monitor.h:10-65 (set for the next calls by
 * xto_set_multi_element_monitor) */
static xtg_multi_element_monitor xto_mem;
static int xto_mem_on = 0;

static void xto_multi_element_monitor(const xto_part* p) {
    const xtg_multi_element_monitor* E = &xto_mem;
    int64_t const at_turn = p->at_turn;
    int64_t const particle_id = p->particle_id;
    if ((at_turn >= E->start_at_turn && at_turn < E->stop_at_turn) &&
        (particle_id >= E->part_id_start && particle_id < E->part_id_end)) {
        int64_t const at_element = p->at_element;
        int64_t store_at = -1;
        if (at_element < E->mapping_len) store_at = E->at_element_mapping[at_element];
        if (store_at >= 0) {
            int64_t const turn_index = at_turn - E->start_at_turn;
            int64_t const particle_index = particle_id - E->part_id_start;
            int64_t const n_part = E->part_id_end - E->part_id_start;
            double const v[7] = {p->x, p->px, p->y, p->py, p->zeta, p->delta, p->s};
            for (int c = 0; c < 7; c++)
                E->data[((turn_index * n_part + particle_index) * 7 + c) * E->n_obs + store_at] = v[c];
        }
    }
}

int32_t xto_set_multi_element_monitor(const xtg_multi_element_monitor* m) {
    if (m) {
        xto_mem = *m;
        xto_mem_on = 1;
    } else {
        xto_mem_on = 0;
    }
    return XTG_OK;
}

/* ---------------------------------------------------------------------- */
/* track_line, per-particle semantics: tracker.py:594-736                  */
/* ---------------------------------------------------------------------- */
typedef struct {
    const xtg_element* els;
    const xtg_config* cfg;
    const xtg_particles* P;
    int32_t num_turns, ele_start, num_ele_track;
    int32_t flag_end_turn_actions, flag_reset_s, flag_monitor, num_ele_line;
    double line_length;
    const xtg_monitor* mon;
    uint64_t flags;
} xto_args;

static void xto_track_one(const xto_args* a, int64_t i) {
    xto_part p;
    xto_load(a->P, i, a->flags, a->line_length, &p);
    int const backtrack = flag_set(&p, XTG_FLAG_BACKTRACK);
    int64_t isactive = p.state > 0;
    for (int64_t iturn = 0; iturn < a->num_turns; iturn++) {
        if (!isactive) break;
        int64_t const ele_stop = (int64_t)a->ele_start + a->num_ele_track;
        int64_t elem_idx, increm;
        if (backtrack) {
            elem_idx = ele_stop - 1;
            increm = -1;
            if (a->flag_end_turn_actions > 0) {
                /* local_particle_custom_api.h:79-94 */
                p.at_turn += -1;
                p.at_element = a->num_ele_line;
                if (a->flag_reset_s > 0) p.s = a->line_length;
            }
        } else {
            if (a->flag_monitor == 1) xto_monitor(a->mon, &p, a->P, i);
            elem_idx = a->ele_start;
            increm = 1;
        }
        for (; (elem_idx >= a->ele_start) && (elem_idx < ele_stop); elem_idx += increm) {
            if (a->flag_monitor == 2) xto_monitor(a->mon, &p, a->P, i);
            if (xto_mem_on) xto_multi_element_monitor(&p);
            if (xto_apply(&a->els[elem_idx], a->cfg, &p, a->P, i)) xto_global_aperture(a->cfg, &p);
            isactive = p.state > 0;
            if (!isactive) break;
            p.at_element += backtrack ? -1 : 1;
        }
        if (a->flag_monitor == 2) xto_monitor(a->mon, &p, a->P, i);
        if (backtrack) {
            if (a->flag_monitor == 1) xto_monitor(a->mon, &p, a->P, i);
        } else if (a->flag_end_turn_actions > 0) {
            if (isactive) {
                /* local_particle_custom_api.h:67-76 */
                p.at_turn += 1;
                p.at_element = 0;
                if (a->flag_reset_s > 0) p.s = 0.;
            }
        }
    }
    xto_store(&p, a->P, i);
}

/* ---------------------------------------------------------------------- */
/* track_line, CPU OpenMP semantics: tracker.py:566-598, 741-748           */
/* ---------------------------------------------------------------------- */

/* LocalParticle_exchange (particles.py:260-280): swaps every per-particle
 * field of two slots. */
static void xto_exchange(const xtg_particles* P, int64_t a, int64_t b) {
#define XTO_SWD(f) if (P->f) { double t = P->f[a]; P->f[a] = P->f[b]; P->f[b] = t; }
#define XTO_SWI(f) if (P->f) { int64_t t = P->f[a]; P->f[a] = P->f[b]; P->f[b] = t; }
    XTO_SWD(p0c) XTO_SWD(gamma0) XTO_SWD(beta0) XTO_SWD(s) XTO_SWD(zeta)
    XTO_SWD(x) XTO_SWD(y) XTO_SWD(px) XTO_SWD(py) XTO_SWD(ptau) XTO_SWD(delta)
    XTO_SWD(rpp) XTO_SWD(rvv) XTO_SWD(chi) XTO_SWD(charge_ratio) XTO_SWD(weight)
    XTO_SWD(ax) XTO_SWD(ay)
    XTO_SWI(pdg_id) XTO_SWI(particle_id) XTO_SWI(at_element) XTO_SWI(at_turn)
    XTO_SWI(state) XTO_SWI(parent_particle_id)
#undef XTO_SWD
#undef XTO_SWI
}

/* local_particle_custom_api.h:133-164 (two-pointer swap compaction) */
static int64_t xto_check_is_active_range(const xtg_particles* P, int64_t ipart, int64_t endpart) {
    int64_t left = ipart;
    int64_t right = endpart - 1;
    int64_t swap_made = 0;
    int64_t has_alive = 0;
    if (endpart <= ipart) return 0;
    if (left == right) return P->state[left] > 0;
    while (left < right) {
        if (P->state[left] > 0) {
            left++;
            has_alive = 1;
        } else if (P->state[right] <= 0) {
            right--;
        } else {
            xto_exchange(P, left, right);
            left++;
            right--;
            swap_made = 1;
        }
    }
    return swap_made || has_alive;
}

/* local_particle_custom_api.h:167-183 */
static int64_t xto_count_active(const xtg_particles* P, int64_t n) {
    int64_t num_active = 0;
    for (int64_t i = 0; i < n; i++) {
        if (P->state[i] <= -999999999) break;
        else if (P->state[i] > 0) num_active++;
    }
    return num_active;
}

static void xto_track_chunk_openmp(const xto_args* a, int64_t ipart, int64_t endpart) {
    const xtg_particles* P = a->P;
    int const backtrack = (int)((a->flags >> XTG_FLAG_BACKTRACK) & 1u);
    int64_t isactive = xto_check_is_active_range(P, ipart, endpart);
    xto_part p;
    for (int64_t iturn = 0; iturn < a->num_turns; iturn++) {
        if (!isactive) break;
        int64_t const ele_stop = (int64_t)a->ele_start + a->num_ele_track;
        int64_t elem_idx, increm;
        if (backtrack) {
            elem_idx = ele_stop - 1;
            increm = -1;
            if (a->flag_end_turn_actions > 0) {
                for (int64_t i = ipart; i < endpart; i++) {
                    if (P->state[i] <= 0) continue;
                    P->at_turn[i] += -1;
                    P->at_element[i] = a->num_ele_line;
                    if (a->flag_reset_s > 0) P->s[i] = a->line_length;
                }
            }
        } else {
            if (a->flag_monitor == 1) {
                for (int64_t i = ipart; i < endpart; i++) {
                    if (P->state[i] <= 0) continue;
                    xto_load(P, i, a->flags, a->line_length, &p);
                    xto_monitor(a->mon, &p, P, i);
                }
            }
            elem_idx = a->ele_start;
            increm = 1;
        }
        for (; (elem_idx >= a->ele_start) && (elem_idx < ele_stop); elem_idx += increm) {
            const xtg_element* e = &a->els[elem_idx];
            for (int64_t i = ipart; i < endpart; i++) {
                if (P->state[i] <= 0) continue;
                xto_load(P, i, a->flags, a->line_length, &p);
                if (a->flag_monitor == 2) xto_monitor(a->mon, &p, P, i);
                if (xto_mem_on) xto_multi_element_monitor(&p);
                if (xto_apply(e, a->cfg, &p, P, i)) xto_global_aperture(a->cfg, &p);
                xto_store(&p, P, i);
            }
            isactive = xto_check_is_active_range(P, ipart, endpart);
            if (!isactive) break;
            for (int64_t i = ipart; i < endpart; i++) {
                if (P->state[i] > 0) P->at_element[i] += backtrack ? -1 : 1;
            }
        }
        if (a->flag_monitor == 2 || (backtrack && a->flag_monitor == 1)) {
            for (int64_t i = ipart; i < endpart; i++) {
                if (P->state[i] <= 0) continue;
                xto_load(P, i, a->flags, a->line_length, &p);
                xto_monitor(a->mon, &p, P, i);
            }
        }
        if (!backtrack && a->flag_end_turn_actions > 0 && isactive) {
            for (int64_t i = ipart; i < endpart; i++) {
                if (P->state[i] <= 0) continue;
                P->at_turn[i] += 1;
                P->at_element[i] = 0;
                if (a->flag_reset_s > 0) P->s[i] = 0.;
            }
        }
    }
}

/* sizeof of the C-ABI structs as this compiler lays them out, for the
 * layout test of the ctypes mirror: element, particles, monitor, config. */
int32_t xto_abi_sizes(int64_t* out) {
    out[0] = (int64_t)sizeof(xtg_element);
    out[1] = (int64_t)sizeof(xtg_particles);
    out[2] = (int64_t)sizeof(xtg_monitor);
    out[3] = (int64_t)sizeof(xtg_config);
    out[4] = (int64_t)offsetof(xtg_element, knl);
    out[5] = (int64_t)offsetof(xtg_element, shift_x);
    out[6] = (int64_t)offsetof(xtg_monitor, data);
    out[7] = (int64_t)sizeof(xtg_element_monitor);
    out[8] = (int64_t)offsetof(xtg_element_monitor, particles);
    out[9] = (int64_t)offsetof(xtg_element, aux);
    out[10] = (int64_t)offsetof(xtg_element, r21);
    out[11] = (int64_t)offsetof(xtg_element, side);
    return 4;
}

int32_t xto_max_threads(void) {
#ifdef _OPENMP
    return (int32_t)omp_get_max_threads();
#else
    return 1;
#endif
}

int32_t xto_track(const xtg_element* els, int64_t n_elements, const xtg_config* cfg,
                  xtg_particles* P, int32_t num_turns, int32_t ele_start,
                  int32_t num_ele_track, int32_t flag_end_turn_actions,
                  int32_t flag_reset_s_at_end_turn, int32_t flag_monitor,
                  int32_t num_ele_line, double line_length, const xtg_monitor* mon,
                  uint64_t track_flags, int32_t mode, int32_t num_threads) {
    if (!els && n_elements > 0) return XTG_E_NULL;
    if (!cfg || !P) return XTG_E_NULL;
    if (!P->x || !P->px || !P->y || !P->py || !P->zeta || !P->delta || !P->ptau
        || !P->rpp || !P->rvv || !P->s || !P->chi || !P->charge_ratio || !P->beta0
        || !P->p0c || !P->state || !P->at_element || !P->at_turn || !P->particle_id)
        return XTG_E_NULL;
    if (ele_start < 0 || num_ele_track < 0 || (int64_t)ele_start + num_ele_track > n_elements)
        return XTG_E_VALUE;
    if (flag_monitor != 0 && !mon) return XTG_E_NULL;
    if (xto_validate(els, n_elements, NULL, 0) != XTG_OK) return XTG_E_UNSUPPORTED;

    xto_args a;
    a.els = els; a.cfg = cfg; a.P = P;
    a.num_turns = num_turns; a.ele_start = ele_start; a.num_ele_track = num_ele_track;
    a.flag_end_turn_actions = flag_end_turn_actions;
    a.flag_reset_s = flag_reset_s_at_end_turn;
    a.flag_monitor = flag_monitor; a.num_ele_line = num_ele_line;
    a.line_length = line_length; a.mon = mon; a.flags = track_flags;

    int nth = num_threads > 0 ? num_threads : xto_max_threads();
    int64_t const capacity = P->capacity;

    if (mode == XTO_MODE_PER_PARTICLE) {
        /* chunks of 64 particles, or single particles when that would leave
           threads idle */
        int const dyn = capacity >= (int64_t)64 * 4 * nth ? 64 : 1;
        (void)dyn;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, dyn) num_threads(nth)
#endif
        for (int64_t i = 0; i < capacity; i++) xto_track_one(&a, i);
        return XTG_OK;
    }

    /* OpenMP semantics: reorganize, chunk, track, reorganize. */
    xto_check_is_active_range(P, 0, capacity);
    int64_t const n_track = xto_count_active(P, capacity);
    int64_t const chunk_size = (n_track + nth - 1) / nth;
#ifdef _OPENMP
#pragma omp parallel for schedule(static, 1) num_threads(nth)
#endif
    for (int chunk = 0; chunk < nth; chunk++) {
        int64_t const ipart = (int64_t)chunk * chunk_size;
        int64_t endpart = (int64_t)(chunk + 1) * chunk_size;
        if (endpart > n_track) endpart = n_track;
        if (ipart < endpart) xto_track_chunk_openmp(&a, ipart, endpart);
    }
    xto_check_is_active_range(P, 0, capacity);
    return XTG_OK;
}
