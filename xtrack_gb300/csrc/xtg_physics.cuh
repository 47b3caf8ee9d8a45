// Device-side element physics of the push, one particle per thread.
//
// Two arithmetic modes share this file (template parameter kExact):
//   kExact = true : the reference's operation order. The translation unit is
//                   compiled with -fmad=false so no product is fused into an
//                   addition; with the per-element constants precomputed by
//                   the host packer in the same order, results equal the
//                   reference's CPU results bit for bit (libm aside).
//   kExact = false: the minimal formulation — one merged complex Horner
//                   polynomial per kick and explicit fma() — for throughput.
// Citations are to xtrack/beam_elements/elements_src/ unless noted.
#pragma once
#include <stdint.h>

#include "xtg_f64emu.cuh"
#include "xtg_table.h"

namespace xtg {

#ifndef XTG_DEV
#define XTG_DEV __device__ __forceinline__
#endif
// Element maps that the common lattices do not use per kick are kept out of
// line so that they cost no registers in the hot loop.
#ifndef XTG_COLD
#define XTG_COLD __device__ __noinline__
#endif

// Products that are not fused into an addition (every product of the
// exact arithmetic; the stand-alone ones of the fast arithmetic) run on the
// integer pipes (emul, xtg_f64emu.cuh: bit-identical to the FP64 unit's)
// unless this is 0. Either way the results are the same bits.
#ifndef XTG_EMUL
#define XTG_EMUL 1
#endif

// A stand-alone product: rounded as the FP64 multiply rounds it.
// XSplit is an operand prepared once for several products (emu_split).
#if XTG_EMUL
typedef F64Split XSplit;
XTG_DEV XSplit xsplit(double v) { return emu_split(v); }
XTG_DEV double xmul(double a, double b) { return emul(a, b); }
XTG_DEV double xmul(const XSplit& a, const XSplit& b) { return emul_split(a, b); }
XTG_DEV double xmul(double a, const XSplit& b) { return emul_split(emu_split(a), b); }
#else
struct XSplit {
    double v;
};
XTG_DEV XSplit xsplit(double v) { return XSplit{v}; }
XTG_DEV double xmul(double a, double b) { return a * b; }
XTG_DEV double xmul(const XSplit& a, const XSplit& b) { return a.v * b.v; }
XTG_DEV double xmul(double a, const XSplit& b) { return a * b.v; }
#endif

// +0.0 + v, as the reference forms a sum that starts from zero: v itself,
// except that -0 becomes +0. Integer operations, off the FP64 pipe.
XTG_DEV double plus_zero(double v) {
    uint64_t const b = emu_bits(v);
    return emu_double(b == 0x8000000000000000ull ? 0ull : b);
}

constexpr double kCLightD = 299792458.0;
constexpr double kPiD = 3.1415926535897932384626433832795028841971693993751;

// Register-resident state of one particle (the LocalParticle of the
// reference, particles.py:96-112, restricted to what the push changes or
// reads). rv0v = 1/rvv and opd = 1 + delta are cached: the reference
// recomputes them in every drift and kick with the same IEEE operations, so
// caching them does not change any result.
struct PState {
    double x, px, y, py, zeta, delta, ptau, rpp, rvv, s;
    double rv0v, opd;
    double chi, charge_ratio, beta0, p0c;
    double ax, ay;
    int64_t state, at_element, at_turn;
    bool chi_one;     // chi == 1: per-element products precomputed at chi = 1 apply
    bool frozen;      // longitudinal coordinates frozen (zeta, ptau, delta, rpp, rvv)
};

XTG_DEV void refresh_energy_cache(PState& p) {
    p.rv0v = 1. / p.rvv;
    p.opd = 1. + p.delta;
}

// The reference's generated setters, adders and scalers of a frozen
// variable are no-ops (particles.py:185-225, FREEZE_VAR_<name>); with the
// longitudinal coordinates frozen, every write to zeta and to the energy
// variables leaves the old value, and later reads in the same element see
// it.
XTG_DEV void set_zeta(PState& p, double v) {
    if (!p.frozen) p.zeta = v;
}
XTG_DEV void set_energy(PState& p, double delta, double rvv, double rpp, double ptau) {
    if (!p.frozen) {
        p.delta = delta;
        p.rvv = rvv;
        p.rpp = rpp;
        p.ptau = ptau;
    }
}

// ---------------------------------------------------------------------------
// Drifts
// ---------------------------------------------------------------------------

// track_drift.h:10-23
template <bool kExact>
XTG_DEV void drift_expanded(PState& p, double length) {
    if (kExact) {
        // 1 + (xp^2 + yp^2) * 0.5 as one fused step: the product with 0.5 is
        // exact, so a single rounding of the sum is the reference's result
        double const xp = xmul(p.px, p.rpp);
        double const yp = xmul(p.py, p.rpp);
        double const dzeta = 1 - xmul(p.rv0v, fma(xmul(xp, xp) + xmul(yp, yp), 0.5, 1.));
        p.x = p.x + xmul(xp, length);
        p.y = p.y + xmul(yp, length);
        p.s = p.s + length;
        set_zeta(p, p.zeta + xmul(length, dzeta));
    } else {
        // the reference's grouping, contracted as its FMA build contracts
        // it: 1 + (xp^2 + yp^2)/2 is rounded before the product with 1/rvv
        // (regrouping it changes zeta by ~1e-12 m per turn on a 6000-drift
        // ring, far outside the reference's own FMA/no-FMA spread)
        double const xp = xmul(p.px, p.rpp);
        double const yp = xmul(p.py, p.rpp);
        double const t = fma(xp, xp, xmul(yp, yp));
        double const dzeta = fma(-p.rv0v, fma(t, 0.5, 1.0), 1.0);
        p.x = fma(xp, length, p.x);
        p.y = fma(yp, length, p.y);
        set_zeta(p, fma(length, dzeta, p.zeta));
        p.s = p.s + length;
    }
}

// Two consecutive expanded drifts of the same length in the exact
// arithmetic (the adjacent half drifts of a uniform magnet body): nothing
// between them changes px, py or the energy, so the slopes, the zeta slip
// and the three increments are those of the first, and only the four sums
// are formed twice, in order. Bit-identical to two drift_expanded<true>.
XTG_DEV void drift_expanded_twice_exact(PState& p, double length) {
    double const xp = xmul(p.px, p.rpp);
    double const yp = xmul(p.py, p.rpp);
    double const dzeta = 1 - xmul(p.rv0v, fma(xmul(xp, xp) + xmul(yp, yp), 0.5, 1.));
    double const dx = xmul(xp, length), dy = xmul(yp, length), dz = xmul(length, dzeta);
    p.x = (p.x + dx) + dx;
    p.y = (p.y + dy) + dy;
    p.s = (p.s + length) + length;
    set_zeta(p, p.zeta + dz);
    set_zeta(p, p.zeta + dz);
}

// track_drift.h:26-42
template <bool kExact>
XTG_DEV void drift_exact(PState& p, double length) {
    double const px = p.px, py = p.py;
    double const opd = p.opd;
    if (kExact) {
        double const one_over_pz = 1. / sqrt(opd * opd - px * px - py * py);
        double const dzeta = 1 - p.rv0v * opd * one_over_pz;
        p.x = p.x + px * one_over_pz * length;
        p.y = p.y + py * one_over_pz * length;
        set_zeta(p, p.zeta + dzeta * length);
        p.s = p.s + length;
    } else {
        double const pz2 = fma(-py, py, fma(-px, px, xmul(opd, opd)));
        double const one_over_pz = 1. / sqrt(pz2);
        double const dzeta = fma(-xmul(p.rv0v, opd), one_over_pz, 1.0);
        double const fl = xmul(one_over_pz, length);
        p.x = fma(px, fl, p.x);
        p.y = fma(py, fl, p.y);
        set_zeta(p, fma(dzeta, length, p.zeta));
        p.s = p.s + length;
    }
}

// track_magnet_drift.h:44-87
XTG_DEV void drift_polar(PState& p, double length, double h) {
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    double const s = length;
    double const opd = p.delta + 1.0;
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
    p.x = new_x;
    p.px = new_px;
    p.y = new_y;
    set_zeta(p, p.zeta + (length - delta_ell / p.rvv));
    p.s = p.s + s;
}

// track_magnet_drift.h:90-213
XTG_DEV void drift_cf_expanded(PState& p, double length, double k0_, double k1_, double h) {
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    double const dp1 = p.delta + 1;
    double const chi = p.chi;
    double const k0 = chi * k0_ / dp1;
    double const k1 = chi * k1_ / dp1;
    double const Kx = k0 * h + k1;
    double const Ky = -k1;
    double Sx, Sy, Cx, Cy;
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
    double x_ = x * Cx + xp * Sx;
    double const y_ = y * Cy + yp * Sy;
    double const px_ = (A * Sx + B * Cx) * dp1;
    double const py_ = (C * Sy + D * Cy) * dp1;
    if (Kx != 0.0) x_ = x_ + (k0 - h) * (Cx - 1.0) / Kx;
    else x_ = x_ - (k0 - h) * 0.5 * ((length) * (length));
    double length_ = length;
    if (Kx != 0.0) {
        length_ -= (h * ((Cx - 1.0) * xp + Sx * A + length * (k0 - h))) / Kx;
        length_ += 0.5 * (-(((A) * (A)) * Cx * Sx) / (2.0 * Kx) + (((B) * (B)) * Cx * Sx) / 2.0 +
                          (((A) * (A)) * length) / (2.0 * Kx) + (((B) * (B)) * length) / 2.0 -
                          (A * B * ((Cx) * (Cx))) / Kx + (A * B) / Kx);
    } else {
        length_ += h * length * (3.0 * length * xp + 6.0 * x - (k0 - h) * ((length) * (length))) / 6.0;
        length_ += 0.5 * (((B) * (B))) * length;
    }
    if (Ky != 0.0) {
        length_ += 0.5 * (-(((C) * (C)) * Cy * Sy) / (2.0 * Ky) + (((D) * (D)) * Cy * Sy) / 2.0 +
                          (((C) * (C)) * length) / (2.0 * Ky) + (((D) * (D)) * length) / 2.0 -
                          (C * D * ((Cy) * (Cy))) / Ky + (C * D) / Ky);
    } else {
        length_ += 0.5 * ((D) * (D)) * length;
    }
    double const dzeta = length - length_ / p.rvv;
    p.x = x_;
    p.px = px_;
    p.y = y_;
    p.py = py_;
    set_zeta(p, p.zeta + dzeta);
    p.s = p.s + length;
}

// track_magnet_drift.h:348-393
XTG_DEV void drift_straight_exact_bend(PState& p, double length, double k0) {
    double const k0_chi = k0 * p.chi;
    if (fabs(k0_chi) < 1e-8) {
        drift_exact<true>(p, length);
        return;
    }
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    double const s = length;
    double const opd = p.delta + 1.0;
    double const A = 1.0 / sqrt((opd) * (opd) - (py) * (py));
    double const pz = sqrt((opd) * (opd) - (px) * (px) - (py) * (py));
    double const new_px = px - k0_chi * s;
    double const new_x = x + (sqrt((opd) * (opd) - (new_px) * (new_px) - (py) * (py)) - pz) / k0_chi;
    double const D = asin(A * px) - asin(A * new_px);
    double const new_y = y + (py / k0_chi) * D;
    double const delta_ell = (opd / k0_chi) * D;
    p.x = new_x;
    p.px = new_px;
    p.y = new_y;
    set_zeta(p, p.zeta + (length - delta_ell / p.rvv));
    p.s = p.s + s;
}

// track_magnet_drift.h:271-345
XTG_DEV void drift_curved_exact_bend(PState& p, double length, double k0, double h) {
    double const k0_chi = k0 * p.chi;
    if (fabs(k0_chi) < 1e-8) {
        drift_polar(p, length, h);
        return;
    }
    double const x0 = p.x, y0 = p.y, px0 = p.px, py = p.py;
    double const s = length;
    double const opd = p.delta + 1.0;
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
    p.x = p.x + delta_x;
    p.px = pxs;
    p.y = new_y;
    set_zeta(p, p.zeta + (length - delta_ell / p.rvv));
    p.s = p.s + s;
}

XTG_COLD PState magnet_drift_curved(PState p, double length, int drift_model, double k0, double k1,
                                    double h);

// track_magnet_drift.h:469-555 (model 6, solenoid, is rejected on the host)
template <bool kExact>
XTG_DEV void magnet_drift(PState& p, double length, int drift_model, double k0, double k1,
                          double h) {
    if (drift_model == -1) return;
    if (length == 0.0) return;
    if (drift_model == 0) {
        drift_expanded<kExact>(p, length);
        return;
    }
    if (drift_model == 1) {
        drift_exact<kExact>(p, length);
        return;
    }
    p = magnet_drift_curved(p, length, drift_model, k0, k1, h);
}

// Drift models 2-8 of track_magnet_drift.h:469-555. Out of line and by
// value, so that the caller's particle state stays in registers.
XTG_COLD PState magnet_drift_curved(PState p, double length, int drift_model, double k0, double k1,
                                    double h) {
    switch (drift_model) {
    case 2: drift_polar(p, length, h); break;
    case 3: drift_cf_expanded(p, length, k0, k1, h); break;
    case 4: drift_curved_exact_bend(p, length, k0, h); break;
    case 5: drift_straight_exact_bend(p, length, k0); break;
    case 7:
        drift_polar(p, 0.6756035959798289 * length, h);
        p.px = p.px - 1.3512071919596578 * k0 * p.chi * length;
        drift_polar(p, -0.17560359597982889 * length, h);
        p.px = p.px - (-1.7024143839193155) * k0 * p.chi * length;
        drift_polar(p, -0.17560359597982889 * length, h);
        p.px = p.px - 1.3512071919596578 * k0 * p.chi * length;
        drift_polar(p, 0.6756035959798289 * length, h);
        break;
    case 8:
        drift_polar(p, 3.922568052387799819591407413100e-01 * length, h);
        p.px = p.px - 7.845136104775599639182814826199e-01 * k0 * p.chi * length;
        drift_polar(p, 5.100434119184584780271052295575e-01 * length, h);
        p.px = p.px - 2.355732133593569921359289764951e-01 * k0 * p.chi * length;
        drift_polar(p, -4.710533854097565531482416645304e-01 * length, h);
        p.px = p.px - (-1.177679984178870098432412305556e+00) * k0 * p.chi * length;
        drift_polar(p, 6.875316825251809316199569366290e-02 * length, h);
        p.px = p.px - 1.315186320683906284756403692882e+00 * k0 * p.chi * length;
        drift_polar(p, 6.875316825251809316199569366290e-02 * length, h);
        p.px = p.px - (-1.177679984178870098432412305556e+00) * k0 * p.chi * length;
        drift_polar(p, -4.710533854097565531482416645304e-01 * length, h);
        p.px = p.px - 2.355732133593569921359289764951e-01 * k0 * p.chi * length;
        drift_polar(p, 5.100434119184584780271052295575e-01 * length, h);
        p.px = p.px - 7.845136104775599639182814826199e-01 * k0 * p.chi * length;
        drift_polar(p, 3.922568052387799819591407413100e-01 * length, h);
        break;
    default: break;
    }
    return p;
}

// ---------------------------------------------------------------------------
// Kicks
// ---------------------------------------------------------------------------

// One kick_simple pass in the reference arithmetic (track_magnet_kick.h:
// 182-260). `co` holds quintuples (A, B, knl, ksl, invf) from `top` down.
// At chi = 1, chi*knl*factor*invf equals the precomputed A (and B).
XTG_DEV void exact_pass_chi1(PState& p, const double* __restrict__ co, int top,
                             double kick_weight, const XSplit& x, const XSplit& y) {
    double dpx_mul = co[0];
    double dpy_mul = co[1];
    for (int i = top; i > 0; i--) {
        co += 5;
        XSplit const a = xsplit(dpx_mul), b = xsplit(dpy_mul);
        double const zre = xmul(a, x) - xmul(b, y);
        double const zim = xmul(a, y) + xmul(b, x);
        dpx_mul = co[0] + zre;
        dpy_mul = co[1] + zim;
    }
    dpx_mul = -dpx_mul;
    p.px = p.px + xmul(kick_weight, dpx_mul);
    p.py = p.py + xmul(kick_weight, dpy_mul);
}

XTG_DEV void exact_pass(PState& p, const double* __restrict__ co, int top, double factor,
                        double kick_weight, double x, double y) {
    double const chi = p.chi;
    double dpx_mul = chi * co[2] * factor * co[4];
    double dpy_mul = chi * co[3] * factor * co[4];
    for (int i = top; i > 0; i--) {
        co += 5;
        double const zre = dpx_mul * x - dpy_mul * y;
        double const zim = dpx_mul * y + dpy_mul * x;
        double const this_knl = chi * co[2] * factor;
        double const this_ksl = chi * co[3] * factor;
        dpx_mul = this_knl * co[4] + zre;
        dpy_mul = this_ksl * co[4] + zim;
    }
    dpx_mul = -dpx_mul;
    p.px = p.px + kick_weight * dpx_mul;
    p.py = p.py + kick_weight * dpy_mul;
}

// The parameters of one kick, read from a MagnetRec (kick-weight slot k) or
// from a compact KickRec.
struct KickArgs {
    const ExactPass* pass;
    int fast_top, fast_coef, curv;
    double kw, hl, C0, C1, htot, Q0, Q1, fscale;
};

XTG_DEV KickArgs kick_args(const MagnetRec& r, int k) {
    KickArgs a;
    a.pass = r.pass;
    a.fast_top = r.fast_top;
    a.fast_coef = r.fast_coef;
    a.curv = r.curv_terms;
    a.kw = r.kw[k];
    a.hl = r.hl[k];
    a.C0 = r.C0[k];
    a.C1 = r.C1[k];
    a.htot = r.htot;
    a.Q0 = r.Q0;
    a.Q1 = r.Q1;
    a.fscale = r.fast_scale[k];
    return a;
}

XTG_DEV KickArgs kick_args(const KickRec& r) {
    KickArgs a;
    a.pass = r.pass;
    a.fast_top = r.fast_top;
    a.fast_coef = r.fast_coef;
    a.curv = r.curv_terms;
    a.kw = r.kw;
    a.hl = r.hl;
    a.C0 = r.C0;
    a.C1 = r.C1;
    a.htot = r.htot;
    a.Q0 = r.Q0;
    a.Q1 = r.Q1;
    a.fscale = 1.0;
    return a;
}

// track_magnet_kick.h:23-144.
template <bool kExact>
XTG_DEV void apply_kick(PState& p, const KickArgs& a, const double* __restrict__ coefs) {
    double const x = p.x, y = p.y;
    if (kExact) {
        double const kw = a.kw;
        XSplit const sx = xsplit(x), sy = xsplit(y);
#pragma unroll 1
        for (int q = 0; q < 3; q++) {
            int const top = a.pass[q].top;
            if (top >= 0) {
                if (p.chi_one) exact_pass_chi1(p, coefs + a.pass[q].coef, top, kw, sx, sy);
                else exact_pass(p, coefs + a.pass[q].coef, top, a.pass[q].factor, kw, x, y);
            }
        }
        int const curv = a.curv;
        if (curv) {
            // track_magnet_kick.h:97-142: dpx, dpy and dzeta start from 0;
            // the first term of each is 0 + v (plus_zero), later ones sum
            double dpx = 0.0, dpy = 0.0, dzeta = 0.0;
            double const chi = p.chi;
            double C0, C1;
            if (p.chi_one) {
                C0 = a.C0;
                C1 = a.C1;
            } else {
                C0 = -chi * a.Q0 * kw * a.htot;
                C1 = a.htot * chi * a.Q1 * kw;
            }
            if (curv & 1) {
                double const hl = a.hl;
                dpx = plus_zero(xmul(hl, p.opd));
                dzeta = plus_zero(xmul(xmul(-p.rv0v, hl), sx));
            }
            if (curv & 2) {
                double const t = xmul(C0, sx);
                dpx = (curv & 1) ? dpx + t : plus_zero(t);
            }
            if (curv & 4) {
                XSplit const nx = xsplit(-x);
                double const t = xmul(C1, xmul(nx, sx) + xmul(xmul(0.5, y), sy));
                dpx = (curv & 3) ? dpx + t : plus_zero(t);
                dpy = plus_zero(xmul(xmul(C1, sx), sy));
            }
            p.px = p.px + dpx;
            p.py = p.py + dpy;
            set_zeta(p, p.zeta + dzeta);
        }
    } else {
        // merged polynomial sum_i (cn_i + i cs_i) z^i, z = x + i y; the
        // (cn_i, cs_i) pairs are 16-byte aligned: one 128-bit load each
        double pr = 0.0, pi = 0.0;
        int const top = a.fast_top;
        if (top >= 0) {
            const double2* __restrict__ c = reinterpret_cast<const double2*>(coefs + a.fast_coef);
            double2 const c0 = c[0];
            pr = c0.x;
            pi = c0.y;
            for (int i = 1; i <= top; i++) {
                double2 const ci = c[i];
                double const nr = fma(pr, x, fma(-pi, y, ci.x));
                double const ni = fma(pr, y, fma(pi, x, ci.y));
                pr = nr;
                pi = ni;
            }
        }
        // every term is accumulated straight into px / py, in the
        // reference's order (multipoles, then curvature terms)
        double const cs = p.chi_one ? a.fscale : xmul(p.chi, a.fscale);
        p.px = fma(-cs, pr, p.px);
        p.py = fma(cs, pi, p.py);
        int const curv = a.curv;
        if (curv) {
            double const chi = p.chi;
            if (curv & 1) {
                double const hl = a.hl;
                p.px = fma(hl, p.opd, p.px);
                set_zeta(p, fma(xmul(-p.rv0v, hl), x, p.zeta));
            }
            if (curv & 2) p.px = fma(p.chi_one ? a.C0 : xmul(chi, a.C0), x, p.px);
            if (curv & 4) {
                double const c1 = p.chi_one ? a.C1 : xmul(chi, a.C1);
                p.px = fma(c1, fma(-x, x, xmul(xmul(0.5, y), y)), p.px);
                p.py = fma(xmul(c1, x), y, p.py);
            }
        }
    }
}

template <bool kExact>
XTG_DEV void magnet_kick(PState& p, const MagnetRec& r, const double* __restrict__ coefs, int k) {
    apply_kick<kExact>(p, kick_args(r, k), coefs);
}

// ---------------------------------------------------------------------------
// Nonlinear edges: the "full" (1) and "dipole-only" (2) edge models of
// track_magnet_edge.h:83-158. Cold code: two calls per magnet at most.
// The parameters of one edge are a FringeRec block of doubles in the
// record's coefficient area (layout: xtg_table.h, FR_*). The arithmetic
// follows the reference expression by expression (this path is shared by
// both arithmetic modes).
// ---------------------------------------------------------------------------

// local_particle_custom_api.h:20-33 (update_delta)
XTG_DEV void set_delta_and_energy(PState& p, double new_delta) {
    double const beta0 = p.beta0;
    double const delta_beta0 = new_delta * beta0;
    double const ptau_beta0 = sqrt(delta_beta0 * delta_beta0 + 2. * delta_beta0 * beta0 + 1.) - 1.;
    set_energy(p, new_delta, (1. + new_delta) / (1. + ptau_beta0), 1. / (1. + new_delta),
               ptau_beta0 / beta0);
}

// local_particle_custom_api.h:248-256
XTG_DEV void kill_particle(PState& p, int64_t kill_state) {
    p.x = 1e30;
    p.px = 1e30;
    p.y = 1e30;
    p.py = 1e30;
    set_zeta(p, 1e30);
    set_delta_and_energy(p, -1.);
    refresh_energy_cache(p);
    p.state = kill_state;
}

// track_yrotation.h:13-48 (spin off)
XTG_DEV void y_rotation(PState& p, double sin_a, double cos_a, double tan_a) {
    double const beta0 = p.beta0;
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    double const t = p.zeta / beta0;
    double const pt = (p.ptau / beta0) * beta0;
    double const pz = sqrt(1.0 + 2.0 * pt / beta0 + pt * pt - px * px - py * py);
    double const ptt = 1.0 + tan_a * px / pz;
    double const x_hat = x / (cos_a * ptt);
    double const px_hat = cos_a * px - sin_a * pz;
    double const y_hat = y - tan_a * x * py / (pz * ptt);
    double const t_hat = t + tan_a * x * (1.0 / beta0 + pt) / (pz * ptt);
    p.x = x_hat;
    p.px = px_hat;
    p.y = y_hat;
    set_zeta(p, t_hat * beta0);
}

// track_dipole_fringe.h:16-82 (MAD-NG form)
XTG_DEV void dipole_fringe(PState& p, double fint, double hgap, double k0) {
    if (fabs(k0) < 10e-10) return;
    double const beta0 = p.beta0;
    double const x = p.x, px = p.px, y = p.y, py = p.py;
    double const t = p.zeta / beta0;
    double const pt = p.ptau;
    double const delta = p.delta;
    double const fh = hgap * fint;
    double const fsad = (fh > 10e-10) ? 1. / (72 * fh) : 0;
    double const b0 = k0 * p.chi;
    double const inv_beta = 1. / beta0;
    double const dpp = (1. + delta) * (1. + delta);
    double const pz = sqrt(dpp - px * px - py * py);
    double const ipz = 1. / pz;
    double const relp = 1. / sqrt(dpp);
    double const tfac = -(inv_beta + pt);
    double const c2 = b0 * fh * 2;
    double const c3 = b0 * b0 * fsad * relp;
    double const xp = px / pz;
    double const yp = py / pz;
    double const xyp = xp * yp;
    double const yp2 = 1. + yp * yp;
    double const xp2 = xp * xp;
    double const iyp2 = 1. / yp2;
    double const fi0 = atan(xp * iyp2) - c2 * (1 + xp2 * (1 + yp2)) * ipz;
    double const cf = cos(fi0);
    double const co2 = b0 / (cf * cf);
    double const xq = xp * iyp2;
    double const co1 = co2 / (1 + xq * xq) * iyp2;
    double const co3 = co2 * c2;
    double const fi1 = co1 - co3 * 2 * xp * (1 + yp2) * ipz;
    double const fi2 = -2 * co1 * xyp * iyp2 - co3 * 2 * xp * xyp * ipz;
    double const fi3 = +co3 * (1 + xp2 * (1 + yp2)) * (ipz * ipz);
    double const kx = fi1 * (1 + xp2) * ipz + fi2 * xyp * ipz - fi3 * xp;
    double const ky = fi1 * xyp * ipz + fi2 * yp2 * ipz - fi3 * yp;
    double const ipz2 = ipz * ipz;
    double const kz = fi1 * tfac * xp * ipz2 + fi2 * tfac * yp * ipz2 - fi3 * tfac * ipz;
    double const new_y = 2 * y / (1 + sqrt(1 - 2 * ky * y));
    double const ny2 = new_y * new_y;
    double const new_x = x + 0.5 * kx * ny2;
    double const new_py = py - 4 * c3 * (ny2 * new_y) - b0 * tan(fi0) * new_y;
    double const new_t = t + 0.5 * kz * ny2 + c3 * (new_y * new_y * new_y * new_y) * (relp * relp) * tfac;
    p.x = new_x;
    p.y = new_y;
    p.py = new_py;
    set_zeta(p, new_t * beta0);
}

// track_mult_fringe.h:12-128 with k_order = 3, min_order = 1
XTG_DEV void mult_fringe(PState& p, const double* kn, const double* ks, const double* knl,
                         const double* ksl, int64_t kl_order, double length, bool is_exit,
                         bool backtrack) {
    if (backtrack) {
        kill_particle(p, -32);
        return;
    }
    int64_t const k_order = 3;
    double const beta0 = p.beta0;
    double const direction = is_exit ? -1 : 1;
    double const x = p.x, px = p.px, y = p.y, py = p.py;
    double const t = p.zeta / beta0;
    double const pt = p.ptau;
    double const rpp = p.rpp;
    double const chi = p.chi;
    double rx = 1, ix = 0;
    double fx = 0, fxx = 0, fxy = 0, fy = 0, fyx = 0, fyy = 0;
    int64_t const order = (k_order > kl_order) ? k_order : kl_order;
    double inv_factorial = 1;
    for (int64_t ii = 0; ii <= order; ii++) {
        if (ii > 1) inv_factorial /= ii;
        double const component = ii + 1;
        double const drx = rx, dix = ix;
        rx = drx * x - dix * y;
        ix = drx * y + dix * x;
        double kn_total = 0, ks_total = 0;
        if (ii >= 1) {
            if (ii <= k_order) {
                kn_total += kn[ii] * inv_factorial;
                ks_total += ks[ii] * inv_factorial;
            }
            if (ii <= kl_order && length != 0.) {
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
    p.x = p.x + -fx * rpp;
    p.y = p.y + -fy * rpp;
    p.px = new_px;
    p.py = new_py;
    set_zeta(p, (t + delta_t) * beta0);
}

// track_wedge.h:14-58 (spin off); the trigonometric values of theta come
// from the host
XTG_DEV void wedge(PState& p, double theta, double sin_t, double cos_t, double tan_t,
                   double sin_2t, double k0) {
    double const b1 = k0 * p.chi;
    if (fabs(b1) < 10e-10) {
        y_rotation(p, -sin_t, cos_t, -tan_t);
        return;
    }
    double const rvv = p.rvv;
    double const x = p.x, px = p.px, py = p.py;
    double const opd = p.delta + 1.0;
    double const A = 1.0 / sqrt(opd * opd - py * py);
    double const pz = sqrt(opd * opd - px * px - py * py);
    double const new_px = px * cos_t + (pz - b1 * x) * sin_t;
    double const new_pz = sqrt(opd * opd - new_px * new_px - py * py);
    double const new_x = x * cos_t +
                         (x * px * sin_2t + (sin_t * sin_t) * (2 * x * pz - b1 * (x * x))) /
                             (new_pz + pz * cos_t - px * sin_t);
    double const D = asin(A * px) - asin(A * new_px);
    double const delta_y = py * (theta + D) / b1;
    double const delta_ell = opd * (theta + D) / b1;
    p.x = new_x;
    p.y = p.y + delta_y;
    p.px = new_px;
    set_zeta(p, p.zeta + -delta_ell / rvv);
}

// track_wedge.h:60-82
XTG_DEV void quad_wedge(PState& p, double theta, double k1) {
    double const b2 = k1 * p.chi;
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    double const new_px = px - b2 * x * x * theta + b2 * y * y / 2 * theta;
    double const new_py = py + b2 * x * y * theta;
    p.px = new_px;
    p.py = new_py;
}

// track_magnet_edge.h:83-158 for one edge; the ax/ay reset of
// track_magnet_edge.h:51-61 is done by the caller. The backtracking
// variants kill the particle (state -32) as the reference does; the kill
// leaves the particle with the kill values (the reference goes on
// applying the map to them).
XTG_COLD PState fringe_edge(PState p, const double* __restrict__ fr, bool backtrack) {
    int const model = (int)fr[FR_MODEL];
    bool const is_exit = fr[FR_IS_EXIT] != 0.;
    if (backtrack) {
        kill_particle(p, -32);
        return p;
    }
    bool const rot = fr[FR_ROTATE] != 0.;
    double const theta = -fr[FR_FACE_ANGLE];
    const double* kn = fr + FR_KNORM;
    const double* ks = fr + FR_KSKEW;
    int64_t const kl_order = (int64_t)fr[FR_KL_ORDER];
    const double* knl = fr + FR_KNL;
    const double* ksl = knl + (kl_order + 1);
    if (!is_exit) {
        if (rot) y_rotation(p, -fr[FR_SIN], fr[FR_COS], -fr[FR_TAN]);
        dipole_fringe(p, fr[FR_FINT], fr[FR_HGAP], fr[FR_K0]);
        if (model == 1) mult_fringe(p, kn, ks, knl, ksl, kl_order, fr[FR_LENGTH], false, false);
        if (model == 1 && rot) quad_wedge(p, theta, kn[1]);
        if (rot) wedge(p, theta, fr[FR_WSIN], fr[FR_WCOS], fr[FR_WTAN], fr[FR_WSIN2], kn[0]);
    } else {
        if (rot) wedge(p, theta, fr[FR_WSIN], fr[FR_WCOS], fr[FR_WTAN], fr[FR_WSIN2], kn[0]);
        if (model == 1 && rot) quad_wedge(p, theta, kn[1]);
        if (model == 1) mult_fringe(p, kn, ks, knl, ksl, kl_order, fr[FR_LENGTH], true, false);
        dipole_fringe(p, fr[FR_FINT], fr[FR_HGAP], fr[FR_K0]);
        if (rot) y_rotation(p, -fr[FR_SIN], fr[FR_COS], -fr[FR_TAN]);
    }
    return p;
}

// track_dipole_edge_linear.h:29-37: px += chi*r21*x, py += chi*r43*y. The
// reference rounds chi*r21 first; at chi == 1 that product is r21 exactly
// and is skipped. The fast mode fuses the remaining product and sum.
template <bool kExact>
XTG_DEV void edge_linear_kick(PState& p, double r21, double r43) {
    double const x = p.x, y = p.y;
    double const c21 = p.chi_one ? r21 : xmul(p.chi, r21);
    double const c43 = p.chi_one ? r43 : xmul(p.chi, r43);
    if (kExact) {
        p.px = p.px + xmul(c21, x);
        p.py = p.py + xmul(c43, y);
    } else {
        p.px = fma(c21, x, p.px);
        p.py = fma(c43, y, p.py);
    }
}

// track_magnet_edge.h:16-80 with the linear model (track_dipole_edge_linear.h);
// the nonlinear models go to fringe_edge
template <bool kExact>
XTG_DEV void magnet_edge(PState& p, int kind, bool is_exit, double r21, double r43,
                         const double* __restrict__ fringe, bool backtrack) {
    if (kind == EDGE_NONE) return;
    if (kind == EDGE_FRINGE) {
        if (is_exit) {
            p.ax = 0.;
            p.ay = 0.;
        } else {
            p.ax = (-0.5 * 0.0) * (p.y - 0.);
            p.ay = (0.5 * 0.0) * (p.x - 0.);
        }
        p = fringe_edge(p, fringe, backtrack);
        return;
    }
    if (is_exit) {
        p.ax = 0.;
        p.ay = 0.;
    } else {
        p.ax = (-0.5 * 0.0) * (p.y - 0.);
        p.ay = (0.5 * 0.0) * (p.x - 0.);
    }
    if (kind == EDGE_LINEAR) edge_linear_kick<kExact>(p, r21, r43);
}

// One drift step of a magnet body: `reps` (1 or 2) consecutive drifts of
// the same length. Consecutive expanded drifts in the exact arithmetic
// share their work (drift_expanded_twice_exact); other models run twice.
template <bool kExact>
XTG_DEV void body_drift(PState& p, double len, int reps, int dm, double k0d, double k1d, double hd) {
    if (kExact && dm == 0 && len != 0.0) {
        if (reps == 2) drift_expanded_twice_exact(p, len);
        else drift_expanded<true>(p, len);
        return;
    }
    for (int q = 0; q < reps; q++) magnet_drift<kExact>(p, len, dm, k0d, k1d, hd);
}

// track_magnet.h:25-285 (body) after the host-side resolution. Every
// integrator is a sequence drift, kick, drift, ..., kick, drift; the body
// walks it in one loop with a single kick and a single drift step in the
// code (a few KB each once the products run on the integer pipes), so that
// the push's instruction footprint stays within the instruction caches.
//   uniform:   d_edge | 2 x d_edge (fast, straight models: d_fast_inside,
//              the two halves composed) | ... | d_edge, kick weight 0;
//   TEAPOT:    d_edge | d_inside | ... | d_edge, kick weight 0;
//   Yoshida-4: slices of 7 kicks with weights 0 1 2 3 2 1 0 and drifts
//              d0 d1 d2 d3 d3 d2 d1 d0; the d0 ending a slice and the d0
//              starting the next are consecutive (one step of 2 x d0).
template <bool kExact>
XTG_DEV void magnet_body(PState& p, const MagnetRec& r, const double* __restrict__ coefs) {
    int const dm = r.drift_model;
    double const k0d = r.k0_drift, k1d = r.k1_drift, hd = r.h_drift;
    if (r.only_drift) {
        magnet_drift<kExact>(p, r.length, dm, k0d, k1d, hd);
        return;
    }
    int const n = r.n_kicks;
    int const integ = r.integrator;
    if (n <= 0) {
        // no kick: the uniform and Yoshida loops run zero times; the TEAPOT
        // sequence keeps its edge drifts and its one kick
        if (integ == INT_TEAPOT) {
            magnet_drift<kExact>(p, r.d_edge, dm, k0d, k1d, hd);
            magnet_kick<kExact>(p, r, coefs, 0);
            magnet_drift<kExact>(p, r.d_edge, dm, k0d, k1d, hd);
        }
        return;
    }
    if (integ != INT_UNIFORM && integ != INT_TEAPOT && integ != INT_YOSHIDA4) return;
    bool const fast_merged = !kExact && (dm == 0 || dm == 1);
    int const nk = (integ == INT_YOSHIDA4) ? 7 * n : n;
#pragma unroll 1
    for (int j = 0; j <= nk; j++) {
        // the drift step before kick j (after the last kick when j == nk)
        double len;
        int reps = 1;
        int kw = 0;
        if (integ == INT_YOSHIDA4) {
            int const m = j % 7;
            int const di = (m == 0) ? 0 : (m <= 3 ? m : 7 - m);
            len = r.d_yoshida[di];
            if (m == 0 && j > 0 && j < nk) reps = 2;
            kw = (m <= 3) ? m : 6 - m;
        } else if (j == 0 || j == nk) {
            len = r.d_edge;
        } else if (integ == INT_TEAPOT) {
            len = r.d_inside;
        } else if (fast_merged) {
            len = r.d_fast_inside;
        } else {
            len = r.d_edge;
            reps = 2;
        }
        body_drift<kExact>(p, len, reps, dm, k0d, k1d, hd);
        if (j == nk) break;
        magnet_kick<kExact>(p, r, coefs, kw);
    }
}

// ---------------------------------------------------------------------------
// RF
// ---------------------------------------------------------------------------

// local_particle_custom_api.h:20-33, 195-217
XTG_DEV void add_to_energy(PState& p, double delta_energy, bool pz_only) {
    double ptau = p.ptau;
    double const mass_ratio = p.charge_ratio / p.chi;
    ptau = ptau + delta_energy / p.p0c / mass_ratio;
    double const old_rpp = p.rpp;
    double const beta0 = p.beta0;
    double const irpp = sqrt(ptau * ptau + 2 * ptau / beta0 + 1);
    double const new_rpp = 1. / irpp;
    double const new_rvv = irpp / (1 + beta0 * ptau);
    set_energy(p, irpp - 1, new_rvv, new_rpp, ptau);
    if (!pz_only) {
        // the reference reads rpp back (frozen: unchanged, f = 1)
        double const f = old_rpp / p.rpp;
        p.px = p.px * f;
        p.py = p.py * f;
    }
    refresh_energy_cache(p);
}

struct RfCtx {
    double q0, t_sim, line_length;
    bool kill, preserve_angle;
};

// track_rf.h:17-167 (order = -1, no transverse voltage)
XTG_DEV void rf_kick(PState& p, const CavityRec& r, double voltage, const RfCtx& c) {
    double arg;
    double const tau = p.zeta / p.beta0;
    if (r.harmonic == 0.0 && r.absolute_time != 1) {
        arg = r.phi_const - r.w_freq * tau;
    } else {
        double phase0 = 0;
        double frequency = r.frequency;
        if (r.harmonic != 0) {
            double const t_rev0 = c.line_length / (p.beta0 * kCLightD);
            frequency = frequency + (r.harmonic / t_rev0);
        }
        if (r.absolute_time == 1) {
            phase0 = phase0 + 2 * kPiD * (double)p.at_turn * frequency * c.t_sim;
        }
        arg = phase0 + r.lag_rad + r.phase - (2.0 * kPiD) / kCLightD * frequency * tau;
    }
    double const q = fabs(c.q0) * p.charge_ratio;
    double const energy_kick = q * voltage * sin(arg);
    if (!c.kill) add_to_energy(p, energy_kick + 0.0, !c.preserve_angle);
}

// track_rf.h:170-290
template <bool kExact>
XTG_DEV void cavity(PState& p, const CavityRec& r, const RfCtx& c) {
    int const dm = r.drift_model;
    int const n = r.n_kicks;
    if (r.integrator == INT_UNIFORM) {
        for (int i = 0; i < n; i++) {
            magnet_drift<kExact>(p, r.d_edge, dm, 0., 0., 0.);
            rf_kick(p, r, r.voltage * r.kw[0], c);
            magnet_drift<kExact>(p, r.d_edge, dm, 0., 0., 0.);
        }
    } else if (r.integrator == INT_TEAPOT) {
        magnet_drift<kExact>(p, r.d_edge, dm, 0., 0., 0.);
        for (int i = 0; i < n - 1; i++) {
            rf_kick(p, r, r.voltage * r.kw[0], c);
            magnet_drift<kExact>(p, r.d_inside, dm, 0., 0., 0.);
        }
        rf_kick(p, r, r.voltage * r.kw[0], c);
        magnet_drift<kExact>(p, r.d_edge, dm, 0., 0., 0.);
    } else if (r.integrator == INT_YOSHIDA4) {
        for (int s = 0; s < n; s++) {
            magnet_drift<kExact>(p, r.d_yoshida[0], dm, 0., 0., 0.);
            for (int j = 0; j < 7; j++) {
                int const kj = (j <= 3) ? j : 6 - j;
                rf_kick(p, r, r.voltage * r.kw[kj], c);
                int const dj = (j < 3) ? j + 1 : (j == 3 ? 3 : 6 - j);
                magnet_drift<kExact>(p, r.d_yoshida[dj], dm, 0., 0., 0.);
            }
        }
    }
}

// Out-of-line entry for the hot loop (one cavity per turn in most rings).
template <bool kExact>
XTG_COLD PState cavity_cold(PState p, const CavityRec& r, const RfCtx c) {
    cavity<kExact>(p, r, c);
    return p;
}

}  // namespace xtg
