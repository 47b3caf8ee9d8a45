// IEEE-754 binary64 multiplication on the integer pipes.
//
// GB300 executes FP64 at 2 lanes per clock per SM, 1/64 of its FP32 rate,
// while its integer pipes (the ALU and the IMAD path of the FMA pipe) are
// an order of magnitude wider. The push in its exact arithmetic is a chain
// of unfused FP64 multiplies and adds and is bound by that one narrow pipe.
// This header computes a binary64 product, correctly rounded to nearest
// even, with 32-bit integer operations, so that the multiplies run on the
// integer pipes while the FP64 pipe keeps the additions and the two proceed
// in parallel (measured on GB300: a chain of multiply+add pairs runs 1.8x
// faster with the multiplies here than with both on the FP64 pipe).
//
// The result is bit-identical to the hardware multiply (__dmul_rn) for
// every pair of operands. Normal operands whose product is normal take the
// integer path; a zero times a finite value gives the signed zero on the
// integer path; everything else (subnormal operands or results, overflow,
// infinities, NaN) goes to the FP64 unit through an out-of-line function,
// so that the common path issues no FP64 instruction even where the
// compiler would otherwise predicate the rare branch. Multiplication is
// commutative, so emul(a, b) == emul(b, a) bit for bit.
//
// An operand used in several products (a particle coordinate across the
// orders of a multipole kick) can be split once (F64Split) and reused.
//
// Shared by the device code (xtg_track.cu) and the host-side check of the
// library (xtg_f64_mul_host), which the tests compare with the CPU's
// multiply.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define XTG_EMU_HD __host__ __device__ __forceinline__
#define XTG_EMU_COLD __host__ __device__ __noinline__
#else
#define XTG_EMU_HD static inline
#define XTG_EMU_COLD static
#endif

namespace xtg {

XTG_EMU_HD uint64_t emu_bits(double v) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    memcpy(&b, &v, sizeof(b));
    return b;
#endif
}

XTG_EMU_HD double emu_double(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double v;
    memcpy(&v, &b, sizeof(v));
    return v;
#endif
}

// high word of (hi:lo) << s, for 0 < s < 32
XTG_EMU_HD uint32_t emu_funnel(uint32_t lo, uint32_t hi, uint32_t s) {
#ifdef __CUDA_ARCH__
    return __funnelshift_l(lo, hi, s);
#else
    return (hi << s) | (lo >> (32u - s));
#endif
}

// The FP64 unit's product, for the operands the integer path leaves out.
XTG_EMU_COLD double emu_mul_special(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    volatile double r = a * b;
    return r;
#endif
}

// One operand split into the fields the integer product needs.
struct F64Split {
    double v;        // the value itself (for the FP64 unit's fallback)
    uint32_t hi;     // high word of the bit pattern (sign, exponent, 20 fraction bits)
    uint32_t lo;     // low 32 fraction bits
    uint32_t mh;     // high 21 bits of the significand, implicit bit included
    uint32_t e;      // biased exponent field
};

XTG_EMU_HD F64Split emu_split(double v) {
    uint64_t const b = emu_bits(v);
    F64Split s;
    s.v = v;
    s.hi = (uint32_t)(b >> 32);
    s.lo = (uint32_t)b;
    s.mh = (s.hi & 0xfffffu) | 0x100000u;
    s.e = (s.hi >> 20) & 0x7ffu;
    return s;
}

// a * b rounded to nearest even, from split operands.
XTG_EMU_HD double emul_split(const F64Split& a, const F64Split& b) {
    // biased exponent field minus one of a product in [1, 2)
    int32_t const e = (int32_t)(a.e + b.e) - 1024;
    uint32_t const sign = (a.hi ^ b.hi) & 0x80000000u;
    uint32_t const ea1 = a.e - 1u, eb1 = b.e - 1u;
    // integer path: both operands normal, and the result's exponent field
    // e + top + 1 within [1, 2046] before rounding (a rounding carry into
    // 2047 gives the correctly rounded infinity)
    if ((ea1 > eb1 ? ea1 : eb1) < 2046u && (uint32_t)e < 2045u) {
        // the 106-bit product of the 53-bit significands (mh:lo) in four
        // 32-bit words w3:w2:w1:w0. The partial products are independent
        // (a short dependency chain for the integer pipes); the two middle
        // ones are below 2^53 (mh has 21 bits), so they and the carry out of
        // the lowest word add up without overflowing 64 bits.
        uint64_t const p0 = (uint64_t)a.lo * b.lo;
        uint64_t const p1 = (uint64_t)a.mh * b.lo;
        uint64_t const p2 = (uint64_t)a.lo * b.mh;
        uint64_t const p3 = (uint64_t)a.mh * b.mh;
        uint64_t const mid = p1 + p2 + (p0 >> 32);
        uint64_t const w = p3 + (mid >> 32);
        uint32_t const w0 = (uint32_t)p0, w1 = (uint32_t)mid;
        uint32_t const w2 = (uint32_t)w, w3 = (uint32_t)(w >> 32);
        // top = 1 when the product lies in [2^105, 2^106): its leading bit
        // is bit 9 of w3; shift the 53 leading bits to mh:ml (implicit bit
        // at bit 20 of mh) and the rest to g (guard bit at bit 31) and w0
        uint32_t const top = w3 >> 9;
        uint32_t const s = 12u - top;
        uint32_t const ml = emu_funnel(w1, w2, s);
        uint32_t const mh = emu_funnel(w2, w3, s);
        uint32_t const g = w1 << s;
        // round to nearest, ties to even: up when g:w0 exceeds half an ulp,
        // or equals it and the significand is odd
        uint64_t const gw = ((uint64_t)g << 32) | w0;
        uint64_t const up = gw >= (0x8000000000000001ull - (ml & 1u));
        uint64_t const m = ((((uint64_t)mh) << 32) | ml) + up;
        // the implicit bit of m adds the missing one to the exponent field,
        // and a rounding carry out of the significand increments it
        return emu_double((((uint64_t)(sign | ((uint32_t)(e + (int32_t)top) << 20))) << 32) + m);
    }
    // a zero times a finite value: the zero with the product's sign
    bool const a_zero = ((a.hi << 1) | a.lo) == 0, b_zero = ((b.hi << 1) | b.lo) == 0;
    if ((a_zero && b.e != 0x7ffu) || (b_zero && a.e != 0x7ffu)) return emu_double((uint64_t)sign << 32);
    return emu_mul_special(a.v, b.v);
}

// a * b rounded to nearest even.
XTG_EMU_HD double emul(double a, double b) {
    return emul_split(emu_split(a), emu_split(b));
}

}  // namespace xtg
