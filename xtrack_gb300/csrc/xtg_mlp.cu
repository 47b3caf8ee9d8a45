// Kernels of the survival surrogate: a small MLP (width 256, GELU in its
// tanh form) with BF16 weights and activations and FP32 accumulation,
// trained with Adam.
//
// No reference counterpart: the reference has no learned component. The
// network screens dynamic-aperture scans so that FP64 tracking is spent
// only on initial conditions near the stability boundary.
//
// The contraction runs on the fifth-generation tensor cores: one CTA of
// 512 threads owns a 128 x BN output tile (BN = 64, 128 or 256) whose FP32
// accumulator lives in tensor memory (TMEM, BN columns allocated per CTA).
// Operand tiles of 64 k-elements are staged in shared memory in the
// 128-byte-swizzled layout, in a two-stage mbarrier pipeline:
//   * TMA path (both operands with a unit stride along k or along the rows,
//     16-byte aligned base and row pitch): one thread issues
//     cp.async.bulk.tensor loads through tensor maps built on the host; an
//     operand stored with unit stride along its rows (a transposed operand
//     of the backward pass) is loaded as it lies and handed to the MMA as
//     MN-major;
//   * thread path (any other strides, e.g. 38-element rows): the 512
//     threads write the same swizzled K-major layout with plain loads,
//     zero outside the matrix.
// One elected thread issues tcgen05.mma (kind::f16, bf16 x bf16 -> f32,
// 128 x BN x 16 per instruction) and releases each stage with
// tcgen05.commit. In the epilogue the 16 warps read the accumulator with
// tcgen05.ld (a warp reaches only its quarter of the TMEM lanes: warp w
// takes rows 32*(w % 4) and up, and a quarter of their columns) and fuse
// bias, GELU, the FP32 pre-activation store, the BF16 activation store and
// an FP32 (accumulating) store, so the forward product X W^T, the input
// gradient dZ W and the weight gradient dZ^T X are one kernel with
// different strides. Every mbarrier wait is bounded:
// on time-out the CTA records XTG_E_TIMEOUT in a device error word
// (xtg_mlp_device_status), skips its stores and frees its TMEM.
//
// Reductions (bias gradients, loss terms) run in a fixed order so results
// are reproducible run to run.
#include <cuda.h>            // CUtensorMap and its enums; the encoder is fetched at run time
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/xtrack_gb300.h"

namespace {

constexpr int TM = 128;             // rows of a tile: the MMA's M
constexpr int TK = 64;              // k per stage: one 128-byte swizzle row of bf16
constexpr int UK = 16;              // k per tcgen05.mma of kind::f16
constexpr int STAGES = 2;
constexpr int GEMM_THREADS = 512;              // 16 warps
constexpr int COL_GROUPS = GEMM_THREADS / 128;   // warps per TMEM lane quarter: 4
constexpr uint32_t A_STAGE_BYTES = TM * TK * 2;   // 16 KB
constexpr uint32_t MN_BOX_BYTES = 64 * TK * 2;    // 8 KB: 64 rows x 64 k, MN-major
constexpr int MAX_BN = 256;
constexpr uint32_t MAX_DSMEM = STAGES * (A_STAGE_BYTES + MAX_BN * TK * 2) + 1024;

enum { LOAD_THREADS = 0, LOAD_TMA = 1 };

#define XTG_MLP_DEV_ERR_TIMEOUT 1

__device__ int32_t g_mlp_dev_err;

struct GemmArgs {
    const __nv_bfloat16* A;   // element (m, k) at A[m*a_sm + k*a_sk]
    int64_t a_sm, a_sk;
    const __nv_bfloat16* B;   // element (n, k) at B[n*b_sn + k*b_sk]
    int64_t b_sn, b_sk;
    int32_t M, N, K;
    const float* bias;        // [N] or NULL
    int32_t act;              // XTG_MLP_ACT_*
    float* Z;                 // pre-activation, fp32 [M, z_ld] or NULL
    int64_t z_ld;
    __nv_bfloat16* Y;         // activation, bf16 [M, y_ld] or NULL
    int64_t y_ld;
    float* C;                 // fp32 [M, c_ld] or NULL
    int64_t c_ld;
    int32_t c_accumulate;     // 1: C += result, 0: C = result
    int32_t bn;               // output columns per CTA: 64, 128 or 256 (= TMEM columns)
    int32_t load;             // LOAD_*
    int32_t a_mn, b_mn;       // TMA path: the operand is stored MN-major
    int32_t vec_z, vec_y, vec_c;   // output base 16-byte aligned and pitch a multiple of 16 bytes
    int32_t vec_bias;              // bias 16-byte aligned
};

// GELU in its tanh form (Hendrycks and Gimpel, 2016):
//   gelu(z) = z/2 (1 + tanh(u)),  u = sqrt(2/pi) (z + 0.044715 z^3),
// with the tanh of the special-function unit (tanh.approx.f32, relative
// error about 2^-11, below the resolution of the BF16 activations). One
// MUFU instruction and a few FMAs per element keep the epilogue off the
// issue limit that an erf-based GELU sets.
constexpr float kGeluS = 0.7978845608028654f;   // sqrt(2/pi)
constexpr float kGeluC = 0.044715f;

__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float gelu_f(float z) {
    float const t = tanh_sfu(kGeluS * fmaf(kGeluC * z, z * z, z));
    float const h = 0.5f * z;
    return fmaf(h, t, h);
}

__device__ __forceinline__ float gelu_grad_f(float z) {
    // d/dz = (1 + t)/2 + z/2 (1 - t^2) sqrt(2/pi) (1 + 3 * 0.044715 z^2)
    float const z2 = z * z;
    float const t = tanh_sfu(kGeluS * fmaf(kGeluC * z, z2, z));
    float const du = kGeluS * fmaf(3.0f * kGeluC, z2, 1.0f);
    return fmaf(0.5f * z * du, fmaf(-t, t, 1.0f), 0.5f * (1.0f + t));
}

// ---------------------------------------------------------------------------
// PTX wrappers: mbarrier, TMA, tcgen05
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// about 1 s at the GB300's 2.07 GHz SM clock
constexpr long long kMlpWaitLimit = 2000000000LL;

// Bounded wait on the phase of `parity`; on time-out records the error word
// and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kMlpWaitLimit) {
    if (mbar_try_wait(bar, parity)) return true;
    long long const t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) {
            atomicExch(&g_mlp_dev_err, XTG_MLP_DEV_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// 2-D tiled TMA load of one box at (c0 = innermost, c1) into shared memory,
// completing on `bar`. c0 is a multiple of 64 elements (128 bytes).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int32_t c0, int32_t c1,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor of a 128-byte-swizzled operand tile
// (start address, leading and stride byte offsets, descriptor version 1,
// layout SWIZZLE_128B). The tile base is 1024-byte aligned.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;
    d |= 2ull << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B,
// K-major (0) or MN-major (1) operands, N = bn, M = 128.
__device__ __forceinline__ uint32_t instr_desc(int bn, int a_mn, int b_mn) {
    uint32_t d = 0;
    d |= 1u << 4;                    // accumulator format F32
    d |= 1u << 7;                    // A format BF16
    d |= 1u << 10;                   // B format BF16
    d |= (uint32_t)(a_mn & 1) << 15;
    d |= (uint32_t)(b_mn & 1) << 16;
    d |= (uint32_t)(bn >> 3) << 17;
    d |= (uint32_t)(TM >> 4) << 24;
    return d;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma this thread issued so far is done.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

// Thread path: a ROWS x 64 tile of a strided operand into the 128-byte-
// swizzled K-major layout (row r at r*128 bytes, its 16-byte chunk c at
// chunk c ^ (r & 7)), zero outside [0, rows) x [0, K). Threads walk the
// unit-stride direction so global reads coalesce.
__device__ __forceinline__ void load_tile_sw128(unsigned char* S, int nrows, const __nv_bfloat16* G, int64_t s_row,
                                                int64_t s_k, int64_t row0, int64_t rows, int k0, int K) {
    int const tid = threadIdx.x;
    bool const k_inner = (s_k == 1 || s_row != 1);
    for (int e = tid; e < nrows * TK; e += GEMM_THREADS) {
        int const r = k_inner ? e / TK : e % nrows;
        int const k = k_inner ? e % TK : e / nrows;
        int64_t const gr = row0 + r;
        int const gk = k0 + k;
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (gr < rows && gk < K) v = G[gr * s_row + (int64_t)gk * s_k];
        uint32_t const off = (uint32_t)r * 128u + ((((uint32_t)k >> 3) ^ ((uint32_t)r & 7u)) << 4) + ((uint32_t)k & 7u) * 2u;
        *reinterpret_cast<__nv_bfloat16*>(S + off) = v;
    }
}

// Epilogue of 16 consecutive columns of one row. A chunk that lies inside
// the matrix is stored with 16-byte vector stores where the host found the
// output's base and pitch aligned (vec_* flags), else element by element.
__device__ __forceinline__ void store_row(const GemmArgs& g, int64_t row, int col0, const float (&v)[16]) {
    bool const full = col0 + 16 <= g.N;
    float z[16];
    if (full && g.vec_bias) {
        const float4* b4 = reinterpret_cast<const float4*>(g.bias + col0);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float4 const b = __ldg(b4 + q);
            z[4 * q] = v[4 * q] + b.x;
            z[4 * q + 1] = v[4 * q + 1] + b.y;
            z[4 * q + 2] = v[4 * q + 2] + b.z;
            z[4 * q + 3] = v[4 * q + 3] + b.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; j++) z[j] = v[j] + ((g.bias && col0 + j < g.N) ? __ldg(g.bias + col0 + j) : 0.0f);
    }
    if (full) {
        if (g.Z && g.vec_z) {
            float4* p = reinterpret_cast<float4*>(g.Z + row * g.z_ld + col0);
#pragma unroll
            for (int q = 0; q < 4; q++) p[q] = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
        }
        if (g.Y && g.vec_y) {
            uint32_t w[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                float const y0 = (g.act == XTG_MLP_ACT_GELU) ? gelu_f(z[2 * q]) : z[2 * q];
                float const y1 = (g.act == XTG_MLP_ACT_GELU) ? gelu_f(z[2 * q + 1]) : z[2 * q + 1];
                __nv_bfloat162 const h = __floats2bfloat162_rn(y0, y1);
                w[q] = *reinterpret_cast<const uint32_t*>(&h);
            }
            uint4* p = reinterpret_cast<uint4*>(g.Y + row * g.y_ld + col0);
            p[0] = make_uint4(w[0], w[1], w[2], w[3]);
            p[1] = make_uint4(w[4], w[5], w[6], w[7]);
        }
        if (g.C && g.vec_c) {
            float4* p = reinterpret_cast<float4*>(g.C + row * g.c_ld + col0);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float4 c = make_float4(z[4 * q], z[4 * q + 1], z[4 * q + 2], z[4 * q + 3]);
                if (g.c_accumulate) {
                    float4 const o = p[q];
                    c.x += o.x;
                    c.y += o.y;
                    c.z += o.z;
                    c.w += o.w;
                }
                p[q] = c;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 16; j++) {
        int const col = col0 + j;
        if (col >= g.N) break;
        if (g.Z && !(full && g.vec_z)) g.Z[row * g.z_ld + col] = z[j];
        if (g.Y && !(full && g.vec_y)) {
            float const y = (g.act == XTG_MLP_ACT_GELU) ? gelu_f(z[j]) : z[j];
            g.Y[row * g.y_ld + col] = __float2bfloat16(y);
        }
        if (g.C && !(full && g.vec_c)) {
            float* p = g.C + row * g.c_ld + col;
            *p = g.c_accumulate ? (*p + z[j]) : z[j];
        }
    }
}

__global__ void __launch_bounds__(GEMM_THREADS, 2) gemm_tc_kernel(const __grid_constant__ CUtensorMap tmA,
                                                               const __grid_constant__ CUtensorMap tmB,
                                                               const GemmArgs g) {
    extern __shared__ unsigned char dsm_raw[];
    __shared__ __align__(8) uint64_t full_bar[STAGES];
    __shared__ __align__(8) uint64_t empty_bar[STAGES];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ volatile int32_t abort_s;

    unsigned char* const dsm =
        dsm_raw + ((1024u - (smem_u32(dsm_raw) & 1023u)) & 1023u);   // 1024-byte aligned stages
    int const tid = threadIdx.x, warp = tid >> 5;
    int64_t const m0 = (int64_t)blockIdx.x * TM;
    int const n0 = blockIdx.y * g.bn;
    uint32_t const b_bytes = (uint32_t)g.bn * TK * 2;
    uint32_t const stage_bytes = A_STAGE_BYTES + b_bytes;
    int const nk = (g.K + TK - 1) / TK;
    bool const tma = g.load == LOAD_TMA;

    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) {
            mbar_init(&full_bar[s], tma ? 1u : (uint32_t)GEMM_THREADS);
            mbar_init(&empty_bar[s], 1u);
        }
        mbar_init(&done_bar, 1u);
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base_s)),
                     "r"((uint32_t)g.bn)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t const tmem = tmem_base_s;
    uint32_t const idesc = instr_desc(g.bn, g.a_mn, g.b_mn);
    // per-MMA advance along k: 32 bytes inside a K-major swizzle row, 16
    // rows of 128 bytes in an MN-major tile
    uint32_t const a_step = g.a_mn ? 16u * 128u : (uint32_t)UK * 2u;
    uint32_t const b_step = g.b_mn ? 16u * 128u : (uint32_t)UK * 2u;
    uint32_t const a_lbo = g.a_mn ? MN_BOX_BYTES : 16u, b_lbo = g.b_mn ? MN_BOX_BYTES : 16u;

    auto issue_mmas = [&](int kt) -> bool {
        int const s = kt % STAGES;
        if (!mbar_wait(&full_bar[s], (uint32_t)(kt / STAGES) & 1u)) return false;
        tc_fence_after();
        uint32_t const a0 = smem_u32(dsm + (size_t)s * stage_bytes);
        uint32_t const b0 = a0 + A_STAGE_BYTES;
#pragma unroll
        for (int kk = 0; kk < TK / UK; kk++) {
            uint64_t const da = smem_desc(a0 + kk * a_step, a_lbo, 1024u);
            uint64_t const db = smem_desc(b0 + kk * b_step, b_lbo, 1024u);
            tc_mma(tmem, da, db, idesc, (kt | kk) != 0 ? 1u : 0u);
        }
        tc_commit(&empty_bar[s]);
        return true;
    };

    if (tma) {
        if (tid == 0) {
            // producer
            int issued = 0;
            for (int kt = 0; kt < nk && !abort_s; kt++) {
                int const s = kt % STAGES;
                if (kt >= STAGES && !mbar_wait(&empty_bar[s], (uint32_t)(kt / STAGES - 1) & 1u)) {
                    abort_s = 1;
                    break;
                }
                unsigned char* const As = dsm + (size_t)s * stage_bytes;
                unsigned char* const Bs = As + A_STAGE_BYTES;
                int32_t const k0 = kt * TK;
                mbar_expect_tx(&full_bar[s], stage_bytes);
                if (!g.a_mn) {
                    tma_load_2d(As, &tmA, k0, (int32_t)m0, &full_bar[s]);
                } else {
                    tma_load_2d(As, &tmA, (int32_t)m0, k0, &full_bar[s]);
                    tma_load_2d(As + MN_BOX_BYTES, &tmA, (int32_t)m0 + 64, k0, &full_bar[s]);
                }
                if (!g.b_mn) {
                    tma_load_2d(Bs, &tmB, k0, n0, &full_bar[s]);
                } else {
                    for (int j = 0; j < g.bn / 64; j++)
                        tma_load_2d(Bs + j * MN_BOX_BYTES, &tmB, n0 + 64 * j, k0, &full_bar[s]);
                }
                issued = kt + 1;
            }
            if (abort_s) {
                // no copy may still write into shared memory when the CTA exits
                for (int kt = issued - STAGES < 0 ? 0 : issued - STAGES; kt < issued; kt++)
                    (void)mbar_wait(&full_bar[kt % STAGES], (uint32_t)(kt / STAGES) & 1u);
            }
        } else if (tid == 32) {
            int kt = 0;
            for (; kt < nk; kt++)
                if (!issue_mmas(kt)) {
                    abort_s = 1;
                    break;
                }
            // done_bar completes when every issued MMA has (plain arrive if none was)
            if (kt > 0) tc_commit(&done_bar);
            else mbar_arrive(&done_bar);
        }
    } else {
        bool issued_any = false;
        for (int kt = 0; kt < nk; kt++) {
            int const s = kt % STAGES;
            if (kt >= STAGES && !mbar_wait(&empty_bar[s], (uint32_t)(kt / STAGES - 1) & 1u)) abort_s = 1;
            __syncthreads();
            if (abort_s) break;
            unsigned char* const As = dsm + (size_t)s * stage_bytes;
            load_tile_sw128(As, TM, g.A, g.a_sm, g.a_sk, m0, g.M, kt * TK, g.K);
            load_tile_sw128(As + A_STAGE_BYTES, g.bn, g.B, g.b_sn, g.b_sk, n0, g.N, kt * TK, g.K);
            fence_proxy_async();
            mbar_arrive(&full_bar[s]);
            if (tid == 32) {
                if (issue_mmas(kt)) issued_any = true;
                else abort_s = 1;
            }
        }
        if (tid == 32) {
            if (issued_any) tc_commit(&done_bar);
            else mbar_arrive(&done_bar);
        }
    }

    // epilogue: a warp may read only the TMEM lanes of its quarter (warp % 4),
    // so warp w takes rows 32*(w % 4) + lane and the column group w / 4
    __syncwarp();
    bool const done = mbar_wait(&done_bar, 0u);
    __syncwarp();
    tc_fence_after();
    __syncthreads();
    if (done && !abort_s) {
        int const lane_q = warp & 3, col_q = warp >> 2;
        int64_t const row = m0 + lane_q * 32 + (tid & 31);
        uint32_t const taddr = tmem + ((uint32_t)(lane_q * 32) << 16);
        int const span = g.bn / COL_GROUPS;
        for (int c0 = col_q * span; c0 < (col_q + 1) * span && n0 + c0 < g.N; c0 += 16) {
            float v[16];
            if (nk > 0) {
                tc_ld16(taddr + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = 0.0f;
            }
            if (row < g.M) store_row(g, row, n0 + c0, v);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)g.bn)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Persistent variant for TMA-staged operands (K > 0). One CTA per SM walks
// the output tiles (tile t = blockIdx.x + j * gridDim.x, row tile t / nN,
// column tile t % nN): warp 0 loads the operand stages (TMA), warp 1 issues
// the MMAs, warps 2-17 run the epilogue. Two accumulators in tensor memory
// (2 x BN columns) let the epilogue of one tile run under the loads and
// MMAs of the next, and four stages keep the loads ahead of the MMAs.
// Warp 2 + w (w = 0..15) reads TMEM lane quarter (2 + w) % 4 and a quarter
// of the tile's columns. Barriers: full / empty per stage (producer <-> MMA), acc_full / acc_empty
// per accumulator (MMA <-> epilogue). Every wait is bounded; a role that
// gives up raises the shared abort flag, the others leave their loops
// (bounded themselves), the MMA thread waits for its MMAs in flight and the
// producer for its copies before the tensor memory is freed.
// ---------------------------------------------------------------------------
constexpr int P_STAGES = 4;
constexpr int P_EPI_WARPS = 16;
constexpr int P_THREADS = 64 + 32 * P_EPI_WARPS;
constexpr uint32_t P_MAX_DSMEM = P_STAGES * (A_STAGE_BYTES + MAX_BN * TK * 2) + 1024;

__global__ void __launch_bounds__(P_THREADS, 1)
    gemm_tc_persistent_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                              const GemmArgs g) {
    extern __shared__ unsigned char dsm_raw[];
    __shared__ __align__(8) uint64_t full_bar[P_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[P_STAGES];
    __shared__ __align__(8) uint64_t acc_full[2];
    __shared__ __align__(8) uint64_t acc_empty[2];
    __shared__ __align__(8) uint64_t mma_done;
    __shared__ uint32_t tmem_base_s;
    __shared__ volatile int32_t abort_s;

    unsigned char* const dsm = dsm_raw + ((1024u - (smem_u32(dsm_raw) & 1023u)) & 1023u);
    int const tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint32_t const stage_bytes = A_STAGE_BYTES + (uint32_t)g.bn * TK * 2;
    int const nk = (g.K + TK - 1) / TK;
    int const n_tn = (g.N + g.bn - 1) / g.bn;
    int64_t const n_total = (((int64_t)g.M + TM - 1) / TM) * n_tn;
    uint32_t const ncols = 2u * (uint32_t)g.bn;

    if (tid == 0) {
        for (int s = 0; s < P_STAGES; s++) {
            mbar_init(&full_bar[s], 1u);
            mbar_init(&empty_bar[s], 1u);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(&acc_full[a], 1u);
            mbar_init(&acc_empty[a], (uint32_t)P_EPI_WARPS);
        }
        mbar_init(&mma_done, 1u);
        abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base_s)),
                     "r"(ncols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    uint32_t const tmem = tmem_base_s;

    if (warp == 0) {
        if (lane == 0) {
            // producer
            int64_t it = 0;
            for (int64_t t = blockIdx.x; t < n_total && !abort_s; t += gridDim.x) {
                int32_t const m0 = (int32_t)((t / n_tn) * TM);
                int32_t const n0 = (int32_t)(t % n_tn) * g.bn;
                for (int kt = 0; kt < nk; kt++, it++) {
                    int const s = (int)(it % P_STAGES);
                    if (it >= P_STAGES && !mbar_wait(&empty_bar[s], (uint32_t)((it / P_STAGES - 1) & 1))) {
                        abort_s = 1;
                        break;
                    }
                    if (abort_s) break;
                    unsigned char* const As = dsm + (size_t)s * stage_bytes;
                    unsigned char* const Bs = As + A_STAGE_BYTES;
                    int32_t const k0 = kt * TK;
                    mbar_expect_tx(&full_bar[s], stage_bytes);
                    if (!g.a_mn) {
                        tma_load_2d(As, &tmA, k0, m0, &full_bar[s]);
                    } else {
                        tma_load_2d(As, &tmA, m0, k0, &full_bar[s]);
                        tma_load_2d(As + MN_BOX_BYTES, &tmA, m0 + 64, k0, &full_bar[s]);
                    }
                    if (!g.b_mn) {
                        tma_load_2d(Bs, &tmB, k0, n0, &full_bar[s]);
                    } else {
                        for (int j = 0; j < g.bn / 64; j++)
                            tma_load_2d(Bs + j * MN_BOX_BYTES, &tmB, n0 + 64 * j, k0, &full_bar[s]);
                    }
                }
            }
            if (abort_s) {
                // no copy may still write into shared memory when the CTA exits
                for (int64_t j = it - P_STAGES < 0 ? 0 : it - P_STAGES; j < it; j++)
                    (void)mbar_wait(&full_bar[j % P_STAGES], (uint32_t)((j / P_STAGES) & 1));
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            uint32_t const idesc = instr_desc(g.bn, g.a_mn, g.b_mn);
            uint32_t const a_step = g.a_mn ? 16u * 128u : (uint32_t)UK * 2u;
            uint32_t const b_step = g.b_mn ? 16u * 128u : (uint32_t)UK * 2u;
            uint32_t const a_lbo = g.a_mn ? MN_BOX_BYTES : 16u, b_lbo = g.b_mn ? MN_BOX_BYTES : 16u;
            int64_t it = 0, i = 0;
            bool issued = false;
            for (int64_t t = blockIdx.x; t < n_total && !abort_s; t += gridDim.x, i++) {
                int const acc = (int)(i & 1);
                if (i >= 2 && !mbar_wait(&acc_empty[acc], (uint32_t)(((i >> 1) - 1) & 1))) {
                    abort_s = 1;
                    break;
                }
                tc_fence_after();
                uint32_t const d = tmem + (uint32_t)(acc * g.bn);
                bool ok = true;
                for (int kt = 0; kt < nk; kt++, it++) {
                    int const s = (int)(it % P_STAGES);
                    if (!mbar_wait(&full_bar[s], (uint32_t)((it / P_STAGES) & 1))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    uint32_t const a0 = smem_u32(dsm + (size_t)s * stage_bytes);
                    uint32_t const b0 = a0 + A_STAGE_BYTES;
#pragma unroll
                    for (int kk = 0; kk < TK / UK; kk++) {
                        uint64_t const da = smem_desc(a0 + kk * a_step, a_lbo, 1024u);
                        uint64_t const db = smem_desc(b0 + kk * b_step, b_lbo, 1024u);
                        tc_mma(d, da, db, idesc, (kt | kk) != 0 ? 1u : 0u);
                    }
                    issued = true;
                    tc_commit(&empty_bar[s]);
                }
                if (!ok) {
                    abort_s = 1;
                    break;
                }
                tc_commit(&acc_full[acc]);
            }
            // every MMA issued has completed before the tensor memory is freed
            if (issued) tc_commit(&mma_done);
            else mbar_arrive(&mma_done);
            if (!mbar_wait(&mma_done, 0u)) abort_s = 1;
        }
    } else {
        // epilogue: a warp reaches only the TMEM lanes of its quarter
        // (warp % 4); the four warps of a quarter take a quarter of the
        // columns each
        int const lane_q = warp & 3, col_g = (warp - 2) >> 2;
        int const span = g.bn / 4;
        int64_t i = 0;
        for (int64_t t = blockIdx.x; t < n_total; t += gridDim.x, i++) {
            int const acc = (int)(i & 1);
            bool const ok = mbar_wait(&acc_full[acc], (uint32_t)((i >> 1) & 1));
            if (__any_sync(0xffffffffu, !ok || abort_s)) {
                abort_s = 1;
                break;
            }
            tc_fence_after();
            int64_t const m0 = (t / n_tn) * TM;
            int const n0 = (int)(t % n_tn) * g.bn;
            int64_t const row = m0 + lane_q * 32 + lane;
            uint32_t const taddr = tmem + ((uint32_t)(lane_q * 32) << 16) + (uint32_t)(acc * g.bn);
            for (int c0 = col_g * span; c0 < (col_g + 1) * span && n0 + c0 < g.N; c0 += 16) {
                float v[16];
                tc_ld16(taddr + (uint32_t)c0, v);
                if (row < g.M) store_row(g, row, n0 + c0, v);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[acc]);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// One wait of the contraction's kind on a barrier that nothing completes:
// thread 0 gives up after `limit` cycles and records the time-out in the
// device error word.
__global__ void mlp_wait_check_kernel(long long limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) (void)mbar_wait(&bar, 0u, limit);
    __syncthreads();
}

// dZ = dY * act'(Z): fp32 and bf16 copies.
__global__ void act_backward_kernel(const float* __restrict__ dY, const float* __restrict__ Z, int64_t n,
                                    int32_t act, float* __restrict__ dZ, __nv_bfloat16* __restrict__ dZ16) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float d = dY[i];
    if (act == XTG_MLP_ACT_GELU) d *= gelu_grad_f(Z[i]);
    if (dZ) dZ[i] = d;
    if (dZ16) dZ16[i] = __float2bfloat16(d);
}

// out[n] (+)= sum over rows of X[m, n] (fp32, fixed summation order).
// Block: 32 columns x 8 row groups.
__global__ void colsum_kernel(const float* __restrict__ X, int64_t M, int32_t N, int64_t ld, float* out,
                              int32_t accumulate) {
    __shared__ float part[8][33];
    int const cx = threadIdx.x & 31, gy = threadIdx.x >> 5;
    int const col = blockIdx.x * 32 + cx;
    float s = 0.0f;
    if (col < N)
        for (int64_t m = gy; m < M; m += 8) s += X[m * ld + col];
    part[gy][cx] = s;
    __syncthreads();
    if (gy == 0 && col < N) {
        float t = 0.0f;
        for (int r = 0; r < 8; r++) t += part[r][cx];
        out[col] = accumulate ? out[col] + t : t;
    }
}

// Loss of the two outputs per sample: out[m*ld + 0] is the logit of
// P(survive), out[m*ld + 1] the predicted normalised log loss turn (the
// other columns of a padded output layer are not read). Binary
// cross-entropy on the logit for every sample, plus w_turn * squared error
// on the loss turn for samples that were lost (survive == 0). Writes the
// gradient with respect to out (scaled by 1/M) into columns 0 and 1 of
// dout / dout16 (row pitch ld) and the per-sample loss.
__global__ void loss_kernel(const float* __restrict__ out, int64_t ld, const float* __restrict__ survive,
                            const float* __restrict__ logturn, int64_t M, float w_turn, float* __restrict__ dout,
                            __nv_bfloat16* __restrict__ dout16, float* __restrict__ loss) {
    int64_t const m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float const z = out[m * ld + 0];
    float const y = survive[m];
    // log(1 + exp(-|z|)) + max(z, 0) - z*y  (stable BCE with logits)
    float const l_bce = fmaxf(z, 0.0f) - z * y + log1pf(expf(-fabsf(z)));
    float const p = 1.0f / (1.0f + expf(-z));
    float const inv_m = 1.0f / (float)M;
    float g0 = (p - y) * inv_m;
    float g1 = 0.0f, l_turn = 0.0f;
    if (y < 0.5f) {
        float const e = out[m * ld + 1] - logturn[m];
        l_turn = w_turn * e * e;
        g1 = 2.0f * w_turn * e * inv_m;
    }
    dout[m * ld + 0] = g0;
    dout[m * ld + 1] = g1;
    dout16[m * ld + 0] = __float2bfloat16(g0);
    dout16[m * ld + 1] = __float2bfloat16(g1);
    loss[m] = l_bce + l_turn;
}

// Adam on fp32 master weights; refreshes the bf16 copy used by the GEMMs.
__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ w16, const float* __restrict__ grad,
                            float* __restrict__ m1, float* __restrict__ m2, int64_t n, float lr, float beta1,
                            float beta2, float eps, float weight_decay, float bc1, float bc2) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g = grad[i];
    float const a = beta1 * m1[i] + (1.0f - beta1) * g;
    float const b = beta2 * m2[i] + (1.0f - beta2) * g * g;
    m1[i] = a;
    m2[i] = b;
    float const mhat = a / bc1;
    float const vhat = b / bc2;
    float x = w[i];
    x -= lr * (mhat / (sqrtf(vhat) + eps) + weight_decay * x);
    w[i] = x;
    if (w16) w16[i] = __float2bfloat16(x);
}

__global__ void to_bf16_kernel(const float* __restrict__ x, int64_t n, __nv_bfloat16* __restrict__ y) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16(x[i]);
}

thread_local char g_mlp_err[256];

int32_t fail(int32_t code, const char* msg) {
    snprintf(g_mlp_err, sizeof(g_mlp_err), "%s", msg);
    return code;
}

int32_t launched(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        snprintf(g_mlp_err, sizeof(g_mlp_err), "%s: %s", what, cudaGetErrorString(e));
        return XTG_E_CUDA;
    }
    return XTG_OK;
}

unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// host: operand staging mode and TMA tensor maps
// ---------------------------------------------------------------------------
enum { MODE_THREADS = 0, MODE_K = 1, MODE_MN = 2 };

// MODE_K: unit stride along k (rows of `row_pitch` elements); MODE_MN: unit
// stride along the rows (k-rows of `k_pitch` elements); both need a 16-byte
// aligned base and pitch. Anything else is staged by the threads.
int operand_mode(const void* p, int64_t s_row, int64_t s_k, int64_t rows, int64_t K) {
    if (K == 0 || ((uintptr_t)p & 15u) != 0) return MODE_THREADS;
    if (s_k == 1 && s_row >= K && s_row % 8 == 0 && s_row * 2 < (1LL << 40)) return MODE_K;
    if (s_row == 1 && s_k >= rows && s_k % 8 == 0 && s_k * 2 < (1LL << 40)) return MODE_MN;
    return MODE_THREADS;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (the library links no libcuda); NULL if unavailable.
EncodeTiledFn encoder() {
    static EncodeTiledFn const fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// 2-D bf16 tensor map: `inner` unit-stride elements by `outer` lines of
// `pitch` elements; boxes of 64 x box_outer, 128-byte swizzle, zero fill
// outside the tensor.
bool encode_map(CUtensorMap* map, const void* base, int64_t inner, int64_t outer, int64_t pitch, uint32_t box_outer) {
    EncodeTiledFn const fn = encoder();
    if (!fn) return false;
    cuuint64_t const dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    cuuint64_t const strides[1] = {(cuuint64_t)pitch * 2u};
    cuuint32_t const box[2] = {(cuuint32_t)TK, box_outer};
    cuuint32_t const estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

extern "C" int64_t xtg_internal_launch_add(int64_t n);

extern "C" {

int32_t xtg_mlp_get_last_error(char* buf, int64_t n) {
    if (!buf || n <= 0) return XTG_E_NULL;
    snprintf(buf, (size_t)n, "%s", g_mlp_err);
    return XTG_OK;
}

int32_t xtg_mlp_gemm(const void* A, int64_t a_sm, int64_t a_sk, const void* B, int64_t b_sn, int64_t b_sk,
                     int32_t M, int32_t N, int32_t K, const float* bias, int32_t act, float* Z, int64_t z_ld,
                     void* Y, int64_t y_ld, float* C, int64_t c_ld, int32_t c_accumulate, void* stream) {
    if (!A || !B) return fail(XTG_E_NULL, "xtg_mlp_gemm: NULL operand");
    if (M < 0 || N < 0 || K < 0) return fail(XTG_E_VALUE, "xtg_mlp_gemm: negative size");
    if (act != XTG_MLP_ACT_NONE && act != XTG_MLP_ACT_GELU) return fail(XTG_E_VALUE, "xtg_mlp_gemm: bad act");
    if (!Z && !Y && !C) return fail(XTG_E_NULL, "xtg_mlp_gemm: no output");
    if (M == 0 || N == 0) return XTG_OK;
    GemmArgs g;
    g.A = (const __nv_bfloat16*)A;
    g.a_sm = a_sm;
    g.a_sk = a_sk;
    g.B = (const __nv_bfloat16*)B;
    g.b_sn = b_sn;
    g.b_sk = b_sk;
    g.M = M;
    g.N = N;
    g.K = K;
    g.bias = bias;
    g.act = act;
    g.Z = Z;
    g.z_ld = z_ld;
    g.Y = (__nv_bfloat16*)Y;
    g.y_ld = y_ld;
    g.C = C;
    g.c_ld = c_ld;
    g.c_accumulate = c_accumulate;
    g.bn = N <= 64 ? 64 : (N <= 128 ? 128 : MAX_BN);
    g.a_mn = g.b_mn = 0;
    g.load = LOAD_THREADS;
    g.vec_z = Z && ((uintptr_t)Z & 15u) == 0 && z_ld % 4 == 0;
    g.vec_y = Y && ((uintptr_t)Y & 15u) == 0 && y_ld % 8 == 0;
    g.vec_c = C && ((uintptr_t)C & 15u) == 0 && c_ld % 4 == 0;
    g.vec_bias = bias && ((uintptr_t)bias & 15u) == 0;

    CUtensorMap ta, tb;
    memset(&ta, 0, sizeof(ta));
    memset(&tb, 0, sizeof(tb));
    int const mode_a = operand_mode(A, a_sm, a_sk, M, K);
    int const mode_b = operand_mode(B, b_sn, b_sk, N, K);
    if (mode_a != MODE_THREADS && mode_b != MODE_THREADS) {
        bool ok = mode_a == MODE_K ? encode_map(&ta, A, K, M, a_sm, TM) : encode_map(&ta, A, M, K, a_sk, 64);
        ok = ok && (mode_b == MODE_K ? encode_map(&tb, B, K, N, b_sn, (uint32_t)g.bn)
                                     : encode_map(&tb, B, N, K, b_sk, 64));
        if (ok) {
            g.load = LOAD_TMA;
            g.a_mn = mode_a == MODE_MN;
            g.b_mn = mode_b == MODE_MN;
        }
    }
    int64_t const m_tiles = ((int64_t)M + TM - 1) / TM;
    int64_t const n_tiles = ((int64_t)N + g.bn - 1) / g.bn;
    if (m_tiles > 0x7FFFFFFFLL || n_tiles > 65535) return fail(XTG_E_CAPACITY, "xtg_mlp_gemm: grid too large");
    if (g.load == LOAD_TMA) {
        // persistent: one CTA per SM over the tiles
        int dev = 0, sms = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(gemm_tc_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)P_MAX_DSMEM);
        if (e != cudaSuccess) {
            snprintf(g_mlp_err, sizeof(g_mlp_err), "xtg_mlp_gemm: %s", cudaGetErrorString(e));
            return XTG_E_CUDA;
        }
        int64_t const total = m_tiles * n_tiles;
        unsigned const grid = (unsigned)(total < (int64_t)sms ? total : (int64_t)sms);
        uint32_t const dsmem = P_STAGES * (A_STAGE_BYTES + (uint32_t)g.bn * TK * 2) + 1024;
        gemm_tc_persistent_kernel<<<grid, P_THREADS, dsmem, (cudaStream_t)stream>>>(ta, tb, g);
        xtg_internal_launch_add(1);
        return launched("gemm_tc_persistent_kernel");
    }
    uint32_t const dsmem = STAGES * (A_STAGE_BYTES + (uint32_t)g.bn * TK * 2) + 1024;
    cudaError_t e = cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MAX_DSMEM);
    if (e != cudaSuccess) {
        snprintf(g_mlp_err, sizeof(g_mlp_err), "xtg_mlp_gemm: %s", cudaGetErrorString(e));
        return XTG_E_CUDA;
    }
    dim3 grid((unsigned)m_tiles, (unsigned)n_tiles);
    gemm_tc_kernel<<<grid, GEMM_THREADS, dsmem, (cudaStream_t)stream>>>(ta, tb, g);
    xtg_internal_launch_add(1);
    return launched("gemm_tc_kernel");
}

int32_t xtg_mlp_act_backward(const float* dY, const float* Z, int64_t n, int32_t act, float* dZ, void* dZ16,
                             void* stream) {
    if (!dY || (act == XTG_MLP_ACT_GELU && !Z)) return fail(XTG_E_NULL, "xtg_mlp_act_backward: NULL input");
    if (n <= 0) return XTG_OK;
    act_backward_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(dY, Z, n, act, dZ,
                                                                            (__nv_bfloat16*)dZ16);
    xtg_internal_launch_add(1);
    return launched("act_backward_kernel");
}

int32_t xtg_mlp_colsum(const float* X, int64_t M, int32_t N, int64_t ld, float* out, int32_t accumulate,
                       void* stream) {
    if (!X || !out) return fail(XTG_E_NULL, "xtg_mlp_colsum: NULL argument");
    if (N <= 0) return XTG_OK;
    colsum_kernel<<<blocks_for(N, 32), 256, 0, (cudaStream_t)stream>>>(X, M, N, ld, out, accumulate);
    xtg_internal_launch_add(1);
    return launched("colsum_kernel");
}

int32_t xtg_mlp_loss(const float* out, int64_t ld, const float* survive, const float* logturn, int64_t M,
                     float w_turn, float* dout, void* dout16, float* loss, void* stream) {
    if (!out || !survive || !logturn || !dout || !dout16 || !loss)
        return fail(XTG_E_NULL, "xtg_mlp_loss: NULL argument");
    if (ld < 2) return fail(XTG_E_VALUE, "xtg_mlp_loss: ld must be >= 2");
    if (M <= 0) return XTG_OK;
    loss_kernel<<<blocks_for(M, 256), 256, 0, (cudaStream_t)stream>>>(out, ld, survive, logturn, M, w_turn, dout,
                                                                    (__nv_bfloat16*)dout16, loss);
    xtg_internal_launch_add(1);
    return launched("loss_kernel");
}

int32_t xtg_mlp_adam(float* w, void* w16, const float* grad, float* m1, float* m2, int64_t n, float lr,
                     float beta1, float beta2, float eps, float weight_decay, int64_t step, void* stream) {
    if (!w || !grad || !m1 || !m2) return fail(XTG_E_NULL, "xtg_mlp_adam: NULL argument");
    if (step < 1) return fail(XTG_E_VALUE, "xtg_mlp_adam: step must be >= 1");
    if (n <= 0) return XTG_OK;
    float const bc1 = 1.0f - powf(beta1, (float)step);
    float const bc2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(w, (__nv_bfloat16*)w16, grad, m1, m2, n, lr,
                                                                    beta1, beta2, eps, weight_decay, bc1, bc2);
    xtg_internal_launch_add(1);
    return launched("adam_kernel");
}

int32_t xtg_mlp_to_bf16(const float* x, int64_t n, void* y, void* stream) {
    if (!x || !y) return fail(XTG_E_NULL, "xtg_mlp_to_bf16: NULL argument");
    if (n <= 0) return XTG_OK;
    to_bf16_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x, n, (__nv_bfloat16*)y);
    xtg_internal_launch_add(1);
    return launched("to_bf16_kernel");
}

int32_t xtg_mlp_check_bounded_wait(int64_t limit_cycles) {
    if (limit_cycles < 1 || limit_cycles > kMlpWaitLimit)
        return fail(XTG_E_VALUE, "xtg_mlp_check_bounded_wait: limit must be in [1, 2e9] cycles");
    mlp_wait_check_kernel<<<1, 32>>>((long long)limit_cycles);
    xtg_internal_launch_add(1);
    int32_t const st = launched("mlp_wait_check_kernel");
    if (st != XTG_OK) return st;
    return xtg_mlp_device_status();
}

int32_t xtg_mlp_device_status(void) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        snprintf(g_mlp_err, sizeof(g_mlp_err), "xtg_mlp_device_status: %s", cudaGetErrorString(e));
        return XTG_E_CUDA;
    }
    int32_t h = 0, zero = 0;
    e = cudaMemcpyFromSymbol(&h, g_mlp_dev_err, sizeof(h));
    if (e == cudaSuccess && h != 0) e = cudaMemcpyToSymbol(g_mlp_dev_err, &zero, sizeof(zero));
    if (e != cudaSuccess) {
        snprintf(g_mlp_err, sizeof(g_mlp_err), "xtg_mlp_device_status: %s", cudaGetErrorString(e));
        return XTG_E_CUDA;
    }
    if (h == XTG_MLP_DEV_ERR_TIMEOUT) return fail(XTG_E_TIMEOUT, "a bounded wait inside an xtg_mlp kernel timed out");
    return XTG_OK;
}

}  // extern "C"
