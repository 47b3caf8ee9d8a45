// Kernels of the survival surrogate: a small MLP (width 256, GELU) with
// BF16 weights and activations and FP32 accumulation, trained with Adam.
//
// No reference counterpart: the reference has no learned component. The
// network screens dynamic-aperture scans so that FP64 tracking is spent
// only on initial conditions near the stability boundary.
//
// The contraction is one generic tile kernel on the tensor cores
// (mma.sync m16n8k16, bf16 x bf16 -> f32) that reads its operands through
// arbitrary (row, k) strides, so forward (X W^T), input gradient (dZ W) and
// weight gradient (dZ^T X) are the same kernel with different strides. Its
// epilogue fuses bias, GELU, the FP32 pre-activation store, the BF16
// activation store and the FP32 (accumulating) store. The layer sizes here
// are tiny next to the tracking that produces the training data, so the
// kernel favours simplicity over peak tensor throughput.
//
// Reductions (bias gradients, loss terms) run in a fixed order so results
// are reproducible run to run.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/xtrack_gb300.h"

namespace {

constexpr int BM = 64, BN = 64, BK = 32;
constexpr int LDS = BK + 8;   // padded row (bf16 elements): conflict-free fragment loads
constexpr int GEMM_THREADS = 128;

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
};

__device__ __forceinline__ float gelu_f(float z) {
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad_f(float z) {
    // d/dz [z Phi(z)] = Phi(z) + z phi(z)
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
           z * 0.39894228040143268f * expf(-0.5f * z * z);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Loads a ROWS x BK tile of a strided operand into shared memory as
// [row][k] (k contiguous), zero outside [0, rows) x [0, K). The thread
// mapping follows whichever stride is 1, so global reads coalesce for both
// plain and transposed operands.
template <int ROWS>
__device__ __forceinline__ void load_tile(__nv_bfloat16 (*S)[LDS], const __nv_bfloat16* G, int64_t s_row,
                                          int64_t s_k, int row0, int rows, int k0, int K) {
    int const tid = threadIdx.x;
    if (s_k == 1 || s_row != 1) {
        for (int e = tid; e < ROWS * BK; e += GEMM_THREADS) {
            int const r = e / BK, k = e % BK;
            int const gr = row0 + r, gk = k0 + k;
            __nv_bfloat16 v = __float2bfloat16(0.0f);
            if (gr < rows && gk < K) v = G[(int64_t)gr * s_row + (int64_t)gk * s_k];
            S[r][k] = v;
        }
    } else {
        for (int e = tid; e < ROWS * BK; e += GEMM_THREADS) {
            int const k = e / ROWS, r = e % ROWS;
            int const gr = row0 + r, gk = k0 + k;
            __nv_bfloat16 v = __float2bfloat16(0.0f);
            if (gr < rows && gk < K) v = G[(int64_t)gr * s_row + (int64_t)gk * s_k];
            S[r][k] = v;
        }
    }
}

__global__ void __launch_bounds__(GEMM_THREADS) gemm_bf16_kernel(const GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][LDS];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][LDS];
    int const m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int const wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    int const gid = lane >> 2, tig = lane & 3;

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[i][j][c] = 0.0f;

    for (int k0 = 0; k0 < g.K; k0 += BK) {
        load_tile<BM>(As, g.A, g.a_sm, g.a_sk, m0, g.M, k0, g.K);
        load_tile<BN>(Bs, g.B, g.b_sn, g.b_sk, n0, g.N, k0, g.K);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                int const r = wm + i * 16 + gid;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + tig * 2]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + tig * 2]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + tig * 2 + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + tig * 2 + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                int const c = wn + j * 8 + gid;
                bf[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + tig * 2]);
                bf[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + tig * 2 + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }

    // epilogue
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
                int const row = m0 + wm + i * 16 + gid + (c >= 2 ? 8 : 0);
                int const col = n0 + wn + j * 8 + tig * 2 + (c & 1);
                if (row >= g.M || col >= g.N) continue;
                float z = acc[i][j][c];
                if (g.bias) z += g.bias[col];
                if (g.Z) g.Z[(int64_t)row * g.z_ld + col] = z;
                if (g.Y) {
                    float const y = (g.act == XTG_MLP_ACT_GELU) ? gelu_f(z) : z;
                    g.Y[(int64_t)row * g.y_ld + col] = __float2bfloat16(y);
                }
                if (g.C) {
                    float* p = g.C + (int64_t)row * g.c_ld + col;
                    *p = g.c_accumulate ? (*p + z) : z;
                }
            }
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

// Loss of the two outputs per sample: out[m, 0] is the logit of P(survive),
// out[m, 1] the predicted normalised log loss turn. Binary cross-entropy on
// the logit for every sample, plus w_turn * squared error on the loss turn
// for samples that were lost (survive == 0). Writes the gradient with
// respect to out (scaled by 1/M) as fp32 and bf16, and the per-sample loss.
__global__ void loss_kernel(const float* __restrict__ out, const float* __restrict__ survive,
                            const float* __restrict__ logturn, int64_t M, float w_turn, float* __restrict__ dout,
                            __nv_bfloat16* __restrict__ dout16, float* __restrict__ loss) {
    int64_t const m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float const z = out[m * 2 + 0];
    float const y = survive[m];
    // log(1 + exp(-|z|)) + max(z, 0) - z*y  (stable BCE with logits)
    float const l_bce = fmaxf(z, 0.0f) - z * y + log1pf(expf(-fabsf(z)));
    float const p = 1.0f / (1.0f + expf(-z));
    float const inv_m = 1.0f / (float)M;
    float g0 = (p - y) * inv_m;
    float g1 = 0.0f, l_turn = 0.0f;
    if (y < 0.5f) {
        float const e = out[m * 2 + 1] - logturn[m];
        l_turn = w_turn * e * e;
        g1 = 2.0f * w_turn * e * inv_m;
    }
    dout[m * 2 + 0] = g0;
    dout[m * 2 + 1] = g1;
    dout16[m * 2 + 0] = __float2bfloat16(g0);
    dout16[m * 2 + 1] = __float2bfloat16(g1);
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
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM);
    if (grid.y > 65535u) return fail(XTG_E_CAPACITY, "xtg_mlp_gemm: M above 4194240");
    gemm_bf16_kernel<<<grid, GEMM_THREADS, 0, (cudaStream_t)stream>>>(g);
    xtg_internal_launch_add(1);
    return launched("gemm_bf16_kernel");
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

int32_t xtg_mlp_loss(const float* out, const float* survive, const float* logturn, int64_t M, float w_turn,
                     float* dout, void* dout16, float* loss, void* stream) {
    if (!out || !survive || !logturn || !dout || !dout16 || !loss)
        return fail(XTG_E_NULL, "xtg_mlp_loss: NULL argument");
    if (M <= 0) return XTG_OK;
    loss_kernel<<<blocks_for(M, 256), 256, 0, (cudaStream_t)stream>>>(out, survive, logturn, M, w_turn, dout,
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

}  // extern "C"
