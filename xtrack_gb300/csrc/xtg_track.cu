// The GB300 push: kernels, launch logic and the C-ABI entry points of
// include/xtrack_gb300.h.
//
// Replaces xtrack's generated `track_line` kernel (xtrack/tracker.py:
// 543-750). One thread owns one particle for a whole launch: its
// coordinates live in registers, elements are read from the packed table
// (xtg_table.h) as warp-uniform records, and particle memory is touched only
// at launch boundaries and monitor records.
//
// Compiled with -fmad=false: the exact-arithmetic path must not have its
// products fused into additions. The fast path uses explicit fma().
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/xtrack_gb300.h"
#include "xtg_lattice.h"
#include "xtg_physics.cuh"

using namespace xtg;

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launch_count{0};

static int32_t set_error(int32_t code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define XTG_CUDA_CHECK(call)                                                         \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess)                                                       \
            return set_error(XTG_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// ---------------------------------------------------------------------------
// lattice handle
// ---------------------------------------------------------------------------
struct DevTable {
    unsigned char* d_bytes = nullptr;
    int64_t* d_offsets = nullptr;
    int64_t n_bytes = 0;
    std::vector<int64_t> h_offsets;
    std::vector<double> flops;
};

struct xtg_lattice {
    std::vector<xtg_element> elements;
    xtg_config config;
    int device = 0;
    DevTable fwd;
    DevTable bwd;          // built on first backtracking call
    bool has_bwd = false;
    int32_t block_size = 256;
    int32_t compact_every = 0;   // turns per launch (0: all turns in one launch)
    std::mutex mu;
};

static int32_t upload_table(const PackedLattice& pl, DevTable* t) {
    t->n_bytes = (int64_t)pl.bytes.size();
    t->h_offsets = pl.offsets;
    t->flops = pl.flops_fast;
    size_t nb = pl.bytes.size() > 0 ? pl.bytes.size() : 16;
    XTG_CUDA_CHECK(cudaMalloc(&t->d_bytes, nb));
    XTG_CUDA_CHECK(cudaMalloc(&t->d_offsets, pl.offsets.size() * sizeof(int64_t)));
    if (!pl.bytes.empty())
        XTG_CUDA_CHECK(cudaMemcpy(t->d_bytes, pl.bytes.data(), pl.bytes.size(), cudaMemcpyHostToDevice));
    XTG_CUDA_CHECK(cudaMemcpy(t->d_offsets, pl.offsets.data(), pl.offsets.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice));
    return XTG_OK;
}

static void free_table(DevTable* t) {
    if (t->d_bytes) cudaFree(t->d_bytes);
    if (t->d_offsets) cudaFree(t->d_offsets);
    t->d_bytes = nullptr;
    t->d_offsets = nullptr;
}

// ---------------------------------------------------------------------------
// kernel
// ---------------------------------------------------------------------------
struct KParams {
    const unsigned char* __restrict__ table;
    int64_t rec_begin;           // byte offset of the first record to track
    int32_t rec_count;           // records per turn
    int32_t num_turns;
    int64_t capacity;
    xtg_particles P;
    xtg_monitor M;
    int32_t flag_monitor;
    int32_t flag_end_turn_actions;
    int32_t flag_reset_s;
    int32_t backtrack;
    int64_t num_ele_line;
    double line_length;
    uint64_t track_flags;
    int32_t has_global;
    int32_t preserve_angle;
    double global_lim;
};

__device__ __forceinline__ bool flag_on(uint64_t flags, int bit) { return (flags >> bit) & 1u; }

// particles_monitor.h:12-77 record (LocalParticle_to_Particles into the
// monitor's data at `store_at`; NULL arrays are not recorded).
__device__ __forceinline__ void monitor_store(const KParams& kp, const PState& p, int64_t i, int64_t k) {
    const xtg_particles& D = kp.M.data;
    const xtg_particles& S = kp.P;
    if (D.x) D.x[k] = p.x;
    if (D.px) D.px[k] = p.px;
    if (D.y) D.y[k] = p.y;
    if (D.py) D.py[k] = p.py;
    if (D.zeta) D.zeta[k] = p.zeta;
    if (D.delta) D.delta[k] = p.delta;
    if (D.ptau) D.ptau[k] = p.ptau;
    if (D.rpp) D.rpp[k] = p.rpp;
    if (D.rvv) D.rvv[k] = p.rvv;
    if (D.s) D.s[k] = p.s;
    if (D.chi) D.chi[k] = p.chi;
    if (D.charge_ratio) D.charge_ratio[k] = p.charge_ratio;
    if (D.beta0) D.beta0[k] = p.beta0;
    if (D.p0c) D.p0c[k] = p.p0c;
    if (D.ax) D.ax[k] = p.ax;
    if (D.ay) D.ay[k] = p.ay;
    if (D.state) D.state[k] = p.state;
    if (D.at_element) D.at_element[k] = p.at_element;
    if (D.at_turn) D.at_turn[k] = p.at_turn;
    if (D.particle_id) D.particle_id[k] = S.particle_id[i];
    if (D.gamma0) D.gamma0[k] = S.gamma0 ? S.gamma0[i] : 0.;
    if (D.weight) D.weight[k] = S.weight ? S.weight[i] : 0.;
    if (D.pdg_id) D.pdg_id[k] = S.pdg_id ? S.pdg_id[i] : 0;
    if (D.parent_particle_id) D.parent_particle_id[k] = S.parent_particle_id ? S.parent_particle_id[i] : 0;
}

__device__ __forceinline__ void monitor(const KParams& kp, const PState& p, int64_t i, int64_t pid) {
    const xtg_monitor& m = kp.M;
    int64_t at_turn;
    if (m.ebe_mode) {
        at_turn = p.at_element;
    } else {
        if (kp.backtrack) return;
        at_turn = p.at_turn;
    }
    int64_t const n_turns_record = m.stop_at_turn - m.start_at_turn;
    if (m.n_repetitions == 1) {
        if (at_turn >= m.start_at_turn && at_turn < m.stop_at_turn && pid < m.part_id_end &&
            pid >= m.part_id_start) {
            int64_t const store_at = n_turns_record * (pid - m.part_id_start) + at_turn - m.start_at_turn;
            if (store_at >= 0 && store_at < m.n_records) monitor_store(kp, p, i, store_at);
        }
    } else if (m.n_repetitions > 1) {
        if (at_turn < m.start_at_turn) return;
        int64_t const i_frame = (at_turn - m.start_at_turn) / m.repetition_period;
        if (i_frame < m.n_repetitions && at_turn >= m.start_at_turn + i_frame * m.repetition_period &&
            at_turn < m.stop_at_turn + i_frame * m.repetition_period && pid < m.part_id_end &&
            pid >= m.part_id_start) {
            int64_t const store_at = n_turns_record * (m.part_id_end - m.part_id_start) * i_frame +
                                     n_turns_record * (pid - m.part_id_start) +
                                     (at_turn - i_frame * m.repetition_period) - m.start_at_turn;
            if (store_at >= 0 && store_at < m.n_records) monitor_store(kp, p, i, store_at);
        }
    }
}

// Applies one packed record; returns whether the global aperture applies.
template <bool kExact>
__device__ __forceinline__ bool apply_record(PState& p, const unsigned char* __restrict__ rec,
                                             const KParams& kp, const RfCtx& rf) {
    const RecHeader& h = *reinterpret_cast<const RecHeader*>(rec);
    switch (h.op) {
    case OP_DRIFT: {
        const DriftRec& r = *reinterpret_cast<const DriftRec*>(rec);
        if (r.exact) drift_exact<kExact>(p, r.length);
        else drift_expanded<kExact>(p, r.length);
        break;
    }
    case OP_MAGNET: {
        const MagnetRec& r = *reinterpret_cast<const MagnetRec*>(rec);
        const double* coefs = reinterpret_cast<const double*>(rec + sizeof(MagnetRec));
        magnet_edge(p, r.edge_entry, false, r.entry_r21, r.entry_r43);
        if (r.body_active) magnet_body<kExact>(p, r, coefs);
        magnet_edge(p, r.edge_exit, true, r.exit_r21, r.exit_r43);
        break;
    }
    case OP_CAVITY: {
        const CavityRec& r = *reinterpret_cast<const CavityRec*>(rec);
        p = cavity_cold<kExact>(p, r, rf);
        break;
    }
    case OP_LIMIT_ELLIPSE: {
        // limitellipse.h:12-38
        if (!flag_on(kp.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE)) {
            const LimitEllipseRec& r = *reinterpret_cast<const LimitEllipseRec*>(rec);
            double const temp = p.x * p.x * r.b_squ + p.y * p.y * r.a_squ;
            if (!(temp <= r.a_b_squ)) p.state = 0;
        }
        break;
    }
    case OP_LIMIT_RECT: {
        // limitrect.h:9-36
        if (!flag_on(kp.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE)) {
            const LimitRectRec& r = *reinterpret_cast<const LimitRectRec*>(rec);
            bool const alive = (p.x >= r.min_x) && (p.x <= r.max_x) && (p.y >= r.min_y) && (p.y <= r.max_y);
            if (!alive) p.state = 0;
        }
        break;
    }
    default:
        break;
    }
    return (h.flags & F_GLOBAL_APER) != 0;
}

template <bool kExact>
__global__ void __launch_bounds__(256) track_kernel(const KParams kp) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.capacity) return;
    const xtg_particles& P = kp.P;
    int64_t const state0 = P.state[i];
    if (state0 <= 0) return;   // inactive: the reference leaves it unchanged

    PState p;
    p.x = P.x[i]; p.px = P.px[i]; p.y = P.y[i]; p.py = P.py[i];
    p.zeta = P.zeta[i]; p.delta = P.delta[i]; p.ptau = P.ptau[i];
    p.rpp = P.rpp[i]; p.rvv = P.rvv[i]; p.s = P.s[i];
    p.chi = P.chi[i]; p.charge_ratio = P.charge_ratio[i];
    p.beta0 = P.beta0[i]; p.p0c = P.p0c[i];
    p.ax = P.ax ? P.ax[i] : 0.;
    p.ay = P.ay ? P.ay[i] : 0.;
    p.state = state0;
    p.at_element = P.at_element[i];
    p.at_turn = P.at_turn[i];
    refresh_energy_cache(p);
    int64_t const pid = (kp.flag_monitor != 0) ? P.particle_id[i] : 0;

    RfCtx rf;
    rf.q0 = P.q0;
    rf.t_sim = P.t_sim;
    rf.line_length = kp.line_length;
    rf.kill = flag_on(kp.track_flags, XTG_FLAG_KILL_CAVITY_KICK);
    rf.preserve_angle = kp.preserve_angle != 0;
    bool const ignore_global = flag_on(kp.track_flags, XTG_FLAG_IGNORE_GLOBAL_APERTURE) || !kp.has_global;
    double const lim = kp.global_lim;
    int64_t const incr = kp.backtrack ? -1 : 1;

    bool active = true;
    for (int32_t iturn = 0; iturn < kp.num_turns && active; iturn++) {
        if (kp.backtrack) {
            if (kp.flag_end_turn_actions > 0) {
                // local_particle_custom_api.h:79-94
                p.at_turn -= 1;
                p.at_element = kp.num_ele_line;
                if (kp.flag_reset_s > 0) p.s = kp.line_length;
            }
        } else if (kp.flag_monitor == 1) {
            monitor(kp, p, i, pid);
        }
        const unsigned char* __restrict__ rec = kp.table + kp.rec_begin;
        for (int32_t e = 0; e < kp.rec_count; e++) {
            if (kp.flag_monitor == 2) monitor(kp, p, i, pid);
            bool const thick = apply_record<kExact>(p, rec, kp, rf);
            if (thick && !ignore_global) {
                // local_particle_custom_api.h:259-287
                bool const within = (p.x >= -lim) && (p.x <= lim) && (p.y >= -lim) && (p.y <= lim);
                if (p.state > 0 && !within) p.state = -1;
            }
            if (p.state <= 0) {
                active = false;
                break;
            }
            p.at_element += incr;
            rec += reinterpret_cast<const RecHeader*>(rec)->nbytes;
        }
        if (kp.flag_monitor == 2) monitor(kp, p, i, pid);
        if (kp.backtrack) {
            if (kp.flag_monitor == 1) monitor(kp, p, i, pid);
        } else if (kp.flag_end_turn_actions > 0 && active) {
            // local_particle_custom_api.h:67-76
            p.at_turn += 1;
            p.at_element = 0;
            if (kp.flag_reset_s > 0) p.s = 0.;
        }
    }

    P.x[i] = p.x; P.px[i] = p.px; P.y[i] = p.y; P.py[i] = p.py;
    P.zeta[i] = p.zeta; P.delta[i] = p.delta; P.ptau[i] = p.ptau;
    P.rpp[i] = p.rpp; P.rvv[i] = p.rvv; P.s[i] = p.s;
    if (P.ax) P.ax[i] = p.ax;
    if (P.ay) P.ay[i] = p.ay;
    P.state[i] = p.state;
    P.at_element[i] = p.at_element;
    P.at_turn[i] = p.at_turn;
}

// ---------------------------------------------------------------------------
// FP64 peak probe: independent DFMA chains; each thread writes one value.
// ---------------------------------------------------------------------------
__global__ void dfma_probe_kernel(double* out, int iters, double a, double b) {
    double r[8];
#pragma unroll
    for (int c = 0; c < 8; c++) r[c] = threadIdx.x * 1e-3 + c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < 8; c++) r[c] = fma(r[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += r[c];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
extern "C" {

int32_t xtg_abi_version(void) { return XTG_ABI_VERSION; }

int32_t xtg_get_last_error(char* buf, int64_t n) {
    if (!buf || n <= 0) return XTG_E_NULL;
    snprintf(buf, (size_t)n, "%s", g_last_error.c_str());
    return XTG_OK;
}

int64_t xtg_launch_count(void) { return g_launch_count.load(); }

int32_t xtg_lattice_create(const xtg_element* elements, int64_t n_elements, const xtg_config* config,
                           xtg_lattice** out) {
    if (!out || !config) return set_error(XTG_E_NULL, "xtg_lattice_create: NULL argument");
    *out = nullptr;
    if (n_elements < 0) return set_error(XTG_E_VALUE, "xtg_lattice_create: n_elements < 0");
    if (n_elements > 0 && !elements) return set_error(XTG_E_NULL, "xtg_lattice_create: elements is NULL");
    if (n_elements > (int64_t)INT32_MAX) return set_error(XTG_E_CAPACITY, "too many elements");
    if (config->arith != XTG_ARITH_EXACT && config->arith != XTG_ARITH_FAST)
        return set_error(XTG_E_VALUE, "xtg_config.arith must be XTG_ARITH_EXACT or XTG_ARITH_FAST");
    std::unique_ptr<xtg_lattice> L(new xtg_lattice());
    L->elements.assign(elements, elements + n_elements);
    L->config = *config;
    // validate and pack before touching the device, so that an unsupported
    // element is reported as such on any host
    PackedLattice pl;
    std::string err;
    int32_t st = pack_lattice(L->elements.data(), n_elements, L->config, false, &pl, &err);
    if (st != XTG_OK) return set_error(st, "%s", err.c_str());
    XTG_CUDA_CHECK(cudaGetDevice(&L->device));
    st = upload_table(pl, &L->fwd);
    if (st != XTG_OK) {
        free_table(&L->fwd);
        return st;
    }
    *out = L.release();
    return XTG_OK;
}

int32_t xtg_lattice_destroy(xtg_lattice* lattice) {
    if (!lattice) return XTG_OK;
    free_table(&lattice->fwd);
    free_table(&lattice->bwd);
    delete lattice;
    return XTG_OK;
}

int32_t xtg_lattice_info(const xtg_lattice* L, int64_t* n_elements, int64_t ele_start, int64_t num_ele,
                         double* flops_per_particle) {
    if (!L) return set_error(XTG_E_NULL, "xtg_lattice_info: NULL lattice");
    int64_t const n = (int64_t)L->elements.size();
    if (n_elements) *n_elements = n;
    if (flops_per_particle) {
        if (ele_start < 0 || num_ele < 0 || ele_start + num_ele > n)
            return set_error(XTG_E_VALUE, "xtg_lattice_info: element range out of bounds");
        double f = 0;
        for (int64_t k = ele_start; k < ele_start + num_ele; k++) f += L->fwd.flops[k];
        *flops_per_particle = f;
    }
    return XTG_OK;
}

int32_t xtg_set_launch_config(xtg_lattice* L, int32_t block_size, int32_t compact_every, int32_t* out_bs,
                              int32_t* out_ce) {
    if (!L) return set_error(XTG_E_NULL, "xtg_set_launch_config: NULL lattice");
    if (block_size != 0) {
        if (block_size < 32 || block_size > 256 || block_size % 32)
            return set_error(XTG_E_VALUE, "block_size must be a multiple of 32 in [32, 256]");
        L->block_size = block_size;
    }
    if (compact_every < 0) return set_error(XTG_E_VALUE, "compact_every must be >= 0");
    if (compact_every > 0) L->compact_every = compact_every;
    if (out_bs) *out_bs = L->block_size;
    if (out_ce) *out_ce = L->compact_every;
    return XTG_OK;
}

int32_t xtg_sync(void* stream) {
    XTG_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
    return XTG_OK;
}

static bool particles_complete(const xtg_particles* P) {
    return P->x && P->px && P->y && P->py && P->zeta && P->delta && P->ptau && P->rpp && P->rvv && P->s &&
           P->chi && P->charge_ratio && P->beta0 && P->p0c && P->state && P->at_element && P->at_turn &&
           P->particle_id;
}

int32_t xtg_track(const xtg_lattice* lattice, const xtg_particles* particles, int32_t num_turns,
                  int32_t ele_start, int32_t num_ele_track, int32_t flag_end_turn_actions,
                  int32_t flag_reset_s_at_end_turn, int32_t flag_monitor, int32_t num_ele_line,
                  double line_length, const xtg_monitor* monitor, uint64_t track_flags, void* stream) {
    if (!lattice || !particles) return set_error(XTG_E_NULL, "xtg_track: NULL lattice or particles");
    xtg_lattice* L = const_cast<xtg_lattice*>(lattice);
    if (!particles_complete(particles)) return set_error(XTG_E_NULL, "xtg_track: a required particle array is NULL");
    int64_t const n = (int64_t)L->elements.size();
    if (num_turns < 0) return set_error(XTG_E_VALUE, "xtg_track: num_turns < 0");
    if (ele_start < 0 || num_ele_track < 0 || (int64_t)ele_start + num_ele_track > n)
        return set_error(XTG_E_VALUE, "xtg_track: element range [%d, %d+%d) outside [0, %lld)", ele_start,
                         ele_start, num_ele_track, (long long)n);
    if (flag_monitor < 0 || flag_monitor > 2) return set_error(XTG_E_VALUE, "xtg_track: flag_monitor must be 0, 1 or 2");
    if (flag_monitor != 0 && !monitor) return set_error(XTG_E_NULL, "xtg_track: flag_monitor set but monitor is NULL");
    if (monitor && flag_monitor != 0) {
        if (monitor->n_repetitions > 1 && monitor->repetition_period <= 0)
            return set_error(XTG_E_VALUE, "xtg_track: repetition_period must be > 0");
        if (monitor->n_records < 0) return set_error(XTG_E_VALUE, "xtg_track: monitor n_records < 0");
    }
    if (particles->capacity < 0) return set_error(XTG_E_VALUE, "xtg_track: capacity < 0");
    if (particles->capacity == 0 || num_turns == 0) return XTG_OK;

    int cur = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&cur));
    if (cur != L->device) return set_error(XTG_E_VALUE, "xtg_track: lattice was built on device %d, current is %d", L->device, cur);

    bool const backtrack = (track_flags >> XTG_FLAG_BACKTRACK) & 1u;
    const DevTable* T = &L->fwd;
    int64_t rec_first = ele_start;
    if (backtrack) {
        std::lock_guard<std::mutex> lock(L->mu);
        if (!L->has_bwd) {
            PackedLattice pl;
            std::string err;
            int32_t st = pack_lattice(L->elements.data(), n, L->config, true, &pl, &err);
            if (st != XTG_OK) return set_error(st, "%s", err.c_str());
            st = upload_table(pl, &L->bwd);
            if (st != XTG_OK) return st;
            L->has_bwd = true;
        }
        T = &L->bwd;
        // reference order ele_stop-1 .. ele_start == reversed-table records
        rec_first = n - ((int64_t)ele_start + num_ele_track);
    }

    KParams kp;
    memset(&kp, 0, sizeof(kp));
    kp.table = T->d_bytes;
    kp.rec_begin = T->h_offsets[rec_first];
    kp.rec_count = num_ele_track;
    kp.capacity = particles->capacity;
    kp.P = *particles;
    if (monitor) kp.M = *monitor;
    kp.flag_monitor = flag_monitor;
    kp.flag_end_turn_actions = flag_end_turn_actions;
    kp.flag_reset_s = flag_reset_s_at_end_turn;
    kp.backtrack = backtrack ? 1 : 0;
    kp.num_ele_line = num_ele_line;
    kp.line_length = line_length;
    kp.track_flags = track_flags;
    kp.has_global = L->config.has_global_xy_limit;
    kp.preserve_angle = L->config.cavity_preserve_angle;
    kp.global_lim = L->config.global_xy_limit;

    cudaStream_t s = (cudaStream_t)stream;
    int const bs = L->block_size;
    int64_t const grid64 = (kp.capacity + bs - 1) / bs;
    if (grid64 > INT32_MAX) return set_error(XTG_E_CAPACITY, "xtg_track: too many particles");
    dim3 grid((unsigned)grid64), block(bs);
    int32_t const per_launch = L->compact_every > 0 ? L->compact_every : num_turns;
    for (int32_t t = 0; t < num_turns; t += per_launch) {
        kp.num_turns = (num_turns - t) < per_launch ? (num_turns - t) : per_launch;
        if (L->config.arith == XTG_ARITH_EXACT) track_kernel<true><<<grid, block, 0, s>>>(kp);
        else track_kernel<false><<<grid, block, 0, s>>>(kp);
        g_launch_count.fetch_add(1);
        XTG_CUDA_CHECK(cudaGetLastError());
    }
    return XTG_OK;
}

int32_t xtg_measure_fp64_peak(double* flops_per_s) {
    if (!flops_per_s) return set_error(XTG_E_NULL, "xtg_measure_fp64_peak: NULL output");
    int dev = 0, sms = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&dev));
    XTG_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int const block = 256, grid = sms * 8, iters = 8192;
    double* out = nullptr;
    XTG_CUDA_CHECK(cudaMalloc(&out, (size_t)grid * block * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        dfma_probe_kernel<<<grid, block>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return set_error(XTG_E_CUDA, "probe failed: %s", cudaGetErrorString(err));
    double const flops = 2.0 * 8.0 * (double)iters * (double)grid * block;
    *flops_per_s = flops / (best * 1e-3);
    return XTG_OK;
}

}  // extern "C"
