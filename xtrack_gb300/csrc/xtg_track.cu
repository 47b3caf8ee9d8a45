// The GB300 push: kernels, launch logic and the C-ABI entry points of
// include/xtrack_gb300.h.
//
// Replaces xtrack's generated `track_line` kernel (xtrack/tracker.py:
// 543-750). The reference launches one thread per particle slot and lets a
// lost particle's thread idle for the rest of the launch; it reads every
// element through a table of references in global memory. Here:
//
//  * rounds: a call is split into rounds of `compact_every` turns. Before
//    each round, a compaction kernel (warp ballot + prefix sum, grouped by
//    lattice with match_any) lists the particles still alive, and a queue
//    kernel cuts that list into work items of one block each;
//  * a persistent kernel pulls work items from the device queue; block b
//    takes item b first (blocks are dispatched breadth-first over the SMs,
//    so a round with fewer items than resident blocks spreads evenly and no
//    FP64 pipe carries two warps while another idles), later items come
//    from an atomic counter. Each thread owns one particle, keeps its
//    coordinates in registers for the whole round and walks the packed
//    element table (xtg_table.h) with warp-uniform records and a
//    warp-uniform switch on the element type;
//  * FP64 is the narrow pipe of this part, so nothing that is not
//    arithmetic goes there: aperture and global-aperture tests compare
//    ordered integer keys of the IEEE bit patterns (ord_key), with the
//    FP64 compare's outcome for signed zeros and NaN;
//  * the element table is staged in shared memory: with one bulk copy per
//    lattice when the tracked range fits, otherwise streamed in chunks
//    through a double-buffered cp.async.bulk + mbarrier pipeline. Every wait
//    is bounded; on time-out the kernel records XTG_E_TIMEOUT and returns;
//  * several lattices (error seeds) share one launch: a work item belongs to
//    one lattice, named by the particles' lattice index;
//  * the rounds of a call can be replayed from a captured CUDA graph.
//
// Compiled with -fmad=false: the exact-arithmetic path must not have its
// products fused into additions. The fast path uses explicit fma().
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <deque>
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

#define XTG_CUDA_CHECK(call)                                                                 \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return set_error(XTG_E_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

// resident blocks of 256 threads per SM the fast push is compiled for (the
// register budget: 1 -> up to 255 registers, 2 -> 128)
#ifndef XTG_FAST_MIN_BLOCKS
#define XTG_FAST_MIN_BLOCKS 1
#endif
// largest block of the fast push the register budget is sized for: 384
// (168 registers: three 128-thread blocks, 12 warps per SM; 1.3 % faster on
// the thick ring than 8 warps) or 256 (214 registers, 8 warps per SM)
#ifndef XTG_FAST_LB_THREADS
#define XTG_FAST_LB_THREADS 384
#endif
// the same for the exact push: 512 (128 registers: four 128-thread blocks,
// 16 warps per SM; the integer-pipe multiplies are latency chains that need
// the warps: 394k particle-turns/s on the thick ring against 382k at 384
// and 328k at 256), 384 (168) or 256 (192)
#ifndef XTG_EXACT_LB_THREADS
#define XTG_EXACT_LB_THREADS 512
#endif

// largest staging chunk: two chunks plus the static shared memory of the
// push kernel stay within the 227 KB a block may use
static constexpr int32_t kMaxChunkBytes = 113 * 1024;

// Every record is read as at least kRecordHead bytes at once (the whole of
// the small records: drifts, apertures, linear dipole edges), so the device
// table and each shared-memory staging area end with kRecordSlack unused
// bytes that such a read of the last record may touch.
static constexpr int32_t kRecordHead = 48;
static constexpr int32_t kRecordSlack = 32;

// smallest block size of the push; the work-item buffers hold one item per
// kMinBlock particles plus one per lattice
static constexpr int32_t kMinBlock = 32;

// device error word values
#define XTG_DEV_ERR_TIMEOUT 1
#define XTG_DEV_ERR_LATTICE_INDEX 2
#define XTG_DEV_ERR_ITEMS 3

// The bit pattern of |limit| shifted left by one (the sign bit dropped) for
// the global-aperture test; a negative or NaN limit, for which |x| <= limit
// holds for no x, is flagged by global_none instead.
static uint64_t global_abs2(double limit) {
    if (!(limit >= 0.0)) return 0;
    uint64_t b;
    memcpy(&b, &limit, sizeof(b));
    return b << 1;
}

// ---------------------------------------------------------------------------
// kernel arguments
// ---------------------------------------------------------------------------
struct TrackArgs {
    const unsigned char* __restrict__ table;   // all lattices' records, concatenated
    const int64_t* __restrict__ lat_base;      // byte offset of each lattice's table
    const int64_t* __restrict__ rec_off;       // per lattice: n+1 record offsets
    const int32_t* __restrict__ chunk_end;     // per lattice: n+1 chunk ends (staging)
    int64_t stride;                            // n+1
    int32_t rec_first;                         // first record of the tracked range
    int32_t rec_count;                         // records per turn
    int32_t num_turns;                         // turns of this round
    int32_t chunk_bytes;                       // 0: read records from global memory
    int32_t smem_bytes;                        // dynamic shared memory of the block
    int32_t flag_monitor;
    int32_t load_pid;                          // a monitor needs particle_id
    int32_t flag_end_turn_actions;
    int32_t flag_reset_s;
    int32_t backtrack;
    int32_t has_global;
    int32_t preserve_angle;
    // global aperture |x|, |y| <= limit as ordered keys: lower_key(-limit), upper_key(limit)
    // |x|, |y| <= limit as one unsigned compare each of the bit patterns
    // shifted left by one (global_abs2); global_none: nothing passes
    uint64_t global_abs2;
    int32_t global_none;
    int32_t reserved_global;
    int64_t num_ele_line;
    double line_length;
    uint64_t track_flags;
    const int32_t* __restrict__ idx;           // active particle indices
    const int4* __restrict__ items;            // (lattice, start, count, -)
    const int32_t* n_items;
    int32_t* item_counter;
    int32_t* err;
    xtg_particles P;
    xtg_monitor M;
    xtg_multi_element_monitor E;               // E.data == NULL: none
};

__device__ __forceinline__ bool flag_on(uint64_t flags, int bit) { return (flags >> bit) & 1u; }

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier and 1-D bulk copies (the TMA engine), shared::cta
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait (about 2 s of SM clock): on time-out records the error word
// and returns false.
// about 2 s at the GB300's 2.07 GHz SM clock
static constexpr long long kWaitLimitCycles = 4000000000LL;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int32_t* err,
                                                  long long limit = kWaitLimitCycles) {
    if (mbar_try_wait(bar, parity)) return true;
    long long const t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) {
            atomicExch(err, XTG_DEV_ERR_TIMEOUT);
            return false;
        }
    }
    return true;
}

// After a timed-out wait: thread 0 waits (again bounded) for the bulk copies
// it issued that were not seen complete, so that no copy still writes into
// the block's shared memory when the block exits.
__device__ __forceinline__ void drain_copies(uint64_t* bars, const uint32_t* phase, uint32_t pending,
                                             int32_t* err) {
    for (int b = 0; b < 2; b++)
        if (pending & (1u << b)) (void)mbar_wait_bounded(&bars[b], phase[b], err);
}

// Copies `bytes` (multiple of 16, at most 1 MB, 16-byte aligned ends) into
// shared memory; the consumers wait on `bar`. Called by one thread.
__device__ __forceinline__ void issue_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    mbar_expect_tx(bar, bytes);
    bulk_copy_g2s(dst, src, bytes, bar);
}

// ---------------------------------------------------------------------------
// monitor (particles_monitor.h:12-77)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void monitor_store(const xtg_monitor& M, const xtg_particles& S, const PState& p,
                                              int64_t i, int64_t k) {
    const xtg_particles& D = M.data;
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

__device__ __forceinline__ void monitor_into(const xtg_monitor& m, const xtg_particles& S, const PState& p,
                                             int64_t i, int64_t pid, bool backtrack) {
    int64_t at_turn;
    if (m.ebe_mode) {
        at_turn = p.at_element;
    } else {
        if (backtrack) return;
        at_turn = p.at_turn;
    }
    int64_t const n_turns_record = m.stop_at_turn - m.start_at_turn;
    if (m.n_repetitions == 1) {
        if (at_turn >= m.start_at_turn && at_turn < m.stop_at_turn && pid < m.part_id_end &&
            pid >= m.part_id_start) {
            int64_t const store_at = n_turns_record * (pid - m.part_id_start) + at_turn - m.start_at_turn;
            if (store_at >= 0 && store_at < m.n_records) monitor_store(m, S, p, i, store_at);
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
            if (store_at >= 0 && store_at < m.n_records) monitor_store(m, S, p, i, store_at);
        }
    }
}

__device__ __forceinline__ void monitor(const TrackArgs& a, const PState& p, int64_t i, int64_t pid) {
    monitor_into(a.M, a.P, p, i, pid, a.backtrack != 0);
}

// LastTurnsMonitor in the line (last_turns_monitor.h:17-55): tracking of a
// particle stops at its loss, so every pass stores the slot offset and the
// last one stored is that of the last pass before the loss
__device__ __noinline__ void monitor_last_turns(const MonLastTurnsRec& r, const PState& p, int64_t pid) {
    int64_t const at_turn = p.at_turn;
    if (at_turn >= 0 && at_turn % r.every_n_turns == 0 && r.particle_id_start <= pid &&
        pid < r.particle_id_stop) {
        int64_t const offset = (at_turn / r.every_n_turns) % r.n_last_turns;
        int64_t const ip = pid - r.particle_id_start;
        int64_t const slot = r.n_last_turns * ip + offset;
        r.lost_at_offset[ip] = (uint32_t)offset;
        r.particle_id[slot] = (uint32_t)pid;
        r.at_turn[slot] = (uint32_t)at_turn;
        r.x[slot] = (float)p.x;
        r.px[slot] = (float)p.px;
        r.y[slot] = (float)p.y;
        r.py[slot] = (float)p.py;
        r.delta[slot] = (float)p.delta;
        r.zeta[slot] = (float)p.zeta;
    }
}

// BeamPositionMonitor in the line (beam_position_monitor.h:16-58)
__device__ __noinline__ void monitor_bpm(const MonBpmRec& r, const PState& p, int64_t pid) {
    if (r.particle_id_stop < 0 || (r.particle_id_start <= pid && pid < r.particle_id_stop)) {
        double const at_turn = (double)p.at_turn;
        int64_t const slot = (int64_t)round(
            r.sampling_frequency * ((at_turn - r.start_at_turn) / r.frev - p.zeta / p.beta0 / kCLightD));
        if (slot >= 0 && slot < r.n_slots) {
            atomicAdd(r.count + slot, 1.0);
            atomicAdd(r.x_sum + slot, p.x);
            atomicAdd(r.y_sum + slot, p.y);
            if (r.x2_sum) {
                // beam_size_monitor.h:16-64
                atomicAdd(r.x2_sum + slot, p.x * p.x);
                atomicAdd(r.y2_sum + slot, p.y * p.y);
            }
        }
    }
}

// BeamProfileMonitor in the line (beam_profile_monitor.h:16-80)
__device__ __noinline__ void monitor_profile(const MonProfileRec& r, const PState& p, int64_t pid) {
    if (r.particle_id_stop < 0 || (r.particle_id_start <= pid && pid < r.particle_id_stop)) {
        double const at_turn = (double)p.at_turn;
        int64_t const sample = (int64_t)round(
            r.sampling_frequency * ((at_turn - r.start_at_turn) / r.frev - p.zeta / p.beta0 / kCLightD));
        if (sample >= 0 && sample < r.sample_size) {
            int64_t const bin_x = (int64_t)floor((p.x - r.x_min) / r.dx);
            int64_t const bin_y = (int64_t)floor((p.y - r.y_min) / r.dy);
            if (bin_x >= 0 && bin_x < r.nx) atomicAdd(r.counts_x + sample * r.nx + bin_x, 1.);
            if (bin_y >= 0 && bin_y < r.ny) atomicAdd(r.counts_y + sample * r.ny + bin_y, 1.);
        }
    }
}

// ---------------------------------------------------------------------------
// one element record
// ---------------------------------------------------------------------------

// multi_element_monitor.h:10-65, before an element
__device__ __noinline__ void multi_element_monitor(const xtg_multi_element_monitor& E, const PState& p,
                                                   int64_t pid) {
    int64_t const at_turn = p.at_turn;
    if (at_turn >= E.start_at_turn && at_turn < E.stop_at_turn && pid >= E.part_id_start &&
        pid < E.part_id_end) {
        int64_t const at_element = p.at_element;
        int64_t store_at = -1;
        if (at_element >= 0 && at_element < E.mapping_len) store_at = E.at_element_mapping[at_element];
        if (store_at >= 0) {
            int64_t const n_part = E.part_id_end - E.part_id_start;
            int64_t const base =
                (((at_turn - E.start_at_turn) * n_part + (pid - E.part_id_start)) * 7) * E.n_obs + store_at;
            double const v[7] = {p.x, p.px, p.y, p.py, p.zeta, p.delta, p.s};
            for (int c = 0; c < 7; c++) E.data[base + (int64_t)c * E.n_obs] = v[c];
        }
    }
}
// limitpolygon.h:64-90: the crossing-number test with the inscribed-circle
// shortcut of the CPU build; out of line (polygons are rare in a turn)
__device__ __noinline__ bool polygon_alive(double x, double y, const unsigned char* __restrict__ rec) {
    const LimitPolygonRec& r = *reinterpret_cast<const LimitPolygonRec*>(rec);
    const double* vx = reinterpret_cast<const double*>(rec + sizeof(LimitPolygonRec));
    const double* vy = vx + r.n;
    if (!(x * x + y * y > r.inner_radius_sq)) return true;
    int64_t ii = 0, jj = r.n - 1;
    bool alive = false;
    while (ii < r.n) {
        double const vx_ii = vx[ii], vx_jj = vx[jj], vy_ii = vy[ii], vy_jj = vy[jj];
        if (((vy_ii > y) != (vy_jj > y)) && (x < (vx_jj - vx_ii) * (y - vy_ii) / (vy_jj - vy_ii) + vx_ii))
            alive = !alive;
        jj = ii;
        ii++;
    }
    return alive;
}

// track_srotation.h:9-37 (no spin)
__device__ __forceinline__ void s_rotation(PState& p, double sin_z, double cos_z) {
    double const x = p.x, y = p.y, px = p.px, py = p.py;
    p.x = cos_z * x + sin_z * y;
    p.y = -sin_z * x + cos_z * y;
    p.px = cos_z * px + sin_z * py;
    p.py = -sin_z * px + cos_z * py;
}
// Transverse shift and tilt of a record (F_SHIFTED, ApertureShift in
// xtg_table.h: apertures, thin Multipoles, DipoleEdges): the entry
// transform for the particle reaching the element, the exit transform only
// if it survives; both also when local apertures are ignored. The block is
// found again from the header at the exit, so that nothing stays live
// across the check. The transforms run out of line, so that the common
// untransformed record keeps a flag test only.
XTG_COLD PState aperture_transform_in(PState p, const ApertureShift* __restrict__ sh) {
    p.x = p.x + sh->in_x;
    p.y = p.y + sh->in_y;
    for (int k = 0; k < sh->n_rot_in; k++) s_rotation(p, sh->rot_in[k][0], sh->rot_in[k][1]);
    return p;
}
XTG_COLD PState aperture_transform_out(PState p, const ApertureShift* __restrict__ sh) {
    for (int k = 0; k < sh->n_rot_out; k++) s_rotation(p, sh->rot_out[k][0], sh->rot_out[k][1]);
    p.x = p.x + sh->out_x;
    p.y = p.y + sh->out_y;
    return p;
}
__device__ __forceinline__ void aperture_shift_in(PState& p, const unsigned char* rec, const RecHeader& h) {
    if (h.flags & F_SHIFTED)
        p = aperture_transform_in(p, reinterpret_cast<const ApertureShift*>(rec + h.nbytes - sizeof(ApertureShift)));
}
__device__ __forceinline__ void aperture_shift_out(PState& p, const unsigned char* rec, const RecHeader& h) {
    if ((h.flags & F_SHIFTED) && p.state > 0)
        p = aperture_transform_out(p, reinterpret_cast<const ApertureShift*>(rec + h.nbytes - sizeof(ApertureShift)));
}

// The first kRecordHead bytes of a record, read with three 16-byte loads
// issued together: the header and, for the small records, every field, so
// that their maps wait on one load latency instead of a header load
// followed by field loads.
union RecHead {
    uint4 w[3];
    RecHeader h;
    DriftRec drift;
    LimitRectRec rect;
    LimitEllipseRec ellipse;
    DipoleEdgeRec dedge;
};
static_assert(sizeof(RecHead) == kRecordHead, "record head");

__device__ __forceinline__ void load_head(RecHead& u, const unsigned char* rec) {
    const uint4* q = reinterpret_cast<const uint4*>(rec);
    u.w[0] = q[0];
    u.w[1] = q[1];
    u.w[2] = q[2];
}

template <bool kExact>
__device__ __forceinline__ bool apply_record(PState& p, const unsigned char* __restrict__ rec, const RecHead& u,
                                             const TrackArgs& a, const RfCtx& rf, int64_t i, int64_t pid) {
    const RecHeader& h = u.h;
    switch (h.op) {
    case OP_DRIFT: {
        const DriftRec& r = u.drift;
        if (r.exact) drift_exact<kExact>(p, r.length);
        else drift_expanded<kExact>(p, r.length);
        break;
    }
    case OP_KICK: {
        const KickRec& r = *reinterpret_cast<const KickRec*>(rec);
        aperture_shift_in(p, rec, h);
        apply_kick<kExact>(p, kick_args(r), reinterpret_cast<const double*>(rec + sizeof(KickRec)));
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_MAGNET: {
        const MagnetRec& r = *reinterpret_cast<const MagnetRec*>(rec);
        const double* coefs = reinterpret_cast<const double*>(rec + sizeof(MagnetRec));
        magnet_edge<kExact>(p, r.edge_entry, false, r.entry_r21, r.entry_r43, coefs + r.entry_fringe,
                    r.backtrack != 0);
        if (p.state <= 0) break;   // killed by a nonlinear edge while backtracking
        if (r.body_active) magnet_body<kExact>(p, r, coefs);
        magnet_edge<kExact>(p, r.edge_exit, true, r.exit_r21, r.exit_r43, coefs + r.exit_fringe,
                    r.backtrack != 0);
        break;
    }
    case OP_DIPOLE_EDGE: {
        // dipoleedge.h:14-71: the linear kick (track_dipole_edge_linear.h:
        // 29-37) or the full model, which kills when backtracking; neither
        // touches ax, ay
        const DipoleEdgeRec& r = u.dedge;
        aperture_shift_in(p, rec, h);
        if (r.model == 0) {
            edge_linear_kick<kExact>(p, r.r21, r.r43);
        } else {
            p = fringe_edge(p, reinterpret_cast<const double*>(rec + sizeof(DipoleEdgeRec)) + r.fringe,
                            r.backtrack != 0);
        }
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_CAVITY: {
        const CavityRec& r = *reinterpret_cast<const CavityRec*>(rec);
        p = cavity_cold<kExact>(p, r, rf);
        break;
    }
    case OP_LIMIT_ELLIPSE: {
        // limitellipse.h:12-38
        aperture_shift_in(p, rec, h);
        if (!flag_on(a.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE)) {
            const LimitEllipseRec& r = u.ellipse;
            double const temp = xmul(xmul(p.x, p.x), r.b_squ) + xmul(xmul(p.y, p.y), r.a_squ);
            int64_t const kt = ord_key(temp);
            if (!(kt >= lower_key(0.0) && kt <= r.key_a_b_squ)) p.state = 0;
        }
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_LIMIT_RECT_ELLIPSE: {
        // limitrectellipse.h:14-44: the sum of squares is formed for every
        // particle, then the rectangle and ellipse tests on ordered keys
        aperture_shift_in(p, rec, h);
        if (!flag_on(a.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE)) {
            const LimitRectEllipseRec& r = *reinterpret_cast<const LimitRectEllipseRec*>(rec);
            double const temp = xmul(xmul(p.x, p.x), r.b_squ) + xmul(xmul(p.y, p.y), r.a_squ);
            int64_t const kx = ord_key(p.x), ky = ord_key(p.y), kt = ord_key(temp);
            bool const alive = (kx <= r.key_max_x) && (kx >= r.key_min_x) && (ky <= r.key_max_y) &&
                               (ky >= r.key_min_y) && (kt >= lower_key(0.0)) && (kt <= r.key_a_b_squ);
            if (!alive) p.state = 0;
        }
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_LIMIT_RECT: {
        // limitrect.h:9-36
        aperture_shift_in(p, rec, h);
        if (!flag_on(a.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE)) {
            // the FP64 compares of the reference as integer compares of
            // ordered keys (ord_key, xtg_table.h): same outcome, NaN lost
            const LimitRectRec& r = u.rect;
            int64_t const kx = ord_key(p.x), ky = ord_key(p.y);
            bool const alive = (kx >= r.key_min_x) && (kx <= r.key_max_x) && (ky >= r.key_min_y) &&
                               (ky <= r.key_max_y);
            if (!alive) p.state = 0;
        }
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_LIMIT_POLYGON: {
        // limitpolygon.h:64-90 (crossing-number test)
        aperture_shift_in(p, rec, h);
        if (!flag_on(a.track_flags, XTG_FLAG_IGNORE_LOCAL_APERTURE) && !polygon_alive(p.x, p.y, rec))
            p.state = 0;
        aperture_shift_out(p, rec, h);
        break;
    }
    case OP_MON_PARTICLES: {
        const MonParticlesRec& r = *reinterpret_cast<const MonParticlesRec*>(rec);
        monitor_into(r.m, a.P, p, i, pid, a.backtrack != 0);
        break;
    }
    case OP_MON_LAST_TURNS:
        monitor_last_turns(*reinterpret_cast<const MonLastTurnsRec*>(rec), p, pid);
        break;
    case OP_MON_BPM:
        monitor_bpm(*reinterpret_cast<const MonBpmRec*>(rec), p, pid);
        break;
    case OP_MON_PROFILE:
        monitor_profile(*reinterpret_cast<const MonProfileRec*>(rec), p, pid);
        break;
    case OP_NOP:
        // a shifted or tilted element with no effect of its own (a thin
        // Multipole of zero strength, a suppressed DipoleEdge) still moves
        // the particle by the entry and exit transforms
        aperture_shift_in(p, rec, h);
        aperture_shift_out(p, rec, h);
        break;
    default:
        break;
    }
    return (h.flags & F_GLOBAL_APER) != 0;
}

// Walks records [rec, rec_end) for one particle; stops at a loss.
template <bool kExact>
__device__ __forceinline__ void walk(PState& p, bool& active, const unsigned char* rec,
                                     const unsigned char* rec_end, const TrackArgs& a, const RfCtx& rf,
                                     bool ignore_global, int64_t i, int64_t pid) {
    int64_t const incr = a.backtrack ? -1 : 1;
    while (active && rec < rec_end) {
        if (a.flag_monitor == 2) monitor(a, p, i, pid);
        if (a.E.data) multi_element_monitor(a.E, p, pid);
        RecHead u;
        load_head(u, rec);
        bool const thick = apply_record<kExact>(p, rec, u, a, rf, i, pid);
        if (thick && !ignore_global) {
            // local_particle_custom_api.h:259-287: |x| <= limit && |y| <= limit.
            // A double's bit pattern shifted left by one drops the sign and
            // orders as its absolute value (+-0 at 0, a NaN above +inf), so
            // each test is one unsigned integer compare, off the FP64 pipe.
            // (Masking the sign bit instead lets the compiler turn the mask
            // into an FP64 absolute value, which keeps a NaN's sign.)
            uint64_t const ax = emu_bits(p.x) << 1, ay = emu_bits(p.y) << 1;
            bool const within = !a.global_none && (ax <= a.global_abs2) && (ay <= a.global_abs2);
            if (p.state > 0 && !within) p.state = -1;
        }
        if (p.state <= 0) {
            active = false;
            break;
        }
        p.at_element += incr;
        rec += u.h.nbytes;
    }
}

__device__ __forceinline__ void begin_turn(const TrackArgs& a, PState& p, int64_t i, int64_t pid) {
    if (a.backtrack) {
        if (a.flag_end_turn_actions > 0) {
            // local_particle_custom_api.h:79-94
            p.at_turn -= 1;
            p.at_element = a.num_ele_line;
            if (a.flag_reset_s > 0) p.s = a.line_length;
        }
    } else if (a.flag_monitor == 1) {
        monitor(a, p, i, pid);
    }
}

__device__ __forceinline__ void end_turn(const TrackArgs& a, PState& p, bool active, int64_t i,
                                         int64_t pid) {
    if (a.flag_monitor == 2) monitor(a, p, i, pid);
    if (a.backtrack) {
        if (a.flag_monitor == 1) monitor(a, p, i, pid);
    } else if (a.flag_end_turn_actions > 0 && active) {
        // local_particle_custom_api.h:67-76
        p.at_turn += 1;
        p.at_element = 0;
        if (a.flag_reset_s > 0) p.s = 0.;
    }
}

// ---------------------------------------------------------------------------
// the persistent push kernel
// ---------------------------------------------------------------------------
template <bool kExact>
__global__ void __launch_bounds__(kExact ? XTG_EXACT_LB_THREADS : XTG_FAST_LB_THREADS, kExact ? 1 : XTG_FAST_MIN_BLOCKS)
    track_kernel(const TrackArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full_bar[2];
    __shared__ int s_item;
    __shared__ int s_abort;
    __shared__ int s_resident;       // lattice whose range is resident, or -1

    int const tid = threadIdx.x;
    bool const staged = a.chunk_bytes > 0;
    if (tid == 0) {
        mbar_init(&full_bar[0], 1);
        mbar_init(&full_bar[1], 1);
        mbar_fence_init();
        s_abort = 0;
        s_resident = -1;
    }
    __syncthreads();
    uint32_t phase[2] = {0u, 0u};   // parity of the next completion of each buffer
    uint32_t pending = 0u;          // thread 0: buffers with a copy in flight

    const xtg_particles& P = a.P;
    RfCtx rf;
    rf.q0 = P.q0;
    rf.t_sim = P.t_sim;
    rf.line_length = a.line_length;
    rf.kill = flag_on(a.track_flags, XTG_FLAG_KILL_CAVITY_KICK);
    rf.preserve_angle = a.preserve_angle != 0;
    bool const ignore_global = flag_on(a.track_flags, XTG_FLAG_IGNORE_GLOBAL_APERTURE) || !a.has_global;

    bool first = true;
    for (;;) {
        if (tid == 0) s_item = first ? (int)blockIdx.x : (int)gridDim.x + atomicAdd(a.item_counter, 1);
        first = false;
        __syncthreads();
        int const it = s_item;
        int const nit = *((volatile const int32_t*)a.n_items);
        __syncthreads();
        if (it >= nit) break;
        int4 const w = a.items[it];
        int const lat = w.x;

        // load the particle
        bool const have = tid < w.z;
        int64_t const i = have ? (int64_t)a.idx[w.y + tid] : 0;
        PState p;
        bool active = false;
        int64_t pid = 0;
        if (have) {
            p.state = P.state[i];
            active = p.state > 0;
        }
        if (active) {
            p.x = P.x[i]; p.px = P.px[i]; p.y = P.y[i]; p.py = P.py[i];
            p.zeta = P.zeta[i]; p.delta = P.delta[i]; p.ptau = P.ptau[i];
            p.rpp = P.rpp[i]; p.rvv = P.rvv[i]; p.s = P.s[i];
            p.chi = P.chi[i]; p.charge_ratio = P.charge_ratio[i];
            p.beta0 = P.beta0[i]; p.p0c = P.p0c[i];
            p.ax = P.ax ? P.ax[i] : 0.;
            p.ay = P.ay ? P.ay[i] : 0.;
            p.at_element = P.at_element[i];
            p.at_turn = P.at_turn[i];
            p.chi_one = (p.chi == 1.0);
            p.frozen = flag_on(a.track_flags, XTG_FLAG_FREEZE_LONGITUDINAL);
            refresh_energy_cache(p);
            if (a.load_pid) pid = P.particle_id[i];
        }
        bool const touched = active;

        const unsigned char* base = a.table + a.lat_base[lat];
        const int64_t* off = a.rec_off + (int64_t)lat * a.stride;
        int32_t const r0 = a.rec_first, r1 = a.rec_first + a.rec_count;
        int64_t const b0 = off[r0];
        int64_t const range_bytes = off[r1] - b0;
        bool const streamed = staged && range_bytes > a.smem_bytes;
        const int32_t* cend = a.chunk_end + (int64_t)lat * a.stride;
        unsigned char* const buf1 = smem + a.chunk_bytes;

        // where the records of a whole turn are read from when not streamed
        const unsigned char* whole = base + b0;
        if (staged && !streamed) {
            // resident: one bulk copy of the whole range, reused by every turn
            // and by every later work item of the same lattice
            if (s_resident != lat) {
                __syncthreads();   // no warp still reads the previous content
                if (tid == 0 && range_bytes > 0) {
                    issue_copy(smem, base + b0, (uint32_t)range_bytes, &full_bar[0]);
                    pending |= 1u;
                }
                if (range_bytes > 0) {
                    if (mbar_wait_bounded(&full_bar[0], phase[0], a.err)) {
                        phase[0] ^= 1u;
                        pending &= ~1u;
                    } else {
                        s_abort = 1;
                    }
                }
                __syncthreads();
                if (s_abort) {
                    if (tid == 0) drain_copies(full_bar, phase, pending, a.err);
                    return;
                }
                if (tid == 0) s_resident = lat;
            }
            whole = smem;
        }
        // producer cursor of the streamed pipeline (used by thread 0 only)
        int32_t pt = 0, pr = r0;
        if (streamed) {
            __syncthreads();   // no warp still reads a resident copy
            if (tid == 0) {
                s_resident = -1;
                for (int b = 0; b < 2 && pt < a.num_turns; b++) {
                    int32_t e = cend[pr];
                    if (e > r1) e = r1;
                    issue_copy(b ? buf1 : smem, base + off[pr], (uint32_t)(off[e] - off[pr]), &full_bar[b]);
                    pending |= 1u << b;
                    pr = e;
                    if (pr >= r1) {
                        pr = r0;
                        pt++;
                    }
                }
            }
        }
        int32_t k = 0;   // chunk counter of this item (streamed)
        for (int32_t t = 0; t < a.num_turns; t++) {
            // a block whose particles are all lost stops early, unless it
            // must keep the streamed pipeline in step
            if (!streamed && !__syncthreads_or(active)) break;
            bool const was_active = active;
            if (active) begin_turn(a, p, i, pid);
            int32_t cr = r0;
            while (cr < r1) {
                int32_t e = r1;
                const unsigned char* sb = whole;
                const unsigned char* se = whole + range_bytes;
                int b = 0;
                if (streamed) {
                    b = k & 1;
                    e = cend[cr];
                    if (e > r1) e = r1;
                    if (mbar_wait_bounded(&full_bar[b], phase[b], a.err)) {
                        phase[b] ^= 1u;
                        pending &= ~(1u << b);
                    } else {
                        s_abort = 1;
                    }
                    __syncthreads();
                    if (s_abort) {
                        if (tid == 0) drain_copies(full_bar, phase, pending, a.err);
                        return;
                    }
                    sb = b ? buf1 : smem;
                    se = sb + (off[e] - off[cr]);
                }
                if (active) walk<kExact>(p, active, sb, se, a, rf, ignore_global, i, pid);
                if (streamed) {
                    __syncthreads();   // buffer b consumed by every warp
                    if (tid == 0 && pt < a.num_turns) {
                        int32_t pe = cend[pr];
                        if (pe > r1) pe = r1;
                        issue_copy(b ? buf1 : smem, base + off[pr], (uint32_t)(off[pe] - off[pr]), &full_bar[b]);
                        pending |= 1u << b;
                        pr = pe;
                        if (pr >= r1) {
                            pr = r0;
                            pt++;
                        }
                    }
                    k++;
                }
                cr = e;
            }
            if (was_active) end_turn(a, p, active, i, pid);
        }

        // write back (inactive particles are left untouched, as in the reference)
        if (touched) {
            P.x[i] = p.x; P.px[i] = p.px; P.y[i] = p.y; P.py[i] = p.py;
            P.zeta[i] = p.zeta; P.delta[i] = p.delta; P.ptau[i] = p.ptau;
            P.rpp[i] = p.rpp; P.rvv[i] = p.rvv; P.s[i] = p.s;
            if (P.ax) P.ax[i] = p.ax;
            if (P.ay) P.ay[i] = p.ay;
            P.state[i] = p.state;
            P.at_element[i] = p.at_element;
            P.at_turn[i] = p.at_turn;
        }
    }
}

// ---------------------------------------------------------------------------
// compaction and work queue
// ---------------------------------------------------------------------------

// Per-lattice particle counts over all slots, so that the index list of
// lattice l lives in [lat_pbase[l], lat_pbase[l+1]).
__global__ void count_lattices_kernel(const int32_t* __restrict__ lat, int64_t n, int32_t n_lat,
                                      int32_t* lat_total, int32_t* err) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t const l = lat[i];
    if (l < 0 || l >= n_lat) {
        atomicExch(err, XTG_DEV_ERR_LATTICE_INDEX);   // the particle is not tracked
        return;
    }
    atomicAdd(&lat_total[l], 1);
}

__global__ void prefix_lattices_kernel(const int32_t* lat_total, int32_t n_lat, int64_t n,
                                       int64_t* lat_pbase, int32_t single) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (single) {
        lat_pbase[0] = 0;
        lat_pbase[1] = n;
        return;
    }
    int64_t acc = 0;
    for (int32_t l = 0; l < n_lat; l++) {
        lat_pbase[l] = acc;
        acc += lat_total[l];
    }
    lat_pbase[n_lat] = acc;
}

// Lists the alive particles of each lattice. Lanes are grouped by lattice
// (match_any); within a group a ballot gives each alive lane its rank (a
// prefix sum of the ballot) and one atomic per group reserves the slots.
__global__ void compact_kernel(const int64_t* __restrict__ state, const int32_t* __restrict__ lat,
                               int64_t n, int32_t n_lat, const int64_t* __restrict__ lat_pbase,
                               int32_t* lat_count, int32_t* __restrict__ idx) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int const lane = threadIdx.x & 31;
    bool const in = i < n;
    int32_t l = 0;
    if (in && lat) l = lat[i];
    bool const alive = in && state[i] > 0 && l >= 0 && l < n_lat;
    unsigned const alive_mask = __ballot_sync(0xffffffffu, alive);
    unsigned const group = __match_any_sync(0xffffffffu, alive ? l : -1) & alive_mask;
    int32_t base = 0;
    int const leader = alive ? (__ffs(group) - 1) : lane;
    if (alive && lane == leader) base = atomicAdd(&lat_count[l], __popc(group));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (alive) {
        int const rank = __popc(group & ((1u << lane) - 1u));
        idx[lat_pbase[l] + base + rank] = (int32_t)i;
    }
}

// threads of the one block of items_kernel
static constexpr int kItemsThreads = 1024;

// Cuts each lattice's list into items of at most `block` particles and
// resets the queue counter. A list that needs more than `items_cap` items
// writes none: the round tracks nothing and the error word says why.
__global__ void items_kernel(const int32_t* lat_count, const int64_t* lat_pbase, int32_t n_lat,
                             int32_t block, int4* items, int64_t items_cap, int32_t* n_items,
                             int32_t* item_counter, int32_t* err) {
    __shared__ int s_fits;
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        for (int32_t l = 0; l < n_lat; l++) acc += (lat_count[l] + block - 1) / block;
        s_fits = acc <= items_cap;
        *n_items = s_fits ? (int32_t)acc : 0;
        *item_counter = 0;
        if (!s_fits) atomicExch(err, XTG_DEV_ERR_ITEMS);
    }
    __syncthreads();
    if (!s_fits) return;
    // lattice by lattice, the block's threads write that lattice's items
    int32_t first = 0;
    for (int32_t l = 0; l < n_lat; l++) {
        int32_t const c = lat_count[l];
        int32_t const ni = (c + block - 1) / block;
        int64_t const pb = lat_pbase[l];
        for (int32_t j = threadIdx.x; j < ni; j += blockDim.x)
            items[first + j] = make_int4(l, (int32_t)(pb + (int64_t)j * block), min(block, c - j * block), 0);
        first += ni;
    }
}

// One wait of the push's kind on a barrier that nothing completes: thread
// 0 gives up after `limit` cycles and records the time-out in `err`.
__global__ void wait_check_kernel(int32_t* err, long long limit) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) (void)mbar_wait_bounded(&bar, 0u, err, limit);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// FP64 peak probe: independent DFMA chains; each thread writes one value.
// ---------------------------------------------------------------------------
// out[i] = a[i] * b[i] by the integer-pipe multiply (xtg_f64emu.cuh)
__global__ void f64_mul_kernel(const double* __restrict__ a, const double* __restrict__ b,
                               double* __restrict__ out, int64_t n) {
    int64_t const i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = emul(a[i], b[i]);
}

// independent chains of (integer-pipe multiply, FP64 add) pairs
__global__ void emul_probe_kernel(double* out, int iters, double m0, double m1, double d0) {
    double v[8];
    for (int c = 0; c < 8; c++) v[c] = 1.0 + 1e-3 * (threadIdx.x + c);
    for (int it = 0; it < iters; it++) {
        double const m = (it & 1) ? m1 : m0;
        double const d = (it & 1) ? -d0 : d0;
#pragma unroll
        for (int c = 0; c < 8; c++) v[c] = __dadd_rn(emul(v[c], m), d);
    }
    double s = 0;
    for (int c = 0; c < 8; c++) s += v[c];
    out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

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
// host side: device tables, workspace, execution context
// ---------------------------------------------------------------------------
struct DevTables {
    unsigned char* d_bytes = nullptr;
    int64_t* d_lat_base = nullptr;
    int64_t* d_rec_off = nullptr;
    int32_t* d_chunk_end = nullptr;
    int32_t chunk_bytes_built = -1;
    int32_t n_lat = 0;
    int64_t n_rec = 0;                         // records per lattice
    std::vector<int64_t> h_rec_off;            // n_lat * (n_rec + 1)
    int64_t max_record = 0;
    bool built = false;
};

static void free_tables(DevTables* t) {
    if (t->d_bytes) cudaFree(t->d_bytes);
    if (t->d_lat_base) cudaFree(t->d_lat_base);
    if (t->d_rec_off) cudaFree(t->d_rec_off);
    if (t->d_chunk_end) cudaFree(t->d_chunk_end);
    *t = DevTables();
}

struct Workspace {
    int64_t cap = 0;
    int32_t n_lat_cap = 0;
    int32_t* idx = nullptr;
    int32_t* lat_total = nullptr;
    int32_t* lat_count = nullptr;
    int64_t* lat_pbase = nullptr;
    int4* items = nullptr;
    int64_t items_cap = 0;
    int32_t* counters = nullptr;   // [0] n_items, [1] item_counter, [2] error word
};

static void free_ws(Workspace* w) {
    cudaFree(w->idx);
    cudaFree(w->lat_total);
    cudaFree(w->lat_count);
    cudaFree(w->lat_pbase);
    cudaFree(w->items);
    cudaFree(w->counters);
    *w = Workspace();
}

struct ExecCtx {
    std::vector<std::vector<xtg_element>> lattices;
    std::deque<xtg_element_monitor> monitors;  // owned copies of the monitor descriptors
    bool has_monitors = false;
    xtg_multi_element_monitor multi_mon;       // data == NULL: none
    xtg_config config;
    int device = 0;
    DevTables fwd, bwd;
    Workspace ws;
    xtg_tuning tune;
    std::vector<double> flops;                 // per element (first lattice)
    std::mutex mu;
    ExecCtx() {
        memset(&multi_mon, 0, sizeof(multi_mon));
        // three 128-thread blocks per SM (12 warps) with 2 x 32 KB chunks each
        tune.block_size = 128;
        tune.compact_every = 0;
        tune.chunk_bytes = 32768;
        tune.use_graph = 0;
    }
    ~ExecCtx() {
        free_tables(&fwd);
        free_tables(&bwd);
        free_ws(&ws);
    }
};

struct xtg_lattice {
    ExecCtx ctx;
};

struct xtg_batch {
    ExecCtx ctx;
};

// Copies the monitor descriptors the elements point at into the context,
// so that the tables can be packed again later (backtracking) without the
// caller's descriptors.
static void own_monitors(ExecCtx* C) {
    for (auto& els : C->lattices)
        for (auto& e : els)
            if (e.cls == XTG_CLS_MONITOR && e.aux) {
                C->monitors.push_back(*reinterpret_cast<const xtg_element_monitor*>(e.aux));
                e.aux = reinterpret_cast<uint64_t>(&C->monitors.back());
                C->has_monitors = true;
            }
}

static int32_t build_tables(ExecCtx* C, bool backtrack, DevTables* T) {
    std::vector<unsigned char> bytes;
    std::vector<int64_t> lat_base, rec_off;
    int64_t n = -1;
    int64_t max_rec = 0;
    for (size_t l = 0; l < C->lattices.size(); l++) {
        PackedLattice pl;
        std::string err;
        const auto& els = C->lattices[l];
        int32_t st = pack_lattice(els.data(), (int64_t)els.size(), C->config, backtrack, &pl, &err);
        if (st != XTG_OK) return set_error(st, "lattice %zu: %s", l, err.c_str());
        if (n < 0) {
            n = (int64_t)els.size();
            if (!backtrack) C->flops = pl.flops_fast;
        }
        lat_base.push_back((int64_t)bytes.size());
        bytes.insert(bytes.end(), pl.bytes.begin(), pl.bytes.end());
        rec_off.insert(rec_off.end(), pl.offsets.begin(), pl.offsets.end());
        for (int64_t r = 0; r < n; r++) max_rec = std::max(max_rec, pl.offsets[r + 1] - pl.offsets[r]);
    }
    free_tables(T);
    T->n_lat = (int32_t)C->lattices.size();
    T->n_rec = n;
    T->h_rec_off = rec_off;
    T->max_record = max_rec;
    size_t const nb = (bytes.empty() ? 16 : bytes.size()) + kRecordSlack;
    XTG_CUDA_CHECK(cudaMalloc(&T->d_bytes, nb));
    XTG_CUDA_CHECK(cudaMemset(T->d_bytes, 0, nb));
    if (!bytes.empty()) XTG_CUDA_CHECK(cudaMemcpy(T->d_bytes, bytes.data(), bytes.size(), cudaMemcpyHostToDevice));
    XTG_CUDA_CHECK(cudaMalloc(&T->d_lat_base, lat_base.size() * sizeof(int64_t)));
    XTG_CUDA_CHECK(cudaMemcpy(T->d_lat_base, lat_base.data(), lat_base.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice));
    XTG_CUDA_CHECK(cudaMalloc(&T->d_rec_off, rec_off.size() * sizeof(int64_t)));
    XTG_CUDA_CHECK(cudaMemcpy(T->d_rec_off, rec_off.data(), rec_off.size() * sizeof(int64_t),
                              cudaMemcpyHostToDevice));
    T->built = true;
    T->chunk_bytes_built = -1;
    return XTG_OK;
}

// chunk_end[r]: the largest r' > r with off[r'] - off[r] <= chunk (records
// are never split; every record fits in a chunk, checked by the caller).
static int32_t build_chunks(DevTables* T, int32_t chunk) {
    if (T->chunk_bytes_built == chunk) return XTG_OK;
    int64_t const stride = T->n_rec + 1;
    std::vector<int32_t> ce((size_t)(stride * T->n_lat));
    for (int32_t l = 0; l < T->n_lat; l++) {
        const int64_t* off = T->h_rec_off.data() + l * stride;
        int64_t e = 0;
        for (int64_t r = 0; r <= T->n_rec; r++) {
            if (r == T->n_rec) {
                ce[l * stride + r] = (int32_t)T->n_rec;
                continue;
            }
            if (e < r + 1) e = r + 1;
            while (e < T->n_rec && off[e + 1] - off[r] <= chunk) e++;
            ce[l * stride + r] = (int32_t)e;
        }
    }
    if (T->d_chunk_end) cudaFree(T->d_chunk_end);
    T->d_chunk_end = nullptr;
    XTG_CUDA_CHECK(cudaMalloc(&T->d_chunk_end, ce.size() * sizeof(int32_t)));
    XTG_CUDA_CHECK(cudaMemcpy(T->d_chunk_end, ce.data(), ce.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    T->chunk_bytes_built = chunk;
    return XTG_OK;
}

static int32_t ensure_ws(Workspace* W, int64_t cap, int32_t n_lat) {
    if (cap > W->cap) {
        if (W->idx) cudaFree(W->idx);
        W->idx = nullptr;
        XTG_CUDA_CHECK(cudaMalloc(&W->idx, (size_t)std::max<int64_t>(cap, 1) * sizeof(int32_t)));
        W->cap = cap;
    }
    int64_t const items_needed = (cap + kMinBlock - 1) / kMinBlock + n_lat + 1;
    if (items_needed > W->items_cap) {
        if (W->items) cudaFree(W->items);
        W->items = nullptr;
        XTG_CUDA_CHECK(cudaMalloc(&W->items, (size_t)items_needed * sizeof(int4)));
        W->items_cap = items_needed;
    }
    if (n_lat > W->n_lat_cap) {
        cudaFree(W->lat_total);
        cudaFree(W->lat_count);
        cudaFree(W->lat_pbase);
        W->lat_total = W->lat_count = nullptr;
        W->lat_pbase = nullptr;
        XTG_CUDA_CHECK(cudaMalloc(&W->lat_total, n_lat * sizeof(int32_t)));
        XTG_CUDA_CHECK(cudaMalloc(&W->lat_count, n_lat * sizeof(int32_t)));
        XTG_CUDA_CHECK(cudaMalloc(&W->lat_pbase, (n_lat + 1) * sizeof(int64_t)));
        W->n_lat_cap = n_lat;
    }
    if (!W->counters) {
        XTG_CUDA_CHECK(cudaMalloc(&W->counters, 4 * sizeof(int32_t)));
        XTG_CUDA_CHECK(cudaMemset(W->counters, 0, 4 * sizeof(int32_t)));
    }
    return XTG_OK;
}

static bool particles_complete(const xtg_particles* P) {
    return P->x && P->px && P->y && P->py && P->zeta && P->delta && P->ptau && P->rpp && P->rvv && P->s &&
           P->chi && P->charge_ratio && P->beta0 && P->p0c && P->state && P->at_element && P->at_turn &&
           P->particle_id;
}

template <bool kExact>
static int32_t configure_kernel(int32_t smem) {
    static int32_t configured = -1;
    if (configured < smem) {
        XTG_CUDA_CHECK(cudaFuncSetAttribute(track_kernel<kExact>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            smem));
        configured = smem;
    }
    return XTG_OK;
}

template <bool kExact>
static int32_t persistent_grid(int32_t block, int32_t smem, int* grid) {
    int dev = 0, sms = 0, per_sm = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&dev));
    XTG_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    XTG_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, track_kernel<kExact>, block, smem));
    if (per_sm < 1)
        return set_error(XTG_E_VALUE, "block size %d with %d B of shared memory does not fit", block, smem);
    *grid = per_sm * sms;
    return XTG_OK;
}

// One round: compact the alive particles, build the work queue, push
// `a.num_turns` turns. All on `s`, no host synchronization.
template <bool kExact>
static int32_t launch_round(ExecCtx* C, const TrackArgs& a, const int32_t* lat, int64_t cap, int32_t block,
                            int grid, int32_t smem, cudaStream_t s) {
    Workspace& W = C->ws;
    int32_t const n_lat = C->fwd.n_lat;
    XTG_CUDA_CHECK(cudaMemsetAsync(W.lat_count, 0, n_lat * sizeof(int32_t), s));
    int64_t const cgrid = (cap + 255) / 256;
    compact_kernel<<<(unsigned)cgrid, 256, 0, s>>>(a.P.state, lat, cap, n_lat, W.lat_pbase, W.lat_count, W.idx);
    items_kernel<<<1, kItemsThreads, 0, s>>>(W.lat_count, W.lat_pbase, n_lat, block, W.items, W.items_cap, W.counters + 0,
                                   W.counters + 1, W.counters + 2);
    track_kernel<kExact><<<grid, block, smem, s>>>(a);
    g_launch_count.fetch_add(3);
    XTG_CUDA_CHECK(cudaGetLastError());
    return XTG_OK;
}

template <bool kExact>
static int32_t run_rounds(ExecCtx* C, TrackArgs a, const int32_t* lat, int64_t cap, int32_t num_turns,
                          cudaStream_t s) {
    int32_t const block = C->tune.block_size;
    int32_t smem = 0;
    if (a.chunk_bytes > 0) {
        // two staging buffers, then the slack of the record-head reads
        smem = 2 * a.chunk_bytes + kRecordSlack;
        int32_t st = configure_kernel<kExact>(smem);
        if (st != XTG_OK) return st;
    }
    a.smem_bytes = smem > 0 ? 2 * a.chunk_bytes : 0;
    int grid = 0;
    int32_t st = persistent_grid<kExact>(block, smem, &grid);
    if (st != XTG_OK) return st;
    int32_t const per = C->tune.compact_every > 0 ? std::min(C->tune.compact_every, num_turns) : num_turns;
    int32_t const full = num_turns / per;
    int32_t const rest = num_turns % per;
    a.num_turns = per;
    if (C->tune.use_graph && full > 1) {
        // capture one round on a side stream and replay it `full` times
        cudaStream_t cs = nullptr;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ex = nullptr;
        XTG_CUDA_CHECK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaError_t ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (ce != cudaSuccess) {
            cudaStreamDestroy(cs);
            return set_error(XTG_E_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
        }
        st = launch_round<kExact>(C, a, lat, cap, block, grid, smem, cs);
        ce = cudaStreamEndCapture(cs, &g);
        if (st == XTG_OK && ce == cudaSuccess) ce = cudaGraphInstantiate(&ex, g, 0);
        if (g) cudaGraphDestroy(g);
        if (st == XTG_OK && ce == cudaSuccess) {
            g_launch_count.fetch_sub(3);   // counted per replay below
            for (int32_t r = 0; r < full && ce == cudaSuccess; r++) {
                ce = cudaGraphLaunch(ex, s);
                g_launch_count.fetch_add(3);
            }
        }
        if (ex) cudaGraphExecDestroy(ex);
        cudaStreamDestroy(cs);
        if (st != XTG_OK) return st;
        if (ce != cudaSuccess) return set_error(XTG_E_CUDA, "graph replay failed: %s", cudaGetErrorString(ce));
    } else {
        for (int32_t r = 0; r < full; r++) {
            st = launch_round<kExact>(C, a, lat, cap, block, grid, smem, s);
            if (st != XTG_OK) return st;
        }
    }
    if (rest > 0) {
        a.num_turns = rest;
        st = launch_round<kExact>(C, a, lat, cap, block, grid, smem, s);
        if (st != XTG_OK) return st;
    }
    return XTG_OK;
}

static int32_t track_impl(ExecCtx* C, const xtg_particles* particles, const int32_t* lattice_index,
                          int32_t num_turns, int32_t ele_start, int32_t num_ele_track,
                          int32_t flag_end_turn_actions, int32_t flag_reset_s_at_end_turn,
                          int32_t flag_monitor, int32_t num_ele_line, double line_length,
                          const xtg_monitor* monitor, uint64_t track_flags, void* stream) {
    if (!particles) return set_error(XTG_E_NULL, "xtg_track: NULL particles");
    if (!particles_complete(particles)) return set_error(XTG_E_NULL, "xtg_track: a required particle array is NULL");
    int64_t const n = C->fwd.n_rec;
    if (num_turns < 0) return set_error(XTG_E_VALUE, "xtg_track: num_turns < 0");
    if (ele_start < 0 || num_ele_track < 0 || (int64_t)ele_start + num_ele_track > n)
        return set_error(XTG_E_VALUE, "xtg_track: element range [%d, %d+%d) outside [0, %lld)", ele_start,
                         ele_start, num_ele_track, (long long)n);
    if (flag_monitor < 0 || flag_monitor > 2)
        return set_error(XTG_E_VALUE, "xtg_track: flag_monitor must be 0, 1 or 2");
    if (flag_monitor != 0 && !monitor)
        return set_error(XTG_E_NULL, "xtg_track: flag_monitor set but monitor is NULL");
    if (monitor && flag_monitor != 0) {
        if (monitor->n_repetitions > 1 && monitor->repetition_period <= 0)
            return set_error(XTG_E_VALUE, "xtg_track: repetition_period must be > 0");
        if (monitor->n_records < 0) return set_error(XTG_E_VALUE, "xtg_track: monitor n_records < 0");
    }
    int64_t const cap = particles->capacity;
    if (cap < 0) return set_error(XTG_E_VALUE, "xtg_track: capacity < 0");
    if (cap > (int64_t)INT32_MAX - 1024) return set_error(XTG_E_CAPACITY, "xtg_track: capacity above 2^31");
    if (cap == 0 || num_turns == 0) return XTG_OK;
    int cur = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&cur));
    if (cur != C->device)
        return set_error(XTG_E_VALUE, "xtg_track: tables were built on device %d, current is %d", C->device, cur);

    std::lock_guard<std::mutex> lock(C->mu);
    bool const backtrack = (track_flags >> XTG_FLAG_BACKTRACK) & 1u;
    DevTables* T = &C->fwd;
    int32_t rec_first = ele_start;
    if (backtrack) {
        if (!C->bwd.built) {
            int32_t st = build_tables(C, true, &C->bwd);
            if (st != XTG_OK) return st;
        }
        T = &C->bwd;
        rec_first = (int32_t)(n - ((int64_t)ele_start + num_ele_track));
    }
    // a chunk holds at least the largest record (records are never split)
    int32_t chunk = C->tune.chunk_bytes;
    if (chunk > 0) {
        if (T->max_record > chunk) chunk = (int32_t)((T->max_record + 15) / 16 * 16);
        if (chunk > kMaxChunkBytes)
            return set_error(XTG_E_CAPACITY, "an element record (%lld B) exceeds the staging limit (%d B)",
                             (long long)T->max_record, kMaxChunkBytes);
        int32_t st = build_chunks(T, chunk);
        if (st != XTG_OK) return st;
    }
    int32_t const n_lat = T->n_lat;
    int32_t st = ensure_ws(&C->ws, cap, n_lat);
    if (st != XTG_OK) return st;
    Workspace& W = C->ws;
    cudaStream_t s = (cudaStream_t)stream;

    // per-lattice regions of the index list
    const int32_t* lat = (lattice_index && n_lat > 1) ? lattice_index : nullptr;
    if (lat) {
        XTG_CUDA_CHECK(cudaMemsetAsync(W.lat_total, 0, n_lat * sizeof(int32_t), s));
        count_lattices_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, s>>>(lat, cap, n_lat, W.lat_total,
                                                                              W.counters + 2);
        prefix_lattices_kernel<<<1, 32, 0, s>>>(W.lat_total, n_lat, cap, W.lat_pbase, 0);
        g_launch_count.fetch_add(2);
    } else {
        prefix_lattices_kernel<<<1, 32, 0, s>>>(W.lat_total, 1, cap, W.lat_pbase, 1);
        g_launch_count.fetch_add(1);
    }
    XTG_CUDA_CHECK(cudaGetLastError());

    TrackArgs a;
    memset(&a, 0, sizeof(a));
    a.table = T->d_bytes;
    a.lat_base = T->d_lat_base;
    a.rec_off = T->d_rec_off;
    a.chunk_end = T->d_chunk_end;
    a.stride = T->n_rec + 1;
    a.rec_first = rec_first;
    a.rec_count = num_ele_track;
    a.chunk_bytes = chunk;
    a.flag_monitor = flag_monitor;
    a.load_pid = (flag_monitor != 0 || C->has_monitors || C->multi_mon.data) ? 1 : 0;
    a.E = C->multi_mon;
    a.flag_end_turn_actions = flag_end_turn_actions;
    a.flag_reset_s = flag_reset_s_at_end_turn;
    a.backtrack = backtrack ? 1 : 0;
    a.has_global = C->config.has_global_xy_limit;
    a.preserve_angle = C->config.cavity_preserve_angle;
    a.global_abs2 = global_abs2(C->config.global_xy_limit);
    a.global_none = !(C->config.global_xy_limit >= 0.0);
    a.num_ele_line = num_ele_line;
    a.line_length = line_length;
    a.track_flags = track_flags;
    a.idx = W.idx;
    a.items = W.items;
    a.n_items = W.counters + 0;
    a.item_counter = W.counters + 1;
    a.err = W.counters + 2;
    a.P = *particles;
    if (monitor) a.M = *monitor;

    if (C->config.arith == XTG_ARITH_EXACT) return run_rounds<true>(C, a, lat, cap, num_turns, s);
    return run_rounds<false>(C, a, lat, cap, num_turns, s);
}

// ---------------------------------------------------------------------------
// allocation-free push: the scratch of the rounds lives in one static device
// array instead of the lattice's workspace
// ---------------------------------------------------------------------------
// Layout (bytes from the 256-aligned start): active-particle index list,
// work items, counters {n_items, item_counter, error word, pad}, lattice
// count, lattice bases.
constexpr int64_t kNoAllocItems = XTG_NOALLOC_MAX_PARTICLES / kMinBlock + 2;
constexpr int64_t kNoAllocIdxOff = 0;
constexpr int64_t kNoAllocItemsOff = kNoAllocIdxOff + XTG_NOALLOC_MAX_PARTICLES * 4;
constexpr int64_t kNoAllocCountersOff = kNoAllocItemsOff + kNoAllocItems * 16;
constexpr int64_t kNoAllocLatCountOff = kNoAllocCountersOff + 16;
constexpr int64_t kNoAllocLatBaseOff = kNoAllocLatCountOff + 16;
constexpr int64_t kNoAllocBytes = kNoAllocLatBaseOff + 16;
static_assert(kNoAllocItemsOff % 16 == 0 && kNoAllocLatBaseOff % 8 == 0, "scratch alignment");
// items_kernel cuts the list into blocks of at least kMinBlock particles:
// the item buffer always has room, so its overflow word is never set here
static_assert(kNoAllocItems >= (XTG_NOALLOC_MAX_PARTICLES + kMinBlock - 1) / kMinBlock + 1,
              "work items of the static scratch");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_addr[64] = {nullptr};

// Set-up, with the device current: the array's address is looked up on
// every call (no allocation; it changes only when the context is created
// anew, e.g. after cudaDeviceReset), and whenever it is new the error word
// is cleared (the rest is rewritten by every round before it is read).
static int32_t noalloc_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= 64) return set_error(XTG_E_VALUE, "xtg_track_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    void* p = nullptr;
    XTG_CUDA_CHECK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (g_noalloc_addr[dev] != (unsigned char*)p) {
        XTG_CUDA_CHECK(cudaMemset((unsigned char*)p + kNoAllocCountersOff, 0, 16));
        g_noalloc_addr[dev] = (unsigned char*)p;
    }
    *out = g_noalloc_addr[dev];
    return XTG_OK;
}

// The device error word of the allocation-free calls on the current device
// (0 when the path was never used there); read and cleared.
static int32_t read_noalloc_status() {
    int dev = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return XTG_OK;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) return XTG_OK;
    int32_t* word = reinterpret_cast<int32_t*>(g_noalloc_addr[dev] + kNoAllocCountersOff) + 2;
    int32_t h = 0;
    XTG_CUDA_CHECK(cudaDeviceSynchronize());
    XTG_CUDA_CHECK(cudaMemcpy(&h, word, sizeof(h), cudaMemcpyDeviceToHost));
    if (h == 0) return XTG_OK;
    XTG_CUDA_CHECK(cudaMemset(word, 0, sizeof(int32_t)));
    if (h == XTG_DEV_ERR_TIMEOUT) return set_error(XTG_E_TIMEOUT, "a bounded device wait timed out (xtg_track_noalloc)");
    if (h == XTG_DEV_ERR_ITEMS) return set_error(XTG_E_VALUE, "the work-item buffer is too small (xtg_track_noalloc)");
    return set_error(XTG_E_VALUE, "device error %d in xtg_track_noalloc", (int)h);
}

template <bool kExact>
static int32_t run_rounds_noalloc(unsigned char* scratch, TrackArgs a, int64_t cap, int32_t num_turns,
                                  int32_t block, int32_t compact_every, cudaStream_t s) {
    int32_t* idx = reinterpret_cast<int32_t*>(scratch + kNoAllocIdxOff);
    int4* items = reinterpret_cast<int4*>(scratch + kNoAllocItemsOff);
    int32_t* counters = reinterpret_cast<int32_t*>(scratch + kNoAllocCountersOff);
    int32_t* lat_count = reinterpret_cast<int32_t*>(scratch + kNoAllocLatCountOff);
    int64_t* lat_pbase = reinterpret_cast<int64_t*>(scratch + kNoAllocLatBaseOff);
    a.idx = idx;
    a.items = items;
    a.n_items = counters + 0;
    a.item_counter = counters + 1;
    a.err = counters + 2;
    a.chunk_bytes = 0;
    a.smem_bytes = 0;
    int grid = 0;
    int32_t st = persistent_grid<kExact>(block, 0, &grid);
    if (st != XTG_OK) return st;
    prefix_lattices_kernel<<<1, 32, 0, s>>>(lat_count, 1, cap, lat_pbase, 1);
    g_launch_count.fetch_add(1);
    int32_t const per = compact_every > 0 ? std::min(compact_every, num_turns) : num_turns;
    for (int32_t done = 0; done < num_turns; done += per) {
        a.num_turns = std::min(per, num_turns - done);
        // the lattice count must start at zero in every round
        XTG_CUDA_CHECK(cudaMemsetAsync(lat_count, 0, sizeof(int32_t), s));
        compact_kernel<<<(unsigned)((cap + 255) / 256), 256, 0, s>>>(a.P.state, nullptr, cap, 1, lat_pbase,
                                                                   lat_count, idx);
        items_kernel<<<1, kItemsThreads, 0, s>>>(lat_count, lat_pbase, 1, block, items, kNoAllocItems, counters + 0,
                                       counters + 1, counters + 2);
        track_kernel<kExact><<<grid, block, 0, s>>>(a);
        g_launch_count.fetch_add(3);
        XTG_CUDA_CHECK(cudaGetLastError());
    }
    return XTG_OK;
}

static int32_t read_device_status(const ExecCtx* C) {
    if (!C->ws.counters) return XTG_OK;
    int32_t h[4] = {0, 0, 0, 0};
    XTG_CUDA_CHECK(cudaDeviceSynchronize());
    XTG_CUDA_CHECK(cudaMemcpy(h, C->ws.counters, sizeof(h), cudaMemcpyDeviceToHost));
    if (h[2] != 0) XTG_CUDA_CHECK(cudaMemset(C->ws.counters + 2, 0, sizeof(int32_t)));
    if (h[2] == XTG_DEV_ERR_TIMEOUT) return set_error(XTG_E_TIMEOUT, "a bounded device wait timed out");
    if (h[2] == XTG_DEV_ERR_LATTICE_INDEX)
        return set_error(XTG_E_VALUE, "a particle has a lattice index outside the batch");
    if (h[2] == XTG_DEV_ERR_ITEMS) return set_error(XTG_E_VALUE, "the work-item buffer is too small");
    return XTG_OK;
}

static int32_t check_tuning(const xtg_tuning* t) {
    if (!(t->block_size == kMinBlock || t->block_size == 64 || t->block_size == 128 || t->block_size == 256))
        return set_error(XTG_E_VALUE, "block_size must be 32, 64, 128 or 256");
    if (t->compact_every < 0) return set_error(XTG_E_VALUE, "compact_every must be >= 0");
    if (t->chunk_bytes < 0 || t->chunk_bytes % 16 || t->chunk_bytes > kMaxChunkBytes)
        return set_error(XTG_E_VALUE, "chunk_bytes must be a multiple of 16 in [0, %d]", kMaxChunkBytes);
    return XTG_OK;
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

// launches of the other translation units of the library (not exported)
__attribute__((visibility("hidden"))) int64_t xtg_internal_launch_add(int64_t n) {
    return g_launch_count.fetch_add(n) + n;
}

int32_t xtg_lattice_create(const xtg_element* elements, int64_t n_elements, const xtg_config* config,
                           xtg_lattice** out) {
    if (!out || !config) return set_error(XTG_E_NULL, "xtg_lattice_create: NULL argument");
    *out = nullptr;
    if (n_elements < 0) return set_error(XTG_E_VALUE, "xtg_lattice_create: n_elements < 0");
    if (n_elements > 0 && !elements) return set_error(XTG_E_NULL, "xtg_lattice_create: elements is NULL");
    if (n_elements > (int64_t)INT32_MAX - 1) return set_error(XTG_E_CAPACITY, "too many elements");
    if (config->arith != XTG_ARITH_EXACT && config->arith != XTG_ARITH_FAST)
        return set_error(XTG_E_VALUE, "xtg_config.arith must be XTG_ARITH_EXACT or XTG_ARITH_FAST");
    // validate and pack before touching the device, so that an unsupported
    // element is reported as such on any host
    {
        PackedLattice pl;
        std::string err;
        int32_t st = pack_lattice(elements, n_elements, *config, false, &pl, &err);
        if (st != XTG_OK) return set_error(st, "%s", err.c_str());
    }
    std::unique_ptr<xtg_lattice> L(new xtg_lattice());
    L->ctx.lattices.emplace_back(elements, elements + n_elements);
    own_monitors(&L->ctx);
    L->ctx.config = *config;
    // the exact push runs four blocks per SM: 2 x 16 KB chunks each fit
    if (config->arith == XTG_ARITH_EXACT) L->ctx.tune.chunk_bytes = 16384;
    XTG_CUDA_CHECK(cudaGetDevice(&L->ctx.device));
    int32_t st = build_tables(&L->ctx, false, &L->ctx.fwd);
    if (st != XTG_OK) return st;
    *out = L.release();
    return XTG_OK;
}

int32_t xtg_lattice_destroy(xtg_lattice* lattice) {
    delete lattice;
    return XTG_OK;
}

int32_t xtg_lattice_info(const xtg_lattice* L, int64_t* n_elements, int64_t ele_start, int64_t num_ele,
                         double* flops_per_particle) {
    if (!L) return set_error(XTG_E_NULL, "xtg_lattice_info: NULL lattice");
    int64_t const n = L->ctx.fwd.n_rec;
    if (n_elements) *n_elements = n;
    if (flops_per_particle) {
        if (ele_start < 0 || num_ele < 0 || ele_start + num_ele > n)
            return set_error(XTG_E_VALUE, "xtg_lattice_info: element range out of bounds");
        double f = 0;
        for (int64_t k = ele_start; k < ele_start + num_ele; k++) f += L->ctx.flops[k];
        *flops_per_particle = f;
    }
    return XTG_OK;
}

int32_t xtg_set_multi_element_monitor(xtg_lattice* L, const xtg_multi_element_monitor* m) {
    if (!L) return set_error(XTG_E_NULL, "xtg_set_multi_element_monitor: NULL lattice");
    if (!m) {
        memset(&L->ctx.multi_mon, 0, sizeof(L->ctx.multi_mon));
        return XTG_OK;
    }
    if (!m->data || !m->at_element_mapping)
        return set_error(XTG_E_NULL, "xtg_set_multi_element_monitor: NULL buffer");
    if (m->mapping_len < 0 || m->n_obs < 1 || m->part_id_end < m->part_id_start ||
        m->stop_at_turn < m->start_at_turn)
        return set_error(XTG_E_VALUE, "xtg_set_multi_element_monitor: inconsistent sizes");
    L->ctx.multi_mon = *m;
    return XTG_OK;
}

int32_t xtg_get_tuning(const xtg_lattice* L, xtg_tuning* out) {
    if (!L || !out) return set_error(XTG_E_NULL, "xtg_get_tuning: NULL argument");
    *out = L->ctx.tune;
    return XTG_OK;
}

int32_t xtg_set_tuning(xtg_lattice* L, const xtg_tuning* t) {
    if (!L || !t) return set_error(XTG_E_NULL, "xtg_set_tuning: NULL argument");
    int32_t st = check_tuning(t);
    if (st != XTG_OK) return st;
    L->ctx.tune = *t;
    return XTG_OK;
}

int32_t xtg_device_status(const xtg_lattice* L) {
    if (!L) return set_error(XTG_E_NULL, "xtg_device_status: NULL lattice");
    int32_t const st = read_device_status(&L->ctx);
    int32_t const st_noalloc = read_noalloc_status();
    return st != XTG_OK ? st : st_noalloc;
}

int32_t xtg_sync(void* stream) {
    XTG_CUDA_CHECK(cudaStreamSynchronize((cudaStream_t)stream));
    return XTG_OK;
}

int32_t xtg_track(const xtg_lattice* lattice, const xtg_particles* particles, int32_t num_turns,
                  int32_t ele_start, int32_t num_ele_track, int32_t flag_end_turn_actions,
                  int32_t flag_reset_s_at_end_turn, int32_t flag_monitor, int32_t num_ele_line,
                  double line_length, const xtg_monitor* monitor, uint64_t track_flags, void* stream) {
    if (!lattice || !particles) return set_error(XTG_E_NULL, "xtg_track: NULL lattice or particles");
    ExecCtx* C = &const_cast<xtg_lattice*>(lattice)->ctx;
    return track_impl(C, particles, nullptr, num_turns, ele_start, num_ele_track, flag_end_turn_actions,
                      flag_reset_s_at_end_turn, flag_monitor, num_ele_line, line_length, monitor, track_flags,
                      stream);
}

int32_t xtg_track_noalloc(const xtg_lattice* lattice, const xtg_particles* particles, int32_t num_turns,
                          int32_t ele_start, int32_t num_ele_track, int32_t flag_end_turn_actions,
                          int32_t flag_reset_s_at_end_turn, int32_t flag_monitor, int32_t num_ele_line,
                          double line_length, const xtg_monitor* monitor, uint64_t track_flags, void* stream) {
    if (!lattice || !particles) return set_error(XTG_E_NULL, "xtg_track_noalloc: NULL lattice or particles");
    int64_t const cap = particles->capacity;
    if (cap < 0) return set_error(XTG_E_VALUE, "xtg_track_noalloc: capacity < 0");
    if (cap > XTG_NOALLOC_MAX_PARTICLES)
        return set_error(XTG_E_CAPACITY,
                         "xtg_track_noalloc: capacity %lld exceeds the static scratch limit of %d particles "
                         "(use xtg_track)",
                         (long long)cap, XTG_NOALLOC_MAX_PARTICLES);
    if (!particles_complete(particles))
        return set_error(XTG_E_NULL, "xtg_track_noalloc: a required particle array is NULL");
    ExecCtx* C = &const_cast<xtg_lattice*>(lattice)->ctx;
    int64_t const n = C->fwd.n_rec;
    if (num_turns < 0) return set_error(XTG_E_VALUE, "xtg_track_noalloc: num_turns < 0");
    if (ele_start < 0 || num_ele_track < 0 || (int64_t)ele_start + num_ele_track > n)
        return set_error(XTG_E_VALUE, "xtg_track_noalloc: element range [%d, %d+%d) outside [0, %lld)",
                         ele_start, ele_start, num_ele_track, (long long)n);
    if (flag_monitor < 0 || flag_monitor > 2)
        return set_error(XTG_E_VALUE, "xtg_track_noalloc: flag_monitor must be 0, 1 or 2");
    if (flag_monitor != 0 && !monitor)
        return set_error(XTG_E_NULL, "xtg_track_noalloc: flag_monitor set but monitor is NULL");
    if (monitor && flag_monitor != 0) {
        if (monitor->n_repetitions > 1 && monitor->repetition_period <= 0)
            return set_error(XTG_E_VALUE, "xtg_track_noalloc: repetition_period must be > 0");
        if (monitor->n_records < 0) return set_error(XTG_E_VALUE, "xtg_track_noalloc: monitor n_records < 0");
    }
    int cur = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&cur));
    if (cur != C->device)
        return set_error(XTG_E_VALUE, "xtg_track_noalloc: tables were built on device %d, current is %d",
                         C->device, cur);
    unsigned char* scratch = nullptr;
    int32_t st = noalloc_scratch(cur, &scratch);
    if (st != XTG_OK) return st;
    if (cap == 0 || num_turns == 0) return XTG_OK;

    std::lock_guard<std::mutex> lock(C->mu);
    bool const backtrack = (track_flags >> XTG_FLAG_BACKTRACK) & 1u;
    const DevTables* T = &C->fwd;
    int32_t rec_first = ele_start;
    if (backtrack) {
        if (!C->bwd.built)
            return set_error(XTG_E_VALUE,
                             "xtg_track_noalloc: the backtracking table of this lattice is not built "
                             "(one xtg_track call with backtracking builds it)");
        T = &C->bwd;
        rec_first = (int32_t)(n - ((int64_t)ele_start + num_ele_track));
    }
    TrackArgs a;
    memset(&a, 0, sizeof(a));
    a.table = T->d_bytes;
    a.lat_base = T->d_lat_base;
    a.rec_off = T->d_rec_off;
    a.chunk_end = nullptr;
    a.stride = T->n_rec + 1;
    a.rec_first = rec_first;
    a.rec_count = num_ele_track;
    a.flag_monitor = flag_monitor;
    a.load_pid = (flag_monitor != 0 || C->has_monitors || C->multi_mon.data) ? 1 : 0;
    a.E = C->multi_mon;
    a.flag_end_turn_actions = flag_end_turn_actions;
    a.flag_reset_s = flag_reset_s_at_end_turn;
    a.backtrack = backtrack ? 1 : 0;
    a.has_global = C->config.has_global_xy_limit;
    a.preserve_angle = C->config.cavity_preserve_angle;
    a.global_abs2 = global_abs2(C->config.global_xy_limit);
    a.global_none = !(C->config.global_xy_limit >= 0.0);
    a.num_ele_line = num_ele_line;
    a.line_length = line_length;
    a.track_flags = track_flags;
    a.P = *particles;
    if (monitor) a.M = *monitor;
    cudaStream_t s = (cudaStream_t)stream;
    if (C->config.arith == XTG_ARITH_EXACT)
        return run_rounds_noalloc<true>(scratch, a, cap, num_turns, C->tune.block_size, C->tune.compact_every, s);
    return run_rounds_noalloc<false>(scratch, a, cap, num_turns, C->tune.block_size, C->tune.compact_every, s);
}

int32_t xtg_batch_create(const xtg_lattice* const* lattices, int32_t n_lattices, xtg_batch** out) {
    if (!lattices || !out) return set_error(XTG_E_NULL, "xtg_batch_create: NULL argument");
    *out = nullptr;
    if (n_lattices < 1) return set_error(XTG_E_VALUE, "xtg_batch_create: no lattices");
    std::unique_ptr<xtg_batch> B(new xtg_batch());
    for (int32_t l = 0; l < n_lattices; l++) {
        if (!lattices[l]) return set_error(XTG_E_NULL, "xtg_batch_create: lattice %d is NULL", l);
        const ExecCtx& c = lattices[l]->ctx;
        if (l == 0) {
            B->ctx.config = c.config;
            B->ctx.device = c.device;
            B->ctx.tune = c.tune;
        } else {
            if (c.lattices[0].size() != B->ctx.lattices[0].size())
                return set_error(XTG_E_VALUE, "xtg_batch_create: lattice %d has %zu elements, lattice 0 %zu", l,
                                 c.lattices[0].size(), B->ctx.lattices[0].size());
            if (memcmp(&c.config, &B->ctx.config, sizeof(xtg_config)) != 0)
                return set_error(XTG_E_VALUE, "xtg_batch_create: lattice %d has a different config", l);
        }
        B->ctx.lattices.push_back(c.lattices[0]);
    }
    own_monitors(&B->ctx);
    int32_t st = build_tables(&B->ctx, false, &B->ctx.fwd);
    if (st != XTG_OK) return st;
    *out = B.release();
    return XTG_OK;
}

int32_t xtg_batch_destroy(xtg_batch* batch) {
    delete batch;
    return XTG_OK;
}

int32_t xtg_batch_get_tuning(const xtg_batch* B, xtg_tuning* out) {
    if (!B || !out) return set_error(XTG_E_NULL, "xtg_batch_get_tuning: NULL argument");
    *out = B->ctx.tune;
    return XTG_OK;
}

int32_t xtg_batch_set_tuning(xtg_batch* B, const xtg_tuning* t) {
    if (!B || !t) return set_error(XTG_E_NULL, "xtg_batch_set_tuning: NULL argument");
    int32_t st = check_tuning(t);
    if (st != XTG_OK) return st;
    B->ctx.tune = *t;
    return XTG_OK;
}

int32_t xtg_batch_device_status(const xtg_batch* B) {
    if (!B) return set_error(XTG_E_NULL, "xtg_batch_device_status: NULL batch");
    return read_device_status(&B->ctx);
}

int32_t xtg_track_batch(xtg_batch* batch, const xtg_particles* particles, const int32_t* lattice_index,
                        int32_t num_turns, int32_t ele_start, int32_t num_ele_track,
                        int32_t flag_end_turn_actions, int32_t flag_reset_s_at_end_turn, int32_t flag_monitor,
                        int32_t num_ele_line, double line_length, const xtg_monitor* monitor,
                        uint64_t track_flags, void* stream) {
    if (!batch || !particles) return set_error(XTG_E_NULL, "xtg_track_batch: NULL batch or particles");
    if (!lattice_index && batch->ctx.fwd.n_lat > 1)
        return set_error(XTG_E_NULL, "xtg_track_batch: lattice_index is required with several lattices");
    return track_impl(&batch->ctx, particles, lattice_index, num_turns, ele_start, num_ele_track,
                      flag_end_turn_actions, flag_reset_s_at_end_turn, flag_monitor, num_ele_line, line_length,
                      monitor, track_flags, stream);
}

int32_t xtg_check_bounded_wait(int64_t limit_cycles) {
    if (limit_cycles < 1 || limit_cycles > kWaitLimitCycles)
        return set_error(XTG_E_VALUE, "xtg_check_bounded_wait: limit must be in [1, %lld] cycles",
                         (long long)kWaitLimitCycles);
    int32_t* d_err = nullptr;
    XTG_CUDA_CHECK(cudaMalloc(&d_err, sizeof(int32_t)));
    int32_t h = 0;
    cudaError_t ce = cudaMemset(d_err, 0, sizeof(int32_t));
    if (ce == cudaSuccess) {
        wait_check_kernel<<<1, 32>>>(d_err, (long long)limit_cycles);
        g_launch_count.fetch_add(1);
        ce = cudaGetLastError();
    }
    if (ce == cudaSuccess) ce = cudaDeviceSynchronize();
    if (ce == cudaSuccess) ce = cudaMemcpy(&h, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_err);
    if (ce != cudaSuccess) return set_error(XTG_E_CUDA, "xtg_check_bounded_wait: %s", cudaGetErrorString(ce));
    if (h == XTG_DEV_ERR_TIMEOUT) return set_error(XTG_E_TIMEOUT, "a bounded device wait timed out");
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

int32_t xtg_f64_mul_host(const double* a, const double* b, double* out, int64_t n) {
    if (n < 0) return set_error(XTG_E_VALUE, "xtg_f64_mul_host: negative n");
    if (n > 0 && (!a || !b || !out)) return set_error(XTG_E_NULL, "xtg_f64_mul_host: NULL array");
    for (int64_t i = 0; i < n; i++) out[i] = emul(a[i], b[i]);
    return XTG_OK;
}

int32_t xtg_f64_mul_device(const double* a, const double* b, double* out, int64_t n, void* stream) {
    if (n < 0) return set_error(XTG_E_VALUE, "xtg_f64_mul_device: negative n");
    if (n == 0) return XTG_OK;
    if (!a || !b || !out) return set_error(XTG_E_NULL, "xtg_f64_mul_device: NULL array");
    int const block = 256;
    int64_t const grid = (n + block - 1) / block;
    if (grid > 0x7fffffffLL) return set_error(XTG_E_VALUE, "xtg_f64_mul_device: n too large");
    f64_mul_kernel<<<(unsigned)grid, block, 0, (cudaStream_t)stream>>>(a, b, out, n);
    g_launch_count++;
    XTG_CUDA_CHECK(cudaGetLastError());
    return XTG_OK;
}

int32_t xtg_measure_emul_rate(double* ops_per_s) {
    if (!ops_per_s) return set_error(XTG_E_NULL, "xtg_measure_emul_rate: NULL output");
    int dev = 0, sms = 0;
    XTG_CUDA_CHECK(cudaGetDevice(&dev));
    XTG_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int const block = 128, grid = sms * 4, iters = 2048;
    double* out = nullptr;
    XTG_CUDA_CHECK(cudaMalloc(&out, (size_t)grid * block * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        emul_probe_kernel<<<grid, block>>>(out, iters, 1.0000001, 0.9999999, 1e-3);
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
    *ops_per_s = 2.0 * 8.0 * (double)iters * (double)grid * block / (best * 1e-3);
    return XTG_OK;
}

}  // extern "C"
