/*
 * xtrack_gb300.h — C-ABI of the GB300-native particle push that replaces
 * xtrack's generated `track_line` kernel.
 *
 * Plain C types only: raw pointers and sizes, no torch or CUDA types apart
 * from an opaque stream handle passed as `void*` (a cudaStream_t; NULL means
 * the legacy default stream).
 *
 * Reference interfaces replaced (paths inside the xtrack source tree):
 *   xtrack/tracker.py:546-564      track_line(...) kernel signature
 *                                  (descriptor tracker.py:793-814)
 *   xtrack/tracker.py:107-118      TrackerData / ElementRefData build
 *                                  (tracker_data.py:65-172, 221-255)
 *   xtrack/base_element.py:130-215 <Elem>_track_particles (per-element kernel)
 *   xtrack/particles/particles.py:26-83   Particles structure-of-arrays
 *   xtrack/monitors/particles_monitor.h:12-77  ParticlesMonitor record layout
 *
 * Error convention: every entry point returns an int32 status; 0 is success,
 * negative values are host-detectable errors (XTG_E_*). Physics outcomes
 * (losses) are reported only through the particles' `state` array, exactly as
 * in the reference. Nothing here aborts or traps. The message of the last
 * error on the calling thread is available from xtg_get_last_error().
 */
#ifndef XTRACK_GB300_H
#define XTRACK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XTG_ABI_VERSION 3

/* Maximum number of multipole coefficients per array (order <= 20). */
#define XTG_MAX_KNL 21

/* ---- status codes ------------------------------------------------------ */
#define XTG_OK               0
#define XTG_E_NULL          -1   /* a required pointer is NULL               */
#define XTG_E_VALUE         -2   /* an argument is out of its valid range    */
#define XTG_E_UNSUPPORTED   -3   /* element feature outside the built set    */
#define XTG_E_CUDA          -4   /* a CUDA runtime call failed               */
#define XTG_E_CAPACITY      -5   /* a size exceeds a compiled-in maximum     */
#define XTG_E_TIMEOUT       -6   /* a bounded device wait gave up            */
#define XTG_E_NOMEM         -7   /* an allocation failed                     */

/* ---- element classes (reference class names, xtrack/beam_elements/) ---- */
#define XTG_CLS_MARKER          0   /* marker.py                             */
#define XTG_CLS_DRIFT           1   /* drift.py, drift.h                     */
#define XTG_CLS_MULTIPOLE       2   /* multipole.py, multipole.h             */
#define XTG_CLS_BEND            3   /* bend.py, bend.h                       */
#define XTG_CLS_QUADRUPOLE      4   /* quadrupole.py, quadrupole.h           */
#define XTG_CLS_SEXTUPOLE       5   /* sextupole.py, sextupole.h             */
#define XTG_CLS_OCTUPOLE        6   /* octupole.py, octupole.h               */
#define XTG_CLS_CAVITY          7   /* cavity.py, cavity.h                   */
#define XTG_CLS_LIMIT_ELLIPSE   8   /* limit_ellipse.py, limitellipse.h      */
#define XTG_CLS_LIMIT_RECT      9   /* limit_rect.py, limitrect.h            */
#define XTG_CLS_MONITOR        10   /* monitors/*.py placed in the line      */
#define XTG_CLS_LIMIT_POLYGON  11   /* limit_polygon.py, limitpolygon.h      */
#define XTG_CLS_DIPOLE_EDGE    12   /* dipole_edge.py, dipoleedge.h          */
#define XTG_CLS_LIMIT_RECT_ELLIPSE 13 /* limit_rect_ellipse.py, limitrectellipse.h */
#define XTG_NUM_CLS            14

/* Slice kind of a record (slice classes of slice_elements_*.py). A slice
 * record carries its parent's parameters plus its own `weight`. */
#define XTG_SLICE_NONE    0   /* the element itself                           */
#define XTG_SLICE_THICK   1   /* ThickSlice<X>  (thick_slice_*.h)             */
#define XTG_SLICE_THIN    2   /* ThinSlice<X>   (thin_slice_*.h)              */
#define XTG_SLICE_DRIFT   3   /* DriftSlice<X>  (drift_slice_*.h)             */
#define XTG_SLICE_ENTRY   4   /* ThinSlice<X>Entry (edge map at entry)        */
#define XTG_SLICE_EXIT    5   /* ThinSlice<X>Exit  (edge map at exit)         */

/* Track flags bit positions (xtrack/track_flags.py:5-12). */
#define XTG_FLAG_BACKTRACK               0
#define XTG_FLAG_KILL_CAVITY_KICK        2
#define XTG_FLAG_IGNORE_GLOBAL_APERTURE  3
#define XTG_FLAG_IGNORE_LOCAL_APERTURE   4
/* Freeze the longitudinal coordinates (zeta, ptau, delta, rpp, rvv) for the
   call: the reference's Line.track(freeze_longitudinal=True), which compiles
   its setters of those variables into no-ops (FREEZE_VAR_<name>,
   particles.py:185-225; line.py:4446-4469). Outside the reference's bits. */
#define XTG_FLAG_FREEZE_LONGITUDINAL     32

/*
 * One lattice element as the reference stores it (the `_xofields` of each
 * class, with slice parents resolved into the record). Fields a class does
 * not have are ignored. Arrays hold `order+1` (knl/ksl) and `order_rel+1`
 * (knl_rel/ksl_rel) valid entries.
 */
typedef struct xtg_element {
    int32_t cls;                 /* XTG_CLS_*                                 */
    int32_t slice;               /* XTG_SLICE_*                               */
    int32_t model;               /* model index (_common.py:20-80)            */
    int32_t integrator;          /* 0 adaptive,1 teapot,2 yoshida4,3 uniform  */
    int64_t num_multipole_kicks; /* magnets; Cavity: num_kicks                */
    int64_t order;               /* len(knl)-1                                */
    int64_t order_rel;           /* len(knl_rel)-1; -1 when absent            */
    int32_t isthick;             /* Multipole.isthick                         */
    int32_t main_is_skew;        /* knl_rel reference component is skew       */
    int32_t main_order;          /* Multipole.main_order                      */
    int32_t edge_entry_active;
    int32_t edge_exit_active;
    int32_t edge_entry_model;    /* -1 suppressed, 0 linear, 1 full, 2 dipole */
    int32_t edge_exit_model;
    int32_t absolute_time;       /* Cavity                                    */
    double weight;               /* slices; 1 for the element itself          */
    double length;
    double h;                    /* Bend curvature angle/length               */
    double hxl;                  /* Multipole                                 */
    double k0, k1, k2, k3;
    double k0s, k1s, k2s, k3s;
    double inv_factorial_order;  /* 1/order!                                  */
    double knl[XTG_MAX_KNL];
    double ksl[XTG_MAX_KNL];
    double knl_rel[XTG_MAX_KNL];
    double ksl_rel[XTG_MAX_KNL];
    double edge_entry_angle, edge_exit_angle;
    double edge_entry_angle_fdown, edge_exit_angle_fdown;
    double edge_entry_fint, edge_exit_fint;
    double edge_entry_hgap, edge_exit_hgap;
    double voltage, frequency, harmonic, lag, phase;   /* Cavity            */
    double a_squ, b_squ, a_b_squ;                      /* LimitEllipse      */
    double min_x, max_x, min_y, max_y;                 /* LimitRect         */
    /* Misalignment fields (base_element.py:274-282). shift_x, shift_y,
     * rot_s_rad and rot_s_rad_no_frame may be nonzero on the apertures, a
     * thin Multipole (isthick 0) and DipoleEdge (the straight transform of
     * zero length, track_misalignments.h:38-130); every other element, and
     * shift_s, rot_x_rad, rot_y_rad everywhere, must be zero
     * (XTG_E_UNSUPPORTED otherwise). */
    double shift_x, shift_y, shift_s;
    double rot_x_rad, rot_y_rad, rot_s_rad, rot_s_rad_no_frame;
    /* Host address of the class's extra description, read by
     * xtg_lattice_create, 0 for the other classes:
     *   XTG_CLS_MONITOR        an xtg_element_monitor (its buffers are
     *                          device pointers kept by the caller for the
     *                          lattice's lifetime);
     *   XTG_CLS_LIMIT_POLYGON  an xtg_polygon (vertices copied). */
    uint64_t aux;
    /* DipoleEdge: k, e1, hgap, fint and the linear coefficients r21, r43 as
     * the class computes them (_update_r21_r43 from k, e1, e1_fd, hgap,
     * fint); side 0 entry, 1 exit; `model` 0 linear, 1 full, -1 suppressed. */
    double k, e1, hgap, fint, r21, r43;
    int32_t side;
    int32_t reserved_dipole_edge;
} xtg_element;

/* Vertices of a LimitPolygon aperture (limit_polygon.py), host arrays. */
typedef struct xtg_polygon {
    int64_t n_vertices;
    const double* x_vertices;
    const double* y_vertices;
} xtg_polygon;

/*
 * Particles structure-of-arrays (particles.py:26-83). Pointers are device
 * pointers for xtg_track and host pointers for the CPU oracle; every array has
 * `capacity` entries. Fields the push does not touch (spin, rng, weight,
 * pdg_id, parent_particle_id, gamma0) may be NULL.
 */
typedef struct xtg_particles {
    int64_t capacity;
    double q0, mass0, t_sim;
    double *p0c, *gamma0, *beta0;
    double *s, *zeta, *x, *y, *px, *py;
    double *ptau, *delta, *rpp, *rvv;
    double *chi, *charge_ratio, *weight;
    double *ax, *ay;
    int64_t *pdg_id, *particle_id, *at_element, *at_turn, *state;
    int64_t *parent_particle_id;
} xtg_particles;

/*
 * Turn-by-turn ParticlesMonitor (particles_monitor.h:12-77). Records have
 * `n_records = (stop-start) * (part_id_end-part_id_start) * n_repetitions`
 * entries in `data`; a record lands at
 *   n_turns*(particle_id - part_id_start) + at_turn - start_at_turn
 * (plus the frame offset when n_repetitions > 1). A NULL array in `data`
 * means that field is not recorded (the reference records all of them).
 */
typedef struct xtg_monitor {
    int64_t start_at_turn, stop_at_turn;
    int64_t part_id_start, part_id_end;
    int64_t ebe_mode;
    int64_t n_repetitions, repetition_period;
    int64_t n_records;
    xtg_particles data;
} xtg_monitor;

/*
 * A monitor placed in the line as an element (monitors/*.py). kind:
 *   XTG_MON_PARTICLES      ParticlesMonitor as an element: the records of
 *                          `particles` (same layout as the turn-by-turn
 *                          monitor), written each time a particle passes;
 *   XTG_MON_LAST_TURNS     LastTurnsMonitor (last_turns_monitor.h): a
 *                          rolling buffer of the last `n_last_turns` passes
 *                          (every `every_n_turns` turns) of particles
 *                          [particle_id_start, +num_particles), float32
 *                          coordinates and uint32 ids/turns;
 *   XTG_MON_BEAM_POSITION  BeamPositionMonitor (beam_position_monitor.h):
 *                          per sample slot, the count and the sums of x and
 *                          y of the particles that pass (atomic adds; the
 *                          summation order is not fixed).
 */
#define XTG_MON_PARTICLES     1
#define XTG_MON_LAST_TURNS    2
#define XTG_MON_BEAM_POSITION 3
#define XTG_MON_BEAM_SIZE     4   /* beam_size_monitor.h: BEAM_POSITION plus
                                     the sums of x^2 and y^2 per slot     */
#define XTG_MON_BEAM_PROFILE  5   /* beam_profile_monitor.h: per sample, the
                                     counts of x and y in nx / ny bins    */

typedef struct xtg_element_monitor {
    int32_t kind;
    int32_t reserved;
    int64_t particle_id_start;      /* LAST_TURNS, BEAM_POSITION              */
    int64_t num_particles;          /* BEAM_POSITION: -1 means all particles  */
    int64_t n_last_turns, every_n_turns;          /* LAST_TURNS              */
    int64_t start_at_turn, n_slots;               /* BEAM_POSITION           */
    double frev, sampling_frequency;              /* BEAM_POSITION           */
    uint32_t *lost_at_offset, *lt_particle_id, *lt_at_turn;   /* LAST_TURNS */
    float *lt_x, *lt_px, *lt_y, *lt_py, *lt_delta, *lt_zeta;
    double *count, *x_sum, *y_sum;                /* BEAM_POSITION, BEAM_SIZE */
    double *x2_sum, *y2_sum;                      /* BEAM_SIZE               */
    int64_t nx, ny;                               /* BEAM_PROFILE: bins;     */
    double x_min, dx, y_min, dy;                  /*   n_slots = sample_size */
    double *counts_x, *counts_y;                  /*   n_slots*nx, *ny       */
    xtg_monitor particles;                        /* PARTICLES               */
} xtg_element_monitor;

/* Compile-time TrackerConfig equivalents (line.py:283-287). */
typedef struct xtg_config {
    int32_t use_exact_drifts;     /* XTRACK_USE_EXACT_DRIFTS                 */
    int32_t cavity_preserve_angle;/* XTRACK_CAVITY_PRESERVE_ANGLE            */
    int32_t has_global_xy_limit;  /* XTRACK_GLOBAL_XY_LIMIT defined          */
    int32_t arith;                /* XTG_ARITH_EXACT or XTG_ARITH_FAST       */
    double global_xy_limit;       /* its value, 1.0 by default               */
} xtg_config;

/* Arithmetic of the push (xtg_config.arith).
 * EXACT: the reference's operation order, no fused multiply-add; results
 *        equal the reference CPU build bit for bit except for the last-ulp
 *        behaviour of sin/cos/atan2/asin/sinh/cosh.
 * FAST:  the minimal formulation (one merged complex Horner polynomial per
 *        kick, fused multiply-adds, merged half drifts); results agree with
 *        the reference to within its own rounding noise. */
#define XTG_ARITH_EXACT 0
#define XTG_ARITH_FAST  1

typedef struct xtg_lattice xtg_lattice;   /* opaque handle */

/* Library / ABI information. */
int32_t xtg_abi_version(void);

/* Copies the last error message of the calling thread into buf (size n). */
int32_t xtg_get_last_error(char* buf, int64_t n);

/*
 * Builds the packed element-parameter table from `n_elements` raw records
 * and uploads it to the current CUDA device. Replaces TrackerData
 * construction (tracker_data.py:65-172) and the per-particle model
 * resolution of track_magnet_particles (track_magnet.h:518-574), which is
 * hoisted here. Allocates device memory; the handle owns it.
 */
int32_t xtg_lattice_create(const xtg_element* elements, int64_t n_elements,
                           const xtg_config* config, xtg_lattice** out);

/* Frees the device table and the handle. Safe on NULL. */
int32_t xtg_lattice_destroy(xtg_lattice* lattice);

/* Number of elements and the FP64 FLOPs one particle spends on elements
 * [ele_start, ele_start+num_ele) in the canonical minimal formulation
 * (FMA = 2, div/sqrt/sin/cos = 1). Used for roofline accounting. */
int32_t xtg_lattice_info(const xtg_lattice* lattice, int64_t* n_elements,
                         int64_t ele_start, int64_t num_ele,
                         double* flops_per_particle);

/*
 * The push: replaces track_line (tracker.py:546-750). Tracks particles
 * [0, capacity) through `num_turns` turns of elements
 * [ele_start, ele_start+num_ele_track), writing the particles in place.
 * `monitor` may be NULL (flag_monitor must then be 0). Asynchronous on
 * `stream`. The lattice owns the scratch of the push (active-particle index
 * list, work queue); it is allocated on the first call and when the particle
 * capacity grows, so steady-state calls allocate nothing.
 */
int32_t xtg_track(const xtg_lattice* lattice, const xtg_particles* particles,
                  int32_t num_turns, int32_t ele_start, int32_t num_ele_track,
                  int32_t flag_end_turn_actions, int32_t flag_reset_s_at_end_turn,
                  int32_t flag_monitor, int32_t num_ele_line, double line_length,
                  const xtg_monitor* monitor, uint64_t track_flags,
                  void* stream);

/*
 * Allocation-free variant of xtg_track. No reference counterpart: the
 * reference's track_line has no scratch to place. The push's scratch (index
 * list, work queue, counters) lives in one static device array sized for
 * XTG_NOALLOC_MAX_PARTICLES particles (about 4.7 MB per device) instead of
 * the lattice's workspace, so a call makes no cudaMalloc/cudaFree and no
 * framework allocation. Same arguments and results as xtg_track; the
 * element table is read from global memory (the tuning's chunk_bytes and
 * use_graph are not used), compact_every and block_size are. Capacities
 * above XTG_NOALLOC_MAX_PARTICLES are rejected with XTG_E_CAPACITY; so is
 * backtracking until an xtg_track call has built the lattice's reversed
 * table. Every call looks up the array's address (no allocation); the
 * first call on a device, and the first after the context is re-created
 * (cudaDeviceReset), also clears its error word: make that call before any
 * stream capture. The array is device memory of the library's module: with
 * CUDA's lazy module loading it is reserved when the module is first loaded
 * on a device (the first call into the push there), so make that call
 * before a framework's allocator takes the device's free memory.
 * xtg_device_status on any lattice of the device reports (and clears) the
 * device-side error word of these calls along with the lattice's own.
 * All calls on a device share the one array: calls that overlap in time
 * (on different streams or host threads) race and must not be issued.
 */
#define XTG_NOALLOC_MAX_PARTICLES 1048576
int32_t xtg_track_noalloc(const xtg_lattice* lattice, const xtg_particles* particles,
                          int32_t num_turns, int32_t ele_start, int32_t num_ele_track,
                          int32_t flag_end_turn_actions, int32_t flag_reset_s_at_end_turn,
                          int32_t flag_monitor, int32_t num_ele_line, double line_length,
                          const xtg_monitor* monitor, uint64_t track_flags, void* stream);

/*
 * Multi-element monitor (monitors/multi_element_monitor.h:10-65; the
 * tracker's `multi_element_monitor_at`, tracker.py:1482-1525): before each
 * element whose index maps to an observation point, the 7 coordinates
 * x, px, y, py, zeta, delta, s of particles [part_id_start, part_id_end)
 * in turns [start_at_turn, stop_at_turn) are stored at
 * data[((turn - start) * n_particles + (id - part_id_start)) * 7 + coord)
 *      * n_obs + obs].
 * `at_element_mapping` (device, mapping_len entries) gives the observation
 * index of each element or -1. Set on a lattice it applies to every later
 * xtg_track / xtg_track_noalloc call on it until cleared with NULL; the
 * struct is copied, its device buffers are the caller's.
 */
typedef struct xtg_multi_element_monitor {
    int64_t start_at_turn, stop_at_turn;
    int64_t part_id_start, part_id_end;
    int64_t mapping_len, n_obs;
    const int64_t* at_element_mapping;
    double* data;
} xtg_multi_element_monitor;

int32_t xtg_set_multi_element_monitor(xtg_lattice* lattice,
                                      const xtg_multi_element_monitor* monitor);

/* Launch tuning of the push. Results do not depend on it. */
/* Defaults of a new lattice: block_size 128, compact_every 0, chunk_bytes
   32768 (fast arithmetic) or 16384 (exact), use_graph 0. */
typedef struct xtg_tuning {
    int32_t block_size;      /* threads per block: 32, 64, 128 or 256        */
    int32_t compact_every;   /* turns between lost-particle compactions;
                                0: only at the start of each call            */
    int32_t chunk_bytes;     /* shared-memory chunk of the element table
                                (double-buffered bulk copies), multiple of
                                16, at most 115712; raised to the largest
                                element record when smaller. A tracked range
                                of at most 2*chunk_bytes is copied once and
                                stays resident. 0: read the table from
                                global memory                                */
    int32_t use_graph;       /* replay the compaction + tracking rounds of a
                                call from a captured CUDA graph              */
} xtg_tuning;

int32_t xtg_get_tuning(const xtg_lattice* lattice, xtg_tuning* out);
int32_t xtg_set_tuning(xtg_lattice* lattice, const xtg_tuning* tuning);

/* Device-side status of the calls on this lattice (or batch) since the last
 * status read: XTG_OK, XTG_E_TIMEOUT when a bounded wait inside a kernel gave
 * up, XTG_E_VALUE when a particle named a lattice outside the batch (that
 * particle is not tracked). Synchronizes the device and clears the status.
 * xtg_device_status also reads and clears the error word of the
 * allocation-free calls (xtg_track_noalloc) on the current device; the
 * lattice's own status is returned first when both are set. */
int32_t xtg_device_status(const xtg_lattice* lattice);

/*
 * Batched push of several lattices that share one element sequence (error
 * seeds of one ring): one persistent launch tracks every particle through
 * the lattice named by its entry in `lattice_index` (device int32 array of
 * `capacity` entries). The batch keeps its own copy of the packed tables;
 * the lattices may be destroyed afterwards. All lattices must have the same
 * number of elements and the same xtg_config.
 */
typedef struct xtg_batch xtg_batch;

int32_t xtg_batch_create(const xtg_lattice* const* lattices, int32_t n_lattices,
                         xtg_batch** out);
int32_t xtg_batch_destroy(xtg_batch* batch);
int32_t xtg_batch_get_tuning(const xtg_batch* batch, xtg_tuning* out);
int32_t xtg_batch_set_tuning(xtg_batch* batch, const xtg_tuning* tuning);
int32_t xtg_batch_device_status(const xtg_batch* batch);
int32_t xtg_track_batch(xtg_batch* batch, const xtg_particles* particles,
                        const int32_t* lattice_index, int32_t num_turns,
                        int32_t ele_start, int32_t num_ele_track,
                        int32_t flag_end_turn_actions,
                        int32_t flag_reset_s_at_end_turn, int32_t flag_monitor,
                        int32_t num_ele_line, double line_length,
                        const xtg_monitor* monitor, uint64_t track_flags,
                        void* stream);

/* Blocks until all work on `stream` is done; returns XTG_E_CUDA on error. */
int32_t xtg_sync(void* stream);

/* Number of kernel launches the library issued since it loaded. */
int64_t xtg_launch_count(void);

/* FP64 peak probe: DFMA throughput of the current device in FLOP/s
 * (FMA = 2), measured with independent FMA chains over the whole GPU. */
int32_t xtg_measure_fp64_peak(double* flops_per_s);

/*
 * Checks of the integer-pipe binary64 multiply that the exact push uses for
 * its products (no reference counterpart: the reference multiplies on the
 * FP64 unit). out[i] = a[i] * b[i], rounded to nearest even, for n pairs.
 * xtg_f64_mul_host computes on the host (host arrays); xtg_f64_mul_device
 * runs the device routine in a kernel on `stream` (device arrays). Both
 * must equal the hardware multiply bit for bit.
 */
int32_t xtg_f64_mul_host(const double* a, const double* b, double* out, int64_t n);
int32_t xtg_f64_mul_device(const double* a, const double* b, double* out, int64_t n,
                           void* stream);

/* Throughput probe of the same multiply: independent multiply+add chains
 * over the whole GPU with the multiplies on the integer pipes and the adds
 * on the FP64 unit. Returns the chains' FP64 operations (multiplies plus
 * adds) per second. */
int32_t xtg_measure_emul_rate(double* ops_per_s);

/*
 * Diagnostic of the push's failure path (no reference counterpart: the
 * reference's kernel has no waits). Runs one shared-memory barrier wait of
 * the kind the push uses to stage its element table, on a barrier that
 * nothing completes, bounded at `limit_cycles` SM clock cycles (1 to
 * 4e9). The wait gives up, records the time-out in a device error word and
 * the kernel returns; the call reads the word as xtg_device_status does and
 * returns XTG_E_TIMEOUT. The context stays usable. Returns XTG_OK only if
 * the wait did not time out.
 */
int32_t xtg_check_bounded_wait(int64_t limit_cycles);

/*
 * Survival surrogate kernels (no reference counterpart: the reference has
 * no learned component). A multilayer perceptron with BF16 weights and
 * activations and FP32 accumulation screens dynamic-aperture scans. All
 * pointers are device pointers; bf16 arrays are passed as void*. All calls
 * are asynchronous on `stream`.
 */
#define XTG_MLP_ACT_NONE 0
#define XTG_MLP_ACT_GELU 1   /* tanh form: z/2 (1 + tanh(sqrt(2/pi)(z + 0.044715 z^3))) */

/* Tensor-core contraction R[m, n] = sum_k A(m, k) B(n, k), with A(m, k) at
 * A[m*a_sm + k*a_sk] and B(n, k) at B[n*b_sn + k*b_sk] (bf16, any strides),
 * FP32 accumulation in tensor memory (tcgen05). Operands with a unit stride
 * along k or along their rows, a 16-byte aligned base and a pitch that is a
 * multiple of 8 elements are staged by TMA (a persistent kernel, one CTA per
 * SM); others by the threads (same results). Epilogue: z = R + bias[n] (bias may be NULL);
 * Z[m*z_ld + n] = z (fp32, optional); Y[m*y_ld + n] = act(z) (bf16,
 * optional); C[m*c_ld + n] = z, or += z with c_accumulate (fp32, optional). */
int32_t xtg_mlp_gemm(const void* A, int64_t a_sm, int64_t a_sk, const void* B,
                     int64_t b_sn, int64_t b_sk, int32_t M, int32_t N, int32_t K,
                     const float* bias, int32_t act, float* Z, int64_t z_ld,
                     void* Y, int64_t y_ld, float* C, int64_t c_ld,
                     int32_t c_accumulate, void* stream);

/* dZ = dY * act'(Z) over n elements; fp32 (dZ) and/or bf16 (dZ16) output. */
int32_t xtg_mlp_act_backward(const float* dY, const float* Z, int64_t n, int32_t act,
                             float* dZ, void* dZ16, void* stream);

/* out[n] (+)= sum_m X[m*ld + n], fp32, fixed summation order. */
int32_t xtg_mlp_colsum(const float* X, int64_t M, int32_t N, int64_t ld, float* out,
                       int32_t accumulate, void* stream);

/* Loss of the two network outputs per sample (out[m*ld+0]: logit of
 * P(survive), out[m*ld+1]: normalised log loss turn; ld >= 2, the other
 * columns of a padded output layer are not read): binary cross-entropy
 * plus w_turn * squared error on the loss turn of lost samples. Writes
 * dLoss/dout / M (fp32 and bf16) into columns 0 and 1 of dout / dout16
 * (row pitch ld) and the per-sample loss. */
int32_t xtg_mlp_loss(const float* out, int64_t ld, const float* survive,
                     const float* logturn, int64_t M, float w_turn, float* dout,
                     void* dout16, float* loss, void* stream);

/* One Adam step (bias-corrected, decoupled weight decay) on fp32 master
 * weights w; refreshes the bf16 copy w16 when not NULL. step >= 1. */
int32_t xtg_mlp_adam(float* w, void* w16, const float* grad, float* m1, float* m2,
                     int64_t n, float lr, float beta1, float beta2, float eps,
                     float weight_decay, int64_t step, void* stream);

/* y = bf16(x) over n elements. */
int32_t xtg_mlp_to_bf16(const float* x, int64_t n, void* y, void* stream);

/* Waits for the device, then reads and clears the xtg_mlp kernels' device
 * error word: XTG_E_TIMEOUT when a bounded wait inside one of them gave up
 * (that kernel's outputs were not written), else XTG_OK. */
int32_t xtg_mlp_device_status(void);

/* Diagnostic of the failure path of the contraction's bounded waits: one
 * wait of its kind on a shared-memory barrier that nothing completes, given
 * up after limit_cycles SM cycles (1 .. 2e9). Returns what
 * xtg_mlp_device_status then reports: XTG_E_TIMEOUT when the wait gave up
 * and the status was read and cleared; the context stays usable. */
int32_t xtg_mlp_check_bounded_wait(int64_t limit_cycles);

/* Message of the last failed xtg_mlp_* call of this thread. */
int32_t xtg_mlp_get_last_error(char* buf, int64_t n);

#ifdef __cplusplus
}
#endif

#endif /* XTRACK_GB300_H */
