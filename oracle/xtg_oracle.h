/*
 * CPU oracle for the xtrack `Line.track` push. TEST INFRASTRUCTURE ONLY:
 * this library is the checker that the CUDA path is compared against and
 * the timed CPU baseline; no product code path calls it.
 *
 * It is a restatement, in plain C99, of the reference's element arithmetic
 * and of its `track_line` driver, written to follow the reference's
 * operation order so that, compiled with -ffp-contract=off, it reproduces
 * the reference's CPU results bit for bit (libm calls aside). Each function
 * in xtg_oracle.c cites the reference file:line it follows.
 */
#ifndef XTG_ORACLE_H
#define XTG_ORACLE_H

#include "../include/xtrack_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Driver structure used by xto_track. */
#define XTO_MODE_PER_PARTICLE 0   /* GPU semantics: one particle at a time,
                                     tracker.py:594-736 (cuda branch)      */
#define XTO_MODE_OPENMP       1   /* CPU OpenMP semantics: per-thread chunks,
                                     element-outer, swap compaction and
                                     final reorganize, tracker.py:566-748 */

/* Checks that every record is inside the implemented feature set.
 * Returns XTG_OK or XTG_E_UNSUPPORTED/XTG_E_VALUE with a message. */
int32_t xto_validate(const xtg_element* elements, int64_t n_elements,
                     char* msg, int64_t msg_len);

/* Restated track_line (tracker.py:543-750) over host arrays. In OPENMP mode
 * the particle arrays are reordered exactly as the reference's CPU path
 * reorders them; compare results keyed by particle_id. num_threads <= 0
 * uses all available threads. */
int32_t xto_track(const xtg_element* elements, int64_t n_elements,
                  const xtg_config* config, xtg_particles* particles,
                  int32_t num_turns, int32_t ele_start, int32_t num_ele_track,
                  int32_t flag_end_turn_actions, int32_t flag_reset_s_at_end_turn,
                  int32_t flag_monitor, int32_t num_ele_line, double line_length,
                  const xtg_monitor* monitor, uint64_t track_flags,
                  int32_t mode, int32_t num_threads);

/* sizeof / offsetof of the C-ABI structs (layout check of foreign mirrors):
 * out[0..11] = element, particles, monitor, config sizes; offsets of
 * element.knl, element.shift_x, monitor.data; element-monitor size, its
 * offset of particles; offsets of element.aux, element.r21, element.side. */
int32_t xto_abi_sizes(int64_t* out);

/* Multi-element monitor applied by the following xto_track calls (NULL
 * clears it); host buffers. */
int32_t xto_set_multi_element_monitor(const xtg_multi_element_monitor* m);

/* Smallest distance to an aperture edge per particle_id (n entries, which
 * the caller fills with +inf) recorded by the following xto_track calls at
 * every aperture a particle reaches; NULL stops the recording. */
int32_t xto_set_edge_distance(double* out, int64_t n);

/* Threads the OpenMP runtime would use (1 when built without OpenMP). */
int32_t xto_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* XTG_ORACLE_H */
