/* dmgb_diag.h: diagnostic and instrumentation entry points of libdmgb.so.
 *
 * These are not part of the drop-in boundary (include/dmgb.h) and have no
 * counterpart in the reference: SeismicMesh's CGAL triangulation exposes no
 * predicate stages, star statistics or timings.  The test-suite uses the
 * dmdbg_* calls to check individual Delaunay stages (predicates, face
 * queries, escalation lists) against exhaustive host computations; bench.py
 * uses the dmprof_* calls to time the star kernels with CUDA events and to
 * count the library's kernel launches.  All return 0 / DM_OK on success.
 */
#ifndef DMGB_DIAG_H
#define DMGB_DIAG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* host evaluation of one predicate stage on FP32 points: kind 0
 * orient3_exact, 1 orient3_slow, 2 insph3_exact, 3 insph3_slow,
 * 4 orient2_exact, 5 incirc2_exact; returns the sign */
int dmdbg_host_pred(int kind, const float *a, const float *b, const float *c,
                    const float *d, const float *e);
/* fixed-point predicate at scale 2^g relative to a (kind 0 orient3, 1
 * insphere with symbolic perturbation, 2 orient2, 3 incircle); -99 when a
 * point has no exact representation at that scale */
int dmdbg_fixed_pred(int kind, int g, const float *a, const float *b,
                     const float *c, const float *d, const float *e);
/* device predicates on m point tuples (indices into pts) */
int dmdbg_predicates(const float *pts, const int32_t *tup, int32_t m,
                     int32_t kind, int32_t *out, void *stream);
/* device FP64 rounding of one operation (0 add, 1 mul, 2 fma, 3 two_sum
 * tail, 4 two_prod tail) */
int dmdbg_fp64(const double *a, const double *b, const double *c, int32_t m,
               int32_t op, double *out, void *stream);
/* level-2 face queries after a dm_delaunay call on the same points and
 * workspace: mode 0 the kernel's query, 1 an exhaustive half-space scan,
 * 2 the hull-candidate scan (3D) */
int dmdbg_face_query(int32_t dim, const float *pts, int64_t n, void *ws,
                     size_t ws_bytes, const int32_t *faces, int32_t m,
                     int32_t *out, void *stream);
int dmdbg_face_query_mode(int32_t dim, const float *pts, int64_t n, void *ws,
                          size_t ws_bytes, const int32_t *faces, int32_t m,
                          int32_t *out, void *stream, int32_t mode);
/* copies of the escalation list / hull-candidate flags of the last call */
int dmdbg_escalations(int32_t dim, int64_t n, void *ws, size_t ws_bytes,
                      int32_t *esc_out, int32_t *seed_out, void *stream);
int dmdbg_hull_candidates(int64_t n, void *ws, size_t ws_bytes, uint8_t *out,
                          void *stream);
/* per-vertex star dumps; DM_ERR_ARG unless built with -DDM_DEBUG_VERTEX */
int dmdbg_watch_vertex(int32_t vertex, int32_t *dbg);

/* CUDA-event timing of the star kernels of the dm_delaunay calls made while
 * enabled: dmprof_enable(1) resets and starts, dmprof_read synchronises and
 * returns the summed level-1 / level-2 milliseconds and the call count */
int dmprof_enable(int32_t on);
int dmprof_read(double *ms_l1, double *ms_l2, int32_t *calls);
/* number of kernels the library has launched in this process */
int64_t dmprof_launches(void);
/* slow-path and per-level statistics (compiled in with -DDM_L2_STATS;
 * otherwise zeros) */
int dmprof_slow_counters(unsigned long long *out8);
int dmprof_l1_stats(unsigned long long *out8);
int dmprof_l2_stats(unsigned long long *out, int64_t nstars);

#ifdef __cplusplus
}
#endif
#endif /* DMGB_DIAG_H */
