/*
 * dmgb.h - C ABI of the GB300 DistMesh engine (libdmgb.so).
 *
 * Every entry point returns an int status (DM_OK == 0).  Pointers marked
 * "device" are CUDA device pointers; "stream" is a cudaStream_t passed as
 * void*.  The library never allocates device memory on the paths declared
 * here: callers pass workspaces sized by the matching *_workspace_size call.
 * Kernels report data-dependent failures through a device counters block
 * (int64_t[DM_NCOUNTERS]) that the caller reads when it synchronises.
 *
 * Point layout: 2D points are float[n][2]; 3D points are float[n][4] (x, y,
 * z, unused) so that one point is one aligned 16-byte load.
 *
 * Each declaration names the reference interface it replaces
 * (path:line inside the SeismicMesh project).
 */
#ifndef DMGB_H
#define DMGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define DM_OK 0
#define DM_ERR_ARG 1           /* bad argument (shape, size, pointer)      */
#define DM_ERR_CUDA 2          /* a CUDA runtime call failed               */
#define DM_ERR_CAPACITY 3      /* an output buffer was too small           */
#define DM_ERR_NOT_CONVERGED 4 /* bounded iteration hit its limit          */
#define DM_ERR_DEGENERATE 5    /* degenerate input (duplicates, flat set)  */
#define DM_ERR_WORKSPACE 6     /* workspace smaller than required          */

/* ---- device counters block: indices into int64_t[DM_NCOUNTERS] --------- */
#define DM_CNT_CELLS 0       /* cells written by dm_delaunay               */
#define DM_CNT_ESCALATED 1   /* vertices resolved by the exhaustive search */
#define DM_CNT_FLAGS 2       /* OR of DM_FLAG_* bits                       */
#define DM_CNT_KEPT 3        /* cells kept by dm_filter_cells              */
#define DM_CNT_EDGES 4       /* unique edges counted by dm_adjacency       */
#define DM_CNT_BAD 5         /* cells flagged by dm_dihedral_flags         */
#define DM_CNT_DUPS 6        /* duplicate points found by dm_delaunay      */
#define DM_CNT_AUX 7
#define DM_CNT_MAXDEG 13     /* largest neighbour count seen by dm_adjacency */
#define DM_NCOUNTERS 16

/* grid_exp value that disables position rounding (dm_update_points,
 * dm_sliver_perturb) */
#define DM_NO_GRID (-1000)

#define DM_FLAG_CELL_OVERFLOW 1   /* cells capacity exceeded               */
#define DM_FLAG_STAR_OVERFLOW 2   /* a vertex star exceeded its capacity   */
#define DM_FLAG_SEED_FAILED 4     /* no Delaunay seed found for a vertex   */
#define DM_FLAG_DUPLICATES 8      /* exactly coincident input points       */
#define DM_FLAG_EXACT_OVERFLOW 16 /* exact arithmetic capacity exceeded    */
#define DM_FLAG_ADJ_OVERFLOW 32   /* adjacency row capacity exceeded       */
#define DM_FLAG_DIVERGED 64       /* max movement >= 1000 h0               */
#define DM_FLAG_NONFINITE 128     /* NaN/Inf in positions                  */

/* ---- signed distance programs ------------------------------------------
 * A domain is a postfix program of primitives and set operations, see
 * seismicmesh_gb300/geometry/signed_distance_functions.py for the encoder.
 * ops/params live in device memory. */
typedef struct dm_sdf_program {
  const int32_t *ops;   /* device: n_ops records of DM_SDF_OPREC ints      */
  const float *params;  /* device: parameter pool                          */
  int32_t n_ops;
  int32_t dim;
} dm_sdf_program;

/* ---- sizing functions ------------------------------------------------- */
#define DM_SIZING_CONST 0 /* h(x) = h                                      */
#define DM_SIZING_GRID 1  /* linear interpolation on a regular grid,        */
                          /* extrapolating (RegularGridInterpolator,        */
                          /* bounds_error=False, fill_value=None)           */
#define DM_SIZING_SLOTS 2 /* per adjacency slot values supplied by caller   */
typedef struct dm_sizing {
  int32_t kind;
  int32_t dim;
  float h;              /* DM_SIZING_CONST                                  */
  const float *grid;    /* device, C order (n0, n1[, n2])                   */
  int32_t n[3];
  float lo[3], hi[3];   /* axis k spans linspace(lo[k], hi[k], n[k])        */
  const float *slot_h;  /* device, [n_points * adj_cap] for DM_SIZING_SLOTS */
} dm_sizing;

/* ---- library ----------------------------------------------------------- */
int dm_version(void);
/* message of the last failing call on this host thread */
const char *dm_last_error(void);
/* number of entry points listed in this header (for loader self-checks) */
int dm_abi_count(void);

/* ---- exact predicates on the host (FP32 inputs) -------------------------
 * Replace the filtered Epick predicates CGAL uses inside the triangulations
 * (generation/cpp/delaunay_class3.cpp:116-129).  Return -1/0/+1; the _sos
 * variants apply the lexicographic symbolic perturbation and return 0 only
 * for five coplanar (four collinear) points. */
int dm_orient2(const float *a, const float *b, const float *c);
int dm_orient3(const float *a, const float *b, const float *c, const float *d);
int dm_incircle_sos(const float *a, const float *b, const float *c,
                    const float *d);
int dm_insphere_sos(const float *a, const float *b, const float *c,
                    const float *d, const float *e);

/* ---- Delaunay triangulation -------------------------------------------
 * Replaces DelaunayTriangulation{,3}.insert + get_finite_cells
 * (generation/cpp/delaunay_class.cpp:108-121,232-265;
 *  generation/cpp/delaunay_class3.cpp:116-129,276-310) as called from
 * generation/mesh_generator.py:465-469.  Writes every finite cell once,
 * positively oriented, as int32[cap_cells][dim+1] (device).  Vertex indices
 * are the input indices (no renumbering).  counters (device, zeroed by the
 * call) receives DM_CNT_CELLS / _ESCALATED / _FLAGS / _DUPS. */
int dm_delaunay_workspace_size(int32_t dim, int64_t n, size_t *bytes);
int dm_delaunay(int32_t dim, const float *points, int64_t n, int32_t *cells,
                int64_t cap_cells, int64_t *counters, void *workspace,
                size_t workspace_bytes, void *stream);

/* ---- cell filter ---------------------------------------------------------
 * Replaces _remove_triangles_outside (generation/mesh_generator.py:734-738):
 * keeps cells whose centroid c has sdf(c) < -geps.  n_cells is read from
 * counters[DM_CNT_CELLS] (device); the kept count goes to
 * counters[DM_CNT_KEPT].  The order of kept cells is unspecified (so is the
 * Delaunay output order; every consumer is order-free). */
int dm_filter_cells_workspace_size(int64_t cap_cells, size_t *bytes);
int dm_filter_cells(int32_t dim, const float *points, const int32_t *cells,
                    int64_t cap_cells, const dm_sdf_program *sdf, float geps,
                    int32_t *cells_out, int64_t *counters, void *workspace,
                    size_t workspace_bytes, void *stream);
/* centroids of the first counters[DM_CNT_CELLS] cells, float[cap][dim] */
int dm_cell_centroids(int32_t dim, const float *points, const int32_t *cells,
                      int64_t cap_cells, const int64_t *counters,
                      float *centroids, void *stream);

/* ---- bars (unique edges) ------------------------------------------------
 * Replaces _get_edges + _fast_geometry.unique_edges
 * (generation/mesh_generator.py:680-688, geometry/cpp/fast_geometry.cpp:30-77)
 * in the adjacency form the force kernels consume: row v of adj
 * (int32[n][adj_cap], device) lists the neighbours of v in increasing order,
 * deg[v] their count.  Cells are read from `cells` with count
 * counters[count_index].  counters[DM_CNT_EDGES] receives the number of
 * unique edges.  A vertex with more than adj_cap neighbours keeps the
 * adj_cap smallest and raises DM_FLAG_ADJ_OVERFLOW (call again with a larger
 * adj_cap).  The workspace holds the raw per-vertex neighbour lists. */
int dm_adjacency_workspace_size(int32_t dim, int64_t n, int64_t cap_cells,
                                size_t *bytes);
int dm_adjacency(int32_t dim, int64_t n, const int32_t *cells,
                 int64_t cap_cells, int32_t count_index, int32_t *adj,
                 int32_t adj_cap, int32_t *deg, int64_t *counters,
                 void *workspace, size_t workspace_bytes, void *stream);
/* Drop-in unique_edges: edges int32[m][2] -> sorted unique (min,max) pairs.
 * Needs the vertex count bound n (max index + 1).  An index outside [0, n)
 * is never used as an address: the call returns DM_ERR_ARG (the output is
 * then unspecified). */
int dm_unique_edges_workspace_size(int64_t n, int64_t m, size_t *bytes);
int dm_unique_edges(const int32_t *edges, int64_t m, int64_t n, int32_t *out,
                    int64_t *n_out_host, void *workspace,
                    size_t workspace_bytes, void *stream);
/* dm_unique_edges without a workspace.  No counterpart in the reference: its
 * unique_edges (geometry/cpp/fast_geometry.cpp:30-77) works on host vectors.
 * Same inputs, outputs and results as dm_unique_edges, but every
 * intermediate array lives in one static device array of the library
 * (about 8.4 MB per device), so the call allocates nothing: no cudaMalloc,
 * no cudaFree, no allocating library routine.  It serves callers that have
 * device buffers but cannot allocate a workspace: a thin FFI binding with no
 * device allocator of its own, or a process whose device memory is held by a
 * caching allocator, where an extra cudaMalloc can fail while the pool still
 * has room and a cudaFree synchronises the whole device.
 * Limits: n <= 131072 vertices and m <= 524288 edges; larger sizes return
 * DM_ERR_CAPACITY with a message naming the limits.
 * The first call on each device looks up the scratch address with
 * cudaGetSymbolAddress (with that device current; a failure returns
 * DM_ERR_CUDA), which may load the library's device code: make that first
 * call (m = 0 is enough) before any stream capture begins.
 * Nothing has to be zero beforehand: each call clears the counters it uses.
 * One scratch exists per device, so calls that overlap in time on the same
 * device (two streams or two host threads) race on it: serialise them.
 * The looked-up address is kept for the life of the process: a
 * cudaDeviceReset after the first call is not supported (the address may
 * then be stale).  Out-of-range indices return DM_ERR_ARG as in
 * dm_unique_edges.
 * Synchronises `stream` to read the output count, like dm_unique_edges. */
int dm_unique_edges_noalloc(const int32_t *edges, int64_t m, int64_t n,
                            int32_t *out, int64_t *n_out_host, void *stream);

/* ---- bar forces and point update ---------------------------------------
 * Replaces _compute_forces + dense scatter + position update + Newton
 * projection (generation/mesh_generator.py:497-506,691-712,762-784,
 * generation/utils.py:48-68).  Two passes over the adjacency:
 *   dm_bar_sums      per-block partial sums of L^dim and h^dim over
 *                    unique bars (v < w), written to partials[2*nblk];
 *   dm_update_points F = sum_w max(L0 - L, 0) / L * (p_v - p_w), with
 *                    L0 = h * L0mult * (sum L^d / sum h^d)^(1/d); points
 *                    with index < nfix keep F = 0;
 *                    p' = p + dt F, then one Newton step back onto the
 *                    zero level set of every program in `levels`
 *                    (level 0: points with d > 0; level k > 0: points with
 *                    0 < d < hmin / 1.5).  Writes points_out, per-block
 *                    maxima of |F| into the leading entries of maxf and
 *                    their maximum into maxf[nblk].  With grid_exp >= -200
 *                    the new positions are rounded to multiples of
 *                    2^grid_exp (DM_NO_GRID disables the rounding); points
 *                    on one such grid let dm_delaunay decide every
 *                    predicate in fixed-point integer arithmetic.
 * dm_bar_blocks gives nblk for n points (the same for 2D and 3D); partials
 * is a workspace of 2*nblk + 3 doubles written by dm_bar_sums and read by
 * dm_update_points. */
int dm_bar_blocks(int64_t n, int32_t *nblk);
int dm_bar_sums(int32_t dim, const float *points, int64_t n,
                const int32_t *adj, int32_t adj_cap, const int32_t *deg,
                const dm_sizing *sizing, double *partials, void *stream);
int dm_update_points(int32_t dim, const float *points, float *points_out,
                     int64_t n, const int32_t *adj, int32_t adj_cap,
                     const int32_t *deg, const dm_sizing *sizing,
                     const double *partials, float L0mult, float delta_t,
                     int64_t nfix, const dm_sdf_program *levels,
                     int32_t n_levels, float hmin, float deps, float *maxf,
                     int32_t grid_exp, void *stream);
/* bar midpoints per adjacency slot (float[n][adj_cap][dim]) for sizing
 * functions that are host callables */
int dm_slot_midpoints(int32_t dim, const float *points, int64_t n,
                      const int32_t *adj, int32_t adj_cap, const int32_t *deg,
                      float *mid, void *stream);

/* ---- signed distance and sizing evaluation ------------------------------
 * Replace geometry.*.eval (geometry/signed_distance_functions.py:89-101,
 * 307-623, geometry/cpp/fast_geometry.cpp:104-214) and SizeFunction.eval
 * (sizing/size_function.py:11-12, sizing/mesh_size_function.py:391-408).
 * x is float[n][x_stride]; grad (optional, may be NULL) float[n][dim]. */
int dm_sdf_eval(const dm_sdf_program *sdf, const float *x, int64_t n,
                int32_t x_stride, float *d, float *grad, void *stream);
int dm_sizing_eval(const dm_sizing *sizing, const float *x, int64_t n,
                   int32_t x_stride, float *h, void *stream);

/* ---- level-set improvement ----------------------------------------------
 * Replaces _improve_level_set_newton (generation/mesh_generator.py:741-759):
 * 5 damped Newton steps on the listed vertices. */
int dm_improve_level_set(int32_t dim, float *points, const int32_t *ids,
                         int64_t n_ids, const dm_sdf_program *sdf, float deps,
                         void *stream);

/* ---- sliver kernels -------------------------------------------------------
 * Replace calc_dihedral_angles / calc_circumsphere_grad
 * (geometry/cpp/fast_geometry.cpp:351-418, 580-666) and the sliver
 * selection of sliver_removal (generation/mesh_generator.py:222-274). */
int dm_dihedral_angles(const float *points, const int32_t *cells, int64_t nc,
                       double *angles, void *stream);
/* calc_dihedral_angles (fast_geometry.cpp:351-418) on caller FP64 points
 * double[n][3], FP64 throughout as in the reference. */
int dm_dihedral_angles_f64(const double *points, const int32_t *cells, int64_t nc,
                           double *angles, void *stream);
int dm_circumsphere_grad(const double *p0, const double *p1, const double *p2,
                         const double *p3, int64_t m, double *grad,
                         void *stream);
/* flags[c] = 1 when a dihedral angle of cell c is outside [min, max]
 * (radians); counters[DM_CNT_BAD] receives the count. */
int dm_dihedral_flags(const float *points, const int32_t *cells,
                      int64_t cap_cells, int32_t count_index, float min_angle,
                      float max_angle, int32_t *flags, int64_t *counters,
                      void *stream);
/* perturb vertex 0 of each flagged cell by step*h0*normalize(grad R^2),
 * all perturbations computed from the pre-update positions; when a vertex is
 * vertex 0 of several flagged cells the highest cell index wins (numpy's
 * buffered fancy-index += keeps the last duplicate).  New positions are
 * rounded to multiples of 2^grid_exp as in dm_update_points. */
int dm_sliver_workspace_size(int64_t n_points, size_t *bytes);
int dm_sliver_perturb(float *points, int64_t n_points, const int32_t *cells,
                      int64_t cap_cells, int32_t count_index,
                      const int32_t *flags, float step_h0, int32_t grid_exp,
                      void *workspace, size_t workspace_bytes,
                      int64_t *counters, void *stream);

/* ---- gradient limiting -----------------------------------------------------
 * Replaces _FastHJ.limgrad (sizing/cpp/FastHJ.cpp:63-157): limits
 * |grad f| <= dfdx on a column-major (dims[0], dims[1], dims[2]) grid with
 * 6-neighbour spacing elen, to the relaxation's fixed point. f is updated in
 * place (device, float64). */
int dm_limgrad(const int32_t *dims_host, double elen, double dfdx,
               int32_t imax, double *f, void *stream);

/* ---- sizing grids ----------------------------------------------------------
 * Elementwise part of get_sizing_function_from_segy
 * (sizing/mesh_size_function.py:146-221): vp (device, float64[n], updated
 * in place) *= scale; when some vp < 1e-3 lies outside the first row_len
 * entries they become vp_water; cell_size = clamp(min(vp/(freq*wl) if wl>0,
 * gradient_term if grad>0), hmin, hmax), then the Courant bound when
 * dt, cr_max and space_order are non-zero.  gradient_term may be NULL when
 * grad == 0.  workspace: >= 4 bytes of device memory. */
/* Gradient sizing term (_gradient_sizing, sizing/mesh_size_function.py:
 * 428-448): grad / (v + 0.1) with v the windowed variance of vp (box means
 * of vp and vp^2 as scipy.ndimage.uniform_filter: per-axis window
 * window_host[k], origin 0, 'reflect' boundaries), divided by its maximum and
 * shifted by its minimum.  vp is a C-order float64 grid of dims_host[0..dim)
 * read with the unit scale and water replacement of dm_size_from_velocity
 * (replace != 0: values below 1e-3 become vp_water).  The result feeds
 * gradient_term of dm_size_from_velocity.  FP64 running sums per grid line. */
int dm_gradient_term_workspace_size(int64_t n, size_t *bytes);
int dm_gradient_term(const double *vp, const int32_t *dims_host, int32_t dim,
                     const int32_t *window_host, double scale, double vp_water,
                     int32_t replace, double grad, double *gradient_term,
                     void *workspace, size_t workspace_bytes, void *stream);
int dm_size_from_velocity(double *vp, int64_t n, int64_t row_len,
                          const double *gradient_term, double scale,
                          double vp_water, double wl, double freq, double grad,
                          double hmin, double hmax, double dt, double cr_max,
                          double space_order, int32_t dim, double *cell_size,
                          int32_t *replaced_host, void *workspace,
                          size_t workspace_bytes, void *stream);
/* numpy.pad of a C-order float64 grid (_pad_it, mesh_size_function.py:
 * 575-587): mode 0 edge, 1 constant, 2 linear_ramp (to cval). */
int dm_pad_grid(const double *src, const int32_t *n_host,
                const int32_t *pre_host, const int32_t *post_host, int32_t dim,
                int32_t mode, double cval, double *dst, void *stream);

/* ---- termination topology ------------------------------------------------
 * dm_boundary replaces get_boundary_edges / get_boundary_facets /
 * get_boundary_vertices (geometry/utils.py:310-326,364-382,421-437): facets
 * (edges in 2D, triangles in 3D) that occur in exactly one of the cells
 * counters[count_index] of `cells`; vertex_flags[v] = 1 for their vertices;
 * faces_out (optional, int32[faces_cap][dim]) receives them, their count in
 * counters[DM_CNT_AUX]. */
int dm_boundary_workspace_size(int32_t dim, int64_t n, int64_t cap_cells,
                               size_t *bytes);
int dm_boundary(int32_t dim, int64_t n, const int32_t *cells, int64_t cap_cells,
                int32_t count_index, int32_t *vertex_flags, int32_t *faces_out,
                int64_t faces_cap, int64_t *counters, void *workspace,
                size_t workspace_bytes, void *stream);
/* fix_mesh(delete_unused=True) for a duplicate-free, positively oriented
 * cell set (geometry/utils.py:204-249): removes vertices no cell uses,
 * renumbers cells in place (order kept), gathers points_out; synchronises
 * and returns the new vertex count in *n_out_host. */
int dm_compact_workspace_size(int64_t n, size_t *bytes);
int dm_compact_vertices(int32_t dim, const float *points, float *points_out,
                        int64_t n, int32_t *cells, int64_t cap_cells,
                        int32_t count_index, int64_t *counters,
                        int64_t *n_out_host, void *workspace,
                        size_t workspace_bytes, void *stream);
/* simp_vol / simp_qual (geometry/utils.py:175-201, 252-274); either output
 * may be NULL.  Float64 outputs computed from the FP32 points. */
/* calc_re_ratios (geometry/utils.py:17-54): circumradius / shortest edge of
 * each of the nc cells, the radius-edge ratio quality metric; points
 * double[n][dim] on the device, arithmetic in FP64. */
int dm_radius_edge_ratios(int32_t dim, const double *points, const int32_t *cells,
                          int64_t nc, double *ratios, void *stream);
/* Cell quality of the reference's benchmark reports (benchmarks/helpers.py
 * print_stats_2d/3d): quality = dim * inradius / circumradius and, in 3D,
 * the minimum sine of the six dihedral angles divided by the regular
 * tetrahedron's (2 sqrt(2) / 3).  points double[n][dim] on the device;
 * min_sin_dihedral may be NULL (always unused in 2D).  FP64. */
int dm_cell_quality(int32_t dim, const double *points, const int32_t *cells, int64_t nc,
                    double *quality, double *min_sin_dihedral, void *stream);
/* do_any_overlap (geometry/utils.py:745-817): points double[n][dim] and
 * cells int32[nc][dim+1] on the device.  The centroid of every cell is tested
 * against every other cell sharing a vertex with it, in FP64 with the
 * reference's operation order (barycentric coordinates in 2D,
 * calc_4x4determinant signs in 3D, fast_geometry.cpp:482-495).  pairs
 * int32[cap][2] receives (cell, other cell) once per shared vertex, ordered
 * by cell, vertex slot, other cell; *n_pairs (host) is the count.  Blocks
 * the calling thread on the stream.  DM_ERR_CAPACITY, with *n_pairs set,
 * when cap is too small; DM_ERR_ARG for a vertex index outside [0, n). */
int dm_overlap_workspace_size(int32_t dim, int64_t n, int64_t nc, size_t *bytes);
int dm_overlap_pairs(int32_t dim, const double *points, int64_t n, const int32_t *cells,
                     int64_t nc, int32_t *pairs, int64_t cap, int64_t *n_pairs,
                     void *workspace, size_t workspace_bytes, void *stream);
/* simp_vol / simp_qual (geometry/utils.py:175-201, 252-274): signed volume
 * and 2 r / R of the first three vertices; volume or quality may be NULL.
 * dm_simplex_metrics reads engine points (float[n][4] in 3D, float[n][2] in
 * 2D); dm_simplex_metrics_f64 reads caller FP64 points double[n][dim] and
 * stays in FP64 throughout, as the reference does. */
int dm_simplex_metrics(int32_t dim, const float *points, const int32_t *cells,
                       int64_t nc, double *volume, double *quality,
                       void *stream);
int dm_simplex_metrics_f64(int32_t dim, const double *points, const int32_t *cells,
                           int64_t nc, double *volume, double *quality,
                           void *stream);

/* laplacian2_fixed_point (geometry/utils.py:494-547) for 2D points
 * float[n][2] (device, updated in place): interior vertices (boundary_flags
 * 0) move to the solution of deg_i x_i - sum_j x_j = 0 with the boundary
 * vertices fixed; Jacobi-preconditioned CG to relative residual rtol. */
int dm_laplacian_workspace_size(int64_t n, size_t *bytes);
int dm_laplacian_smooth(float *points, int64_t n, const int32_t *adj,
                        int32_t adj_cap, const int32_t *deg,
                        const int32_t *boundary_flags, int32_t max_iter,
                        double rtol, int32_t *iters_host, void *workspace,
                        size_t workspace_bytes, void *stream);

/* ---- isosurface SDF of a gridded field (salt bodies) ---------------------
 * No counterpart in the reference: its domains are analytic primitives and
 * their CSG (geometry/signed_distance_functions.py:307-593).  This is the
 * domain of a body given by a gridded field B (e.g. a salt indicator derived
 * from a velocity model): inside where the piecewise-linear interpolant of B
 * over the Kuhn split of every grid cell (6 tetrahedra along the cell's main
 * diagonal) is >= level.  The surface is extracted by marching tetrahedra;
 * dm_iso_eval returns the exact signed distance to it (negative inside) and
 * its gradient.  All pointers in the struct are device pointers. */
typedef struct dm_iso {
  const float *field;    /* B at the nodes, float[n0][n1][n2], C order      */
  float level;
  int32_t n[3];          /* nodes per axis (>= 2)                           */
  float origin[3];       /* node (0,0,0)                                    */
  float h[3];            /* node spacing                                    */
  const float *tris;     /* float[ntri][3][4]: vertices (x, y, z, 0)        */
  int64_t ntri;
  const int32_t *bstart; /* [nb0*nb1*nb2 + 1] triangles by box (CSR)        */
  const int32_t *btri;   /* [ntri] triangle ids, ascending within a box     */
  const int32_t *bring;  /* [nb] Chebyshev ring of the nearest non-empty box*/
  int32_t nb[3];         /* boxes per axis                                  */
  float bsize[3];        /* box edge lengths (boxes start at origin)        */
  float rho;             /* how far a triangle reaches out of its box       */
  int32_t cf;            /* coarse level: blocks of cf^3 boxes (>= 1)       */
  int32_t ncb[3];        /* blocks per axis: ceil(nb / cf)                  */
  const int32_t *cocc;   /* [ncb] triangles in the block                    */
  const int32_t *cring;  /* [ncb] Chebyshev ring of the nearest non-empty   */
                         /* block                                           */
} dm_iso;
/* triangle count of the surface: rowstart int32[2*(n0-1)*(n1-1) + 1]
 * receives the exclusive scan of the per-row counts in its first
 * (n0-1)*(n1-1) + 1 entries; tmp holds >= 2 (R/1024 + 3) + R/2^20 + 17 ints
 * for R = (n0-1)*(n1-1) rows.
 * Synchronises the stream. */
int dm_iso_count(const dm_iso *iso, int32_t *rowstart, int32_t *tmp,
                 int64_t *ntri_host, void *stream);
/* the triangles, float[ntri][3][4], in a fixed order (row, cell, tet) */
int dm_iso_emit(const dm_iso *iso, const int32_t *rowstart, float *tris,
                void *stream);
/* boxes of the triangles: fills bstart/btri/bring, the coarse level
 * (coarse: int32[2 * ncb0*ncb1*ncb2], occupancy then rings) and iso->rho
 * (host struct updated, stream synchronised); iso->tris, ntri, nb, bsize,
 * cf and ncb are set by the caller.  A query scans the rings of blocks
 * around it and descends only into blocks holding triangles. */
int dm_iso_bucket_workspace_size(int64_t ntri, int64_t n_boxes, size_t *bytes);
int dm_iso_bucket(dm_iso *iso, int32_t *bstart, int32_t *btri, int32_t *bring,
                  int32_t *coarse, void *workspace, size_t workspace_bytes,
                  void *stream);
/* signed distance d[i] (and grad float[n][4], may be NULL) of the points
 * float[n][stride]; with idx only the listed points are evaluated, and with
 * count (device) their number is read on the device (n is then an upper
 * bound used for the launch shape). */
int dm_iso_eval(const dm_iso *iso, const float *points, int32_t stride,
                int64_t n, const int32_t *idx, const int64_t *count,
                float *d, float *grad, void *stream);

/* ---- batched-SDF steps of the DistMesh loop --------------------------------
 * The counterparts of dm_filter_cells and of the projection inside
 * dm_update_points for domains whose distances are computed by a separate
 * batched evaluation (dm_iso_eval, dm_mlp_eval) rather than an inline
 * program: _remove_triangles_outside (generation/mesh_generator.py:734-738)
 * keeps cell c when d[c] < -geps (cells_out, count in
 * counters[DM_CNT_KEPT]); _project_points_back_newton (762-784) moves every
 * point with d > 0 by -d grad (grad float[n][4], unit length, as the exact
 * SDF returns), then rounds to the position grid as dm_update_points does. */
int dm_filter_cells_by_value(int32_t dim, const int32_t *cells, int64_t cap_cells,
                             const float *d, float geps, int32_t *cells_out,
                             int64_t *counters, void *stream);
int dm_project_by_value(int32_t dim, float *points, int64_t n, const float *d,
                        const float *grad, int32_t grid_exp, void *stream);
/* _improve_level_set_newton (generation/mesh_generator.py:741-759) step on
 * the m listed points: p -= alpha d grad, rounded to the position grid */
int dm_newton_by_value(int32_t dim, float *points, const int32_t *idx, int64_t m,
                       const float *d, const float *grad, float alpha, int32_t grid_exp,
                       void *stream);
/* indices i < n with lo < d[i] < hi, appended to idx; *count (device) is
 * set to their number */
int dm_select_band(const float *d, int64_t n, float lo, float hi, int32_t *idx,
                   int64_t *count, void *stream);

/* ---- neural signed distance (Fourier-feature MLP) ------------------------
 * No counterpart in the reference.  A learned stand-in for an expensive SDF
 * (dm_iso): x_n = (x - center) * inv_scale; features sin(2 pi F x_n),
 * cos(2 pi F x_n) for the 32 rows of F; 4 hidden layers of 128 (ReLU);
 * d = out_scale * (w5 . h4 + b5).  Parameters are FP32 (training), with
 * BF16 copies of W1..W4 for the tensor-core inference kernel.
 * Parameter layout (DM_MLP_NPARAMS floats): W1[128][64] b1[128]
 * W2[128][128] b2[128] W3[128][128] b3[128] W4[128][128] b4[128] w5[128]
 * b5[1]. */
#define DM_MLP_NFREQ 32
#define DM_MLP_NFEAT 64
#define DM_MLP_WIDTH 128
#define DM_MLP_NPARAMS (128 * 64 + 128 + 3 * (128 * 128 + 128) + 128 + 1)
#define DM_MLP_NBF16 (128 * 64 + 3 * 128 * 128)
typedef struct dm_mlp {
  float freq[DM_MLP_NFREQ * 3]; /* Fourier frequencies F[32][3] (host values) */
  float center[3];
  float inv_scale;
  float out_scale;
  const float *params;   /* device, DM_MLP_NPARAMS FP32                      */
  const uint16_t *wbf16; /* device, DM_MLP_NBF16 BF16 (W1, W2, W3, W4)       */
} dm_mlp;
/* one training step's gradient: forward and backward of the batch x
 * float[batch][4] against target float[batch] (in units of out_scale) with
 * per-sample weights (may be NULL), loss = sum w (y - t)^2 / batch;
 * grads float[DM_MLP_NPARAMS] (device) receives d loss / d params and
 * loss_dev (device, may be NULL) the loss.  FP32 throughout. */
int dm_mlp_train_workspace_size(int64_t batch, size_t *bytes);
int dm_mlp_forward_backward(const dm_mlp *mlp, const float *x, const float *target,
                            const float *weight, int64_t batch, float *grads,
                            float *loss_dev, void *workspace, size_t workspace_bytes,
                            void *stream);
/* Adam (Kingma & Ba 2015) on n parameters, step t >= 1 */
int dm_mlp_adam(float *params, const float *grads, float *m1, float *m2, int64_t n,
                float lr, float beta1, float beta2, float eps, int32_t t, void *stream);
/* BF16 copies of W1..W4 (round to nearest even) */
int dm_mlp_to_bf16(const float *params, uint16_t *wbf16, void *stream);
/* FP32 forward (the training path's arithmetic): d[i] for points
 * float[n][stride] */
int dm_mlp_eval_fp32(const dm_mlp *mlp, const float *points, int32_t stride, int64_t n,
                     float *d, void *workspace, size_t workspace_bytes, void *stream);
/* inference on the 5th-generation tensor cores: BF16 weights and
 * activations, FP32 accumulation in tensor memory (tcgen05.mma, weights
 * staged by TMA); one persistent CTA per SM.  d[i] for points
 * float[n][stride].  Every wait inside the kernel gives up after 2 s and
 * records it; dm_mlp_eval_status (synchronises the stream) returns 1 in
 * *timed_out_host when that happened since the last status call. */
int dm_mlp_eval(const dm_mlp *mlp, const float *points, int32_t stride, int64_t n,
                float *d, void *stream);
int dm_mlp_eval_status(int32_t *timed_out_host, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DMGB_H */
