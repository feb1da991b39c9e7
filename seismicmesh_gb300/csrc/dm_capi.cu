// extern "C" entry points of libdmgb.so (declared in include/dmgb.h).
#include "dm_common.cuh"
#include "dm_predicates.cuh"
#include "dm_fixed.cuh"

namespace dm {
int delaunay_workspace(int dim, int64_t n, size_t *bytes);
int delaunay(int dim, const float *pts, int64_t n, int32_t *cells,
             int64_t cap_cells, int64_t *counters, void *ws, size_t ws_bytes,
             cudaStream_t s);
int filter_cells(int dim, const float *P, const int32_t *cells, int64_t cap,
                 const dm_sdf_program *sdf, float geps, int32_t *out,
                 int64_t *counters, cudaStream_t s);
int cell_centroids(int dim, const float *P, const int32_t *cells, int64_t cap,
                   const int64_t *counters, float *cen, cudaStream_t s);
size_t adjacency_workspace(int dim, int64_t n, int64_t cap_cells);
int adjacency(int dim, int64_t n, const int32_t *cells, int64_t cap_cells,
              int count_index, int32_t *adj, int adj_cap, int32_t *deg,
              int64_t *counters, void *ws, size_t ws_bytes, cudaStream_t s);
int bar_blocks(int dim, int64_t n);
int bar_sums(int dim, const float *P, int64_t n, const int32_t *adj,
             int adj_cap, const int32_t *deg, const dm_sizing *sz,
             double *partials, cudaStream_t s);
int update_points(int dim, const float *P, float *Pout, int64_t n,
                  const int32_t *adj, int adj_cap, const int32_t *deg,
                  const dm_sizing *sz, const double *partials, float L0mult,
                  float dt, int64_t nfix, const dm_sdf_program *levels,
                  int n_levels, float hmin, float deps, float *maxf,
                  int grid_exp, cudaStream_t s);
int slot_midpoints(int dim, const float *P, int64_t n, const int32_t *adj,
                   int adj_cap, const int32_t *deg, float *mid, cudaStream_t s);
int sdf_eval_launch(const dm_sdf_program *p, const float *x, int64_t n,
                    int stride, float *d, float *grad, cudaStream_t s);
int sizing_eval_launch(const dm_sizing *sz, const float *x, int64_t n,
                       int stride, float *h, cudaStream_t s);
int improve_level_set(int dim, float *P, const int32_t *ids, int64_t m,
                      const dm_sdf_program *sdf, float deps, cudaStream_t s);
int dihedral_angles(const float *P, const int32_t *cells, int64_t nc,
                    double *ang, cudaStream_t s);
int dihedral_angles_f64(const double *X, const int32_t *cells, int64_t nc,
                        double *ang, cudaStream_t s);
int circumsphere_grad(const double *p0, const double *p1, const double *p2,
                      const double *p3, int64_t m, double *g, cudaStream_t s);
int dihedral_flags(const float *P, const int32_t *cells, int64_t cap,
                   int count_index, float amin, float amax, int32_t *flags,
                   int64_t *counters, cudaStream_t s);
int sliver_perturb(float *P, int64_t n_points, const int32_t *cells,
                   int64_t cap, int count_index, const int32_t *flags,
                   float step_h0, int grid_exp, void *ws, size_t ws_bytes,
                   int64_t *counters, cudaStream_t s);
size_t sliver_workspace(int64_t n_points);
int limgrad(const int32_t *dims, double elen, double dfdx, int imax, double *f,
            cudaStream_t s);
int unique_edges_workspace(int64_t n, int64_t m, size_t *bytes);
size_t gradient_term_workspace(int64_t n);
int gradient_term(const double *vp, const int32_t *dims, int dim, const int32_t *window,
                  double scale, double vp_water, int replace, double grad, double *g,
                  void *ws, size_t ws_bytes, cudaStream_t s);
int unique_edges(const int32_t *edges, int64_t m, int64_t n, int32_t *out,
                 int64_t *n_out, void *ws, size_t ws_bytes, cudaStream_t s);
int unique_edges_noalloc(const int32_t *edges, int64_t m, int64_t n,
                         int32_t *out, int64_t *n_out, cudaStream_t s);
size_t boundary_workspace(int dim, int64_t n, int64_t cap_cells);
int boundary(int dim, int64_t n, const int32_t *cells, int64_t cap,
             int count_index, int32_t *vflag, int32_t *faces_out,
             int64_t faces_cap, int64_t *counters, void *ws, size_t ws_bytes,
             cudaStream_t s);
size_t compact_workspace(int64_t n);
int compact_vertices(int dim, const float *P, float *Pout, int64_t n,
                     int32_t *cells, int64_t cap, int count_index,
                     int64_t *counters, int64_t *n_out, void *ws,
                     size_t ws_bytes, cudaStream_t s);
int re_ratios(int dim, const double *P, const int32_t *cells, int64_t nc, double *out,
              cudaStream_t s);
size_t overlap_workspace(int dim, int64_t n, int64_t nc);
int cell_quality(int dim, const double *X, const int32_t *cells, int64_t nc, double *quality,
                 double *min_sin, cudaStream_t s);
int overlap_pairs(int dim, const double *X, int64_t n, const int32_t *cells, int64_t nc,
                  int32_t *pairs, int64_t cap, int64_t *n_pairs, void *ws, size_t ws_bytes,
                  cudaStream_t s);
int simplex_metrics(int dim, const float *P, const int32_t *cells, int64_t nc,
                    double *vol, double *qual, cudaStream_t s);
int simplex_metrics_f64(int dim, const double *X, const int32_t *cells, int64_t nc,
                        double *vol, double *qual, cudaStream_t s);
size_t laplacian_workspace(int64_t n);
struct SizeParams {
  double scale, vp_water;
  int replace;
  double wl, freq, grad, hmin, hmax, dt, cr_max, space_order;
  int dim;
};
int size_from_velocity(double *vp, int64_t n, int64_t row_len,
                       const double *gterm, const SizeParams *sp, double *cell,
                       int *replaced_host, void *ws, cudaStream_t s);
int pad_grid(const double *src, const int *n, const int *pre, const int *post,
             int dim, int mode, double cval, double *dst, cudaStream_t s);
int laplacian_smooth(float *P, int64_t n, const int32_t *adj, int cap,
                     const int32_t *deg, const int32_t *bflag, int max_iter,
                     double rtol, int *iters_out, void *ws, size_t ws_bytes,
                     cudaStream_t s);
int iso_count(const dm_iso *I, int32_t *rowstart, int32_t *tmp, int64_t *ntri, cudaStream_t s);
int iso_emit(const dm_iso *I, const int32_t *rowstart, float *tris, cudaStream_t s);
size_t iso_bucket_workspace(int64_t ntri, int64_t nbk);
int iso_bucket(dm_iso *I, int32_t *bstart, int32_t *btri, int32_t *bring, int32_t *coarse,
               void *ws, size_t ws_bytes, cudaStream_t s);
int iso_eval(const dm_iso *I, const float *pts, int stride, int64_t n, const int32_t *idx,
             const int64_t *count_dev, float *d, float *grad, cudaStream_t s);
int filter_by_value(int dim, const int32_t *cells, int64_t cap, const float *d, float geps,
                    int32_t *out, int64_t *counters, cudaStream_t s);
int project_by_value(int dim, float *P, int64_t n, const float *d, const float *grad,
                     int grid_exp, cudaStream_t s);
int select_band(const float *d, int64_t n, float lo, float hi, int32_t *idx, int64_t *count,
                cudaStream_t s);
int newton_by_value(int dim, float *P, const int32_t *idx, int64_t m, const float *d,
                    const float *grad, float alpha, int grid_exp, cudaStream_t s);
size_t mlp_train_workspace(int64_t batch);
int mlp_forward_backward(const dm_mlp *m, const float *x, const float *target,
                         const float *weight, int64_t batch, float *grads, float *loss,
                         void *ws, size_t ws_bytes, cudaStream_t s);
int mlp_adam(float *params, const float *grads, float *m1, float *m2, int64_t n, float lr,
             float b1, float b2, float eps, int t, cudaStream_t s);
int mlp_to_bf16(const float *params, uint16_t *w, cudaStream_t s);
int mlp_eval_fp32(const dm_mlp *m, const float *pts, int stride, int64_t n, float *d,
                  void *ws, size_t ws_bytes, cudaStream_t s);
int mlp_eval_tc(const dm_mlp *m, const float *pts, int stride, int64_t n, float *d,
                cudaStream_t s);
int mlp_tc_status(cudaStream_t s, int *status);
}  // namespace dm

#define S(x) reinterpret_cast<cudaStream_t>(x)

extern "C" {

int dm_version(void) { return 10000; }
const char *dm_last_error(void) { return dm::last_error(); }
int dm_abi_count(void) { return 63; }

int dm_orient2(const float *a, const float *b, const float *c) {
  dmp::ExactScratch W;
  return dmp::orient2(a, b, c, &W);
}
int dm_orient3(const float *a, const float *b, const float *c, const float *d) {
  dmp::ExactScratch W;
  return dmp::orient3(a, b, c, d, &W);
}
int dm_incircle_sos(const float *a, const float *b, const float *c,
                    const float *d) {
  int ovf = 0;
  dmp::ExactScratch W;
  return dmp::incirc2_sos(a, b, c, d, &ovf, &W);
}
int dm_insphere_sos(const float *a, const float *b, const float *c,
                    const float *d, const float *e) {
  int ovf = 0;
  dmp::ExactScratch W;
  return dmp::insph3_sos(a, b, c, d, e, &ovf, &W);
}

int dm_delaunay_workspace_size(int32_t dim, int64_t n, size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  return dm::delaunay_workspace(dim, n, bytes);
}
int dm_delaunay(int32_t dim, const float *points, int64_t n, int32_t *cells,
                int64_t cap_cells, int64_t *counters, void *workspace,
                size_t workspace_bytes, void *stream) {
  return dm::delaunay(dim, points, n, cells, cap_cells, counters, workspace,
                      workspace_bytes, S(stream));
}

int dm_filter_cells_workspace_size(int64_t cap_cells, size_t *bytes) {
  (void)cap_cells;
  if (!bytes) return DM_ERR_ARG;
  *bytes = 0;
  return DM_OK;
}
int dm_filter_cells(int32_t dim, const float *points, const int32_t *cells,
                    int64_t cap_cells, const dm_sdf_program *sdf, float geps,
                    int32_t *cells_out, int64_t *counters, void *workspace,
                    size_t workspace_bytes, void *stream) {
  (void)workspace;
  (void)workspace_bytes;
  return dm::filter_cells(dim, points, cells, cap_cells, sdf, geps, cells_out,
                          counters, S(stream));
}
int dm_cell_centroids(int32_t dim, const float *points, const int32_t *cells,
                      int64_t cap_cells, const int64_t *counters,
                      float *centroids, void *stream) {
  return dm::cell_centroids(dim, points, cells, cap_cells, counters, centroids,
                            S(stream));
}

int dm_adjacency_workspace_size(int32_t dim, int64_t n, int64_t cap_cells,
                                size_t *bytes) {
  if (!bytes || (dim != 2 && dim != 3) || n < 0 || cap_cells < 0) return DM_ERR_ARG;
  *bytes = dm::adjacency_workspace(dim, n, cap_cells);
  return DM_OK;
}
int dm_adjacency(int32_t dim, int64_t n, const int32_t *cells,
                 int64_t cap_cells, int32_t count_index, int32_t *adj,
                 int32_t adj_cap, int32_t *deg, int64_t *counters,
                 void *workspace, size_t workspace_bytes, void *stream) {
  return dm::adjacency(dim, n, cells, cap_cells, count_index, adj, adj_cap, deg,
                       counters, workspace, workspace_bytes, S(stream));
}

int dm_unique_edges_workspace_size(int64_t n, int64_t m, size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  return dm::unique_edges_workspace(n, m, bytes);
}
int dm_unique_edges(const int32_t *edges, int64_t m, int64_t n, int32_t *out,
                    int64_t *n_out_host, void *workspace,
                    size_t workspace_bytes, void *stream) {
  return dm::unique_edges(edges, m, n, out, n_out_host, workspace,
                          workspace_bytes, S(stream));
}
int dm_unique_edges_noalloc(const int32_t *edges, int64_t m, int64_t n,
                            int32_t *out, int64_t *n_out_host, void *stream) {
  return dm::unique_edges_noalloc(edges, m, n, out, n_out_host, S(stream));
}

int dm_gradient_term_workspace_size(int64_t n, size_t *bytes) {
  if (!bytes || n < 0) return DM_ERR_ARG;
  *bytes = dm::gradient_term_workspace(n);
  return DM_OK;
}
int dm_gradient_term(const double *vp, const int32_t *dims_host, int32_t dim,
                     const int32_t *window_host, double scale, double vp_water,
                     int32_t replace, double grad, double *gradient_term,
                     void *workspace, size_t workspace_bytes, void *stream) {
  return dm::gradient_term(vp, dims_host, dim, window_host, scale, vp_water, replace,
                           grad, gradient_term, workspace, workspace_bytes, S(stream));
}

int dm_bar_blocks(int64_t n, int32_t *nblk) {
  if (!nblk) return DM_ERR_ARG;
  // both dimensions use the same vertices-per-block bound for sizing buffers
  int a = dm::bar_blocks(2, n), b = dm::bar_blocks(3, n);
  *nblk = a > b ? a : b;
  return DM_OK;
}
int dm_bar_sums(int32_t dim, const float *points, int64_t n,
                const int32_t *adj, int32_t adj_cap, const int32_t *deg,
                const dm_sizing *sizing, double *partials, void *stream) {
  return dm::bar_sums(dim, points, n, adj, adj_cap, deg, sizing, partials,
                      S(stream));
}
int dm_update_points(int32_t dim, const float *points, float *points_out,
                     int64_t n, const int32_t *adj, int32_t adj_cap,
                     const int32_t *deg, const dm_sizing *sizing,
                     const double *partials, float L0mult, float delta_t,
                     int64_t nfix, const dm_sdf_program *levels,
                     int32_t n_levels, float hmin, float deps, float *maxf,
                     int32_t grid_exp, void *stream) {
  return dm::update_points(dim, points, points_out, n, adj, adj_cap, deg,
                           sizing, partials, L0mult, delta_t, nfix, levels,
                           n_levels, hmin, deps, maxf, grid_exp, S(stream));
}
int dm_slot_midpoints(int32_t dim, const float *points, int64_t n,
                      const int32_t *adj, int32_t adj_cap, const int32_t *deg,
                      float *mid, void *stream) {
  return dm::slot_midpoints(dim, points, n, adj, adj_cap, deg, mid, S(stream));
}

int dm_sdf_eval(const dm_sdf_program *sdf, const float *x, int64_t n,
                int32_t x_stride, float *d, float *grad, void *stream) {
  return dm::sdf_eval_launch(sdf, x, n, x_stride, d, grad, S(stream));
}
int dm_sizing_eval(const dm_sizing *sizing, const float *x, int64_t n,
                   int32_t x_stride, float *h, void *stream) {
  return dm::sizing_eval_launch(sizing, x, n, x_stride, h, S(stream));
}
int dm_improve_level_set(int32_t dim, float *points, const int32_t *ids,
                         int64_t n_ids, const dm_sdf_program *sdf, float deps,
                         void *stream) {
  return dm::improve_level_set(dim, points, ids, n_ids, sdf, deps, S(stream));
}

int dm_dihedral_angles(const float *points, const int32_t *cells, int64_t nc,
                       double *angles, void *stream) {
  return dm::dihedral_angles(points, cells, nc, angles, S(stream));
}
int dm_dihedral_angles_f64(const double *points, const int32_t *cells, int64_t nc,
                           double *angles, void *stream) {
  return dm::dihedral_angles_f64(points, cells, nc, angles, S(stream));
}
int dm_circumsphere_grad(const double *p0, const double *p1, const double *p2,
                         const double *p3, int64_t m, double *grad,
                         void *stream) {
  return dm::circumsphere_grad(p0, p1, p2, p3, m, grad, S(stream));
}
int dm_dihedral_flags(const float *points, const int32_t *cells,
                      int64_t cap_cells, int32_t count_index, float min_angle,
                      float max_angle, int32_t *flags, int64_t *counters,
                      void *stream) {
  return dm::dihedral_flags(points, cells, cap_cells, count_index, min_angle,
                            max_angle, flags, counters, S(stream));
}
int dm_sliver_workspace_size(int64_t n_points, size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  *bytes = dm::sliver_workspace(n_points);
  return DM_OK;
}
int dm_sliver_perturb(float *points, int64_t n_points, const int32_t *cells,
                      int64_t cap_cells, int32_t count_index,
                      const int32_t *flags, float step_h0, int32_t grid_exp,
                      void *workspace, size_t workspace_bytes,
                      int64_t *counters, void *stream) {
  return dm::sliver_perturb(points, n_points, cells, cap_cells, count_index,
                            flags, step_h0, grid_exp, workspace,
                            workspace_bytes, counters, S(stream));
}

int dm_limgrad(const int32_t *dims, double elen, double dfdx, int32_t imax,
               double *f, void *stream) {
  return dm::limgrad(dims, elen, dfdx, imax, f, S(stream));
}

int dm_boundary_workspace_size(int32_t dim, int64_t n, int64_t cap_cells,
                               size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  *bytes = dm::boundary_workspace(dim, n, cap_cells);
  return DM_OK;
}
int dm_boundary(int32_t dim, int64_t n, const int32_t *cells, int64_t cap_cells,
                int32_t count_index, int32_t *vertex_flags, int32_t *faces_out,
                int64_t faces_cap, int64_t *counters, void *workspace,
                size_t workspace_bytes, void *stream) {
  return dm::boundary(dim, n, cells, cap_cells, count_index, vertex_flags,
                      faces_out, faces_cap, counters, workspace,
                      workspace_bytes, S(stream));
}
int dm_compact_workspace_size(int64_t n, size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  *bytes = dm::compact_workspace(n);
  return DM_OK;
}
int dm_compact_vertices(int32_t dim, const float *points, float *points_out,
                        int64_t n, int32_t *cells, int64_t cap_cells,
                        int32_t count_index, int64_t *counters,
                        int64_t *n_out_host, void *workspace,
                        size_t workspace_bytes, void *stream) {
  return dm::compact_vertices(dim, points, points_out, n, cells, cap_cells,
                              count_index, counters, n_out_host, workspace,
                              workspace_bytes, S(stream));
}
int dm_radius_edge_ratios(int32_t dim, const double *points, const int32_t *cells,
                          int64_t nc, double *ratios, void *stream) {
  return dm::re_ratios(dim, points, cells, nc, ratios, S(stream));
}
int dm_cell_quality(int32_t dim, const double *points, const int32_t *cells, int64_t nc,
                    double *quality, double *min_sin_dihedral, void *stream) {
  return dm::cell_quality(dim, points, cells, nc, quality, min_sin_dihedral, S(stream));
}
int dm_overlap_workspace_size(int32_t dim, int64_t n, int64_t nc, size_t *bytes) {
  DM_ARG_CHECK(bytes && n >= 0 && nc >= 0, "arguments");
  *bytes = dm::overlap_workspace(dim, n, nc);
  return DM_OK;
}
int dm_overlap_pairs(int32_t dim, const double *points, int64_t n, const int32_t *cells,
                     int64_t nc, int32_t *pairs, int64_t cap, int64_t *n_pairs,
                     void *workspace, size_t workspace_bytes, void *stream) {
  return dm::overlap_pairs(dim, points, n, cells, nc, pairs, cap, n_pairs, workspace,
                           workspace_bytes, S(stream));
}
int dm_simplex_metrics(int32_t dim, const float *points, const int32_t *cells,
                       int64_t nc, double *volume, double *quality,
                       void *stream) {
  return dm::simplex_metrics(dim, points, cells, nc, volume, quality, S(stream));
}
int dm_simplex_metrics_f64(int32_t dim, const double *points, const int32_t *cells,
                           int64_t nc, double *volume, double *quality,
                           void *stream) {
  return dm::simplex_metrics_f64(dim, points, cells, nc, volume, quality, S(stream));
}

int dm_laplacian_workspace_size(int64_t n, size_t *bytes) {
  if (!bytes) return DM_ERR_ARG;
  *bytes = dm::laplacian_workspace(n);
  return DM_OK;
}
int dm_laplacian_smooth(float *points, int64_t n, const int32_t *adj,
                        int32_t adj_cap, const int32_t *deg,
                        const int32_t *boundary_flags, int32_t max_iter,
                        double rtol, int32_t *iters_host, void *workspace,
                        size_t workspace_bytes, void *stream) {
  return dm::laplacian_smooth(points, n, adj, adj_cap, deg, boundary_flags,
                              max_iter, rtol, iters_host, workspace,
                              workspace_bytes, S(stream));
}

int dm_size_from_velocity(double *vp, int64_t n, int64_t row_len,
                          const double *gradient_term, double scale,
                          double vp_water, double wl, double freq, double grad,
                          double hmin, double hmax, double dt, double cr_max,
                          double space_order, int32_t dim, double *cell_size,
                          int32_t *replaced_host, void *workspace,
                          size_t workspace_bytes, void *stream) {
  if (!workspace || workspace_bytes < sizeof(int)) {
    dm::set_error("size_from_velocity: workspace must hold 4 bytes");
    return DM_ERR_WORKSPACE;
  }
  dm::SizeParams sp;
  sp.scale = scale;
  sp.vp_water = vp_water;
  sp.replace = 0;
  sp.wl = wl;
  sp.freq = freq;
  sp.grad = grad;
  sp.hmin = hmin;
  sp.hmax = hmax;
  sp.dt = dt;
  sp.cr_max = cr_max;
  sp.space_order = space_order;
  sp.dim = dim;
  return dm::size_from_velocity(vp, n, row_len, gradient_term, &sp, cell_size,
                                replaced_host, workspace, S(stream));
}
int dm_pad_grid(const double *src, const int32_t *n_host,
                const int32_t *pre_host, const int32_t *post_host, int32_t dim,
                int32_t mode, double cval, double *dst, void *stream) {
  return dm::pad_grid(src, n_host, pre_host, post_host, dim, mode, cval, dst,
                      S(stream));
}

}  // extern "C"

// Debug aid (not part of the public ABI): host evaluation of the individual
// predicate stages (0 orient3_exact, 1 orient3_slow, 2 insph3_exact,
// 3 insph3_slow, 4 orient2_exact, 5 incirc2_exact).
// Debug aid: fixed-point predicates on points converted at scale 2^g
// (relative to a).  Returns -99 when a point has no exact representation.
extern "C" int dmdbg_fixed_pred(int kind, int g, const float *a, const float *b,
                                const float *c, const float *d, const float *e) {
  const float *pts[4] = {b, c, d, e};
  int4 q[4];
  int dim = kind >= 2 ? 2 : 3;
  int npts = kind == 0 ? 3 : kind == 1 ? 4 : kind == 2 ? 2 : 3;
  for (int i = 0; i < npts; ++i) {
    long long v[3] = {0, 0, 0};
    for (int k = 0; k < dim; ++k) {
      long long X, P;
      if (!dmp::float_to_fixed(pts[i][k], g, &X) || !dmp::float_to_fixed(a[k], g, &P))
        return -99;
      v[k] = X - P;
      if (v[k] <= -(1ll << 30) || v[k] >= (1ll << 30)) return -99;
    }
    q[i] = make_int4((int)v[0], (int)v[1], (int)v[2], 1);
  }
  switch (kind) {
    case 0: return dmp::orient3_fx(q[0], q[1], q[2]);
    case 1: return dmp::insph3_fx_sos(q[0], q[1], q[2], q[3]);
    case 2: return dmp::orient2_fx(q[0], q[1]);
    case 3: return dmp::incirc2_fx_sos(q[0], q[1], q[2]);
  }
  return -98;
}

extern "C" int dmdbg_host_pred(int kind, const float *a, const float *b,
                               const float *c, const float *d, const float *e) {
  int ovf = 0;
  dmp::ExactScratch W;
  switch (kind) {
    case 0: return dmp::orient3_exact(a, b, c, d, &W);
    case 1: return dmp::orient3_slow(a, b, c, d, &W);
    case 2: return dmp::insph3_exact(a, b, c, d, e, &ovf, &W);
    case 3: return dmp::insph3_slow(a, b, c, d, e, &ovf, &W);
    case 4: return dmp::orient2_exact(a, b, c, &W);
    case 5: return dmp::incirc2_exact(a, b, c, d, &ovf, &W);
  }
  return -99;
}

// ---- isosurface SDF, batched-SDF steps, neural SDF -------------------------
extern "C" {
int dm_iso_count(const dm_iso *iso, int32_t *rowstart, int32_t *tmp, int64_t *ntri_host,
                 void *stream) {
  return dm::iso_count(iso, rowstart, tmp, ntri_host, S(stream));
}
int dm_iso_emit(const dm_iso *iso, const int32_t *rowstart, float *tris, void *stream) {
  return dm::iso_emit(iso, rowstart, tris, S(stream));
}
int dm_iso_bucket_workspace_size(int64_t ntri, int64_t n_boxes, size_t *bytes) {
  if (!bytes || ntri < 0 || n_boxes <= 0) return DM_ERR_ARG;
  *bytes = dm::iso_bucket_workspace(ntri, n_boxes);
  return DM_OK;
}
int dm_iso_bucket(dm_iso *iso, int32_t *bstart, int32_t *btri, int32_t *bring, int32_t *coarse,
                  void *workspace, size_t workspace_bytes, void *stream) {
  return dm::iso_bucket(iso, bstart, btri, bring, coarse, workspace, workspace_bytes, S(stream));
}
int dm_iso_eval(const dm_iso *iso, const float *points, int32_t stride, int64_t n,
                const int32_t *idx, const int64_t *count, float *d, float *grad, void *stream) {
  return dm::iso_eval(iso, points, stride, n, idx, count, d, grad, S(stream));
}
int dm_filter_cells_by_value(int32_t dim, const int32_t *cells, int64_t cap_cells,
                             const float *d, float geps, int32_t *cells_out,
                             int64_t *counters, void *stream) {
  return dm::filter_by_value(dim, cells, cap_cells, d, geps, cells_out, counters, S(stream));
}
int dm_project_by_value(int32_t dim, float *points, int64_t n, const float *d,
                        const float *grad, int32_t grid_exp, void *stream) {
  return dm::project_by_value(dim, points, n, d, grad, grid_exp, S(stream));
}
int dm_newton_by_value(int32_t dim, float *points, const int32_t *idx, int64_t m,
                       const float *d, const float *grad, float alpha, int32_t grid_exp,
                       void *stream) {
  return dm::newton_by_value(dim, points, idx, m, d, grad, alpha, grid_exp, S(stream));
}
int dm_select_band(const float *d, int64_t n, float lo, float hi, int32_t *idx,
                   int64_t *count, void *stream) {
  return dm::select_band(d, n, lo, hi, idx, count, S(stream));
}
int dm_mlp_train_workspace_size(int64_t batch, size_t *bytes) {
  if (!bytes || batch <= 0) return DM_ERR_ARG;
  *bytes = dm::mlp_train_workspace(batch);
  return DM_OK;
}
int dm_mlp_forward_backward(const dm_mlp *mlp, const float *x, const float *target,
                            const float *weight, int64_t batch, float *grads, float *loss_dev,
                            void *workspace, size_t workspace_bytes, void *stream) {
  return dm::mlp_forward_backward(mlp, x, target, weight, batch, grads, loss_dev, workspace,
                                  workspace_bytes, S(stream));
}
int dm_mlp_adam(float *params, const float *grads, float *m1, float *m2, int64_t n, float lr,
                float beta1, float beta2, float eps, int32_t t, void *stream) {
  return dm::mlp_adam(params, grads, m1, m2, n, lr, beta1, beta2, eps, t, S(stream));
}
int dm_mlp_to_bf16(const float *params, uint16_t *wbf16, void *stream) {
  return dm::mlp_to_bf16(params, wbf16, S(stream));
}
int dm_mlp_eval_fp32(const dm_mlp *mlp, const float *points, int32_t stride, int64_t n,
                     float *d, void *workspace, size_t workspace_bytes, void *stream) {
  return dm::mlp_eval_fp32(mlp, points, stride, n, d, workspace, workspace_bytes, S(stream));
}
int dm_mlp_eval(const dm_mlp *mlp, const float *points, int32_t stride, int64_t n, float *d,
                void *stream) {
  return dm::mlp_eval_tc(mlp, points, stride, n, d, S(stream));
}
int dm_mlp_eval_status(int32_t *timed_out_host, void *stream) {
  return dm::mlp_tc_status(S(stream), timed_out_host);
}
}  // extern "C"
