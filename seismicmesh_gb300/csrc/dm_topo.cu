// Mesh topology kernels used once per run (termination) and by the mesh
// utilities: boundary facets, unused-vertex compaction, simplex volumes and
// qualities.
//
// Follows geometry/utils.py: get_boundary_edges 310-326 / get_boundary_facets
// 421-437 (facets that occur once), get_boundary_vertices 364-382,
// fix_mesh 204-249 (delete_unused), simp_vol 175-201, simp_qual 252-274.
#include "dm_common.cuh"

namespace dm {

// faces of a cell: all vertex subsets of size DIM, stored sorted.
// key of a face with sorted vertices (a < b [< c]) is bucketed by a, and
// its remaining vertices packed into 64 bits (b << 32 | c).
template <int DIM>
__device__ __forceinline__ void cell_face(const int32_t *c, int f, int *v) {
  // face f omits vertex f
  int k = 0;
  for (int i = 0; i <= DIM; ++i)
    if (i != f) v[k++] = c[i];
  // sort DIM values
  for (int i = 1; i < DIM; ++i) {
    int x = v[i], j = i - 1;
    while (j >= 0 && v[j] > x) {
      v[j + 1] = v[j];
      --j;
    }
    v[j + 1] = x;
  }
}

template <int DIM>
__global__ void k_face_count(const int32_t *cells, int64_t cap,
                             const int64_t *counters, int count_index,
                             int32_t *cnt, int32_t *slot) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < nc * (DIM + 1); i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = i / (DIM + 1);
    int f = (int)(i % (DIM + 1));
    int v[3];
    cell_face<DIM>(cells + (DIM + 1) * c, f, v);
    slot[i] = atomicAdd(&cnt[v[0]], 1);
  }
}

template <int DIM>
__global__ void k_face_scatter(const int32_t *cells, int64_t cap,
                               const int64_t *counters, int count_index,
                               const int32_t *start, const int32_t *slot,
                               uint64_t *keys) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < nc * (DIM + 1); i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = i / (DIM + 1);
    int f = (int)(i % (DIM + 1));
    int v[3];
    cell_face<DIM>(cells + (DIM + 1) * c, f, v);
    uint64_t key = DIM == 3 ? ((uint64_t)(uint32_t)v[1] << 32) | (uint32_t)v[2]
                            : (uint64_t)(uint32_t)v[1];
    keys[start[v[0]] + slot[i]] = key;
  }
}

// per bucket: sort, find keys that occur once, flag their vertices and
// optionally append the boundary face
template <int DIM>
__global__ void k_face_boundary(int64_t n, const int32_t *start, uint64_t *keys,
                                int32_t *vflag, int32_t *faces_out,
                                int64_t faces_cap, int64_t *counters) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n;
       a += (int64_t)gridDim.x * blockDim.x) {
    int b = start[a], e = start[a + 1];
    for (int i = b + 1; i < e; ++i) {
      uint64_t x = keys[i];
      int j = i - 1;
      while (j >= b && keys[j] > x) {
        keys[j + 1] = keys[j];
        --j;
      }
      keys[j + 1] = x;
    }
    for (int i = b; i < e;) {
      int j = i + 1;
      while (j < e && keys[j] == keys[i]) ++j;
      if (j - i == 1) {
        uint64_t k = keys[i];
        int v1 = DIM == 3 ? (int)(k >> 32) : (int)k;
        int v2 = DIM == 3 ? (int)(uint32_t)k : -1;
        vflag[a] = 1;
        vflag[v1] = 1;
        if (DIM == 3) vflag[v2] = 1;
        if (faces_out) {
          unsigned long long q =
              atomicAdd((unsigned long long *)&counters[DM_CNT_AUX], 1ull);
          if ((int64_t)q < faces_cap) {
            faces_out[DIM * q] = (int)a;
            faces_out[DIM * q + 1] = v1;
            if (DIM == 3) faces_out[DIM * q + 2] = v2;
          }
        }
      }
      i = j;
    }
  }
}

static size_t carve_faces(Carve &c, int64_t n, int64_t nf, int32_t **cnt,
                          int32_t **start, int32_t **slot, uint64_t **keys,
                          int32_t **tmp) {
  *cnt = c.take<int32_t>(n);
  *start = c.take<int32_t>(n + 1);
  *slot = c.take<int32_t>(nf);
  *keys = c.take<uint64_t>(nf);
  *tmp = c.take<int32_t>(scan_tmp_elems(n));
  return c.used;
}

size_t boundary_workspace(int dim, int64_t n, int64_t cap_cells) {
  Carve c(nullptr, 0);
  int32_t *a, *b, *d, *t;
  uint64_t *k;
  return carve_faces(c, n, cap_cells * (dim + 1), &a, &b, &d, &k, &t) + 256;
}

int boundary(int dim, int64_t n, const int32_t *cells, int64_t cap,
             int count_index, int32_t *vflag, int32_t *faces_out,
             int64_t faces_cap, int64_t *counters, void *ws, size_t ws_bytes,
             cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  Carve c(ws, ws_bytes);
  int32_t *cnt, *start, *slot, *tmp;
  uint64_t *keys;
  carve_faces(c, n, cap * (dim + 1), &cnt, &start, &slot, &keys, &tmp);
  if (!c.ok() || !ws) {
    set_error("boundary: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  DM_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n, s));
  DM_CUDA_TRY(cudaMemsetAsync(vflag, 0, sizeof(int32_t) * n, s));
  DM_CUDA_TRY(cudaMemsetAsync(&counters[DM_CNT_AUX], 0, sizeof(int64_t), s));
  int nb = grid_for(cap * (dim + 1), 256);
  if (dim == 3)
    k_face_count<3><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, cnt, slot);
  else
    k_face_count<2><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, cnt, slot);
  int rc = exclusive_scan_i32(cnt, start, n, tmp, s);
  if (rc) return rc;
  if (dim == 3)
    k_face_scatter<3><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, start, slot, keys);
  else
    k_face_scatter<2><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, start, slot, keys);
  int nv = grid_for(n, 128);
  if (dim == 3)
    k_face_boundary<3><<<nv, 128, 0, s>>>(n, start, keys, vflag, faces_out, faces_cap, counters);
  else
    k_face_boundary<2><<<nv, 128, 0, s>>>(n, start, keys, vflag, faces_out, faces_cap, counters);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// ---------------------------------------------------------------------------
// delete unused vertices: used[v] = 1 if v is in a cell; new index by scan;
// cells renumbered in place, points gathered into points_out.
template <int NV>
__global__ void k_mark_used(const int32_t *cells, int64_t cap,
                            const int64_t *counters, int count_index,
                            int32_t *used) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc * NV;
       i += (int64_t)gridDim.x * blockDim.x)
    used[cells[i]] = 1;
}

template <int NV>
__global__ void k_renumber(int32_t *cells, int64_t cap, const int64_t *counters,
                           int count_index, const int32_t *newidx) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc * NV;
       i += (int64_t)gridDim.x * blockDim.x)
    cells[i] = newidx[cells[i]];
}

__global__ void k_gather_points(const float *P, float *Pout, int64_t n, int width,
                                const int32_t *used, const int32_t *newidx) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    if (used[v])
      for (int j = 0; j < width; ++j) Pout[(int64_t)newidx[v] * width + j] = P[v * width + j];
}

size_t compact_workspace(int64_t n) {
  Carve c(nullptr, 0);
  c.take<int32_t>(n);
  c.take<int32_t>(n + 1);
  c.take<int32_t>(scan_tmp_elems(n));
  return c.used + 256;
}

int compact_vertices(int dim, const float *P, float *Pout, int64_t n,
                     int32_t *cells, int64_t cap, int count_index,
                     int64_t *counters, int64_t *n_out, void *ws,
                     size_t ws_bytes, cudaStream_t s) {
  Carve c(ws, ws_bytes);
  int32_t *used = c.take<int32_t>(n);
  int32_t *newidx = c.take<int32_t>(n + 1);
  int32_t *tmp = c.take<int32_t>(scan_tmp_elems(n));
  if (!c.ok() || !ws) {
    set_error("compact: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  DM_CUDA_TRY(cudaMemsetAsync(used, 0, sizeof(int32_t) * n, s));
  int nb = grid_for(cap * (dim + 1), 256);
  if (dim == 3)
    k_mark_used<4><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, used);
  else
    k_mark_used<3><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, used);
  int rc = exclusive_scan_i32(used, newidx, n, tmp, s);
  if (rc) return rc;
  if (dim == 3)
    k_renumber<4><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, newidx);
  else
    k_renumber<3><<<nb, 256, 0, s>>>(cells, cap, counters, count_index, newidx);
  k_gather_points<<<grid_for(n, 256), 256, 0, s>>>(P, Pout, n, dim == 3 ? 4 : 2, used, newidx);
  DM_LAUNCH_CHECK();
  int32_t total = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&total, newidx + n, sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  *n_out = total;
  return DM_OK;
}

// ---------------------------------------------------------------------------
// simplex signed volume and simp_qual (2 * inradius / circumradius of the
// triangle formed by the first three vertices)
template <int DIM>
__device__ __forceinline__ void load_vertex(const float *P, int64_t v, double *x) {
  if (DIM == 3) {
    float4 q = reinterpret_cast<const float4 *>(P)[v];
    x[0] = q.x;
    x[1] = q.y;
    x[2] = q.z;
  } else {
    float2 q = reinterpret_cast<const float2 *>(P)[v];
    x[0] = q.x;
    x[1] = q.y;
  }
}
// caller FP64 points: DIM doubles per row
template <int DIM>
__device__ __forceinline__ void load_vertex(const double *X, int64_t v, double *x) {
  for (int d = 0; d < DIM; ++d) x[d] = X[v * DIM + d];
}

template <int DIM, typename PT>
__global__ void k_simplex_metrics(const PT *P, const int32_t *cells,
                                  int64_t nc, double *vol, double *qual) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[4][3] = {};
    for (int k = 0; k <= DIM; ++k) load_vertex<DIM>(P, cells[(DIM + 1) * c + k], x[k]);
    if (vol) {
      double d1[3], d2[3], d3[3];
      for (int j = 0; j < 3; ++j) {
        d1[j] = x[1][j] - x[0][j];
        d2[j] = x[2][j] - x[0][j];
        d3[j] = x[DIM == 3 ? 3 : 0][j] - x[0][j];
      }
      if (DIM == 2)
        vol[c] = (d1[0] * d2[1] - d1[1] * d2[0]) / 2;
      else
        vol[c] = ((d1[1] * d2[2] - d1[2] * d2[1]) * d3[0] +
                  (d1[2] * d2[0] - d1[0] * d2[2]) * d3[1] +
                  (d1[0] * d2[1] - d1[1] * d2[0]) * d3[2]) / 6;
    }
    if (qual) {
      auto len = [&](int i, int j) {
        double s = 0;
        for (int k = 0; k < DIM; ++k) s += (x[i][k] - x[j][k]) * (x[i][k] - x[j][k]);
        return sqrt(s);
      };
      double a = len(1, 0), b = len(2, 0), cc = len(2, 1);
      double r = 0.5 * sqrt((b + cc - a) * (cc + a - b) * (a + b - cc) / (a + b + cc));
      double R = a * b * cc / sqrt((a + b + cc) * (b + cc - a) * (cc + a - b) * (a + b - cc));
      qual[c] = 2 * r / R;
    }
  }
}

// calc_re_ratios (geometry/utils.py:17-54): circumradius / shortest edge of
// each simplex, in FP64 (circumcentre from the normal equations of the edge
// vectors relative to the first vertex)
template <int DIM>
__global__ void k_re_ratios(const double *X, const int32_t *cells, int64_t nc, double *out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[4][3] = {};
    for (int k = 0; k <= DIM; ++k) {
      const int64_t v = cells[(DIM + 1) * c + k];
      for (int d = 0; d < DIM; ++d) x[k][d] = X[v * DIM + d];
    }
    double minl2 = 1e300;
    for (int i = 0; i <= DIM; ++i)
      for (int j = i + 1; j <= DIM; ++j) {
        double l2 = 0;
        for (int k = 0; k < DIM; ++k) l2 += (x[i][k] - x[j][k]) * (x[i][k] - x[j][k]);
        minl2 = fmin(minl2, l2);
      }
    double r2;
    if (DIM == 2) {
      double a0 = x[1][0] - x[0][0], a1 = x[1][1] - x[0][1];
      double b0 = x[2][0] - x[0][0], b1 = x[2][1] - x[0][1];
      double d = 2 * (a0 * b1 - a1 * b0);
      double la = a0 * a0 + a1 * a1, lb = b0 * b0 + b1 * b1;
      double ux = (b1 * la - a1 * lb) / d, uy = (a0 * lb - b0 * la) / d;
      r2 = ux * ux + uy * uy;
    } else {
      double a[3], b[3], e[3];
      for (int k = 0; k < 3; ++k) {
        a[k] = x[1][k] - x[0][k];
        b[k] = x[2][k] - x[0][k];
        e[k] = x[3][k] - x[0][k];
      }
      double bc[3] = {b[1] * e[2] - b[2] * e[1], b[2] * e[0] - b[0] * e[2], b[0] * e[1] - b[1] * e[0]};
      double ca[3] = {e[1] * a[2] - e[2] * a[1], e[2] * a[0] - e[0] * a[2], e[0] * a[1] - e[1] * a[0]};
      double ab[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
      double det = 2 * (a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2]);
      double la = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
      double lb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
      double le = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
      r2 = 0;
      for (int k = 0; k < 3; ++k) {
        double u = (la * bc[k] + lb * ca[k] + le * ab[k]) / det;
        r2 += u * u;
      }
    }
    out[c] = sqrt(r2) / sqrt(minl2);
  }
}

int re_ratios(int dim, const double *P, const int32_t *cells, int64_t nc, double *out,
              cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(nc >= 0 && (nc == 0 || (P && cells && out)), "arguments");
  if (nc == 0) return DM_OK;
  if (dim == 3)
    k_re_ratios<3><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, out);
  else
    k_re_ratios<2><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, out);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

template <typename PT>
static int simplex_metrics_t(int dim, const PT *P, const int32_t *cells, int64_t nc,
                             double *vol, double *qual, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  if (nc == 0) return DM_OK;
  if (dim == 3)
    k_simplex_metrics<3, PT><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, vol, qual);
  else
    k_simplex_metrics<2, PT><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, vol, qual);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int simplex_metrics(int dim, const float *P, const int32_t *cells, int64_t nc,
                    double *vol, double *qual, cudaStream_t s) {
  return simplex_metrics_t(dim, P, cells, nc, vol, qual, s);
}

int simplex_metrics_f64(int dim, const double *X, const int32_t *cells, int64_t nc,
                        double *vol, double *qual, cudaStream_t s) {
  return simplex_metrics_t(dim, X, cells, nc, vol, qual, s);
}

}  // namespace dm

namespace dm {

// ---------------------------------------------------------------------------
// laplacian2_fixed_point (geometry/utils.py:494-547): solve the graph
// Laplacian with Dirichlet rows on the boundary vertices,
//   interior i:  deg_i x_i - sum_j x_j = 0,   boundary b:  x_b = p_b.
// The reference assembles it from triangle edges (interior edges weigh 2 on
// both sides of every interior row, so the rows are the unweighted graph
// Laplacian) and solves with algebraic multigrid.  Here: Jacobi-
// preconditioned conjugate gradients on the symmetric interior system, both
// coordinates at once, on the device.
struct LapState {
  double2 *x, *r, *z, *p, *q;
  double *part;  // per-block partial sums: [nblk][4]
  double *sc;    // scalars: rz.x rz.y alpha.x alpha.y beta.x beta.y rr.x rr.y rr0
};

__device__ __forceinline__ void block_sum4(double *v, double *out) {
  __shared__ double sh[4][8];
  for (int k = 0; k < 4; ++k)
    for (int o = 16; o; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int k = 0; k < 4; ++k) sh[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; ++k) {
      double s = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[k][i];
      out[k] = s;
    }
  __syncthreads();
}

__global__ void k_lap_init(const float *P, int64_t n, const int32_t *adj,
                           int cap, const int32_t *deg, const int32_t *bflag,
                           LapState S) {
  double acc[4] = {0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float2 pi = reinterpret_cast<const float2 *>(P)[i];
    S.x[i] = make_double2(pi.x, pi.y);
    double2 r = make_double2(0, 0), z = r;
    if (!bflag[i] && deg[i] > 0) {
      double sx = 0, sy = 0;
      for (int k = 0; k < deg[i]; ++k) {
        float2 pj = reinterpret_cast<const float2 *>(P)[adj[i * cap + k]];
        sx += pj.x;
        sy += pj.y;
      }
      r = make_double2(sx - deg[i] * (double)pi.x, sy - deg[i] * (double)pi.y);
      z = make_double2(r.x / deg[i], r.y / deg[i]);
    }
    S.r[i] = r;
    S.z[i] = z;
    S.p[i] = z;
    acc[0] += r.x * z.x;
    acc[1] += r.y * z.y;
    acc[2] += r.x * r.x;
    acc[3] += r.y * r.y;
  }
  block_sum4(acc, S.part + 4 * blockIdx.x);
}

// q = A_II p, partial p.q
__global__ void k_lap_spmv(int64_t n, const int32_t *adj, int cap,
                           const int32_t *deg, const int32_t *bflag, LapState S) {
  double acc[4] = {0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 q = make_double2(0, 0);
    if (!bflag[i] && deg[i] > 0) {
      double2 pi = S.p[i];
      double sx = 0, sy = 0;
      for (int k = 0; k < deg[i]; ++k) {
        int j = adj[i * cap + k];
        if (bflag[j]) continue;
        double2 pj = S.p[j];
        sx += pj.x;
        sy += pj.y;
      }
      q = make_double2(deg[i] * pi.x - sx, deg[i] * pi.y - sy);
      acc[0] += pi.x * q.x;
      acc[1] += pi.y * q.y;
    }
    S.q[i] = q;
  }
  block_sum4(acc, S.part + 4 * blockIdx.x);
}

// reduce partials; mode 0: init (rz, rr0), 1: alpha = rz / pq, 2: beta
__global__ void k_lap_scalars(LapState S, int nblk, int mode) {
  __shared__ double sh[4][1024];
  double a[4] = {0, 0, 0, 0};
  for (int i = threadIdx.x; i < nblk; i += blockDim.x)
    for (int k = 0; k < 4; ++k) a[k] += S.part[4 * i + k];
  for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < 4; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  double t0 = sh[0][0], t1 = sh[1][0], t2 = sh[2][0], t3 = sh[3][0];
  if (mode == 0) {
    S.sc[0] = t0;
    S.sc[1] = t1;
    S.sc[6] = t2;
    S.sc[7] = t3;
    S.sc[8] = fmax(t2 + t3, 1e-300);
  } else if (mode == 1) {
    S.sc[2] = t0 > 0 ? S.sc[0] / t0 : 0;
    S.sc[3] = t1 > 0 ? S.sc[1] / t1 : 0;
  } else {
    S.sc[4] = S.sc[0] > 0 ? t0 / S.sc[0] : 0;
    S.sc[5] = S.sc[1] > 0 ? t1 / S.sc[1] : 0;
    S.sc[0] = t0;
    S.sc[1] = t1;
    S.sc[6] = t2;
    S.sc[7] = t3;
  }
}

__global__ void k_lap_update(int64_t n, const int32_t *deg,
                             const int32_t *bflag, LapState S) {
  double ax = S.sc[2], ay = S.sc[3];
  double acc[4] = {0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (bflag[i] || deg[i] == 0) continue;
    double2 x = S.x[i], r = S.r[i], p = S.p[i], q = S.q[i];
    x.x += ax * p.x;
    x.y += ay * p.y;
    r.x -= ax * q.x;
    r.y -= ay * q.y;
    double2 z = make_double2(r.x / deg[i], r.y / deg[i]);
    S.x[i] = x;
    S.r[i] = r;
    S.z[i] = z;
    acc[0] += r.x * z.x;
    acc[1] += r.y * z.y;
    acc[2] += r.x * r.x;
    acc[3] += r.y * r.y;
  }
  block_sum4(acc, S.part + 4 * blockIdx.x);
}

__global__ void k_lap_dir(int64_t n, LapState S) {
  double bx = S.sc[4], by = S.sc[5];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 z = S.z[i], p = S.p[i];
    S.p[i] = make_double2(z.x + bx * p.x, z.y + by * p.y);
  }
}

__global__ void k_lap_write(float *P, int64_t n, LapState S) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double2 x = S.x[i];
    reinterpret_cast<float2 *>(P)[i] = make_float2((float)x.x, (float)x.y);
  }
}

size_t laplacian_workspace(int64_t n) {
  Carve c(nullptr, 0);
  for (int k = 0; k < 5; ++k) c.take<double2>(n);
  c.take<double>(4 * (size_t)grid_for(n, 256) + 4);
  c.take<double>(16);
  return c.used + 256;
}

int laplacian_smooth(float *P, int64_t n, const int32_t *adj, int cap,
                     const int32_t *deg, const int32_t *bflag, int max_iter,
                     double rtol, int *iters_out, void *ws, size_t ws_bytes,
                     cudaStream_t s) {
  Carve c(ws, ws_bytes);
  LapState S;
  S.x = c.take<double2>(n);
  S.r = c.take<double2>(n);
  S.z = c.take<double2>(n);
  S.p = c.take<double2>(n);
  S.q = c.take<double2>(n);
  int nblk = grid_for(n, 256);
  S.part = c.take<double>(4 * (size_t)nblk + 4);
  S.sc = c.take<double>(16);
  if (!c.ok() || !ws) {
    set_error("laplacian: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  k_lap_init<<<nblk, 256, 0, s>>>(P, n, adj, cap, deg, bflag, S);
  k_lap_scalars<<<1, 1024, 0, s>>>(S, nblk, 0);
  int it = 0;
  double hs[16];
  for (; it < max_iter; ++it) {
    k_lap_spmv<<<nblk, 256, 0, s>>>(n, adj, cap, deg, bflag, S);
    k_lap_scalars<<<1, 1024, 0, s>>>(S, nblk, 1);
    k_lap_update<<<nblk, 256, 0, s>>>(n, deg, bflag, S);
    k_lap_scalars<<<1, 1024, 0, s>>>(S, nblk, 2);
    k_lap_dir<<<nblk, 256, 0, s>>>(n, S);
    if ((it & 15) == 15) {
      DM_CUDA_TRY(cudaMemcpyAsync(hs, S.sc, sizeof(double) * 16,
                                  cudaMemcpyDeviceToHost, s));
      DM_CUDA_TRY(cudaStreamSynchronize(s));
      if (hs[6] + hs[7] <= rtol * rtol * hs[8]) {
        ++it;
        break;
      }
    }
  }
  k_lap_write<<<nblk, 256, 0, s>>>(P, n, S);
  DM_LAUNCH_CHECK();
  if (iters_out) *iters_out = it;
  if (it >= max_iter) {
    set_error("laplacian: no convergence in %d iterations", max_iter);
    return DM_ERR_NOT_CONVERGED;
  }
  return DM_OK;
}

}  // namespace dm

namespace dm {

// ---------------------------------------------------------------------------
// do_any_overlap (geometry/utils.py:745-817): the centroid of every cell is
// tested against every other cell in its 1-ring (the cells sharing one of its
// vertices, vertex_to_entities 97-130).  The arithmetic follows the
// reference operation by operation in FP64 with explicit round-to-nearest
// intrinsics, so no multiply-add is contracted and every decision matches
// the reference's double-precision evaluation:
//   centroid      get_centroids 729-742: ((v0 + v1) + v2 [+ v3]) / (dim + 1)
//   2D inclusion  vertex_in_entity2 657-679: barycentric a, b, c = 1 - a - b,
//                 all three in [0, 1]
//   3D inclusion  vertex_in_entity3 682-726: the five 4x4 determinants of
//                 calc_4x4determinant (fast_geometry.cpp:482-495), each
//                 summed left to right, must share one non-zero sign
// A pair (ie, ele) is reported once per vertex the two cells share, as the
// reference's loop over the vertices of ie does; pairs are ordered by ie,
// then by the vertex slot in ie, then by ele.

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// calc_4x4determinant on a row-major 4x4 matrix: 24 four-factor products,
// each multiplied left to right, accumulated left to right with the signs
// of the reference expression
__device__ double det4x4_ref(const double *m) {
  // {i0, i1, i2, i3, sign}
  constexpr int T[24][5] = {
      {12, 9, 6, 3, 1},    {8, 13, 6, 3, -1},   {12, 5, 10, 3, -1},  {4, 13, 10, 3, 1},
      {8, 5, 14, 3, 1},    {4, 9, 14, 3, -1},   {12, 9, 2, 7, -1},   {8, 13, 2, 7, 1},
      {12, 1, 10, 7, 1},   {0, 13, 10, 7, -1},  {8, 1, 14, 7, -1},   {0, 9, 14, 7, 1},
      {12, 5, 2, 11, 1},   {4, 13, 2, 11, -1},  {12, 1, 6, 11, -1},  {0, 13, 6, 11, 1},
      {4, 1, 14, 11, 1},   {0, 5, 14, 11, -1},  {8, 5, 2, 15, -1},   {4, 9, 2, 15, 1},
      {8, 1, 6, 15, 1},    {0, 9, 6, 15, -1},   {4, 1, 10, 15, -1},  {0, 5, 10, 15, 1}};
  double s = 0;
#pragma unroll
  for (int k = 0; k < 24; ++k) {
    double t = dmul(dmul(dmul(m[T[k][0]], m[T[k][1]]), m[T[k][2]]), m[T[k][3]]);
    s = k == 0 ? t : (T[k][4] > 0 ? dadd(s, t) : dsub(s, t));
  }
  return s;
}

__device__ __forceinline__ int sign_d(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

template <int DIM>
__device__ void centroid_ref(const double *X, const int32_t *c, double *cent) {
  for (int d = 0; d < DIM; ++d) {
    double s = X[(int64_t)c[0] * DIM + d];
    for (int k = 1; k <= DIM; ++k) s = dadd(s, X[(int64_t)c[k] * DIM + d]);
    cent[d] = __ddiv_rn(s, (double)(DIM + 1));
  }
}

template <int DIM>
__device__ bool inside_ref(const double *X, const int32_t *c, const double *q) {
  if (DIM == 2) {
    const double x1 = X[2 * (int64_t)c[0]], y1 = X[2 * (int64_t)c[0] + 1];
    const double x2 = X[2 * (int64_t)c[1]], y2 = X[2 * (int64_t)c[1] + 1];
    const double x3 = X[2 * (int64_t)c[2]], y3 = X[2 * (int64_t)c[2] + 1];
    const double x = q[0], y = q[1];
    const double den = dadd(dmul(dsub(y2, y3), dsub(x1, x3)), dmul(dsub(x3, x2), dsub(y1, y3)));
    const double a =
        __ddiv_rn(dadd(dmul(dsub(y2, y3), dsub(x, x3)), dmul(dsub(x3, x2), dsub(y, y3))), den);
    const double b =
        __ddiv_rn(dadd(dmul(dsub(y3, y1), dsub(x, x3)), dmul(dsub(x1, x3), dsub(y, y3))), den);
    const double cc = dsub(dsub(1.0, a), b);
    return 0 <= a && a <= 1 && 0 <= b && b <= 1 && 0 <= cc && cc <= 1;
  } else {
    double m[16];
    for (int r = 0; r < 4; ++r) {
      for (int d = 0; d < 3; ++d) m[4 * r + d] = X[3 * (int64_t)c[r] + d];
      m[4 * r + 3] = 1.0;
    }
    const int s0 = sign_d(det4x4_ref(m));
    int prev = s0;
    for (int r = 0; r < 4; ++r) {
      double save[3];
      for (int d = 0; d < 3; ++d) {
        save[d] = m[4 * r + d];
        m[4 * r + d] = q[d];
      }
      const int s = sign_d(det4x4_ref(m));
      for (int d = 0; d < 3; ++d) m[4 * r + d] = save[d];
      if (s != prev) return false;
      prev = s;
    }
    return s0 != 0;
  }
}

__global__ void k_v2c_count(const int32_t *cells, int64_t ne, int64_t n, int32_t *cnt,
                            int32_t *status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = cells[i];
    if (v < 0 || v >= n)
      atomicOr(status, 1);
    else
      atomicAdd(&cnt[v], 1);
  }
}

__global__ void k_v2c_fill(const int32_t *cells, int64_t ne, int nv, int64_t n,
                           const int32_t *ptr, int32_t *cursor, int32_t *vtoe) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = cells[i];
    if (v < 0 || v >= n) continue;
    vtoe[ptr[v] + atomicAdd(&cursor[v], 1)] = (int32_t)(i / nv);
  }
}

// each row ascending (insertion sort; rows are the cells around one vertex)
__global__ void k_v2c_sort(int64_t n, const int32_t *ptr, int32_t *vtoe) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int32_t b = ptr[v], e = ptr[v + 1];
    for (int32_t i = b + 1; i < e; ++i) {
      const int32_t x = vtoe[i];
      int32_t j = i - 1;
      while (j >= b && vtoe[j] > x) {
        vtoe[j + 1] = vtoe[j];
        --j;
      }
      vtoe[j + 1] = x;
    }
  }
}

// FILL = false: count the pairs of every cell; true: write them at ptr[ie]
template <int DIM, bool FILL>
__global__ void k_overlap(const double *X, const int32_t *cells, int64_t nc,
                          const int32_t *vptr, const int32_t *vtoe, int32_t *cnt,
                          const int32_t *cptr, int32_t *pairs) {
  for (int64_t ie = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; ie < nc;
       ie += (int64_t)gridDim.x * blockDim.x) {
    const int32_t *c = cells + (DIM + 1) * ie;
    double cent[DIM];
    centroid_ref<DIM>(X, c, cent);
    int32_t k = 0;
    const int32_t base = FILL ? cptr[ie] : 0;
    for (int s = 0; s <= DIM; ++s) {
      const int32_t v = c[s];
      for (int32_t j = vptr[v]; j < vptr[v + 1]; ++j) {
        const int32_t ele = vtoe[j];
        if (ele == ie) continue;
        if (inside_ref<DIM>(X, cells + (int64_t)(DIM + 1) * ele, cent)) {
          if (FILL) {
            pairs[2 * (int64_t)(base + k)] = (int32_t)ie;
            pairs[2 * (int64_t)(base + k) + 1] = ele;
          }
          ++k;
        }
      }
    }
    if (!FILL) cnt[ie] = k;
  }
}

struct OverlapWs {
  int32_t *vcnt, *vptr, *cursor, *vtoe, *ccnt, *cptr, *tmp, *status;
};

static size_t carve_overlap(Carve &c, int dim, int64_t n, int64_t nc, OverlapWs &w) {
  w.vcnt = c.take<int32_t>(n + 1);
  w.vptr = c.take<int32_t>(n + 1);
  w.cursor = c.take<int32_t>(n + 1);
  w.vtoe = c.take<int32_t>(nc * (dim + 1) + 1);
  w.ccnt = c.take<int32_t>(nc + 1);
  w.cptr = c.take<int32_t>(nc + 1);
  w.tmp = c.take<int32_t>(scan_tmp_elems(n > nc ? n + 1 : nc + 1));
  w.status = c.take<int32_t>(4);
  return c.used;
}

size_t overlap_workspace(int dim, int64_t n, int64_t nc) {
  Carve c(nullptr, 0);
  OverlapWs w;
  return carve_overlap(c, dim, n, nc, w) + 256;
}

int overlap_pairs(int dim, const double *X, int64_t n, const int32_t *cells, int64_t nc,
                  int32_t *pairs, int64_t cap, int64_t *n_pairs, void *ws, size_t ws_bytes,
                  cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(n >= 0 && nc >= 0 && cap >= 0 && n_pairs, "arguments");
  DM_ARG_CHECK(nc == 0 || (X && cells), "null points or cells");
  DM_ARG_CHECK(cap == 0 || pairs, "null pairs");
  *n_pairs = 0;
  if (nc == 0) return DM_OK;
  Carve c(ws, ws_bytes);
  OverlapWs w;
  carve_overlap(c, dim, n, nc, w);
  if (!c.ok() || !ws) {
    set_error("overlap_pairs: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  const int nv = dim + 1;
  const int64_t ne = nc * nv;
  DM_CUDA_TRY(cudaMemsetAsync(w.vcnt, 0, sizeof(int32_t) * (n + 1), s));
  DM_CUDA_TRY(cudaMemsetAsync(w.cursor, 0, sizeof(int32_t) * (n + 1), s));
  DM_CUDA_TRY(cudaMemsetAsync(w.status, 0, sizeof(int32_t) * 4, s));
  k_v2c_count<<<grid_for(ne, 256), 256, 0, s>>>(cells, ne, n, w.vcnt, w.status);
  int rc = exclusive_scan_i32(w.vcnt, w.vptr, n, w.tmp, s);
  if (rc) return rc;
  k_v2c_fill<<<grid_for(ne, 256), 256, 0, s>>>(cells, ne, nv, n, w.vptr, w.cursor, w.vtoe);
  k_v2c_sort<<<grid_for(n, 128), 128, 0, s>>>(n, w.vptr, w.vtoe);
  int32_t status = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&status, w.status, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  if (status) {
    set_error("overlap_pairs: a cell vertex is outside [0, %lld)", (long long)n);
    return DM_ERR_ARG;
  }
  const int nb = grid_for(nc, 128);
  if (dim == 3)
    k_overlap<3, false><<<nb, 128, 0, s>>>(X, cells, nc, w.vptr, w.vtoe, w.ccnt, nullptr, nullptr);
  else
    k_overlap<2, false><<<nb, 128, 0, s>>>(X, cells, nc, w.vptr, w.vtoe, w.ccnt, nullptr, nullptr);
  rc = exclusive_scan_i32(w.ccnt, w.cptr, nc, w.tmp, s);
  if (rc) return rc;
  int32_t total = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&total, w.cptr + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  *n_pairs = total;
  if (total > cap) {
    set_error("overlap_pairs: %d pairs exceed capacity %lld", total, (long long)cap);
    return DM_ERR_CAPACITY;
  }
  if (total == 0) return DM_OK;
  if (dim == 3)
    k_overlap<3, true><<<nb, 128, 0, s>>>(X, cells, nc, w.vptr, w.vtoe, nullptr, w.cptr, pairs);
  else
    k_overlap<2, true><<<nb, 128, 0, s>>>(X, cells, nc, w.vptr, w.vtoe, nullptr, w.cptr, pairs);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

}  // namespace dm

namespace dm {

// ---------------------------------------------------------------------------
// Cell quality of the reference's benchmark reports (benchmarks/helpers.py
// print_stats_2d / print_stats_3d, which take meshplex's cell_quality and
// q_min_sin_dihedral_angles), in FP64:
//   quality   = dim * inradius / circumradius   (1 for the regular simplex)
//             inradius = dim * volume / (sum of facet measures)
//   3D        sin of the dihedral angle at edge (i, j), whose two faces are
//             the ones opposite the other two vertices k, l:
//               sin = 3 V |x_i - x_j| / (2 A_k A_l)
//             min over the six edges / sin(regular) = min / (2 sqrt(2) / 3)
template <int DIM>
__global__ void k_cell_quality(const double *X, const int32_t *cells, int64_t nc,
                               double *quality, double *min_sin) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[DIM + 1][DIM];
    for (int k = 0; k <= DIM; ++k) {
      const int64_t v = cells[(DIM + 1) * c + k];
      for (int d = 0; d < DIM; ++d) x[k][d] = X[v * DIM + d];
    }
    if (DIM == 2) {
      double l[3];
      for (int k = 0; k < 3; ++k) {
        const double dx = x[(k + 1) % 3][0] - x[(k + 2) % 3][0];
        const double dy = x[(k + 1) % 3][1] - x[(k + 2) % 3][1];
        l[k] = sqrt(dx * dx + dy * dy);
      }
      const double area = 0.5 * fabs((x[1][0] - x[0][0]) * (x[2][1] - x[0][1]) -
                                     (x[1][1] - x[0][1]) * (x[2][0] - x[0][0]));
      const double r = 2 * area / (l[0] + l[1] + l[2]);
      const double R = l[0] * l[1] * l[2] / (4 * area);
      quality[c] = 2 * r / R;
    } else {
      double e[4][4][3];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          for (int d = 0; d < 3; ++d) e[i][j][d] = x[j][d] - x[i][d];
      // facet areas: A[k] = area of the face opposite vertex k
      double A[4];
      for (int k = 0; k < 4; ++k) {
        const int a = (k + 1) & 3, b = (k + 2) & 3, cc = (k + 3) & 3;
        const double *u = e[a][b], *w = e[a][cc];
        const double n0 = u[1] * w[2] - u[2] * w[1], n1 = u[2] * w[0] - u[0] * w[2],
                     n2 = u[0] * w[1] - u[1] * w[0];
        A[k] = 0.5 * sqrt(n0 * n0 + n1 * n1 + n2 * n2);
      }
      const double *a = e[0][1], *b = e[0][2], *d = e[0][3];
      const double det = a[0] * (b[1] * d[2] - b[2] * d[1]) - a[1] * (b[0] * d[2] - b[2] * d[0]) +
                         a[2] * (b[0] * d[1] - b[1] * d[0]);
      const double V = fabs(det) / 6;
      const double r = 3 * V / (A[0] + A[1] + A[2] + A[3]);
      // circumradius: |u| with u = (la (b x d) + lb (d x a) + ld (a x b)) / (2 det)
      const double la = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
      const double lb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
      const double ld = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      double R2 = 0;
      for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        const double bd = b[k1] * d[k2] - b[k2] * d[k1];
        const double da = d[k1] * a[k2] - d[k2] * a[k1];
        const double ab = a[k1] * b[k2] - a[k2] * b[k1];
        const double u = (la * bd + lb * da + ld * ab) / (2 * det);
        R2 += u * u;
      }
      quality[c] = 3 * r / sqrt(R2);
      if (min_sin) {
        double m = 1e300;
        for (int i = 0; i < 4; ++i)
          for (int j = i + 1; j < 4; ++j) {
            int k = -1, l = -1;
            for (int q = 0; q < 4; ++q)
              if (q != i && q != j) (k < 0 ? k : l) = q;
            const double *g = e[i][j];
            const double len = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
            m = fmin(m, 3 * V * len / (2 * A[k] * A[l]));
          }
        min_sin[c] = m / (2 * 1.4142135623730951 / 3);
      }
    }
  }
}

int cell_quality(int dim, const double *X, const int32_t *cells, int64_t nc, double *quality,
                 double *min_sin, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(nc >= 0 && (nc == 0 || (X && cells && quality)), "arguments");
  if (nc == 0) return DM_OK;
  if (dim == 3)
    k_cell_quality<3><<<grid_for(nc, 128), 128, 0, s>>>(X, cells, nc, quality, min_sin);
  else
    k_cell_quality<2><<<grid_for(nc, 128), 128, 0, s>>>(X, cells, nc, quality, nullptr);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

}  // namespace dm
