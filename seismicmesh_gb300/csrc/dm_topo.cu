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
__global__ void k_simplex_metrics(const float *P, const int32_t *cells,
                                  int64_t nc, double *vol, double *qual) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[4][3] = {};
    for (int k = 0; k <= DIM; ++k) {
      int v = cells[(DIM + 1) * c + k];
      if (DIM == 3) {
        float4 q = reinterpret_cast<const float4 *>(P)[v];
        x[k][0] = q.x;
        x[k][1] = q.y;
        x[k][2] = q.z;
      } else {
        float2 q = reinterpret_cast<const float2 *>(P)[v];
        x[k][0] = q.x;
        x[k][1] = q.y;
      }
    }
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

int simplex_metrics(int dim, const float *P, const int32_t *cells, int64_t nc,
                    double *vol, double *qual, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  if (nc == 0) return DM_OK;
  if (dim == 3)
    k_simplex_metrics<3><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, vol, qual);
  else
    k_simplex_metrics<2><<<grid_for(nc, 256), 256, 0, s>>>(P, cells, nc, vol, qual);
  DM_LAUNCH_CHECK();
  return DM_OK;
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
