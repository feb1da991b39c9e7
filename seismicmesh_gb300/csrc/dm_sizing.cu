// Gradient limiting of mesh-size grids and the drop-in unique_edges.
#include <mutex>

#include "dm_common.cuh"

namespace dm {

// ---------------------------------------------------------------------------
// limgrad.  The reference (sizing/cpp/FastHJ.cpp:63-157) relaxes
//   f_i <- min(f_i, f_j + elen * dfdx)
// over the 6-neighbour stencil of a column-major grid with an active set
// until no value drops by more than ftol = min(f) * sqrt(eps).  Its fixed
// point is the min-plus distance transform f_i = min_k f_k + c |i - k|_1
// (c = elen * dfdx, grid steps counted in L1), which is separable by axis.
// Each axis is one forward and one backward sweep per grid line; the result
// is that fixed point exactly (the reference stops within ftol of it).
__global__ void k_limgrad_axis(double *f, int d0, int d1, int d2, int axis,
                               double c) {
  int64_t nlines, len, stride;
  if (axis == 0) {
    nlines = (int64_t)d1 * d2;
    len = d0;
    stride = 1;
  } else if (axis == 1) {
    nlines = (int64_t)d0 * d2;
    len = d1;
    stride = d0;
  } else {
    nlines = (int64_t)d0 * d1;
    len = d2;
    stride = (int64_t)d0 * d1;
  }
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nlines;
       l += (int64_t)gridDim.x * blockDim.x) {
    int64_t base;
    if (axis == 0)
      base = l * d0;
    else if (axis == 1)
      base = (l % d0) + (l / d0) * (int64_t)d0 * d1;
    else
      base = l;
    double prev = f[base];
    for (int64_t i = 1; i < len; ++i) {
      double *q = f + base + i * stride;
      double v = fmin(*q, prev + c);
      *q = v;
      prev = v;
    }
    prev = f[base + (len - 1) * stride];
    for (int64_t i = len - 2; i >= 0; --i) {
      double *q = f + base + i * stride;
      double v = fmin(*q, prev + c);
      *q = v;
      prev = v;
    }
  }
}

int limgrad(const int32_t *dims, double elen, double dfdx, int imax, double *f,
            cudaStream_t s) {
  DM_ARG_CHECK(dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0, "dims");
  DM_ARG_CHECK(imax >= 0, "imax");
  double c = elen * dfdx;
  for (int axis = 0; axis < 3; ++axis) {
    int64_t nl = axis == 0 ? (int64_t)dims[1] * dims[2]
                           : axis == 1 ? (int64_t)dims[0] * dims[2]
                                       : (int64_t)dims[0] * dims[1];
    if ((axis == 0 ? dims[0] : axis == 1 ? dims[1] : dims[2]) < 2) continue;
    k_limgrad_axis<<<grid_for(nl, 128), 128, 0, s>>>(f, dims[0], dims[1], dims[2],
                                                     axis, c);
  }
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// ---------------------------------------------------------------------------
// unique_edges (geometry/cpp/fast_geometry.cpp:30-77): (min, max) pairs,
// sorted lexicographically, duplicates removed.  Counting sort by the first
// key, then each bucket is sorted and deduplicated on the second key.  An
// index outside [0, n) is skipped and recorded in *bad, so a malformed edge
// list can never write outside the workspace; the host returns DM_ERR_ARG.
__global__ void k_ue_count(const int32_t *e, int64_t m, int64_t n, int32_t *cnt,
                           int32_t *key, int32_t *slot, int32_t *bad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int a = e[2 * i], b = e[2 * i + 1];
    if (a < 0 || b < 0 || a >= n || b >= n) {
      key[i] = -1;
      atomicExch(bad, 1);
      continue;
    }
    int lo = min(a, b);
    key[i] = lo;
    slot[i] = atomicAdd(&cnt[lo], 1);
  }
}

__global__ void k_ue_scatter(const int32_t *e, int64_t m, const int32_t *start,
                             const int32_t *key, const int32_t *slot,
                             int32_t *val) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int k = key[i];
    if (k < 0) continue;
    int a = e[2 * i], b = e[2 * i + 1];
    val[start[k] + slot[i]] = max(a, b);
  }
}

// buckets up to kUeSmall entries: one thread, insertion sort + unique in
// place, ucnt[v] = unique count.  Larger buckets are left to k_ue_sort_big.
constexpr int kUeSmall = 32;
__global__ void k_ue_sort(int64_t n, const int32_t *start, int32_t *val,
                          int32_t *ucnt) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int b = start[v], e = start[v + 1];
    if (e - b > kUeSmall) continue;
    for (int i = b + 1; i < e; ++i) {
      int x = val[i], j = i - 1;
      while (j >= b && val[j] > x) {
        val[j + 1] = val[j];
        --j;
      }
      val[j + 1] = x;
    }
    int u = 0;
    for (int i = b; i < e; ++i)
      if (i == b || val[i] != val[i - 1]) val[b + u++] = val[i];
    ucnt[v] = u;
  }
}

// Buckets above kUeSmall entries (hub vertices): a block per bucket, bottom-up
// merge sort in which every element finds its merged position by a binary
// search in the other run, ping-ponging between val[b, e) and the same range
// of tmp (the per-edge slot array, free once k_ue_scatter has run).  Each
// block scans kUeBigSpan consecutive buckets for large ones.
constexpr int kUeBigSpan = 256;
__global__ void k_ue_sort_big(int64_t n, const int32_t *start, int32_t *val,
                              int32_t *tmp, int32_t *ucnt) {
  __shared__ int32_t big[kUeBigSpan];
  __shared__ int nbig;
  const int64_t v0 = (int64_t)blockIdx.x * kUeBigSpan;
  if (threadIdx.x == 0) nbig = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < kUeBigSpan; k += blockDim.x) {
    int64_t v = v0 + k;
    if (v < n && start[v + 1] - start[v] > kUeSmall) big[atomicAdd(&nbig, 1)] = (int32_t)v;
  }
  __syncthreads();
  for (int q = 0; q < nbig; ++q) {
    const int v = big[q];
    const int b = start[v], s = start[v + 1] - b;
    int32_t *src = val + b, *dst = tmp + b;
    for (int w = 1; w < s; w *= 2) {
      for (int i = threadIdx.x; i < s; i += blockDim.x) {
        const int lo = (i / (2 * w)) * (2 * w);
        const int mid = min(lo + w, s), hi = min(lo + 2 * w, s);
        const int x = src[i];
        int pos;
        if (i < mid) {  // left run: count right-run elements < x
          int l = mid, r = hi;
          while (l < r) {
            int m = (l + r) >> 1;
            if (src[m] < x) l = m + 1; else r = m;
          }
          pos = lo + (i - lo) + (l - mid);
        } else {        // right run: count left-run elements <= x
          int l = lo, r = mid;
          while (l < r) {
            int m = (l + r) >> 1;
            if (src[m] <= x) l = m + 1; else r = m;
          }
          pos = lo + (i - mid) + (l - lo);
        }
        dst[pos] = x;
      }
      __syncthreads();
      int32_t *t = src;
      src = dst;
      dst = t;
    }
    if (src != val + b)
      for (int i = threadIdx.x; i < s; i += blockDim.x) val[b + i] = src[i];
    __syncthreads();
    if (threadIdx.x == 0) {
      int u = 0;
      for (int i = b; i < b + s; ++i)
        if (i == b || val[i] != val[i - 1]) val[b + u++] = val[i];
      ucnt[v] = u;
    }
    __syncthreads();
  }
}

__global__ void k_ue_write(int64_t n, const int32_t *start, const int32_t *val,
                           const int32_t *ustart, int32_t *out) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    int b = start[v], o = ustart[v], u = ustart[v + 1] - o;
    for (int i = 0; i < u; ++i) {
      out[2 * (o + i)] = (int32_t)v;
      out[2 * (o + i) + 1] = val[b + i];
    }
  }
}

// cnt carries one extra slot, cnt[n], the bad-index flag
static size_t carve_ue(Carve &c, int64_t n, int64_t m, int32_t **cnt,
                       int32_t **start, int32_t **key, int32_t **slot,
                       int32_t **val, int32_t **ucnt, int32_t **ustart,
                       int32_t **tmp) {
  *cnt = c.take<int32_t>(n + 1);
  *start = c.take<int32_t>(n + 1);
  *key = c.take<int32_t>(m);
  *slot = c.take<int32_t>(m);
  *val = c.take<int32_t>(m);
  *ucnt = c.take<int32_t>(n);
  *ustart = c.take<int32_t>(n + 1);
  *tmp = c.take<int32_t>(scan_tmp_elems(n));
  return c.used;
}

// the kernel sequence shared by both entry points, on carved arrays
static int unique_edges_run(const int32_t *edges, int64_t m, int64_t n, int32_t *out,
                            int64_t *n_out, int32_t *cnt, int32_t *start, int32_t *key,
                            int32_t *slot, int32_t *val, int32_t *ucnt, int32_t *ustart,
                            int32_t *tmp, const char *who, cudaStream_t s) {
  int32_t *bad = cnt + n;
  DM_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (n + 1), s));
  int nb = grid_for(m, 256);
  k_ue_count<<<nb, 256, 0, s>>>(edges, m, n, cnt, key, slot, bad);
  int rc = exclusive_scan_i32(cnt, start, n, tmp, s);
  if (rc) return rc;
  k_ue_scatter<<<nb, 256, 0, s>>>(edges, m, start, key, slot, val);
  k_ue_sort<<<grid_for(n, 128), 128, 0, s>>>(n, start, val, ucnt);
  k_ue_sort_big<<<(int)((n + kUeBigSpan - 1) / kUeBigSpan), 256, 0, s>>>(n, start, val,
                                                                         slot, ucnt);
  rc = exclusive_scan_i32(ucnt, ustart, n, tmp, s);
  if (rc) return rc;
  k_ue_write<<<grid_for(n, 128), 128, 0, s>>>(n, start, val, ustart, out);
  DM_LAUNCH_CHECK();
  int32_t total = 0, flag = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&total, ustart + n, sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaMemcpyAsync(&flag, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag) {
    set_error("%s: an edge index lies outside [0, n = %lld)", who, (long long)n);
    return DM_ERR_ARG;
  }
  *n_out = total;
  return DM_OK;
}

int unique_edges_workspace(int64_t n, int64_t m, size_t *bytes) {
  Carve c(nullptr, 0);
  int32_t *a, *b, *d, *e, *f, *g, *h, *t;
  *bytes = carve_ue(c, n, m, &a, &b, &d, &e, &f, &g, &h, &t) + 256;
  return DM_OK;
}

int unique_edges(const int32_t *edges, int64_t m, int64_t n, int32_t *out,
                 int64_t *n_out, void *ws, size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(n >= 0 && m >= 0, "sizes");
  DM_ARG_CHECK(n_out != nullptr, "n_out");
  Carve c(ws, ws_bytes);
  int32_t *cnt, *start, *key, *slot, *val, *ucnt, *ustart, *tmp;
  carve_ue(c, n, m, &cnt, &start, &key, &slot, &val, &ucnt, &ustart, &tmp);
  if (!c.ok() || !ws) {
    set_error("unique_edges: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  *n_out = 0;
  if (m == 0 || n == 0) return DM_OK;
  return unique_edges_run(edges, m, n, out, n_out, cnt, start, key, slot, val, ucnt,
                          ustart, tmp, "unique_edges", s);
}

// ---------------------------------------------------------------------------
// unique_edges on library-owned scratch: the same kernels as unique_edges,
// with every intermediate array carved from one static device array instead
// of a caller workspace.  Nothing is allocated.  Limits: n <= 131072
// vertices, m <= 524288 edges.  The bucket counters are cleared at the start
// of every call, so nothing has to be zero beforehand.  One scratch exists
// per device: calls that overlap in time on the same device race on it.
constexpr int64_t kUeStaticMaxN = int64_t(1) << 17;
constexpr int64_t kUeStaticMaxM = int64_t(1) << 19;
constexpr size_t kUeStaticBytes =
    4 * (4 * (size_t)kUeStaticMaxN + 3 * (size_t)kUeStaticMaxM) + (64 << 10);
constexpr int kUeMaxDevices = 64;

static __device__ __align__(256) unsigned char g_ue_scratch[kUeStaticBytes];

static std::mutex g_ue_mu;
static void *g_ue_addr[kUeMaxDevices];  // by device ordinal, set on first use

// Address of g_ue_scratch on the current device, looked up once per device
// with that device current.
static int ue_static_scratch(void **out) {
  int dev = -1;
  DM_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kUeMaxDevices) {
    set_error("unique_edges_noalloc: device ordinal %d outside [0, %d)", dev,
              kUeMaxDevices);
    return DM_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_ue_mu);
  if (!g_ue_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_ue_scratch);
    if (e != cudaSuccess || !p) {
      set_error("unique_edges_noalloc: cudaGetSymbolAddress on device %d "
                "failed: %s", dev, cudaGetErrorString(e));
      return DM_ERR_CUDA;
    }
    g_ue_addr[dev] = p;
  }
  *out = g_ue_addr[dev];
  return DM_OK;
}

int unique_edges_noalloc(const int32_t *edges, int64_t m, int64_t n,
                         int32_t *out, int64_t *n_out, cudaStream_t s) {
  DM_ARG_CHECK(n >= 0 && m >= 0, "sizes");
  DM_ARG_CHECK(n_out != nullptr, "n_out");
  if (n > kUeStaticMaxN || m > kUeStaticMaxM) {
    set_error("unique_edges_noalloc: n = %lld vertices, m = %lld edges "
              "exceed the static scratch limits n <= %lld, m <= %lld; use "
              "dm_unique_edges with a workspace", (long long)n, (long long)m,
              (long long)kUeStaticMaxN, (long long)kUeStaticMaxM);
    return DM_ERR_CAPACITY;
  }
  void *base = nullptr;
  int rc = ue_static_scratch(&base);
  if (rc) return rc;
  Carve c(base, kUeStaticBytes);
  int32_t *cnt, *start, *key, *slot, *val, *ucnt, *ustart, *tmp;
  carve_ue(c, n, m, &cnt, &start, &key, &slot, &val, &ucnt, &ustart, &tmp);
  if (!c.ok()) {
    set_error("unique_edges_noalloc: static scratch %zu < required %zu",
              kUeStaticBytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  *n_out = 0;
  if (m == 0 || n == 0) return DM_OK;
  return unique_edges_run(edges, m, n, out, n_out, cnt, start, key, slot, val, ucnt,
                          ustart, tmp, "unique_edges_noalloc", s);
}

}  // namespace dm

namespace dm {

// ---------------------------------------------------------------------------
// Mesh size from a velocity grid (sizing/mesh_size_function.py:146-221):
// unit scale, water replacement, wavelength / gradient sizing, [hmin, hmax]
// clamp and the Courant bound, elementwise in FP64.
struct SizeParams {
  double scale;       // unit conversion factor applied to vp
  double vp_water;    // replacement for vp < 1e-3 (if replace != 0)
  int replace;
  double wl, freq;    // wavelength sizing when wl > 0
  double grad;        // gradient sizing when grad > 0 (uses gterm)
  double hmin, hmax;
  double dt, cr_max, space_order;
  int dim;
};

__global__ void k_size_from_vp(double *vp, int64_t n, const double *gterm,
                               SizeParams sp, double *cell) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = vp[i] * sp.scale;
    if (sp.replace && v < 1e-3) v = sp.vp_water;
    vp[i] = v;
    double h = sp.hmin;
    if (sp.wl > 0 || sp.grad > 0) {
      double a = sp.wl > 0 ? v / (sp.freq * sp.wl) : 99999.0;
      double b = sp.grad > 0 ? gterm[i] : 99999.0;
      h = fmin(a, b);
    }
    if (h < sp.hmin) h = sp.hmin;
    if (h > sp.hmax) h = sp.hmax;
    if (sp.cr_max != 0.0 && sp.dt != 0.0 && sp.space_order != 0.0) {
      double cr_old = (v * sp.dt) / (sp.dim * h);
      double crm = sp.cr_max / (sp.dim * sp.space_order);
      double dxn = (v * sp.dt) / (sp.dim * crm);
      if (cr_old > crm) h = dxn;
    }
    cell[i] = h;
  }
}

// flag: some vp < 1e-3 (after unit scaling) outside the first row (the
// reference replaces water velocities only when such a cell exists,
// sizing/mesh_size_function.py:154-165)
__global__ void k_water_flag(const double *vp, int64_t n, int64_t row_len,
                             double scale, int *flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (vp[i] * scale < 1e-3 && i >= row_len) *flag = 1;
}

// ---------------------------------------------------------------------------
// Gradient sizing (sizing/mesh_size_function.py:428-448):
//   g = grad / (v + 0.10),  v = var / max(var) - min(var / max(var)),
//   var = box_mean(vp^2) - box_mean(vp)^2
// with the box means of scipy.ndimage.uniform_filter: separable, applied
// axis by axis in order, window w per axis, origin 0 (covers i - w/2 ..
// i - w/2 + w - 1) and 'reflect' boundaries (d c b a | a b c d | d c b a).
// vp is read with the unit scale and water replacement of
// dm_size_from_velocity.  Running sums in FP64, one thread per grid line.
__device__ __forceinline__ int64_t reflect_index(int64_t j, int64_t L) {
  const int64_t p = 2 * L;
  j %= p;
  if (j < 0) j += p;
  return j < L ? j : p - 1 - j;
}

__global__ void k_box_mean_axis(const double *src_m, const double *src_s, double *dst_m,
                                double *dst_s, int64_t nlines, int64_t L, int64_t st,
                                int w, int first, double scale, double vp_water,
                                int replace) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nlines;
       l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = (l / st) * (st * L) + (l % st);
    auto val = [&](int64_t j, double &m, double &q) {
      int64_t k = base + reflect_index(j, L) * st;
      if (first) {
        double v = src_m[k] * scale;
        if (replace && v < 1e-3) v = vp_water;
        m = v;
        q = v * v;
      } else {
        m = src_m[k];
        q = src_s[k];
      }
    };
    const int64_t h = w / 2;
    double sm = 0, sq = 0, a, b;
    for (int64_t k = 0; k < w; ++k) {
      val(k - h, a, b);
      sm += a;
      sq += b;
    }
    const double inv = 1.0 / w;
    for (int64_t i = 0; i < L; ++i) {
      dst_m[base + i * st] = sm * inv;
      dst_s[base + i * st] = sq * inv;
      if (i + 1 < L) {
        double a1, b1, a0, b0;
        val(i + 1 - h + w - 1, a1, b1);
        val(i - h, a0, b0);
        sm += a1 - a0;
        sq += b1 - b0;
      }
    }
  }
}

// var = s - m^2 into m; block maxima / minima of var into part
__global__ void k_variance(double *m, const double *sq, int64_t n, double *part) {
  double mx = -1e300, mn = 1e300;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = sq[i] - m[i] * m[i];
    m[i] = v;
    mx = fmax(mx, v);
    mn = fmin(mn, v);
  }
  for (int o = 16; o; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  }
  __shared__ double smx[8], smn[8];
  if ((threadIdx.x & 31) == 0) {
    smx[threadIdx.x >> 5] = mx;
    smn[threadIdx.x >> 5] = mn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mx = smx[0];
    mn = smn[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
      mx = fmax(mx, smx[k]);
      mn = fmin(mn, smn[k]);
    }
    part[2 * blockIdx.x] = mx;
    part[2 * blockIdx.x + 1] = mn;
  }
}

// g = grad / (var / max - min(var / max) + 0.1), in the order of the reference
__global__ void k_gradient_term(const double *var, int64_t n, const double *part, int nb,
                                double grad, double *g) {
  double mx = -1e300, mn = 1e300;
  for (int k = 0; k < nb; ++k) {
    mx = fmax(mx, part[2 * k]);
    mn = fmin(mn, part[2 * k + 1]);
  }
  const double lo = mn / mx;  // min of var / max (division is monotone for mx > 0)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = var[i] / mx;
    v -= lo;
    g[i] = grad / (v + 0.10);
  }
}

size_t gradient_term_workspace(int64_t n) {
  Carve c(nullptr, 0);
  c.take<double>(n);
  c.take<double>(n);
  c.take<double>(n);
  c.take<double>(2 * 256);
  return c.used + 256;
}

int gradient_term(const double *vp, const int32_t *dims, int dim, const int32_t *window,
                  double scale, double vp_water, int replace, double grad, double *g,
                  void *ws, size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(dims && window, "dims / window");
  int64_t n = 1;
  for (int k = 0; k < dim; ++k) {
    DM_ARG_CHECK(dims[k] > 0 && window[k] > 0, "dims and window must be positive");
    n *= dims[k];
  }
  DM_ARG_CHECK(grad > 0, "grad must be > 0");
  Carve c(ws, ws_bytes);
  double *ms = c.take<double>(n), *ss = c.take<double>(n), *tm = c.take<double>(n);
  double *part = c.take<double>(2 * 256);
  if (!c.ok() || !ws) {
    set_error("gradient_term: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  // ping-pong: (g, ms) <-> (tm, ss); the output array g serves as a buffer
  double *cur_m = nullptr, *cur_s = nullptr;
  double *bufm[2] = {g, tm}, *bufs[2] = {ms, ss};
  for (int axis = 0; axis < dim; ++axis) {
    int64_t st = 1;
    for (int k = axis + 1; k < dim; ++k) st *= dims[k];
    const int64_t L = dims[axis], nlines = n / L;
    double *om = bufm[axis & 1], *os = bufs[axis & 1];
    k_box_mean_axis<<<grid_for(nlines, 128), 128, 0, s>>>(
        axis == 0 ? vp : cur_m, cur_s, om, os, nlines, L, st, window[axis], axis == 0,
        scale, vp_water, replace);
    cur_m = om;
    cur_s = os;
  }
  const int nb = 256;
  k_variance<<<nb, 256, 0, s>>>(cur_m, cur_s, n, part);
  k_gradient_term<<<grid_for(n, 256), 256, 0, s>>>(cur_m, n, part, nb, grad, g);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int size_from_velocity(double *vp, int64_t n, int64_t row_len,
                       const double *gterm, const SizeParams *sp_in,
                       double *cell, int *replaced_host, void *ws,
                       cudaStream_t s) {
  SizeParams sp = *sp_in;
  int *flag = (int *)ws;
  DM_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), s));
  k_water_flag<<<grid_for(n, 256), 256, 0, s>>>(vp, n, row_len, sp.scale, flag);
  int h = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  sp.replace = h;
  if (h && (sp.vp_water < 1300 || sp.vp_water > 1800)) {
    set_error("vp_water is None or out of bounds. It should be >1300 and <1800 m/s");
    return DM_ERR_ARG;
  }
  if (replaced_host) *replaced_host = h;
  k_size_from_vp<<<grid_for(n, 256), 256, 0, s>>>(vp, n, gterm, sp, cell);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// ---------------------------------------------------------------------------
// domain pad (sizing/mesh_size_function.py:526-587): pad a C-order grid by
// pre[k] / post[k] cells per axis; mode 0 = edge, 1 = constant (value
// cval), 2 = linear ramp to cval (numpy.pad semantics).
struct PadArgs {
  int n[3], pre[3], post[3];
};

__global__ void k_pad(const double *src, PadArgs a, int dim, int mode,
                      double cval, double *dst) {
  int m[3];
  for (int k = 0; k < 3; ++k) m[k] = a.n[k] + a.pre[k] + a.post[k];
  int64_t total = (int64_t)m[0] * m[1] * m[2];
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * blockDim.x) {
    int idx[3] = {(int)(o / ((int64_t)m[1] * m[2])), (int)((o / m[2]) % m[1]),
                  (int)(o % m[2])};
    int sidx[3], c[3];
    bool inside = true;
    for (int k = 0; k < 3; ++k) {
      sidx[k] = idx[k] - a.pre[k];
      if (sidx[k] < 0 || sidx[k] >= a.n[k]) inside = false;
      c[k] = min(max(sidx[k], 0), a.n[k] - 1);
    }
    double v = src[((int64_t)c[0] * a.n[1] + c[1]) * a.n[2] + c[2]];
    if (!inside && mode == 1) {
      v = cval;
    } else if (!inside && mode == 2) {
      // numpy.pad linear_ramp, applied axis by axis: the outermost pad cell
      // equals cval, the ramp is linear in the distance to the edge.
      for (int k = 0; k < dim; ++k) {
        int i = sidx[k];
        if (i < 0)
          v = v + (cval - v) * ((double)(-i) / a.pre[k]);
        else if (i >= a.n[k])
          v = v + (cval - v) * ((double)(i - a.n[k] + 1) / a.post[k]);
      }
    }
    dst[o] = v;
  }
}

int pad_grid(const double *src, const int *n, const int *pre, const int *post,
             int dim, int mode, double cval, double *dst, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(mode >= 0 && mode <= 2, "mode");
  PadArgs a;
  int64_t total = 1;
  for (int k = 0; k < 3; ++k) {
    a.n[k] = k < dim ? n[k] : 1;
    a.pre[k] = k < dim ? pre[k] : 0;
    a.post[k] = k < dim ? post[k] : 0;
    total *= (int64_t)(a.n[k] + a.pre[k] + a.post[k]);
  }
  k_pad<<<grid_for(total, 256), 256, 0, s>>>(src, a, dim, mode, cval, dst);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

}  // namespace dm
