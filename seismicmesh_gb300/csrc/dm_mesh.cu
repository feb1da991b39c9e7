// Per-iteration DistMesh kernels: cell filter, bar adjacency, bar forces with
// the fused point update and Newton projection, and the sliver kernels.
#include <float.h>

#include "dm_common.cuh"
#include "dm_sdf.cuh"

namespace dm {

void note_launches(int k);

struct SdfDev {
  const int32_t *ops;
  const float *params;
  int n_ops;
};

struct SizingDev {
  int kind;
  float h;
  const float *grid;
  int n[3];
  float lo[3], hi[3];
  const float *slot_h;
};

static SizingDev to_dev(const dm_sizing *s) {
  SizingDev d;
  d.kind = s->kind;
  d.h = s->h;
  d.grid = s->grid;
  for (int k = 0; k < 3; ++k) {
    d.n[k] = s->n[k];
    d.lo[k] = s->lo[k];
    d.hi[k] = s->hi[k];
  }
  d.slot_h = s->slot_h;
  return d;
}

template <int DIM>
__device__ __forceinline__ void ldpt(const float *P, int64_t i, float *x) {
  if (DIM == 3) {
    float4 v = __ldg(reinterpret_cast<const float4 *>(P) + i);
    x[0] = v.x;
    x[1] = v.y;
    x[2] = v.z;
  } else {
    float2 v = __ldg(reinterpret_cast<const float2 *>(P) + i);
    x[0] = v.x;
    x[1] = v.y;
  }
}

template <int DIM>
__device__ __forceinline__ float sizing_at(const SizingDev &s, const float *x,
                                           int64_t slot) {
  if (s.kind == DM_SIZING_CONST) return s.h;
  if (s.kind == DM_SIZING_GRID)
    return grid_interp<DIM>(s.grid, s.n, s.lo, s.hi, x, nullptr);
  return __ldg(s.slot_h + slot);
}

// ---------------------------------------------------------------------------
// cell filter: keep cells with sdf(centroid) < -geps
template <int DIM>
__global__ void k_filter_cells(const float *P, const int32_t *cells,
                               int64_t cap, SdfDev sdf, float geps,
                               int32_t *out, int64_t *counters) {
  int64_t nc = min(counters[DM_CNT_CELLS], cap);
  const int NV = DIM + 1;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t base = blockIdx.x * (int64_t)blockDim.x;
  for (int64_t c0 = base; c0 < nc; c0 += stride) {
    int64_t c = c0 + threadIdx.x;
    bool keep = false;
    int v[4] = {0, 0, 0, 0};
    if (c < nc) {
      float cen[3] = {0, 0, 0};
      for (int k = 0; k < NV; ++k) {
        v[k] = cells[NV * c + k];
        float x[3];
        ldpt<DIM>(P, v[k], x);
        for (int j = 0; j < DIM; ++j) cen[j] += x[j];
      }
      for (int j = 0; j < DIM; ++j) cen[j] = cen[j] / (float)NV;
      Dual d = sdf_eval<DIM, false>(sdf.ops, sdf.params, sdf.n_ops, cen);
      keep = d.v < -geps;
    }
    int64_t k = warp_append(&counters[DM_CNT_KEPT], keep);
    if (keep)
      for (int j = 0; j < NV; ++j) out[NV * k + j] = v[j];
  }
}

template <int DIM>
__global__ void k_centroids(const float *P, const int32_t *cells, int64_t cap,
                            const int64_t *counters, float *cen_out) {
  int64_t nc = min(counters[DM_CNT_CELLS], cap);
  const int NV = DIM + 1;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    float cen[3] = {0, 0, 0};
    for (int k = 0; k < NV; ++k) {
      float x[3];
      ldpt<DIM>(P, cells[NV * c + k], x);
      for (int j = 0; j < DIM; ++j) cen[j] += x[j];
    }
    for (int j = 0; j < DIM; ++j) cen_out[DIM * c + j] = cen[j] / (float)NV;
  }
}

// ---------------------------------------------------------------------------
// adjacency: scatter every cell edge into both endpoint rows, then sort and
// deduplicate each row in shared memory.
// Adjacency rows from cells (replaces _get_edges + unique_edges of the
// reference, generation/mesh_generator.py:680-688): CSR of the raw neighbour
// lists (NV-1 entries per incident cell), then one warp per vertex sorts and
// deduplicates its segment into a fixed-stride row.
template <int NV>
__global__ void k_adj_count(const int32_t *cells, int64_t cap_cells,
                            const int64_t *counters, int count_index, int32_t *cnt) {
  int64_t nc = min(counters[count_index], cap_cells);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x)
    for (int k = 0; k < NV; ++k) atomicAdd(&cnt[cells[NV * c + k]], NV - 1);
}

template <int NV>
__global__ void k_adj_fill(const int32_t *cells, int64_t cap_cells,
                           const int64_t *counters, int count_index,
                           const int32_t *off, int32_t *cursor, int32_t *raw) {
  int64_t nc = min(counters[count_index], cap_cells);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    int v[NV];
    for (int k = 0; k < NV; ++k) v[k] = cells[NV * c + k];
    for (int i = 0; i < NV; ++i) {
      int pos = off[v[i]] + atomicAdd(&cursor[v[i]], NV - 1);
      for (int j = 0; j < NV; ++j)
        if (j != i) raw[pos++] = v[j];
    }
  }
}

constexpr int ADJ_WARPS = 8;
constexpr int ADJ_SORTMAX = 1024;  // raw segment sorted in shared memory

// bitonic sort of b[0..size) (size a power of two) by one warp
__device__ __forceinline__ void warp_bitonic(int *b, int size, int lane) {
  for (int kk = 2; kk <= size; kk <<= 1)
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < size; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          int x = b[i], y = b[ixj];
          bool up = (i & kk) == 0;
          if ((x > y) == up) {
            b[i] = y;
            b[ixj] = x;
          }
        }
      }
      __syncwarp();
    }
}

// One thread per vertex: its raw segment goes into a sorted, duplicate-free
// array by insertion.  A vertex whose segment exceeds kAdjRaw entries or
// whose unique neighbours exceed kAdjLocal is appended to big[] for the warp
// kernel below.  The row keeps the adj_cap smallest neighbours either way.
constexpr int kAdjLocal = 32, kAdjRaw = 160;
__global__ void __launch_bounds__(256)
    k_adj_dedup_thread(int64_t n, const int32_t *off, const int32_t *raw, int32_t *adj,
                       int adj_cap, int32_t *deg, int32_t *big, int32_t *nbig,
                       int64_t *counters) {
  unsigned long long ecount = 0;
  bool ovf = false;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int o = off[v], L = off[v + 1] - o;
    int u[kAdjLocal];
    int m = 0;
    bool spill = L > kAdjRaw;
    for (int k = 0; k < L && !spill; ++k) {
      const int x = raw[o + k];
      int j = m;
      while (j > 0 && u[j - 1] > x) --j;
      if (j > 0 && u[j - 1] == x) continue;
      if (m == kAdjLocal) {
        spill = true;
        break;
      }
      for (int t = m; t > j; --t) u[t] = u[t - 1];
      u[j] = x;
      ++m;
    }
    if (spill) {
      big[atomicAdd(nbig, 1)] = (int32_t)v;
      continue;
    }
    if (m > adj_cap) atomicMax((unsigned long long *)&counters[DM_CNT_MAXDEG], (unsigned long long)m);
    int32_t *row = adj + v * adj_cap;
    const int keep = min(m, adj_cap);
    for (int i = 0; i < keep; ++i) row[i] = u[i];
    deg[v] = keep;
    if (m > adj_cap) ovf = true;
    ecount += m;
  }
  for (int o = 16; o; o >>= 1) ecount += __shfl_xor_sync(0xffffffffu, ecount, o);
  if ((threadIdx.x & 31) == 0 && ecount)
    atomicAdd((unsigned long long *)&counters[DM_CNT_EDGES], ecount);
  if (__any_sync(0xffffffffu, ovf) && (threadIdx.x & 31) == 0)
    flag_or(counters, DM_FLAG_ADJ_OVERFLOW);
}

// One warp per listed vertex (the high-incidence ones): bitonic sort of the
// segment in shared memory, then unique and compaction into the row.
__global__ void __launch_bounds__(32 * ADJ_WARPS)
    k_adj_dedup(const int32_t *list, const int32_t *nlist, const int32_t *off,
                const int32_t *raw, int32_t *adj, int adj_cap, int32_t *deg,
                int64_t *counters) {
  __shared__ int buf[ADJ_WARPS][ADJ_SORTMAX];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int *b = buf[w];
  unsigned long long ecount = 0;
  bool ovf = false;
  const int64_t nl = *nlist;
  for (int64_t q = (int64_t)blockIdx.x * ADJ_WARPS + w; q < nl;
       q += (int64_t)gridDim.x * ADJ_WARPS) {
    const int64_t v = list[q];
    const int o = off[v], L = off[v + 1] - o;
    int m;  // entries staged in b
    if (L <= ADJ_SORTMAX) {
      for (int k = lane; k < L; k += 32) b[k] = raw[o + k];
      m = L;
    } else {
      // very high incidence: stage first occurrences only (quadratic scan)
      m = 0;
      for (int k0 = 0; k0 < L; k0 += 32) {
        int k = k0 + lane;
        int x = k < L ? raw[o + k] : 0;
        bool first = k < L;
        for (int j = 0; j < k0 + lane && first; ++j) first = raw[o + j] != x;
        unsigned mk = __ballot_sync(0xffffffffu, first);
        int pos = m + __popc(mk & ((1u << lane) - 1));
        if (first && pos < ADJ_SORTMAX) b[pos] = x;
        m += __popc(mk);
      }
      if (m > ADJ_SORTMAX) {
        ovf = true;
        m = ADJ_SORTMAX;
      }
    }
    int size = 1;
    while (size < m) size <<= 1;
    for (int k = m + lane; k < size; k += 32) b[k] = 0x7fffffff;
    __syncwarp();
    warp_bitonic(b, size, lane);
    // unique + compact into the row
    int32_t *row = adj + v * adj_cap;
    int base = 0;
    for (int k0 = 0; k0 < m; k0 += 32) {
      int k = k0 + lane;
      bool keep = k < m && (k == 0 || b[k] != b[k - 1]);
      unsigned mk = __ballot_sync(0xffffffffu, keep);
      int pos = base + __popc(mk & ((1u << lane) - 1));
      if (keep && pos < adj_cap) row[pos] = b[k];
      base += __popc(mk);
    }
    if (base > adj_cap) ovf = true;
    if (lane == 0 && base > adj_cap)
      atomicMax((unsigned long long *)&counters[DM_CNT_MAXDEG], (unsigned long long)base);
    if (lane == 0) deg[v] = min(base, adj_cap);
    ecount += base;
    __syncwarp();
  }
  if (lane == 0 && ecount)
    atomicAdd((unsigned long long *)&counters[DM_CNT_EDGES], ecount);
  if (ovf && lane == 0) flag_or(counters, DM_FLAG_ADJ_OVERFLOW);
}

__global__ void k_half_edges(int64_t *counters) {
  counters[DM_CNT_EDGES] /= 2;
}

// ---------------------------------------------------------------------------
// bar forces.  G lanes cooperate on one vertex.
template <int DIM>
struct BarCfg {
  static constexpr int G = DIM == 3 ? 8 : 4;
  static constexpr int THREADS = 256;
  static constexpr int VPB = THREADS / G;  // vertices per block
};

template <int DIM>
__global__ void __launch_bounds__(256)
    k_bar_sums(const float *P, int64_t n, const int32_t *adj, int adj_cap,
               const int32_t *deg, SizingDev sz, double *partials) {
  constexpr int G = BarCfg<DIM>::G;
  const int sub = threadIdx.x % G;
  int64_t v = (int64_t)blockIdx.x * BarCfg<DIM>::VPB + threadIdx.x / G;
  double sL = 0.0, sH = 0.0;
  if (v < n) {
    float pv[3];
    ldpt<DIM>(P, v, pv);
    int dg = deg[v];
    for (int k = sub; k < dg; k += G) {
      int w = adj[v * adj_cap + k];
      if (w <= v) continue;
      float pw[3], mid[3], L2 = 0.f;
      ldpt<DIM>(P, w, pw);
      for (int j = 0; j < DIM; ++j) {
        float d = pv[j] - pw[j];
        L2 += d * d;
        mid[j] = (pv[j] + pw[j]) * 0.5f;
      }
      float L = sqrtf(L2);
      float h = sizing_at<DIM>(sz, mid, v * adj_cap + k);
      double Ld = L, hd = h;
      sL += DIM == 3 ? Ld * Ld * Ld : Ld * Ld;
      sH += DIM == 3 ? hd * hd * hd : hd * hd;
    }
  }
  // deterministic block reduction
  for (int o = 16; o; o >>= 1) {
    sL += __shfl_xor_sync(0xffffffffu, sL, o);
    sH += __shfl_xor_sync(0xffffffffu, sH, o);
  }
  __shared__ double rs[2][8];
  int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    rs[0][w] = sL;
    rs[1][w] = sH;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int i = 0; i < 8; ++i) {
      a += rs[0][i];
      b += rs[1][i];
    }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

// scale = (sum L^d / sum h^d)^(1/d), written to partials[2 * nblk]
__global__ void k_bar_scale(double *partials, int nblk, int dim) {
  __shared__ double ra[1024], rb[1024];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += partials[2 * i];
    b += partials[2 * i + 1];
  }
  ra[threadIdx.x] = a;
  rb[threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      ra[threadIdx.x] += ra[threadIdx.x + s];
      rb[threadIdx.x] += rb[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double r = ra[0] / rb[0];
    partials[2 * nblk] = dim == 3 ? cbrt(r) : sqrt(r);
    partials[2 * nblk + 1] = ra[0];
    partials[2 * nblk + 2] = rb[0];
  }
}

struct Levels {
  SdfDev lv[4];
  int n;
};

template <int DIM>
__device__ __forceinline__ void newton_project(const Levels &L, float *x,
                                               float hmin, float deps) {
  for (int l = 0; l < L.n; ++l) {
    Dual d = sdf_eval<DIM, true>(L.lv[l].ops, L.lv[l].params, L.lv[l].n_ops, x);
    bool sel = l == 0 ? d.v > 0.f : (d.v > 0.f && d.v < hmin / 1.5f);
    if (!sel) continue;
    float g2 = 0.f;
    for (int j = 0; j < DIM; ++j) g2 += d.g[j] * d.g[j];
    if (g2 < deps) g2 = deps;
    for (int j = 0; j < DIM; ++j) x[j] -= d.v * d.g[j] / g2;
  }
}

// round x to a multiple of 2^e (exact: power-of-two scaling and rint);
// e < -200 leaves x unchanged
__device__ __forceinline__ float to_grid(float x, int e) {
  return e < -200 ? x : ldexpf(rintf(ldexpf(x, -e)), e);
}

template <int DIM>
__global__ void __launch_bounds__(256)
    k_update(const float *P, float *Pout, int64_t n, const int32_t *adj,
             int adj_cap, const int32_t *deg, SizingDev sz,
             const double *partials, int nblk, float L0mult, float dt,
             int64_t nfix, Levels lv, float hmin, float deps, float *maxf,
             int grid_exp) {
  constexpr int G = BarCfg<DIM>::G;
  const int sub = threadIdx.x % G;
  int64_t v = (int64_t)blockIdx.x * BarCfg<DIM>::VPB + threadIdx.x / G;
  const float scale = (float)partials[2 * nblk];
  float F[3] = {0, 0, 0};
  float pv[3] = {0, 0, 0};
  if (v < n) {
    ldpt<DIM>(P, v, pv);
    int dg = deg[v];
    for (int k = sub; k < dg; k += G) {
      int w = adj[v * adj_cap + k];
      float pw[3], bar[3], mid[3], L2 = 0.f;
      ldpt<DIM>(P, w, pw);
      for (int j = 0; j < DIM; ++j) {
        bar[j] = pv[j] - pw[j];
        L2 += bar[j] * bar[j];
        mid[j] = (pv[j] + pw[j]) * 0.5f;
      }
      float L = sqrtf(L2);
      if (L == 0.f) L = FLT_EPSILON;
      float h = sizing_at<DIM>(sz, mid, v * adj_cap + k);
      float L0 = h * L0mult * scale;
      float f = fmaxf(L0 - L, 0.f) / L;
      for (int j = 0; j < DIM; ++j) F[j] += f * bar[j];
    }
  }
  // reduce over the G lanes of this vertex (fixed order)
  for (int o = G / 2; o; o >>= 1)
    for (int j = 0; j < DIM; ++j) F[j] += __shfl_xor_sync(0xffffffffu, F[j], o);
  float fn = 0.f;
  if (v < n && sub == 0) {
    if (v < nfix) F[0] = F[1] = F[2] = 0.f;
    float x[3];
    for (int j = 0; j < DIM; ++j) {
      x[j] = pv[j] + dt * F[j];
      fn += F[j] * F[j];
    }
    newton_project<DIM>(lv, x, hmin, deps);
    for (int j = 0; j < DIM; ++j) x[j] = to_grid(x[j], grid_exp);
    if (DIM == 3)
      reinterpret_cast<float4 *>(Pout)[v] = make_float4(x[0], x[1], x[2], 0.f);
    else
      reinterpret_cast<float2 *>(Pout)[v] = make_float2(x[0], x[1]);
  }
  fn = sqrtf(fn);
  for (int o = 16; o; o >>= 1) fn = fmaxf(fn, __shfl_xor_sync(0xffffffffu, fn, o));
  __shared__ float rm[8];
  if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = fn;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int i = 0; i < 8; ++i) m = fmaxf(m, rm[i]);
    maxf[blockIdx.x] = m;
  }
}

// maximum of the nblk block maxima, written to maxf[slot]
__global__ void k_max_reduce(float *maxf, int nblk, int slot) {
  __shared__ float r[1024];
  float m = 0.f;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) m = fmaxf(m, maxf[i]);
  r[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) r[threadIdx.x] = fmaxf(r[threadIdx.x], r[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) maxf[slot] = r[0];
}

template <int DIM>
__global__ void k_slot_mid(const float *P, int64_t n, const int32_t *adj,
                           int adj_cap, const int32_t *deg, float *mid) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
       i < n * adj_cap; i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = i / adj_cap;
    int k = (int)(i % adj_cap);
    if (k >= deg[v]) continue;
    int w = adj[i];
    float pv[3], pw[3];
    ldpt<DIM>(P, v, pv);
    ldpt<DIM>(P, w, pw);
    for (int j = 0; j < DIM; ++j) mid[i * DIM + j] = (pv[j] + pw[j]) * 0.5f;
  }
}

// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_sdf_eval(SdfDev sdf, const float *x, int64_t n, int stride,
                           float *d, float *grad) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float q[3] = {0, 0, 0};
    for (int j = 0; j < DIM; ++j) q[j] = x[i * stride + j];
    if (grad) {
      Dual r = sdf_eval<DIM, true>(sdf.ops, sdf.params, sdf.n_ops, q);
      d[i] = r.v;
      for (int j = 0; j < DIM; ++j) grad[i * DIM + j] = r.g[j];
    } else {
      d[i] = sdf_eval<DIM, false>(sdf.ops, sdf.params, sdf.n_ops, q).v;
    }
  }
}

template <int DIM>
__global__ void k_sizing_eval(SizingDev sz, const float *x, int64_t n,
                              int stride, float *h) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float q[3] = {0, 0, 0};
    for (int j = 0; j < DIM; ++j) q[j] = x[i * stride + j];
    h[i] = sz.kind == DM_SIZING_CONST
               ? sz.h
               : grid_interp<DIM>(sz.grid, sz.n, sz.lo, sz.hi, q, nullptr);
  }
}

// _improve_level_set_newton: 5 damped Newton steps, alpha = 1,1,1/2,1/6,1/24
template <int DIM>
__global__ void k_improve_level_set(float *P, const int32_t *ids, int64_t m,
                                    SdfDev sdf, float deps) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t v = ids[i];
    float x[3];
    ldpt<DIM>(P, v, x);
    float alpha = 1.f;
    for (int it = 0; it < 5; ++it) {
      Dual d = sdf_eval<DIM, true>(sdf.ops, sdf.params, sdf.n_ops, x);
      float g2 = 0.f;
      for (int j = 0; j < DIM; ++j) g2 += d.g[j] * d.g[j];
      if (g2 < deps) g2 = deps;
      for (int j = 0; j < DIM; ++j) x[j] -= alpha * d.v * d.g[j] / g2;
      alpha /= (float)(it + 1);
    }
    if (DIM == 3)
      reinterpret_cast<float4 *>(P)[v] = make_float4(x[0], x[1], x[2], 0.f);
    else
      reinterpret_cast<float2 *>(P)[v] = make_float2(x[0], x[1]);
  }
}

// ---------------------------------------------------------------------------
// dihedral angles (fast_geometry.cpp:351-418 layout: 6 per cell, edge i
// between vertices E[i] with the opposite edge E[5-i])
__constant__ int kDhE[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};

template <typename T>
__device__ __forceinline__ T dihedral(const T *p0, const T *p1, const T *p2,
                                      const T *p3) {
  T v1[3], v2[3], v3[3];
  for (int j = 0; j < 3; ++j) {
    v1[j] = p1[j] - p0[j];
    v2[j] = p2[j] - p0[j];
    v3[j] = p3[j] - p0[j];
  }
  T n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
  T n2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
  T n3 = sqrt(v3[0] * v3[0] + v3[1] * v3[1] + v3[2] * v3[2]);
  for (int j = 0; j < 3; ++j) {
    v1[j] /= n1;
    v2[j] /= n2;
    v3[j] /= n3;
  }
  T d23 = v2[0] * v3[0] + v2[1] * v3[1] + v2[2] * v3[2];
  T d12 = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
  T d13 = v1[0] * v3[0] + v1[1] * v3[1] + v1[2] * v3[2];
  T c12[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
              v1[0] * v2[1] - v1[1] * v2[0]};
  T c13[3] = {v1[1] * v3[2] - v1[2] * v3[1], v1[2] * v3[0] - v1[0] * v3[2],
              v1[0] * v3[1] - v1[1] * v3[0]};
  T m12 = sqrt(c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2]);
  T m13 = sqrt(c13[0] * c13[0] + c13[1] * c13[1] + c13[2] * c13[2]);
  return acos((d23 - d12 * d13) / (m12 * m13));
}

// vertex v of a cell as FP64: engine points (float4 rows) or caller FP64
// points (3 doubles per row, as the reference's numpy arrays)
__device__ __forceinline__ void load_xyz(const float *P, int64_t v, double *x) {
  float4 q = __ldg(reinterpret_cast<const float4 *>(P) + v);
  x[0] = q.x;
  x[1] = q.y;
  x[2] = q.z;
}
__device__ __forceinline__ void load_xyz(const double *X, int64_t v, double *x) {
  x[0] = X[3 * v];
  x[1] = X[3 * v + 1];
  x[2] = X[3 * v + 2];
}

template <typename PT>
__global__ void k_dihedral(const PT *P, const int32_t *cells, int64_t nc,
                           double *ang) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc * 6;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t c = i / 6;
    int e = (int)(i % 6);
    double x[4][3];
    int vid[4] = {kDhE[e][0], kDhE[e][1], kDhE[5 - e][0], kDhE[5 - e][1]};
    for (int k = 0; k < 4; ++k) load_xyz(P, cells[4 * c + vid[k]], x[k]);
    ang[i] = dihedral<double>(x[0], x[1], x[2], x[3]);
  }
}

__global__ void k_dihedral_flags(const float *P, const int32_t *cells,
                                 int64_t cap, int count_index, float amin,
                                 float amax, int32_t *flags, int64_t *counters) {
  int64_t nc = min(counters[count_index], cap);
  unsigned long long bad = 0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    float x[4][3];
    for (int k = 0; k < 4; ++k) {
      float4 q = __ldg(reinterpret_cast<const float4 *>(P) + cells[4 * c + k]);
      x[k][0] = q.x;
      x[k][1] = q.y;
      x[k][2] = q.z;
    }
    int f = 0;
    for (int e = 0; e < 6; ++e) {
      float a = dihedral<float>(x[kDhE[e][0]], x[kDhE[e][1]], x[kDhE[5 - e][0]],
                                x[kDhE[5 - e][1]]);
      if (a < amin || a > amax || !(a == a)) f = 1;
    }
    flags[c] = f;
    bad += f;
  }
  for (int o = 16; o; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
  if ((threadIdx.x & 31) == 0 && bad)
    atomicAdd((unsigned long long *)&counters[DM_CNT_BAD], bad);
}

// gradient of the squared circumradius of (p0,p1,p2,p3) with respect to p0
// (geometry/cpp/fast_geometry.cpp:580-666: explicit circumcentre formula in
// coordinates translated to p3)
template <typename T>
__device__ __forceinline__ void circum_grad(const T *p0, const T *p1,
                                            const T *p2, const T *p3, T *g) {
  T x1 = p0[0] - p3[0], y1 = p0[1] - p3[1], z1 = p0[2] - p3[2];
  T x2 = p1[0] - p3[0], y2 = p1[1] - p3[1], z2 = p1[2] - p3[2];
  T x3 = p2[0] - p3[0], y3 = p2[1] - p3[1], z3 = p2[2] - p3[2];
  T s1 = x1 * x1 + y1 * y1 + z1 * z1;
  T s2 = x2 * x2 + y2 * y2 + z2 * z2;
  T s3 = x3 * x3 + y3 * y3 + z3 * z3;
  // a = det(rows p0', p1', p2'); its partials w.r.t. p0' are the cofactors
  T ax = y2 * z3 - y3 * z2, ay = z2 * x3 - x2 * z3, az = x2 * y3 - x3 * y2;
  T a = x1 * ax + y1 * ay + z1 * az;
  // D = sum_i s_i * (cross of the other two rows), signs as for the
  // circumcentre numerator; the reference's Dx, Dy, Dz
  T u = s2 * z3 - s3 * z2, vq = s2 * y3 - s3 * y2, wq = s2 * x3 - s3 * x2;
  T Dx = -s1 * ax + y1 * u - z1 * vq;
  T Dy = -s1 * ay - x1 * u + z1 * wq;
  T Dz = -s1 * az + x1 * vq - y1 * wq;
  // partial derivatives of D w.r.t. (x1, y1, z1)
  T dDx[3] = {-2 * x1 * ax, -2 * y1 * ax + u, -2 * z1 * ax - vq};
  T dDy[3] = {-2 * x1 * ay - u, -2 * y1 * ay, -2 * z1 * ay + wq};
  T dDz[3] = {-2 * x1 * az + vq, -2 * y1 * az - wq, -2 * z1 * az};
  T da[3] = {ax, ay, az};
  T sD = Dx * Dx + Dy * Dy + Dz * Dz;
  for (int k = 0; k < 3; ++k)
    g[k] = (Dx * dDx[k] + Dy * dDy[k] + Dz * dDz[k]) / (2 * a * a) -
           (da[k] * sD) / (2 * a * a * a);
}

__global__ void k_circum_grad(const double *p0, const double *p1,
                              const double *p2, const double *p3, int64_t m,
                              double *g) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    circum_grad<double>(p0 + 3 * i, p1 + 3 * i, p2 + 3 * i, p3 + 3 * i, g + 3 * i);
}

// winner[v] = largest flagged cell index whose vertex 0 is v (numpy's
// buffered fancy-index += keeps the last duplicate)
__global__ void k_sliver_winner(const int32_t *cells, int64_t cap, int count_index,
                                const int32_t *flags, const int64_t *counters,
                                int32_t *winner) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x)
    if (flags[c]) atomicMax(&winner[cells[4 * c]], (int)c);
}

__global__ void k_sliver_delta(const float *P, const int32_t *cells, int64_t cap,
                               int count_index, const int32_t *flags,
                               const int64_t *counters, const int32_t *winner,
                               float step_h0, float4 *delta) {
  int64_t nc = min(counters[count_index], cap);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nc;
       c += (int64_t)gridDim.x * blockDim.x) {
    if (!flags[c]) continue;
    int v0 = cells[4 * c];
    if (winner[v0] != (int)c) continue;
    double xd[4][3];
    for (int k = 0; k < 4; ++k) {
      float4 q = __ldg(reinterpret_cast<const float4 *>(P) + cells[4 * c + k]);
      xd[k][0] = q.x;
      xd[k][1] = q.y;
      xd[k][2] = q.z;
    }
    double g[3];
    circum_grad<double>(xd[0], xd[1], xd[2], xd[3], g);
    for (int j = 0; j < 3; ++j)
      if (isinf(g[j])) g[j] = 1.0;
    double nrm = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    delta[v0] = make_float4((float)(step_h0 * (g[0] / nrm)),
                            (float)(step_h0 * (g[1] / nrm)),
                            (float)(step_h0 * (g[2] / nrm)), 0.f);
  }
}

__global__ void k_sliver_apply(float *P, int64_t n, const int32_t *winner,
                               const float4 *delta, int grid_exp) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    if (winner[v] < 0) continue;
    float4 p = reinterpret_cast<float4 *>(P)[v], d = delta[v];
    reinterpret_cast<float4 *>(P)[v] =
        make_float4(to_grid(p.x + d.x, grid_exp), to_grid(p.y + d.y, grid_exp),
                    to_grid(p.z + d.z, grid_exp), 0.f);
  }
}

// ---------------------------------------------------------------------------
// host launchers
static SdfDev to_sdf(const dm_sdf_program *p) {
  SdfDev s;
  s.ops = p->ops;
  s.params = p->params;
  s.n_ops = p->n_ops;
  return s;
}

int filter_cells(int dim, const float *P, const int32_t *cells, int64_t cap,
                 const dm_sdf_program *sdf, float geps, int32_t *out,
                 int64_t *counters, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(sdf && sdf->dim == dim, "sdf program dimension");
  DM_CUDA_TRY(cudaMemsetAsync(&counters[DM_CNT_KEPT], 0, sizeof(int64_t), s));
  int nb = grid_for(cap, 256);
  if (dim == 3)
    k_filter_cells<3><<<nb, 256, 0, s>>>(P, cells, cap, to_sdf(sdf), geps, out, counters);
  else
    k_filter_cells<2><<<nb, 256, 0, s>>>(P, cells, cap, to_sdf(sdf), geps, out, counters);
  DM_LAUNCH_CHECK();
  note_launches(1);
  return DM_OK;
}

int cell_centroids(int dim, const float *P, const int32_t *cells, int64_t cap,
                   const int64_t *counters, float *cen, cudaStream_t s) {
  int nb = grid_for(cap, 256);
  if (dim == 3)
    k_centroids<3><<<nb, 256, 0, s>>>(P, cells, cap, counters, cen);
  else
    k_centroids<2><<<nb, 256, 0, s>>>(P, cells, cap, counters, cen);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// cnt: counts, then fill cursors, then the list of high-incidence vertices;
// tmp: scan scratch followed by the list length
static size_t carve_adj(Carve &c, int dim, int64_t n, int64_t cap_cells, int32_t **cnt,
                        int32_t **off, int32_t **raw, int32_t **tmp, int32_t **nbig) {
  const int NV = dim + 1;
  *cnt = c.take<int32_t>(n);
  *off = c.take<int32_t>(n + 1);
  *raw = c.take<int32_t>((size_t)NV * (NV - 1) * cap_cells);
  *tmp = c.take<int32_t>(scan_tmp_elems(n));
  *nbig = c.take<int32_t>(1);
  return c.used;
}

size_t adjacency_workspace(int dim, int64_t n, int64_t cap_cells) {
  Carve c(nullptr, 0);
  int32_t *a, *b, *d, *e, *f;
  return carve_adj(c, dim, n, cap_cells, &a, &b, &d, &e, &f) + 256;
}

int adjacency(int dim, int64_t n, const int32_t *cells, int64_t cap_cells,
              int count_index, int32_t *adj, int adj_cap, int32_t *deg,
              int64_t *counters, void *ws, size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(adj_cap > 0, "adj_cap must be positive");
  DM_ARG_CHECK(count_index >= 0 && count_index < DM_NCOUNTERS, "count_index");
  DM_ARG_CHECK(n >= 0 && n < (1 << 30) && cap_cells >= 0, "sizes");
  DM_ARG_CHECK((dim + 1) * dim * cap_cells < (1ll << 31), "too many cells");
  Carve c(ws, ws_bytes);
  int32_t *cnt, *off, *raw, *tmp, *nbig;
  carve_adj(c, dim, n, cap_cells, &cnt, &off, &raw, &tmp, &nbig);
  if (!c.ok() || !ws) {
    set_error("adjacency: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  DM_CUDA_TRY(cudaMemsetAsync(&counters[DM_CNT_EDGES], 0, sizeof(int64_t), s));
  DM_CUDA_TRY(cudaMemsetAsync(&counters[DM_CNT_MAXDEG], 0, sizeof(int64_t), s));
  if (n == 0) return DM_OK;
  DM_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n, s));
  int nb = grid_for(cap_cells, 256);
  if (dim == 3)
    k_adj_count<4><<<nb, 256, 0, s>>>(cells, cap_cells, counters, count_index, cnt);
  else
    k_adj_count<3><<<nb, 256, 0, s>>>(cells, cap_cells, counters, count_index, cnt);
  int rc = exclusive_scan_i32(cnt, off, n, tmp, s);
  if (rc) return rc;
  DM_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n, s));
  if (dim == 3)
    k_adj_fill<4><<<nb, 256, 0, s>>>(cells, cap_cells, counters, count_index, off, cnt, raw);
  else
    k_adj_fill<3><<<nb, 256, 0, s>>>(cells, cap_cells, counters, count_index, off, cnt, raw);
  DM_CUDA_TRY(cudaMemsetAsync(nbig, 0, sizeof(int32_t), s));
  k_adj_dedup_thread<<<grid_for(n, 256), 256, 0, s>>>(n, off, raw, adj, adj_cap, deg, cnt, nbig,
                                                      counters);
  k_adj_dedup<<<kSMs * 4, 32 * ADJ_WARPS, 0, s>>>(cnt, nbig, off, raw, adj, adj_cap, deg,
                                                   counters);
  k_half_edges<<<1, 1, 0, s>>>(counters);
  DM_LAUNCH_CHECK();
  note_launches(8);
  return DM_OK;
}

int bar_blocks(int dim, int64_t n) {
  int vpb = dim == 3 ? BarCfg<3>::VPB : BarCfg<2>::VPB;
  int64_t b = (n + vpb - 1) / vpb;
  return (int)(b < 1 ? 1 : b);
}

int bar_sums(int dim, const float *P, int64_t n, const int32_t *adj,
             int adj_cap, const int32_t *deg, const dm_sizing *sz,
             double *partials, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(sz != nullptr, "sizing");
  int nblk = bar_blocks(dim, n);
  DM_ARG_CHECK(nblk <= 1 << 24, "too many points");
  SizingDev d = to_dev(sz);
  if (dim == 3)
    k_bar_sums<3><<<nblk, 256, 0, s>>>(P, n, adj, adj_cap, deg, d, partials);
  else
    k_bar_sums<2><<<nblk, 256, 0, s>>>(P, n, adj, adj_cap, deg, d, partials);
  k_bar_scale<<<1, 1024, 0, s>>>(partials, nblk, dim);
  DM_LAUNCH_CHECK();
  note_launches(2);
  return DM_OK;
}

int update_points(int dim, const float *P, float *Pout, int64_t n,
                  const int32_t *adj, int adj_cap, const int32_t *deg,
                  const dm_sizing *sz, const double *partials, float L0mult,
                  float dt, int64_t nfix, const dm_sdf_program *levels,
                  int n_levels, float hmin, float deps, float *maxf,
                  int grid_exp, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(n_levels >= 0 && n_levels <= 4, "at most 4 levels");
  Levels L;
  L.n = n_levels;
  for (int i = 0; i < n_levels; ++i) {
    DM_ARG_CHECK(levels[i].dim == dim, "level dimension");
    L.lv[i] = to_sdf(&levels[i]);
  }
  int nblk = bar_blocks(dim, n);
  SizingDev d = to_dev(sz);
  if (dim == 3)
    k_update<3><<<nblk, 256, 0, s>>>(P, Pout, n, adj, adj_cap, deg, d, partials,
                                     nblk, L0mult, dt, nfix, L, hmin, deps, maxf,
                                     grid_exp);
  else
    k_update<2><<<nblk, 256, 0, s>>>(P, Pout, n, adj, adj_cap, deg, d, partials,
                                     nblk, L0mult, dt, nfix, L, hmin, deps, maxf,
                                     grid_exp);
  // the result goes to maxf[dm_bar_blocks(n)], the slot callers size
  // (and read) independently of the dimension
  const int slot = max(bar_blocks(2, n), bar_blocks(3, n));
  k_max_reduce<<<1, 1024, 0, s>>>(maxf, nblk, slot);
  DM_LAUNCH_CHECK();
  note_launches(2);
  return DM_OK;
}

int slot_midpoints(int dim, const float *P, int64_t n, const int32_t *adj,
                   int adj_cap, const int32_t *deg, float *mid, cudaStream_t s) {
  int nb = grid_for(n * adj_cap, 256);
  if (dim == 3)
    k_slot_mid<3><<<nb, 256, 0, s>>>(P, n, adj, adj_cap, deg, mid);
  else
    k_slot_mid<2><<<nb, 256, 0, s>>>(P, n, adj, adj_cap, deg, mid);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int sdf_eval_launch(const dm_sdf_program *p, const float *x, int64_t n,
                    int stride, float *d, float *grad, cudaStream_t s) {
  DM_ARG_CHECK(p && (p->dim == 2 || p->dim == 3), "sdf program");
  DM_ARG_CHECK(stride >= p->dim, "x_stride < dim");
  int nb = grid_for(n, 256);
  if (p->dim == 3)
    k_sdf_eval<3><<<nb, 256, 0, s>>>(to_sdf(p), x, n, stride, d, grad);
  else
    k_sdf_eval<2><<<nb, 256, 0, s>>>(to_sdf(p), x, n, stride, d, grad);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int sizing_eval_launch(const dm_sizing *sz, const float *x, int64_t n,
                       int stride, float *h, cudaStream_t s) {
  DM_ARG_CHECK(sz && (sz->dim == 2 || sz->dim == 3), "sizing");
  DM_ARG_CHECK(sz->kind == DM_SIZING_CONST || sz->kind == DM_SIZING_GRID,
               "sizing kind must be const or grid");
  int nb = grid_for(n, 256);
  if (sz->dim == 3)
    k_sizing_eval<3><<<nb, 256, 0, s>>>(to_dev(sz), x, n, stride, h);
  else
    k_sizing_eval<2><<<nb, 256, 0, s>>>(to_dev(sz), x, n, stride, h);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int improve_level_set(int dim, float *P, const int32_t *ids, int64_t m,
                      const dm_sdf_program *sdf, float deps, cudaStream_t s) {
  DM_ARG_CHECK(sdf && sdf->dim == dim, "sdf program dimension");
  int nb = grid_for(m, 256);
  if (dim == 3)
    k_improve_level_set<3><<<nb, 256, 0, s>>>(P, ids, m, to_sdf(sdf), deps);
  else
    k_improve_level_set<2><<<nb, 256, 0, s>>>(P, ids, m, to_sdf(sdf), deps);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int dihedral_angles(const float *P, const int32_t *cells, int64_t nc,
                    double *ang, cudaStream_t s) {
  if (nc == 0) return DM_OK;
  k_dihedral<float><<<grid_for(nc * 6, 256), 256, 0, s>>>(P, cells, nc, ang);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int dihedral_angles_f64(const double *X, const int32_t *cells, int64_t nc,
                        double *ang, cudaStream_t s) {
  if (nc == 0) return DM_OK;
  k_dihedral<double><<<grid_for(nc * 6, 256), 256, 0, s>>>(X, cells, nc, ang);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int circumsphere_grad(const double *p0, const double *p1, const double *p2,
                      const double *p3, int64_t m, double *g, cudaStream_t s) {
  k_circum_grad<<<grid_for(m, 256), 256, 0, s>>>(p0, p1, p2, p3, m, g);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int dihedral_flags(const float *P, const int32_t *cells, int64_t cap,
                   int count_index, float amin, float amax, int32_t *flags,
                   int64_t *counters, cudaStream_t s) {
  DM_CUDA_TRY(cudaMemsetAsync(&counters[DM_CNT_BAD], 0, sizeof(int64_t), s));
  k_dihedral_flags<<<grid_for(cap, 256), 256, 0, s>>>(P, cells, cap, count_index,
                                                     amin, amax, flags, counters);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int sliver_perturb(float *P, int64_t n_points, const int32_t *cells,
                   int64_t cap, int count_index, const int32_t *flags,
                   float step_h0, int grid_exp, void *ws, size_t ws_bytes,
                   int64_t *counters, cudaStream_t s) {
  Carve c(ws, ws_bytes);
  int32_t *winner = c.take<int32_t>(n_points);
  float4 *delta = c.take<float4>(n_points);
  if (!c.ok() || !ws) {
    set_error("sliver_perturb: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  DM_CUDA_TRY(cudaMemsetAsync(winner, 0xff, sizeof(int32_t) * n_points, s));
  int nb = grid_for(cap, 256);
  k_sliver_winner<<<nb, 256, 0, s>>>(cells, cap, count_index, flags, counters, winner);
  k_sliver_delta<<<nb, 256, 0, s>>>(P, cells, cap, count_index, flags, counters,
                                    winner, step_h0, delta);
  k_sliver_apply<<<grid_for(n_points, 256), 256, 0, s>>>(P, n_points, winner, delta,
                                                          grid_exp);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

size_t sliver_workspace(int64_t n_points) {
  Carve c(nullptr, 0);
  c.take<int32_t>(n_points);
  c.take<float4>(n_points);
  return c.used + 256;
}

}  // namespace dm
