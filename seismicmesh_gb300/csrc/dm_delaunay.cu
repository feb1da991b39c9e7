// GPU Delaunay triangulation by independent vertex stars.
//
// Replaces the CGAL rebuild the reference performs every DistMesh iteration
// (generation/mesh_generator.py:465-469 -> DelaunayTriangulation{,3}.insert,
// generation/cpp/delaunay_class.cpp:108-121, delaunay_class3.cpp:116-129,
// and get_finite_cells, delaunay_class.cpp:232-265, delaunay_class3.cpp:
// 276-310).  The Delaunay triangulation of points in general position (and
// of any point set under a fixed symbolic perturbation) is unique, so it can
// be assembled from the stars of its vertices computed independently:
//
//   star(p) = all Delaunay cells incident to p.
//
// One warp computes one star by gift wrapping around p: starting from a
// certified seed cell, every face through p is crossed by a query that
// returns the point whose sphere through the face is smallest on the far
// side (an insphere total order).  All predicates are exact (see
// dm_predicates.cuh), so stars of different vertices agree and every cell is
// emitted once, by its smallest vertex index.
//
// Level 1 runs the queries on the points within distance R of p, held in
// shared memory.  A cell found this way whose circumball lies inside B(p, R)
// is certified (every point that could invalidate it was examined).  A star
// with an uncertified cell or an open (convex-hull) face is handed to level 2,
// whose queries walk the uniform grid and its coarse blocks and are exact
// over the whole point set.
#include <float.h>
#include <limits.h>
#include <string.h>

#include "dm_common.cuh"
#include "dm_predicates.cuh"
#include "dm_fixed.cuh"

namespace dm {

using dmp::insph3_sos;
using dmp::incirc2_sos;

struct GridParams {
  float lo[3];
  float cs, inv_cs;
  int dims[3];
  int ncells;
  int bs;  // coarse block edge (cells)
  int bdims[3];
  int nblocks;
  int dim;
  // every coordinate is a multiple of 2^gfix and |coordinate| < 2^(gfix+29):
  // all predicates can use the fixed-point path; kNoFix otherwise
  int gfix;
};

constexpr int kNoFix = -100000;

// level-3 star storage: per-warp slots in the workspace
constexpr int L3_CAP_TRI = 16384, L3_CAP_OPEN = 8192, L3_WARPS = 4, L3_BLOCKS = 38;
constexpr int kCntL3 = 11;  // counters slot: stars deferred to level 3
constexpr int kCntL2Next = 12;  // counters slot: next escalated star for level 2

struct DTArgs {
  int dim;
  int64_t n;
  const float *P;  // float4 (3D) or float2 (2D)
  GridParams *gp;
  int *bbox;          // 6 ordered ints
  int *occ;           // occupied cells of the first grid
  int32_t *cell_of;   // [n]
  int32_t *slot;      // [n]
  int32_t *cell_cnt;  // [cap_cells]
  int32_t *cell_start;  // [cap_cells + 1]
  int32_t *sorted;    // [n]
  int32_t *scan_tmp;
  int32_t *blk_cnt;   // [cap_blocks]
  float *blk_box;     // [cap_blocks * 6]
  uint8_t *dup;       // [n]
  float4 *spts;       // [n] points in cell order: x, y, z, id bits (-1: duplicate)
  int32_t *l3_list;   // [n] escalated stars deferred to level 3
  int3 *l3_tri, *l3_open;  // level-3 star storage, one slot per warp
  int32_t *l3_cnt;
  int32_t *esc;       // [n]
  int4 *esc_seed;     // [n]
  // hull candidates (3D): vertices whose level-1 star was not closed,
  // bucketed by coarse block (o_start: nullptr until they are built)
  uint8_t *hullc;     // [n]
  int32_t *o_cnt;     // [cap_blocks] counts, then fill cursors
  int32_t *o_start;   // [cap_blocks + 1]
  int *o_box;         // [cap_blocks * 6] order-preserving ints (f2o)
  float4 *o_pts;      // [n] x, y, z, id bits
  float4 *o_tab;      // [2 * cap_blocks] non-empty candidate blocks: (lo, start bits),
                      // (hi, count bits)
  int32_t *o_ntab;    // [1] entries of o_tab
  int use_o;          // hull scans read the hull candidates
  int32_t *cells;
  int64_t cap_cells_out;
  int64_t *counters;
  int64_t cap_cells, cap_blocks;
  int dbg_vertex;  // debug aid: level-1 state of this vertex goes to dbg
  int32_t *dbg;
  int dbg_full;    // debug aid: face queries always scan the whole half-space
};

static size_t carve_dt(Carve &c, DTArgs &a, int dim, int64_t n) {
  a.cap_cells = 2 * n + 4096;
  a.cap_blocks = a.cap_cells;
  a.gp = c.take<GridParams>(1);
  a.bbox = c.take<int>(8);
  a.occ = c.take<int>(1);
  a.cell_of = c.take<int32_t>(n);
  a.slot = c.take<int32_t>(n);
  a.cell_cnt = c.take<int32_t>(a.cap_cells);
  a.cell_start = c.take<int32_t>(a.cap_cells + 1);
  a.sorted = c.take<int32_t>(n);
  a.scan_tmp = c.take<int32_t>(scan_tmp_elems(a.cap_cells));
  a.blk_cnt = c.take<int32_t>(a.cap_blocks);
  a.blk_box = c.take<float>(a.cap_blocks * 6);
  a.dup = c.take<uint8_t>(n);
  a.spts = c.take<float4>(n);
  a.l3_list = c.take<int32_t>(n);
  a.l3_tri = c.take<int3>((size_t)L3_BLOCKS * L3_WARPS * L3_CAP_TRI);
  a.l3_open = c.take<int3>((size_t)L3_BLOCKS * L3_WARPS * L3_CAP_OPEN);
  a.l3_cnt = c.take<int32_t>((size_t)L3_BLOCKS * L3_WARPS * 4);
  a.esc = c.take<int32_t>(n);
  a.esc_seed = c.take<int4>(n);
  a.hullc = c.take<uint8_t>(n);
  a.o_cnt = c.take<int32_t>(a.cap_blocks);
  a.o_start = c.take<int32_t>(a.cap_blocks + 1);
  a.o_box = c.take<int>(a.cap_blocks * 6);
  a.o_pts = c.take<float4>(n);
  a.o_tab = c.take<float4>(2 * a.cap_blocks);
  a.o_ntab = c.take<int32_t>(4);
  return c.used;
}

// ---------------------------------------------------------------------------
// point access
template <int DIM>
__device__ __forceinline__ void load_pt(const float *P, int i, float *x) {
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

// ---------------------------------------------------------------------------
// grid build
__global__ void k_bbox_init(int *bbox) {
  if (threadIdx.x < 3) {
    bbox[threadIdx.x] = f2o(FLT_MAX);
    bbox[3 + threadIdx.x] = f2o(-FLT_MAX);
  }
  if (threadIdx.x == 0) bbox[6] = INT_MAX;  // smallest lowest-set-bit exponent
}

// exponent of the lowest set bit of a finite non-zero float; INT_MAX for 0
__device__ __forceinline__ int lsb_exponent(float x) {
  uint32_t u = __float_as_uint(x);
  int e = (int)((u >> 23) & 0xffu);
  uint32_t m = u & 0x7fffffu;
  if (e == 0) return m ? -149 + __ffs(m) - 1 : INT_MAX;
  return e - 150 + __ffs(m | 0x800000u) - 1;
}

template <int DIM>
__global__ void k_bbox(const float *P, int64_t n, int *bbox, int64_t *counters) {
  float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  bool bad = false;
  int lsb = INT_MAX;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x[3];
    load_pt<DIM>(P, (int)i, x);
    for (int k = 0; k < DIM; ++k) {
      if (!isfinite(x[k])) bad = true;
      mn[k] = fminf(mn[k], x[k]);
      mx[k] = fmaxf(mx[k], x[k]);
      lsb = min(lsb, lsb_exponent(x[k]));
    }
  }
  for (int o = 16; o; o >>= 1) lsb = min(lsb, __shfl_xor_sync(0xffffffffu, lsb, o));
  if ((threadIdx.x & 31) == 0 && lsb != INT_MAX) atomicMin(&bbox[6], lsb);
  for (int k = 0; k < DIM; ++k) {
    for (int o = 16; o; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < DIM; ++k) {
      atomicMin(&bbox[k], f2o(mn[k]));
      atomicMax(&bbox[3 + k], f2o(mx[k]));
    }
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0)
    flag_or(counters, DM_FLAG_NONFINITE);
}

__global__ void k_grid_params(GridParams *gp, const int *bbox, int64_t n,
                              int dim, int64_t cap_cells, int64_t cap_blocks) {
  if (threadIdx.x != 0) return;
  double lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
  double maxext = 0;
  bool finite = true;
  for (int k = 0; k < dim; ++k) {
    lo[k] = o2f(bbox[k]);
    double hi = o2f(bbox[3 + k]);
    ext[k] = hi - lo[k];
    if (!isfinite(lo[k]) || !isfinite(hi)) finite = false;
    if (!(ext[k] >= 0) || !isfinite(ext[k])) ext[k] = 0;
    maxext = fmax(maxext, ext[k]);
  }
  if (!finite) {
    // non-finite input (already flagged): one cell, no triangulation work
    for (int k = 0; k < dim; ++k) {
      lo[k] = 0;
      ext[k] = 0;
    }
    maxext = 0;
  }
  if (maxext <= 0) maxext = 1;
  double vol = 1;
  for (int k = 0; k < dim; ++k) vol *= fmax(ext[k], maxext * 1e-3);
  double nn = (double)(n > 0 ? n : 1);
  double cs = pow(vol / nn, 1.0 / dim);
  if (!(cs > 0)) cs = maxext;
  int dims[3] = {1, 1, 1};
  for (int it = 0; it < 200; ++it) {
    double cells = 1;
    for (int k = 0; k < dim; ++k) {
      double q = fmin(floor(ext[k] / cs), 1e9);
      dims[k] = (int)q + 1;
      cells *= dims[k];
    }
    if (cells <= (double)cap_cells) break;
    cs *= 1.1;
  }
  // round cs up to a float that keeps floor((x-lo)/cs) within dims
  GridParams g;
  g.dim = dim;
  // common power-of-two grid of the coordinates (fixed-point predicates)
  g.gfix = kNoFix;
  if (finite) {
    double E = 0;
    for (int k = 0; k < dim; ++k) E = fmax(E, fmax(fabs(lo[k]), fabs(lo[k] + ext[k])));
    int lsb = bbox[6];
    if (E > 0 && lsb != INT_MAX && lsb >= ilogb(E) - 28) g.gfix = lsb;
  }
  g.cs = (float)cs;
  g.inv_cs = (float)(1.0 / cs);
  g.ncells = 1;
  g.bs = dim == 3 ? 4 : 8;
  g.nblocks = 1;
  for (int k = 0; k < 3; ++k) {
    g.lo[k] = k < dim ? (float)lo[k] : 0.f;
    g.dims[k] = k < dim ? dims[k] : 1;
    g.ncells *= g.dims[k];
    g.bdims[k] = (g.dims[k] + g.bs - 1) / g.bs;
    g.nblocks *= g.bdims[k];
  }
  *gp = g;
}

// occupied cells of the first grid (cells holding at least one point)
__global__ void k_occupancy(const int32_t *cnt, const GridParams *gp, int *occ) {
  const int64_t nc = gp->ncells;
  int c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc;
       i += (int64_t)gridDim.x * blockDim.x)
    c += cnt[i] > 0;
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(occ, c);
}

// The first cell size assumes the points fill their bounding box.  When they
// fill only part of it (a ball fills half of its cube, a salt body much
// less), every occupied cell holds several points and the level-1 gathers
// overflow their candidate slots.  Shrink the cells so that an occupied cell
// holds about one point, cs *= (occupied / n)^(1/dim), within the cell
// capacity.
__global__ void k_grid_refine(GridParams *gp, const int *bbox, const int *occ, int64_t n,
                              int64_t cap_cells) {
  if (threadIdx.x != 0) return;
  GridParams g = *gp;
  const double ppc = (double)n / (double)max(*occ, 1);
  if (!(ppc > 1.25)) return;
  double ext[3] = {0, 0, 0};
  for (int k = 0; k < g.dim; ++k) {
    ext[k] = (double)o2f(bbox[3 + k]) - (double)o2f(bbox[k]);
    if (!(ext[k] >= 0) || !isfinite(ext[k])) return;
  }
  double cs = g.cs * pow(1.0 / ppc, 1.0 / g.dim);
  int dims[3] = {1, 1, 1};
  for (int it = 0; it < 200; ++it) {
    double cells = 1;
    for (int k = 0; k < g.dim; ++k) {
      dims[k] = (int)fmin(floor(ext[k] / cs), 1e9) + 1;
      cells *= dims[k];
    }
    if (cells <= (double)cap_cells) break;
    cs *= 1.05;
  }
  if (!(cs < g.cs)) return;
  g.cs = (float)cs;
  g.inv_cs = (float)(1.0 / cs);
  g.ncells = 1;
  g.nblocks = 1;
  for (int k = 0; k < 3; ++k) {
    g.dims[k] = k < g.dim ? dims[k] : 1;
    g.ncells *= g.dims[k];
    g.bdims[k] = (g.dims[k] + g.bs - 1) / g.bs;
    g.nblocks *= g.bdims[k];
  }
  *gp = g;
}

__device__ __forceinline__ int cell_coord(const GridParams &g, float x, int k) {
  int c = (int)floorf((x - g.lo[k]) * g.inv_cs);
  return min(max(c, 0), g.dims[k] - 1);
}

template <int DIM>
__global__ void k_cell_count(const float *P, int64_t n, const GridParams *gp,
                             int32_t *cell_of, int32_t *slot, int32_t *cnt) {
  GridParams g = *gp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x[3];
    load_pt<DIM>(P, (int)i, x);
    int c = cell_coord(g, x[0], 0) +
            g.dims[0] * (cell_coord(g, x[1], 1) +
                         (DIM == 3 ? g.dims[1] * cell_coord(g, x[2], 2) : 0));
    cell_of[i] = c;
    slot[i] = atomicAdd(&cnt[c], 1);
  }
}

__global__ void k_cell_scatter(int64_t n, const int32_t *cell_of,
                               const int32_t *slot, const int32_t *start,
                               int32_t *sorted) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    sorted[start[cell_of[i]] + slot[i]] = (int32_t)i;
}

// sort each cell's points by index (deterministic order) and mark exact
// duplicates: every point equal to a lower-index point gets dup = 1.
template <int DIM>
__global__ void k_cell_sort(const float *P, const GridParams *gp,
                            const int32_t *start, int32_t *sorted,
                            uint8_t *dup, int64_t *counters) {
  int nc = gp->ncells;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc;
       c += gridDim.x * blockDim.x) {
    int b = start[c], e = start[c + 1];
    for (int i = b + 1; i < e; ++i) {
      int v = sorted[i], j = i - 1;
      while (j >= b && sorted[j] > v) {
        sorted[j + 1] = sorted[j];
        --j;
      }
      sorted[j + 1] = v;
    }
    int ndup = 0;
    for (int i = b; i < e; ++i) {
      int vi = sorted[i];
      float xi[3];
      load_pt<DIM>(P, vi, xi);
      uint8_t d = 0;
      for (int j = b; j < i; ++j) {
        float xj[3];
        load_pt<DIM>(P, sorted[j], xj);
        bool same = xi[0] == xj[0] && xi[1] == xj[1] && (DIM == 2 || xi[2] == xj[2]);
        if (same) {
          d = 1;
          break;
        }
      }
      dup[vi] = d;
      ndup += d;
    }
    if (ndup) {
      atomicAdd((unsigned long long *)&counters[DM_CNT_DUPS], (unsigned long long)ndup);
      flag_or(counters, DM_FLAG_DUPLICATES);
    }
  }
}

// cell-ordered copy of the points: one 16-byte load per visited point
template <int DIM>
__global__ void k_sorted_points(const float *P, int64_t n, const int32_t *sorted,
                                const uint8_t *dup, float4 *spts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int j = sorted[i];
    float x[3] = {0.f, 0.f, 0.f};
    load_pt<DIM>(P, j, x);
    spts[i] = make_float4(x[0], x[1], x[2], __int_as_float(dup[j] ? -1 : j));
  }
}

template <int DIM>
__global__ void k_block_boxes(const float *P, const GridParams *gp,
                              const int32_t *start, const int32_t *sorted,
                              int32_t *blk_cnt, float *blk_box) {
  GridParams g = *gp;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < g.nblocks;
       b += gridDim.x * blockDim.x) {
    int bx = b % g.bdims[0], by = (b / g.bdims[0]) % g.bdims[1],
        bz = b / (g.bdims[0] * g.bdims[1]);
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    int cnt = 0;
    int z0 = DIM == 3 ? bz * g.bs : 0, z1 = DIM == 3 ? min(z0 + g.bs, g.dims[2]) : 1;
    for (int cz = z0; cz < z1; ++cz)
      for (int cy = by * g.bs; cy < min(by * g.bs + g.bs, g.dims[1]); ++cy)
        for (int cx = bx * g.bs; cx < min(bx * g.bs + g.bs, g.dims[0]); ++cx) {
          int c = cx + g.dims[0] * (cy + g.dims[1] * cz);
          for (int i = start[c]; i < start[c + 1]; ++i) {
            float x[3];
            load_pt<DIM>(P, sorted[i], x);
            for (int k = 0; k < DIM; ++k) {
              mn[k] = fminf(mn[k], x[k]);
              mx[k] = fmaxf(mx[k], x[k]);
            }
            ++cnt;
          }
        }
    blk_cnt[b] = cnt;
    for (int k = 0; k < 3; ++k) {
      blk_box[6 * b + k] = mn[k];
      blk_box[6 * b + 3 + k] = mx[k];
    }
  }
}

// ---------------------------------------------------------------------------
// Hull candidates (3D).  Level 1 flags every vertex whose star it could not
// close among its candidates (an open star, no seed, or over capacity).  A
// vertex of the convex hull of the point set (symbolically perturbed, as
// every predicate here is) lies on the hull of any subset that contains it,
// so its level-1 star is open: the flagged set holds every hull vertex.  The
// maximum of an affine function over the points is reached at a hull
// vertex, so a half-space that holds no flagged vertex holds no point at
// all.  Hull scans (face queries whose half-space has no point near the
// face) read the flagged vertices, bucketed by coarse block with tight
// boxes, instead of every cell of every block the half-space crosses.
__device__ __forceinline__ int block_of_cell(const GridParams &g, int c) {
  const int cx = c % g.dims[0], cy = (c / g.dims[0]) % g.dims[1],
            cz = c / (g.dims[0] * g.dims[1]);
  return cx / g.bs + g.bdims[0] * (cy / g.bs + g.bdims[1] * (cz / g.bs));
}

__global__ void k_hc_init(const GridParams *gp, int32_t *o_cnt, int *o_box) {
  const int nb = gp->nblocks;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    o_cnt[b] = 0;
    for (int k = 0; k < 3; ++k) {
      o_box[6 * b + k] = f2o(FLT_MAX);
      o_box[6 * b + 3 + k] = f2o(-FLT_MAX);
    }
  }
}

__global__ void k_hc_count(int64_t n, const uint8_t *hullc, const int32_t *cell_of,
                           const GridParams *gp, int32_t *o_cnt) {
  const GridParams g = *gp;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x)
    if (hullc[v]) atomicAdd(&o_cnt[block_of_cell(g, cell_of[v])], 1);
}

__global__ void k_hc_fill(int64_t n, const float *P, const uint8_t *hullc,
                          const int32_t *cell_of, const GridParams *gp,
                          const int32_t *o_start, int32_t *o_cur, int *o_box,
                          float4 *o_pts) {
  const GridParams g = *gp;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    if (!hullc[v]) continue;
    const int b = block_of_cell(g, cell_of[v]);
    const int pos = o_start[b] + atomicAdd(&o_cur[b], 1);
    float x[3];
    load_pt<3>(P, (int)v, x);
    o_pts[pos] = make_float4(x[0], x[1], x[2], __int_as_float((int)v));
    for (int k = 0; k < 3; ++k) {
      atomicMin(&o_box[6 * b + k], f2o(x[k]));
      atomicMax(&o_box[6 * b + 3 + k], f2o(x[k]));
    }
  }
}

// table of the non-empty candidate blocks (tight box, range); hull scans
// walk it instead of every block index
__global__ void k_hc_table(const GridParams *gp, const int32_t *o_start, const int *o_box,
                           float4 *o_tab, int32_t *o_ntab) {
  const int nb = gp->nblocks;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const int s0 = o_start[b], s1 = o_start[b + 1];
    if (s0 == s1) continue;
    const int e = atomicAdd(o_ntab, 1);
    o_tab[2 * e] = make_float4(o2f(o_box[6 * b]), o2f(o_box[6 * b + 1]), o2f(o_box[6 * b + 2]),
                               __int_as_float(s0));
    o_tab[2 * e + 1] = make_float4(o2f(o_box[6 * b + 3]), o2f(o_box[6 * b + 4]),
                                   o2f(o_box[6 * b + 5]), __int_as_float(s1 - s0));
  }
}

// ---------------------------------------------------------------------------
// Level 1: shared-memory neighbourhoods
template <int DIM>
struct L1 {};
template <>
struct L1<3> {
  static constexpr int CAP = 128, PER = 4, K = 2, MAXTRI = 128, MAXOPEN = 96;
};
template <>
struct L1<2> {
  static constexpr int CAP = 64, PER = 2, K = 3, MAXTRI = 64, MAXOPEN = 4;
};

constexpr int L1_WARPS = 4;
// minimum resident blocks per SM requested from the register allocator
#ifndef DM_L1_MINB
#define DM_L1_MINB 4  // 128 registers: 4 blocks per SM measured 23 % faster than 1
#endif
#ifndef DM_L2_MINB
#define DM_L2_MINB 4  // 128 registers: measured 10 % faster than 5 blocks per SM (96)
#endif

template <int DIM>
struct WarpL1 {
  float4 c[L1<DIM>::CAP];  // relative coords (x,y,z) and lift (w)
  int4 ci[L1<DIM>::CAP];   // exact fixed-point relative coords; w = 1 if valid
  int id[L1<DIM>::CAP];    // global index
  uint32_t tri[L1<DIM>::MAXTRI];
  uint32_t open[L1<DIM>::MAXOPEN];
  int nc, ntri, nopen;
  int flags;
  float reff;
  int capped;  // the candidate radius was cut below the covered radius
};

__device__ __forceinline__ uint32_t pack3(int a, int b, int c) {
  return (uint32_t)a | ((uint32_t)b << 8) | ((uint32_t)c << 16);
}
__device__ __forceinline__ int un0(uint32_t t) { return t & 0xff; }
__device__ __forceinline__ int un1(uint32_t t) { return (t >> 8) & 0xff; }
__device__ __forceinline__ int un2(uint32_t t) { return (t >> 16) & 0xff; }

// warp argmin over (key, id); lanes with no candidate pass key=+inf, j=-1
__device__ __forceinline__ void warp_argmin(float &key, int &j, int &gid) {
  for (int o = 16; o; o >>= 1) {
    float k2 = __shfl_xor_sync(0xffffffffu, key, o);
    int j2 = __shfl_xor_sync(0xffffffffu, j, o);
    int g2 = __shfl_xor_sync(0xffffffffu, gid, o);
    bool take = (j2 >= 0) && (j < 0 || k2 < key || (k2 == key && g2 < gid));
    if (take) {
      key = k2;
      j = j2;
      gid = g2;
    }
  }
}

// ---- 3D level-1 predicates on shared candidates (p is the origin)
// exact orient3(p, a, b, c) once the filter has failed
__device__ __forceinline__ int o3L_exact(const WarpL1<3> &S, const float *P, int ip,
                                         int a, int b, int c, dmp::ExactScratch *W) {
  const int4 IA = S.ci[a], IB = S.ci[b], IC = S.ci[c];
  if (IA.w & IB.w & IC.w) return dmp::orient3_fx(IA, IB, IC);
  load_pt<3>(P, ip, W->pt[0]);
  load_pt<3>(P, S.id[a], W->pt[1]);
  load_pt<3>(P, S.id[b], W->pt[2]);
  load_pt<3>(P, S.id[c], W->pt[3]);
  return dmp::orient3_slow(W->pt[0], W->pt[1], W->pt[2], W->pt[3], W);
}

__device__ __forceinline__ int o3L(const WarpL1<3> &S, const float *P, int ip,
                                   int a, int b, int c, dmp::ExactScratch *W) {
  float4 A = S.c[a], B = S.c[b], C = S.c[c];
  int s = dmp::orient3_rel_filter<float>(A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y,
                                         C.z, 16.0f * DMP_U32);
  if (s) return s;
  return o3L_exact(S, P, ip, a, b, c, W);
}

// sign of det with |error| <= c * perm; 0 when undecided (including
// overflow, underflow and NaN, which go to the exact stages)
__device__ __forceinline__ int filter_sign(float det, float perm, float c) {
  if (!(perm < 1e30f) || !(perm >= 1e-30f)) return 0;
  float err = c * perm;
  return det > err ? 1 : (det < -err ? -1 : 0);
}

// 3x3 determinant of rows (a, b, c) and its permanent
__device__ __forceinline__ float det3p(float a0, float a1, float a2, float b0, float b1,
                                       float b2, float c0, float c1, float c2, float &perm) {
  float m0 = b1 * c2 - b2 * c1, m1 = b2 * c0 - b0 * c2, m2 = b0 * c1 - b1 * c0;
  float p0 = fabsf(b1 * c2) + fabsf(b2 * c1), p1 = fabsf(b2 * c0) + fabsf(b0 * c2),
        p2 = fabsf(b0 * c1) + fabsf(b1 * c0);
  perm = fabsf(a0) * p0 + fabsf(a1) * p1 + fabsf(a2) * p2;
  return a0 * m0 + a1 * m1 + a2 * m2;
}

// insph3(p, a, b, c, y) for a fixed (a, b, c) and many y: expansion along
// the row of y, det = -y.x Mx + y.y My - y.z Mz + y.w Mw, with the 3x3
// minors of rows (a, b, c).  With FP32 inputs (relative coordinates and
// lifts rounded once) the error is below 17u * sum |y_k| perm(M_k); the
// filter uses 48u.
struct SphereRows {
  float mx, my, mz, mw, px, py, pz, pw;
};
__device__ __forceinline__ void sphere_rows(SphereRows &R, float4 A, float4 B, float4 C) {
  R.mx = det3p(A.y, A.z, A.w, B.y, B.z, B.w, C.y, C.z, C.w, R.px);
  R.my = det3p(A.x, A.z, A.w, B.x, B.z, B.w, C.x, C.z, C.w, R.py);
  R.mz = det3p(A.x, A.y, A.w, B.x, B.y, B.w, C.x, C.y, C.w, R.pz);
  R.mw = det3p(A.x, A.y, A.z, B.x, B.y, B.z, C.x, C.y, C.z, R.pw);
}
__device__ __forceinline__ int sphere_filter(const SphereRows &R, float4 Y) {
  float det = -Y.x * R.mx + Y.y * R.my - Y.z * R.mz + Y.w * R.mw;
  float perm = fabsf(Y.x) * R.px + fabsf(Y.y) * R.py + fabsf(Y.z) * R.pz + fabsf(Y.w) * R.pw;
  return filter_sign(det, perm, 48.0f * DMP_U32);
}

__device__ __forceinline__ int is3L_exact(const WarpL1<3> &S, const float *P, int ip,
                                          int a, int b, int c, int d, int &ovf,
                                          dmp::ExactScratch *W);

__device__ __forceinline__ int is3L(const WarpL1<3> &S, const float *P, int ip,
                                    int a, int b, int c, int d, int &ovf,
                                    dmp::ExactScratch *W) {
  float4 A = S.c[a], B = S.c[b], C = S.c[c], D = S.c[d];
  float X[3] = {A.x, A.y, A.z}, Y[3] = {B.x, B.y, B.z}, Z[3] = {C.x, C.y, C.z},
        Q[3] = {D.x, D.y, D.z};
  int s = dmp::insph3_rel_filter<float>(X, Y, Z, Q, A.w, B.w, C.w, D.w,
                                        48.0f * DMP_U32);
  if (s) return s;
  return is3L_exact(S, P, ip, a, b, c, d, ovf, W);
}

// exact perturbed insph3(p, a, b, c, d) once the filter has failed
__device__ __forceinline__ int is3L_exact(const WarpL1<3> &S, const float *P, int ip,
                                          int a, int b, int c, int d, int &ovf,
                                          dmp::ExactScratch *W) {
  const int4 IA = S.ci[a], IB = S.ci[b], IC = S.ci[c], ID = S.ci[d];
  if (IA.w & IB.w & IC.w & ID.w) return dmp::insph3_fx_sos(IA, IB, IC, ID);
  float(*pt)[3] = W->pt;
  load_pt<3>(P, ip, pt[0]);
  load_pt<3>(P, S.id[a], pt[1]);
  load_pt<3>(P, S.id[b], pt[2]);
  load_pt<3>(P, S.id[c], pt[3]);
  load_pt<3>(P, S.id[d], pt[4]);
  int s = dmp::insph3_slow(pt[0], pt[1], pt[2], pt[3], pt[4], &ovf, W);
  return s ? s : dmp::insph3_sos_tail(pt[0], pt[1], pt[2], pt[3], pt[4], W);
}

// gift-wrap query on face (p, a, b): winner among candidates y with
// orient3(p,a,b,y) > 0 whose sphere through the face is smallest; -1 if none.
// out of line: one copy serves the seed search and the walk (instruction
// cache); it owns no arrays (exact-stage temporaries live in W)
#ifdef DM_GW3L_INLINE
static __device__ __forceinline__ int gw3L(const WarpL1<3> &S, const float *P, int ip,
#else
static __device__ __noinline__ int gw3L(const WarpL1<3> &S, const float *P, int ip,
#endif
                                        int a, int b, int lane, int &ovf,
                                        dmp::ExactScratch *W) {
  const int nc = S.nc;
  float4 A = S.c[a], B = S.c[b];
  float nx = A.y * B.z - A.z * B.y, ny = A.z * B.x - A.x * B.z,
        nz = A.x * B.y - A.y * B.x;
  float nn = nx * nx + ny * ny + nz * nz;
  float tx = A.w * B.x - B.w * A.x, ty = A.w * B.y - B.w * A.y,
        tz = A.w * B.z - B.w * A.z;
  float inv = nn > 0.f ? 0.5f / nn : 0.f;
  float cx = (ty * nz - tz * ny) * inv, cy = (tz * nx - tx * nz) * inv,
        cz = (tx * ny - ty * nx) * inv;
  // orientation of every candidate against the face: Y . (A x B), with the
  // permanent terms of A x B for the error bound (16u, as orient3 filters)
  const float pnx = fabsf(A.y * B.z) + fabsf(A.z * B.y), pny = fabsf(A.z * B.x) + fabsf(A.x * B.z),
              pnz = fabsf(A.x * B.y) + fabsf(A.y * B.x);
  uint32_t pos = 0, und = 0;
  float bk = FLT_MAX;
  int bj = -1, bg = 0x7fffffff;
  // filtered orientations; the undecided ones go to one exact call site
  // below (keeps the unrolled loop small)
#pragma unroll
  for (int s = 0; s < L1<3>::PER; ++s) {
    int j = lane + 32 * s;
    if (j < nc && j != a && j != b) {
      float4 Y = S.c[j];
      float den = Y.x * nx + Y.y * ny + Y.z * nz;
      int o = filter_sign(den, fabsf(Y.x) * pnx + fabsf(Y.y) * pny + fabsf(Y.z) * pnz,
                          16.0f * DMP_U32);
      if (o > 0) pos |= 1u << s;
      if (o == 0) und |= 1u << s;
    }
  }
  while (und) {
    const int s = __ffs(und) - 1;
    und &= und - 1;
    if (o3L_exact(S, P, ip, a, b, lane + 32 * s, W) > 0) pos |= 1u << s;
  }
  for (uint32_t m = pos; m; m &= m - 1) {
    const int j = lane + 32 * (__ffs(m) - 1);
    float4 Y = S.c[j];
    float den = Y.x * nx + Y.y * ny + Y.z * nz;
    float tau = (Y.w - 2.f * (Y.x * cx + Y.y * cy + Y.z * cz)) / den;
    if (!(tau == tau) || !(den > 0.f)) tau = FLT_MAX;
    int g = S.id[j];
    if (bj < 0 || tau < bk || (tau == bk && g < bg)) {
      bk = tau;
      bj = j;
      bg = g;
    }
  }
  warp_argmin(bk, bj, bg);
  if (bj < 0) return -1;
  // verification: no positive candidate inside the sphere (p, a, b, bj)
  for (int it = 0; it < nc + 1; ++it) {
    SphereRows R;
    sphere_rows(R, A, B, S.c[bj]);
    int found = -1;
    uint32_t und2 = 0;
#pragma unroll
    for (int s = 0; s < L1<3>::PER; ++s) {
      int j = lane + 32 * s;
      if (found < 0 && (pos >> s & 1u) && j != bj) {
        int v = sphere_filter(R, S.c[j]);
        if (v < 0) found = j;
        if (v == 0) und2 |= 1u << s;
      }
    }
    while (found < 0 && und2) {
      const int s = __ffs(und2) - 1;
      und2 &= und2 - 1;
      if (is3L_exact(S, P, ip, a, b, bj, lane + 32 * s, ovf, W) < 0) found = lane + 32 * s;
    }
    unsigned m = __ballot_sync(0xffffffffu, found >= 0);
    if (!m) return bj;
    bj = __shfl_sync(0xffffffffu, found, __ffs(m) - 1);
  }
  return bj;
}

// find open edge (t -> s) (reverse of s -> t); returns index or -1
template <int DIM>
__device__ __forceinline__ int find_rev(const WarpL1<DIM> &S, int s, int t,
                                        int lane) {
  int hit = -1;
  for (int k = lane; k < S.nopen; k += 32) {
    uint32_t e = S.open[k];
    if (un0(e) == t && un1(e) == s) hit = k;
  }
  unsigned m = __ballot_sync(0xffffffffu, hit >= 0);
  if (!m) return -1;
  return __shfl_sync(0xffffffffu, hit, __ffs(m) - 1);
}

// circumball of cell (p, A, B, C) inside B(p, reff)?  Requires a well
// conditioned orientation so the float circumradius is trustworthy.
__device__ __forceinline__ bool certified3(float4 A, float4 B, float4 C,
                                           float reff) {
  float bcx = B.y * C.z - B.z * C.y, bcy = B.z * C.x - B.x * C.z,
        bcz = B.x * C.y - B.y * C.x;
  float cax = C.y * A.z - C.z * A.y, cay = C.z * A.x - C.x * A.z,
        caz = C.x * A.y - C.y * A.x;
  float abx = A.y * B.z - A.z * B.y, aby = A.z * B.x - A.x * B.z,
        abz = A.x * B.y - A.y * B.x;
  float det = A.x * bcx + A.y * bcy + A.z * bcz;
  float perm = fabsf(A.x) * (fabsf(B.y * C.z) + fabsf(B.z * C.y)) +
               fabsf(A.y) * (fabsf(B.z * C.x) + fabsf(B.x * C.z)) +
               fabsf(A.z) * (fabsf(B.x * C.y) + fabsf(B.y * C.x));
  if (!(fabsf(det) > 1e4f * 16.0f * DMP_U32 * perm)) return false;
  float nx = A.w * bcx + B.w * cax + C.w * abx;
  float ny = A.w * bcy + B.w * cay + C.w * aby;
  float nz = A.w * bcz + B.w * caz + C.w * abz;
  float num2 = nx * nx + ny * ny + nz * nz;  // (2 r det)^2 * ... = 4 r^2 det^2
  float lim = 0.99f * reff;
  return num2 <= lim * lim * det * det;
}

// Collect the candidate set Q of vertex p: every point within reff of p,
// reff chosen so |Q| <= CAP.  The cells within K of p's cell are scanned; the
// covered radius rcov is p's distance to the faces of that block (sides
// clipped by the grid need no limit).  A 16-bin histogram of d / r picks the
// largest radius whose ball holds <= CAP points; when the first bin alone
// overflows (dense clusters) the radius is divided by 16 and re-histogrammed.
// Fixed-point frame: coordinates relative to p at scale 2^g, where
// g = exponent(extent) - 28 keeps |relative coordinate| < 2^30 for points
// within `extent` of p (per axis).  Points that are not multiples of 2^g or
// fall outside the range get w = 0 and use the floating-point exact path.
struct FxFrame {
  int g;
  bool ok;  // p itself is representable
  long long P0[3];
};

// gfix != kNoFix: every point shares the grid 2^gfix (range checked when the
// grid was built), so that scale serves every star
template <int DIM>
__device__ __forceinline__ void fx_frame(FxFrame &fr, const float *p, float extent, int gfix) {
  if (gfix != kNoFix) {
    fr.g = gfix;
    fr.ok = true;
  } else {
    fr.g = dmp::float_exponent(extent) - 28;
    fr.ok = extent > 0.f && dmp::float_exponent(extent) > -100;
  }
  for (int k = 0; k < 3; ++k) fr.P0[k] = 0;
  for (int k = 0; k < DIM; ++k) fr.ok = fr.ok && dmp::float_to_fixed(p[k], fr.g, &fr.P0[k]);
}

template <int DIM>
__device__ __forceinline__ int4 fx_point(const FxFrame &fr, const float *x) {
  int v[3] = {0, 0, 0};
  if (!fr.ok) return make_int4(0, 0, 0, 0);
  for (int k = 0; k < DIM; ++k) {
    long long X;
    if (!dmp::float_to_fixed(x[k], fr.g, &X)) return make_int4(0, 0, 0, 0);
    long long d = X - fr.P0[k];
    if (d <= -(1ll << 30) || d >= (1ll << 30)) return make_int4(0, 0, 0, 0);
    v[k] = (int)d;
  }
  return make_int4(v[0], v[1], v[2], 1);
}

// Exact fixed-point coordinates of the candidates relative to p: scale 2^g
// with g chosen so that |relative coordinate| < 2^30.  A candidate (or the
// whole star, when p itself is not a multiple of 2^g) without an exact
// representation keeps w = 0 and uses the floating-point exact path.
template <int DIM>
__device__ __forceinline__ void fixed_coords(WarpL1<DIM> &S, const DTArgs &A,
                                             const float *px, int lane, int gfix) {
  const int nc = S.nc;
  float m = 0.f;
  for (int j = lane; j < nc; j += 32) {
    float4 c = S.c[j];
    m = fmaxf(m, fmaxf(fabsf(c.x), fmaxf(fabsf(c.y), DIM == 3 ? fabsf(c.z) : 0.f)));
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  FxFrame fr;
  fx_frame<DIM>(fr, px, m, gfix);
  for (int j = lane; j < nc; j += 32) {
    float xq[3];
    load_pt<DIM>(A.P, S.id[j], xq);
    S.ci[j] = fx_point<DIM>(fr, xq);
  }
  __syncwarp();
}

template <int DIM>
__device__ __forceinline__ void gather_l1(WarpL1<DIM> &S, const DTArgs &A, const GridParams &g,
                                          int ip, const float *px, int lane, int K) {
  const int W = 2 * K + 1;
  const int NCELL = DIM == 3 ? W * W * W : W * W;
  int cc[3];
  for (int k = 0; k < DIM; ++k) cc[k] = cell_coord(g, px[k], k);
  float rcov = FLT_MAX;
  for (int k = 0; k < DIM; ++k) {
    if (cc[k] - K > 0) rcov = fminf(rcov, px[k] - (g.lo[k] + (cc[k] - K) * g.cs));
    if (cc[k] + K + 1 < g.dims[k])
      rcov = fminf(rcov, (g.lo[k] + (cc[k] + K + 1) * g.cs) - px[k]);
  }
  // a block clipped on every side holds every point: any radius beyond the
  // grid diagonal is covered
  rcov = fminf(rcov, g.cs * (float)(g.dims[0] + g.dims[1] + g.dims[2] + 1));
  rcov = rcov * (1.f - 1e-5f);
  float rcnt = rcov;
  int bmax = -1;
  // the first pass also stores its points: when they fit (the usual case)
  // no second pass is needed
  if (lane == 0) S.nc = 0;
  __syncwarp();
  bool stored = false;
  for (int round = 0; round < 6 && bmax < 0; ++round, rcnt *= (1.f / 16.f)) {
    const float rc2 = rcnt * rcnt;
    int bins[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) bins[k] = 0;
    int total = 0;
    for (int t = lane; t < NCELL; t += 32) {
      int d0 = t % W - K, d1 = (t / W) % W - K, d2 = DIM == 3 ? t / (W * W) - K : 0;
      int x = cc[0] + d0, y = cc[1] + d1, z = DIM == 3 ? cc[2] + d2 : 0;
      if (x < 0 || y < 0 || z < 0 || x >= g.dims[0] || y >= g.dims[1] ||
          (DIM == 3 && z >= g.dims[2]))
        continue;
      int c = x + g.dims[0] * (y + g.dims[1] * z);
      for (int i = A.cell_start[c]; i < A.cell_start[c + 1]; ++i) {
        const float4 sq = A.spts[i];
        int q = __float_as_int(sq.w);
        if (q == ip || q < 0) continue;
        float xq[3] = {sq.x, sq.y, sq.z};
        float d2s = 0.f;
        for (int k = 0; k < DIM; ++k) {
          float dd = xq[k] - px[k];
          d2s += dd * dd;
        }
        if (d2s <= rc2) {
          ++total;
          int bidx = min(15, (int)(sqrtf(d2s) / rcnt * 16.f));
#pragma unroll
          for (int k = 0; k < 16; ++k) bins[k] += (k == bidx);
          if (round == 0) {
            const int slot = atomicAdd(&S.nc, 1);
            if (slot < L1<DIM>::CAP) {
              float r[3] = {0.f, 0.f, 0.f};
              for (int k = 0; k < DIM; ++k) r[k] = xq[k] - px[k];
              S.c[slot] = make_float4(r[0], r[1], r[2],
                                      DIM == 3 ? r[0] * r[0] + r[1] * r[1] + r[2] * r[2]
                                               : r[0] * r[0] + r[1] * r[1]);
              S.id[slot] = q;
            }
          }
        }
      }
    }
    for (int o = 16; o; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    if (total <= L1<DIM>::CAP) {
      bmax = 15;
      stored = round == 0;
      break;
    }
    int cum = 0;
    for (int k = 0; k < 16; ++k) {
      int v = bins[k];
      for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      cum += v;
      if (cum <= L1<DIM>::CAP) bmax = k;
    }
    if (bmax >= 0) break;
  }
  const float reff = bmax == 15 ? rcnt : rcnt * (bmax + 1) / 16.f * (1.f - 1e-5f);
  __syncwarp();
  if (lane == 0) {
    if (!stored) S.nc = 0;
    S.reff = bmax < 0 ? 0.f : reff;
    S.capped = bmax != 15 || rcnt < rcov;
  }
  __syncwarp();
  if (bmax < 0) return;
  if (stored) {
    fixed_coords<DIM>(S, A, px, lane, g.gfix);
    return;
  }
  const float rc2 = rcnt * rcnt;
  for (int t = lane; t < NCELL; t += 32) {
    int d0 = t % W - K, d1 = (t / W) % W - K, d2 = DIM == 3 ? t / (W * W) - K : 0;
    int x = cc[0] + d0, y = cc[1] + d1, z = DIM == 3 ? cc[2] + d2 : 0;
    if (x < 0 || y < 0 || z < 0 || x >= g.dims[0] || y >= g.dims[1] ||
        (DIM == 3 && z >= g.dims[2]))
      continue;
    int c = x + g.dims[0] * (y + g.dims[1] * z);
    for (int i = A.cell_start[c]; i < A.cell_start[c + 1]; ++i) {
      const float4 sq = A.spts[i];
      int q = __float_as_int(sq.w);
      if (q == ip || q < 0) continue;
      float xq[3] = {sq.x, sq.y, sq.z};
      float r[3] = {0, 0, 0}, d2s = 0.f;
      for (int k = 0; k < DIM; ++k) {
        r[k] = xq[k] - px[k];
        d2s += r[k] * r[k];
      }
      if (d2s > rc2) continue;
      int bidx = min(15, (int)(sqrtf(d2s) / rcnt * 16.f));
      if (bidx > bmax) continue;
      int slot = atomicAdd(&S.nc, 1);
      if (slot < L1<DIM>::CAP) {
        S.c[slot] = make_float4(r[0], r[1], r[2],
                                DIM == 3 ? r[0] * r[0] + r[1] * r[1] + r[2] * r[2]
                                         : r[0] * r[0] + r[1] * r[1]);
        S.id[slot] = q;
      }
    }
  }
  __syncwarp();
  if (lane == 0 && S.nc > L1<DIM>::CAP) S.nc = L1<DIM>::CAP;  // cannot happen
  __syncwarp();
  fixed_coords<DIM>(S, A, px, lane, g.gfix);
}

// is the cell (p, a, b, c) of a packed link triangle empty w.r.t. every
// candidate?  (exact, warp-cooperative)
__device__ __forceinline__ bool empty3L(const WarpL1<3> &S, const float *P, int ip,
                                        uint32_t tr, int lane, int &ovf,
                                        dmp::ExactScratch *W) {
  int a = un0(tr), b = un1(tr), c = un2(tr);
  SphereRows R;
  sphere_rows(R, S.c[a], S.c[b], S.c[c]);
  bool inside = false;
  for (int j = lane; j < S.nc; j += 32)
    if (!inside && j != a && j != b && j != c) {
      int v = sphere_filter(R, S.c[j]);
      if (v == 0) v = is3L_exact(S, P, ip, a, b, c, j, ovf, W);
      inside = v < 0;
    }
  return !__any_sync(0xffffffffu, inside);
}

// seed search (3D): returns packed link triangle or 0xffffffff
__device__ __forceinline__ uint32_t seed3L(const WarpL1<3> &S, const float *P,
                                           int ip, int lane, int &ovf,
                                           dmp::ExactScratch *W) {
  const int nc = S.nc;
  float pk1 = -1.f;
  int pg1 = -1;
  for (int t1 = 0; t1 < 3; ++t1) {
    // next nearest after (pk1, pg1)
    float bk = FLT_MAX;
    int bj = -1, bg = 0x7fffffff;
    for (int s = 0; s < L1<3>::PER; ++s) {
      int j = lane + 32 * s;
      if (j >= nc) continue;
      float k = S.c[j].w;
      int g = S.id[j];
      bool after = k > pk1 || (k == pk1 && g > pg1);
      if (after && (bj < 0 || k < bk || (k == bk && g < bg))) {
        bk = k;
        bj = j;
        bg = g;
      }
    }
    warp_argmin(bk, bj, bg);
    if (bj < 0) return 0xffffffffu;
    int q1 = bj;
    pk1 = bk;
    pg1 = bg;
    float4 Q = S.c[q1];
    float pk2 = -1.f;
    int pg2 = -1;
    for (int t2 = 0; t2 < 6; ++t2) {
      float ck = FLT_MAX;
      int cj = -1, cg = 0x7fffffff;
      for (int s = 0; s < L1<3>::PER; ++s) {
        int j = lane + 32 * s;
        if (j >= nc || j == q1) continue;
        float4 Y = S.c[j];
        float cx = Q.y * Y.z - Q.z * Y.y, cy = Q.z * Y.x - Q.x * Y.z,
              cz = Q.x * Y.y - Q.y * Y.x;
        float cr = cx * cx + cy * cy + cz * cz;
        if (!(cr > 0.f)) continue;
        float dx = Q.x - Y.x, dy = Q.y - Y.y, dz = Q.z - Y.z;
        float k = Q.w * Y.w * (dx * dx + dy * dy + dz * dz) / cr;
        int g = S.id[j];
        bool after = k > pk2 || (k == pk2 && g > pg2);
        if (after && (cj < 0 || k < ck || (k == ck && g < cg))) {
          ck = k;
          cj = j;
          cg = g;
        }
      }
      warp_argmin(ck, cj, cg);
      if (cj < 0) break;
      pk2 = ck;
      pg2 = cg;
      int q2 = cj;
      // the cell on one side of face (p, q1, q2) is accepted once no
      // candidate lies inside its circumsphere (this also rejects faces with
      // a coplanar point inside their circumcircle)
      uint32_t cand;
      int xp = gw3L(S, P, ip, q1, q2, lane, ovf, W);
      if (xp >= 0) {
        cand = pack3(q1, q2, xp);
      } else {
        int xm = gw3L(S, P, ip, q2, q1, lane, ovf, W);
        if (xm < 0) continue;
        cand = pack3(q2, q1, xm);
      }
      if (empty3L(S, P, ip, cand, lane, ovf, W)) return cand;
    }
  }
  return 0xffffffffu;
}

// seed search (2D): link edge (a, b) of a positive triangle (p, a, b)

__device__ __forceinline__ int o2L(const WarpL1<2> &S, const float *P, int ip,
                                   int a, int b, dmp::ExactScratch *W) {
  float4 A = S.c[a], B = S.c[b];
  int s = dmp::orient2_rel_filter<float>(A.x, A.y, B.x, B.y, 8.0f * DMP_U32);
  if (s) return s;
  const int4 IA = S.ci[a], IB = S.ci[b];
  if (IA.w & IB.w) return dmp::orient2_fx(IA, IB);
  float pr[2], ar[2], br[2];
  load_pt<2>(P, ip, pr);
  load_pt<2>(P, S.id[a], ar);
  load_pt<2>(P, S.id[b], br);
  return dmp::orient2_slow(pr, ar, br, W);
}

// incirc2(p, a, b, d)
__device__ __forceinline__ int ic2L(const WarpL1<2> &S, const float *P, int ip,
                                    int a, int b, int d, int &ovf,
                                    dmp::ExactScratch *W) {
  float4 A = S.c[a], B = S.c[b], D = S.c[d];
  float X[2] = {A.x, A.y}, Y[2] = {B.x, B.y}, Z[2] = {D.x, D.y};
  int s = dmp::incirc2_rel_filter<float>(X, Y, Z, A.w, B.w, D.w, 16.0f * DMP_U32);
  if (s) return s;
  const int4 IA = S.ci[a], IB = S.ci[b], ID = S.ci[d];
  if (IA.w & IB.w & ID.w) return dmp::incirc2_fx_sos(IA, IB, ID);
  float pr[2], ar[2], br[2], dr[2];
  load_pt<2>(P, ip, pr);
  load_pt<2>(P, S.id[a], ar);
  load_pt<2>(P, S.id[b], br);
  load_pt<2>(P, S.id[d], dr);
  return incirc2_sos(pr, ar, br, dr, &ovf, W);
}

// 2D gift-wrap across edge (p, x): sgn=+1 candidates with orient2(p,x,y)>0
// (triangle (p,x,y)); sgn=-1 candidates with orient2(p,y,x)>0 (triangle
// (p,y,x)).  Winner has the smallest circle through p and x on that side.
__device__ __forceinline__ int gw2L(const WarpL1<2> &S, const float *P, int ip,
                                    int x, int sgn, int lane, int &ovf,
                                    dmp::ExactScratch *W) {
  const int nc = S.nc;
  float4 X = S.c[x];
  float nx = -X.y * sgn, ny = X.x * sgn;
  uint32_t pos = 0;
  float bk = FLT_MAX;
  int bj = -1, bg = 0x7fffffff;
#pragma unroll
  for (int s = 0; s < L1<2>::PER; ++s) {
    int j = lane + 32 * s;
    if (j < nc && j != x) {
      int o = sgn > 0 ? o2L(S, P, ip, x, j, W) : o2L(S, P, ip, j, x, W);
      if (o > 0) {
        pos |= 1u << s;
        float4 Y = S.c[j];
        float den = Y.x * nx + Y.y * ny;
        float tau = (Y.w - (Y.x * X.x + Y.y * X.y)) / den;
        if (!(tau == tau) || !(den > 0.f)) tau = FLT_MAX;
        int g = S.id[j];
        if (bj < 0 || tau < bk || (tau == bk && g < bg)) {
          bk = tau;
          bj = j;
          bg = g;
        }
      }
    }
  }
  warp_argmin(bk, bj, bg);
  if (bj < 0) return -1;
  for (int it = 0; it < nc + 1; ++it) {
    int found = -1;
#pragma unroll
    for (int s = 0; s < L1<2>::PER; ++s) {
      int j = lane + 32 * s;
      if (found < 0 && (pos >> s & 1u) && j != bj) {
        int r = sgn > 0 ? ic2L(S, P, ip, x, bj, j, ovf, W) : ic2L(S, P, ip, bj, x, j, ovf, W);
        if (r < 0) found = j;
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, found >= 0);
    if (!m) return bj;
    bj = __shfl_sync(0xffffffffu, found, __ffs(m) - 1);
  }
  return bj;
}

__device__ __forceinline__ bool certified2(float4 A, float4 B, float reff) {
  float det = A.x * B.y - A.y * B.x;
  float perm = fabsf(A.x * B.y) + fabsf(A.y * B.x);
  if (!(fabsf(det) > 1e4f * 8.0f * DMP_U32 * perm)) return false;
  float nx = B.y * A.w - A.y * B.w, ny = A.x * B.w - B.x * A.w;
  float lim = 0.99f * reff;
  return nx * nx + ny * ny <= lim * lim * det * det;
}

// 2D seed: returns packed (q1, x) with triangle (p, q1, x) positive, or ~0
__device__ __forceinline__ uint32_t seed2L(const WarpL1<2> &S, const float *P,
                                           int ip, int lane, int &ovf,
                                           dmp::ExactScratch *W) {
  const int nc = S.nc;
  float pk = -1.f;
  int pg = -1;
  for (int t = 0; t < 6; ++t) {
    float bk = FLT_MAX;
    int bj = -1, bg = 0x7fffffff;
    for (int s = 0; s < L1<2>::PER; ++s) {
      int j = lane + 32 * s;
      if (j >= nc) continue;
      float k = S.c[j].w;
      int g = S.id[j];
      bool after = k > pk || (k == pk && g > pg);
      if (after && (bj < 0 || k < bk || (k == bk && g < bg))) {
        bk = k;
        bj = j;
        bg = g;
      }
    }
    warp_argmin(bk, bj, bg);
    if (bj < 0) return 0xffffffffu;
    pk = bk;
    pg = bg;
    int q1 = bj;
    uint32_t cand;
    int xp = gw2L(S, P, ip, q1, +1, lane, ovf, W);
    if (xp >= 0) {
      cand = pack3(q1, xp, 0);
    } else {
      int xm = gw2L(S, P, ip, q1, -1, lane, ovf, W);
      if (xm < 0) continue;
      cand = pack3(xm, q1, 0);
    }
    // accept once no candidate lies inside the triangle's circumcircle
    int a = un0(cand), b = un1(cand);
    bool inside = false;
    for (int j = lane; j < nc; j += 32)
      if (!inside && j != a && j != b) inside = ic2L(S, P, ip, a, b, j, ovf, W) < 0;
    if (!__any_sync(0xffffffffu, inside)) return cand;
  }
  return 0xffffffffu;
}

// Level-1 outcome counts of the 3D kernel, compiled in only with
// -DDM_L2_STATS: {no seed, open star, capacity, certification failed, stars,
// candidates, stars with a capped candidate radius, link triangles}
#ifdef DM_L2_STATS
static __device__ unsigned long long g_l1s[16];
#define L1S_ADD(i, v) atomicAdd(&g_l1s[i], (unsigned long long)(v))
#define L1S_CLOCK() clock64()
#else
#define L1S_ADD(i, v) ((void)0)
#define L1S_CLOCK() 0ll
#endif

// escalation record: (p, a, b, c) global ids; c < 0 means "no seed";
// bit 30 of p marks a certified seed cell.
__device__ __forceinline__ void escalate(const DTArgs &A, int p, int4 seed,
                                         int lane) {
  int64_t k = warp_append(&A.counters[DM_CNT_ESCALATED], lane == 0);
  if (lane == 0) {
    A.esc[k] = p;
    A.esc_seed[k] = seed;
  }
}

__global__ void __launch_bounds__(32 * L1_WARPS, DM_L1_MINB) k_star3_l1(DTArgs A) {
  __shared__ WarpL1<3> sm[L1_WARPS];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpL1<3> &S = sm[w];
  const GridParams g = *A.gp;
  for (int64_t pv = (int64_t)blockIdx.x * L1_WARPS + w; pv < A.n;
       pv += (int64_t)gridDim.x * L1_WARPS) {
    const int ip = (int)pv;
    if (A.dup[ip]) continue;
    float px[3];
    load_pt<3>(A.P, ip, px);
    [[maybe_unused]] long long t0 = L1S_CLOCK();
    gather_l1<3>(S, A, g, ip, px, lane, L1<3>::K);
    [[maybe_unused]] long long t1 = L1S_CLOCK();
    int ovf = 0;
    uint32_t seed = S.nc >= 3 ? seed3L(S, A.P, ip, lane, ovf, W) : 0xffffffffu;
    [[maybe_unused]] long long t2 = L1S_CLOCK();
    if (lane == 0) {
      L1S_ADD(8, t1 - t0);
      L1S_ADD(9, t2 - t1);
      L1S_ADD(4, 1);
      L1S_ADD(5, S.nc);
      L1S_ADD(6, S.capped);
    }
    if (seed == 0xffffffffu) {
      if (lane == 0) {
        L1S_ADD(0, 1);
        A.hullc[ip] = 1;
      }
      escalate(A, ip, make_int4(ip, -1, -1, -1), lane);
      continue;
    }
    if (lane == 0) {
      S.ntri = 1;
      S.tri[0] = seed;
      int a = un0(seed), b = un1(seed), c = un2(seed);
      S.open[0] = pack3(a, b, c);
      S.open[1] = pack3(b, c, a);
      S.open[2] = pack3(c, a, b);
      S.nopen = 3;
      S.flags = 0;
    }
    __syncwarp();
    int hull = 0;
    while (S.nopen > 0) {
      uint32_t e = S.open[S.nopen - 1];
      __syncwarp();
      if (lane == 0) S.nopen--;
      __syncwarp();
      int u = un0(e), v = un1(e);
      int y = gw3L(S, A.P, ip, v, u, lane, ovf, W);
      if (y < 0) {
        hull = 1;
        continue;
      }
      if (S.ntri >= L1<3>::MAXTRI) {
        if (lane == 0) S.flags |= 1;
        __syncwarp();
        break;
      }
      if (lane == 0) S.tri[S.ntri++] = pack3(v, u, y);
      __syncwarp();
      // new directed edges (u, y | v) and (y, v | u)
      int es[2][3] = {{u, y, v}, {y, v, u}};
      for (int k = 0; k < 2; ++k) {
        int r = find_rev<3>(S, es[k][0], es[k][1], lane);
        if (lane == 0) {
          if (r >= 0) {
            S.open[r] = S.open[S.nopen - 1];
            S.nopen--;
          } else if (S.nopen < L1<3>::MAXOPEN) {
            S.open[S.nopen++] = pack3(es[k][0], es[k][1], es[k][2]);
          } else {
            S.flags |= 1;
          }
        }
        __syncwarp();
      }
      if (S.flags) break;
    }
#ifdef DM_DEBUG_VERTEX
    if (ip == A.dbg_vertex && A.dbg) {
      // [nc, ntri, hull, flags, reff bits, ids[nc]..., tri[ntri] (3 ids each)]
      if (lane == 0) {
        A.dbg[0] = S.nc;
        A.dbg[1] = S.ntri;
        A.dbg[2] = hull;
        A.dbg[3] = S.flags;
        A.dbg[4] = __float_as_int(S.reff);
      }
      for (int k = lane; k < S.nc; k += 32) A.dbg[8 + k] = S.id[k];
      for (int t = lane; t < S.ntri; t += 32) {
        uint32_t tr = S.tri[t];
        A.dbg[8 + 128 + 3 * t] = S.id[un0(tr)];
        A.dbg[8 + 128 + 3 * t + 1] = S.id[un1(tr)];
        A.dbg[8 + 128 + 3 * t + 2] = S.id[un2(tr)];
      }
      __syncwarp();
    }
#endif
    [[maybe_unused]] long long t3 = L1S_CLOCK();
    if (lane == 0) L1S_ADD(10, t3 - t2);
    // certification
    bool allok = !hull && !S.flags;
    int cert_any = -1;
    for (int t = lane; t < S.ntri; t += 32) {
      uint32_t tr = S.tri[t];
      bool ok = certified3(S.c[un0(tr)], S.c[un1(tr)], S.c[un2(tr)], S.reff);
      if (!ok) allok = false;
      else if (cert_any < 0) cert_any = t;
    }
    allok = __all_sync(0xffffffffu, allok);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
    if (lane == 0) {
      L1S_ADD(7, S.ntri);
      if (!allok) L1S_ADD(hull ? 1 : (S.flags ? 2 : 3), 1);
      if (hull || S.flags) A.hullc[ip] = 1;
    }
    if (!allok) {
      unsigned m = S.flags ? 0u : __ballot_sync(0xffffffffu, cert_any >= 0);
      int4 sd;
      if (m) {
        int t = __shfl_sync(0xffffffffu, cert_any, __ffs(m) - 1);
        uint32_t tr = S.tri[t];
        sd = make_int4(ip | (1 << 30), S.id[un0(tr)], S.id[un1(tr)], S.id[un2(tr)]);
      } else {
        uint32_t tr = S.tri[0];
        sd = make_int4(ip, S.id[un0(tr)], S.id[un1(tr)], S.id[un2(tr)]);
      }
      escalate(A, ip, sd, lane);
      continue;
    }
    if (lane == 0) L1S_ADD(11, L1S_CLOCK() - t3);
    // emit cells owned by p (p has the smallest index)
    for (int t0 = 0; t0 < S.ntri; t0 += 32) {
      int t = t0 + lane;
      bool own = false;
      int ga = 0, gb = 0, gc = 0;
      if (t < S.ntri) {
        uint32_t tr = S.tri[t];
        ga = S.id[un0(tr)];
        gb = S.id[un1(tr)];
        gc = S.id[un2(tr)];
        own = ip < ga && ip < gb && ip < gc;
      }
      int64_t k = warp_append(&A.counters[DM_CNT_CELLS], own);
      if (own) {
        if (k < A.cap_cells_out) {
          int4 *out = reinterpret_cast<int4 *>(A.cells);
          out[k] = make_int4(ip, ga, gb, gc);
        } else {
          flag_or(A.counters, DM_FLAG_CELL_OVERFLOW);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(32 * L1_WARPS) k_star2_l1(DTArgs A) {
  __shared__ WarpL1<2> sm[L1_WARPS];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  WarpL1<2> &S = sm[w];
  const GridParams g = *A.gp;
  for (int64_t pv = (int64_t)blockIdx.x * L1_WARPS + w; pv < A.n;
       pv += (int64_t)gridDim.x * L1_WARPS) {
    const int ip = (int)pv;
    if (A.dup[ip]) continue;
    float px[2];
    load_pt<2>(A.P, ip, px);
    gather_l1<2>(S, A, g, ip, px, lane, L1<2>::K);
    int ovf = 0;
    uint32_t seed = S.nc >= 2 ? seed2L(S, A.P, ip, lane, ovf, W) : 0xffffffffu;
    if (seed == 0xffffffffu) {
      escalate(A, ip, make_int4(ip, -1, -1, -1), lane);
      continue;
    }
    // forward walk: v0 = a, v1 = b, v_{i+1} = gw(v_i, +1) until closed
    int a = un0(seed), b = un1(seed);
    if (lane == 0) {
      S.ntri = 1;
      S.tri[0] = pack3(a, b, 0);
      S.flags = 0;
    }
    __syncwarp();
    bool hull = false;
    int cur = b;
    while (true) {
      int nx = gw2L(S, A.P, ip, cur, +1, lane, ovf, W);
      if (nx < 0) {
        hull = true;
        break;
      }
      if (S.ntri >= L1<2>::MAXTRI) {
        if (lane == 0) S.flags |= 1;
        __syncwarp();
        break;
      }
      if (nx == a) {
        // closing triangle (p, cur, a)
        if (lane == 0) S.tri[S.ntri++] = pack3(cur, nx, 0);
        __syncwarp();
        break;
      }
      if (S.ntri >= L1<2>::MAXTRI) {
        if (lane == 0) S.flags |= 1;
        __syncwarp();
        break;
      }
      if (lane == 0) S.tri[S.ntri++] = pack3(cur, nx, 0);
      __syncwarp();
      cur = nx;
    }
    if (hull && !S.flags) {
      cur = a;
      while (true) {
        int pv2 = gw2L(S, A.P, ip, cur, -1, lane, ovf, W);
        if (pv2 < 0) break;
        if (S.ntri >= L1<2>::MAXTRI) {
          if (lane == 0) S.flags |= 1;
          __syncwarp();
          break;
        }
        if (lane == 0) S.tri[S.ntri++] = pack3(pv2, cur, 0);
        __syncwarp();
        cur = pv2;
      }
    }
    bool allok = !hull && !S.flags;
    int cert_any = -1;
    for (int t = lane; t < S.ntri; t += 32) {
      uint32_t tr = S.tri[t];
      bool ok = certified2(S.c[un0(tr)], S.c[un1(tr)], S.reff);
      if (!ok) allok = false;
      else if (cert_any < 0) cert_any = t;
    }
    allok = __all_sync(0xffffffffu, allok);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
    if (!allok) {
      unsigned m = S.flags ? 0u : __ballot_sync(0xffffffffu, cert_any >= 0);
      int4 sd;
      int t = m ? __shfl_sync(0xffffffffu, cert_any, __ffs(m) - 1) : 0;
      uint32_t tr = S.tri[t];
      sd = make_int4(ip | (m ? (1 << 30) : 0), S.id[un0(tr)], S.id[un1(tr)], 0);
      escalate(A, ip, sd, lane);
      continue;
    }
    for (int t0 = 0; t0 < S.ntri; t0 += 32) {
      int t = t0 + lane;
      bool own = false;
      int ga = 0, gb = 0;
      if (t < S.ntri) {
        uint32_t tr = S.tri[t];
        ga = S.id[un0(tr)];
        gb = S.id[un1(tr)];
        own = ip < ga && ip < gb;
      }
      int64_t k = warp_append(&A.counters[DM_CNT_CELLS], own);
      if (own) {
        if (k < A.cap_cells_out) {
          A.cells[3 * k] = ip;
          A.cells[3 * k + 1] = ga;
          A.cells[3 * k + 2] = gb;
        } else {
          flag_or(A.counters, DM_FLAG_CELL_OVERFLOW);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Level 2: exhaustive queries over the grid
constexpr int L2_WARPS = 4;
constexpr int L2_MAXTRI = 192, L2_MAXOPEN = 128;

struct WarpL2 {
  int3 tri[L2_MAXTRI];
  int3 open[L2_MAXOPEN];
  int ntri, nopen, flags;
};

struct GQ {
  const DTArgs *A;
  GridParams g;
};

// Level-2 per-star statistics, compiled in only with -DDM_L2_STATS:
// g_l2s[star] = {cycles, ntri | ip << 32, hull scans, region cells, points
// considered, kind-1 regions, kind-2 regions, widened local searches}
#ifdef DM_L2_STATS
constexpr int kL2StatStars = 1 << 17, kL2StatWarps = 152 * 8 * 4;
static __device__ unsigned long long g_l2s[kL2StatStars][8];
static __device__ unsigned long long g_l2w[kL2StatWarps][8];
__device__ __forceinline__ void l2s_add(int i, unsigned long long v) {
  int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w < kL2StatWarps) atomicAdd(&g_l2w[w][i], v);
}
#define L2S_ADD(i, v) l2s_add(i, v)
#else
#define L2S_ADD(i, v) ((void)0)
#endif

template <int DIM>
__device__ __forceinline__ void ldp(const DTArgs &A, int i, float *x) {
  load_pt<DIM>(A.P, i, x);
}

// 3D: compare candidate j against current best on face (p,a,b)
struct Face3 {
  int ip, ia, ib;
  int gfix;  // GridParams::gfix (the exact stages rebuild their frame from it)
  float p[3], a[3], b[3];
  float V[3], U[3];
};

__device__ __forceinline__ void face3_frame(Face3 &F, int gfix) { F.gfix = gfix; }

// Exact stages of the face predicates.  They run only when the FP32 filter
// cannot decide, so they are compiled once, out of line, and take scalars
// (the face stays in registers at every inlined filter).  The fixed-point
// frame is the one at p covering 8x the face size (its largest coordinate
// difference), in which a and b and the query points are exact or flagged.
struct FaceFx {
  FxFrame fr;
  int4 IA, IB;
};

__device__ __forceinline__ void face_fx(FaceFx &X, const float *p, const float *a,
                                        const float *b, int gfix) {
  float e = 0.f;
  for (int k = 0; k < 3; ++k) e = fmaxf(e, fmaxf(fabsf(a[k] - p[k]), fabsf(b[k] - p[k])));
  fx_frame<3>(X.fr, p, 8.f * e, gfix);
  X.IA = fx_point<3>(X.fr, a);
  X.IB = fx_point<3>(X.fr, b);
}

static __device__ __noinline__ int side3_exact(float p0, float p1, float p2, float a0, float a1,
                                               float a2, float b0, float b1, float b2, float y0,
                                               float y1, float y2, int gfix,
                                               dmp::ExactScratch *W) {
  const float p[3] = {p0, p1, p2}, a[3] = {a0, a1, a2}, b[3] = {b0, b1, b2}, y[3] = {y0, y1, y2};
  FaceFx X;
  face_fx(X, p, a, b, gfix);
  const int4 IY = fx_point<3>(X.fr, y);
  if (X.IA.w & X.IB.w & IY.w) return dmp::orient3_fx(X.IA, X.IB, IY);
  return dmp::orient3_slow(p, a, b, y, W);
}

// perturbed insph3(p, a, b, c, d): the sign in bits 0-1 (sign + 1), bit 2
// set when an expansion overflowed
static __device__ __noinline__ int insph_face3_exact(float p0, float p1, float p2, float a0,
                                                     float a1, float a2, float b0, float b1,
                                                     float b2, float c0, float c1, float c2,
                                                     float d0, float d1, float d2, int gfix,
                                                     dmp::ExactScratch *W) {
  const float p[3] = {p0, p1, p2}, a[3] = {a0, a1, a2}, b[3] = {b0, b1, b2};
  const float c[3] = {c0, c1, c2}, d[3] = {d0, d1, d2};
  FaceFx X;
  face_fx(X, p, a, b, gfix);
  const int4 IC = fx_point<3>(X.fr, c), ID = fx_point<3>(X.fr, d);
  if (X.IA.w & X.IB.w & IC.w & ID.w) return dmp::insph3_fx_sos(X.IA, X.IB, IC, ID) + 1;
  int ovf = 0;
  int s = dmp::insph3_slow(p, a, b, c, d, &ovf, W);
  if (!s) s = dmp::insph3_sos_tail(p, a, b, c, d, W);
  return (s + 1) | (ovf ? 4 : 0);
}

__device__ __forceinline__ int side3(const Face3 &F, const float *y,
                                     dmp::ExactScratch *W) {
  float Y[3] = {y[0] - F.p[0], y[1] - F.p[1], y[2] - F.p[2]};
  int s = dmp::orient3_rel_filter<float>(F.V[0], F.V[1], F.V[2], F.U[0], F.U[1],
                                         F.U[2], Y[0], Y[1], Y[2], 16.0f * DMP_U32);
  if (s) return s;
  return side3_exact(F.p[0], F.p[1], F.p[2], F.a[0], F.a[1], F.a[2], F.b[0], F.b[1], F.b[2], y[0],
                     y[1], y[2], F.gfix, W);
}

// perturbed insph3(p, a, b, c, d) of a face query
__device__ __forceinline__ int insph_face3(const Face3 &F, const float *c, const float *d,
                                           int &ovf, dmp::ExactScratch *W) {
  float Z[3] = {c[0] - F.p[0], c[1] - F.p[1], c[2] - F.p[2]};
  float Q[3] = {d[0] - F.p[0], d[1] - F.p[1], d[2] - F.p[2]};
  float wx = F.V[0] * F.V[0] + F.V[1] * F.V[1] + F.V[2] * F.V[2];
  float wy = F.U[0] * F.U[0] + F.U[1] * F.U[1] + F.U[2] * F.U[2];
  float wz = Z[0] * Z[0] + Z[1] * Z[1] + Z[2] * Z[2];
  float wq = Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2];
  int s = dmp::insph3_rel_filter<float>(F.V, F.U, Z, Q, wx, wy, wz, wq, 48.0f * DMP_U32);
  if (s) return s;
  const int r = insph_face3_exact(F.p[0], F.p[1], F.p[2], F.a[0], F.a[1], F.a[2], F.b[0], F.b[1],
                                  F.b[2], c[0], c[1], c[2], d[0], d[1], d[2], F.gfix, W);
  if (r & 4) ovf = 1;
  return (r & 3) - 1;
}

#ifdef DM_C3_NOINLINE
static __device__ __noinline__ void consider3(const DTArgs &A, const Face3 &F, int j,
#else
__device__ __forceinline__ void consider3(const DTArgs &A, const Face3 &F, int j,
#endif
                                          float4 q, int &best, float *bx, int &ovf,
                                          dmp::ExactScratch *W) {
  if (j == F.ip || j == F.ia || j == F.ib) return;
  L2S_ADD(3, 1);
  float y[3] = {q.x, q.y, q.z};
  if (side3(F, y, W) <= 0) return;
  if (best < 0 || insph_face3(F, bx, y, ovf, W) < 0) {
    best = j;
    bx[0] = y[0];
    bx[1] = y[1];
    bx[2] = y[2];
  }
}

// Warp tournament: every lane ends with the winner of the lanes' bests and
// its coordinates (bx holds each lane's best point).  Not unrolled: one
// copy of the face predicate per call site.
__device__ __forceinline__ int tourney3(const DTArgs &A, const Face3 &F,
                                        int best, float *bx, int &ovf,
                                        dmp::ExactScratch *W) {
#pragma unroll 1
  for (int o = 16; o; o >>= 1) {
    const int other = __shfl_xor_sync(0xffffffffu, best, o);
    float ox[3];
    for (int k = 0; k < 3; ++k) ox[k] = __shfl_xor_sync(0xffffffffu, bx[k], o);
    if (other >= 0 && other != best && (best < 0 || insph_face3(F, bx, ox, ovf, W) < 0)) {
      best = other;
      for (int k = 0; k < 3; ++k) bx[k] = ox[k];
    }
  }
  return best;
}

__device__ __forceinline__ bool in_local(const int *cc, int x, int y, int z,
                                         int dim) {
  return abs(x - cc[0]) <= 1 && abs(y - cc[1]) <= 1 && (dim == 2 || abs(z - cc[2]) <= 1);
}

// cells [lo, hi] on axis k covering [c - r, c + r], padded by one cell and
// clipped to the grid (computed in double: r may be huge); lo > hi when the
// interval misses the grid
__device__ __forceinline__ void cell_range(const GridParams &g, double c, double r,
                                           int k, int &lo, int &hi) {
  double a = floor((c - r - g.lo[k]) * g.inv_cs) - 1;
  double b = floor((c + r - g.lo[k]) * g.inv_cs) + 1;
  lo = (int)fmax(0.0, fmin(a, (double)g.dims[k]));
  hi = (int)fmin((double)(g.dims[k] - 1), fmax(b, -1.0));
}

// the points of cell c
template <typename F>
__device__ __forceinline__ void for_cell(const DTArgs &A, int c, F f) {
  const int e = A.cell_start[c + 1];
  for (int i = A.cell_start[c]; i < e; ++i) {
    const float4 q = A.spts[i];
    const int j = __float_as_int(q.w);
    if (j >= 0) f(j, q);  // duplicates are skipped
  }
}

// Search region of a gift-wrap query on face (p, a, b) with current winner y:
// every point that beats y lies in sphere(p, a, b, y) on the positive side
// H+ of the face.  Kinds:
//  1: the face circumcircle (cc, r) is well conditioned.  With z(x) the
//     height over the face, the region is {x in H+ : |x-cc|^2 - r^2 <= 2 Z z(x)}
//     for any Z >= z0 (the sphere centre's height).  Z < 0 gives a thin lens.
//  2: ill-conditioned face, well-conditioned tetrahedron: the circumsphere
//     (s, R) of (p, a, b, y) intersected with H+.
//  0: neither: all of H+ (culling only by the face plane when its normal is
//     resolvable).
struct Region3 {
  int kind;
  bool cull;          // the unit normal un is accurate (plane culling allowed)
  double p[3], un[3];
  double cc[3], r2, Z, dcc;  // kind 1 (cc absolute), dcc: error bound of cc
  double s[3], R2;           // kind 2
  double lo[3], hi[3];       // bounding box of the region (kinds 1, 2)
  // FP32 copies for the per-box tests (FP64 stays out of the scan loops)
  float fp[3], fun[3], fc[3], fr2, fZ, fR2, fdcc;
};

// double-precision region from the exact face/winner differences
__device__ __forceinline__ void make_region3(Region3 &R, const float *fp, const double *a,
                                             const double *b, const double *n, double nn,
                                             double la, double lb, const float *y) {
  const double u = 1.2e-16;
  for (int k = 0; k < 3; ++k) R.p[k] = fp[k];
  R.cull = nn > 1e-20 * la * lb;
  const double inl = R.cull ? 1.0 / sqrt(nn) : 0.0;
  for (int k = 0; k < 3; ++k) R.un[k] = n[k] * inl;
  R.kind = 0;
  if (!y) return;
  double c[3];
  for (int k = 0; k < 3; ++k) c[k] = (double)y[k] - fp[k];
  if (nn > 1e-12 * la * lb) {
    // |dn| <= 4u|a||b|; |dcc| <= 16u (la|b| + lb|a|)|a||b| / nn + 1e-9 r
    double al = sqrt(la), bl = sqrt(lb), nl = sqrt(nn);
    double t[3] = {la * b[0] - lb * a[0], la * b[1] - lb * a[1], la * b[2] - lb * a[2]};
    double inv = 0.5 / nn;
    double cc[3] = {(t[1] * n[2] - t[2] * n[1]) * inv, (t[2] * n[0] - t[0] * n[2]) * inv,
                    (t[0] * n[1] - t[1] * n[0]) * inv};
    double r2 = cc[0] * cc[0] + cc[1] * cc[1] + cc[2] * cc[2];
    double r = sqrt(r2);
    double dcc = 16 * u * (la * bl + lb * al) * al * bl / nn + 4 * u * r;
    double w[3] = {c[0] - cc[0], c[1] - cc[1], c[2] - cc[2]};
    double lw = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    double q = lw - r2;
    double eq = 4 * (sqrt(lw) + r + dcc) * dcc + 1e-14 * (lw + r2);
    double lc = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    double hgt = (c[0] * n[0] + c[1] * n[1] + c[2] * n[2]) / nl;  // > 0 exactly
    double dh = 2 * lc * u * (4 * al * bl / nl + 3);
    double Z;
    bool ok = true;
    if (q + eq <= 0) {
      Z = (q + eq) / (2 * (hgt + dh));  // <= 0: an upper bound of z0
    } else if (hgt > 2 * dh) {
      Z = (q + eq) / (2 * (hgt - dh));
    } else {
      ok = false;
    }
    if (ok && Z < 1e30) {
      R.kind = 1;
      for (int k = 0; k < 3; ++k) R.cc[k] = cc[k] + fp[k];
      R.r2 = r2;
      R.Z = Z;
      R.dcc = dcc + 1e-7 * (fabs(R.cc[0]) + fabs(R.cc[1]) + fabs(R.cc[2]));
      // the region lies in B(cc, r) when Z <= 0, else in the sphere itself
      double ctr[3], rb;
      if (Z <= 0) {
        for (int k = 0; k < 3; ++k) ctr[k] = R.cc[k];
        rb = r;
      } else {
        for (int k = 0; k < 3; ++k) ctr[k] = R.cc[k] + Z * n[k] / nl;
        rb = sqrt(r2 + Z * Z);
      }
      rb = rb * (1 + 1e-6) + R.dcc;
      for (int k = 0; k < 3; ++k) {
        R.lo[k] = ctr[k] - rb;
        R.hi[k] = ctr[k] + rb;
      }
      return;
    }
  }
  // circumsphere of the tetrahedron (p, a, b, y)
  double bc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2],
                  b[0] * c[1] - b[1] * c[0]};
  double ca[3] = {c[1] * a[2] - c[2] * a[1], c[2] * a[0] - c[0] * a[2],
                  c[0] * a[1] - c[1] * a[0]};
  double det = a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2];
  double perm = fabs(a[0]) * (fabs(b[1] * c[2]) + fabs(b[2] * c[1])) +
                fabs(a[1]) * (fabs(b[2] * c[0]) + fabs(b[0] * c[2])) +
                fabs(a[2]) * (fabs(b[0] * c[1]) + fabs(b[1] * c[0]));
  if (fabs(det) > 1e-9 * perm) {
    double lc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    double s[3];
    for (int k = 0; k < 3; ++k) s[k] = (la * bc[k] + lb * ca[k] + lc * n[k]) / (2 * det);
    double rad = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    for (int k = 0; k < 3; ++k) s[k] += fp[k];
    rad = rad * (1 + 1e-6) + 1e-7 * (fabs(s[0]) + fabs(s[1]) + fabs(s[2]));
    if (rad < 1e30) {
      R.kind = 2;
      R.R2 = rad * rad;
      for (int k = 0; k < 3; ++k) {
        R.s[k] = s[k];
        R.lo[k] = s[k] - rad;
        R.hi[k] = s[k] + rad;
      }
    }
  }
}

__device__ __forceinline__ void region3_floats(Region3 &R) {
  for (int k = 0; k < 3; ++k) {
    R.fp[k] = (float)R.p[k];
    R.fun[k] = (float)R.un[k];
    R.fc[k] = (float)(R.kind == 2 ? R.s[k] : R.cc[k]);
  }
  R.fr2 = (float)R.r2;
  R.fZ = (float)fmax(fmin(R.Z, 1e30), -1e30);
  R.fR2 = (float)fmin(R.R2, 1e36);
  R.fdcc = (float)R.dcc;
}

// May the box [lo, hi] hold a point of the region?  Conservative FP32 test:
// every rounding error (a few ulps per term, relative 6e-8) is covered by
// margins of relative 1e-5 and by the error bound of the region itself.
__device__ __forceinline__ bool region_hits3(const Region3 &R, const float *lo,
                                             const float *hi) {
  // heights of the box corners over the face plane, distance bound to p
  float zmin = FLT_MAX, zmax = -FLT_MAX, dp2 = 0.f;
  for (int corner = 0; corner < 8; ++corner) {
    float z = 0.f, d2 = 0.f;
    for (int k = 0; k < 3; ++k) {
      float v = ((corner >> k) & 1 ? hi[k] : lo[k]) - R.fp[k];
      z = fmaf(v, R.fun[k], z);
      d2 = fmaf(v, v, d2);
    }
    zmin = fminf(zmin, z);
    zmax = fmaxf(zmax, z);
    dp2 = fmaxf(dp2, d2);
  }
  const float dp = sqrtf(dp2);
  const float tz = 1e-5f * dp;  // height error (normal direction and rounding)
  if (R.cull && zmax < -tz) return false;  // entirely below the face
  if (R.kind == 0) return true;
  float d2 = 0.f;
  for (int k = 0; k < 3; ++k) {
    float e = fmaxf(fmaxf(lo[k] - R.fc[k], R.fc[k] - hi[k]), 0.f);
    d2 = fmaf(e, e, d2);
  }
  if (R.kind == 2) return d2 <= R.fR2 * (1.f + 1e-5f) + 1e-30f;
  // kind 1: lower bound of |x-cc|^2 - 2 Z z(x) - r^2 over the box within H+
  float zb = R.fZ > 0.f ? zmax + tz : fmaxf(zmin - tz, 0.f);
  float t = 2.f * R.fZ * zb;
  float gl = d2 - t - R.fr2;
  float tol = 2.f * dp * R.fdcc + 1e-5f * (d2 + R.fr2 + fabsf(t)) + 1e-30f;
  return gl <= tol;
}

// Chebyshev distance of cell (x, y, z) from cell cc
__device__ __forceinline__ int cheb3(const int *cc, int x, int y, int z) {
  return max(abs(x - cc[0]), max(abs(y - cc[1]), abs(z - cc[2])));
}

// Every point of each lane's range [off, off + len) of pts, visited by the
// whole warp: an inclusive prefix sum flattens the 32 ranges and each lane
// takes one point at a time (a binary search over the prefix finds its
// range).  A warp whose hits are few and uneven keeps all lanes busy, and
// the point loads are independent.
template <typename F>
__device__ __forceinline__ void warp_ranges(const float4 *pts, int off, int len, int lane, F f) {
  int incl = len;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  const int base = off - (incl - len);  // point t of the flat list is pts[base_r + t]
  for (int t0 = 0; t0 < total; t0 += 32) {
    const int t = t0 + lane;
    int r = 0;  // first range whose inclusive sum exceeds t
    for (int s = 16; s; s >>= 1)
      if (__shfl_sync(0xffffffffu, incl, r + s - 1) <= t) r += s;
    const int b = __shfl_sync(0xffffffffu, base, r);
    if (t < total) f(pts[b + t]);
  }
}

// Box of the cell row x0 <= x < x1 at (y, z), padded for the rounding of the
// cell assignment (floor((x - lo) / cs) in FP32 may place a point a few
// ulps of the grid extent outside its cell's nominal box).
__device__ __forceinline__ void row_box3(const GridParams &g, int x0, int x1, int y, int z,
                                         float *lo, float *hi) {
  const int c0[3] = {x0, y, z}, c1[3] = {x1, y + 1, z + 1};
  for (int k = 0; k < 3; ++k) {
    const float pad = (fabsf(g.lo[k]) + (float)g.dims[k] * g.cs) * 1e-6f;
    lo[k] = g.lo[k] + (float)c0[k] * g.cs - pad;
    hi[k] = g.lo[k] + (float)c1[k] * g.cs + pad;
  }
}

// The points of coarse blocks b0 and b1 (b1 < 0: none) that may lie in the
// region, visited by the whole warp: lane l holds cell row l % 16 (the 4
// cells along x at one (y, z)) of block l < 16 ? b0 : b1.  A row whose box
// misses the region, or whose cells all lie within Chebyshev distance rex of
// cell cc (already scanned), is dropped; a point in such a cell is skipped.
constexpr int kBs3 = 4;  // coarse block edge in 3D (GridParams::bs)
template <typename F>
__device__ __forceinline__ void scan_block_pair3(const DTArgs &A, const GridParams &g,
                                                 const Region3 &R, int b0, int b1,
                                                 const int *cc, int rex, int lane, F f) {
  const int b = lane < 16 ? b0 : b1, r = lane & 15;
  int off = 0, len = 0;
  if (b >= 0) {
    const int bxi = b % g.bdims[0], byi = (b / g.bdims[0]) % g.bdims[1],
              bzi = b / (g.bdims[0] * g.bdims[1]);
    const int y = byi * kBs3 + (r & 3), z = bzi * kBs3 + (r >> 2);
    const int x0 = bxi * kBs3, x1 = min(x0 + kBs3, g.dims[0]);
    const bool done = abs(y - cc[1]) <= rex && abs(z - cc[2]) <= rex && x0 >= cc[0] - rex &&
                      x1 - 1 <= cc[0] + rex;
    if (y < g.dims[1] && z < g.dims[2] && !done) {
      float lo[3], hi[3];
      row_box3(g, x0, x1, y, z, lo, hi);
      if (region_hits3(R, lo, hi)) {
        const int c0 = x0 + g.dims[0] * (y + g.dims[1] * z);
        off = A.cell_start[c0];
        len = A.cell_start[c0 + (x1 - x0)] - off;
      }
    }
  }
  warp_ranges(A.spts, off, len, lane, [&](float4 q) {
    const int j = __float_as_int(q.w);
    if (j < 0) return;  // duplicate
    if (cheb3(cc, cell_coord(g, q.x, 0), cell_coord(g, q.y, 1), cell_coord(g, q.z, 2)) <= rex)
      return;
    f(j, q);
  });
}

// Every point of the coarse blocks [blo, bhi] (block coordinates) whose
// tight box meets the region: lanes test 32 blocks at a time and the hits
// are scanned two by two by the whole warp.
template <typename F>
__device__ __forceinline__ void scan_blocks3(const DTArgs &A, const GridParams &g,
                                             const Region3 &R, const int *blo, const int *bhi,
                                             const int *cc, int rex, int lane, F f) {
  const int sx = bhi[0] - blo[0] + 1, sy = bhi[1] - blo[1] + 1, sz = bhi[2] - blo[2] + 1;
  if (sx <= 0 || sy <= 0 || sz <= 0) return;
  const int64_t nb = (int64_t)sx * sy * sz;
  int pending = -1;  // a hit block waiting for a partner (warp-uniform)
  for (int64_t t0 = 0; t0 < nb; t0 += 32) {
    const int64_t t = t0 + lane;
    int bid = -1;
    if (t < nb) {
      const int bxi = blo[0] + (int)(t % sx), byi = blo[1] + (int)((t / sx) % sy),
                bzi = blo[2] + (int)(t / ((int64_t)sx * sy));
      bid = bxi + g.bdims[0] * (byi + g.bdims[1] * bzi);
      if (A.blk_cnt[bid] == 0 || !region_hits3(R, A.blk_box + 6 * bid, A.blk_box + 6 * bid + 3))
        bid = -1;
    }
    unsigned m = __ballot_sync(0xffffffffu, bid >= 0);
    while (m) {
      const int h = __shfl_sync(0xffffffffu, bid, __ffs(m) - 1);
      m &= m - 1;
      if (pending < 0) {
        pending = h;
        continue;
      }
      scan_block_pair3(A, g, R, pending, h, cc, rex, lane, f);
      pending = -1;
    }
  }
  if (pending >= 0) scan_block_pair3(A, g, R, pending, -1, cc, rex, lane, f);
}

// exhaustive gift-wrap query on face (p, a, b), 3D
__device__ __forceinline__ int gq3(const DTArgs &A, const GridParams &g, int ip,
                                   int ia, int ib, int lane, int &ovf,
                                   dmp::ExactScratch *W) {
  Face3 F;
  F.ip = ip;
  F.ia = ia;
  F.ib = ib;
  load_pt<3>(A.P, ip, F.p);
  load_pt<3>(A.P, ia, F.a);
  load_pt<3>(A.P, ib, F.b);
  for (int k = 0; k < 3; ++k) {
    F.V[k] = F.a[k] - F.p[k];
    F.U[k] = F.b[k] - F.p[k];
  }
  face3_frame(F, g.gfix);
  // face normal from the exact differences
  double a[3], b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = (double)F.a[k] - F.p[k];
    b[k] = (double)F.b[k] - F.p[k];
  }
  const double n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                       a[0] * b[1] - a[1] * b[0]};
  const double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
  const double la = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  const double lb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
  int best = -1;
  float bx[3] = {0.f, 0.f, 0.f};
  int cc[3];
  for (int k = 0; k < 3; ++k)
    cc[k] = cell_coord(g, (F.p[k] + F.a[k] + F.b[k]) * (1.f / 3.f), k);
  auto scan_cell = [&](int x, int y, int z) {
    if (x >= 0 && y >= 0 && z >= 0 && x < g.dims[0] && y < g.dims[1] && z < g.dims[2])
      for_cell(A, x + g.dims[0] * (y + g.dims[1] * z),
               [&](int j, float4 q) { consider3(A, F, j, q, best, bx, ovf, W); });
  };
  // local search: the 27 cells around the face centroid
  if (lane < 27) scan_cell(cc[0] + lane % 3 - 1, cc[1] + (lane / 3) % 3 - 1, cc[2] + lane / 9 - 1);
  // after a tournament every lane holds the same winner: reload its point
  best = tourney3(A, F, best, bx, ovf, W);
  if (best >= 0) load_pt<3>(A.P, best, bx);
  // no point near the face: if no hull candidate lies in H+, no point does
  // (a hull face); a candidate that does bounds the region of the search
  bool h_empty = false;
  if (best < 0 && A.use_o && !A.dbg_full) {
    if (lane == 0) L2S_ADD(1, 1);
    Region3 H;
    make_region3(H, F.p, a, b, n, nn, la, lb, nullptr);
    region3_floats(H);
    const int ntab = *A.o_ntab;
    for (int e0 = 0; e0 < ntab; e0 += 32) {
      const int e = e0 + lane;
      int s0 = 0, cnt = 0;
      if (e < ntab) {
        const float4 t0 = A.o_tab[2 * e], t1 = A.o_tab[2 * e + 1];
        const float blo[3] = {t0.x, t0.y, t0.z}, bhi[3] = {t1.x, t1.y, t1.z};
        if (region_hits3(H, blo, bhi)) {
          s0 = __float_as_int(t0.w);
          cnt = __float_as_int(t1.w);
        }
      }
      warp_ranges(A.o_pts, s0, cnt, lane,
                  [&](float4 q) { consider3(A, F, __float_as_int(q.w), q, best, bx, ovf, W); });
    }
    best = tourney3(A, F, best, bx, ovf, W);
    if (best >= 0)
      load_pt<3>(A.P, best, bx);
    else
      h_empty = true;
  }
#ifdef DM_L2_STATS
  const long long tr_t0 = clock64();
  const int tr_local = best;
  int tr_wide = -2;
  const int tr_w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const unsigned long long tr_c0 = tr_w < kL2StatWarps ? g_l2w[tr_w][3] : 0;
#endif
  Region3 R;
  make_region3(R, F.p, a, b, n, nn, la, lb, best >= 0 ? bx : nullptr);
  region3_floats(R);
  int rex = 1;  // cells with Chebyshev distance <= rex are done
  // a large region: widen the local search to the 5^3 cells first
  bool large = R.kind == 0;
  for (int k = 0; k < 3 && !large; ++k)
    large = (R.hi[k] - R.lo[k]) * g.inv_cs > 5.0;
  large = large && !h_empty;
  if (large) {
    for (int t = lane; t < 125; t += 32) {
      int dx = t % 5 - 2, dy = (t / 5) % 5 - 2, dz = t / 25 - 2;
      if (max(abs(dx), max(abs(dy), abs(dz))) == 2) scan_cell(cc[0] + dx, cc[1] + dy, cc[2] + dz);
    }
    best = tourney3(A, F, best, bx, ovf, W);
    rex = 2;
    if (best >= 0) load_pt<3>(A.P, best, bx);
    make_region3(R, F.p, a, b, n, nn, la, lb, best >= 0 ? bx : nullptr);
    region3_floats(R);
#ifdef DM_L2_STATS
    tr_wide = best;
#endif
  }
  if (A.dbg_full) {
    R.kind = 0;
    rex = 1;
  }
  if (lane == 0) {
    if (R.kind == 1) L2S_ADD(4, 1);
    if (R.kind == 2) L2S_ADD(5, 1);
    if (large) L2S_ADD(6, 1);
  }
  if (h_empty) {
    // every point in H+ would have shown a hull candidate in H+
  } else if (R.kind != 0) {
    int lo[3], hi[3];
    int64_t ncell = 1;
    for (int k = 0; k < 3; ++k) {
      double c0 = 0.5 * (R.lo[k] + R.hi[k]), r0 = 0.5 * (R.hi[k] - R.lo[k]);
      cell_range(g, c0, r0, k, lo[k], hi[k]);
      ncell *= max(0, hi[k] - lo[k] + 1);
    }
    if (lane == 0) L2S_ADD(2, ncell);
    if (ncell <= 4096) {
      int sx = hi[0] - lo[0] + 1, sy = hi[1] - lo[1] + 1;
      for (int t = lane; t < ncell; t += 32) {
        int x = lo[0] + t % sx, y = lo[1] + (t / sx) % sy, z = lo[2] + t / (sx * sy);
        if (cheb3(cc, x, y, z) <= rex) continue;
        float blo[3], bhi[3];
        row_box3(g, x, x + 1, y, z, blo, bhi);
        if (!region_hits3(R, blo, bhi)) continue;
        for_cell(A, x + g.dims[0] * (y + g.dims[1] * z),
                 [&](int j, float4 q) { consider3(A, F, j, q, best, bx, ovf, W); });
      }
    } else {
      int blo[3], bhi[3];
      for (int k = 0; k < 3; ++k) {
        blo[k] = lo[k] / kBs3;
        bhi[k] = hi[k] / kBs3;
      }
      scan_blocks3(A, g, R, blo, bhi, cc, rex, lane,
                   [&](int j, float4 q) { consider3(A, F, j, q, best, bx, ovf, W); });
    }
  } else {
    // every block that may hold a point on the positive side
    if (lane == 0) L2S_ADD(1, 1);
    const int blo[3] = {0, 0, 0}, bhi[3] = {g.bdims[0] - 1, g.bdims[1] - 1, g.bdims[2] - 1};
    scan_blocks3(A, g, R, blo, bhi, cc, rex, lane,
                 [&](int j, float4 q) { consider3(A, F, j, q, best, bx, ovf, W); });
  }
  best = tourney3(A, F, best, bx, ovf, W);
#ifdef DM_L2_STATS
  // per-face trace of the watched vertex: dbg[1999] counts faces, record
  // i at dbg[2000 + 16 i]
  if (ip == A.dbg_vertex && A.dbg && lane == 0) {
    int i = atomicAdd(&A.dbg[1999], 1);
    if (i < 256) {
      int32_t *t = A.dbg + 2000 + 16 * i;
      int64_t ncell = 1;
      for (int k = 0; k < 3; ++k) ncell *= max(1, (int)((R.hi[k] - R.lo[k]) * g.inv_cs) + 1);
      t[0] = ia;
      t[1] = ib;
      t[2] = R.kind;
      t[3] = (int)min(ncell, (int64_t)INT32_MAX);
      t[4] = tr_local;
      t[5] = tr_wide;
      t[6] = best;
      t[7] = (int)min(clock64() - tr_t0, (long long)INT32_MAX);
      t[8] = tr_w < kL2StatWarps ? (int)(g_l2w[tr_w][3] - tr_c0) : -1;
      t[9] = __float_as_int((float)R.Z);
      t[10] = __float_as_int((float)R.r2);
      t[11] = __float_as_int((float)R.R2);
      t[12] = rex;
      FaceFx X;
      face_fx(X, F.p, F.a, F.b, F.gfix);
      t[13] = X.IA.w | (X.IB.w << 1) | ((int)X.fr.ok << 2);
      t[14] = X.fr.g;
    }
  }
#endif
  return best;
}

// ---- 2D exhaustive query across edge (p, x): sgn=+1 triangles (p,x,y),
// sgn=-1 triangles (p,y,x)
struct Edge2 {
  int ip, ix, sgn;
  float p[2], x[2];
  float X[2];
  FxFrame fr;  // fixed-point frame at p covering 8x the edge length
  int4 IX;
};

__device__ __forceinline__ void edge2_frame(Edge2 &E, int gfix) {
  fx_frame<2>(E.fr, E.p, 8.f * fmaxf(fabsf(E.X[0]), fabsf(E.X[1])), gfix);
  E.IX = fx_point<2>(E.fr, E.x);
}

__device__ __forceinline__ int side2(const Edge2 &E, const float *y,
                                     dmp::ExactScratch *W) {
  float Y[2] = {y[0] - E.p[0], y[1] - E.p[1]};
  int s = dmp::orient2_rel_filter<float>(E.X[0], E.X[1], Y[0], Y[1], 8.0f * DMP_U32);
  if (!s) {
    const int4 IY = fx_point<2>(E.fr, y);
    s = (E.IX.w & IY.w) ? dmp::orient2_fx(E.IX, IY) : dmp::orient2_slow(E.p, E.x, y, W);
  }
  return s * E.sgn;
}

// perturbed incirc2(p, b, c, d) of an edge query
__device__ __forceinline__ int incirc_edge2(const Edge2 &E, const float *b, const float *c,
                                            const float *d, int &ovf, dmp::ExactScratch *W) {
  float X[2] = {b[0] - E.p[0], b[1] - E.p[1]}, Y[2] = {c[0] - E.p[0], c[1] - E.p[1]},
        Z[2] = {d[0] - E.p[0], d[1] - E.p[1]};
  int s = dmp::incirc2_rel_filter<float>(X, Y, Z, X[0] * X[0] + X[1] * X[1],
                                         Y[0] * Y[0] + Y[1] * Y[1], Z[0] * Z[0] + Z[1] * Z[1],
                                         16.0f * DMP_U32);
  if (s) return s;
  const int4 IB = fx_point<2>(E.fr, b), IC = fx_point<2>(E.fr, c), ID = fx_point<2>(E.fr, d);
  if (IB.w & IC.w & ID.w) return dmp::incirc2_fx_sos(IB, IC, ID);
  s = dmp::incirc2_slow(E.p, b, c, d, &ovf, W);
  if (s) return s;
  return dmp::incirc2_sos_tail(E.p, b, c, d, W);
}

__device__ __forceinline__ int cmp2(const Edge2 &E, const float *bx,
                                    const float *y, int &ovf,
                                    dmp::ExactScratch *W) {
  // <0 when y lies inside the circle of the current triangle
  return E.sgn > 0 ? incirc_edge2(E, E.x, bx, y, ovf, W)
                   : incirc_edge2(E, bx, E.x, y, ovf, W);
}

__device__ __forceinline__ void consider2(const DTArgs &A, const Edge2 &E, int j,
                                          float4 q, int &best, float *bx, int &ovf,
                                          dmp::ExactScratch *W) {
  if (j == E.ip || j == E.ix) return;
  float y[2] = {q.x, q.y};
  if (side2(E, y, W) <= 0) return;
  if (best < 0 || cmp2(E, bx, y, ovf, W) < 0) {
    best = j;
    bx[0] = y[0];
    bx[1] = y[1];
  }
}

__device__ __forceinline__ int tourney2(const DTArgs &A, const Edge2 &E,
                                        int best, int &ovf,
                                        dmp::ExactScratch *W) {
  for (int o = 16; o; o >>= 1) {
    int other = __shfl_xor_sync(0xffffffffu, best, o);
    if (other >= 0 && other != best) {
      if (best < 0) {
        best = other;
      } else {
        float bx[2], ox[2];
        load_pt<2>(A.P, best, bx);
        load_pt<2>(A.P, other, ox);
        if (cmp2(E, bx, ox, ovf, W) < 0) best = other;
      }
    }
  }
  return best;
}

// Search region of a 2D edge query: the circle (c, r2) bounding every point
// that may beat the current winner, or (full) the positive half-plane of the
// edge p -> p + X with normal n when there is no winner yet.
struct Region2 {
  bool full;
  float c[2], r2;
  float p[2], n[2], nrm;
};

// May the box [lo, hi] hold a point of the region?  The tolerances are those
// of the per-cell and per-block tests of the queries.
__device__ __forceinline__ bool region_hits2(const Region2 &R, const GridParams &g,
                                             const float *lo, const float *hi) {
  if (!R.full) {
    float dd = 0.f;
    for (int k = 0; k < 2; ++k) {
      const float e = R.c[k] < lo[k] ? lo[k] - R.c[k] : (R.c[k] > hi[k] ? R.c[k] - hi[k] : 0.f);
      dd += e * e;
    }
    return dd <= R.r2 * 1.0001f + 1e-6f * g.cs * g.cs;
  }
  float mx = -FLT_MAX, scale = 0.f;
  for (int corner = 0; corner < 4; ++corner) {
    const float v0 = ((corner & 1) ? hi[0] : lo[0]) - R.p[0];
    const float v1 = ((corner >> 1) & 1 ? hi[1] : lo[1]) - R.p[1];
    mx = fmaxf(mx, v0 * R.n[0] + v1 * R.n[1]);
    scale = fmaxf(scale, fmaxf(fabsf(v0), fabsf(v1)));
  }
  return !(mx < -1e-4f * R.nrm * scale);
}

// The points of up to four coarse blocks (b0..b3, < 0: none) that may lie in
// the region, visited by the whole warp: lane l holds cell row l % 8 (the 8
// cells along x at one y) of block b(l / 8).  Points of the 3x3 cells
// around cc (already scanned) are skipped.
constexpr int kBs2 = 8;  // coarse block edge in 2D (GridParams::bs)
template <typename F>
__device__ __forceinline__ void scan_block_quad2(const DTArgs &A, const GridParams &g,
                                                 const Region2 &R, int b0, int b1, int b2, int b3,
                                                 const int *cc, int lane, F f) {
  const int slot = lane >> 3, r = lane & 7;
  const int b = slot == 0 ? b0 : slot == 1 ? b1 : slot == 2 ? b2 : b3;
  int off = 0, len = 0;
  if (b >= 0) {
    const int bxi = b % g.bdims[0], byi = b / g.bdims[0];
    const int y = byi * kBs2 + r, x0 = bxi * kBs2, x1 = min(x0 + kBs2, g.dims[0]);
    if (y < g.dims[1]) {
      float lo[2], hi[2];
      const int c0[2] = {x0, y}, c1[2] = {x1, y + 1};
      for (int k = 0; k < 2; ++k) {
        const float pad = (fabsf(g.lo[k]) + (float)g.dims[k] * g.cs) * 1e-6f;
        lo[k] = g.lo[k] + (float)c0[k] * g.cs - pad;
        hi[k] = g.lo[k] + (float)c1[k] * g.cs + pad;
      }
      if (region_hits2(R, g, lo, hi)) {
        const int cs0 = x0 + g.dims[0] * y;
        off = A.cell_start[cs0];
        len = A.cell_start[cs0 + (x1 - x0)] - off;
      }
    }
  }
  warp_ranges(A.spts, off, len, lane, [&](float4 q) {
    const int j = __float_as_int(q.w);
    if (j < 0) return;  // duplicate
    if (in_local(cc, cell_coord(g, q.x, 0), cell_coord(g, q.y, 1), 0, 2)) return;
    f(j, q);
  });
}

// Every point of the coarse blocks [blo, bhi] whose tight box meets the
// region: lanes test 32 blocks at a time and the hits are scanned four by
// four by the whole warp.
template <typename F>
__device__ __forceinline__ void scan_blocks2(const DTArgs &A, const GridParams &g,
                                             const Region2 &R, const int *blo, const int *bhi,
                                             const int *cc, int lane, F f) {
  const int sx = bhi[0] - blo[0] + 1, sy = bhi[1] - blo[1] + 1;
  if (sx <= 0 || sy <= 0) return;
  const int64_t nb = (int64_t)sx * sy;
  int q0 = -1, q1 = -1, q2 = -1, nq = 0;  // queued hits (warp-uniform)
  for (int64_t t0 = 0; t0 < nb; t0 += 32) {
    const int64_t t = t0 + lane;
    int bid = -1;
    if (t < nb) {
      const int bxi = blo[0] + (int)(t % sx), byi = blo[1] + (int)(t / sx);
      bid = bxi + g.bdims[0] * byi;
      if (A.blk_cnt[bid] == 0) {
        bid = -1;
      } else {
        const float lo[2] = {A.blk_box[6 * bid], A.blk_box[6 * bid + 1]};
        const float hi[2] = {A.blk_box[6 * bid + 3], A.blk_box[6 * bid + 4]};
        if (!region_hits2(R, g, lo, hi)) bid = -1;
      }
    }
    unsigned m = __ballot_sync(0xffffffffu, bid >= 0);
    while (m) {
      const int h = __shfl_sync(0xffffffffu, bid, __ffs(m) - 1);
      m &= m - 1;
      if (nq == 3) {
        scan_block_quad2(A, g, R, q0, q1, q2, h, cc, lane, f);
        q0 = q1 = q2 = -1;
        nq = 0;
      } else {
        if (nq == 0) q0 = h;
        else if (nq == 1) q1 = h;
        else q2 = h;
        ++nq;
      }
    }
  }
  if (nq) scan_block_quad2(A, g, R, q0, q1, q2, -1, cc, lane, f);
}

__device__ __forceinline__ int gq2(const DTArgs &A, const GridParams &g, int ip,
                                   int ix, int sgn, int lane, int &ovf,
                                   dmp::ExactScratch *W) {
  Edge2 E;
  E.ip = ip;
  E.ix = ix;
  E.sgn = sgn;
  load_pt<2>(A.P, ip, E.p);
  load_pt<2>(A.P, ix, E.x);
  E.X[0] = E.x[0] - E.p[0];
  E.X[1] = E.x[1] - E.p[1];
  edge2_frame(E, g.gfix);
  int best = -1;
  float bx[2];
  int cc[3] = {cell_coord(g, 0.5f * (E.p[0] + E.x[0]), 0),
               cell_coord(g, 0.5f * (E.p[1] + E.x[1]), 1), 0};
  if (lane < 9) {
    int x = cc[0] + lane % 3 - 1, y = cc[1] + lane / 3 - 1;
    if (x >= 0 && y >= 0 && x < g.dims[0] && y < g.dims[1])
      for_cell(A, x + g.dims[0] * y, [&](int j, float4 q) { consider2(A, E, j, q, best, bx, ovf, W); });
  }
  best = tourney2(A, E, best, ovf, W);
  // Search region (as in gq3): a point beating the winner y lies inside
  // circle(p, x, y) on the positive side of the edge, which lies inside
  // B(m + Z n^, sqrt(r^2 + Z^2)) with m, r the midpoint and half length of
  // the edge and Z >= max(z0, 0), z0 = (|y - m|^2 - r^2) / (2 h).
  bool full = true;
  double cen[2] = {0, 0}, rad = 0;
  if (best >= 0) {
    load_pt<2>(A.P, best, bx);
    const double u = 1.2e-16;
    double a[2] = {(double)E.x[0] - E.p[0], (double)E.x[1] - E.p[1]};
    double c[2] = {(double)bx[0] - E.p[0], (double)bx[1] - E.p[1]};
    double la = a[0] * a[0] + a[1] * a[1];
    if (la > 0) {
      double al = sqrt(la);
      double r2 = 0.25 * la;
      double w[2] = {c[0] - 0.5 * a[0], c[1] - 0.5 * a[1]};
      double lw = w[0] * w[0] + w[1] * w[1];
      double q = lw - r2;
      double eq = 1e-14 * (lw + r2 + la);
      double lc = sqrt(c[0] * c[0] + c[1] * c[1]);
      double hgt = E.sgn * (a[0] * c[1] - a[1] * c[0]) / al;
      double dh = 8 * u * lc;
      double Z = -1;
      if (q + eq <= 0) {
        Z = 0;
      } else if (hgt > 2 * dh) {
        Z = (q + eq) / (2 * (hgt - dh));
      }
      if (Z >= 0 && Z < 1e30) {
        double nx = -E.sgn * a[1] / al, ny = E.sgn * a[0] / al;
        cen[0] = 0.5 * a[0] + Z * nx + E.p[0];
        cen[1] = 0.5 * a[1] + Z * ny + E.p[1];
        rad = sqrt(r2 + Z * Z);
        rad = rad * (1 + 1e-6) + 1e-7 * (fabs(cen[0]) + fabs(cen[1]));
        full = !(rad < 1e30);
      }
    }
  }
  if (!full) {
    int lo[2], hi[2];
    int64_t ncell = 1;
    for (int k = 0; k < 2; ++k) {
      cell_range(g, cen[k], rad, k, lo[k], hi[k]);
      ncell *= max(0, hi[k] - lo[k] + 1);
    }
    float r2 = (float)(rad * rad) * 1.0001f;
    if (lane == 0) L2S_ADD(2, ncell);
    if (ncell <= 4096) {
      int sx = hi[0] - lo[0] + 1;
      for (int t = lane; t < ncell; t += 32) {
        int x = lo[0] + t % sx, y = lo[1] + t / sx;
        if (in_local(cc, x, y, 0, 2)) continue;
        float dd = 0.f;
        int ci[2] = {x, y};
        for (int k = 0; k < 2; ++k) {
          float b0 = g.lo[k] + ci[k] * g.cs, b1 = b0 + g.cs;
          float c = (float)cen[k];
          float e = c < b0 ? b0 - c : (c > b1 ? c - b1 : 0.f);
          dd += e * e;
        }
        if (dd > r2 + 1e-6f * g.cs * g.cs) continue;
        for_cell(A, x + g.dims[0] * y, [&](int j, float4 q) { consider2(A, E, j, q, best, bx, ovf, W); });
      }
    } else {
      Region2 R;
      R.full = false;
      R.c[0] = (float)cen[0];
      R.c[1] = (float)cen[1];
      R.r2 = r2;
      const int blo[2] = {lo[0] / kBs2, lo[1] / kBs2}, bhi[2] = {hi[0] / kBs2, hi[1] / kBs2};
      scan_blocks2(A, g, R, blo, bhi, cc, lane,
                   [&](int j, float4 q) { consider2(A, E, j, q, best, bx, ovf, W); });
    }
  } else {
    // every block that may hold a point on the positive side
    Region2 R;
    R.full = true;
    R.p[0] = E.p[0];
    R.p[1] = E.p[1];
    R.n[0] = -E.X[1] * sgn;
    R.n[1] = E.X[0] * sgn;
    R.nrm = sqrtf(E.X[0] * E.X[0] + E.X[1] * E.X[1]);
    const int blo[2] = {0, 0}, bhi[2] = {g.bdims[0] - 1, g.bdims[1] - 1};
    scan_blocks2(A, g, R, blo, bhi, cc, lane,
                 [&](int j, float4 q) { consider2(A, E, j, q, best, bx, ovf, W); });
  }
  return tourney2(A, E, best, ovf, W);
}

// exact emptiness of a circumsphere (circle) over the whole point set: every
// point in a cell that meets the ball is tested with the perturbed predicate.
template <int DIM>
__device__ __forceinline__ bool gempty(const DTArgs &A, const GridParams &g, int ip,
                                       const int *v, int lane, int &ovf,
                                       dmp::ExactScratch *W) {
  float P0[3], X[3][3];
  load_pt<DIM>(A.P, ip, P0);
  for (int k = 0; k < DIM; ++k) load_pt<DIM>(A.P, v[k], X[k]);
  double a[3][3];
  for (int k = 0; k < DIM; ++k)
    for (int j = 0; j < DIM; ++j) a[k][j] = (double)X[k][j] - P0[j];
  double cen[3] = {0, 0, 0}, rad;
  if (DIM == 3) {
    double bc[3] = {a[1][1] * a[2][2] - a[1][2] * a[2][1], a[1][2] * a[2][0] - a[1][0] * a[2][2],
                    a[1][0] * a[2][1] - a[1][1] * a[2][0]};
    double ca[3] = {a[2][1] * a[0][2] - a[2][2] * a[0][1], a[2][2] * a[0][0] - a[2][0] * a[0][2],
                    a[2][0] * a[0][1] - a[2][1] * a[0][0]};
    double ab[3] = {a[0][1] * a[1][2] - a[0][2] * a[1][1], a[0][2] * a[1][0] - a[0][0] * a[1][2],
                    a[0][0] * a[1][1] - a[0][1] * a[1][0]};
    double det = a[0][0] * bc[0] + a[0][1] * bc[1] + a[0][2] * bc[2];
    double l0 = a[0][0] * a[0][0] + a[0][1] * a[0][1] + a[0][2] * a[0][2];
    double l1 = a[1][0] * a[1][0] + a[1][1] * a[1][1] + a[1][2] * a[1][2];
    double l2 = a[2][0] * a[2][0] + a[2][1] * a[2][1] + a[2][2] * a[2][2];
    if (!(fabs(det) > 1e-9 * sqrt(l0 * l1 * l2))) return false;  // flat: reject
    for (int k = 0; k < 3; ++k) cen[k] = (l0 * bc[k] + l1 * ca[k] + l2 * ab[k]) / (2 * det);
  } else {
    double det = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    double l0 = a[0][0] * a[0][0] + a[0][1] * a[0][1], l1 = a[1][0] * a[1][0] + a[1][1] * a[1][1];
    if (!(fabs(det) > 1e-9 * sqrt(l0 * l1))) return false;
    cen[0] = (a[1][1] * l0 - a[0][1] * l1) / (2 * det);
    cen[1] = (a[0][0] * l1 - a[1][0] * l0) / (2 * det);
  }
  rad = sqrt(cen[0] * cen[0] + cen[1] * cen[1] + cen[2] * cen[2]);
  for (int k = 0; k < DIM; ++k) cen[k] += P0[k];
  rad = rad * (1 + 1e-6) + 1e-7 * (fabs(cen[0]) + fabs(cen[1]) + fabs(cen[2]));
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  int64_t ncell = 1;
  for (int k = 0; k < DIM; ++k) {
    cell_range(g, cen[k], rad, k, lo[k], hi[k]);
    ncell *= max(0, hi[k] - lo[k] + 1);
  }
  const float r2 = (float)(rad * rad) * 1.0001f;
  const int sx = hi[0] - lo[0] + 1, sy = hi[1] - lo[1] + 1;
  bool inside = false;
  for (int64_t t = lane; t < ncell && !inside; t += 32) {
    int x = lo[0] + (int)(t % sx), y = lo[1] + (int)((t / sx) % sy),
        z = DIM == 3 ? lo[2] + (int)(t / ((int64_t)sx * sy)) : 0;
    float dd = 0.f;
    int ci[3] = {x, y, z};
    for (int k = 0; k < DIM; ++k) {
      float b0 = g.lo[k] + ci[k] * g.cs, b1 = b0 + g.cs;
      float cc = (float)cen[k];
      float e = cc < b0 ? b0 - cc : (cc > b1 ? cc - b1 : 0.f);
      dd += e * e;
    }
    if (dd > r2 + 1e-6f * g.cs * g.cs) continue;
    int c = x + g.dims[0] * (y + g.dims[1] * z);
    for (int i = A.cell_start[c]; i < A.cell_start[c + 1] && !inside; ++i) {
      int j = A.sorted[i];
      if (j == ip || j == v[0] || j == v[1] || (DIM == 3 && j == v[2]) || A.dup[j]) continue;
      float y3[3];
      load_pt<DIM>(A.P, j, y3);
      int s = DIM == 3 ? insph3_sos(P0, X[0], X[1], X[2], y3, &ovf, W)
                       : incirc2_sos(P0, X[0], X[1], y3, &ovf, W);
      inside = s < 0;
    }
  }
  return !__any_sync(0xffffffffu, inside);
}

// Warp-cooperative ring search around cell cc: visits cells at Chebyshev
// distance k = 0, 1, ... and calls f(j) for their points; after ring k,
// every point within guard(k) of the centre x was visited.  Stops once
// done(guard) is true or the grid is exhausted.
template <int DIM, typename F, typename D>
__device__ __forceinline__ void ring_search(const DTArgs &A, const GridParams &g,
                                            const float *x, int lane, F f, D done) {
  int cc[3] = {0, 0, 0};
  for (int k = 0; k < DIM; ++k) cc[k] = cell_coord(g, x[k], k);
  int kmax = 0;
  for (int k = 0; k < DIM; ++k) kmax = max(kmax, max(cc[k], g.dims[k] - 1 - cc[k]));
  for (int r = 0; r <= kmax; ++r) {
    const int w = 2 * r + 1;
    const int64_t ncell = DIM == 3 ? (int64_t)w * w * w : (int64_t)w * w;
    for (int64_t t = lane; t < ncell; t += 32) {
      int d0 = (int)(t % w) - r, d1 = (int)((t / w) % w) - r,
          d2 = DIM == 3 ? (int)(t / ((int64_t)w * w)) - r : 0;
      if (max(abs(d0), max(abs(d1), abs(d2))) != r) continue;  // ring only
      int xx = cc[0] + d0, yy = cc[1] + d1, zz = DIM == 3 ? cc[2] + d2 : 0;
      if (xx < 0 || yy < 0 || zz < 0 || xx >= g.dims[0] || yy >= g.dims[1] ||
          (DIM == 3 && zz >= g.dims[2]))
        continue;
      int c = xx + g.dims[0] * (yy + g.dims[1] * zz);
      for (int i = A.cell_start[c]; i < A.cell_start[c + 1]; ++i) f(A.sorted[i]);
    }
    float guard = FLT_MAX;
    for (int k = 0; k < DIM; ++k) {
      if (cc[k] - r > 0) guard = fminf(guard, x[k] - (g.lo[k] + (cc[k] - r) * g.cs));
      if (cc[k] + r + 1 < g.dims[k]) guard = fminf(guard, (g.lo[k] + (cc[k] + r + 1) * g.cs) - x[k]);
    }
    guard *= (1.f - 1e-5f);
    if (done(guard)) return;
  }
}

// global seed from a nearest neighbour q1 and a smallest circumcircle
// through (p, q1): for points in general position the triangle (p, q1, q2)
// is Delaunay and both cells on its sides are found by exhaustive queries;
// the candidate cell is verified empty over the whole point set.  On
// degenerate sets (a lattice: many neighbours at the same distance, many
// circles of the same radius) the first pick may be a triangle the
// perturbed triangulation does not contain, so the next candidates are
// tried: up to kSeedQ2 choices of q2 for each of up to kSeedQ1 choices of
// q1, each excluding the ones already tried.
constexpr int kSeedQ1 = 4, kSeedQ2 = 8;
__device__ __forceinline__ bool gseed3_nn(const DTArgs &A, const GridParams &g, int ip,
                                          int lane, int &ovf, dmp::ExactScratch *W,
                                          int3 &out) {
  float px[3];
  load_pt<3>(A.P, ip, px);
  int ex1[kSeedQ1];
  for (int a1 = 0; a1 < kSeedQ1; ++a1) {
    float bk = FLT_MAX;
    int bj = -1, bg = 0x7fffffff;
    ring_search<3>(A, g, px, lane,
                   [&](int j) {
                     if (j == ip || A.dup[j]) return;
                     for (int e = 0; e < a1; ++e)
                       if (ex1[e] == j) return;
                     float y[3];
                     load_pt<3>(A.P, j, y);
                     float d = (y[0] - px[0]) * (y[0] - px[0]) + (y[1] - px[1]) * (y[1] - px[1]) +
                               (y[2] - px[2]) * (y[2] - px[2]);
                     if (bj < 0 || d < bk || (d == bk && j < bg)) {
                       bk = d;
                       bj = j;
                       bg = j;
                     }
                   },
                   [&](float guard) {
                     float k2 = bk;
                     int j2 = bj, g2 = bg;
                     warp_argmin(k2, j2, g2);
                     return j2 >= 0 && sqrtf(k2) < guard;
                   });
    warp_argmin(bk, bj, bg);
    if (bj < 0) return false;
    const int q1 = bj;
    ex1[a1] = q1;
    float a[3];
    load_pt<3>(A.P, q1, a);
    const float A3[3] = {a[0] - px[0], a[1] - px[1], a[2] - px[2]};
    const float m[3] = {0.5f * (a[0] + px[0]), 0.5f * (a[1] + px[1]), 0.5f * (a[2] + px[2])};
    int ex2[kSeedQ2];
    for (int a2 = 0; a2 < kSeedQ2; ++a2) {
      float ck = FLT_MAX;
      int cj = -1, cg = 0x7fffffff;
      ring_search<3>(A, g, m, lane,
                     [&](int j) {
                       if (j == ip || j == q1 || A.dup[j]) return;
                       for (int e = 0; e < a2; ++e)
                         if (ex2[e] == j) return;
                       float y[3];
                       load_pt<3>(A.P, j, y);
                       float B[3] = {y[0] - px[0], y[1] - px[1], y[2] - px[2]};
                       float cx = A3[1] * B[2] - A3[2] * B[1], cy = A3[2] * B[0] - A3[0] * B[2],
                             cz = A3[0] * B[1] - A3[1] * B[0];
                       float cr = cx * cx + cy * cy + cz * cz;
                       if (!(cr > 0.f)) return;
                       float la = A3[0] * A3[0] + A3[1] * A3[1] + A3[2] * A3[2];
                       float lb = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
                       float dx = A3[0] - B[0], dy = A3[1] - B[1], dz = A3[2] - B[2];
                       float R2 = la * lb * (dx * dx + dy * dy + dz * dz) / (4.f * cr);
                       if (cj < 0 || R2 < ck || (R2 == ck && j < cg)) {
                         ck = R2;
                         cj = j;
                         cg = j;
                       }
                     },
                     [&](float guard) {
                       float k2 = ck;
                       int j2 = cj, g2 = cg;
                       warp_argmin(k2, j2, g2);
                       // a smaller circumcircle through p and q1 lies within 2R of m
                       return j2 >= 0 && 2.f * sqrtf(k2) * 1.0001f < guard;
                     });
      warp_argmin(ck, cj, cg);
      if (cj < 0) break;
      const int q2 = cj;
      ex2[a2] = q2;
      for (int side = 0; side < 2; ++side) {
        int u = side ? q2 : q1, v = side ? q1 : q2;
        int x = gq3(A, g, ip, u, v, lane, ovf, W);
        if (x < 0) continue;
        int vv[3] = {u, v, x};
        if (gempty<3>(A, g, ip, vv, lane, ovf, W)) {
          out = make_int3(u, v, x);
          return true;
        }
      }
    }
  }
  return false;
}

__device__ __forceinline__ bool gseed2_nn(const DTArgs &A, const GridParams &g, int ip,
                                          int lane, int &ovf, dmp::ExactScratch *W,
                                          int &oa, int &ob) {
  float px[3];
  load_pt<2>(A.P, ip, px);
  float bk = FLT_MAX;
  int bj = -1, bg = 0x7fffffff;
  ring_search<2>(A, g, px, lane,
                 [&](int j) {
                   if (j == ip || A.dup[j]) return;
                   float y[3];
                   load_pt<2>(A.P, j, y);
                   float d = (y[0] - px[0]) * (y[0] - px[0]) + (y[1] - px[1]) * (y[1] - px[1]);
                   if (bj < 0 || d < bk || (d == bk && j < bg)) {
                     bk = d;
                     bj = j;
                     bg = j;
                   }
                 },
                 [&](float guard) {
                   float k2 = bk;
                   int j2 = bj, g2 = bg;
                   warp_argmin(k2, j2, g2);
                   return j2 >= 0 && sqrtf(k2) < guard;
                 });
  warp_argmin(bk, bj, bg);
  if (bj < 0) return false;
  const int q1 = bj;
  for (int sgn = 1; sgn >= -1; sgn -= 2) {
    int x = gq2(A, g, ip, q1, sgn, lane, ovf, W);
    if (x < 0) continue;
    int a = sgn > 0 ? q1 : x, b = sgn > 0 ? x : q1;
    int vv[3] = {a, b, -1};
    if (gempty<2>(A, g, ip, vv, lane, ovf, W)) {
      oa = a;
      ob = b;
      return true;
    }
  }
  return false;
}

// Seed for the exhaustive level: local candidate pools of growing size,
// the local seed cell kept when its circumball lies inside the pool's
// covered radius or when it is empty over the whole point set.
__device__ __forceinline__ bool gseed3(WarpL1<3> &Q, const DTArgs &A, const GridParams &g,
                                       int ip, int lane, int &ovf, dmp::ExactScratch *W,
                                       int3 &out) {
  float px[3];
  load_pt<3>(A.P, ip, px);
  for (int K = 2; K <= 8; K *= 2) {
    gather_l1<3>(Q, A, g, ip, px, lane, K);
    if (Q.nc < 3) continue;
    uint32_t t = seed3L(Q, A.P, ip, lane, ovf, W);
    if (t == 0xffffffffu) continue;
    int v[3] = {Q.id[un0(t)], Q.id[un1(t)], Q.id[un2(t)]};
    bool ok = certified3(Q.c[un0(t)], Q.c[un1(t)], Q.c[un2(t)], Q.reff);
    if (!ok) ok = gempty<3>(A, g, ip, v, lane, ovf, W);
    if (ok) {
      out = make_int3(v[0], v[1], v[2]);
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ bool gseed2(WarpL1<2> &Q, const DTArgs &A, const GridParams &g,
                                       int ip, int lane, int &ovf, dmp::ExactScratch *W,
                                       int &oa, int &ob) {
  float px[3];
  load_pt<2>(A.P, ip, px);
  for (int K = 3; K <= 12; K *= 2) {
    gather_l1<2>(Q, A, g, ip, px, lane, K);
    if (Q.nc < 2) continue;
    uint32_t t = seed2L(Q, A.P, ip, lane, ovf, W);
    if (t == 0xffffffffu) continue;
    int v[3] = {Q.id[un0(t)], Q.id[un1(t)], -1};
    bool ok = certified2(Q.c[un0(t)], Q.c[un1(t)], Q.reff);
    if (!ok) ok = gempty<2>(A, g, ip, v, lane, ovf, W);
    if (ok) {
      oa = v[0];
      ob = v[1];
      return true;
    }
  }
  return false;
}

// Storage of one star under construction: link triangles, open link edges
// (3D) and counters cnt = {ntri, nopen, flags}.  Level 2 keeps it in shared
// memory (192 triangles); stars that outgrow it are finished by level 3 in a
// per-warp slot of global memory (L3_CAP_TRI triangles).
struct StarStore {
  int3 *tri, *open;
  int *cnt;
  int cap_tri, cap_open;
};


__device__ __forceinline__ int find_rev_s(const StarStore &S, int s, int t, int lane) {
  const int nopen = S.cnt[1];
  int hit = -1;
  for (int k = lane; k < nopen; k += 32) {
    int3 e = S.open[k];
    if (e.x == t && e.y == s) hit = k;
  }
  unsigned m = __ballot_sync(0xffffffffu, hit >= 0);
  if (!m) return -1;
  return __shfl_sync(0xffffffffu, hit, __ffs(m) - 1);
}

// exhaustive gift-wrap walk of the star of ip (3D) from a seed link triangle;
// false when the storage overflowed
__device__ __forceinline__ bool walk3(const DTArgs &A, const GridParams &g, int ip, int3 seed,
                                      int lane, int &ovf, dmp::ExactScratch *W,
                                      const StarStore &S) {
  if (lane == 0) {
    S.cnt[0] = 1;
    S.tri[0] = seed;
    S.open[0] = make_int3(seed.x, seed.y, seed.z);
    S.open[1] = make_int3(seed.y, seed.z, seed.x);
    S.open[2] = make_int3(seed.z, seed.x, seed.y);
    S.cnt[1] = 3;
    S.cnt[2] = 0;
  }
  __syncwarp();
  while (S.cnt[1] > 0) {
    int3 e = S.open[S.cnt[1] - 1];
    __syncwarp();
    if (lane == 0) S.cnt[1]--;
    __syncwarp();
    int u = e.x, v = e.y;
    int y = gq3(A, g, ip, v, u, lane, ovf, W);
    if (y < 0) continue;  // convex-hull face
    if (S.cnt[0] >= S.cap_tri) {
      if (lane == 0) S.cnt[2] |= 1;
      __syncwarp();
      break;
    }
    if (lane == 0) S.tri[S.cnt[0]++] = make_int3(v, u, y);
    __syncwarp();
    int es[2][3] = {{u, y, v}, {y, v, u}};
    for (int q = 0; q < 2; ++q) {
      int r = find_rev_s(S, es[q][0], es[q][1], lane);
      if (lane == 0) {
        if (r >= 0) {
          S.open[r] = S.open[S.cnt[1] - 1];
          S.cnt[1]--;
        } else if (S.cnt[1] < S.cap_open) {
          S.open[S.cnt[1]++] = make_int3(es[q][0], es[q][1], es[q][2]);
        } else {
          S.cnt[2] |= 1;
        }
      }
      __syncwarp();
    }
    if (S.cnt[2]) break;
  }
  __syncwarp();
  return S.cnt[2] == 0;
}

// cells of a finished star owned by ip (smallest index)
__device__ __forceinline__ void emit3(const DTArgs &A, int ip, const StarStore &S, int lane) {
  const int ntri = S.cnt[0];
  for (int t0 = 0; t0 < ntri; t0 += 32) {
    int t = t0 + lane;
    bool own = false;
    int3 tr = make_int3(0, 0, 0);
    if (t < ntri) {
      tr = S.tri[t];
      own = ip < tr.x && ip < tr.y && ip < tr.z;
    }
    int64_t q = warp_append(&A.counters[DM_CNT_CELLS], own);
    if (own) {
      if (q < A.cap_cells_out) {
        reinterpret_cast<int4 *>(A.cells)[q] = make_int4(ip, tr.x, tr.y, tr.z);
      } else {
        flag_or(A.counters, DM_FLAG_CELL_OVERFLOW);
      }
    }
  }
  __syncwarp();
}

// seed of escalated star k: the certified level-1 cell, else a global search
__device__ __forceinline__ bool seed_of3(const DTArgs &A, const GridParams &g, int64_t k,
                                         WarpL1<3> &Q1, int lane, int &ovf,
                                         dmp::ExactScratch *W, int &ip, int3 &seed) {
  int4 sd = A.esc_seed[k];
  ip = sd.x & ~(1 << 30);
  const bool certified = (sd.x >> 30) & 1;
  seed = make_int3(-1, -1, -1);
  if (certified) {
    seed = make_int3(sd.y, sd.z, sd.w);
  } else if (!gseed3(Q1, A, g, ip, lane, ovf, W, seed) &&
             !gseed3_nn(A, g, ip, lane, ovf, W, seed)) {
    seed = make_int3(-1, -1, -1);
  }
  return seed.x >= 0;
}

__global__ void __launch_bounds__(32 * L2_WARPS, DM_L2_MINB) k_star3_l2(DTArgs A) {
  __shared__ WarpL2 sm[L2_WARPS];
  __shared__ WarpL1<3> sm1[L2_WARPS];
  __shared__ int scnt[L2_WARPS][4];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const StarStore S = {sm[w].tri, sm[w].open, scnt[w], L2_MAXTRI, L2_MAXOPEN};
  auto &Q1 = sm1[w];
  const GridParams g = *A.gp;
  const int64_t nesc = A.counters[DM_CNT_ESCALATED];
  // stars are taken one at a time from a shared counter: their costs vary by
  // orders of magnitude, so a static split leaves a long tail
  for (;;) {
    unsigned long long kk = 0;
    if (lane == 0) kk = atomicAdd((unsigned long long *)&A.counters[kCntL2Next], 1ull);
    const int64_t k = (int64_t)__shfl_sync(0xffffffffu, kk, 0);
    if (k >= nesc) break;
#ifdef DM_L2_STATS
    long long t_start = clock64();
    if (lane < 8) g_l2w[blockIdx.x * L2_WARPS + w][lane] = 0;
    __syncwarp();
#endif
    int ovf = 0, ip;
    int3 seed;
    if (!seed_of3(A, g, k, Q1, lane, ovf, W, ip, seed)) {
      if (lane == 0) flag_or(A.counters, DM_FLAG_SEED_FAILED);
      continue;
    }
    const bool done = walk3(A, g, ip, seed, lane, ovf, W, S);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
#ifdef DM_DEBUG_VERTEX
    if (ip == A.dbg_vertex && A.dbg) {
      // level-2 walk of the watched vertex: [1000] ntri, [1002..1004] seed,
      // [1008 + 3t ..] triangles in walk order
      if (lane == 0) {
        A.dbg[1000] = S.cnt[0];
        A.dbg[1002] = seed.x;
        A.dbg[1003] = seed.y;
        A.dbg[1004] = seed.z;
      }
      for (int t = lane; t < S.cnt[0]; t += 32) {
        A.dbg[1008 + 3 * t] = S.tri[t].x;
        A.dbg[1008 + 3 * t + 1] = S.tri[t].y;
        A.dbg[1008 + 3 * t + 2] = S.tri[t].z;
      }
      __syncwarp();
    }
#endif
#ifdef DM_L2_STATS
    if (lane == 0 && k < kL2StatStars) {
      g_l2s[k][0] = clock64() - t_start;
      g_l2s[k][1] = S.cnt[0] | ((unsigned long long)ip << 32);
      for (int q = 1; q < 7; ++q) g_l2s[k][q + 1] = g_l2w[blockIdx.x * L2_WARPS + w][q];
    }
#endif
    if (!done) {
      // too large for shared memory: finished by level 3
      if (lane == 0) {
        int64_t k3 = atomicAdd((unsigned long long *)&A.counters[kCntL3], 1ull);
        A.l3_list[k3] = (int32_t)k;
      }
      __syncwarp();
      continue;
    }
    emit3(A, ip, S, lane);
  }
}

__global__ void __launch_bounds__(32 * L3_WARPS) k_star3_l3(DTArgs A) {
  __shared__ WarpL1<3> sm1[L3_WARPS];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gw = blockIdx.x * L3_WARPS + w;
  const StarStore S = {A.l3_tri + (int64_t)gw * L3_CAP_TRI, A.l3_open + (int64_t)gw * L3_CAP_OPEN,
                       A.l3_cnt + 4 * gw, L3_CAP_TRI, L3_CAP_OPEN};
  const GridParams g = *A.gp;
  const int64_t n3 = A.counters[kCntL3];
  for (int64_t k3 = gw; k3 < n3; k3 += (int64_t)gridDim.x * L3_WARPS) {
    const int64_t k = A.l3_list[k3];
    int ovf = 0, ip;
    int3 seed;
    if (!seed_of3(A, g, k, sm1[w], lane, ovf, W, ip, seed)) {
      if (lane == 0) flag_or(A.counters, DM_FLAG_SEED_FAILED);
      continue;
    }
    const bool done = walk3(A, g, ip, seed, lane, ovf, W, S);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
    if (!done) {
      if (lane == 0) {
        flag_or(A.counters, DM_FLAG_STAR_OVERFLOW);
        A.counters[8] = ip;
        A.counters[9] = S.cnt[0];
        A.counters[10] = S.cnt[1];
      }
      __syncwarp();
      continue;
    }
    emit3(A, ip, S, lane);
  }
}

// linear walk of the star of ip (2D) from the link edge (a, b): forward
// around p, then backward from a when a hull edge stops it
__device__ __forceinline__ bool walk2(const DTArgs &A, const GridParams &g, int ip, int a, int b,
                                      int lane, int &ovf, dmp::ExactScratch *W,
                                      const StarStore &S) {
  if (lane == 0) {
    S.cnt[0] = 1;
    S.tri[0] = make_int3(a, b, 0);
    S.cnt[2] = 0;
  }
  __syncwarp();
  bool hull = false;
  int cur = b;
  while (true) {
    int nx = gq2(A, g, ip, cur, +1, lane, ovf, W);
    if (nx < 0) {
      hull = true;
      break;
    }
    if (S.cnt[0] >= S.cap_tri) {
      if (lane == 0) S.cnt[2] |= 1;
      __syncwarp();
      break;
    }
    if (lane == 0) S.tri[S.cnt[0]++] = make_int3(cur, nx, 0);
    __syncwarp();
    if (nx == a) break;  // closing triangle (p, cur, a)
    cur = nx;
  }
  if (hull && !S.cnt[2]) {
    cur = a;
    while (true) {
      int pv = gq2(A, g, ip, cur, -1, lane, ovf, W);
      if (pv < 0) break;
      if (S.cnt[0] >= S.cap_tri) {
        if (lane == 0) S.cnt[2] |= 1;
        __syncwarp();
        break;
      }
      if (lane == 0) S.tri[S.cnt[0]++] = make_int3(pv, cur, 0);
      __syncwarp();
      cur = pv;
    }
  }
  __syncwarp();
  return S.cnt[2] == 0;
}

__device__ __forceinline__ void emit2(const DTArgs &A, int ip, const StarStore &S, int lane) {
  const int ntri = S.cnt[0];
  for (int t0 = 0; t0 < ntri; t0 += 32) {
    int t = t0 + lane;
    bool own = false;
    int3 tr = make_int3(0, 0, 0);
    if (t < ntri) {
      tr = S.tri[t];
      own = ip < tr.x && ip < tr.y;
    }
    int64_t q = warp_append(&A.counters[DM_CNT_CELLS], own);
    if (own) {
      if (q < A.cap_cells_out) {
        A.cells[3 * q] = ip;
        A.cells[3 * q + 1] = tr.x;
        A.cells[3 * q + 2] = tr.y;
      } else {
        flag_or(A.counters, DM_FLAG_CELL_OVERFLOW);
      }
    }
  }
  __syncwarp();
}

__device__ __forceinline__ bool seed_of2(const DTArgs &A, const GridParams &g, int64_t k,
                                         WarpL1<2> &Q1, int lane, int &ovf,
                                         dmp::ExactScratch *W, int &ip, int &a, int &b) {
  int4 sd = A.esc_seed[k];
  ip = sd.x & ~(1 << 30);
  const bool certified = (sd.x >> 30) & 1;
  a = -1;
  b = -1;
  if (certified) {
    a = sd.y;
    b = sd.z;
  } else if (!gseed2(Q1, A, g, ip, lane, ovf, W, a, b) &&
             !gseed2_nn(A, g, ip, lane, ovf, W, a, b)) {
    a = -1;
  }
  return a >= 0;
}

__global__ void __launch_bounds__(32 * L2_WARPS) k_star2_l2(DTArgs A) {
  __shared__ WarpL2 sm[L2_WARPS];
  __shared__ WarpL1<2> sm1[L2_WARPS];
  __shared__ int scnt[L2_WARPS][4];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const StarStore S = {sm[w].tri, sm[w].open, scnt[w], L2_MAXTRI, L2_MAXOPEN};
  auto &Q1 = sm1[w];
  const GridParams g = *A.gp;
  const int64_t nesc = A.counters[DM_CNT_ESCALATED];
  // stars are taken one at a time from a shared counter, as in 3D
  for (;;) {
    unsigned long long kk = 0;
    if (lane == 0) kk = atomicAdd((unsigned long long *)&A.counters[kCntL2Next], 1ull);
    const int64_t k = (int64_t)__shfl_sync(0xffffffffu, kk, 0);
    if (k >= nesc) break;
    int ovf = 0, ip, a, b;
    if (!seed_of2(A, g, k, Q1, lane, ovf, W, ip, a, b)) {
      if (lane == 0) flag_or(A.counters, DM_FLAG_SEED_FAILED);
      continue;
    }
    const bool done = walk2(A, g, ip, a, b, lane, ovf, W, S);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
    if (!done) {
      if (lane == 0) {
        int64_t k3 = atomicAdd((unsigned long long *)&A.counters[kCntL3], 1ull);
        A.l3_list[k3] = (int32_t)k;
      }
      __syncwarp();
      continue;
    }
    emit2(A, ip, S, lane);
  }
}

__global__ void __launch_bounds__(32 * L3_WARPS) k_star2_l3(DTArgs A) {
  __shared__ WarpL1<2> sm1[L3_WARPS];
  dmp::ExactScratch WS;
  dmp::ExactScratch *W = &WS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int gw = blockIdx.x * L3_WARPS + w;
  const StarStore S = {A.l3_tri + (int64_t)gw * L3_CAP_TRI, A.l3_open + (int64_t)gw * L3_CAP_OPEN,
                       A.l3_cnt + 4 * gw, L3_CAP_TRI, L3_CAP_OPEN};
  const GridParams g = *A.gp;
  const int64_t n3 = A.counters[kCntL3];
  for (int64_t k3 = gw; k3 < n3; k3 += (int64_t)gridDim.x * L3_WARPS) {
    const int64_t k = A.l3_list[k3];
    int ovf = 0, ip, a, b;
    if (!seed_of2(A, g, k, sm1[w], lane, ovf, W, ip, a, b)) {
      if (lane == 0) flag_or(A.counters, DM_FLAG_SEED_FAILED);
      continue;
    }
    const bool done = walk2(A, g, ip, a, b, lane, ovf, W, S);
    if (ovf) flag_or(A.counters, DM_FLAG_EXACT_OVERFLOW);
    if (!done) {
      if (lane == 0) {
        flag_or(A.counters, DM_FLAG_STAR_OVERFLOW);
        A.counters[8] = ip;
        A.counters[9] = S.cnt[0];
      }
      __syncwarp();
      continue;
    }
    emit2(A, ip, S, lane);
  }
}

// ---------------------------------------------------------------------------
static int g_dbg_vertex = -1;
static int32_t *g_dbg = nullptr;

// Optional timing of the star kernels (events on the caller's stream).
constexpr int kProfMax = 256;
static bool g_prof_on = false;
static int g_prof_n = 0;
static cudaEvent_t g_prof_ev[kProfMax][3];
static int64_t g_launches = 0;

void note_launches(int k) { g_launches += k; }

static void prof_mark(int slot, cudaStream_t s) {
  if (!g_prof_on || g_prof_n >= kProfMax) return;
  cudaEvent_t &e = g_prof_ev[g_prof_n][slot];
  if (!e) cudaEventCreate(&e);
  // inside a stream capture the mark becomes an event-record node of the
  // graph, re-recorded (with its timestamp) at every replay
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &st);
  if (st == cudaStreamCaptureStatusActive)
    cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
  else
    cudaEventRecord(e, s);
}

int delaunay_workspace(int dim, int64_t n, size_t *bytes) {
  Carve c(nullptr, 0);
  DTArgs a;
  *bytes = carve_dt(c, a, dim, n) + 256;
  return DM_OK;
}

int delaunay(int dim, const float *pts, int64_t n, int32_t *cells,
             int64_t cap_cells, int64_t *counters, void *ws, size_t ws_bytes,
             cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim must be 2 or 3");
  DM_ARG_CHECK(n >= 0 && n < (1 << 30), "n out of range");
  DM_ARG_CHECK(pts != nullptr || n == 0, "points is null");
  DM_ARG_CHECK(cells != nullptr && counters != nullptr, "null output");
  DM_ARG_CHECK(((uintptr_t)pts & (dim == 3 ? 15 : 7)) == 0, "points misaligned");
  DM_ARG_CHECK(((uintptr_t)cells & 15) == 0, "cells misaligned");
  Carve c(ws, ws_bytes);
  DTArgs a;
  memset(&a, 0, sizeof(a));
  carve_dt(c, a, dim, n);
  if (!c.ok() || ws == nullptr) {
    set_error("delaunay: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  a.dim = dim;
  a.n = n;
  a.P = pts;
  a.cells = cells;
  a.cap_cells_out = cap_cells;
  a.counters = counters;
  a.dbg_vertex = g_dbg_vertex;
  a.dbg = g_dbg;
  DM_CUDA_TRY(cudaMemsetAsync(counters, 0, sizeof(int64_t) * DM_NCOUNTERS, s));
  if (n == 0) return DM_OK;
  DM_CUDA_TRY(cudaMemsetAsync(a.cell_cnt, 0, sizeof(int32_t) * a.cap_cells, s));
  int nb = grid_for(n, 256);
  k_bbox_init<<<1, 32, 0, s>>>(a.bbox);
  if (dim == 3)
    k_bbox<3><<<nb, 256, 0, s>>>(pts, n, a.bbox, counters);
  else
    k_bbox<2><<<nb, 256, 0, s>>>(pts, n, a.bbox, counters);
  k_grid_params<<<1, 32, 0, s>>>(a.gp, a.bbox, n, dim, a.cap_cells, a.cap_blocks);
  // count once on the bounding-box grid to measure occupancy, refine the
  // cell size, count again on the final grid
  for (int pass = 0; pass < 2; ++pass) {
    if (pass) {
      DM_CUDA_TRY(cudaMemsetAsync(a.occ, 0, sizeof(int), s));
      k_occupancy<<<grid_for(a.cap_cells, 256), 256, 0, s>>>(a.cell_cnt, a.gp, a.occ);
      k_grid_refine<<<1, 32, 0, s>>>(a.gp, a.bbox, a.occ, n, a.cap_cells);
      DM_CUDA_TRY(cudaMemsetAsync(a.cell_cnt, 0, sizeof(int32_t) * a.cap_cells, s));
    }
    if (dim == 3)
      k_cell_count<3><<<nb, 256, 0, s>>>(pts, n, a.gp, a.cell_of, a.slot, a.cell_cnt);
    else
      k_cell_count<2><<<nb, 256, 0, s>>>(pts, n, a.gp, a.cell_of, a.slot, a.cell_cnt);
  }
  DM_LAUNCH_CHECK();
  int rc = exclusive_scan_i32(a.cell_cnt, a.cell_start, a.cap_cells, a.scan_tmp, s);
  if (rc) return rc;
  k_cell_scatter<<<nb, 256, 0, s>>>(n, a.cell_of, a.slot, a.cell_start, a.sorted);
  int ncb = grid_for(a.cap_cells, 256);
  if (dim == 3) {
    k_cell_sort<3><<<ncb, 256, 0, s>>>(pts, a.gp, a.cell_start, a.sorted, a.dup, counters);
    k_sorted_points<3><<<nb, 256, 0, s>>>(pts, n, a.sorted, a.dup, a.spts);
    k_block_boxes<3><<<grid_for(a.cap_blocks, 128), 128, 0, s>>>(
        pts, a.gp, a.cell_start, a.sorted, a.blk_cnt, a.blk_box);
  } else {
    k_cell_sort<2><<<ncb, 256, 0, s>>>(pts, a.gp, a.cell_start, a.sorted, a.dup, counters);
    k_sorted_points<2><<<nb, 256, 0, s>>>(pts, n, a.sorted, a.dup, a.spts);
    k_block_boxes<2><<<grid_for(a.cap_blocks, 128), 128, 0, s>>>(
        pts, a.gp, a.cell_start, a.sorted, a.blk_cnt, a.blk_box);
  }
  DM_LAUNCH_CHECK();
  // (non-finite coordinates are reported through DM_FLAG_NONFINITE; the star
  // kernels still run on the single-cell grid and stay bounded)
  int64_t nwb = (n + L1_WARPS - 1) / L1_WARPS;
  int g1 = (int)std::min<int64_t>(nwb, (int64_t)kSMs * 16);
  if (dim == 3) DM_CUDA_TRY(cudaMemsetAsync(a.hullc, 0, n, s));
  prof_mark(0, s);
  if (dim == 3)
    k_star3_l1<<<g1, 32 * L1_WARPS, 0, s>>>(a);
  else
    k_star2_l1<<<g1, 32 * L1_WARPS, 0, s>>>(a);
  DM_LAUNCH_CHECK();
  prof_mark(1, s);
  int launches = 17;
  if (dim == 3) {
    // hull candidates bucketed by coarse block
    DM_CUDA_TRY(cudaMemsetAsync(a.o_cnt, 0, sizeof(int32_t) * a.cap_blocks, s));
    k_hc_init<<<grid_for(a.cap_blocks, 256), 256, 0, s>>>(a.gp, a.o_cnt, a.o_box);
    k_hc_count<<<nb, 256, 0, s>>>(n, a.hullc, a.cell_of, a.gp, a.o_cnt);
    rc = exclusive_scan_i32(a.o_cnt, a.o_start, a.cap_blocks, a.scan_tmp, s);
    if (rc) return rc;
    DM_CUDA_TRY(cudaMemsetAsync(a.o_cnt, 0, sizeof(int32_t) * a.cap_blocks, s));
    k_hc_fill<<<nb, 256, 0, s>>>(n, pts, a.hullc, a.cell_of, a.gp, a.o_start, a.o_cnt,
                                 a.o_box, a.o_pts);
    DM_CUDA_TRY(cudaMemsetAsync(a.o_ntab, 0, sizeof(int32_t), s));
    k_hc_table<<<grid_for(a.cap_blocks, 256), 256, 0, s>>>(a.gp, a.o_start, a.o_box, a.o_tab,
                                                           a.o_ntab);
    DM_LAUNCH_CHECK();
    a.use_o = 1;
    launches += 7;
  }
  int g2 = kSMs * 8;
  if (dim == 3) {
    k_star3_l2<<<g2, 32 * L2_WARPS, 0, s>>>(a);
    k_star3_l3<<<L3_BLOCKS, 32 * L3_WARPS, 0, s>>>(a);
  } else {
    k_star2_l2<<<g2, 32 * L2_WARPS, 0, s>>>(a);
    k_star2_l3<<<L3_BLOCKS, 32 * L3_WARPS, 0, s>>>(a);
  }
  DM_LAUNCH_CHECK();
  prof_mark(2, s);
  if (g_prof_on && g_prof_n < kProfMax) ++g_prof_n;
  note_launches(launches);
  return DM_OK;
}

}  // namespace dm

namespace dm {
// Debug aid (not part of the public ABI): run exhaustive face queries on the
// grid of the last dm_delaunay call.  faces: int32[m][3] (p, a, b) device;
// out: int32[m] winner (or -1).
__global__ void k_debug_gq(DTArgs A, const int32_t *faces, int m, int32_t *out) {
  const int lane = threadIdx.x & 31;
  const GridParams g = *A.gp;
  int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (w >= m) return;
  int ovf = 0;
  dmp::ExactScratch WS;
  int r = A.dim == 3 ? gq3(A, g, faces[3 * w], faces[3 * w + 1], faces[3 * w + 2], lane, ovf, &WS)
                     : gq2(A, g, faces[3 * w], faces[3 * w + 1], faces[3 * w + 2], lane, ovf, &WS);
  if (lane == 0) out[w] = r;
}
}  // namespace dm

extern "C" int dmdbg_face_query_mode(int32_t dim, const float *pts, int64_t n,
                                     void *ws, size_t ws_bytes, const int32_t *faces,
                                     int32_t m, int32_t *out, void *stream, int32_t mode);
extern "C" int dmdbg_face_query(int32_t dim, const float *pts, int64_t n,
                                void *ws, size_t ws_bytes, const int32_t *faces,
                                int32_t m, int32_t *out, void *stream) {
  return dmdbg_face_query_mode(dim, pts, n, ws, ws_bytes, faces, m, out, stream, 0);
}

// mode 1: exhaustive half-space scan for every face (ground truth, 3D);
// mode 2: hull scans through the hull candidates of the last dm_delaunay
// call on the same points and workspace (3D)
extern "C" int dmdbg_face_query_mode(int32_t dim, const float *pts, int64_t n,
                                     void *ws, size_t ws_bytes, const int32_t *faces,
                                     int32_t m, int32_t *out, void *stream, int32_t mode) {
  using namespace dm;
  Carve c(ws, ws_bytes);
  DTArgs a;
  memset(&a, 0, sizeof(a));
  carve_dt(c, a, dim, n);
  a.dim = dim;
  a.n = n;
  a.P = pts;
  a.dbg_vertex = -1;
  a.dbg_full = mode == 1;
  a.use_o = mode == 2 && dim == 3;
  k_debug_gq<<<(m + 3) / 4, 128, 0, (cudaStream_t)stream>>>(a, faces, m, out);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

namespace dm {
// Debug aid: device evaluation of orient3 (kind 0) / insph3_sos (kind 1) /
// the float orient filter alone (kind 2) on index tuples int32[m][5].
__global__ void k_debug_pred(const float *P, const int32_t *tup, int m, int kind,
                             int32_t *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  float x[5][3];
  for (int k = 0; k < 5; ++k) load_pt<3>(P, tup[5 * i + k], x[k]);
  int ovf = 0;
  dmp::ExactScratch WS;
  if (kind == 0) {
    out[i] = dmp::orient3(x[0], x[1], x[2], x[3], &WS);
  } else if (kind == 1) {
    out[i] = dmp::insph3_sos(x[0], x[1], x[2], x[3], x[4], &ovf, &WS);
  } else if (kind == 2) {
    float V[3], U[3], Y[3];
    for (int k = 0; k < 3; ++k) {
      V[k] = x[1][k] - x[0][k];
      U[k] = x[2][k] - x[0][k];
      Y[k] = x[3][k] - x[0][k];
    }
    out[i] = dmp::orient3_rel_filter<float>(V[0], V[1], V[2], U[0], U[1], U[2],
                                            Y[0], Y[1], Y[2], 16.0f * DMP_U32);
  } else if (kind == 3) {
    out[i] = dmp::orient3_slow(x[0], x[1], x[2], x[3], &WS);
  } else {
    out[i] = dmp::orient3_exact(x[0], x[1], x[2], x[3], &WS);
  }
}
}  // namespace dm

extern "C" int dmdbg_predicates(const float *pts, const int32_t *tup, int32_t m,
                                int32_t kind, int32_t *out, void *stream) {
  dm::k_debug_pred<<<(m + 127) / 128, 128, 0, (cudaStream_t)stream>>>(pts, tup, m, kind, out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

namespace dm {
// Debug aid: FP64 rounding behaviour of the device (op 0 add, 1 mul, 2 fma,
// 3 two_sum tail, 4 two_prod tail).
__global__ void k_debug_fp64(const double *a, const double *b, const double *c,
                             int m, int op, double *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double x, y;
  switch (op) {
    case 0: out[i] = __dadd_rn(a[i], b[i]); break;
    case 1: out[i] = __dmul_rn(a[i], b[i]); break;
    case 2: out[i] = fma(a[i], b[i], c[i]); break;
    case 3: dmp::two_sum(a[i], b[i], x, y); out[i] = y; break;
    case 4: dmp::two_prod(a[i], b[i], x, y); out[i] = y; break;
    case 5: out[i] = a[i] - b[i]; break;
  }
}
}  // namespace dm
extern "C" int dmdbg_fp64(const double *a, const double *b, const double *c,
                          int32_t m, int32_t op, double *out, void *stream) {
  dm::k_debug_fp64<<<(m + 127) / 128, 128, 0, (cudaStream_t)stream>>>(a, b, c, m, op, out);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Debug aid: copy the escalation list and seeds of the last dm_delaunay call.
extern "C" int dmdbg_escalations(int32_t dim, int64_t n, void *ws, size_t ws_bytes,
                                 int32_t *esc_out, int32_t *seed_out, void *stream) {
  using namespace dm;
  Carve c(ws, ws_bytes);
  DTArgs a;
  carve_dt(c, a, dim, n);
  cudaMemcpyAsync(esc_out, a.esc, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  cudaMemcpyAsync(seed_out, a.esc_seed, sizeof(int4) * n, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Debug aid: copy the hull-candidate flags of the last 3D dm_delaunay call.
extern "C" int dmdbg_hull_candidates(int64_t n, void *ws, size_t ws_bytes, uint8_t *out,
                                     void *stream) {
  using namespace dm;
  Carve c(ws, ws_bytes);
  DTArgs a;
  carve_dt(c, a, 3, n);
  cudaMemcpyAsync(out, a.hullc, n, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// Debug aid: make the next dm_delaunay calls dump the level-1 state of one
// vertex into dbg (device, >= 8 + 128 + 3*128 ints); vertex -1 disables.
// The dumps are compiled in only with -DDM_DEBUG_VERTEX; otherwise the call
// returns DM_ERR_ARG.
extern "C" int dmdbg_watch_vertex(int32_t vertex, int32_t *dbg) {
#ifdef DM_DEBUG_VERTEX
  dm::g_dbg_vertex = vertex;
  dm::g_dbg = dbg;
  return 0;
#else
  (void)vertex;
  (void)dbg;
  return DM_ERR_ARG;
#endif
}

// Timing of the star kernels of the dm_delaunay calls made while enabled:
// dmprof_enable(1) resets and starts; dmprof_read synchronises the events and
// returns the summed milliseconds of level 1 and level 2 and the call count.
extern "C" int dmprof_enable(int32_t on) {
  dm::g_prof_on = on != 0;
  if (on) dm::g_prof_n = 0;
  return 0;
}
extern "C" int dmprof_read(double *ms_l1, double *ms_l2, int32_t *calls) {
  double a = 0, b = 0;
  for (int i = 0; i < dm::g_prof_n; ++i) {
    float t1 = 0, t2 = 0;
    cudaEventSynchronize(dm::g_prof_ev[i][2]);
    cudaEventElapsedTime(&t1, dm::g_prof_ev[i][0], dm::g_prof_ev[i][1]);
    cudaEventElapsedTime(&t2, dm::g_prof_ev[i][1], dm::g_prof_ev[i][2]);
    a += t1;
    b += t2;
  }
  *ms_l1 = a;
  *ms_l2 = b;
  *calls = dm::g_prof_n;
  return 0;
}
// number of kernels libdmgb.so has launched in this process
extern "C" int64_t dmprof_launches(void) { return dm::g_launches; }

// Debug aid: read and reset the slow-path counters of the Delaunay kernels.
extern "C" int dmprof_slow_counters(unsigned long long *out8) {
  cudaMemcpyFromSymbol(out8, dmp::g_slow, sizeof(unsigned long long) * 8);
  unsigned long long z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaMemcpyToSymbol(dmp::g_slow, z, sizeof(z));
  return 0;
}

// Debug aid: copy level-2 statistics of the last dm_delaunay (stars < 2^17,
// 8 values each); returns 0 when the statistics are not compiled in.
extern "C" int dmprof_l1_stats(unsigned long long *out8) {
#ifdef DM_L2_STATS
  cudaMemcpyFromSymbol(out8, dm::g_l1s, sizeof(unsigned long long) * 16);
  unsigned long long z[16] = {};
  cudaMemcpyToSymbol(dm::g_l1s, z, sizeof(z));
  return 1;
#else
  (void)out8;
  return 0;
#endif
}
extern "C" int dmprof_l2_stats(unsigned long long *out, int64_t nstars) {
#ifdef DM_L2_STATS
  if (nstars > dm::kL2StatStars) nstars = dm::kL2StatStars;
  cudaMemcpyFromSymbol(out, dm::g_l2s, sizeof(unsigned long long) * 8 * nstars);
  return 1;
#else
  (void)out;
  (void)nstars;
  return 0;
#endif
}
