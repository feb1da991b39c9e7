// Isosurface signed distance of a gridded field (the salt-body domain of a
// velocity model).  The surface is the zero set of the piecewise-linear
// interpolant of f = B - level over the Kuhn (Freudenthal) split of every
// grid cell into 6 tetrahedra along its main diagonal; it is extracted as
// triangles by marching tetrahedra.  The exact signed distance of a query
// point is the distance to the nearest triangle, negative where the
// interpolant is >= level (inside).
//
// Layout (device):
//   field  float[n0][n1][n2], C order; node (i,j,k) sits at origin + (i,j,k)*h
//   tris   float4[ntri][3]: the three vertices (x, y, z, 0)
//   buckets: a uniform grid of nb0*nb1*nb2 boxes of bsize; each triangle is
//   listed once, in the box of its centroid (CSR bstart/btri, ids ascending),
//   and rho bounds how far a triangle reaches out of its box.  bring[b] is
//   the Chebyshev ring of the nearest non-empty box, so a query starts its
//   ring search there.
#include <cstring>

#include "dm_common.cuh"

namespace dm {

// corners of a grid cell: bit 0 -> +1 along axis 0, bit 1 -> axis 1, bit 2
// -> axis 2.  Tetrahedron p of the Kuhn split is the chain 0 -> 1<<a ->
// 1<<a | 1<<b -> 7 for the axis permutation (a, b, c) = kPerm[p].
__constant__ int kKuhn[6][4] = {{0, 1, 3, 7}, {0, 1, 5, 7}, {0, 2, 3, 7},
                                {0, 2, 6, 7}, {0, 4, 5, 7}, {0, 4, 6, 7}};

__device__ __forceinline__ int64_t node_id(const int32_t *n, int i, int j, int k) {
  return ((int64_t)i * n[1] + j) * n[2] + k;
}

__device__ __forceinline__ int tet_triangles(int s) {
  return (s == 1 || s == 3) ? 1 : (s == 2 ? 2 : 0);
}

// the 8 corner values of cell (i, j, k) minus level
__device__ __forceinline__ void cell_values(const dm_iso &I, int i, int j, int k,
                                            float *fv) {
#pragma unroll
  for (int q = 0; q < 8; ++q)
    fv[q] = __ldg(I.field + node_id(I.n, i + (q & 1), j + ((q >> 1) & 1),
                                    k + ((q >> 2) & 1))) - I.level;
}

__device__ __forceinline__ int cell_triangles(const float *fv) {
  int cnt = 0;
#pragma unroll
  for (int p = 0; p < 6; ++p) {
    int s = 0;
#pragma unroll
    for (int v = 0; v < 4; ++v) s += fv[kKuhn[p][v]] >= 0.f;
    cnt += tet_triangles(s);
  }
  return cnt;
}

// point where the interpolant crosses zero on the edge from corner u to
// corner v (bits(u) a subset of bits(v): the edge is always evaluated from
// its lower node, so the cells sharing it compute the same point)
__device__ __forceinline__ float4 edge_point(const dm_iso &I, int i, int j, int k,
                                             const float *fv, int u, int v) {
  float t = fv[u] / (fv[u] - fv[v]);
  float xu[3] = {I.origin[0] + (float)(i + (u & 1)) * I.h[0],
                 I.origin[1] + (float)(j + ((u >> 1) & 1)) * I.h[1],
                 I.origin[2] + (float)(k + ((u >> 2) & 1)) * I.h[2]};
  float xv[3] = {I.origin[0] + (float)(i + (v & 1)) * I.h[0],
                 I.origin[1] + (float)(j + ((v >> 1) & 1)) * I.h[1],
                 I.origin[2] + (float)(k + ((v >> 2) & 1)) * I.h[2]};
  return make_float4(xu[0] + t * (xv[0] - xu[0]), xu[1] + t * (xv[1] - xu[1]),
                     xu[2] + t * (xv[2] - xu[2]), 0.f);
}

__device__ __forceinline__ float4 tet_edge(const dm_iso &I, int i, int j, int k,
                                           const float *fv, const int *tv, int a, int b) {
  int u = tv[a], v = tv[b];
  return u < v ? edge_point(I, i, j, k, fv, u, v) : edge_point(I, i, j, k, fv, v, u);
}

// triangles of cell (i, j, k) in a fixed order (tetrahedron, then case)
__device__ int emit_cell(const dm_iso &I, int i, int j, int k, const float *fv,
                         float4 *out) {
  int m = 0;
  for (int p = 0; p < 6; ++p) {
    int tv[4] = {kKuhn[p][0], kKuhn[p][1], kKuhn[p][2], kKuhn[p][3]};
    int in[4], nin = 0, outv[4], nout = 0;
    for (int v = 0; v < 4; ++v) {
      if (fv[tv[v]] >= 0.f) in[nin++] = v; else outv[nout++] = v;
    }
    if (nin == 1 || nin == 3) {
      int lone = nin == 1 ? in[0] : outv[0];
      int o[3], no = 0;
      for (int v = 0; v < 4; ++v)
        if (v != lone) o[no++] = v;
      out[3 * m] = tet_edge(I, i, j, k, fv, tv, lone, o[0]);
      out[3 * m + 1] = tet_edge(I, i, j, k, fv, tv, lone, o[1]);
      out[3 * m + 2] = tet_edge(I, i, j, k, fv, tv, lone, o[2]);
      ++m;
    } else if (nin == 2) {
      // quad a-c, a-d, b-d, b-c (a, b inside; c, d outside)
      float4 ac = tet_edge(I, i, j, k, fv, tv, in[0], outv[0]);
      float4 ad = tet_edge(I, i, j, k, fv, tv, in[0], outv[1]);
      float4 bd = tet_edge(I, i, j, k, fv, tv, in[1], outv[1]);
      float4 bc = tet_edge(I, i, j, k, fv, tv, in[1], outv[0]);
      out[3 * m] = ac;
      out[3 * m + 1] = ad;
      out[3 * m + 2] = bd;
      out[3 * m + 3] = ac;
      out[3 * m + 4] = bd;
      out[3 * m + 5] = bc;
      m += 2;
    }
  }
  return m;
}

// one warp per row of cells (i, j, *): triangle count of the row
__global__ void k_iso_count(dm_iso I, int32_t *rowcnt) {
  const int lane = threadIdx.x & 31;
  const int64_t nrow = (int64_t)(I.n[0] - 1) * (I.n[1] - 1);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < nrow;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int i = (int)(r / (I.n[1] - 1)), j = (int)(r % (I.n[1] - 1));
    int cnt = 0;
    for (int k = lane; k < I.n[2] - 1; k += 32) {
      float fv[8];
      cell_values(I, i, j, k, fv);
      cnt += cell_triangles(fv);
    }
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) rowcnt[r] = cnt;
  }
}

// same traversal; the row's triangles go to rowstart[r].. in cell order
__global__ void k_iso_emit(dm_iso I, const int32_t *rowstart, float4 *tris) {
  const int lane = threadIdx.x & 31;
  const int64_t nrow = (int64_t)(I.n[0] - 1) * (I.n[1] - 1);
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < nrow;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int i = (int)(r / (I.n[1] - 1)), j = (int)(r % (I.n[1] - 1));
    int64_t base = rowstart[r];
    for (int k0 = 0; k0 < I.n[2] - 1; k0 += 32) {
      const int k = k0 + lane;
      float fv[8];
      int cnt = 0;
      if (k < I.n[2] - 1) {
        cell_values(I, i, j, k, fv);
        cnt = cell_triangles(fv);
      }
      int incl = cnt;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (cnt) emit_cell(I, i, j, k, fv, tris + 3 * (base + incl - cnt));
      base += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

__device__ __forceinline__ int bucket_of(const dm_iso &I, float x, int d) {
  int b = (int)floorf((x - I.origin[d]) / I.bsize[d]);
  return min(max(b, 0), I.nb[d] - 1);
}

__global__ void k_iso_bucket_count(dm_iso I, const float4 *tris, int64_t ntri,
                                   int32_t *cnt, int32_t *key, int32_t *slot,
                                   int *rho_bits) {
  float rmax = 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntri;
       t += (int64_t)gridDim.x * blockDim.x) {
    float4 a = tris[3 * t], b = tris[3 * t + 1], c = tris[3 * t + 2];
    float cx = (a.x + b.x + c.x) / 3.f, cy = (a.y + b.y + c.y) / 3.f,
          cz = (a.z + b.z + c.z) / 3.f;
    int bb = (bucket_of(I, cx, 0) * I.nb[1] + bucket_of(I, cy, 1)) * I.nb[2] +
             bucket_of(I, cz, 2);
    key[t] = bb;
    slot[t] = atomicAdd(&cnt[bb], 1);
    float4 v[3] = {a, b, c};
    for (int q = 0; q < 3; ++q) {
      float dx = v[q].x - cx, dy = v[q].y - cy, dz = v[q].z - cz;
      rmax = fmaxf(rmax, sqrtf(dx * dx + dy * dy + dz * dz));
    }
  }
  for (int o = 16; o; o >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
  if ((threadIdx.x & 31) == 0) atomicMax(rho_bits, __float_as_int(rmax));
}

__global__ void k_iso_bucket_scatter(int64_t ntri, const int32_t *key, const int32_t *slot,
                                     const int32_t *start, int32_t *btri) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntri;
       t += (int64_t)gridDim.x * blockDim.x)
    btri[start[key[t]] + slot[t]] = (int32_t)t;
}

// ids of each box in ascending order (deterministic nearest-triangle ties)
__global__ void k_iso_bucket_sort(int64_t nbk, const int32_t *start, int32_t *btri,
                                  int32_t *ring) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbk;
       b += (int64_t)gridDim.x * blockDim.x) {
    int s = start[b], e = start[b + 1];
    for (int i = s + 1; i < e; ++i) {
      int x = btri[i], j = i - 1;
      while (j >= s && btri[j] > x) {
        btri[j + 1] = btri[j];
        --j;
      }
      btri[j + 1] = x;
    }
    ring[b] = e > s ? 0 : (1 << 30);
  }
}

// one Jacobi pass of the Chebyshev distance transform of the non-empty
// cells of a grid of nb.x x nb.y x nb.z
__global__ void k_iso_ring_pass(int3 nb, const int32_t *in, int32_t *out) {
  const int64_t nbk = (int64_t)nb.x * nb.y * nb.z;
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbk;
       b += (int64_t)gridDim.x * blockDim.x) {
    int z = (int)(b % nb.z), y = (int)((b / nb.z) % nb.y), x = (int)(b / ((int64_t)nb.z * nb.y));
    int best = in[b];
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          int X = x + dx, Y = y + dy, Z = z + dz;
          if (X < 0 || Y < 0 || Z < 0 || X >= nb.x || Y >= nb.y || Z >= nb.z) continue;
          int v = in[((int64_t)X * nb.y + Y) * nb.z + Z];
          if (v < (1 << 30)) best = min(best, v + 1);
        }
    out[b] = best;
  }
}

// coarse block occupancy (triangles in the block's boxes) and the ring seed
__global__ void k_iso_coarse(dm_iso I, const int32_t *bstart, int32_t *cocc, int32_t *cring) {
  const int64_t ncb = (int64_t)I.ncb[0] * I.ncb[1] * I.ncb[2];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncb;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int cz = (int)(c % I.ncb[2]), cy = (int)((c / I.ncb[2]) % I.ncb[1]),
              cx = (int)(c / ((int64_t)I.ncb[2] * I.ncb[1]));
    int tot = 0;
    for (int x = cx * I.cf; x < min(I.nb[0], (cx + 1) * I.cf); ++x)
      for (int y = cy * I.cf; y < min(I.nb[1], (cy + 1) * I.cf); ++y) {
        const int64_t b0 = ((int64_t)x * I.nb[1] + y) * I.nb[2];
        const int z0 = cz * I.cf, z1 = min(I.nb[2], (cz + 1) * I.cf);
        tot += bstart[b0 + z1] - bstart[b0 + z0];
      }
    cocc[c] = tot;
    cring[c] = tot ? 0 : (1 << 30);
  }
}

// ---------------------------------------------------------------------------
// queries

// Closest point of triangle (a, b, c) to p by the Voronoi-region tests of
// Ericson, "Real-Time Collision Detection" (2005), section 5.1.5; degenerate
// (zero-area) triangles fall back to their edges.
__device__ __forceinline__ float3 sub3(float3 a, float3 b) {
  return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float dot3(float3 a, float3 b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float3 madd3(float3 a, float3 d, float t) {
  return make_float3(a.x + t * d.x, a.y + t * d.y, a.z + t * d.z);
}
__device__ __forceinline__ float3 closest_on_segment(float3 p, float3 a, float3 b) {
  float3 ab = sub3(b, a);
  float l2 = dot3(ab, ab);
  float t = l2 > 0.f ? fminf(fmaxf(dot3(sub3(p, a), ab) / l2, 0.f), 1.f) : 0.f;
  return madd3(a, ab, t);
}
__device__ float3 closest_on_triangle(float3 p, float3 a, float3 b, float3 c) {
  float3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
  float d1 = dot3(ab, ap), d2 = dot3(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) return a;
  float3 bp = sub3(p, b);
  float d3 = dot3(ab, bp), d4 = dot3(ac, bp);
  if (d3 >= 0.f && d4 <= d3) return b;
  float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return madd3(a, ab, d1 / (d1 - d3));
  float3 cp = sub3(p, c);
  float d5 = dot3(ab, cp), d6 = dot3(ac, cp);
  if (d6 >= 0.f && d5 <= d6) return c;
  float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return madd3(a, ac, d2 / (d2 - d6));
  float va = d3 * d6 - d5 * d4;
  if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f)
    return madd3(b, sub3(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6)));
  float den = va + vb + vc;
  if (!(den > 0.f)) {  // degenerate: nearest of the three edges
    float3 q0 = closest_on_segment(p, a, b), q1 = closest_on_segment(p, b, c),
           q2 = closest_on_segment(p, a, c);
    float e0 = dot3(sub3(p, q0), sub3(p, q0)), e1 = dot3(sub3(p, q1), sub3(p, q1)),
          e2 = dot3(sub3(p, q2), sub3(p, q2));
    return e0 <= e1 ? (e0 <= e2 ? q0 : q2) : (e1 <= e2 ? q1 : q2);
  }
  float v = vb / den, w = vc / den;
  return make_float3(a.x + ab.x * v + ac.x * w, a.y + ab.y * v + ac.y * w,
                     a.z + ab.z * v + ac.z * w);
}

// value of the piecewise-linear interpolant (minus level) at x, and its
// gradient; points outside the node box are outside the body (-1)
__device__ float iso_field(const dm_iso &I, float3 x, float3 *grad) {
  float xs[3] = {x.x, x.y, x.z};
  int c[3];
  float u[3];
  for (int d = 0; d < 3; ++d) {
    float t = (xs[d] - I.origin[d]) / I.h[d];
    if (!(t >= 0.f && t <= (float)(I.n[d] - 1))) {
      if (grad) *grad = make_float3(0.f, 0.f, 0.f);
      return -1.f;
    }
    c[d] = min((int)floorf(t), I.n[d] - 2);
    u[d] = t - (float)c[d];
  }
  // axes by decreasing local coordinate: the Kuhn tetrahedron holding x
  int a0 = 0, a1 = 1, a2 = 2, s;
  if (u[a0] < u[a1]) { s = a0; a0 = a1; a1 = s; }
  if (u[a1] < u[a2]) { s = a1; a1 = a2; a2 = s; }
  if (u[a0] < u[a1]) { s = a0; a0 = a1; a1 = s; }
  int q1 = 1 << a0, q2 = q1 | (1 << a1);
  auto val = [&](int q) {
    return __ldg(I.field + node_id(I.n, c[0] + (q & 1), c[1] + ((q >> 1) & 1),
                                   c[2] + ((q >> 2) & 1))) - I.level;
  };
  float f0 = val(0), f1 = val(q1), f2 = val(q2), f3 = val(7);
  if (grad) {
    float g[3];
    g[a0] = (f1 - f0) / I.h[a0];
    g[a1] = (f2 - f1) / I.h[a1];
    g[a2] = (f3 - f2) / I.h[a2];
    *grad = make_float3(g[0], g[1], g[2]);
  }
  return f0 + u[a0] * (f1 - f0) + u[a1] * (f2 - f1) + u[a2] * (f3 - f2);
}

__device__ __forceinline__ float box_dist2(const dm_iso &I, float3 x, int bx, int by, int bz) {
  float lo[3] = {I.origin[0] + bx * I.bsize[0], I.origin[1] + by * I.bsize[1],
                 I.origin[2] + bz * I.bsize[2]};
  float xs[3] = {x.x, x.y, x.z}, d2 = 0.f;
  for (int d = 0; d < 3; ++d) {
    float e = fmaxf(fmaxf(lo[d] - xs[d], xs[d] - (lo[d] + I.bsize[d])), 0.f);
    d2 += e * e;
  }
  return d2;
}

__device__ __forceinline__ void scan_box(const dm_iso &I, float3 x, int64_t b, float &best2,
                                         float3 &bestp) {
  const int s = __ldg(I.bstart + b), e = __ldg(I.bstart + b + 1);
  for (int q = s; q < e; ++q) {
    const int t = __ldg(I.btri + q);
    const float4 A = __ldg(reinterpret_cast<const float4 *>(I.tris) + 3 * t);
    const float4 B = __ldg(reinterpret_cast<const float4 *>(I.tris) + 3 * t + 1);
    const float4 C = __ldg(reinterpret_cast<const float4 *>(I.tris) + 3 * t + 2);
    float3 cp = closest_on_triangle(x, make_float3(A.x, A.y, A.z), make_float3(B.x, B.y, B.z),
                                    make_float3(C.x, C.y, C.z));
    float3 dv = sub3(x, cp);
    float d2 = dot3(dv, dv);
    if (d2 < best2) {
      best2 = d2;
      bestp = cp;
    }
  }
}

// squared distance from x to block (cx, cy, cz) of cf^3 boxes (a lower bound
// for a block cut short at the grid's end)
__device__ __forceinline__ float block_dist2(const dm_iso &I, float3 x, int cx, int cy, int cz) {
  float lo[3] = {I.origin[0] + cx * I.cf * I.bsize[0], I.origin[1] + cy * I.cf * I.bsize[1],
                 I.origin[2] + cz * I.cf * I.bsize[2]};
  float xs[3] = {x.x, x.y, x.z}, d2 = 0.f;
  for (int d = 0; d < 3; ++d) {
    float e = fmaxf(fmaxf(lo[d] - xs[d], xs[d] - (lo[d] + I.cf * I.bsize[d])), 0.f);
    d2 += e * e;
  }
  return d2;
}

// signed distance and (optionally) its gradient at x: first the 27 boxes
// around x (for a point near the surface they hold the nearest triangle, so
// the bound is tight from the start), then rings of blocks around x
// (starting at the block ring bound), descending into the boxes of blocks
// that hold triangles and may hold a nearer one
__device__ float iso_distance(const dm_iso &I, float3 x, float3 *grad) {
  const int bx = bucket_of(I, x.x, 0), by = bucket_of(I, x.y, 1), bz = bucket_of(I, x.z, 2);
  const int cx = bx / I.cf, cy = by / I.cf, cz = bz / I.cf;
  const int r0 = __ldg(I.cring + ((int64_t)cx * I.ncb[1] + cy) * I.ncb[2] + cz);
  const int rmax = max(max(max(cx, I.ncb[0] - 1 - cx), max(cy, I.ncb[1] - 1 - cy)),
                       max(cz, I.ncb[2] - 1 - cz));
  const float cmin = I.cf * fminf(fminf(I.bsize[0], I.bsize[1]), I.bsize[2]);
  float best2 = INFINITY;
  float3 bestp = x;
  const bool near = __ldg(I.bring + ((int64_t)bx * I.nb[1] + by) * I.nb[2] + bz) <= 1;
  if (near) {
    for (int q = 0; q < 27; ++q) {  // the box of x first
      const int k = (q + 13) % 27;
      const int fx = bx + k / 9 - 1, fy = by + (k / 3) % 3 - 1, fz = bz + k % 3 - 1;
      if (fx < 0 || fy < 0 || fz < 0 || fx >= I.nb[0] || fy >= I.nb[1] || fz >= I.nb[2])
        continue;
      const float fd = sqrtf(box_dist2(I, x, fx, fy, fz)) - I.rho;
      if (fd > 0.f && fd * fd >= best2) continue;
      scan_box(I, x, ((int64_t)fx * I.nb[1] + fy) * I.nb[2] + fz, best2, bestp);
    }
  }
  for (int r = min(r0, rmax); r <= rmax; ++r) {
    const float lower = (float)(r - 1) * cmin - I.rho;
    if (lower > 0.f && lower * lower >= best2) break;
    for (int dx = -r; dx <= r; ++dx) {
      const int X = cx + dx;
      if (X < 0 || X >= I.ncb[0]) continue;
      for (int dy = -r; dy <= r; ++dy) {
        const int Y = cy + dy;
        if (Y < 0 || Y >= I.ncb[1]) continue;
        const bool shell = (dx == -r || dx == r || dy == -r || dy == r);
        const int step = shell ? 1 : max(2 * r, 1);
        for (int dz = -r; dz <= r; dz += step) {
          const int Z = cz + dz;
          if (Z < 0 || Z >= I.ncb[2]) continue;
          if (__ldg(I.cocc + ((int64_t)X * I.ncb[1] + Y) * I.ncb[2] + Z) == 0) continue;
          float bd = sqrtf(block_dist2(I, x, X, Y, Z)) - I.rho;
          if (bd > 0.f && bd * bd >= best2) continue;
          for (int fx = X * I.cf; fx < min(I.nb[0], (X + 1) * I.cf); ++fx)
            for (int fy = Y * I.cf; fy < min(I.nb[1], (Y + 1) * I.cf); ++fy)
              for (int fz = Z * I.cf; fz < min(I.nb[2], (Z + 1) * I.cf); ++fz) {
                if (near && abs(fx - bx) <= 1 && abs(fy - by) <= 1 && abs(fz - bz) <= 1)
                  continue;  // scanned above
                float fd = sqrtf(box_dist2(I, x, fx, fy, fz)) - I.rho;
                if (fd > 0.f && fd * fd >= best2) continue;
                scan_box(I, x, ((int64_t)fx * I.nb[1] + fy) * I.nb[2] + fz, best2, bestp);
              }
        }
      }
    }
  }
  float3 gf;
  const float f = iso_field(I, x, grad ? &gf : nullptr);
  const float sgn = f >= 0.f ? -1.f : 1.f;
  const float dist = sqrtf(best2);
  if (grad) {
    if (dist > 0.f) {
      float3 dv = sub3(x, bestp);
      *grad = make_float3(sgn * dv.x / dist, sgn * dv.y / dist, sgn * dv.z / dist);
    } else {  // on the surface: the interpolant's outward normal
      float gl = sqrtf(dot3(gf, gf));
      *grad = gl > 0.f ? make_float3(-gf.x / gl, -gf.y / gl, -gf.z / gl)
                       : make_float3(0.f, 0.f, 0.f);
    }
  }
  return sgn * dist;
}

// points float[..][stride]; idx (optional) selects which, count_dev
// (optional, device) overrides n
__global__ void k_iso_eval(dm_iso I, const float *pts, int stride, int64_t n,
                           const int32_t *idx, const int64_t *count_dev, float *d,
                           float *grad) {
  const int64_t m = count_dev ? *count_dev : n;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx ? idx[q] : q;
    const float *x = pts + i * stride;
    float3 g;
    float v = iso_distance(I, make_float3(x[0], x[1], x[2]), grad ? &g : nullptr);
    d[i] = v;
    if (grad) {
      grad[4 * i] = g.x;
      grad[4 * i + 1] = g.y;
      grad[4 * i + 2] = g.z;
      grad[4 * i + 3] = 0.f;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
void note_launches(int k);

static bool iso_grid_ok(const dm_iso *I) {
  return I && I->field && I->n[0] >= 2 && I->n[1] >= 2 && I->n[2] >= 2 && I->h[0] > 0 &&
         I->h[1] > 0 && I->h[2] > 0;
}

int iso_count(const dm_iso *I, int32_t *rowstart, int32_t *tmp, int64_t *ntri,
              cudaStream_t s) {
  DM_ARG_CHECK(iso_grid_ok(I) && rowstart && tmp && ntri, "iso grid");
  const int64_t nrow = (int64_t)(I->n[0] - 1) * (I->n[1] - 1);
  k_iso_count<<<grid_for(nrow * 32, 256), 256, 0, s>>>(*I, rowstart + nrow + 1);
  int rc = exclusive_scan_i32(rowstart + nrow + 1, rowstart, nrow, tmp, s);
  if (rc) return rc;
  note_launches(1);
  DM_LAUNCH_CHECK();
  int32_t total = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&total, rowstart + nrow, sizeof(int32_t),
                              cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  *ntri = total;
  return DM_OK;
}

int iso_emit(const dm_iso *I, const int32_t *rowstart, float *tris, cudaStream_t s) {
  DM_ARG_CHECK(iso_grid_ok(I) && rowstart && tris, "iso grid");
  const int64_t nrow = (int64_t)(I->n[0] - 1) * (I->n[1] - 1);
  k_iso_emit<<<grid_for(nrow * 32, 256), 256, 0, s>>>(*I, rowstart,
                                                      reinterpret_cast<float4 *>(tris));
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

size_t iso_bucket_workspace(int64_t ntri, int64_t nbk) {
  Carve c(nullptr, 0);
  c.take<int32_t>(nbk);                  // counts
  c.take<int32_t>(ntri);                 // key
  c.take<int32_t>(ntri);                 // slot
  c.take<int32_t>(nbk);                  // ring ping-pong
  c.take<int32_t>(scan_tmp_elems(nbk));  // scan
  c.take<int32_t>(1);                    // rho
  return c.used + 256;
}

int iso_bucket(dm_iso *I, int32_t *bstart, int32_t *btri, int32_t *bring, int32_t *coarse,
               void *ws, size_t ws_bytes, cudaStream_t s) {
  DM_ARG_CHECK(iso_grid_ok(I) && I->tris && I->ntri >= 0 && bstart && btri && bring && coarse,
               "iso buckets");
  DM_ARG_CHECK(I->nb[0] > 0 && I->nb[1] > 0 && I->nb[2] > 0 && I->bsize[0] > 0 &&
                   I->bsize[1] > 0 && I->bsize[2] > 0, "bucket grid");
  DM_ARG_CHECK(I->cf >= 1 && I->ncb[0] == (I->nb[0] + I->cf - 1) / I->cf &&
                   I->ncb[1] == (I->nb[1] + I->cf - 1) / I->cf &&
                   I->ncb[2] == (I->nb[2] + I->cf - 1) / I->cf, "coarse grid");
  const int64_t ncb = (int64_t)I->ncb[0] * I->ncb[1] * I->ncb[2];
  const int64_t nbk = (int64_t)I->nb[0] * I->nb[1] * I->nb[2];
  Carve c(ws, ws_bytes);
  int32_t *cnt = c.take<int32_t>(nbk), *key = c.take<int32_t>(I->ntri),
          *slot = c.take<int32_t>(I->ntri), *ring2 = c.take<int32_t>(nbk),
          *tmp = c.take<int32_t>(scan_tmp_elems(nbk)), *rho = c.take<int32_t>(1);
  if (!c.ok() || !ws) {
    set_error("iso_bucket: workspace %zu < required %zu", ws_bytes, c.used);
    return DM_ERR_WORKSPACE;
  }
  DM_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * nbk, s));
  DM_CUDA_TRY(cudaMemsetAsync(rho, 0, sizeof(int32_t), s));
  const float4 *T = reinterpret_cast<const float4 *>(I->tris);
  k_iso_bucket_count<<<grid_for(I->ntri, 256), 256, 0, s>>>(*I, T, I->ntri, cnt, key, slot, rho);
  int rc = exclusive_scan_i32(cnt, bstart, nbk, tmp, s);
  if (rc) return rc;
  k_iso_bucket_scatter<<<grid_for(I->ntri, 256), 256, 0, s>>>(I->ntri, key, slot, bstart, btri);
  k_iso_bucket_sort<<<grid_for(nbk, 128), 128, 0, s>>>(nbk, bstart, btri, bring);
  I->bstart = bstart;
  I->btri = btri;
  const int passes = max(max(I->nb[0], I->nb[1]), I->nb[2]);
  int32_t *a = bring, *b = ring2;
  for (int p = 0; p < passes; ++p) {
    k_iso_ring_pass<<<grid_for(nbk, 256), 256, 0, s>>>(make_int3(I->nb[0], I->nb[1], I->nb[2]),
                                                       a, b);
    int32_t *t = a;
    a = b;
    b = t;
  }
  if (a != bring)
    DM_CUDA_TRY(cudaMemcpyAsync(bring, a, sizeof(int32_t) * nbk, cudaMemcpyDeviceToDevice, s));
  // coarse level: occupancy, then its ring transform (ping-pong through ring2)
  int32_t *cocc = coarse, *cring = coarse + ncb;
  k_iso_coarse<<<grid_for(ncb, 128), 128, 0, s>>>(*I, bstart, cocc, cring);
  const int cpasses = max(max(I->ncb[0], I->ncb[1]), I->ncb[2]);
  a = cring;
  b = ring2;
  for (int p = 0; p < cpasses; ++p) {
    k_iso_ring_pass<<<grid_for(ncb, 256), 256, 0, s>>>(
        make_int3(I->ncb[0], I->ncb[1], I->ncb[2]), a, b);
    int32_t *t = a;
    a = b;
    b = t;
  }
  if (a != cring)
    DM_CUDA_TRY(cudaMemcpyAsync(cring, a, sizeof(int32_t) * ncb, cudaMemcpyDeviceToDevice, s));
  I->cocc = cocc;
  I->cring = cring;
  note_launches(5 + passes + cpasses);
  DM_LAUNCH_CHECK();
  int rho_bits = 0;
  DM_CUDA_TRY(cudaMemcpyAsync(&rho_bits, rho, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  DM_CUDA_TRY(cudaStreamSynchronize(s));
  float r;
  memcpy(&r, &rho_bits, sizeof(float));
  // a little slack for the rounding of centroids and box bounds
  I->rho = r * 1.0001f + 1e-4f * fmaxf(fmaxf(I->bsize[0], I->bsize[1]), I->bsize[2]);
  I->bring = bring;
  return DM_OK;
}

int iso_eval(const dm_iso *I, const float *pts, int stride, int64_t n, const int32_t *idx,
             const int64_t *count_dev, float *d, float *grad, cudaStream_t s) {
  DM_ARG_CHECK(iso_grid_ok(I) && I->tris && I->bstart && I->btri && I->bring && I->cocc &&
                   I->cring && I->cf >= 1, "iso sdf");
  DM_ARG_CHECK(pts && d && n >= 0 && stride >= 3, "points");
  if (n == 0 && !count_dev) return DM_OK;
  k_iso_eval<<<grid_for(n, 128, kSMs * 32), 128, 0, s>>>(*I, pts, stride, n, idx, count_dev,
                                                          d, grad);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

// ---------------------------------------------------------------------------
// DistMesh steps on batched SDF values

template <int NV>
__global__ void k_filter_by_value(const int32_t *cells, int64_t cap, const float *d,
                                  float geps, int32_t *out, int64_t *counters) {
  const int64_t nc = min(counters[DM_CNT_CELLS], cap);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c0 = blockIdx.x * (int64_t)blockDim.x; c0 < nc; c0 += stride) {
    const int64_t c = c0 + threadIdx.x;
    const bool keep = c < nc && d[c] < -geps;
    const int64_t k = warp_append(&counters[DM_CNT_KEPT], keep);
    if (keep)
      for (int j = 0; j < NV; ++j) out[NV * k + j] = cells[NV * c + j];
  }
}

__device__ __forceinline__ float round_to_grid(float x, int e) {
  return e < -200 ? x : ldexpf(rintf(ldexpf(x, -e)), e);
}

template <int DIM>
__global__ void k_project_by_value(float *P, int64_t n, const float *d, const float *grad,
                                   int grid_exp) {
  constexpr int W = DIM == 3 ? 4 : 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float di = d[i];
    if (!(di > 0.f)) continue;
    for (int j = 0; j < DIM; ++j)
      P[W * i + j] = round_to_grid(P[W * i + j] - di * grad[4 * i + j], grid_exp);
  }
}

template <int DIM>
__global__ void k_newton_by_value(float *P, const int32_t *idx, int64_t m, const float *d,
                                  const float *grad, float alpha, int grid_exp) {
  constexpr int W = DIM == 3 ? 4 : 2;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[q];
    const float di = d[i];
    for (int j = 0; j < DIM; ++j)
      P[W * i + j] = round_to_grid(P[W * i + j] - alpha * di * grad[4 * i + j], grid_exp);
  }
}

__global__ void k_select_band(const float *d, int64_t n, float lo, float hi, int32_t *idx,
                              int64_t *count) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = blockIdx.x * (int64_t)blockDim.x; i0 < n; i0 += stride) {
    const int64_t i = i0 + threadIdx.x;
    const bool in = i < n && d[i] > lo && d[i] < hi;
    const int64_t k = warp_append(count, in);
    if (in) idx[k] = (int32_t)i;
  }
}

int filter_by_value(int dim, const int32_t *cells, int64_t cap, const float *d, float geps,
                    int32_t *out, int64_t *counters, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(cells && d && out && counters, "pointers");
  DM_CUDA_TRY(cudaMemsetAsync(counters + DM_CNT_KEPT, 0, sizeof(int64_t), s));
  if (dim == 3)
    k_filter_by_value<4><<<grid_for(cap, 256), 256, 0, s>>>(cells, cap, d, geps, out, counters);
  else
    k_filter_by_value<3><<<grid_for(cap, 256), 256, 0, s>>>(cells, cap, d, geps, out, counters);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int project_by_value(int dim, float *P, int64_t n, const float *d, const float *grad,
                     int grid_exp, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(P && d && grad, "pointers");
  if (n == 0) return DM_OK;
  if (dim == 3)
    k_project_by_value<3><<<grid_for(n, 256), 256, 0, s>>>(P, n, d, grad, grid_exp);
  else
    k_project_by_value<2><<<grid_for(n, 256), 256, 0, s>>>(P, n, d, grad, grid_exp);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int newton_by_value(int dim, float *P, const int32_t *idx, int64_t m, const float *d,
                    const float *grad, float alpha, int grid_exp, cudaStream_t s) {
  DM_ARG_CHECK(dim == 2 || dim == 3, "dim");
  DM_ARG_CHECK(P && idx && d && grad && m >= 0, "pointers");
  if (m == 0) return DM_OK;
  if (dim == 3)
    k_newton_by_value<3><<<grid_for(m, 256), 256, 0, s>>>(P, idx, m, d, grad, alpha, grid_exp);
  else
    k_newton_by_value<2><<<grid_for(m, 256), 256, 0, s>>>(P, idx, m, d, grad, alpha, grid_exp);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

int select_band(const float *d, int64_t n, float lo, float hi, int32_t *idx, int64_t *count,
                cudaStream_t s) {
  DM_ARG_CHECK(d && idx && count && n >= 0, "pointers");
  DM_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(int64_t), s));
  if (n == 0) return DM_OK;
  k_select_band<<<grid_for(n, 256), 256, 0, s>>>(d, n, lo, hi, idx, count);
  note_launches(1);
  DM_LAUNCH_CHECK();
  return DM_OK;
}

}  // namespace dm
