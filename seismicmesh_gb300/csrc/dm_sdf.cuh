// Signed distance programs: a postfix list of primitives and set operations
// evaluated per point with forward-mode gradients.
//
// Follows geometry/signed_distance_functions.py: the inverse rigid
// transforms of _manipulate (89-101: translate back, Rx^-1, Ry^-1, Rz^-1,
// stretch back), the primitives Disk (429-447, _ddisk 596-598), Ball
// (450-471, dball 601-603), Rectangle (474-492 -> drectangle_fast,
// geometry/cpp/fast_geometry.cpp:165-214), Cube (495-519 -> dblock_fast,
// fast_geometry.cpp:104-163), Torus (522-543), Prism (546-566), Cylinder
// (569-593), and the sharp / smooth set operations Union (307-344),
// Intersection (347-384) and Difference (387-426).  Gradients replace the
// one-sided finite differences of _project_points_back_newton
// (generation/mesh_generator.py:762-784): with FP32 coordinates the
// reference step sqrt(eps_f64)*h0 is below the coordinate resolution, so the
// analytic derivative is used instead (it is the limit the reference's
// difference quotient approximates).
#pragma once
#include <math.h>
#include <stdint.h>

namespace dm {

enum SdfOp : int32_t {
  SDF_DISK = 1,
  SDF_BALL = 2,
  SDF_RECT = 3,
  SDF_CUBE = 4,
  SDF_TORUS = 5,
  SDF_PRISM = 6,
  SDF_CYLINDER = 7,
  SDF_GRID = 8,
  SDF_UNION = 20,
  SDF_INTERSECTION = 21,
  SDF_DIFFERENCE = 22,
};
enum SdfXform : int32_t {
  XF_TRANSLATE = 1,
  XF_RX = 2,
  XF_RY = 4,
  XF_RZ = 8,
  XF_STRETCH = 16,
  XF_REPEAT = 32,  // periodic repetition, applied before the other transforms
};
constexpr int SDF_OPREC = 4;  // {op, param offset, child count, xform flags}
constexpr int SDF_STACK = 16;

struct Dual {
  float v, g[3];
};

__device__ __forceinline__ float sgnf(float x) { return (x > 0.f) - (x < 0.f); }

// apply M^T to g (M row-major dim x dim)
template <int DIM>
__device__ __forceinline__ void mt_apply(const float *M, float *g) {
  float r[3] = {0, 0, 0};
  for (int i = 0; i < DIM; ++i)
    for (int j = 0; j < DIM; ++j) r[i] += M[j * DIM + i] * g[j];
  for (int i = 0; i < DIM; ++i) g[i] = r[i];
}
template <int DIM>
__device__ __forceinline__ void m_apply(const float *M, float *x) {
  float r[3] = {0, 0, 0};
  for (int i = 0; i < DIM; ++i)
    for (int j = 0; j < DIM; ++j) r[i] += M[i * DIM + j] * x[j];
  for (int i = 0; i < DIM; ++i) x[i] = r[i];
}

// bilinear / trilinear interpolation of a regular grid with extrapolation
// (scipy RegularGridInterpolator, method="linear", fill_value=None)
template <int DIM>
__device__ __forceinline__ float grid_interp(const float *grid, const int *n,
                                             const float *lo, const float *hi,
                                             const float *x, float *grad) {
  int i[3] = {0, 0, 0};
  float t[3] = {0, 0, 0}, inv[3] = {0, 0, 0};
  for (int k = 0; k < DIM; ++k) {
    float step = (hi[k] - lo[k]) / (float)(n[k] - 1);
    inv[k] = 1.f / step;
    float u = (x[k] - lo[k]) * inv[k];
    int ii = (int)floorf(u);
    ii = min(max(ii, 0), n[k] - 2);
    i[k] = ii;
    t[k] = u - (float)ii;
  }
  if (DIM == 2) {
    const float *r0 = grid + (size_t)i[0] * n[1] + i[1];
    const float *r1 = r0 + n[1];
    float f00 = __ldg(r0), f01 = __ldg(r0 + 1), f10 = __ldg(r1), f11 = __ldg(r1 + 1);
    float a0 = f00 + (f01 - f00) * t[1], a1 = f10 + (f11 - f10) * t[1];
    if (grad) {
      grad[0] = (a1 - a0) * inv[0];
      grad[1] = ((1.f - t[0]) * (f01 - f00) + t[0] * (f11 - f10)) * inv[1];
    }
    return a0 + (a1 - a0) * t[0];
  } else {
    size_t s1 = n[2], s0 = (size_t)n[1] * n[2];
    const float *b = grid + i[0] * s0 + i[1] * s1 + i[2];
    float c[8];
    for (int q = 0; q < 8; ++q)
      c[q] = __ldg(b + ((q >> 2) & 1) * s0 + ((q >> 1) & 1) * s1 + (q & 1));
    float c00 = c[0] + (c[1] - c[0]) * t[2], c01 = c[2] + (c[3] - c[2]) * t[2];
    float c10 = c[4] + (c[5] - c[4]) * t[2], c11 = c[6] + (c[7] - c[6]) * t[2];
    float c0 = c00 + (c01 - c00) * t[1], c1 = c10 + (c11 - c10) * t[1];
    if (grad) {
      grad[0] = (c1 - c0) * inv[0];
      float d0 = (c01 - c00), d1 = (c11 - c10);
      grad[1] = ((1.f - t[0]) * d0 + t[0] * d1) * inv[1];
      float e00 = c[1] - c[0], e01 = c[3] - c[2], e10 = c[5] - c[4], e11 = c[7] - c[6];
      float e0 = e00 + (e01 - e00) * t[1], e1 = e10 + (e11 - e10) * t[1];
      grad[2] = ((1.f - t[0]) * e0 + t[0] * e1) * inv[2];
    }
    return c0 + (c1 - c0) * t[0];
  }
}

// primitive value and local gradient at q
template <int DIM, bool GRAD>
__device__ __forceinline__ Dual prim_eval(int op, const float *pp,
                                          const float *q) {
  Dual r;
  r.g[0] = r.g[1] = r.g[2] = 0.f;
  switch (op) {
    case SDF_DISK:
    case SDF_BALL: {
      float d[3] = {0, 0, 0}, s = 0.f;
      for (int k = 0; k < DIM; ++k) {
        d[k] = q[k] - pp[k];
        s += d[k] * d[k];
      }
      float l = sqrtf(s);
      r.v = l - pp[DIM];
      if (GRAD && l > 0.f)
        for (int k = 0; k < DIM; ++k) r.g[k] = d[k] / l;
      break;
    }
    case SDF_RECT:
    case SDF_CUBE: {
      // -min(lower/upper slab distances) = max(x1 - x, x - x2, ...)
      float best = -INFINITY;
      int bk = 0;
      float bs = 0.f;
      // reference evaluation order: z-slabs, y-slabs, x-slabs
      for (int kk = DIM - 1; kk >= 0; --kk) {
        float lo = pp[2 * kk] - q[kk], hi = q[kk] - pp[2 * kk + 1];
        if (lo > best) {
          best = lo;
          bk = kk;
          bs = -1.f;
        }
        if (hi > best) {
          best = hi;
          bk = kk;
          bs = 1.f;
        }
      }
      r.v = best;
      if (GRAD) r.g[bk] = bs;
      break;
    }
    case SDF_TORUS: {
      // xz = (x, z); qq = (|xz| - r1, y); d = |qq| - r2
      float lxz = sqrtf(q[0] * q[0] + q[2] * q[2]);
      float a = lxz - pp[0], b = q[1];
      float l = sqrtf(a * a + b * b);
      r.v = l - pp[1];
      if (GRAD && l > 0.f) {
        float da = a / l, db = b / l;
        if (lxz > 0.f) {
          r.g[0] = da * q[0] / lxz;
          r.g[2] = da * q[2] / lxz;
        }
        r.g[1] = db;
      }
      break;
    }
    case SDF_PRISM: {
      // max(|z| - h, max(|x| * 0.866025 + y * 0.5, -y) - b * 0.5)
      float t1 = fabsf(q[2]) - pp[1];
      float u1 = fabsf(q[0]) * 0.866025f + q[1] * 0.5f, u2 = -q[1];
      float u = fmaxf(u1, u2) - pp[0] * 0.5f;
      if (t1 >= u) {
        r.v = t1;
        if (GRAD) r.g[2] = sgnf(q[2]);
      } else {
        r.v = u;
        if (GRAD) {
          if (u1 >= u2) {
            r.g[0] = 0.866025f * sgnf(q[0]);
            r.g[1] = 0.5f;
          } else {
            r.g[1] = -1.f;
          }
        }
      }
      break;
    }
    case SDF_CYLINDER: {
      // d = (|(|xz|, y)| - (r, h)); min(max(d0, d1), 0) + |max(d, 0)|
      float lxz = sqrtf(q[0] * q[0] + q[2] * q[2]);
      float d0 = fabsf(lxz) - pp[0], d1 = fabsf(q[1]) - pp[1];
      float m0 = fmaxf(d0, 0.f), m1 = fmaxf(d1, 0.f);
      float ln = sqrtf(m0 * m0 + m1 * m1);
      r.v = fminf(fmaxf(d0, d1), 0.f) + ln;
      if (GRAD) {
        float g0 = 0.f, g1 = 0.f;  // derivative w.r.t. d0, d1
        if (fmaxf(d0, d1) < 0.f) {
          if (d0 >= d1) g0 = 1.f; else g1 = 1.f;
        }
        if (ln > 0.f) {
          g0 += m0 / ln;
          g1 += m1 / ln;
        }
        if (lxz > 0.f) {
          r.g[0] = g0 * q[0] / lxz;
          r.g[2] = g0 * q[2] / lxz;
        }
        r.g[1] = g1 * sgnf(q[1]);
      }
      break;
    }
    case SDF_GRID: {
      // params: n0 n1 n2 (as floats), lo[3], hi[3], offset of data (float)
      int n[3] = {(int)pp[0], (int)pp[1], (int)pp[2]};
      const float *lo = pp + 3, *hi = pp + 6;
      const float *data = pp + (int)pp[9];
      float g[3] = {0, 0, 0};
      r.v = grid_interp<DIM>(data, n, lo, hi, q, GRAD ? g : nullptr);
      if (GRAD)
        for (int k = 0; k < DIM; ++k) r.g[k] = g[k];
      break;
    }
    default:
      r.v = NAN;
  }
  return r;
}

template <int DIM>
__device__ __forceinline__ int prim_nparams(int op) {
  switch (op) {
    case SDF_DISK:
    case SDF_BALL: return DIM + 1;
    case SDF_RECT:
    case SDF_CUBE: return 2 * DIM;
    case SDF_TORUS:
    case SDF_PRISM:
    case SDF_CYLINDER: return 2;
    case SDF_GRID: return 10;
  }
  return 0;
}

template <int DIM, bool GRAD>
__device__ __forceinline__ Dual eval_primitive(int op, const float *pp,
                                               int xf, const float *x) {
  float q[3] = {x[0], x[1], DIM == 3 ? x[2] : 0.f};
  const float *t = pp + prim_nparams<DIM>(op);
  const float *T = nullptr, *RX = nullptr, *RY = nullptr, *RZ = nullptr,
              *SV = nullptr;
  if (xf & XF_REPEAT) {
    // Repeat (geometry/signed_distance_functions.py:283-297):
    // q = mod(x + p/2, p) - p/2 with a floor-based mod (numpy's np.mod)
    for (int k = 0; k < DIM; ++k) {
      const float p = t[k], y = q[k] + 0.5f * p;
      q[k] = y - p * floorf(y / p) - 0.5f * p;
    }
    t += DIM;
  }
  if (xf & XF_TRANSLATE) {
    T = t;
    t += DIM;
  }
  if (xf & XF_RX) {
    RX = t;
    t += DIM * DIM;
  }
  if (xf & XF_RY) {
    RY = t;
    t += DIM * DIM;
  }
  if (xf & XF_RZ) {
    RZ = t;
    t += DIM * DIM;
  }
  if (xf & XF_STRETCH) {
    SV = t;
    t += DIM + 1;
  }
  if (T)
    for (int k = 0; k < DIM; ++k) q[k] -= T[k];
  if (RX) m_apply<DIM>(RX, q);
  if (RY) m_apply<DIM>(RY, q);
  if (RZ) m_apply<DIM>(RZ, q);
  float vx = 0.f, sa = 0.f;
  if (SV) {
    // x' = (v.x) v / alpha + (x - (v.x) v)
    for (int k = 0; k < DIM; ++k) vx += SV[k] * q[k];
    sa = 1.f / SV[DIM] - 1.f;
    for (int k = 0; k < DIM; ++k) q[k] += sa * vx * SV[k];
  }
  Dual r = prim_eval<DIM, GRAD>(op, pp, q);
  if (GRAD) {
    if (SV) {
      float vg = 0.f;
      for (int k = 0; k < DIM; ++k) vg += SV[k] * r.g[k];
      for (int k = 0; k < DIM; ++k) r.g[k] += sa * vg * SV[k];
    }
    if (RZ) mt_apply<DIM>(RZ, r.g);
    if (RY) mt_apply<DIM>(RY, r.g);
    if (RX) mt_apply<DIM>(RX, r.g);
  }
  return r;
}

// smooth fold operators on duals (signed distance k-smoothing)
template <bool GRAD>
__device__ __forceinline__ Dual smooth_union(const Dual &a, const Dual &b,
                                             float k) {
  Dual r;
  float diff = a.v - b.v;
  float h = fmaxf(k - fabsf(diff), 0.f);
  bool amin = a.v <= b.v;
  r.v = fminf(a.v, b.v) - h * h * 0.25f / k;
  if (GRAD)
    for (int i = 0; i < 3; ++i) {
      float gm = amin ? a.g[i] : b.g[i];
      float hg = h > 0.f ? -sgnf(diff) * (a.g[i] - b.g[i]) : 0.f;
      r.g[i] = gm - 0.5f * h * hg / k;
    }
  return r;
}
template <bool GRAD>
__device__ __forceinline__ Dual smooth_inter(const Dual &a, const Dual &b,
                                             float k) {
  Dual r;
  float diff = a.v - b.v;
  float h = fmaxf(k - fabsf(diff), 0.f);
  bool amax = a.v >= b.v;
  r.v = fmaxf(a.v, b.v) + h * h * 0.25f / k;
  if (GRAD)
    for (int i = 0; i < 3; ++i) {
      float gm = amax ? a.g[i] : b.g[i];
      float hg = h > 0.f ? -sgnf(diff) * (a.g[i] - b.g[i]) : 0.f;
      r.g[i] = gm + 0.5f * h * hg / k;
    }
  return r;
}
// _smooth_difference(d1, d2): h = max(k - |-d1 - d2|, 0);
// max(-d1, d2) + h^2 / 4k
template <bool GRAD>
__device__ __forceinline__ Dual smooth_diff(const Dual &a, const Dual &b,
                                            float k) {
  Dual r;
  float s = -a.v - b.v;
  float h = fmaxf(k - fabsf(s), 0.f);
  bool first = -a.v >= b.v;
  r.v = fmaxf(-a.v, b.v) + h * h * 0.25f / k;
  if (GRAD)
    for (int i = 0; i < 3; ++i) {
      float gm = first ? -a.g[i] : b.g[i];
      float hg = h > 0.f ? -sgnf(s) * (-a.g[i] - b.g[i]) : 0.f;
      r.g[i] = gm + 0.5f * h * hg / k;
    }
  return r;
}

// Evaluate a program at x.  Returns NaN on a malformed program.
template <int DIM, bool GRAD>
__device__ Dual sdf_eval(const int32_t *ops, const float *params, int n_ops,
                         const float *x) {
  Dual st[SDF_STACK];
  int sp = 0;
  for (int o = 0; o < n_ops; ++o) {
    int op = __ldg(ops + SDF_OPREC * o);
    int off = __ldg(ops + SDF_OPREC * o + 1);
    int cnt = __ldg(ops + SDF_OPREC * o + 2);
    int xf = __ldg(ops + SDF_OPREC * o + 3);
    if (op < SDF_UNION) {
      if (sp >= SDF_STACK) break;
      st[sp++] = eval_primitive<DIM, GRAD>(op, params + off, xf, x);
      continue;
    }
    if (cnt < 1 || cnt > sp) {
      sp = -1;
      break;
    }
    float k = __ldg(params + off);
    Dual *c = st + sp - cnt;
    Dual r = c[0];
    if (op == SDF_UNION) {
      if (k == 0.f) {
        for (int i = 1; i < cnt; ++i)
          if (c[i].v < r.v) r = c[i];
      } else {
        for (int i = 1; i < cnt; ++i) r = smooth_union<GRAD>(r, c[i], k);
      }
    } else if (op == SDF_INTERSECTION) {
      if (k == 0.f) {
        for (int i = 1; i < cnt; ++i)
          if (c[i].v > r.v) r = c[i];
      } else {
        for (int i = 1; i < cnt; ++i) r = smooth_inter<GRAD>(r, c[i], k);
      }
    } else if (op == SDF_DIFFERENCE) {
      if (k == 0.f) {
        for (int i = 1; i < cnt; ++i) {
          if (-c[i].v > r.v) {
            r.v = -c[i].v;
            for (int j = 0; j < 3; ++j) r.g[j] = -c[i].g[j];
          }
        }
      } else {
        // fold over the reversed child list: tmp = d[m]; tmp = f(tmp, d[i])
        r = c[cnt - 1];
        for (int i = cnt - 2; i >= 0; --i) r = smooth_diff<GRAD>(r, c[i], k);
      }
    } else {
      sp = -1;
      break;
    }
    sp -= cnt;
    st[sp++] = r;
  }
  if (sp != 1) {
    Dual bad;
    bad.v = NAN;
    bad.g[0] = bad.g[1] = bad.g[2] = 0.f;
    return bad;
  }
  return st[0];
}

}  // namespace dm
