// Robust geometric predicates for the Delaunay kernels.
//
// The reference triangulates with CGAL's Epick kernel (filtered predicates
// with an exact fallback), generation/cpp/delaunay_class.cpp:108-121 and
// generation/cpp/delaunay_class3.cpp:116-129.  CGAL is a third-party
// dependency (>= 5.0, CMakeLists.txt:19-21) that is not vendored, so the
// published methods it relies on are restated here:
//
//  * adaptive exact arithmetic on floating-point expansions
//    (J. R. Shewchuk, "Adaptive Precision Floating-Point Arithmetic and Fast
//    Robust Geometric Predicates", DCG 18, 1997): Two-Sum, Two-Product,
//    Grow/Fast-Expansion-Sum, Scale-Expansion, Compress;
//  * symbolic perturbation of the lifted coordinate with points ordered
//    lexicographically (O. Devillers, M. Teillaud, "Perturbations for
//    Delaunay and weighted Delaunay 3D triangulations", CGTA 44, 2011).
//
// Evaluation order of every predicate: FP32 filter on coordinates already
// translated to the star centre -> FP64 filter on exactly translated
// coordinates -> exact expansion arithmetic on the raw float inputs.
// Inputs are FP32 coordinates, so every product of two inputs is exact in FP64.
//
// Sign conventions (all rows, all translated by the first argument a):
//   orient3(a,b,c,d)  = det[b-a; c-a; d-a]
//   insph3(a,b,c,d,e) = det[[b-a,|b-a|^2]; [c-a,..]; [d-a,..]; [e-a,..]]
//   with orient3(a,b,c,d) > 0, e is inside sphere(a,b,c,d) iff insph3 < 0.
//   orient2(a,b,c)    = det[b-a; c-a]
//   incirc2(a,b,c,d)  = det[[b-a,|b-a|^2]; [c-a,..]; [d-a,..]]
//   with orient2(a,b,c) > 0, d is inside circle(a,b,c) iff incirc2 < 0.
// Symbolic perturbation raises the lifted coordinate of each point by an
// infinitesimal whose order follows the lexicographic order of the points
// (lexicographically largest point = largest perturbation).  Under it a
// sphere/circle test against a non-degenerate simplex never returns zero.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define DM_HD __host__ __device__ __forceinline__
// The exact stages are out-of-line functions that keep every expansion in a
// caller-provided ExactScratch (allocated once in the kernel's own frame).
// Out-of-line device functions that owned local arrays computed wrong
// results with nvcc 13.0 for sm_103a; the scratch form is exact and keeps a
// single copy of each stage per translation unit.
#define DM_HD_NI static __host__ __device__ __noinline__
#else
#define DM_HD static inline
#define DM_HD_NI static
#endif

namespace dmp {

// Slow-path event counters (device side, per translation unit), compiled in
// only with -DDMP_SLOW_COUNTERS: [0] orient fp64 stage, [1] orient exact,
// [2] insphere fp64 stage, [3] insphere exact, [4] symbolic perturbation.
static __device__ unsigned long long g_slow[8];
#if defined(__CUDA_ARCH__) && defined(DMP_SLOW_COUNTERS)
#define DMP_COUNT(i) atomicAdd(&g_slow[i], 1ull)
#else
#define DMP_COUNT(i) ((void)0)
#endif

// Every operation of the error-free transformations must round on its own:
// a multiply fused into a following add (FMA contraction, nvcc's default)
// breaks Two-Sum.  Device code uses the explicitly rounded intrinsics, which
// are never contracted; host code is compiled with -ffp-contract=off.
#if defined(__CUDA_ARCH__)
#define DMP_MUL(a, b) __dmul_rn((a), (b))
#define DMP_ADD(a, b) __dadd_rn((a), (b))
#define DMP_SUB(a, b) __dsub_rn((a), (b))
#else
#define DMP_MUL(a, b) ((a) * (b))
#define DMP_ADD(a, b) ((a) + (b))
#define DMP_SUB(a, b) ((a) - (b))
#endif

// ---------------------------------------------------------------------------
// Error-free transformations (round-to-nearest-even FP64 arithmetic).
DM_HD void two_sum(double a, double b, double &x, double &y) {
  x = DMP_ADD(a, b);
  double bv = DMP_SUB(x, a);
  double av = DMP_SUB(x, bv);
  double br = DMP_SUB(b, bv);
  double ar = DMP_SUB(a, av);
  y = DMP_ADD(ar, br);
}
DM_HD void fast_two_sum(double a, double b, double &x, double &y) {
  x = DMP_ADD(a, b);
  double bv = DMP_SUB(x, a);
  y = DMP_SUB(b, bv);
}
DM_HD void two_prod(double a, double b, double &x, double &y) {
  x = DMP_MUL(a, b);
  y = fma(a, b, -x);
}

// h = e + b  (e: nonoverlapping, increasing magnitude).  |h| <= elen + 1.
DM_HD int grow_expansion(int elen, const double *e, double b, double *h) {
  double q = b;
  int hi = 0;
  for (int i = 0; i < elen; ++i) {
    double qn, hh;
    two_sum(q, e[i], qn, hh);
    q = qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  if (q != 0.0 || hi == 0) h[hi++] = q;
  return hi;
}

// h = e + f by magnitude-ordered merge followed by a Two-Sum sweep.
// |h| <= elen + flen.  h must not alias e or f.
DM_HD int expansion_sum(int elen, const double *e, int flen, const double *f,
                        double *h) {
  int ei = 0, fi = 0, hi = 0;
  double q;
  // first component: smallest magnitude of the two heads
  if (ei < elen && (fi >= flen || fabs(e[ei]) <= fabs(f[fi])))
    q = e[ei++];
  else
    q = f[fi++];
  while (ei < elen || fi < flen) {
    double g;
    if (ei < elen && (fi >= flen || fabs(e[ei]) <= fabs(f[fi])))
      g = e[ei++];
    else
      g = f[fi++];
    double qn, hh;
    two_sum(q, g, qn, hh);
    q = qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  if (q != 0.0 || hi == 0) h[hi++] = q;
  return hi;
}

// h = b * e.  |h| <= 2 elen.
DM_HD int scale_expansion(int elen, const double *e, double b, double *h) {
  double q, hh;
  int hi = 0;
  two_prod(e[0], b, q, hh);
  if (hh != 0.0) h[hi++] = hh;
  for (int i = 1; i < elen; ++i) {
    double p1, p0, s;
    two_prod(e[i], b, p1, p0);
    two_sum(q, p0, s, hh);
    if (hh != 0.0) h[hi++] = hh;
    fast_two_sum(p1, s, q, hh);
    if (hh != 0.0) h[hi++] = hh;
  }
  if (q != 0.0 || hi == 0) h[hi++] = q;
  return hi;
}

// In-place compression to a nonadjacent expansion; returns new length.
DM_HD int compress(int elen, double *e) {
  if (elen <= 1) return elen;
  // top-down pass: write survivors from the top of e downwards
  int bottom = elen - 1;
  double q = e[bottom];
  for (int i = elen - 2; i >= 0; --i) {
    double qn, qq;
    fast_two_sum(q, e[i], qn, qq);
    if (qq != 0.0) {
      e[bottom--] = qn;
      q = qq;
    } else {
      q = qn;
    }
  }
  e[bottom] = q;
  // bottom-up pass
  int top = 0;
  for (int i = bottom + 1; i < elen; ++i) {
    double qn, qq;
    fast_two_sum(e[i], q, qn, qq);
    q = qn;
    if (qq != 0.0) e[top++] = qq;
  }
  e[top++] = q;
  return top;
}

DM_HD int expansion_sign(int elen, const double *e) {
  double v = e[elen - 1];
  return (v > 0.0) - (v < 0.0);
}

DM_HD void negate(int n, double *e) {
  for (int i = 0; i < n; ++i) e[i] = -e[i];
}

// ---------------------------------------------------------------------------
// Exact predicates on raw FP32 coordinates.
// xy-minor m(X,Y) = X_x Y_y - Y_x X_y as an expansion of <= 2 terms.
DM_HD int minor2(const float *X, const float *Y, double *m) {
  double p = DMP_MUL((double)X[0], (double)Y[1]);  // exact: float*float
  double q = DMP_MUL((double)Y[0], (double)X[1]);
  double hi, lo;
  two_sum(p, -q, hi, lo);
  int n = 0;
  if (lo != 0.0) m[n++] = lo;
  if (hi != 0.0 || n == 0) m[n++] = hi;
  return n;
}

// det3 of raw rows [A;B;C] (<= 12 terms), given its three xy-minors;
// t (>= 20 doubles) is scratch.
DM_HD int det3_from_minors(const float *A, const float *B, const float *C,
                           const double *mBC, int nBC, const double *mAC,
                           int nAC, const double *mAB, int nAB, double *out,
                           double *t) {
  double *t1 = t, *t2 = t + 4, *t3 = t + 8, *s12 = t + 12;
  int n1 = scale_expansion(nBC, mBC, (double)A[2], t1);
  int n2 = scale_expansion(nAC, mAC, -(double)B[2], t2);
  int n3 = scale_expansion(nAB, mAB, (double)C[2], t3);
  int n12 = expansion_sum(n1, t1, n2, t2, s12);
  return expansion_sum(n12, s12, n3, t3, out);
}

DM_HD int lex_greater(const float *p, const float *q, int dim) {
  for (int i = 0; i < dim; ++i) {
    if (p[i] > q[i]) return 1;
    if (p[i] < q[i]) return 0;
  }
  return 0;
}

// point r of (a, b, c, d, e) without a local pointer array
DM_HD const float *sel5(int r, const float *a, const float *b, const float *c,
                        const float *d, const float *e) {
  return r == 0 ? a : r == 1 ? b : r == 2 ? c : r == 3 ? d : e;
}
// rank of pair (i < j) among pairs of n items, enumerated i-major
DM_HD int pair_index(int i, int j, int n) { return i * (2 * n - i - 1) / 2 + (j - i - 1); }
// rank of triple (i < j < k) among triples of 5 items, enumerated i-major
DM_HD int triple_index5(int i, int j, int k) {
  int base = i == 0 ? 0 : i == 1 ? 6 : i == 2 ? 9 : 10;
  int m = 4 - i, jj = j - i - 1, kk = k - i - 1;
  return base + jj * (2 * m - jj - 1) / 2 + (kk - jj - 1);
}

// Work space of the exact stages (about 4.6 KB).
#define DMP_ACC_CAP 112
struct ExactScratch {
  double m[10][2];
  int nm[10];
  double D3[10][12];
  int nD3[10];
  double o1[24], o2[24], o[48], tneg[12];
  double acc[DMP_ACC_CAP], tmp[DMP_ACC_CAP], tmp2[DMP_ACC_CAP];
  double w[3];
  double e2[2];
  double d3tmp[20];
  double dx[4][3];  // exact differences of the FP64 filter stages
  float pt[5][3];   // raw points handed to the exact stages by the star kernels
};

// orient3(a,b,c,d) = det3(b,c,d) - det3(a,c,d) + det3(a,b,d) - det3(a,b,c)
// (Laplace expansion of det[[x y z 1]] along the ones column).
DM_HD_NI int orient3_exact(const float *a, const float *b, const float *c,
                           const float *d, ExactScratch *W) {
  DMP_COUNT(1);
  double(*m)[2] = W->m;  // pairs ab ac ad bc bd cd
  int nab = minor2(a, b, m[0]), nac = minor2(a, c, m[1]), nad = minor2(a, d, m[2]);
  int nbc = minor2(b, c, m[3]), nbd = minor2(b, d, m[4]), ncd = minor2(c, d, m[5]);
  double *bcd = W->D3[0], *acd = W->D3[1], *abd = W->D3[2], *abc = W->D3[3];
  int n_bcd = det3_from_minors(b, c, d, m[5], ncd, m[4], nbd, m[3], nbc, bcd, W->d3tmp);
  int n_acd = det3_from_minors(a, c, d, m[5], ncd, m[2], nad, m[1], nac, acd, W->d3tmp);
  int n_abd = det3_from_minors(a, b, d, m[4], nbd, m[2], nad, m[0], nab, abd, W->d3tmp);
  int n_abc = det3_from_minors(a, b, c, m[3], nbc, m[1], nac, m[0], nab, abc, W->d3tmp);
  negate(n_acd, acd);
  negate(n_abc, abc);
  int k1 = expansion_sum(n_bcd, bcd, n_acd, acd, W->o1);
  int k2 = expansion_sum(n_abd, abd, n_abc, abc, W->o2);
  int k = expansion_sum(k1, W->o1, k2, W->o2, W->o);
  k = compress(k, W->o);
  return expansion_sign(k, W->o);
}

// orient2(a,b,c) = m(b,c) - m(a,c) + m(a,b)
DM_HD_NI int orient2_exact(const float *a, const float *b, const float *c,
                           ExactScratch *W) {
  double *mbc = W->m[0], *mac = W->m[1], *mab = W->m[2];
  int nbc = minor2(b, c, mbc), nac = minor2(a, c, mac), nab = minor2(a, b, mab);
  negate(nac, mac);
  int k1 = expansion_sum(nbc, mbc, nac, mac, W->o1);
  int k = expansion_sum(k1, W->o1, nab, mab, W->o);
  k = compress(k, W->o);
  return expansion_sign(k, W->o);
}

// exact lifted coordinate x^2 + y^2 (+ z^2) as an expansion (<= 3 terms);
// e (2 doubles) is scratch.
DM_HD int lift_exact(const float *X, int dim, double *w, double *e) {
  double x2 = DMP_MUL((double)X[0], (double)X[0]);
  double y2 = DMP_MUL((double)X[1], (double)X[1]);
  double hi, lo;
  two_sum(x2, y2, hi, lo);
  int n = 0;
  if (lo != 0.0) e[n++] = lo;
  if (hi != 0.0 || n == 0) e[n++] = hi;
  if (dim == 2) {
    for (int i = 0; i < n; ++i) w[i] = e[i];
    return n;
  }
  double z2 = DMP_MUL((double)X[2], (double)X[2]);
  return grow_expansion(n, e, z2, w);
}

// accumulate acc += coef * w  (coef, w expansions); acc kept compressed.
// Returns new accumulator length, or -1 when a capacity would overflow.
DM_HD int acc_add_product(int nacc, double *acc, int ncoef, const double *coef,
                          int nw, const double *w, double *tmp, double *tmp2) {
  for (int j = 0; j < nw; ++j) {
    if (2 * ncoef + nacc > DMP_ACC_CAP) return -1;
    int ns = scale_expansion(ncoef, coef, w[j], tmp);
    int nn = expansion_sum(nacc, acc, ns, tmp, tmp2);
    nn = compress(nn, tmp2);
    for (int i = 0; i < nn; ++i) acc[i] = tmp2[i];
    nacc = nn;
  }
  return nacc;
}

// insph3(a,b,c,d,e) = w_a o(b,c,d,e) - w_b o(a,c,d,e) + w_c o(a,b,d,e)
//                   - w_d o(a,b,c,e) + w_e o(a,b,c,d)
// Returns the sign; *overflow set to 1 if an expansion would exceed its
// capacity (never happens for finite FP32 inputs of realistic range).
DM_HD_NI int insph3_exact(const float *a, const float *b, const float *c,
                          const float *d, const float *e, int *overflow,
                          ExactScratch *W) {
  DMP_COUNT(3);
  for (int i = 0; i < 5; ++i)
    for (int j = i + 1; j < 5; ++j) {
      int t = pair_index(i, j, 5);
      W->nm[t] = minor2(sel5(i, a, b, c, d, e), sel5(j, a, b, c, d, e), W->m[t]);
    }
  for (int i = 0; i < 5; ++i)
    for (int j = i + 1; j < 5; ++j)
      for (int k = j + 1; k < 5; ++k) {
        int t = triple_index5(i, j, k);
        int mjk = pair_index(j, k, 5), mik = pair_index(i, k, 5), mij = pair_index(i, j, 5);
        W->nD3[t] = det3_from_minors(sel5(i, a, b, c, d, e), sel5(j, a, b, c, d, e),
                                     sel5(k, a, b, c, d, e), W->m[mjk], W->nm[mjk],
                                     W->m[mik], W->nm[mik], W->m[mij], W->nm[mij], W->D3[t],
                                     W->d3tmp);
        W->nD3[t] = compress(W->nD3[t], W->D3[t]);
      }
  W->acc[0] = 0.0;
  int nacc = 1;
  for (int r = 0; r < 5; ++r) {
    // the other four points in argument order
    int q0 = 0 + (0 >= r), q1 = 1 + (1 >= r), q2 = 2 + (2 >= r), q3 = 3 + (3 >= r);
    // o(q0,q1,q2,q3) = det3(q1q2q3) - det3(q0q2q3) + det3(q0q1q3) - det3(q0q1q2)
    int t0 = triple_index5(q1, q2, q3), t1 = triple_index5(q0, q2, q3);
    int t2 = triple_index5(q0, q1, q3), t3 = triple_index5(q0, q1, q2);
    for (int i = 0; i < W->nD3[t1]; ++i) W->tneg[i] = -W->D3[t1][i];
    int k1 = expansion_sum(W->nD3[t0], W->D3[t0], W->nD3[t1], W->tneg, W->o1);
    for (int i = 0; i < W->nD3[t3]; ++i) W->tneg[i] = -W->D3[t3][i];
    int k2 = expansion_sum(W->nD3[t2], W->D3[t2], W->nD3[t3], W->tneg, W->o2);
    int ko = expansion_sum(k1, W->o1, k2, W->o2, W->o);
    ko = compress(ko, W->o);
    if ((r & 1) == 1) negate(ko, W->o);  // alternating signs: +a -b +c -d +e
    int nw = lift_exact(sel5(r, a, b, c, d, e), 3, W->w, W->e2);
    nacc = acc_add_product(nacc, W->acc, ko, W->o, nw, W->w, W->tmp, W->tmp2);
    if (nacc < 0) {
      *overflow = 1;
      return 0;
    }
  }
  return expansion_sign(nacc, W->acc);
}

// incirc2(a,b,c,d) = -w_a o(b,c,d) + w_b o(a,c,d) - w_c o(a,b,d) + w_d o(a,b,c)
DM_HD_NI int incirc2_exact(const float *a, const float *b, const float *c,
                           const float *d, int *overflow, ExactScratch *W) {
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j) {
      int t = pair_index(i, j, 4);
      W->nm[t] = minor2(sel5(i, a, b, c, d, d), sel5(j, a, b, c, d, d), W->m[t]);
    }
  W->acc[0] = 0.0;
  int nacc = 1;
  for (int r = 0; r < 4; ++r) {
    int q0 = 0 + (0 >= r), q1 = 1 + (1 >= r), q2 = 2 + (2 >= r);
    // o(q0,q1,q2) = m(q1,q2) - m(q0,q2) + m(q0,q1)
    int a12 = pair_index(q1, q2, 4), a02 = pair_index(q0, q2, 4), a01 = pair_index(q0, q1, 4);
    for (int i = 0; i < W->nm[a02]; ++i) W->tneg[i] = -W->m[a02][i];
    int k1 = expansion_sum(W->nm[a12], W->m[a12], W->nm[a02], W->tneg, W->o1);
    int ko = expansion_sum(k1, W->o1, W->nm[a01], W->m[a01], W->o);
    ko = compress(ko, W->o);
    if ((r & 1) == 0) negate(ko, W->o);  // -a +b -c +d
    int nw = lift_exact(sel5(r, a, b, c, d, d), 2, W->w, W->e2);
    nacc = acc_add_product(nacc, W->acc, ko, W->o, nw, W->w, W->tmp, W->tmp2);
    if (nacc < 0) {
      *overflow = 1;
      return 0;
    }
  }
  return expansion_sign(nacc, W->acc);
}

// ---------------------------------------------------------------------------
// Filters.  Relative (translated) coordinates, permanent-based error bounds.
// Return +1/-1 when certain, 0 when uncertain.
#define DMP_U32 5.9604644775390625e-08f  /* 2^-24 */
#define DMP_U64 1.1102230246251565e-16   /* 2^-53 */

template <typename T>
DM_HD int orient3_rel_filter(T xx, T xy, T xz, T yx, T yy, T yz, T zx, T zy,
                             T zz, T c) {
  // det[X;Y;Z] = X . (Y x Z)
  T nx = yy * zz - yz * zy, ny = yz * zx - yx * zz, nz = yx * zy - yy * zx;
  T det = xx * nx + xy * ny + xz * nz;
  T px = fabs(yy * zz) + fabs(yz * zy), py = fabs(yz * zx) + fabs(yx * zz),
    pz = fabs(yx * zy) + fabs(yy * zx);
  T perm = fabs(xx) * px + fabs(xy) * py + fabs(xz) * pz;
  if (!(perm < (T)1e30) ) return 0;        // overflow / NaN
  if (perm == (T)0) return 0;             // exact zero is decided exactly
  if (perm < (T)1e-30) return 0;          // underflow risk
  T err = c * perm;
  if (det > err) return 1;
  if (det < -err) return -1;
  return 0;
}

// det of 4x4 rows (x,y,z,w) by Laplace expansion on the (x,y) columns.
template <typename T>
DM_HD int insph3_rel_filter(const T *X, const T *Y, const T *Z, const T *W,
                            T wX, T wY, T wZ, T wW, T c) {
  const T *R[4] = {X, Y, Z, W};
  T w[4] = {wX, wY, wZ, wW};
  T M[4][4], PM[4][4], N[4][4], PN[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j) {
      T p = R[i][0] * R[j][1], q = R[j][0] * R[i][1];
      M[i][j] = p - q;
      PM[i][j] = fabs(p) + fabs(q);
      T r = R[i][2] * w[j], s = R[j][2] * w[i];
      N[i][j] = r - s;
      PN[i][j] = fabs(r) + fabs(s);
    }
  T det = M[0][1] * N[2][3] - M[0][2] * N[1][3] + M[0][3] * N[1][2] +
          M[1][2] * N[0][3] - M[1][3] * N[0][2] + M[2][3] * N[0][1];
  T perm = PM[0][1] * PN[2][3] + PM[0][2] * PN[1][3] + PM[0][3] * PN[1][2] +
           PM[1][2] * PN[0][3] + PM[1][3] * PN[0][2] + PM[2][3] * PN[0][1];
  if (!(perm < (T)1e30)) return 0;
  if (perm == (T)0) return 0;
  if (perm < (T)1e-30) return 0;
  T err = c * perm;
  if (det > err) return 1;
  if (det < -err) return -1;
  return 0;
}

template <typename T>
DM_HD int orient2_rel_filter(T xx, T xy, T yx, T yy, T c) {
  T p = xx * yy, q = xy * yx;
  T det = p - q;
  T perm = fabs(p) + fabs(q);
  if (!(perm < (T)1e30)) return 0;
  if (perm == (T)0) return 0;
  if (perm < (T)1e-30) return 0;
  T err = c * perm;
  if (det > err) return 1;
  if (det < -err) return -1;
  return 0;
}

// det3 rows (x,y,w) by expansion along w
template <typename T>
DM_HD int incirc2_rel_filter(const T *X, const T *Y, const T *Z, T wX, T wY,
                             T wZ, T c) {
  T a1 = Y[0] * Z[1], a2 = Z[0] * Y[1];
  T b1 = X[0] * Z[1], b2 = Z[0] * X[1];
  T c1 = X[0] * Y[1], c2 = Y[0] * X[1];
  T mYZ = a1 - a2, mXZ = b1 - b2, mXY = c1 - c2;
  T det = wX * mYZ - wY * mXZ + wZ * mXY;
  T perm = fabs(wX) * (fabs(a1) + fabs(a2)) + fabs(wY) * (fabs(b1) + fabs(b2)) +
           fabs(wZ) * (fabs(c1) + fabs(c2));
  if (!(perm < (T)1e30)) return 0;
  if (perm == (T)0) return 0;
  if (perm < (T)1e-30) return 0;
  T err = c * perm;
  if (det > err) return 1;
  if (det < -err) return -1;
  return 0;
}

// exact translation test: returns 1 and the differences if b - a is exact
DM_HD int exact_diff(const float *b, const float *a, int dim, double *out) {
  for (int i = 0; i < dim; ++i) {
    double x, y;
    two_sum((double)b[i], -(double)a[i], x, y);
    if (y != 0.0) return 0;
    out[i] = x;
  }
  return 1;
}

// ---------------------------------------------------------------------------
// Full predicates on raw coordinates (FP64 filter then exact).
DM_HD_NI int orient3_slow(const float *a, const float *b, const float *c,
                          const float *d, ExactScratch *W) {
  DMP_COUNT(0);
  double *X = W->dx[0], *Y = W->dx[1], *Z = W->dx[2];
  if (exact_diff(b, a, 3, X) && exact_diff(c, a, 3, Y) && exact_diff(d, a, 3, Z)) {
    int s = orient3_rel_filter<double>(X[0], X[1], X[2], Y[0], Y[1], Y[2], Z[0],
                                       Z[1], Z[2], 16.0 * DMP_U64);
    if (s) return s;
    // all-zero permanent means an exactly zero determinant
    if (((X[0] == 0 && X[1] == 0 && X[2] == 0) || (Y[0] == 0 && Y[1] == 0 && Y[2] == 0) ||
         (Z[0] == 0 && Z[1] == 0 && Z[2] == 0)))
      return 0;
  }
  return orient3_exact(a, b, c, d, W);
}

DM_HD int orient3(const float *a, const float *b, const float *c,
                  const float *d, ExactScratch *W) {
  int s = orient3_rel_filter<float>(b[0] - a[0], b[1] - a[1], b[2] - a[2], c[0] - a[0],
                                    c[1] - a[1], c[2] - a[2], d[0] - a[0], d[1] - a[1],
                                    d[2] - a[2], 16.0f * DMP_U32);
  if (s) return s;
  return orient3_slow(a, b, c, d, W);
}

DM_HD_NI int orient2_slow(const float *a, const float *b, const float *c,
                          ExactScratch *W) {
  double *X = W->dx[0], *Y = W->dx[1];
  if (exact_diff(b, a, 2, X) && exact_diff(c, a, 2, Y)) {
    int s = orient2_rel_filter<double>(X[0], X[1], Y[0], Y[1], 8.0 * DMP_U64);
    if (s) return s;
  }
  return orient2_exact(a, b, c, W);
}

DM_HD int orient2(const float *a, const float *b, const float *c,
                  ExactScratch *W) {
  int s = orient2_rel_filter<float>(b[0] - a[0], b[1] - a[1], c[0] - a[0], c[1] - a[1],
                                    8.0f * DMP_U32);
  if (s) return s;
  return orient2_slow(a, b, c, W);
}


// unperturbed sign of insph3 (FP64 filter, then exact)
DM_HD_NI int insph3_slow(const float *a, const float *b, const float *c,
                         const float *d, const float *e, int *overflow,
                         ExactScratch *W) {
  DMP_COUNT(2);
  double *X = W->dx[0], *Y = W->dx[1], *Z = W->dx[2], *Q = W->dx[3];
  if (exact_diff(b, a, 3, X) && exact_diff(c, a, 3, Y) && exact_diff(d, a, 3, Z) &&
      exact_diff(e, a, 3, Q)) {
    double wx = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
    double wy = Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2];
    double wz = Z[0] * Z[0] + Z[1] * Z[1] + Z[2] * Z[2];
    double ww = Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2];
    int s = insph3_rel_filter<double>(X, Y, Z, Q, wx, wy, wz, ww, 48.0 * DMP_U64);
    if (s) return s;
  }
  return insph3_exact(a, b, c, d, e, overflow, W);
}

// perturbed insph3: never 0 unless all five points are coplanar (or overflow).
// The coefficient of the lifted coordinate of point X (translated form):
//   e: +o(a,b,c,d)  d: -o(a,b,c,e)  c: +o(a,b,d,e)  b: -o(a,c,d,e)  a: +o(b,c,d,e)
// Points are visited from the lexicographically largest (largest
// perturbation) down; the first non-zero coefficient decides.
DM_HD_NI int insph3_sos_tail(const float *a, const float *b, const float *c,
                          const float *d, const float *e, ExactScratch *W) {
  DMP_COUNT(4);
  int done = 0;  // bit mask of visited points
  for (int step = 0; step < 5; ++step) {
    int best = -1;
    for (int r = 0; r < 5; ++r) {
      if (done >> r & 1) continue;
      if (best < 0 || lex_greater(sel5(r, a, b, c, d, e), sel5(best, a, b, c, d, e), 3)) best = r;
    }
    done |= 1 << best;
    int s = 0;
    switch (best) {
      case 4: s = orient3(a, b, c, d, W); break;
      case 3: s = -orient3(a, b, c, e, W); break;
      case 2: s = orient3(a, b, d, e, W); break;
      case 1: s = -orient3(a, c, d, e, W); break;
      case 0: s = orient3(b, c, d, e, W); break;
    }
    if (s) return s;
  }
  return 0;
}

DM_HD int insph3_sos(const float *a, const float *b, const float *c,
                     const float *d, const float *e, int *overflow,
                     ExactScratch *W) {
  float X[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  float Y[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  float Z[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
  float Q[3] = {e[0] - a[0], e[1] - a[1], e[2] - a[2]};
  float wx = X[0] * X[0] + X[1] * X[1] + X[2] * X[2];
  float wy = Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2];
  float wz = Z[0] * Z[0] + Z[1] * Z[1] + Z[2] * Z[2];
  float ww = Q[0] * Q[0] + Q[1] * Q[1] + Q[2] * Q[2];
  int s = insph3_rel_filter<float>(X, Y, Z, Q, wx, wy, wz, ww, 48.0f * DMP_U32);
  if (s) return s;
  s = insph3_slow(a, b, c, d, e, overflow, W);
  if (s) return s;
  return insph3_sos_tail(a, b, c, d, e, W);
}

DM_HD_NI int incirc2_slow(const float *a, const float *b, const float *c,
                          const float *d, int *overflow, ExactScratch *W) {
  double *X = W->dx[0], *Y = W->dx[1], *Z = W->dx[2];
  if (exact_diff(b, a, 2, X) && exact_diff(c, a, 2, Y) && exact_diff(d, a, 2, Z)) {
    double wx = X[0] * X[0] + X[1] * X[1];
    double wy = Y[0] * Y[0] + Y[1] * Y[1];
    double wz = Z[0] * Z[0] + Z[1] * Z[1];
    int s = incirc2_rel_filter<double>(X, Y, Z, wx, wy, wz, 16.0 * DMP_U64);
    if (s) return s;
  }
  return incirc2_exact(a, b, c, d, overflow, W);
}

// perturbation coefficients of incirc2 (translated form):
//   d: +o(a,b,c)  c: -o(a,b,d)  b: +o(a,c,d)  a: -o(b,c,d)
DM_HD_NI int incirc2_sos_tail(const float *a, const float *b, const float *c,
                           const float *d, ExactScratch *W) {
  int done = 0;
  for (int step = 0; step < 4; ++step) {
    int best = -1;
    for (int r = 0; r < 4; ++r) {
      if (done >> r & 1) continue;
      if (best < 0 || lex_greater(sel5(r, a, b, c, d, d), sel5(best, a, b, c, d, d), 2)) best = r;
    }
    done |= 1 << best;
    int s = 0;
    switch (best) {
      case 3: s = orient2(a, b, c, W); break;
      case 2: s = -orient2(a, b, d, W); break;
      case 1: s = orient2(a, c, d, W); break;
      case 0: s = -orient2(b, c, d, W); break;
    }
    if (s) return s;
  }
  return 0;
}

DM_HD int incirc2_sos(const float *a, const float *b, const float *c,
                      const float *d, int *overflow, ExactScratch *W) {
  float X[2] = {b[0] - a[0], b[1] - a[1]};
  float Y[2] = {c[0] - a[0], c[1] - a[1]};
  float Z[2] = {d[0] - a[0], d[1] - a[1]};
  float wx = X[0] * X[0] + X[1] * X[1];
  float wy = Y[0] * Y[0] + Y[1] * Y[1];
  float wz = Z[0] * Z[0] + Z[1] * Z[1];
  int s = incirc2_rel_filter<float>(X, Y, Z, wx, wy, wz, 16.0f * DMP_U32);
  if (s) return s;
  s = incirc2_slow(a, b, c, d, overflow, W);
  if (s) return s;
  return incirc2_sos_tail(a, b, c, d, W);
}

}  // namespace dmp
