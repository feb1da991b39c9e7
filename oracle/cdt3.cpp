// Host 3D Delaunay tetrahedralisation with exact predicates.
//
// TEST INFRASTRUCTURE ONLY: the second CPU triangulation stub of the
// reference loop's CPU baseline (bench.py's reference arm and cpu_baseline,
// tests/).  The reference rebuilds a CGAL Delaunay_triangulation_3 every
// DistMesh iteration (generation/mesh_generator.py:465-469 ->
// generation/cpp/delaunay_class3.cpp:116-129, get_finite_cells 276-310);
// CGAL cannot be built here, so the oracle's loop uses Qhull, and this file
// is the project's own exact-predicate triangulator plugged in at the same
// place.  Published methods, written here:
//
//  * Bowyer-Watson insertion (Bowyer 1981, Watson 1981): the tetrahedra whose
//    circumsphere contains the new point form a star-shaped cavity, which is
//    replaced by the cone from the point to the cavity's boundary faces;
//  * point location by a visibility walk from the last tetrahedron created
//    (terminates in a Delaunay triangulation: Edelsbrunner's acyclicity
//    theorem), with points inserted in Morton (Z-order) order;
//  * exact orientation and in-sphere predicates by floating-point filters
//    with the error bounds of Shewchuk, "Adaptive precision floating-point
//    arithmetic and fast robust geometric predicates" (1997), falling back
//    to his expansion arithmetic (two-sum, two-product, expansion sum and
//    scaling with zero elimination): on the translated determinant when the
//    coordinate differences are exact (nearby points, the usual case), else
//    on the untranslated 4x4 / 5x5 determinants;
//  * symbolic perturbation of the lifted coordinate (points ordered by a
//    hash of their index, see sos_key), which decides cospherical ties, so
//    that the degenerate initial lattice of DistMesh has well-defined
//    cavities (Edelsbrunner and Muecke, simulation of simplicity, 1990);
//  * a bounding super-tetrahedron 1e5 times the points' extent: the result
//    is the Delaunay tetrahedralisation of the points except tetrahedra on
//    the convex hull whose circumsphere would reach that far (exactly flat
//    hull configurations).
//
// Entry points (C ABI, for ctypes):
//   cdt3_delaunay(xyz, n, out, cap): tetrahedra into out[cap][4]; returns
//     their number, or -(number) when cap is too small (out untouched past
//     cap), or a code at or below -2^41 on errors (bad n, a non-finite
//     coordinate, a cavity that did not close);
//   cdt3_orient4 / cdt3_insphere: the predicates, for tests.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// expansion arithmetic (components in increasing magnitude, nonoverlapping)
inline void two_sum(double a, double b, double &x, double &y) {
  x = a + b;
  const double bv = x - a;
  const double av = x - bv;
  y = (a - av) + (b - bv);
}

inline void fast_two_sum(double a, double b, double &x, double &y) {
  x = a + b;
  y = b - (x - a);
}

inline void two_prod(double a, double b, double &x, double &y) {
  x = a * b;
  y = std::fma(a, b, -x);
}

// h = e + f with zero elimination; h has room for elen + flen components
int expansion_sum(int elen, const double *e, int flen, const double *f, double *h) {
  int ei = 0, fi = 0, hi = 0;
  double Q, Qn, hh;
  double en = e[0], fn = f[0];
  auto take_e = [&]() { return (fn > en) == (fn > -en); };
  if (take_e()) {
    Q = en;
    en = ++ei < elen ? e[ei] : 0.0;
  } else {
    Q = fn;
    fn = ++fi < flen ? f[fi] : 0.0;
  }
  if (ei < elen && fi < flen) {
    if (take_e()) {
      fast_two_sum(en, Q, Qn, hh);
      en = ++ei < elen ? e[ei] : 0.0;
    } else {
      fast_two_sum(fn, Q, Qn, hh);
      fn = ++fi < flen ? f[fi] : 0.0;
    }
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
    while (ei < elen && fi < flen) {
      if (take_e()) {
        two_sum(Q, en, Qn, hh);
        en = ++ei < elen ? e[ei] : 0.0;
      } else {
        two_sum(Q, fn, Qn, hh);
        fn = ++fi < flen ? f[fi] : 0.0;
      }
      Q = Qn;
      if (hh != 0.0) h[hi++] = hh;
    }
  }
  while (ei < elen) {
    two_sum(Q, en, Qn, hh);
    en = ++ei < elen ? e[ei] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  while (fi < flen) {
    two_sum(Q, fn, Qn, hh);
    fn = ++fi < flen ? f[fi] : 0.0;
    Q = Qn;
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

// h = b * e with zero elimination; h has room for 2 elen components
int scale_expansion(int elen, const double *e, double b, double *h) {
  int hi = 0;
  double Q, hh, p1, p0, s;
  two_prod(e[0], b, Q, hh);
  if (hh != 0.0) h[hi++] = hh;
  for (int i = 1; i < elen; ++i) {
    two_prod(e[i], b, p1, p0);
    two_sum(Q, p0, s, hh);
    if (hh != 0.0) h[hi++] = hh;
    fast_two_sum(p1, s, Q, hh);
    if (hh != 0.0) h[hi++] = hh;
  }
  if (Q != 0.0 || hi == 0) h[hi++] = Q;
  return hi;
}

inline int sign_of(int len, const double *e) {
  const double t = e[len - 1];
  return (t > 0.0) - (t < 0.0);
}

inline int negate(int len, const double *e, double *h) {
  for (int i = 0; i < len; ++i) h[i] = -e[i];
  return len;
}

// xy minor p.x q.y - p.y q.x, exact (<= 4 components)
int minor_xy(const double *p, const double *q, double *h) {
  double a1, a0, b1, b0;
  two_prod(p[0], q[1], a1, a0);
  two_prod(p[1], q[0], b1, b0);
  const double A[2] = {a0, a1}, B[2] = {-b0, -b1};
  return expansion_sum(2, A, 2, B, h);
}

// det3 of the xyz rows p, q, r, exact (<= 24 components), expanded along z:
// pz m(q, r) - qz m(p, r) + rz m(p, q)
int det3_exact(const double *p, const double *q, const double *r, double *h) {
  double m_qr[4], m_pr[4], m_pq[4], t1[8], t2[8], t3[8], s12[16];
  const int lqr = minor_xy(q, r, m_qr), lpr = minor_xy(p, r, m_pr), lpq = minor_xy(p, q, m_pq);
  const int l1 = scale_expansion(lqr, m_qr, p[2], t1);
  const int l2 = scale_expansion(lpr, m_pr, -q[2], t2);
  const int l3 = scale_expansion(lpq, m_pq, r[2], t3);
  const int l12 = expansion_sum(l1, t1, l2, t2, s12);
  return expansion_sum(l12, s12, l3, t3, h);
}

// orient4(a, b, c, d) = det of the rows (x, y, z, 1), exact (<= 96 components):
// -det3(b,c,d) + det3(a,c,d) - det3(a,b,d) + det3(a,b,c)
int orient4_exact(const double *a, const double *b, const double *c, const double *d, double *h) {
  double d1[24], d2[24], d3[24], d4[24], n1[24], n3[24], s1[48], s2[48];
  const int l1 = det3_exact(b, c, d, d1), l2 = det3_exact(a, c, d, d2);
  const int l3 = det3_exact(a, b, d, d3), l4 = det3_exact(a, b, c, d4);
  negate(l1, d1, n1);
  negate(l3, d3, n3);
  const int ls1 = expansion_sum(l1, n1, l2, d2, s1);
  const int ls2 = expansion_sum(l3, n3, l4, d4, s2);
  return expansion_sum(ls1, s1, ls2, s2, h);
}

// exact difference a - b when the rounding error is zero (Sterbenz: within a
// factor of two, or equal exponents), else false
inline bool exact_diff(double a, double b, double &d) {
  d = a - b;
  const double bv = a - d;
  const double av = d + bv;
  return (a - av) + (bv - b) == 0.0;
}

constexpr double kEps = 1.1102230246251565e-16;  // 2^-53
// Shewchuk's first-stage bounds, doubled as a margin for evaluation order
const double kO3Bound = 2.0 * (7.0 + 56.0 * kEps) * kEps;
const double kISBound = 2.0 * (16.0 + 224.0 * kEps) * kEps;

// sign of orient4(a, b, c, d) = -det3(b - a, c - a, d - a)
int orient4(const double *a, const double *b, const double *c, const double *d) {
  const double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
  const double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
  const double wx = d[0] - a[0], wy = d[1] - a[1], wz = d[2] - a[2];
  const double vywz = vy * wz, vzwy = vz * wy, vzwx = vz * wx, vxwz = vx * wz;
  const double vxwy = vx * wy, vywx = vy * wx;
  const double det = ux * (vywz - vzwy) + uy * (vzwx - vxwz) + uz * (vxwy - vywx);
  const double perm = std::fabs(ux) * (std::fabs(vywz) + std::fabs(vzwy)) +
                      std::fabs(uy) * (std::fabs(vzwx) + std::fabs(vxwz)) +
                      std::fabs(uz) * (std::fabs(vxwy) + std::fabs(vywx));
  const double bound = kO3Bound * perm;
  if (det > bound) return -1;
  if (-det > bound) return 1;
  // the differences to a are usually exact: then -det3 of them is the
  // value (<= 24 components instead of 96)
  double U[3], V[3], W[3];
  bool ex = true;
  for (int k = 0; k < 3 && ex; ++k)
    ex = exact_diff(b[k], a[k], U[k]) && exact_diff(c[k], a[k], V[k]) &&
         exact_diff(d[k], a[k], W[k]);
  if (ex) {
    double h[24];
    return -sign_of(det3_exact(U, V, W, h), h);
  }
  double h[96];
  return sign_of(orient4_exact(a, b, c, d, h), h);
}

// D = det of the rows (x - e, |x - e|^2) for x = a, b, c, d: for orient4(a, b,
// c, d) > 0, D > 0 iff e lies inside the circumsphere.  Unperturbed sign.
int insphere_plain(const double *a, const double *b, const double *c, const double *d,
                   const double *e) {
  const double *P[4] = {a, b, c, d};
  double X[4], Y[4], Z[4], L[4];
  for (int i = 0; i < 4; ++i) {
    X[i] = P[i][0] - e[0];
    Y[i] = P[i][1] - e[1];
    Z[i] = P[i][2] - e[2];
    L[i] = X[i] * X[i] + Y[i] * Y[i] + Z[i] * Z[i];
  }
  // det3 of rows i, j, k of (X, Y, Z) along z, with its permanent
  auto d3 = [&](int i, int j, int k, double &perm) {
    const double mjk = X[j] * Y[k] - Y[j] * X[k], mik = X[i] * Y[k] - Y[i] * X[k];
    const double mij = X[i] * Y[j] - Y[i] * X[j];
    perm = std::fabs(Z[i]) * (std::fabs(X[j] * Y[k]) + std::fabs(Y[j] * X[k])) +
           std::fabs(Z[j]) * (std::fabs(X[i] * Y[k]) + std::fabs(Y[i] * X[k])) +
           std::fabs(Z[k]) * (std::fabs(X[i] * Y[j]) + std::fabs(Y[i] * X[j]));
    return Z[i] * mjk - Z[j] * mik + Z[k] * mij;
  };
  double pa, pb, pc, pd;
  const double bcd = d3(1, 2, 3, pa), acd = d3(0, 2, 3, pb), abd = d3(0, 1, 3, pc),
               abc = d3(0, 1, 2, pd);
  const double det = (L[3] * abc - L[2] * abd) + (L[1] * acd - L[0] * bcd);
  const double perm = L[3] * pd + L[2] * pc + L[1] * pb + L[0] * pa;
  const double bound = kISBound * perm;
  if (det > bound) return 1;
  if (-det > bound) return -1;
  // exact, when the differences to e are exact (the usual case for nearby
  // points): D = -L_a det3(b,c,d) + L_b det3(a,c,d) - L_c det3(a,b,d)
  // + L_d det3(a,b,c) over the difference rows, L_i = |x_i - e|^2
  {
    double R[4][3];
    bool ex = true;
    for (int i = 0; i < 4 && ex; ++i)
      for (int k = 0; k < 3 && ex; ++k) ex = exact_diff(P[i][k], e[k], R[i][k]);
    if (ex) {
      // at most 4 terms of 6 x 48 components
      double buf0[1160], buf1[1160];
      double *acc2 = buf0, *tmp2 = buf1;
      acc2[0] = 0.0;
      int alen2 = 1;
      for (int i = 0; i < 4; ++i) {
        const double *o[3];
        for (int j = 0, k = 0; j < 4; ++j)
          if (j != i) o[k++] = R[j];
        double dm[24];
        const int dl = det3_exact(o[0], o[1], o[2], dm);
        if (dl == 1 && dm[0] == 0.0) continue;
        double s0[2], s1[2], s2[2], s01[4], w[6];
        two_prod(R[i][0], R[i][0], s0[1], s0[0]);
        two_prod(R[i][1], R[i][1], s1[1], s1[0]);
        two_prod(R[i][2], R[i][2], s2[1], s2[0]);
        const int l01 = expansion_sum(2, s0, 2, s1, s01);
        const int wl = expansion_sum(l01, s01, 2, s2, w);
        const double sg = (i % 2 == 0) ? -1.0 : 1.0;  // (-1)^(i+4), i from 1
        for (int k = 0; k < wl; ++k) {
          double part[48];
          const int pl = scale_expansion(dl, dm, sg * w[k], part);
          alen2 = expansion_sum(alen2, acc2, pl, part, tmp2);
          std::swap(acc2, tmp2);
        }
      }
      return sign_of(alen2, acc2);
    }
  }
  // exact: the 5x5 determinant of the rows (x, y, z, w, 1), w = |x|^2, for
  // a, b, c, d, e, expanded along w: sum_i (-1)^i w_i orient4(others)
  const double *Q[5] = {a, b, c, d, e};
  static thread_local std::vector<double> acc, tmp, term;
  acc.assign(1, 0.0);
  int alen = 1;
  for (int i = 0; i < 5; ++i) {
    const double *o[4];
    for (int j = 0, k = 0; j < 5; ++j)
      if (j != i) o[k++] = Q[j];
    double om[96];
    const int ol = orient4_exact(o[0], o[1], o[2], o[3], om);
    if (ol == 1 && om[0] == 0.0) continue;
    // w_i exact (<= 6 components)
    double s0[2], s1[2], s2[2], s01[4], w[6];
    two_prod(Q[i][0], Q[i][0], s0[1], s0[0]);
    two_prod(Q[i][1], Q[i][1], s1[1], s1[0]);
    two_prod(Q[i][2], Q[i][2], s2[1], s2[0]);
    const int l01 = expansion_sum(2, s0, 2, s1, s01);
    const int wl = expansion_sum(l01, s01, 2, s2, w);
    // term = w * om (sign (-1)^i, i counted from 1: a is 1)
    const double sg = (i % 2 == 0) ? -1.0 : 1.0;
    term.assign(1, 0.0);
    int tl = 1;
    for (int k = 0; k < wl; ++k) {
      double part[192];
      const int pl = scale_expansion(ol, om, sg * w[k], part);
      tmp.resize(tl + pl);
      tl = expansion_sum(tl, term.data(), pl, part, tmp.data());
      term.assign(tmp.begin(), tmp.begin() + tl);
    }
    tmp.resize(alen + tl);
    alen = expansion_sum(alen, acc.data(), tl, term.data(), tmp.data());
    acc.assign(tmp.begin(), tmp.begin() + alen);
  }
  return sign_of(alen, acc.data());
}

struct Tri {
  const double *xyz;  // [n + 4][3]
};

// Order of the perturbations: a bijective mix of the point's index (xor-
// shifts and odd multipliers, each invertible modulo 2^32), so a strict
// total order that looks random.  Ordering by the index itself also gives a
// valid triangulation, but on DistMesh's lattice it breaks ties in a
// regular pattern, the forces keep the lattice's symmetry and the next
// iterations stay cospherical (about ten times more exact evaluations; a
// single multiplier keeps the pattern quasi-periodic).
inline uint32_t sos_key(int i) {
  uint32_t h = (uint32_t)i;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

// in-sphere with symbolic perturbation of the lifted coordinate: point with
// the larger sos_key perturbed more; the coefficient of point i's
// perturbation (i = 1..5 for a..e) is (-1)^i orient4(the other four)
int insphere_sos(const double *xyz, const int *v, int ie) {
  const double *a = xyz + 3 * v[0], *b = xyz + 3 * v[1], *c = xyz + 3 * v[2],
               *d = xyz + 3 * v[3], *e = xyz + 3 * ie;
  const int s = insphere_plain(a, b, c, d, e);
  if (s) return s;
  const int id[5] = {v[0], v[1], v[2], v[3], ie};
  const double *Q[5] = {a, b, c, d, e};
  int order[5] = {0, 1, 2, 3, 4};
  std::sort(order, order + 5, [&](int x, int y) { return sos_key(id[x]) > sos_key(id[y]); });
  for (int r = 0; r < 5; ++r) {
    const int i = order[r];
    const double *o[4];
    for (int j = 0, k = 0; j < 5; ++j)
      if (j != i) o[k++] = Q[j];
    const int so = orient4(o[0], o[1], o[2], o[3]);
    if (so) return (i % 2 == 0) ? -so : so;  // (-1)^(i+1) with i from 0
  }
  return 0;
}

// ---------------------------------------------------------------------------
// triangulation
struct Tet {
  int v[4];
  int nb[4];  // neighbour opposite v[k]; -1 outside the super-tetrahedron
};

struct DT {
  const double *P;  // points, [n + 4][3]; the last four are the super vertices
  int n;
  std::vector<Tet> tets;
  std::vector<int> freel;
  std::vector<int> mark;  // insertion stamp of cavity membership / visit
  int last = 0;
  uint32_t rng = 12345u;
  bool broken = false;  // a cavity boundary that did not close (never expected)
  std::vector<int> made, outf;
  std::vector<Tet> newt;
  std::vector<uint64_t> slot_key;
  std::vector<int> slot_val;

  int fresh() {
    if (!freel.empty()) {
      const int t = freel.back();
      freel.pop_back();
      return t;
    }
    tets.push_back(Tet{});
    mark.push_back(0);
    return (int)tets.size() - 1;
  }

  int conflict(int t, int p) const { return insphere_sos(P, tets[t].v, p) > 0; }

  // walk to a tetrahedron holding p (closed); -1 when p leaves the hull
  int locate(int p) {
    int t = last;
    const double *q = P + 3 * p;
    for (int steps = 0; steps < 1 << 26; ++steps) {
      const Tet &T = tets[t];
      rng = rng * 1664525u + 1013904223u;
      const int r0 = (int)(rng >> 30);
      int next = -2;
      for (int s = 0; s < 4; ++s) {
        const int k = (r0 + s) & 3;
        const double *w[4];
        for (int j = 0; j < 4; ++j) w[j] = j == k ? q : P + 3 * T.v[j];
        if (orient4(w[0], w[1], w[2], w[3]) < 0) {
          next = T.nb[k];
          break;
        }
      }
      if (next == -2) return t;
      if (next < 0) return -1;
      t = next;
    }
    return -1;
  }

  // insert point p; false for an exact duplicate of a vertex
  bool insert(int p, int stamp, std::vector<int> &cav, std::vector<int> &bnd_t,
              std::vector<int> &bnd_k) {
    int t = locate(p);
    if (t < 0) return false;
    const double *q = P + 3 * p;
    for (int j = 0; j < 4; ++j) {
      const double *x = P + 3 * tets[t].v[j];
      if (x[0] == q[0] && x[1] == q[1] && x[2] == q[2]) return false;
    }
    if (!conflict(t, p)) {
      // cannot happen with exact predicates; search every live tetrahedron
      t = -1;
      for (int u = 0; u < (int)tets.size() && t < 0; ++u)
        if (tets[u].v[0] >= 0 && conflict(u, p)) t = u;
      if (t < 0) return false;
    }
    cav.clear();
    bnd_t.clear();
    bnd_k.clear();
    cav.push_back(t);
    mark[t] = stamp;
    for (size_t i = 0; i < cav.size(); ++i) {
      const int c = cav[i];
      for (int k = 0; k < 4; ++k) {
        const int u = tets[c].nb[k];
        if (u >= 0 && mark[u] == stamp) continue;
        if (u >= 0 && mark[u] == -stamp) {  // already found outside
          bnd_t.push_back(c);
          bnd_k.push_back(k);
          continue;
        }
        if (u >= 0 && conflict(u, p)) {
          mark[u] = stamp;
          cav.push_back(u);
        } else {
          if (u >= 0) mark[u] = -stamp;
          bnd_t.push_back(c);
          bnd_k.push_back(k);
        }
      }
    }
    // new tetrahedra: cavity tetrahedron c with its vertex k replaced by p.
    // Every boundary face is read first: the cavity's slots are reused for
    // the new cone (they were just read, so they are in cache), and the face
    // of the outside neighbour is found by its vertices, not by the slot.
    const size_t nb = bnd_t.size();
    newt.resize(nb);
    outf.resize(nb);
    made.resize(nb);
    for (size_t i = 0; i < nb; ++i) {
      const int c = bnd_t[i], k = bnd_k[i];
      Tet T = tets[c];
      T.v[k] = p;
      int jj = -1;
      const int out = T.nb[k];
      if (out >= 0) {
        const Tet &O = tets[out];
        for (int j = 0; j < 4 && jj < 0; ++j) {
          bool in_face = false;
          for (int l = 0; l < 4; ++l) in_face = in_face || (l != k && T.v[l] == O.v[j]);
          if (!in_face) jj = j;
        }
      }
      newt[i] = T;
      outf[i] = jj;
    }
    for (size_t i = 0; i < nb; ++i) made[i] = i < cav.size() ? cav[i] : fresh();
    for (size_t r = nb; r < cav.size(); ++r) {
      tets[cav[r]].v[0] = -1;
      freel.push_back(cav[r]);
    }
    // faces through p are matched by their edge (the two other vertices) in
    // an open-addressing table; each edge of the cavity boundary is met twice
    size_t cap2 = 16;
    while (cap2 < 4 * nb) cap2 <<= 1;
    if (slot_key.size() < cap2) {
      slot_key.resize(cap2);
      slot_val.resize(cap2);
    }
    for (size_t i = 0; i < cap2; ++i) slot_key[i] = ~0ull;
    size_t unmatched = 0;
    for (size_t i = 0; i < nb; ++i) {
      const int k = bnd_k[i], m = made[i];
      Tet T = newt[i];
      const int out = T.nb[k];
      if (out >= 0) tets[out].nb[outf[i]] = m;
      for (int j = 0; j < 4; ++j) {
        if (j == k) continue;
        int e0 = -1, e1 = -1;
        for (int l = 0; l < 4; ++l) {
          if (l == j || l == k) continue;
          if (e0 < 0) e0 = T.v[l];
          else e1 = T.v[l];
        }
        if (e0 > e1) std::swap(e0, e1);
        const uint64_t key = (uint64_t)(uint32_t)e0 << 32 | (uint32_t)e1;
        size_t h = (size_t)((key * 0x9e3779b97f4a7c15ull) >> 40) & (cap2 - 1);
        while (slot_key[h] != ~0ull && slot_key[h] != key) h = (h + 1) & (cap2 - 1);
        if (slot_key[h] == key) {
          const int ot = slot_val[h] >> 2, ok = slot_val[h] & 3;
          T.nb[j] = ot;
          tets[ot].nb[ok] = m;
          slot_key[h] = ~1ull;  // matched: a tombstone keeps the probe chains intact
          --unmatched;
        } else {
          T.nb[j] = -1;
          slot_key[h] = key;
          slot_val[h] = m << 2 | j;
          ++unmatched;
        }
      }
      tets[m] = T;
      mark[m] = 0;
    }
    if (unmatched) broken = true;
    last = made[0];
    return true;
  }
};

uint64_t spread3(uint32_t x) {
  uint64_t v = x & 0x1fffff;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

}  // namespace

extern "C" {

int cdt3_orient4(const double *a, const double *b, const double *c, const double *d) {
  return orient4(a, b, c, d);
}

int cdt3_insphere(const double *a, const double *b, const double *c, const double *d,
                  const double *e) {
  return insphere_plain(a, b, c, d, e);
}

// perturbed in-sphere of the points xyz[v[0..3]] and xyz[ie] (indices order
// the perturbation)
int cdt3_insphere_sos(const double *xyz, const int *v, int ie) { return insphere_sos(xyz, v, ie); }

int64_t cdt3_delaunay(const double *xyz, int64_t n64, int32_t *out, int64_t cap) {
  if (n64 < 0 || n64 > (1ll << 30)) return -(1ll << 41);
  const int n = (int)n64;
  if (n < 4) return 0;
  std::vector<double> P(3 * ((size_t)n + 4));
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const double x = xyz[3 * i + k];
      if (!std::isfinite(x)) return -(1ll << 42);
      P[3 * i + k] = x;
      lo[k] = std::min(lo[k], x);
      hi[k] = std::max(hi[k], x);
    }
  double ext = 0.0, c[3];
  for (int k = 0; k < 3; ++k) {
    ext = std::max(ext, hi[k] - lo[k]);
    c[k] = 0.5 * (lo[k] + hi[k]);
  }
  if (!(ext > 0.0)) ext = 1.0;
  const double R = 1e5 * ext;
  const double sv[4][3] = {{R, R, R}, {R, -R, -R}, {-R, R, -R}, {-R, -R, R}};
  for (int s = 0; s < 4; ++s)
    for (int k = 0; k < 3; ++k) P[3 * ((size_t)n + s) + k] = c[k] + sv[s][k];
  DT dt;
  dt.P = P.data();
  dt.n = n;
  dt.tets.reserve((size_t)7 * n + 64);
  dt.mark.reserve((size_t)7 * n + 64);
  Tet T0;
  T0.v[0] = n;
  T0.v[1] = n + 1;
  T0.v[2] = n + 2;
  T0.v[3] = n + 3;
  if (orient4(&P[3 * (size_t)n], &P[3 * ((size_t)n + 1)], &P[3 * ((size_t)n + 2)],
              &P[3 * ((size_t)n + 3)]) < 0)
    std::swap(T0.v[0], T0.v[1]);
  for (int k = 0; k < 4; ++k) T0.nb[k] = -1;
  dt.tets.push_back(T0);
  dt.mark.push_back(0);
  // insertion order: Morton code of the quantised coordinates
  std::vector<std::pair<uint64_t, int>> ord(n);
  for (int i = 0; i < n; ++i) {
    uint64_t code = 0;
    for (int k = 0; k < 3; ++k) {
      const double f = (P[3 * i + k] - lo[k]) / (hi[k] > lo[k] ? hi[k] - lo[k] : 1.0);
      const uint32_t q = (uint32_t)std::min(2097151.0, std::max(0.0, f * 2097151.0));
      code |= spread3(q) << k;
    }
    ord[i] = {code, i};
  }
  std::sort(ord.begin(), ord.end());
  std::vector<int> cav, bt, bk;
  int stamp = 1;
  for (int i = 0; i < n; ++i) dt.insert(ord[i].second, stamp++, cav, bt, bk);
  if (dt.broken) return -(1ll << 43);
  int64_t m = 0;
  for (const Tet &T : dt.tets) {
    if (T.v[0] < 0) continue;
    if (T.v[0] >= n || T.v[1] >= n || T.v[2] >= n || T.v[3] >= n) continue;
    if (m < cap)
      for (int k = 0; k < 4; ++k) out[4 * m + k] = T.v[k];
    ++m;
  }
  return m <= cap ? m : -m;
}

}  // extern "C"
