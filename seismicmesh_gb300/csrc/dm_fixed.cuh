// Exact predicates on fixed-point coordinates.
//
// Inside one vertex star the points are close together.  When every
// coordinate involved is an integer multiple of a common power of two 2^g,
// the coordinates relative to the star centre are exact integers at that
// scale.  Within |coordinate| < 2^30 the orientation and in-sphere
// determinants are evaluated exactly in 64/128/192-bit integer arithmetic
// instead of floating-point expansions.  The results are the same exact
// signs as the expansion predicates in dm_predicates.cuh (same conventions,
// same symbolic perturbation), so both paths can be mixed freely.
//
// Conventions (p = star centre = origin, rows relative to p):
//   orient3(p,a,b,c)   = det[A; B; C]
//   insph3(p,a,b,c,d)  = det[[A,|A|^2]; [B,|B|^2]; [C,|C|^2]; [D,|D|^2]]
//                      = -|A|^2 o(B,C,D) + |B|^2 o(A,C,D) - |C|^2 o(A,B,D)
//                        + |D|^2 o(A,B,C)      (expansion on the lift column)
//   orient2(p,a,b)     = det[A; B]
//   incirc2(p,a,b,c)   = |A|^2 o(B,C) - |B|^2 o(A,C) + |C|^2 o(A,B)
// Magnitudes: |coord| < 2^30, lifts < 2^62 (3D) / 2^61 (2D); 3x3 cofactors
// < 2^93; 4x4 terms < 2^155 (192-bit accumulator); 2D terms < 2^122.
#pragma once
#include <stdint.h>
#include <string.h>

#include "dm_predicates.cuh"

namespace dmp {

typedef __int128 i128;
typedef unsigned __int128 u128;

DM_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

// largest e with 2^e <= |f| for a finite non-zero normal float; -200 else
DM_HD int float_exponent(float f) {
  int e = (int)((f2u(f) >> 23) & 0xffu);
  return (e == 0 || e == 0xff) ? -200 : e - 127;
}

// f as an integer multiple of 2^g.  False when f is not such a multiple,
// when |f| / 2^g >= 2^62, or when f is not finite.
DM_HD bool float_to_fixed(float f, int g, long long *out) {
  uint32_t u = f2u(f);
  int e = (int)((u >> 23) & 0xffu);
  if (e == 0xff) return false;
  long long m = (long long)(u & 0x7fffffu);
  int ex;
  if (e == 0) {
    if (m == 0) {
      *out = 0;
      return true;
    }
    ex = -149;
  } else {
    m |= 0x800000;
    ex = e - 150;
  }
  int sh = ex - g;  // value = m * 2^sh at scale 2^g
  long long v;
  if (sh >= 0) {
    if (sh > 38) return false;  // m < 2^24: keeps |v| < 2^62
    v = m << sh;
  } else {
    if (sh < -24) return false;  // m != 0 here and m < 2^24
    if (m & ((1ll << -sh) - 1)) return false;
    v = m >> -sh;
  }
  *out = (u >> 31) ? -v : v;
  return true;
}

// ---- 3D ------------------------------------------------------------------
// det[a; b; c] for |coordinates| < 2^30
DM_HD i128 det3_fx(int4 a, int4 b, int4 c) {
  long long m0 = (long long)b.y * c.z - (long long)b.z * c.y;
  long long m1 = (long long)b.z * c.x - (long long)b.x * c.z;
  long long m2 = (long long)b.x * c.y - (long long)b.y * c.x;
  return (i128)a.x * m0 + (i128)a.y * m1 + (i128)a.z * m2;
}

// det[a; b; c] for |coordinates| < 2^31 (differences of fixed coordinates)
DM_HD i128 det3_fx_wide(long long a0, long long a1, long long a2, long long b0,
                        long long b1, long long b2, long long c0, long long c1,
                        long long c2) {
  i128 m0 = (i128)b1 * c2 - (i128)b2 * c1;
  i128 m1 = (i128)b2 * c0 - (i128)b0 * c2;
  i128 m2 = (i128)b0 * c1 - (i128)b1 * c0;
  return a0 * m0 + a1 * m1 + a2 * m2;
}

DM_HD int sign128(i128 v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

DM_HD int orient3_fx(int4 a, int4 b, int4 c) { return sign128(det3_fx(a, b, c)); }

// 192-bit two's complement accumulator
struct I192 {
  unsigned long long w0, w1, w2;
};

// r += l * o  (0 <= l < 2^63, |o| < 2^126)
DM_HD void mad192(I192 &r, unsigned long long l, i128 o) {
  const bool neg = o < 0;
  const u128 m = neg ? (u128)(-o) : (u128)o;
  const u128 p0 = (u128)l * (unsigned long long)m;
  const u128 p1 = (u128)l * (unsigned long long)(m >> 64);
  unsigned long long w0 = (unsigned long long)p0;
  const u128 t = (p0 >> 64) + (unsigned long long)p1;
  unsigned long long w1 = (unsigned long long)t;
  unsigned long long w2 = (unsigned long long)(p1 >> 64) + (unsigned long long)(t >> 64);
  if (neg) {
    w0 = ~w0;
    w1 = ~w1;
    w2 = ~w2;
    if (++w0 == 0 && ++w1 == 0) ++w2;
  }
  const u128 s0 = (u128)r.w0 + w0;
  const u128 s1 = (u128)r.w1 + w1 + (unsigned long long)(s0 >> 64);
  r.w0 = (unsigned long long)s0;
  r.w1 = (unsigned long long)s1;
  r.w2 = r.w2 + w2 + (unsigned long long)(s1 >> 64);
}

DM_HD int sign192(const I192 &r) {
  if ((long long)r.w2 < 0) return -1;
  return (r.w0 | r.w1 | r.w2) ? 1 : 0;
}

DM_HD unsigned long long lift3_fx(int4 a) {
  return (unsigned long long)((long long)a.x * a.x + (long long)a.y * a.y +
                              (long long)a.z * a.z);
}

// unperturbed insph3(p, a, b, c, d) with p at the origin
DM_HD int insph3_fx(int4 a, int4 b, int4 c, int4 d) {
  I192 r = {0, 0, 0};
  mad192(r, lift3_fx(a), -det3_fx(b, c, d));
  mad192(r, lift3_fx(b), det3_fx(a, c, d));
  mad192(r, lift3_fx(c), -det3_fx(a, b, d));
  mad192(r, lift3_fx(d), det3_fx(a, b, c));
  return sign192(r);
}

DM_HD bool lex_greater_fx(int4 p, int4 q) {
  if (p.x != q.x) return p.x > q.x;
  if (p.y != q.y) return p.y > q.y;
  return p.z > q.z;
}

// symbolic perturbation of insph3 (same coefficients and order as
// insph3_sos_tail): e=d: +o(A,B,C), d=c: -o(A,B,D), c=b: +o(A,C,D),
// b=a: -o(B,C,D), a=p: +o(B-A, C-A, D-A)
DM_HD int insph3_fx_sos_tail(int4 a, int4 b, int4 c, int4 d) {
  const int4 z = make_int4(0, 0, 0, 0);
  int done = 0;
  for (int step = 0; step < 5; ++step) {
    int best = -1;
    int4 bp = z;
    for (int r = 0; r < 5; ++r) {
      if (done >> r & 1) continue;
      int4 q = r == 0 ? z : r == 1 ? a : r == 2 ? b : r == 3 ? c : d;
      if (best < 0 || lex_greater_fx(q, bp)) {
        best = r;
        bp = q;
      }
    }
    done |= 1 << best;
    int s = 0;
    switch (best) {
      case 4: s = orient3_fx(a, b, c); break;
      case 3: s = -orient3_fx(a, b, d); break;
      case 2: s = orient3_fx(a, c, d); break;
      case 1: s = -orient3_fx(b, c, d); break;
      case 0:
        s = sign128(det3_fx_wide((long long)b.x - a.x, (long long)b.y - a.y,
                                 (long long)b.z - a.z, (long long)c.x - a.x,
                                 (long long)c.y - a.y, (long long)c.z - a.z,
                                 (long long)d.x - a.x, (long long)d.y - a.y,
                                 (long long)d.z - a.z));
        break;
    }
    if (s) return s;
  }
  return 0;
}

// out of line: the filters decide most calls, this keeps the kernels small
DM_HD_NI int insph3_fx_sos(int4 a, int4 b, int4 c, int4 d) {
  int s = insph3_fx(a, b, c, d);
  return s ? s : insph3_fx_sos_tail(a, b, c, d);
}

// ---- 2D ------------------------------------------------------------------
DM_HD long long det2_fx(int4 a, int4 b) {
  return (long long)a.x * b.y - (long long)a.y * b.x;
}
DM_HD int orient2_fx(int4 a, int4 b) {
  long long v = det2_fx(a, b);
  return v > 0 ? 1 : (v < 0 ? -1 : 0);
}
DM_HD long long lift2_fx(int4 a) { return (long long)a.x * a.x + (long long)a.y * a.y; }

DM_HD int incirc2_fx(int4 a, int4 b, int4 c) {
  i128 v = (i128)lift2_fx(a) * det2_fx(b, c) - (i128)lift2_fx(b) * det2_fx(a, c) +
           (i128)lift2_fx(c) * det2_fx(a, b);
  return sign128(v);
}

DM_HD bool lex_greater2_fx(int4 p, int4 q) {
  if (p.x != q.x) return p.x > q.x;
  return p.y > q.y;
}

// perturbation of incirc2 (as incirc2_sos_tail): d=c: +o(A,B), c=b: -o(A,C),
// b=a: +o(B,C), a=p: -o(B-A, C-A)
DM_HD int incirc2_fx_sos_tail(int4 a, int4 b, int4 c) {
  const int4 z = make_int4(0, 0, 0, 0);
  int done = 0;
  for (int step = 0; step < 4; ++step) {
    int best = -1;
    int4 bp = z;
    for (int r = 0; r < 4; ++r) {
      if (done >> r & 1) continue;
      int4 q = r == 0 ? z : r == 1 ? a : r == 2 ? b : c;
      if (best < 0 || lex_greater2_fx(q, bp)) {
        best = r;
        bp = q;
      }
    }
    done |= 1 << best;
    int s = 0;
    switch (best) {
      case 3: s = orient2_fx(a, b); break;
      case 2: s = -orient2_fx(a, c); break;
      case 1: s = orient2_fx(b, c); break;
      case 0: {
        long long X0 = (long long)b.x - a.x, X1 = (long long)b.y - a.y;
        long long Y0 = (long long)c.x - a.x, Y1 = (long long)c.y - a.y;
        i128 v = (i128)X0 * Y1 - (i128)X1 * Y0;
        s = -sign128(v);
        break;
      }
    }
    if (s) return s;
  }
  return 0;
}

DM_HD_NI int incirc2_fx_sos(int4 a, int4 b, int4 c) {
  int s = incirc2_fx(a, b, c);
  return s ? s : incirc2_fx_sos_tail(a, b, c);
}

}  // namespace dmp
