/*
 * Gradient limiting by active-set relaxation, plain C.
 * TEST INFRASTRUCTURE ONLY (oracle of dm_limgrad).
 *
 * Restates sizing/cpp/FastHJ.cpp:63-157 of the reference: nodes of a
 * column-major (d0, d1, d2) grid are relaxed against their six axis
 * neighbours (clamped at the border, order j+1, j-1, i+1, i-1, k+1, k-1),
 *   f_hi <- f_lo + elen * dfdx   when f_hi exceeds it by more than ftol,
 * ftol = min(f) * sqrt(DBL_EPSILON); pass `it` visits, in increasing index
 * order, the nodes changed in pass it - 1 (every node in pass 0) and stops
 * when a pass changes nothing or after imax passes.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>

int oracle_limgrad(const int *dims, double elen, double dfdx, int imax, double *f) {
  const long n0 = dims[0], n1 = dims[1], n2 = dims[2];
  const long n = n0 * n1 * n2;
  int *last = (int *)malloc(sizeof(int) * n);
  long *active = (long *)malloc(sizeof(long) * n);
  if (!last || !active) {
    free(last);
    free(active);
    return -1;
  }
  double fmin = f[0];
  for (long i = 0; i < n; ++i) {
    last[i] = -1;
    if (f[i] < fmin) fmin = f[i];
  }
  const double ftol = fmin * sqrt(DBL_EPSILON);
  const double step = elen * dfdx;
  int passes = 0;
  for (int it = 0; it < imax; ++it) {
    long na = 0;
    for (long i = 0; i < n; ++i)
      if (last[i] == it - 1) active[na++] = i;
    if (na == 0) break;
    ++passes;
    for (long q = 0; q < na; ++q) {
      long node = active[q];
      long i = node % n0, j = (node / n0) % n1, k = node / (n0 * n1);
      long nb[6];
      long jp = j + 1 < n1 ? j + 1 : n1 - 1, jm = j - 1 >= 0 ? j - 1 : 0;
      long ip = i + 1 < n0 ? i + 1 : n0 - 1, im = i - 1 >= 0 ? i - 1 : 0;
      long kp = k + 1 < n2 ? k + 1 : n2 - 1, km = k - 1 >= 0 ? k - 1 : 0;
      nb[0] = i + n0 * (jp + n1 * k);
      nb[1] = i + n0 * (jm + n1 * k);
      nb[2] = ip + n0 * (j + n1 * k);
      nb[3] = im + n0 * (j + n1 * k);
      nb[4] = i + n0 * (j + n1 * kp);
      nb[5] = i + n0 * (j + n1 * km);
      for (int u = 0; u < 6; ++u) {
        long other = nb[u];
        if (f[node] > f[other]) {
          double lim = f[other] + step;
          if (f[node] > lim + ftol) {
            f[node] = lim;
            last[node] = it;
          }
        } else {
          double lim = f[node] + step;
          if (f[other] > lim + ftol) {
            f[other] = lim;
            last[other] = it;
          }
        }
      }
    }
  }
  free(last);
  free(active);
  return passes;
}
