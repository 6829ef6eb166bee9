// Exponential of a small symmetric tridiagonal matrix applied to e_1, the
// projected step of the Krylov exponential integrators (the expm of the
// projected matrix T in scikit_tt/solvers/ode.py:1750-1752 and the Krylov
// replacement of scipy's expm_multiply, ode.py:1435 and 1525).
//
// tri_ql_warp: T = Z diag(d) Z^T by the implicit QL iteration with Wilkinson
//   shifts (Bowdler, Martin, Reinsch and Wilkinson, Numer. Math. 11 (1968)).
//   Lane 0 runs the scalar recurrence of each bulge chase and stores its
//   rotations; the whole warp then applies them to the rows of Z.
// tri_expv_apply: c = Z diag(exp(h d)) Z^T e_1, scaled by exp(max h d) so that
//   only the final factor can overflow.
#pragma once

#include <float.h>

#include "ttals_device.cuh"

namespace ttals {

// d: k diagonal entries, e: k-1 off-diagonal entries (+1 slot of work), both
// overwritten (d -> eigenvalues).  Z: k x k row-major.  rc, rs: k doubles of
// rotation storage.  Returns false when an eigenvalue needed more than 60
// iterations (uniform over the warp).
static __device__ __noinline__ bool tri_ql_warp(double* d, double* e, int k, double* Z, double* rc, double* rs) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < k * k; i += 32) Z[i] = (i / k == i % k) ? 1.0 : 0.0;
  if (lane == 0) e[k - 1] = 0.0;
  __syncwarp();
  for (int l = 0; l < k; ++l) {
    for (int iter = 0;; ++iter) {
      int m = l, lo = l, bad = 0;
      if (lane == 0) {
        for (m = l; m < k - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= DBL_EPSILON * dd) break;
        }
        if (m != l && iter >= 60) bad = 1;
        if (m != l && !bad) {
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + e[l] / (g + copysign(r, g));
          double s = 1.0, c = 1.0, p = 0.0;
          bool split = false;
          int i;
          for (i = m - 1; i >= l; --i) {
            const double f = s * e[i];
            const double b = c * e[i];
            r = hypot(f, g);
            e[i + 1] = r;
            if (r == 0.0) {
              // the chase decoupled the matrix: restart from the split
              d[i + 1] -= p;
              e[m] = 0.0;
              split = true;
              break;
            }
            s = f / r;
            c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * b;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - b;
            rc[i] = c;
            rs[i] = s;
          }
          lo = split ? i + 1 : l;
          if (!split) {
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
          }
        }
      }
      m = __shfl_sync(0xffffffffu, m, 0);
      lo = __shfl_sync(0xffffffffu, lo, 0);
      bad = __shfl_sync(0xffffffffu, bad, 0);
      if (bad) return false;
      if (m == l) break;
      __syncwarp();
      // Z <- Z G_{m-1} ... G_lo, each rotation mixing columns i and i+1
      for (int q = lane; q < k; q += 32) {
        double* zr = Z + q * k;
        for (int i = m - 1; i >= lo; --i) {
          const double f = zr[i + 1];
          zr[i + 1] = rs[i] * zr[i] + rc[i] * f;
          zr[i] = rc[i] * zr[i] - rs[i] * f;
        }
      }
      __syncwarp();
    }
  }
  __syncwarp();
  return true;
}

// c = Z diag(exp(h lam)) Z^T e_1 (k entries), computed by lane 0.  Returns
// |c| (2-norm).
static __device__ __forceinline__ double tri_expv_apply(const double* lam, const double* Z, int k, double h,
                                                        double* c) {
  double sh = -DBL_MAX;
  for (int q = 0; q < k; ++q) sh = fmax(sh, h * lam[q]);
  double nrm = 0.0;
  const double big = exp(sh);
  for (int j = 0; j < k; ++j) {
    double acc = 0.0;
    for (int q = 0; q < k; ++q) acc += Z[j * k + q] * exp(h * lam[q] - sh) * Z[q];
    c[j] = acc * big;
    nrm += c[j] * c[j];
  }
  return sqrt(nrm);
}

}  // namespace ttals
