// Symmetric tridiagonal eigen-helpers shared by the Lanczos solvers:
// Sturm-count multisection for selected eigenvalues (one warp) and inverse
// iteration for their eigenvectors (one thread).
#pragma once

#include <float.h>

#include "ttals_device.cuh"

namespace ttals {

// ---------------------------------------------------------------------------
// symmetric tridiagonal helpers (one warp)
// ---------------------------------------------------------------------------

// Number of eigenvalues of T (diag al, off-diag be) smaller than x
// (Sylvester inertia of T - x I through its LDL^T pivots).
__device__ __forceinline__ int sturm_count(const double* al, const double* be, int n, double x, double pivmin) {
  int c = 0;
  double d = al[0] - x;
  if (fabs(d) < pivmin) d = -pivmin;
  c += d < 0.0;
  for (int i = 1; i < n; ++i) {
    d = (al[i] - x) - be[i - 1] * be[i - 1] / d;
    if (fabs(d) < pivmin) d = -pivmin;
    c += d < 0.0;
  }
  return c;
}

// Eigenvalue number idx (ascending, 0-based) by 33-way multisection of
// [lo, hi] with the 32 lanes of the calling warp; uniform result.
static __device__ __noinline__ double tri_eigval(const double* al, const double* be, int n, int idx, double lo, double hi,
                             double pivmin) {
  const int lane = threadIdx.x & 31;
  for (int round = 0; round < 24; ++round) {
    const double width = hi - lo;
    if (width <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const double x = lo + width * (double)(lane + 1) / 33.0;
    const int c = sturm_count(al, be, n, x, pivmin);
    const unsigned mask = __ballot_sync(0xffffffffu, c > idx);
    const int first = mask ? (__ffs(mask) - 1) : 32;
    const double nlo = (first == 0) ? lo : lo + width * (double)first / 33.0;
    const double nhi = (first == 32) ? hi : lo + width * (double)(first + 1) / 33.0;
    lo = nlo;
    hi = nhi;
  }
  return 0.5 * (lo + hi);
}

// Inverse iteration for the eigenvector of T at theta (one thread).  Partial
// pivoting Gaussian elimination of the tridiagonal T - theta I; z (n) out,
// work: 5 n doubles + n ints.
static __device__ __noinline__ void tri_eigvec(const double* al, const double* be, int n, double theta, double tnorm, double* z,
                           double* wk, int* piv) {
  double* d = wk;
  double* du = wk + n;
  double* du2 = wk + 2 * n;
  double* dl = wk + 3 * n;
  double* b = wk + 4 * n;
  const double tiny = DBL_EPSILON * tnorm + 1e-300;
  for (int i = 0; i < n; ++i) {
    d[i] = al[i] - theta;
    du[i] = (i < n - 1) ? be[i] : 0.0;
    dl[i] = (i < n - 1) ? be[i] : 0.0;
    du2[i] = 0.0;
  }
  for (int i = 0; i < n - 1; ++i) {
    if (fabs(d[i]) >= fabs(dl[i])) {
      if (d[i] == 0.0) d[i] = tiny;
      const double fct = dl[i] / d[i];
      dl[i] = fct;
      d[i + 1] -= fct * du[i];
      piv[i] = 0;
    } else {
      const double fct = d[i] / dl[i];
      d[i] = dl[i];
      dl[i] = fct;
      const double tmp = du[i];
      du[i] = d[i + 1];
      d[i + 1] = tmp - fct * d[i + 1];
      if (i < n - 2) {
        du2[i] = du[i + 1];
        du[i + 1] = -fct * du[i + 1];
      }
      piv[i] = 1;
    }
  }
  if (d[n - 1] == 0.0) d[n - 1] = tiny;
  for (int i = 0; i < n; ++i) z[i] = 1.0 / sqrt((double)n) * (1.0 + 0.01 * (double)(i % 7));
  for (int it = 0; it < 3; ++it) {
    for (int i = 0; i < n; ++i) b[i] = z[i];
    for (int i = 0; i < n - 1; ++i) {
      if (!piv[i]) {
        b[i + 1] -= dl[i] * b[i];
      } else {
        const double t = b[i];
        b[i] = b[i + 1];
        b[i + 1] = t - dl[i] * b[i];
      }
    }
    z[n - 1] = b[n - 1] / d[n - 1];
    if (n > 1) z[n - 2] = (b[n - 2] - du[n - 2] * z[n - 1]) / d[n - 2];
    for (int i = n - 3; i >= 0; --i) z[i] = (b[i] - du[i] * z[i + 1] - du2[i] * z[i + 2]) / d[i];
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
    nrm = sqrt(nrm);
    if (!(nrm > 0.0) || !isfinite(nrm)) {
      for (int i = 0; i < n; ++i) z[i] = (i == 0) ? 1.0 : 0.0;
      return;
    }
    for (int i = 0; i < n; ++i) z[i] /= nrm;
  }
}

}  // namespace ttals
