// Small nonsymmetric (upper Hessenberg) eigen-helpers for the Arnoldi mode of
// the local eigensolver:
//
// * hess_eigvals_warp: all eigenvalues of an n x n upper Hessenberg matrix by
//   the implicitly double-shifted Francis QR iteration (eigenvalues only, so
//   each bulge-chasing step touches only the active block).  Shifts are the
//   eigenvalues of the trailing 2 x 2 block, with the customary exceptional
//   shifts after 10 and 20 iterations without deflation; a subdiagonal entry
//   is set to zero once it is below machine epsilon times its two diagonal
//   neighbours.  One warp: the row and column updates of every 3 x 3
//   Householder reflector are spread over the lanes, all scalar work is done
//   redundantly by every lane (uniform control flow).
// * hess_eigvec: eigenvector of H at a real Ritz value theta by inverse
//   iteration with the O(n^2) partially pivoted LU of the Hessenberg H - theta I
//   (one thread).
//
// These replace the dense LAPACK geev call of scikit_tt/solvers/evp.py:423 on
// the projected (Arnoldi) matrix, which is at most a few dozen rows.
#pragma once

#include <float.h>

#include "ttals_device.cuh"

namespace ttals {

// H: row-major with leading dimension ld, destroyed.  Returns false when some
// eigenvalue needed more than 60 iterations.
static __device__ __noinline__ bool hess_eigvals_warp(double* H, int ld, int n, double* wr, double* wi) {
  const int lane = threadIdx.x & 31;
  auto h = [&](int i, int j) -> double& { return H[(int64_t)i * ld + j]; };
  double anorm = 0.0;
  for (int i = lane; i < n; i += 32)
    for (int j = (i > 0 ? i - 1 : 0); j < n; ++j) anorm += fabs(h(i, j));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) anorm += __shfl_xor_sync(0xffffffffu, anorm, o);
  __syncwarp();
  int nn = n - 1;
  double t = 0.0;
  while (nn >= 0) {
    int its = 0;
    for (;;) {
      int l;
      for (l = nn; l >= 1; --l) {
        double s = fabs(h(l - 1, l - 1)) + fabs(h(l, l));
        if (s == 0.0) s = anorm;
        if (fabs(h(l, l - 1)) <= DBL_EPSILON * s) break;
      }
      __syncwarp();
      if (l >= 1 && lane == 0) h(l, l - 1) = 0.0;
      __syncwarp();
      double x = h(nn, nn);
      if (l == nn) {
        if (lane == 0) {
          wr[nn] = x + t;
          wi[nn] = 0.0;
        }
        --nn;
        break;
      }
      double y = h(nn - 1, nn - 1);
      double w = h(nn, nn - 1) * h(nn - 1, nn);
      if (l == nn - 1) {
        const double p = 0.5 * (y - x);
        const double q = p * p + w;
        double z = sqrt(fabs(q));
        x += t;
        if (lane == 0) {
          if (q >= 0.0) {
            z = p + copysign(z, p);
            wr[nn - 1] = wr[nn] = x + z;
            if (z != 0.0) wr[nn] = x - w / z;
            wi[nn - 1] = wi[nn] = 0.0;
          } else {
            wr[nn - 1] = wr[nn] = x + p;
            wi[nn - 1] = -z;
            wi[nn] = z;
          }
        }
        nn -= 2;
        break;
      }
      if (its == 60) {
        __syncwarp();
        return false;
      }
      if (its == 10 || its == 20) {
        t += x;
        __syncwarp();
        for (int i = lane; i <= nn; i += 32) h(i, i) -= x;
        __syncwarp();
        const double s = fabs(h(nn, nn - 1)) + fabs(h(nn - 1, nn - 2));
        x = y = 0.75 * s;
        w = -0.4375 * s * s;
      }
      ++its;
      // start of the double-shift sweep: two consecutive small subdiagonals
      int m;
      double p = 0.0, q = 0.0, r = 0.0, z;
      for (m = nn - 2; m >= l; --m) {
        z = h(m, m);
        r = x - z;
        double s = y - z;
        p = (r * s - w) / h(m + 1, m) + h(m, m + 1);
        q = h(m + 1, m + 1) - z - r - s;
        r = h(m + 2, m + 1);
        s = fabs(p) + fabs(q) + fabs(r);
        p /= s;
        q /= s;
        r /= s;
        if (m == l) break;
        const double u = fabs(h(m, m - 1)) * (fabs(q) + fabs(r));
        const double v = fabs(p) * (fabs(h(m - 1, m - 1)) + fabs(z) + fabs(h(m + 1, m + 1)));
        if (u <= DBL_EPSILON * v) break;
      }
      __syncwarp();
      for (int i = m + 2 + lane; i <= nn; i += 32) {
        h(i, i - 2) = 0.0;
        if (i != m + 2) h(i, i - 3) = 0.0;
      }
      __syncwarp();
      for (int k = m; k <= nn - 1; ++k) {
        if (k != m) {
          p = h(k, k - 1);
          q = h(k + 1, k - 1);
          r = (k != nn - 1) ? h(k + 2, k - 1) : 0.0;
          x = fabs(p) + fabs(q) + fabs(r);
          if (x != 0.0) {
            p /= x;
            q /= x;
            r /= x;
          }
        }
        const double s = copysign(sqrt(p * p + q * q + r * r), p);
        __syncwarp();
        if (s != 0.0) {
          if (lane == 0) {
            if (k == m) {
              if (l != m) h(k, k - 1) = -h(k, k - 1);
            } else {
              h(k, k - 1) = -s * x;
            }
          }
          p += s;
          x = p / s;
          y = q / s;
          z = r / s;
          q /= p;
          r /= p;
          __syncwarp();
          for (int j = k + lane; j <= nn; j += 32) {
            double pp = h(k, j) + q * h(k + 1, j);
            if (k != nn - 1) {
              pp += r * h(k + 2, j);
              h(k + 2, j) -= pp * z;
            }
            h(k + 1, j) -= pp * y;
            h(k, j) -= pp * x;
          }
          __syncwarp();
          const int mmin = nn < k + 3 ? nn : k + 3;
          for (int i = l + lane; i <= mmin; i += 32) {
            double pp = x * h(i, k) + y * h(i, k + 1);
            if (k != nn - 1) {
              pp += z * h(i, k + 2);
              h(i, k + 2) -= pp * r;
            }
            h(i, k + 1) -= pp * q;
            h(i, k) -= pp;
          }
          __syncwarp();
        }
      }
    }
  }
  __syncwarp();
  return true;
}

// Unit eigenvector z of the n x n Hessenberg H (row-major, ld) for the real
// eigenvalue theta: inverse iteration, three steps.  U: n*n doubles of work
// (row-major, leading dimension n), piv: n ints.  One thread.
static __device__ __noinline__ void hess_eigvec(const double* H, int ld, int n, double theta, double hnorm, double* z,
                                                double* U, int* piv) {
  const double tiny = DBL_EPSILON * hnorm + 1e-300;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) U[i * n + j] = (j >= i - 1) ? H[(int64_t)i * ld + j] - (i == j ? theta : 0.0) : 0.0;
  // LU with partial pivoting; only rows i and i+1 compete for the pivot of column i
  for (int i = 0; i < n - 1; ++i) {
    piv[i] = 0;
    if (fabs(U[(i + 1) * n + i]) > fabs(U[i * n + i])) {
      piv[i] = 1;
      for (int j = i; j < n; ++j) {
        const double tmp = U[i * n + j];
        U[i * n + j] = U[(i + 1) * n + j];
        U[(i + 1) * n + j] = tmp;
      }
    }
    if (U[i * n + i] == 0.0) U[i * n + i] = tiny;
    const double li = U[(i + 1) * n + i] / U[i * n + i];
    for (int j = i + 1; j < n; ++j) U[(i + 1) * n + j] -= li * U[i * n + j];
    U[(i + 1) * n + i] = li;
  }
  if (U[(n - 1) * n + n - 1] == 0.0) U[(n - 1) * n + n - 1] = tiny;
  for (int i = 0; i < n; ++i) z[i] = 1.0 / sqrt((double)n) * (1.0 + 0.01 * (double)(i % 7));
  for (int it = 0; it < 3; ++it) {
    // forward: apply the row swaps and the unit lower bidiagonal factor
    for (int i = 0; i < n - 1; ++i) {
      if (piv[i]) {
        const double tmp = z[i];
        z[i] = z[i + 1];
        z[i + 1] = tmp;
      }
      z[i + 1] -= U[(i + 1) * n + i] * z[i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double acc = z[i];
      for (int j = i + 1; j < n; ++j) acc -= U[i * n + j] * z[j];
      z[i] = acc / U[i * n + i];
    }
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
