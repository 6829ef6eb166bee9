// Exponential of a small symmetric tridiagonal matrix applied to e_1, the
// projected step of the Krylov exponential integrators (the expm of the
// projected matrix T in scikit_tt/solvers/ode.py:1750-1752 and the Krylov
// replacement of scipy's expm_multiply, ode.py:1435 and 1525).
//
// tri_expv_warp: c = exp(h T) e_1 by the truncated Taylor series with scaling
//   (the method family of scipy's expm_multiply, Al-Mohy and Higham 2011):
//   h T is split into s pieces with |h T / s|_inf <= 1/2, and each piece's
//   series is cut after 16 terms (remainder <= 0.5^17 / 17! e^0.5 < 2^-60 of
//   the piece's result, whose norm is at least e^-0.5 of its input).  One warp:
//   lane L holds entries 2L and 2L+1 (k <= 64), a tridiagonal product is two
//   shuffles and three FMAs per entry, so a check costs a few hundred cycles
//   (an eigendecomposition by a serial QL chase costs 10^5 here: FP64
//   division and square root run at a small fraction of the FMA rate).
#pragma once

#include <float.h>

#include "ttals_device.cuh"

namespace ttals {

// 1 / q for q = 0..17 (entry 0 unused)
__device__ __constant__ const double kInvInt[18] = {0.0,       1.0,        1.0 / 2,  1.0 / 3,  1.0 / 4,  1.0 / 5,
                                                    1.0 / 6,   1.0 / 7,    1.0 / 8,  1.0 / 9,  1.0 / 10, 1.0 / 11,
                                                    1.0 / 12,  1.0 / 13,   1.0 / 14, 1.0 / 15, 1.0 / 16, 1.0 / 17};

// al: k diagonal entries, be: k-1 off-diagonal entries (be[i] couples i and
// i+1).  c: k outputs (written by the lanes owning them).  Returns |c|_2 to
// every lane; false in *ok when the scaling would need more than 2^16 pieces
// or the result is not finite.
static __device__ __noinline__ double tri_expv_warp(const double* al, const double* be, int k, double h, double* c,
                                                    bool* ok) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int i0 = 2 * lane, i1 = 2 * lane + 1;
  // local entries of h T (zero outside k)
  const double a0 = i0 < k ? h * al[i0] : 0.0, a1 = i1 < k ? h * al[i1] : 0.0;
  const double b0 = i0 + 1 < k ? h * be[i0] : 0.0;   // couples i0, i1
  const double b1 = i1 + 1 < k ? h * be[i1] : 0.0;   // couples i1, i1+1 (next lane's i0)
  const double bm = __shfl_up_sync(full, b1, 1);     // couples i0-1, i0
  const double bmin = lane > 0 ? bm : 0.0;
  double nrm = fmax(fabs(a0) + fabs(b0) + fabs(bmin), fabs(a1) + fabs(b0) + fabs(b1));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nrm = fmax(nrm, __shfl_xor_sync(full, nrm, o));
  double s = ceil(2.0 * nrm);
  if (!(s >= 1.0)) s = 1.0;
  *ok = s <= 65536.0;
  const int pieces = *ok ? (int)s : 1;
  const double inv = 1.0 / (double)pieces;
  double x0 = lane == 0 ? 1.0 : 0.0, x1 = 0.0;  // e_1
  for (int p = 0; p < pieces; ++p) {
    double t0 = x0, t1 = x1, s0 = x0, s1 = x1;
    double f = inv;  // inv / q
#pragma unroll 4
    for (int q = 1; q <= 16; ++q) {
      // t_q = (h T / pieces)^q e / q!, accumulated into s
      const double left = __shfl_up_sync(full, t1, 1);    // t[i0 - 1]
      const double right = __shfl_down_sync(full, t0, 1); // t[i1 + 1]
      const double n0 = (a0 * t0 + b0 * t1 + (lane > 0 ? bmin * left : 0.0)) * f;
      const double n1 = (a1 * t1 + b0 * t0 + (lane < 31 ? b1 * right : 0.0)) * f;
      t0 = n0;
      t1 = n1;
      s0 += t0;
      s1 += t1;
      f = inv * kInvInt[q + 1];
    }
    x0 = s0;
    x1 = s1;
  }
  if (i0 < k) c[i0] = x0;
  if (i1 < k) c[i1] = x1;
  double n2 = (i0 < k ? x0 * x0 : 0.0) + (i1 < k ? x1 * x1 : 0.0);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(full, n2, o);
  __syncwarp();
  const double cn = sqrt(n2);
  if (!isfinite(cn)) *ok = false;
  return cn;
}

}  // namespace ttals
