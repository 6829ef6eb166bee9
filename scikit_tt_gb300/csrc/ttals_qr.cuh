// Householder QR executed by one CTA (any block size that is a multiple of 32).
// Column-major working copy W (rows x cols) and reflectors Vh (rows x k) live in
// global scratch (L2 resident at ALS sizes).  Reflector j: H_j = I - tau_j v_j v_j^T
// with v_j[j] = x_j - alpha_j, alpha_j = -sign(x_j) ||x||, so R[j][j] = alpha_j
// (the LAPACK sign choice).  The input may alias the Q output: it is read
// completely before the first barrier.
#pragma once

#include "ttals_internal.h"

namespace ttals {

// G: the two-group form of the batch kernels (ttals_device.cuh); false: the whole CTA.
template <bool G = false>
__device__ __forceinline__ void cta_householder_qr(const QrArgs& a) {
  const int64_t rows = a.rows, cols = a.cols;
  const int64_t k = rows < cols ? rows : cols;
  double* W = a.work;
  double* Vh = W + rows * cols;
  double* Qw = Vh + rows * k;
  double* tau = Qw + rows * k;
  const int tid = gtid<G>(), nt = gsize<G>();
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  __shared__ double red_g[kGroups<G>][32];
  __shared__ double s_alpha_g[kGroups<G>], s_tau_g[kGroups<G>], s_v0_g[kGroups<G>];
  double* red = red_g[gidx<G>()];
  double& s_alpha = s_alpha_g[gidx<G>()];
  double& s_tau = s_tau_g[gidx<G>()];
  double& s_v0 = s_v0_g[gidx<G>()];

  for (int64_t e = tid; e < rows * cols; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    W[e] = a.in[i * a.ris + c * a.rjs];
  }
  gsync<G>();

  for (int64_t j = 0; j < k; ++j) {
    const double* col = W + j * rows;
    double s = 0.0;
    for (int64_t i = j + tid; i < rows; i += nt) s += col[i] * col[i];
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    gsync<G>();
    if (tid == 0) {
      double tot = 0.0;
      for (int w = 0; w < nw; ++w) tot += red[w];
      const double x0 = col[j];
      const double nrm = sqrt(tot);
      if (nrm == 0.0) {
        s_alpha = 0.0; s_tau = 0.0; s_v0 = 1.0;
      } else {
        const double alpha = (x0 >= 0.0) ? -nrm : nrm;
        const double v0 = x0 - alpha;
        const double vn2 = tot - x0 * x0 + v0 * v0;
        s_alpha = alpha; s_v0 = v0; s_tau = (vn2 > 0.0) ? 2.0 / vn2 : 0.0;
      }
      tau[j] = s_tau;
    }
    gsync<G>();
    double* v = Vh + j * rows;
    for (int64_t i = j + tid; i < rows; i += nt) v[i] = (i == j) ? s_v0 : col[i];
    gsync<G>();
    const double tj = s_tau;
    for (int64_t c = j + 1 + warp; c < cols; c += nw) {
      double* wc = W + c * rows;
      double dot = 0.0;
      for (int64_t i = j + lane; i < rows; i += 32) dot += v[i] * wc[i];
      dot = warp_sum(dot) * tj;
      for (int64_t i = j + lane; i < rows; i += 32) wc[i] -= dot * v[i];
    }
    gsync<G>();
    if (tid == 0) W[j * rows + j] = s_alpha;
    gsync<G>();
  }

  // R (k x cols, upper trapezoidal) and optional normalisation
  double rscale = 1.0;
  if (a.normalize_r) {
    double s = 0.0;
    for (int64_t e = tid; e < k * cols; e += nt) {
      const int64_t i = e / cols, c = e % cols;
      if (i <= c) { const double v = W[c * rows + i]; s += v * v; }
    }
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    gsync<G>();
    double tot = 0.0;
    for (int w = 0; w < nw; ++w) tot += red[w];
    gsync<G>();
    const double nrm = sqrt(tot);
    if (a.rnorm && tid == 0) *a.rnorm = nrm;
    rscale = (nrm > 0.0) ? 1.0 / nrm : 1.0;
  }
  if (a.r) {
    for (int64_t e = tid; e < k * cols; e += nt) {
      const int64_t i = e / cols, c = e % cols;
      a.r[i * a.r_is + c * a.r_js] = (i <= c) ? W[c * rows + i] * rscale : 0.0;
    }
  }

  // Q = H_0 ... H_{k-1} [I_k; 0], accumulated backwards (column-major Qw)
  for (int64_t e = tid; e < rows * k; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    Qw[e] = (i == c) ? 1.0 : 0.0;
  }
  gsync<G>();
  for (int64_t j = k - 1; j >= 0; --j) {
    const double* v = Vh + j * rows;
    const double tj = tau[j];
    for (int64_t c = j + warp; c < k; c += nw) {
      double* qc = Qw + c * rows;
      double dot = 0.0;
      for (int64_t i = j + lane; i < rows; i += 32) dot += v[i] * qc[i];
      dot = warp_sum(dot) * tj;
      for (int64_t i = j + lane; i < rows; i += 32) qc[i] -= dot * v[i];
    }
    gsync<G>();
  }
  for (int64_t e = tid; e < rows * k; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    a.q[i * a.qis + c * a.qjs] = Qw[e];
  }
  gsync<G>();
}

// The same factorisation for a matrix that fits in shared memory (W: rows x
// cols doubles, column-major), in compact form: reflector j is kept below the
// diagonal of column j scaled to a unit leading entry (v / v_j, tau v_j^2, the
// LAPACK convention) and Q is formed in place, backwards, after R is written
// out.  Two group barriers per column, no global-memory round trips; the
// reflectors are the ones of cta_householder_qr (same sign choice).
constexpr int kQrSharedMaxK = 128;
template <bool G>
__device__ __noinline__ void cta_householder_qr_shared(const QrArgs& a, double* W) {
  const int64_t rows = a.rows, cols = a.cols;
  const int64_t k = rows < cols ? rows : cols;
  const int tid = gtid<G>(), nt = gsize<G>();
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  __shared__ double red_g[kGroups<G>][32];
  __shared__ double tau_g[kGroups<G>][kQrSharedMaxK];
  double* red = red_g[gidx<G>()];
  double* tau = tau_g[gidx<G>()];
  for (int64_t e = tid; e < rows * cols; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    W[e] = a.in[i * a.ris + c * a.rjs];
  }
  gsync<G>();
  for (int64_t j = 0; j < k; ++j) {
    double* col = W + j * rows;
    double s = 0.0;
    for (int64_t i = j + 1 + tid; i < rows; i += nt) s += col[i] * col[i];
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    gsync<G>();
    double sigma = 0.0;
    for (int w = 0; w < nw; ++w) sigma += red[w];
    const double x0 = col[j];
    const double nrm = sqrt(x0 * x0 + sigma);
    double alpha = 0.0, scale = 1.0, tj = 0.0;
    if (nrm != 0.0) {
      alpha = (x0 >= 0.0) ? -nrm : nrm;
      const double v0 = x0 - alpha;
      const double vn2 = sigma + v0 * v0;
      if (vn2 > 0.0 && v0 != 0.0) {
        tj = 2.0 * v0 * v0 / vn2;
        scale = 1.0 / v0;
      }
    }
    if (tid == 0) tau[j] = tj;
    for (int64_t i = j + 1 + tid; i < rows; i += nt) col[i] *= scale;
    gsync<G>();  // every thread has read x0; the scaled reflector is complete
    for (int64_t c = j + 1 + warp; c < cols; c += nw) {
      double* wc = W + c * rows;
      double dot = (lane == 0) ? wc[j] : 0.0;
      for (int64_t i = j + 1 + lane; i < rows; i += 32) dot += col[i] * wc[i];
      dot = warp_sum(dot) * tj;
      if (lane == 0) wc[j] -= dot;
      for (int64_t i = j + 1 + lane; i < rows; i += 32) wc[i] -= dot * col[i];
    }
    if (tid == 0) col[j] = alpha;
    gsync<G>();
  }
  double rscale = 1.0;
  if (a.normalize_r) {
    double s = 0.0;
    for (int64_t e = tid; e < k * cols; e += nt) {
      const int64_t i = e / cols, c = e % cols;
      if (i <= c) {
        const double v = W[c * rows + i];
        s += v * v;
      }
    }
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    gsync<G>();
    double tot = 0.0;
    for (int w = 0; w < nw; ++w) tot += red[w];
    const double nrm = sqrt(tot);
    if (a.rnorm && tid == 0) *a.rnorm = nrm;
    rscale = (nrm > 0.0) ? 1.0 / nrm : 1.0;
  }
  if (a.r) {
    for (int64_t e = tid; e < k * cols; e += nt) {
      const int64_t i = e / cols, c = e % cols;
      a.r[i * a.r_is + c * a.r_js] = (i <= c) ? W[c * rows + i] * rscale : 0.0;
    }
  }
  gsync<G>();  // R is out (and red read) before Q overwrites W
  // Q = H_0 ... H_{k-1} [I_k; 0] in place: column j becomes H_j applied to e_j
  // after H_j has been applied to the later columns (rows >= j)
  for (int64_t j = k - 1; j >= 0; --j) {
    double* col = W + j * rows;
    const double tj = tau[j];
    for (int64_t c = j + 1 + warp; c < k; c += nw) {
      double* qc = W + c * rows;
      double dot = (lane == 0) ? qc[j] : 0.0;
      for (int64_t i = j + 1 + lane; i < rows; i += 32) dot += col[i] * qc[i];
      dot = warp_sum(dot) * tj;
      if (lane == 0) qc[j] -= dot;
      for (int64_t i = j + 1 + lane; i < rows; i += 32) qc[i] -= dot * col[i];
    }
    gsync<G>();
    for (int64_t i = tid; i < rows; i += nt) col[i] = (i < j) ? 0.0 : (i == j ? 1.0 - tj : -tj * col[i]);
    gsync<G>();
  }
  for (int64_t e = tid; e < rows * k; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    a.q[i * a.qis + c * a.qjs] = W[e];
  }
  gsync<G>();
}

}  // namespace ttals
