// Rank-r orthonormal bases of the local eigenvector blocks (number_ev > 1).
//
// The reference re-gauges a block of k local eigenvectors by an SVD and keeps
// the r leading singular vectors (scikit_tt/solvers/evp.py:455-468 forward:
// left singular vectors of the (a n) x (s k) reshape, r = min(s, u.shape[1]);
// evp.py:470-486 backward: right singular vectors of the (k a) x (n s)
// reshape of the transposed block, r = min(a, v.shape[0])).  Only the spanned
// subspace matters to the sweep (the next micro problem is a Galerkin
// projection onto it), so this kernel computes an orthonormal basis of the
// same r-dimensional dominant singular subspace without a full SVD:
//
//   * the Gram matrix of the smaller side (at most a few hundred rows) is
//     diagonalised by the cyclic Jacobi method, parallel over disjoint
//     rotation pairs (round-robin ordering), one CTA;
//   * if the Gram matrix lives on the wanted side its r leading eigenvectors
//     are the basis; otherwise they are mapped through M and re-orthonormalised
//     by Householder QR (span(M w_1..w_r) = span(u_1..u_r)).
#include <float.h>

#include <algorithm>

#include "ttals_internal.h"
#include "ttals_qr.cuh"

namespace ttals {

constexpr int kTrThreads = 1024;
constexpr int kTrMaxGram = 1024;

struct TruncK {
  const double* M;  // row-major p x q, or (transposed) the N x k eigenvector block, see tr
  int64_t p, q;
  int tr_k;         // > 0: M(x, y) = E[(ai * q + y) * tr_k + e], x = e * (p / tr_k) + ai
  int r, side;      // side 0: left basis (p x r) out; 1: right basis (r x q) out
  double* G;        // n x n
  double* V;        // n x n
  double* B;        // max(p, q) x r
  double* qrwork;
  double* out;
  int* status;
};

__device__ __forceinline__ double tr_get(const TruncK& a, int64_t x, int64_t y) {
  if (a.tr_k > 0) {
    const int64_t pa = a.p / a.tr_k;
    const int64_t e = x / pa, ai = x - e * pa;
    return a.M[(ai * a.q + y) * a.tr_k + e];
  }
  return a.M[x * a.q + y];
}

__global__ void __launch_bounds__(kTrThreads) trunc_basis_kernel(TruncK a) {
  __shared__ double s_c[kTrMaxGram / 2], s_s[kTrMaxGram / 2];
  __shared__ int s_a[kTrMaxGram / 2], s_b[kTrMaxGram / 2];
  __shared__ double red[64];
  __shared__ int s_sel[kTrMaxGram];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int64_t p = a.p, q = a.q;
  // Gram side: gram_rows = true -> G = M M^T (p x p), else G = M^T M (q x q)
  const bool gram_rows = p <= q;
  const int n = (int)(gram_rows ? p : q);
  const int64_t other = gram_rows ? q : p;
  double* G = a.G;
  double* V = a.V;
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    if (j < i) continue;
    double acc = 0.0;
    for (int64_t z = 0; z < other; ++z)
      acc += gram_rows ? tr_get(a, i, z) * tr_get(a, j, z) : tr_get(a, z, i) * tr_get(a, z, j);
    G[(int64_t)i * n + j] = acc;
    G[(int64_t)j * n + i] = acc;
  }
  for (int64_t e = tid; e < (int64_t)n * n; e += nt) V[e] = (e / n == e % n) ? 1.0 : 0.0;
  __syncthreads();
  // cyclic Jacobi, round-robin pairs over nn (even) positions; position n is a dummy
  const int nn = (n + 1) & ~1;
  const int npairs = nn / 2;
  for (int sweep = 0; sweep < 40 && n > 1; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int64_t e = tid; e < (int64_t)n * n; e += nt) {
      const double g = G[e];
      if (e / n == e % n) dia += g * g;
      else off += g * g;
    }
    off = warp_sum(off);
    dia = warp_sum(dia);
    if (lane == 0) {
      red[warp] = off;
      red[32 + warp] = dia;
    }
    __syncthreads();
    double to = 0.0, td = 0.0;
    for (int w = 0; w < (nt >> 5); ++w) {
      to += red[w];
      td += red[32 + w];
    }
    __syncthreads();
    if (!(to > 1e-30 * td) || !(td > 0.0)) break;
    for (int step = 0; step < nn - 1; ++step) {
      for (int pi = tid; pi < npairs; pi += nt) {
        auto pos = [&](int j) { return j == 0 ? 0 : ((j - 1 + step) % (nn - 1)) + 1; };
        int ia = pos(pi), ib = pos(nn - 1 - pi);
        if (ia > ib) {
          const int t = ia;
          ia = ib;
          ib = t;
        }
        double c = 1.0, s = 0.0;
        if (ib < n) {
          const double apq = G[(int64_t)ia * n + ib];
          if (apq != 0.0) {
            const double tau = (G[(int64_t)ib * n + ib] - G[(int64_t)ia * n + ia]) / (2.0 * apq);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        }
        s_a[pi] = ia;
        s_b[pi] = ib;
        s_c[pi] = c;
        s_s[pi] = s;
      }
      __syncthreads();
      // rows: G <- J^T G
      for (int64_t e = tid; e < (int64_t)npairs * n; e += nt) {
        const int pi = (int)(e / n), j = (int)(e - (int64_t)pi * n);
        const int ia = s_a[pi], ib = s_b[pi];
        if (ib >= n || s_s[pi] == 0.0) continue;
        const double c = s_c[pi], s = s_s[pi];
        const double ga = G[(int64_t)ia * n + j], gb = G[(int64_t)ib * n + j];
        G[(int64_t)ia * n + j] = c * ga - s * gb;
        G[(int64_t)ib * n + j] = s * ga + c * gb;
      }
      __syncthreads();
      // columns: G <- G J, V <- V J
      for (int64_t e = tid; e < (int64_t)npairs * n; e += nt) {
        const int pi = (int)(e / n), i = (int)(e - (int64_t)pi * n);
        const int ia = s_a[pi], ib = s_b[pi];
        if (ib >= n || s_s[pi] == 0.0) continue;
        const double c = s_c[pi], s = s_s[pi];
        const double ga = G[(int64_t)i * n + ia], gb = G[(int64_t)i * n + ib];
        G[(int64_t)i * n + ia] = c * ga - s * gb;
        G[(int64_t)i * n + ib] = s * ga + c * gb;
        const double va = V[(int64_t)i * n + ia], vb = V[(int64_t)i * n + ib];
        V[(int64_t)i * n + ia] = c * va - s * vb;
        V[(int64_t)i * n + ib] = s * va + c * vb;
      }
      __syncthreads();
    }
  }
  // the r largest eigenvalues, descending
  const int r = a.r;
  if (tid == 0) {
    for (int i = 0; i < n; ++i) s_sel[i] = i;
    for (int c = 0; c < r; ++c) {
      int best = c;
      for (int i = c + 1; i < n; ++i)
        if (G[(int64_t)s_sel[i] * n + s_sel[i]] > G[(int64_t)s_sel[best] * n + s_sel[best]]) best = i;
      const int t = s_sel[c];
      s_sel[c] = s_sel[best];
      s_sel[best] = t;
    }
  }
  __syncthreads();
  const bool direct = (a.side == 0) == gram_rows;  // eigenvectors already on the wanted side
  if (direct) {
    if (a.side == 0) {
      for (int64_t e = tid; e < p * r; e += nt) {
        const int64_t x = e / r;
        const int c = (int)(e - x * r);
        a.out[e] = V[x * n + s_sel[c]];
      }
    } else {
      for (int64_t e = tid; e < (int64_t)r * q; e += nt) {
        const int c = (int)(e / q);
        const int64_t y = e - (int64_t)c * q;
        a.out[e] = V[y * n + s_sel[c]];
      }
    }
    return;
  }
  // map through M: B = M W (left side wanted, Gram of columns) or M^T Y (right side wanted)
  const int64_t rows = a.side == 0 ? p : q;
  for (int64_t e = tid; e < rows * r; e += nt) {
    const int64_t x = e / r;
    const int c = (int)(e - x * r);
    const int col = s_sel[c];
    double acc = 0.0;
    if (a.side == 0)
      for (int64_t y = 0; y < q; ++y) acc += tr_get(a, x, y) * V[y * n + col];
    else
      for (int64_t y = 0; y < p; ++y) acc += tr_get(a, y, x) * V[y * n + col];
    a.B[e] = acc;
  }
  __syncthreads();
  // Householder QR of B (rows x r); Q -> out (p x r) or out^T (r x q)
  QrArgs qa{a.B, r, 1, a.out, a.side == 0 ? r : 1, a.side == 0 ? 1 : q, a.G, r, 1, rows, r, 0, nullptr, a.qrwork};
  cta_householder_qr(qa);
}

size_t trunc_work_doubles(int64_t p, int64_t q, int64_t r) {
  const int64_t n = p < q ? p : q, rows = p > q ? p : q;
  return (size_t)(2 * n * n + rows * r + (rows * r + 2 * rows * r + r) + 64);
}

cudaError_t launch_trunc_basis(const double* M, int64_t p, int64_t q, int tr_k, int r, int side, double* work,
                               double* out, int* status, cudaStream_t st) {
  const int64_t n = p < q ? p : q, rows = p > q ? p : q;
  if (n > kTrMaxGram || r < 1 || r > n) return cudaErrorInvalidValue;
  TruncK a{};
  a.M = M;
  a.p = p;
  a.q = q;
  a.tr_k = tr_k;
  a.r = r;
  a.side = side;
  a.G = work;
  a.V = a.G + n * n;
  a.B = a.V + n * n;
  a.qrwork = a.B + rows * r;
  a.out = out;
  a.status = status;
  trunc_basis_kernel<<<1, kTrThreads, 0, st>>>(a);
  ++launch_counter();
  return cudaGetLastError();
}

}  // namespace ttals

namespace ttals {

// ---------------------------------------------------------------------------
// Truncated SVD of one TT core (TT.ortho_left / ortho_right with threshold or
// max_rank, scikit_tt/tensor_train.py:1150-1181 and 1262-1296).
//
// One-sided (Hestenes) Jacobi on the columns of X = M (q <= p) or X = M^T:
// column pairs are rotated until mutually orthogonal to machine precision;
// then the column norms are the singular values (computed to high relative
// accuracy, which the relative cut sigma_i / sigma_0 > threshold needs), the
// normalised columns the left singular vectors of X and the accumulated
// rotations its right singular vectors.  Rotation pairs follow the round-robin
// ordering, one warp per pair, one CTA.  Kept rank k = #{sigma_i / sigma_0 >
// threshold} (all when threshold == 0), capped at max_rank, at least 1.
// Outputs for M = U S V^T:
//   side 0 (left):  core = U (p x k),    r = S V^T (k x q)
//   side 1 (right): core = V^T (k x q),  r = U S (p x k)
// ---------------------------------------------------------------------------

struct SvdK {
  const double* M;   // p x q row-major
  int64_t p, q;
  int side;
  double threshold;
  int64_t max_rank;  // <= 0: no cap
  double* W;         // working columns, n_rows x ncols column-major
  double* Vr;        // ncols x ncols rotations (column-major)
  double* core;
  double* r;
  int* kept;         // out: k
  int* status;
  float* W32;        // FP32 copies for the preconditioning sweeps
  float* V32;
  int in_smem;       // bits: 1 W, 2 W32, 4 Vr, 8 V32 in dynamic shared memory (in that order)
  const int* skip;   // nonzero *skip: the factorisation is not needed (return at once); may be null
};

__global__ void __launch_bounds__(kTrThreads) svd_trunc_kernel(SvdK a) {
  if (a.skip && *a.skip) return;
  extern __shared__ double s_dyn[];
  __shared__ int s_a[kTrMaxGram / 2], s_b[kTrMaxGram / 2];
  __shared__ double s_sig[kTrMaxGram];
  __shared__ int s_ord[kTrMaxGram];
  __shared__ int s_rot;
  __shared__ int s_k;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const bool tr = a.q > a.p;                 // work on M^T when M is wide
  const int64_t rows = tr ? a.q : a.p;       // length of a working column
  const int ncols = (int)(tr ? a.p : a.q);   // number of working columns
  // the rotation steps re-read every column: shared memory where it fits
  char* sp = reinterpret_cast<char*>(s_dyn);
  auto carve = [&](int bit, int64_t bytes) {
    char* p = sp;
    if (a.in_smem & bit) sp += (bytes + 7) / 8 * 8;
    return p;
  };
  double* W = (a.in_smem & 1) ? reinterpret_cast<double*>(carve(1, 8 * rows * ncols)) : a.W;
  float* W32 = (a.in_smem & 2) ? reinterpret_cast<float*>(carve(2, 4 * rows * ncols)) : a.W32;
  double* V = (a.in_smem & 4) ? reinterpret_cast<double*>(carve(4, 8 * (int64_t)ncols * ncols)) : a.Vr;
  float* V32 = (a.in_smem & 8) ? reinterpret_cast<float*>(carve(8, 4 * (int64_t)ncols * ncols)) : a.V32;
  for (int64_t e = tid; e < rows * ncols; e += nt) {
    const int64_t c = e / rows, i = e - c * rows;
    W[e] = tr ? a.M[c * a.q + i] : a.M[i * a.q + c];
  }
  for (int64_t e = tid; e < (int64_t)ncols * ncols; e += nt) V[e] = (e / ncols == e % ncols) ? 1.0 : 0.0;
  // |M|_F^2: columns below 1e-30 of it (singular values below 1e-15 |M|) are
  // rounding noise that a rotation only regenerates; rotations of such pairs
  // do not keep the sweeps going
  __shared__ double s_red[32], s_fro2;
  {
    double f2 = 0.0;
    for (int64_t e = tid; e < rows * ncols; e += nt) f2 += W[e] * W[e];
    f2 = warp_sum(f2);
    if (lane == 0) s_red[warp] = f2;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += s_red[w];
      s_fro2 = t;
    }
  }
  __syncthreads();
  const double live_floor = 1e-30 * s_fro2;
  const int nn = (ncols + 1) & ~1, npairs = nn / 2;
  // pair (ia, ib) of warp-slot pi in round-robin step `step`
  auto pair_of = [&](int pi, int step, int& ia, int& ib) {
    auto pos = [&](int j) { return j == 0 ? 0 : ((j - 1 + step) % (nn - 1)) + 1; };
    ia = pos(pi);
    ib = pos(nn - 1 - pi);
    if (ia > ib) {
      const int t = ia;
      ia = ib;
      ib = t;
    }
  };
  if (ncols > 1) {
    // Preconditioning in FP32 (57x the FP64 rate here): Jacobi sweeps on a
    // power-of-two scaled FP32 copy until the columns are orthogonal to ~1e-6,
    // then V = the FP32 rotations re-orthonormalised in FP64 and W = M V in
    // FP64.  The FP64 sweeps below start from nearly orthogonal columns; their
    // stopping rule and accuracy are unchanged.
    double amax = 0.0;
    for (int64_t e = tid; e < rows * ncols; e += nt) amax = fmax(amax, fabs(W[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) s_red[warp] = amax;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t = fmax(t, s_red[w]);
      s_red[0] = t;
    }
    __syncthreads();
    const double sc = s_red[0] > 0.0 ? ldexp(1.0, -ilogb(s_red[0])) : 1.0;
    for (int64_t e = tid; e < rows * ncols; e += nt) W32[e] = (float)(W[e] * sc);
    for (int64_t e = tid; e < (int64_t)ncols * ncols; e += nt) V32[e] = (e / ncols == e % ncols) ? 1.f : 0.f;
    const float live32 = (float)(1e-12 * s_fro2 * sc * sc);
    __syncthreads();
    for (int sweep = 0; sweep < 40; ++sweep) {
      if (tid == 0) s_rot = 0;
      __syncthreads();
      for (int step = 0; step < nn - 1; ++step) {
        for (int pi = warp; pi < npairs; pi += nw) {
          int ia, ib;
          pair_of(pi, step, ia, ib);
          if (ib >= ncols) continue;
          float* ca = W32 + (int64_t)ia * rows;
          float* cb = W32 + (int64_t)ib * rows;
          float al = 0.f, be = 0.f, ga = 0.f;
          for (int64_t i = lane; i < rows; i += 32) {
            al += ca[i] * ca[i];
            be += cb[i] * cb[i];
            ga += ca[i] * cb[i];
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            al += __shfl_xor_sync(0xffffffffu, al, o);
            be += __shfl_xor_sync(0xffffffffu, be, o);
            ga += __shfl_xor_sync(0xffffffffu, ga, o);
          }
          if (ga != 0.f && ga * ga > 1e-12f * al * be) {
            const float zeta = (be - al) / (2.f * ga);
            const float t = fabsf(zeta) > 1e18f ? 0.5f / zeta
                                                : (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
            const float cs = rsqrtf(1.f + t * t), sn = cs * t;
            for (int64_t i = lane; i < rows; i += 32) {
              const float x = ca[i], y = cb[i];
              ca[i] = cs * x - sn * y;
              cb[i] = sn * x + cs * y;
            }
            float* va = V32 + (int64_t)ia * ncols;
            float* vb = V32 + (int64_t)ib * ncols;
            for (int i = lane; i < ncols; i += 32) {
              const float x = va[i], y = vb[i];
              va[i] = cs * x - sn * y;
              vb[i] = sn * x + cs * y;
            }
            // a sweep whose live pairs were all within 1e-3 leaves them within ~1e-6
            if (lane == 0 && fminf(al, be) > live32 && ga * ga > 1e-6f * al * be) s_rot = 1;
          }
        }
        __syncthreads();
      }
      if (!s_rot) break;
      __syncthreads();
    }
    // V = FP64 Gram-Schmidt (two passes) of the FP32 rotations, column by column
    __shared__ double s_d[kTrMaxGram];
    for (int c = 0; c < ncols; ++c) {
      double* vc = V + (int64_t)c * ncols;
      for (int i = tid; i < ncols; i += nt) vc[i] = (double)V32[(int64_t)c * ncols + i];
      __syncthreads();
      for (int pass = 0; pass < 2 && c > 0; ++pass) {
        for (int q = warp; q < c; q += nw) {
          const double* vq = V + (int64_t)q * ncols;
          double dt = 0.0;
          for (int i = lane; i < ncols; i += 32) dt += vq[i] * vc[i];
          dt = warp_sum(dt);
          if (lane == 0) s_d[q] = dt;
        }
        __syncthreads();
        for (int i = tid; i < ncols; i += nt) {
          double acc = vc[i];
          for (int q = 0; q < c; ++q) acc -= s_d[q] * V[(int64_t)q * ncols + i];
          vc[i] = acc;
        }
        __syncthreads();
      }
      double n2 = 0.0;
      for (int i = tid; i < ncols; i += nt) n2 += vc[i] * vc[i];
      n2 = warp_sum(n2);
      if (lane == 0) s_red[warp] = n2;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += s_red[w];
        s_red[0] = t > 0.0 ? 1.0 / sqrt(t) : 0.0;
      }
      __syncthreads();
      const double inv = s_red[0];
      for (int i = tid; i < ncols; i += nt) vc[i] *= inv;
      __syncthreads();
    }
    // W = M V (working orientation of M): from the FP64 copy when W sits in
    // shared memory (the global work area is free then), else from M
    if (a.in_smem & 1) {
      for (int64_t e = tid; e < rows * ncols; e += nt) {
        const int64_t c = e / rows, i = e - c * rows;
        const double* vc = V + c * ncols;
        double acc = 0.0;
        for (int q = 0; q < ncols; ++q) acc += W[(int64_t)q * rows + i] * vc[q];
        a.W[e] = acc;
      }
      __syncthreads();
      for (int64_t e = tid; e < rows * ncols; e += nt) W[e] = a.W[e];
    } else {
      for (int64_t e = tid; e < rows * ncols; e += nt) {
        const int64_t c = e / rows, i = e - c * rows;
        const double* vc = V + c * ncols;
        double acc = 0.0;
        for (int q = 0; q < ncols; ++q) acc += (tr ? a.M[(int64_t)q * a.q + i] : a.M[i * a.q + q]) * vc[q];
        W[e] = acc;
      }
    }
    __syncthreads();
  }
  for (int sweep = 0; sweep < 60 && ncols > 1; ++sweep) {
    if (tid == 0) s_rot = 0;
    __syncthreads();
    for (int step = 0; step < nn - 1; ++step) {
      if (tid < npairs) {
        auto pos = [&](int j) { return j == 0 ? 0 : ((j - 1 + step) % (nn - 1)) + 1; };
        int ia = pos(tid), ib = pos(nn - 1 - tid);
        if (ia > ib) {
          const int t = ia;
          ia = ib;
          ib = t;
        }
        s_a[tid] = ia;
        s_b[tid] = ib;
      }
      __syncthreads();
      for (int pi = warp; pi < npairs; pi += nw) {
        const int ia = s_a[pi], ib = s_b[pi];
        if (ib >= ncols) continue;
        double* ca = W + (int64_t)ia * rows;
        double* cb = W + (int64_t)ib * rows;
        double alpha = 0.0, beta = 0.0, gamma = 0.0;
        for (int64_t i = lane; i < rows; i += 32) {
          alpha += ca[i] * ca[i];
          beta += cb[i] * cb[i];
          gamma += ca[i] * cb[i];
        }
        alpha = warp_sum(alpha);
        beta = warp_sum(beta);
        gamma = warp_sum(gamma);
        // rotation angle by lane 0 only (FP64 division and square root are
        // scarce on this part), then broadcast
        double c = 1.0, s = 0.0;
        int rot = 0;
        if (lane == 0 && gamma != 0.0 && gamma * gamma > 1e-30 * alpha * beta) {
          const double zeta = (beta - alpha) / (2.0 * gamma);
          const double t = fabs(zeta) > 1e150 ? 0.5 / zeta
                                              : (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
          c = rsqrt(1.0 + t * t);
          s = c * t;
          rot = 1;
        }
        rot = __shfl_sync(0xffffffffu, rot, 0);
        if (rot) {
          c = __shfl_sync(0xffffffffu, c, 0);
          s = __shfl_sync(0xffffffffu, s, 0);
          for (int64_t i = lane; i < rows; i += 32) {
            const double x = ca[i], y = cb[i];
            ca[i] = c * x - s * y;
            cb[i] = s * x + c * y;
          }
          double* va = V + (int64_t)ia * ncols;
          double* vb = V + (int64_t)ib * ncols;
          for (int i = lane; i < ncols; i += 32) {
            const double x = va[i], y = vb[i];
            va[i] = c * x - s * y;
            vb[i] = s * x + c * y;
          }
          // quadratic convergence: a sweep whose live pairs were all within 1e-9
          // (relative) leaves them within ~1e-18, so no further sweep is needed
          if (lane == 0 && fmin(alpha, beta) > live_floor && gamma * gamma > 1e-18 * alpha * beta) s_rot = 1;
        }
      }
      __syncthreads();
    }
    if (!s_rot) break;
    __syncthreads();
  }
  // singular values, descending order, kept rank
  for (int c = warp; c < ncols; c += nw) {
    const double* cc = W + (int64_t)c * rows;
    double s = 0.0;
    for (int64_t i = lane; i < rows; i += 32) s += cc[i] * cc[i];
    s = warp_sum(s);
    if (lane == 0) s_sig[c] = sqrt(s);
  }
  __syncthreads();
  if (tid == 0) {
    for (int i = 0; i < ncols; ++i) s_ord[i] = i;
    for (int i = 1; i < ncols; ++i) {  // insertion sort, descending, stable
      const int v = s_ord[i];
      int j = i - 1;
      while (j >= 0 && s_sig[s_ord[j]] < s_sig[v]) {
        s_ord[j + 1] = s_ord[j];
        --j;
      }
      s_ord[j + 1] = v;
    }
    const double s0 = s_sig[s_ord[0]];
    int k = ncols;
    if (a.threshold != 0.0) {
      k = 0;
      while (k < ncols && s0 > 0.0 && s_sig[s_ord[k]] / s0 > a.threshold) ++k;
    }
    if (a.max_rank > 0 && k > a.max_rank) k = (int)a.max_rank;
    if (k < 1) k = 1;
    s_k = k;
    *a.kept = k;
  }
  __syncthreads();
  const int k = s_k;
  // M = U S V^T.  Working X (= M or M^T) = Ux S Vx^T with Ux = W[:, c] / sigma_c, Vx = V[:, c].
  // not transposed: U = Ux, V = Vx.  transposed: U = Vx, V = Ux.
  const int64_t p = a.p, q = a.q;
  auto Uel = [&](int64_t i, int j) -> double {  // U[i][j] * sigma_j   (unnormalised left vector)
    const int c = s_ord[j];
    return tr ? V[(int64_t)c * ncols + i] * s_sig[c] : W[(int64_t)c * rows + i];
  };
  auto Vel = [&](int64_t i, int j) -> double {  // V[i][j] * sigma_j
    const int c = s_ord[j];
    return tr ? W[(int64_t)c * rows + i] : V[(int64_t)c * ncols + i] * s_sig[c];
  };
  for (int64_t e = tid; e < p * k; e += nt) {
    const int64_t i = e / k;
    const int j = (int)(e - i * k);
    const double sg = s_sig[s_ord[j]];
    const double u = Uel(i, j);
    if (a.side == 0) a.core[e] = sg > 0.0 ? u / sg : (i == j ? 1.0 : 0.0);
    else a.r[e] = u;
  }
  for (int64_t e = tid; e < (int64_t)k * q; e += nt) {
    const int j = (int)(e / q);
    const int64_t i = e - (int64_t)j * q;
    const double sg = s_sig[s_ord[j]];
    const double v = Vel(i, j);
    if (a.side == 0) a.r[e] = v;
    else a.core[e] = sg > 0.0 ? v / sg : (i == j ? 1.0 : 0.0);
  }
}

// Minimum-norm least-squares solution from the truncated SVD of R (the
// gelss step of scipy.linalg.lstsq, used by scikit_tt/data_driven/
// regression.py:487): R (kq x N) = U S V^T with the r = *kept leading
// singular values, c = Q^T y:  x = V S^-1 U^T c = (S V^T)^T S^-2 (U^T c).
// U: kq x r (row-major, leading dimension r), SVt: r x N.  One CTA.
__global__ void __launch_bounds__(1024) lstsq_combine_kernel(const double* U, const double* SVt, const double* c,
                                                              int64_t kq, int64_t N, const int* kept, double* x,
                                                              const int* skip) {
  if (skip && *skip) return;
  __shared__ double w[kTrMaxGram];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int r = *kept;
  for (int i = warp; i < r; i += nw) {
    double dot = 0.0, s2 = 0.0;
    for (int64_t q = lane; q < kq; q += 32) dot += U[q * r + i] * c[q];
    for (int64_t p = lane; p < N; p += 32) s2 += SVt[i * N + p] * SVt[i * N + p];
    dot = warp_sum(dot);
    s2 = warp_sum(s2);
    if (lane == 0) w[i] = s2 > 0.0 ? dot / s2 : 0.0;
  }
  __syncthreads();
  for (int64_t p = tid; p < N; p += nt) {
    double acc = 0.0;
    for (int i = 0; i < r; ++i) acc += SVt[i * N + p] * w[i];
    x[p] = acc;
  }
}

cudaError_t launch_lstsq_combine(const double* U, const double* SVt, const double* c, int64_t kq, int64_t N,
                                 const int* kept, double* x, cudaStream_t st, const int* skip) {
  if (std::min(kq, N) > kTrMaxGram) return cudaErrorInvalidValue;
  lstsq_combine_kernel<<<1, 1024, 0, st>>>(U, SVt, c, kq, N, kept, x, skip);
  ++launch_counter();
  return cudaGetLastError();
}

// Least squares through the triangular factor when that is safe: R (N x N,
// upper triangular, row-major) from the QR of the m x N micro matrix (m >= N)
// and c = Q^T y.  gelss (scipy.linalg.lstsq as regression.py:487 calls it)
// treats singular values below rcond * s_max as zero; when
// ||R||_F ||R^-1||_F <= 1e-2 / rcond no singular value is that small, and when
// it is also <= 1e5 the two solutions agree to rounding, so x = R^-1 c.  R^-1
// is formed column by column (thread j back-substitutes e_j) into Z (N x N);
// *fast = 1 then and x is written, else *fast = 0 and the SVD path solves.
__global__ void __launch_bounds__(1024) lstsq_tri_kernel(const double* R, const double* c, int64_t N, double rcond,
                                                          double* Z, double* x, int* fast) {
  __shared__ double rinv[kTrMaxGram];
  __shared__ double red[32];
  __shared__ int s_ok;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  auto block_sum = [&](double v) {
    v = warp_sum(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[w];
    __syncthreads();
    return t;
  };
  if (tid == 0) s_ok = 1;
  __syncthreads();
  for (int64_t i = tid; i < N; i += nt) {
    const double d = R[i * N + i];
    if (!(fabs(d) > 0.0) || !isfinite(d)) s_ok = 0;
    rinv[i] = 1.0 / d;
  }
  __syncthreads();
  if (!s_ok) {
    if (tid == 0) *fast = 0;
    return;
  }
  double sr = 0.0;
  for (int64_t e = tid; e < N * N; e += nt) {
    const int64_t i = e / N, k = e - i * N;
    if (k >= i) sr += R[e] * R[e];
  }
  sr = block_sum(sr);
  for (int64_t j = tid; j < N; j += nt) {
    Z[j * N + j] = rinv[j];
    for (int64_t i = j - 1; i >= 0; --i) {
      double acc = 0.0;
      for (int64_t k = i + 1; k <= j; ++k) acc += R[i * N + k] * Z[k * N + j];
      Z[i * N + j] = -acc * rinv[i];
    }
  }
  __syncthreads();
  double sz = 0.0;
  for (int64_t e = tid; e < N * N; e += nt) {
    const int64_t i = e / N, k = e - i * N;
    if (k >= i) sz += Z[e] * Z[e];
  }
  sz = block_sum(sz);
  const double kf = sqrt(sr) * sqrt(sz);
  const int ok = isfinite(kf) && kf <= 1e5 && kf * rcond <= 1e-2;
  if (ok) {
    for (int64_t i = tid; i < N; i += nt) {
      double acc = 0.0;
      for (int64_t k = i; k < N; ++k) acc += Z[i * N + k] * c[k];
      x[i] = acc;
    }
  }
  if (tid == 0) *fast = ok;
}

cudaError_t launch_lstsq_tri(const double* R, const double* c, int64_t N, double rcond, double* Z, double* x,
                             int* fast, cudaStream_t st) {
  if (N > kTrMaxGram || N < 1) return cudaErrorInvalidValue;
  lstsq_tri_kernel<<<1, 1024, 0, st>>>(R, c, N, rcond, Z, x, fast);
  ++launch_counter();
  return cudaGetLastError();
}

constexpr size_t kSvdSmemMax = 196 * 1024;  // plus ~25 KB of static shared memory

size_t svd_trunc_work_doubles(int64_t p, int64_t q) {
  const int64_t n = p < q ? p : q, rows = p > q ? p : q;
  return (size_t)(rows * n + n * n + (rows * n + 1) / 2 + (n * n + 1) / 2 + 64);
}

cudaError_t launch_svd_trunc(const double* M, int64_t p, int64_t q, int side, double threshold, int64_t max_rank,
                             double* work, double* core, double* r, int* kept, int* status, cudaStream_t st,
                             const int* skip) {
  const int64_t n = p < q ? p : q, rows = p > q ? p : q;
  if (n > kTrMaxGram || n < 1) return cudaErrorInvalidValue;
  // the dots read W at every rotation step: W first, then V if both fit
  // shared memory for W, then its FP32 copy, then V and its copy, while they fit
  const size_t part[4] = {8 * (size_t)(rows * n), ((4 * (size_t)(rows * n)) + 7) / 8 * 8, 8 * (size_t)(n * n),
                          ((4 * (size_t)(n * n)) + 7) / 8 * 8};
  int in_smem = 0;
  size_t bytes = 0;
  for (int b = 0; b < 4; ++b)
    if (bytes + part[b] <= kSvdSmemMax) {
      bytes += part[b];
      in_smem |= 1 << b;
    }
  double* w32 = work + rows * n + n * n;
  double* v32 = w32 + (rows * n + 1) / 2;
  SvdK a{M,    p,    q, side, threshold, max_rank, work, work + rows * n, core, r, kept, status,
         reinterpret_cast<float*>(w32), reinterpret_cast<float*>(v32), in_smem, skip};
  if (in_smem) {
    cudaError_t e = cudaFuncSetAttribute(svd_trunc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSvdSmemMax);
    if (e != cudaSuccess) return e;
  }
  svd_trunc_kernel<<<1, kTrThreads, bytes, st>>>(a);
  ++launch_counter();
  return cudaGetLastError();
}

}  // namespace ttals
