// Non-persistent kernels of the ALS engine: strided contractions (interface
// stacks, local right-hand sides, gauge pushes, operator-core products),
// elementwise helpers and the Householder QR used for the sweep's QR/RQ
// re-gauging (scikit_tt/solvers/sle.py:514-547).
#include <algorithm>

#include "ttals_desc.cuh"
#include "ttals_internal.h"
#include "ttals_qr.cuh"

namespace ttals {

int64_t& launch_counter() {
  static thread_local int64_t n = 0;
  return n;
}

Contraction make_contraction(const std::vector<Axis>& out, const std::vector<Axis>& k) {
  Ax o[kMaxOut], kk[kMaxK];
  for (size_t q = 0; q < out.size(); ++q) o[q] = {out[q].dim, out[q].sa, out[q].sb, out[q].sc};
  for (size_t q = 0; q < k.size(); ++q) kk[q] = {k[q].dim, k[q].sa, k[q].sb, 0};
  return desc_make((int)out.size(), o, (int)k.size(), kk);
}

// Three phases of y -> M y (see LocalShape and desc_apply).
void local_apply_descs(const LocalShape& sh, Contraction* p1, Contraction* p2, Contraction* p3) {
  desc_apply(sh.a, sh.n, sh.s, sh.R0, sh.R1, p1, p2, p3);
}

template <typename T>
__global__ void __launch_bounds__(256) contract_kernel(Contraction c, const T* __restrict__ A,
                                                       const T* __restrict__ B, T* __restrict__ C,
                                                       T alpha, T beta) {
  const int64_t first = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  contract_range(c, A, B, C, alpha, beta, first, step);
}

template <typename T>
cudaError_t launch_contract(const Contraction& c, const T* A, const T* B, T* C, T alpha, T beta,
                            cudaStream_t st) {
  if (c.total <= 0) return cudaSuccess;
  if (c.total >= (int64_t(1) << 31)) return cudaErrorInvalidValue;  // 32-bit index arithmetic
  // Spread the outputs over every SM: FP64 runs at two lanes a clock per SM, so a
  // small contraction in 256-thread blocks would sit on a few SMs.  Blocks shrink
  // (down to one warp) until there are about two per SM.
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && sms[dev] == 0) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    sms[dev] = v > 0 ? v : 1;
  }
  const int64_t nsm = (dev >= 0 && dev < 64) ? sms[dev] : 1;
  int64_t threads = (c.total + 2 * nsm - 1) / (2 * nsm);
  threads = std::max<int64_t>(32, std::min<int64_t>(256, (threads + 31) / 32 * 32));
  int64_t blocks = (c.total + threads - 1) / threads;
  blocks = std::min<int64_t>(blocks, 65535);
  contract_kernel<T><<<(unsigned)blocks, (unsigned)threads, 0, st>>>(c, A, B, C, alpha, beta);
  ++launch_counter();
  return cudaGetLastError();
}
template cudaError_t launch_contract<double>(const Contraction&, const double*, const double*, double*,
                                             double, double, cudaStream_t);
template cudaError_t launch_contract<float>(const Contraction&, const float*, const float*, float*, float,
                                            float, cudaStream_t);

__global__ void fill_kernel(double* p, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = v;
}
cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
  fill_kernel<<<blocks, 256, 0, st>>>(p, n, v);
  ++launch_counter();
  return cudaGetLastError();
}

__global__ void to_float_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}
cudaError_t launch_to_float(const double* src, float* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
  to_float_kernel<<<blocks, 256, 0, st>>>(src, dst, n);
  ++launch_counter();
  return cudaGetLastError();
}

__global__ void scale_kernel(double* p, int64_t n, const double* sc, int invert) {
  double f = *sc;
  if (invert) f = (f != 0.0) ? 1.0 / f : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] *= f;
}
cudaError_t launch_scale(double* p, int64_t n, const double* scale_dev, int invert, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
  scale_kernel<<<blocks, 256, 0, st>>>(p, n, scale_dev, invert);
  ++launch_counter();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Householder QR, one CTA (body in ttals_qr.cuh, shared with the batch kernel)
// ---------------------------------------------------------------------------

constexpr int kQrThreads = 512;

__global__ void __launch_bounds__(kQrThreads) qr_kernel(QrArgs a) { cta_householder_qr(a); }

cudaError_t launch_qr(const QrArgs& a, cudaStream_t st) {
  if (a.rows <= 0 || a.cols <= 0) return cudaSuccess;
  qr_kernel<<<1, kQrThreads, 0, st>>>(a);
  ++launch_counter();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// CholeskyQR2 for the single-solve path (tall-skinny cores, many CTAs)
// ---------------------------------------------------------------------------
//
// The economic QR of an ALS core (e.g. 256 x 32) on one CTA is a chain of
// 32 reductions and barriers; CholeskyQR spreads it over the GPU:
//   G = X^T X (row chunks on kCqrChunks CTAs, partial Gram matrices reduced in a
//   fixed order), G = R^T R (Cholesky, one CTA), Q = X R^-1 (parallel over rows),
// twice (the second pass restores orthogonality to working precision), then
// R = R2 R1.  A Cholesky pivot below 1e-15 of the largest diagonal (cond(X) >~
// 3e7) sets a device flag: the same call then runs the Householder kernel on
// the untouched input instead, without a host round trip.  Q keeps the span of
// X; R carries a positive diagonal (a gauge of the reference's QR).  The
// Cholesky factor and its inverse live in shared memory (cols <= 64).
// Work layout: [flag | partials kCqrChunks*c^2 | (spare) c^2 | Rinv c^2 | R1 c^2 | (spare) c^2].

constexpr int kCqrChunks = 16;
constexpr int kCqrThreads = 256;
constexpr int kCqrMaxCols = 64;  // G and R^-1 of the Cholesky step live in shared memory

__global__ void __launch_bounds__(kCqrThreads) cqr_gram_kernel(const double* __restrict__ X, int64_t ris,
                                                               int64_t rjs, int64_t rows, int cols, double* work,
                                                               int pass) {
  const int* flag = reinterpret_cast<const int*>(work);
  if (*flag != 0) return;
  double* part = work + 8 + (int64_t)blockIdx.x * cols * cols;
  const int64_t chunk = (rows + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * chunk, r1 = r0 + chunk < rows ? r0 + chunk : rows;
  for (int e = threadIdx.x; e < cols * cols; e += blockDim.x) {
    const int i = e / cols, j = e - i * cols;
    if (j < i) continue;
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r) acc += X[r * ris + i * rjs] * X[r * ris + j * rjs];
    part[i * cols + j] = acc;
    part[j * cols + i] = acc;
  }
  (void)pass;
}

__global__ void __launch_bounds__(kCqrThreads) cqr_chol_kernel(int cols, double* work, int pass, double* r,
                                                               int64_t r_is, int64_t r_js) {
  extern __shared__ double sh[];
  int* flag = reinterpret_cast<int*>(work);
  if (*flag != 0) return;
  const int cc = cols * cols;
  const double* part = work + 8;
  double* Rig = work + 8 + (int64_t)kCqrChunks * cc + cc;  // R^-1 for the apply kernel
  double* R1g = Rig + cc;
  double* G = sh;        // Cholesky in place: upper factor
  double* Ri = sh + cc;  // R^-1
  // FP64 runs at two lanes a clock per SM on this part: every FP64 operation
  // of this single-CTA step is counted, divisions are done once and shared
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  __shared__ double s_inv, s_max;
  __shared__ int s_fail;
  __shared__ double s_dinv[kCqrMaxCols];
  for (int e = tid; e < cc; e += nt) {
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < kCqrChunks; ++b) acc += part[(int64_t)b * cc + e];
    G[e] = acc;
  }
  __syncthreads();
  if (tid == 0) {
    double m = 0.0;
    for (int i = 0; i < cols; ++i) m = fmax(m, G[i * cols + i]);
    s_max = m;
    s_fail = !(m > 0.0) || !isfinite(m);
  }
  __syncthreads();
  for (int k = 0; k < cols && !s_fail; ++k) {
    if (tid == 0) {
      const double d = G[k * cols + k];
      if (!(d > 1e-15 * s_max)) {
        s_fail = 1;
      } else {
        // 1/sqrt(d) by Newton-Raphson on y^-2 = d (each step doubles the correct
        // bits: 24 -> 48 -> FP64), instead of the long dependent FP64 sqrt and
        // division sequences.  The FP32 seed is taken from the mantissa: d = m 4^t
        // with m in [1, 4) (integer exponent arithmetic), y0 = rsqrt(m) 2^-t, so
        // Gram entries far outside the FP32 range (cores of norm 1e40) are fine.
        double y;
        const uint64_t db = (uint64_t)__double_as_longlong(d);
        const int ex = (int)((db >> 52) & 0x7ff);
        if (ex == 0) {
          y = 1.0 / sqrt(d);  // subnormal pivot: exact path
        } else {
          const int t = (ex - 1023) >> 1;  // floor((e) / 2)
          const double m = __longlong_as_double((long long)(db - ((uint64_t)(int64_t)(2 * t) << 52)));
          y = (double)rsqrtf((float)m);
          y = __longlong_as_double((long long)((uint64_t)__double_as_longlong(y) - ((uint64_t)(int64_t)t << 52)));
          y = y * (1.5 - 0.5 * d * y * y);
          y = y * (1.5 - 0.5 * d * y * y);
        }
        G[k * cols + k] = d * y;
        s_inv = y;
        s_dinv[k] = y;
      }
    }
    __syncthreads();
    if (s_fail) break;
    const double inv = s_inv;
    for (int j = k + 1 + tid; j < cols; j += nt) G[k * cols + j] *= inv;
    __syncthreads();
    // trailing update of the upper triangle: rows by warps, columns by lanes
    for (int i = k + 1 + warp; i < cols; i += nw) {
      const double gki = G[k * cols + i];
      for (int j = i + lane; j < cols; j += 32) G[i * cols + j] -= gki * G[k * cols + j];
    }
    __syncthreads();
  }
  if (s_fail) {
    if (tid == 0) *flag = pass;  // 1: fall back to Householder on X; 2: keep the first pass
    return;
  }
  // R^-1 of the upper factor, one column per thread (back substitution with the
  // shared reciprocal diagonal)
  for (int j = tid; j < cols; j += nt) {
    for (int i = cols - 1; i >= 0; --i) {
      if (i > j) {
        Ri[i * cols + j] = 0.0;
        continue;
      }
      double acc = (i == j) ? 1.0 : 0.0;
      for (int l = i + 1; l <= j; ++l) acc -= G[i * cols + l] * Ri[l * cols + j];
      Ri[i * cols + j] = acc * s_dinv[i];
    }
  }
  __syncthreads();
  for (int e = tid; e < cc; e += nt) Rig[e] = Ri[e];
  if (pass == 1) {
    for (int e = tid; e < cc; e += nt) {
      const int i = e / cols, j = e - i * cols;
      R1g[e] = (j >= i) ? G[e] : 0.0;
    }
  } else if (r) {
    // R = R2 R1 (both upper triangular)
    for (int e = tid; e < cc; e += nt) {
      const int i = e / cols, j = e - i * cols;
      double acc = 0.0;
      for (int l = i; l <= j; ++l) acc += G[i * cols + l] * R1g[l * cols + j];
      r[i * r_is + j * r_js] = (j >= i) ? acc : 0.0;
    }
  }
}

// Q = X R^-1: kCqrRows rows per CTA staged in shared memory with R^-1 (X may alias Q)
constexpr int kCqrRows = 8;
__global__ void __launch_bounds__(kCqrThreads) cqr_apply_kernel(const double* X, int64_t ris, int64_t rjs,
                                                                double* Q, int64_t qis, int64_t qjs, int64_t rows,
                                                                int cols, const double* work) {
  extern __shared__ double sh[];
  const int* flag = reinterpret_cast<const int*>(work);
  if (*flag != 0) return;
  const int cc = cols * cols;
  const double* Rig = work + 8 + (int64_t)kCqrChunks * cc + cc;
  double* Ri = sh;
  double* sx = sh + cc;
  const int64_t r0 = (int64_t)blockIdx.x * kCqrRows;
  const int nr = (int)(r0 + kCqrRows <= rows ? kCqrRows : rows - r0);
  if (nr <= 0) return;
  for (int e = threadIdx.x; e < cc; e += blockDim.x) Ri[e] = Rig[e];
  for (int e = threadIdx.x; e < nr * cols; e += blockDim.x) {
    const int i = e / cols, j = e - i * cols;
    sx[e] = X[(r0 + i) * ris + j * rjs];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nr * cols; e += blockDim.x) {
    const int i = e / cols, j = e - i * cols;
    double acc = 0.0;
    for (int l = 0; l <= j; ++l) acc += sx[i * cols + l] * Ri[l * cols + j];
    Q[(r0 + i) * qis + j * qjs] = acc;
  }
}

// pass 2 failed (flag 2): R = R1, Q = the first pass's Q
__global__ void cqr_keep_first_kernel(int cols, const double* work, double* r, int64_t r_is, int64_t r_js) {
  if (*reinterpret_cast<const int*>(work) != 2) return;
  const int cc = cols * cols;
  const double* R1g = work + 8 + (int64_t)kCqrChunks * cc + 2 * (int64_t)cc;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cc; e += gridDim.x * blockDim.x) {
    const int i = e / cols, j = e - i * cols;
    r[i * r_is + j * r_js] = R1g[e];
  }
}

__global__ void __launch_bounds__(kQrThreads) qr_fallback_kernel(QrArgs a, const double* work) {
  if (*reinterpret_cast<const int*>(work) != 1) return;
  cta_householder_qr(a);
}

int64_t cqr_work_doubles(int64_t cols) { return 8 + ((int64_t)kCqrChunks + 4) * cols * cols; }

bool cqr_applicable(const QrArgs& a) {
  return a.rows >= a.cols && a.cols >= 1 && a.cols <= kCqrMaxCols && !a.normalize_r && !a.rnorm &&
         a.rows >= 2 * kCqrChunks;
}

// a.work must hold max(qr_work(rows, cols), cqr_work_doubles(cols)) + 8 doubles
cudaError_t launch_qr_fast(const QrArgs& a, cudaStream_t st) {
  if (a.rows <= 0 || a.cols <= 0) return cudaSuccess;
  if (!cqr_applicable(a)) return launch_qr(a, st);
  double* work = a.work;
  const int cols = (int)a.cols;
  const size_t cc = (size_t)cols * cols;
  const size_t chol_smem = sizeof(double) * 2 * cc;
  const size_t apply_smem = sizeof(double) * (cc + (size_t)kCqrRows * cols);
  cudaError_t e = cudaFuncSetAttribute(cqr_chol_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)chol_smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(cqr_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)apply_smem);
  if (e == cudaSuccess) e = cudaMemsetAsync(work, 0, sizeof(double), st);
  if (e != cudaSuccess) return e;
  const int nblk = (int)((a.rows + kCqrRows - 1) / kCqrRows);
  // pass 1: X -> Q (a.in -> a.q); pass 2: Q -> Q, R = R2 R1
  cqr_gram_kernel<<<kCqrChunks, kCqrThreads, 0, st>>>(a.in, a.ris, a.rjs, a.rows, cols, work, 1);
  cqr_chol_kernel<<<1, kCqrThreads, chol_smem, st>>>(cols, work, 1, nullptr, 0, 0);
  cqr_apply_kernel<<<nblk, kCqrThreads, apply_smem, st>>>(a.in, a.ris, a.rjs, a.q, a.qis, a.qjs, a.rows, cols, work);
  cqr_gram_kernel<<<kCqrChunks, kCqrThreads, 0, st>>>(a.q, a.qis, a.qjs, a.rows, cols, work, 2);
  cqr_chol_kernel<<<1, kCqrThreads, chol_smem, st>>>(cols, work, 2, a.r, a.r_is, a.r_js);
  cqr_apply_kernel<<<nblk, kCqrThreads, apply_smem, st>>>(a.q, a.qis, a.qjs, a.q, a.qis, a.qjs, a.rows, cols, work);
  if (a.r) cqr_keep_first_kernel<<<1, 256, 0, st>>>(cols, work, a.r, a.r_is, a.r_js);
  QrArgs fb = a;
  fb.work = work + 8;
  qr_fallback_kernel<<<1, kQrThreads, 0, st>>>(fb, work);
  launch_counter() += a.r ? 8 : 7;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// failure-detection probe: the engine's bounded wait on a flag
// ---------------------------------------------------------------------------

// Waits (bounded) for *flag to leave 0; records ST_TIMEOUT in *status when the
// limit runs out.  With a flag that nothing sets this exercises the timeout
// path of every device-side wait without hanging or faulting anything.
__global__ void wait_probe_kernel(const unsigned* flag, unsigned limit, int* status) {
  if (threadIdx.x == 0 && !bounded_wait_change(flag, 0u, limit)) atomicCAS(status, ST_OK, ST_TIMEOUT);
}

cudaError_t launch_wait_probe(const unsigned* flag, unsigned limit, int* status, cudaStream_t st) {
  wait_probe_kernel<<<1, 32, 0, st>>>(flag, limit, status);
  ++launch_counter();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// arithmetic peak microbenchmark: 8 independent FMA chains per thread
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(512) fma_chain_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
    x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
    x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t measure_fma_peaks(cudaStream_t st, int num_sms, double* fp64, double* fp32) {
  const int blocks = num_sms * 4, threads = 512;
  void* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double));
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto run = [&](bool dbl, int iters) -> double {
    cudaEventRecord(e0, st);
    if (dbl)
      fma_chain_kernel<double><<<blocks, threads, 0, st>>>((double*)buf, iters, 0.999, 0.001);
    else
      fma_chain_kernel<float><<<blocks, threads, 0, st>>>((float*)buf, iters, 0.999f, 0.001f);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e9;
  };
  run(true, 200);
  *fp64 = std::max(run(true, 4000), run(true, 4000));
  run(false, 200);
  *fp32 = std::max(run(false, 40000), run(false, 40000));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  return cudaGetLastError();
}

}  // namespace ttals
