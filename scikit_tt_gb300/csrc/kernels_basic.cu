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
  int64_t blocks = (c.total + 255) / 256;
  blocks = std::min<int64_t>(blocks, 65535);
  contract_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(c, A, B, C, alpha, beta);
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
