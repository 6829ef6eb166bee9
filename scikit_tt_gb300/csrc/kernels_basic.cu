// Non-persistent kernels of the ALS engine: strided contractions (interface
// stacks, local right-hand sides, gauge pushes, operator-core products),
// elementwise helpers and the Householder QR used for the sweep's QR/RQ
// re-gauging (scikit_tt/solvers/sle.py:514-547).
#include <algorithm>

#include "ttals_internal.h"

namespace ttals {

int64_t& launch_counter() {
  static thread_local int64_t n = 0;
  return n;
}

Contraction make_contraction(const std::vector<Axis>& out, const std::vector<Axis>& k) {
  Contraction c{};
  c.nout = (int)out.size();
  c.nk = (int)k.size();
  c.total = 1;
  for (int q = 0; q < c.nout; ++q) {
    c.out_dim[q] = (int)out[q].dim;
    c.a_os[q] = out[q].sa;
    c.b_os[q] = out[q].sb;
    c.c_os[q] = out[q].sc;
    c.total *= out[q].dim;
  }
  c.ktotal = 1;
  for (int q = 0; q < c.nk; ++q) {
    c.k_dim[q] = (int)k[q].dim;
    c.a_ks[q] = k[q].sa;
    c.b_ks[q] = k[q].sb;
    c.ktotal *= k[q].dim;
  }
  return c;
}

// Three phases of y -> M y (see LocalShape):
//   P1  T1[R, a', n, s]  = sum_a      L[a, R, a'] y[a, n, s]
//   P2  T2[a', m, s, R'] = sum_{R,n}  T1[R, a', n, s] A[R, m, n, R']
//   P3  out[a', m, s']   = sum_{s,R'} T2[a', m, s, R'] Rt[s, R', s']
void local_apply_descs(const LocalShape& sh, Contraction* p1, Contraction* p2, Contraction* p3) {
  const int64_t a = sh.a, n = sh.n, s = sh.s, R0 = sh.R0, R1 = sh.R1;
  // P1: A-operand L (strides a: R0*a, R: a, a': 1), B-operand y (a: n*s, n: s, s: 1)
  *p1 = make_contraction({{R0, a, 0, a * n * s}, {a, 1, 0, n * s}, {n, 0, s, s}, {s, 0, 1, 1}},
                         {{a, R0 * a, n * s, 0}});
  // P2: A-operand T1 (R: a*n*s, a': n*s, n: s, s: 1), B-operand A (R: n*n*R1, m: n*R1, n: R1, R': 1)
  *p2 = make_contraction(
      {{a, n * s, 0, n * s * R1}, {n, 0, n * R1, s * R1}, {s, 1, 0, R1}, {R1, 0, 1, 1}},
      {{R0, a * n * s, n * n * R1, 0}, {n, s, R1, 0}});
  // P3: A-operand T2 (a': n*s*R1, m: s*R1, s: R1, R': 1), B-operand Rt (s: R1*s, R': s, s': 1)
  *p3 = make_contraction({{a, n * s * R1, 0, n * s}, {n, s * R1, 0, s}, {s, 0, 1, 1}},
                         {{s, R1, R1 * s, 0}, {R1, 1, s, 0}});
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
// Householder QR, one CTA.  Column-major working copy W (rows x cols) and
// reflectors Vh (rows x k) live in global scratch (L2 resident at ALS sizes).
// Reflector j: H_j = I - tau_j v_j v_j^T with v_j[j] = x_j - alpha_j,
// alpha_j = -sign(x_j) ||x||, so R[j][j] = alpha_j (the LAPACK sign choice).
// ---------------------------------------------------------------------------

constexpr int kQrThreads = 512;

__global__ void __launch_bounds__(kQrThreads) qr_kernel(QrArgs a) {
  const int64_t rows = a.rows, cols = a.cols;
  const int64_t k = rows < cols ? rows : cols;
  double* W = a.work;
  double* Vh = W + rows * cols;
  double* Qw = Vh + rows * k;
  double* tau = Qw + rows * k;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  __shared__ double red[32];
  __shared__ double s_alpha, s_tau, s_v0;

  for (int64_t e = tid; e < rows * cols; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    W[e] = a.in[i * a.ris + c * a.rjs];
  }
  __syncthreads();

  for (int64_t j = 0; j < k; ++j) {
    const double* col = W + j * rows;
    double s = 0.0;
    for (int64_t i = j + tid; i < rows; i += nt) s += col[i] * col[i];
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    __syncthreads();
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
    __syncthreads();
    double* v = Vh + j * rows;
    for (int64_t i = j + tid; i < rows; i += nt) v[i] = (i == j) ? s_v0 : col[i];
    __syncthreads();
    const double tj = s_tau;
    for (int64_t c = j + 1 + warp; c < cols; c += nw) {
      double* wc = W + c * rows;
      double dot = 0.0;
      for (int64_t i = j + lane; i < rows; i += 32) dot += v[i] * wc[i];
      dot = warp_sum(dot) * tj;
      for (int64_t i = j + lane; i < rows; i += 32) wc[i] -= dot * v[i];
    }
    __syncthreads();
    if (tid == 0) W[j * rows + j] = s_alpha;
    __syncthreads();
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
    __syncthreads();
    double tot = 0.0;
    for (int w = 0; w < nw; ++w) tot += red[w];
    __syncthreads();
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
  __syncthreads();
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
    __syncthreads();
  }
  for (int64_t e = tid; e < rows * k; e += nt) {
    const int64_t i = e % rows, c = e / rows;
    a.q[i * a.qis + c * a.qjs] = Qw[e];
  }
}

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
