// Host-side declarations shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "ttals_device.cuh"

namespace ttals {

// ---------------------------------------------------------------------------
// contraction descriptors (host builders)
// ---------------------------------------------------------------------------

struct Axis {          // one output or contraction axis
  int64_t dim;
  int64_t sa, sb, sc;  // strides in A, B, C (sc unused for contraction axes)
};

Contraction make_contraction(const std::vector<Axis>& out, const std::vector<Axis>& k);

// y -> M y for the local operator M[(a',m,s'),(a,n,s)] =
//   sum_{R,R'} L[a,R,a'] A[R,m,n,R'] Rt[s,R',s']  (square: a'=a, s'=s, m=n)
struct LocalShape {
  int64_t a, n, s, R0, R1;
  int64_t N() const { return a * n * s; }
  int64_t t1() const { return R0 * a * n * s; }  // T1[R, a', n, s]
  int64_t t2() const { return a * n * s * R1; }  // T2[a', m, s, R']
};
void local_apply_descs(const LocalShape& sh, Contraction* p1, Contraction* p2, Contraction* p3);

// ---------------------------------------------------------------------------
// kernel launchers (kernels_basic.cu)
// ---------------------------------------------------------------------------

// Kernels launched by this host thread since the last reset (every launch_*
// wrapper counts itself).
int64_t& launch_counter();

// FMA-chain throughput of the device in GFLOP/s (FP64 and FP32).
cudaError_t measure_fma_peaks(cudaStream_t st, int num_sms, double* fp64, double* fp32);

template <typename T>
cudaError_t launch_contract(const Contraction& c, const T* A, const T* B, T* C, T alpha, T beta,
                            cudaStream_t st);
cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t st);
cudaError_t launch_to_float(const double* src, float* dst, int64_t n, cudaStream_t st);
cudaError_t launch_scale(double* p, int64_t n, const double* scale_dev, int invert, cudaStream_t st);

// Householder QR of the rows x cols matrix M(i, j) = in[i*ris + j*rjs].
// Writes Q (rows x k, k = min(rows, cols)) to q[i*qis + j*qjs] and R
// (k x cols) to r[i*ris_r + j*rjs_r] (r may be null).  If normalize_r, R is
// divided by its Frobenius norm (used where only the gauge matters) and the
// norm is stored in *rnorm (may be null).  work: rows*cols + 2*rows*k + k
// doubles.
struct QrArgs {
  const double* in; int64_t ris, rjs;
  double* q; int64_t qis, qjs;
  double* r; int64_t r_is, r_js;
  int64_t rows, cols;
  int normalize_r;
  double* rnorm;
  double* work;
};
cudaError_t launch_qr(const QrArgs& a, cudaStream_t st);
// CholeskyQR2 over many CTAs for tall cores (Householder fallback on the device
// when the Gram matrix is not numerically SPD); a.work: qr_work_fast doubles
cudaError_t launch_qr_fast(const QrArgs& a, cudaStream_t st);
int64_t cqr_work_doubles(int64_t cols);

// ---------------------------------------------------------------------------
// persistent Krylov solvers (kernels_krylov.cu)
// ---------------------------------------------------------------------------

struct GmresLaunch {
  LocalShape sh;
  const double *L64, *A64, *R64;
  const void *Li, *Ai, *Ri;  // inner-precision copies (float for MIXED; == *64 for FP64)
  double *T1_64, *T2_64;
  void *T1i, *T2i;
  const double* f;
  double* x;
  double* r;
  void* V;
  void* w;
  double* partials;
  int m, max_cycles;
  double tol, inner_floor;
  unsigned* bar;  // 2 unsigned: count, generation
  int* status;
  double* report;  // 4 doubles: rel residual, cycles, inner iterations, flag
  int precision;   // 0 fp64, 1 mixed
};
// grid: one CTA per SM (cooperative launch)
cudaError_t launch_gmres(const GmresLaunch& g, int num_sms, cudaStream_t st);
size_t gmres_partials_doubles(int m, int num_sms);

struct LanczosLaunch {
  LocalShape sh;
  const double *L, *A, *R;
  double *T1, *T2;
  int nprev;               // deflation vectors: M += shift * t t^T
  const double* prevt;     // nprev x N
  double shift;
  double* x;               // in: start vector (N); out: eigenvectors (N x k, column k contiguous)
  double* vals;            // out: k eigenvalues
  double* V;               // (m+1) x N
  double* w;               // N
  double* partials;
  int m, k, mode;          // mode 0: largest, 1: closest to sigma, 2: smallest,
                           // 3: closest to sigma, farthest of the k first (eigs order)
  int nonsym;              // Arnoldi (nonsymmetric operator), m <= 64
  double sigma;
  int max_restarts;
  double tol;
  unsigned* bar;
  int* status;
  double* report;          // rel residual, restarts, iterations
};
cudaError_t launch_lanczos(const LanczosLaunch& l, int num_sms, cudaStream_t st);
size_t lanczos_partials_doubles(int m, int num_sms);
size_t lanczos_smem_bytes(int m, int nonsym);

// x <- exp(tau M) x on the local operator M (kernels_krylov.cu): literal = 1
// runs the fixed m-dimensional recurrence of the reference's local Krylov
// method, literal = 0 a converged Krylov approximation (relative tol) with at
// most max_substeps substeps; m <= 64
struct ExpmLaunch {
  LocalShape sh;
  const double *L, *A, *R;
  double *T1, *T2;
  double* x;
  double* V;               // (m+1) x N
  double* w;               // N
  double* partials;        // lanczos_partials_doubles(m, num_sms)
  int m, literal, max_substeps;
  double tau, tol;
  unsigned* bar;
  int* status;
  double* report;          // rel error estimate, substeps, iterations, basis size
};
cudaError_t launch_expm(const ExpmLaunch& l, int num_sms, cudaStream_t st);

// rank-r orthonormal basis of an eigenvector block (kernels_evp.cu): side 0 ->
// left basis (p x r) of M (p x q), side 1 -> right basis (r x q); tr_k > 0 reads
// M as the transposed-and-reshaped N x tr_k block (backward sweep)
size_t trunc_work_doubles(int64_t p, int64_t q, int64_t r);
cudaError_t launch_trunc_basis(const double* M, int64_t p, int64_t q, int tr_k, int r, int side, double* work,
                               double* out, int* status, cudaStream_t st);

// truncated SVD of one core (kernels_evp.cu): M (p x q) = U S V^T, kept rank k
// -> side 0: core = U (p x k), r = S V^T (k x q); side 1: core = V^T, r = U S
size_t svd_trunc_work_doubles(int64_t p, int64_t q);
cudaError_t launch_svd_trunc(const double* M, int64_t p, int64_t q, int side, double threshold, int64_t max_rank,
                             double* work, double* core, double* r, int* kept, int* status, cudaStream_t st,
                             const int* skip = nullptr);

// x = V S^-1 U^T c from the truncated SVD of R (kernels_evp.cu, least squares)
cudaError_t launch_lstsq_combine(const double* U, const double* SVt, const double* c, int64_t kq, int64_t N,
                                 const int* kept, double* x, cudaStream_t st, const int* skip = nullptr);
// x = R^-1 c when the square triangular R is safely invertible for gelss's
// rcond (kernels_evp.cu); *fast = 1 then (the SVD path is skipped), else 0
cudaError_t launch_lstsq_tri(const double* R, const double* c, int64_t N, double rcond, double* Z, double* x,
                             int* fast, cudaStream_t st);

// failure-detection probe (kernels_basic.cu): bounded wait on *flag leaving 0
cudaError_t launch_wait_probe(const unsigned* flag, unsigned limit, int* status, cudaStream_t st);

// engine.cu helpers used by the allocation-free entry point (noalloc.cu)
}  // namespace ttals
struct ttals_ctx;
namespace ttals {
int ctx_device(const ttals_ctx* c);
void ctx_set_error(ttals_ctx* c, const std::string& msg);
int stack_op_on_stream(ttals_ctx* c, int32_t left, const double* stack, const double* x, const double* op,
                       int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1, double* t1, double* t2,
                       double* out);
}  // namespace ttals
