// Shared host/device structures of the batched ALS kernel (kernels_batch.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ttals {

// One instance.  meta (int64, at meta + meta_off) holds, in order:
// n[d], R[d+1], rb[d+1], rx0[d+1], cap[d+1], op_off[d], rhs_off[d], x0_off[d],
// X_off[d], L_off[d], Rt_off[d], Lb_off[d], Rb_off[d].
struct BatchInst {
  int32_t d, repeats;
  int32_t kind;  // 0: linear system (sle.als), 1: eigenproblem (evp.als)
  int32_t mode;  // EVP selection: 0 largest (eigh), 1 closest to sigma (eig/eigs), 2 smallest
  double sigma, conv_eps;
  int64_t meta_off;
  const double *op, *rhs, *x0;
  double *X, *L, *Rt, *Lb, *Rb;
  double* Xopt;    // EVP: cores of the best sweep (evp.py:151-155)
  double* out;     // final cores, packed
  int* done;       // per-request completion flag in host-mapped memory (may be null)
  double* report;  // [max rel residual, local solves, Krylov its, refinement cycles, status, flops64, flops32,
                   //  eigenvalue, ranks[d+1], sweeps run, phase cycles[8], tensor-core GEMMs, fallbacks,
                   //  inner-solve cycles in operator applications]
};

// Largest per-CTA scratch needs over the batch (elements).
struct BatchSizes {
  int64_t T, U, N, R, Q, core, stack, opcore;
  int64_t Ng;  // N when the batch holds a generalised eigenproblem, else 0 (its extra scratch)
  int64_t oz_a, oz_b, oz_r, oz_c;  // emulated-FP64 GEMM scratch: slice arrays and exponent vectors
};

// Adds the emulated-FP64 (Ozaki) scratch needs of one site's contractions
// (apply, left and right stack updates) to z.
void oz_need_site(BatchSizes& z, int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1);

struct BatchArgs {
  const BatchInst* inst;
  int count;
  const int64_t* meta;
  int* next;  // work counter (zeroed before launch)
  char* scratch;
  int64_t scratch_stride;
  BatchSizes sizes;
  int m;      // GMRES restart length
  int m_evp;  // Lanczos basis size
  int prec;
  double tol;      // local linear solves
  double tol_evp;  // local eigen solves (Ritz residual relative to |T|)
  int use_tc;      // mixed precision on tcgen05 (batch_sle_tc_kernel)
};

size_t batch_smem_bytes(int m, int m_evp, int use_tc, int gevp = 0);
int batch_blocks_per_sm(int m, int m_evp, int use_tc, cudaError_t* err = nullptr, int gevp = 0);
int batch_threads(int use_tc);
// independent solves one CTA of the variant runs side by side (scratch slots per CTA)
int batch_solves_per_cta(int use_tc);
int64_t batch_scratch_stride(const BatchSizes& z, int m, int m_evp);
cudaError_t launch_batch_sle(const BatchArgs& a, int grid, cudaStream_t st);
cudaError_t launch_apply_f64emu(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1, const double* L,
                                const double* A, const double* R, const double* y, double* T1, double* T2,
                                double* out, char* ozmem, size_t ozbytes, int use_tc, cudaStream_t st);
size_t apply_f64emu_scratch_bytes(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1);
cudaError_t launch_apply_f32(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1, const float* L, const float* A,
                             const float* R, const float* y, float* T1, float* T2, float* out, int* ktab,
                             int use_tc, cudaStream_t st);

cudaError_t launch_umma_selftest(int kind, int N, int K, const float* A, const float* Bt, float* C, int* status,
                                 cudaStream_t st);

}  // namespace ttals
