/*
 * ttals.h -- C ABI of the GB300 (sm_103a) tensor-train ALS engine.
 *
 * The engine is a drop-in for scikit_tt's ALS hot path.  Each entry point
 * names the reference function it replaces (paths are relative to the
 * scikit_tt project root).  All functions return an int status (TTALS_OK on
 * success); ttals_last_error() gives a one-line message for the last failure
 * on a context.  No torch or CUDA types appear in the signatures: tensors are
 * plain double pointers, either host memory (copied to/from the device inside
 * the call) or device memory (on_device = 1).
 *
 * A tensor train is described by ttals_tt: `order` cores, core i of shape
 * (ranks[i], row_dims[i], col_dims[i], ranks[i+1]) in C order, all cores
 * concatenated in `data` (the layout of scikit_tt/tensor_train.py:184-188).
 */
#ifndef TTALS_H_
#define TTALS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TTALS_OK 0
#define TTALS_ERR_ARG 1         /* malformed shapes / arguments (ValueError)   */
#define TTALS_ERR_CUDA 2        /* CUDA runtime failure                         */
#define TTALS_ERR_NOMEM 3       /* device memory budget exceeded                */
#define TTALS_ERR_SINGULAR 4    /* local system singular / Krylov breakdown     */
#define TTALS_ERR_NONFINITE 5   /* NaN/Inf met in a local solve                 */
#define TTALS_ERR_TIMEOUT 6     /* a device-side wait gave up                   */
#define TTALS_ERR_NOCONV 7      /* local solve missed its tolerance             */
#define TTALS_ERR_UNSUPPORTED 8 /* feature outside the implemented path         */

/* arithmetic of the local solves */
#define TTALS_PREC_FP64 0  /* plain FP64 everywhere                                   */
#define TTALS_PREC_MIXED 1 /* FP32 Krylov inner solves + FP64 refinement residual     */

/* sle.als `solver` argument (scikit_tt/solvers/sle.py:505-509) */
#define TTALS_SLE_SOLVE 0
#define TTALS_SLE_LU 1

/* evp.als `solver` argument (scikit_tt/solvers/evp.py:417-439) */
#define TTALS_EVP_EIG 0
#define TTALS_EVP_EIGS 1
#define TTALS_EVP_EIGH 2

typedef struct ttals_ctx ttals_ctx;
typedef struct ttals_job ttals_job;

/* request kinds of the batched / served entry points */
#define TTALS_REQ_SLE 0 /* scikit_tt/solvers/sle.py:10 als */
#define TTALS_REQ_EVP 1 /* scikit_tt/solvers/evp.py:17 als (symmetric, number_ev == 1) */
/* scikit_tt/solvers/evp.py:17 als with operator_gevp (evp.py:272-287, 314-329,
 * 367-368): A x = lambda B x with A symmetric and B symmetric positive
 * definite, number_ev == 1; the request's rhs carries operator_gevp */
#define TTALS_REQ_GEVP 2

typedef struct {
  int32_t order;
  const int64_t* row_dims; /* [order]     */
  const int64_t* col_dims; /* [order]     */
  const int64_t* ranks;    /* [order + 1] */
  const double* data;      /* concatenated cores */
  int32_t on_device;       /* 0: host pointer, 1: device pointer */
} ttals_tt;

/* One ALS problem of a batch.  out_data receives the solution cores (ranks
 * from ttals_als_ranks; for EVP the best sweep's eigentensor, evp.py:151-155);
 * out_value the eigenvalue and out_iterations the sweeps run (EVP, may be
 * NULL).  rhs is ignored for EVP; for GEVP it is operator_gevp (an operator
 * train with the operator's mode sizes). */
typedef struct {
  int32_t kind;
  ttals_tt op, x0, rhs;
  int32_t repeats;
  int32_t solver;
  double sigma;
  double conv_eps;
  double* out_data;
  double* out_value;
  int32_t* out_iterations;
} ttals_request;

typedef struct {
  int64_t local_solves;       /* micro systems solved                          */
  int64_t krylov_iterations;  /* inner Krylov iterations, all local solves     */
  int64_t refinement_steps;   /* FP64 residual evaluations, all local solves   */
  double max_local_residual;  /* worst final relative residual of a local solve */
  double device_ms;           /* device time of the call (CUDA events)         */
  int64_t kernel_launches;    /* kernels the call launched                      */
  /* filled only while profiling is on (ttals_set_profiling):                  */
  int64_t solver_launches;    /* local-solve kernel launches                    */
  double solver_ms;           /* their summed duration (CUDA events)            */
  double solver_flops64;      /* algorithmic FP64 flops of the local solves     */
  double solver_flops32;      /* algorithmic FP32 flops of the local solves     */
  /* batched calls: SM cycles summed over requests, per phase: guess
   * orthonormalisation, operator/RHS stacks, local right-hand sides, FP64
   * residuals, inner Krylov iterations, QR/RQ + gauge push, eigensolves, total */
  double phase_cycles[8];
  /* batched mixed-precision calls: GEMM-shaped contractions that ran on the
   * fifth-generation tensor cores (tcgen05), and those that fell back to the
   * SIMT path (non-finite operands, or a tensor-core wait that gave up)      */
  int64_t tc_gemms;
  int64_t tc_fallbacks;
  /* batched calls: the part of phase_cycles[4] (inner Krylov iterations)
   * spent applying the local operator                                      */
  double inner_apply_cycles;
  /* batched calls: the launch variant the engine used (chosen by its
   * autotuner unless fixed by ttals_set_batch_variant): 1 = tensor-core
   * kernel (tcgen05), 0 = SIMT / warp-MMA kernel; and its CTAs per SM       */
  int32_t batch_tensor_cores;
  int32_t batch_ctas_per_sm;
  /* ... and the solves one of its CTAs runs side by side (2 on the
   * tensor-core kernel's two-group variant, else 1)                        */
  int32_t batch_solves_per_cta;
} ttals_stats;

/* Context: one device, one stream, one device-memory arena capped at
 * budget_bytes (0 = 90% of free memory).  No reference counterpart: the
 * reference is single-process NumPy (scikit_tt/solvers/sle.py:10). */
int ttals_create(ttals_ctx** ctx, int device, size_t budget_bytes);
int ttals_destroy(ttals_ctx* ctx);
const char* ttals_last_error(const ttals_ctx* ctx);
/* Run on a caller-provided cudaStream_t (passed as void*); NULL restores the
 * context's own stream. */
int ttals_set_stream(ttals_ctx* ctx, void* stream);

/* Time every local-solve launch with CUDA events (adds two event records
 * per launch) and report it in ttals_stats.  No reference counterpart. */
int ttals_set_profiling(ttals_ctx* ctx, int32_t enable);

/* Failure-detection probe: one device thread waits, through the engine's
 * bounded spin (the one every grid barrier uses), for a flag to leave 0 --
 * set beforehand when preset != 0, never set otherwise.  *status_out receives
 * TTALS_OK or TTALS_ERR_TIMEOUT (limit polls of ~64 ns, at most 2^22).  The
 * context stays usable either way.  No reference counterpart. */
int ttals_wait_probe(ttals_ctx* ctx, int32_t preset, uint32_t limit, int32_t* status_out);

/* Measured arithmetic peaks of this device (FMA-chain microbenchmarks), in
 * GFLOP/s.  Used to state roofline fractions.  No reference counterpart. */
int ttals_measure_peaks(ttals_ctx* ctx, double* fp64_gflops, double* fp32_gflops);

/* Rank schedule of one ALS run: the ranks of the returned solution for
 * dims/x_ranks, following the economic QR/RQ rank rule of
 * scikit_tt/solvers/sle.py:517-541 (identical for evp.py:452-487 when
 * number_ev == 1).  Host-only, no device work. */
int ttals_als_ranks(int32_t order, const int64_t* dims, const int64_t* x_ranks, int64_t* out_ranks);

/* scikit_tt/solvers/sle.py:10 `als(operator, initial_guess, right_hand_side,
 * repeats, solver)`.  out_data receives the solution cores (ranks from
 * ttals_als_ranks, written to out_ranks).  tol is the relative residual each
 * local system is solved to (<= 0 selects 1e-13 for FP64, 1e-10 for MIXED). */
int ttals_sle_als(ttals_ctx* ctx, const ttals_tt* op, const ttals_tt* x0, const ttals_tt* rhs,
                  int32_t repeats, int32_t solver, int32_t precision, double tol,
                  double* out_data, int32_t out_on_device, int64_t* out_ranks, ttals_stats* stats);

/* scikit_tt/solvers/sle.py:98-191 (`mals`): two-site ALS with a truncated SVD
 * split (sle.py:550-650): singular values with sigma_k / sigma_0 <= threshold
 * are dropped (none when threshold == 0) and at most max_rank (<= 0: no cap)
 * are kept.  The two-site micro system is solved matrix-free in FP64 (tol <= 0
 * picks 1e-13).  With out_data == NULL and out_capacity != NULL the call only
 * stores in *out_capacity the number of doubles the output may need. */
int ttals_sle_mals(ttals_ctx* ctx, const ttals_tt* op, const ttals_tt* x0, const ttals_tt* rhs, int32_t repeats,
                   int32_t solver, double threshold, int64_t max_rank, double tol, double* out_data,
                   int32_t out_on_device, int64_t* out_ranks, int64_t* out_capacity, ttals_stats* stats);

/* Number of requests one batched launch runs at the same time on this device
 * (SMs x resident CTAs per SM x solves per CTA, for the default launch
 * variant): a batch of this size keeps every SM busy.  No reference
 * counterpart. */
int ttals_batch_slots(ttals_ctx* ctx, int32_t* slots);

/* Launch variant of the batched calls (ttals_sle_als_batch, ttals_solve_batch,
 * ttals_submit).  -1 (default): autotuned -- per workload bucket (precision,
 * request kinds, largest local system, stack and operator core, and whether
 * the batch holds two requests per SM) the first
 * batches try each candidate once (every one of them solves its batch in
 * full), later ones use the fastest by kernel time per solve.  Candidates,
 * mixed precision: 0 tensor-core kernel (one CTA per SM running two requests
 * side by side, one per 256-thread group), 1 the tensor-core kernel running
 * one request on all 512 threads, 2 warp-MMA kernel at full occupancy, 3 the
 * same with one CTA per SM less; plain FP64: 0 full occupancy, 1 one CTA per
 * SM less.  -2 forgets every bucket's timings and
 * autotunes afresh.  No reference counterpart. */
int ttals_set_batch_variant(ttals_ctx* ctx, int32_t variant);

/* Batched scikit_tt/solvers/sle.py:10 `als`: `count` independent systems
 * (each with its own order, mode sizes and ranks) solved in one launch, one
 * CTA per system (one 256-thread group of a CTA on the tensor-core variant).  out_data[j] receives system j's cores with the ranks
 * ttals_als_ranks gives; all systems use `precision` and `tol`. */
int ttals_sle_als_batch(ttals_ctx* ctx, int32_t count, const ttals_tt* ops, const ttals_tt* x0s,
                        const ttals_tt* rhss, const int32_t* repeats, int32_t precision, double tol,
                        double* const* out_data, int32_t out_on_device, ttals_stats* stats);

/* Mixed batch of SLE and EVP requests (each `als` of sle.py:10 / evp.py:17),
 * one CTA (or CTA group) per request, synchronous.  Outputs follow out_on_device. */
int ttals_solve_batch(ttals_ctx* ctx, int32_t count, const ttals_request* reqs, int32_t precision, double tol,
                      int32_t out_on_device, ttals_stats* stats);

/* Serving: the same as ttals_solve_batch but asynchronous.  The call copies
 * the inputs, reserves the batch's device memory (TTALS_ERR_NOMEM, with
 * nothing allocated, when the context's budget would be exceeded -- retry
 * after finishing a job), launches on a stream of its own and returns; jobs
 * submitted while others run share the GPU.  ttals_job_poll reports
 * completion without blocking; ttals_job_finish waits, writes the outputs to
 * the requests' host pointers, releases the memory and frees the job.
 * No reference counterpart (the reference has no serving layer). */
int ttals_submit(ttals_ctx* ctx, int32_t count, const ttals_request* reqs, int32_t precision, double tol,
                 ttals_job** job);
int ttals_job_poll(ttals_job* job, int32_t* done);
/* Per-request completion: done[i] = 1 once request i's CTA has finished
 * (host-mapped flags, no device call).  ttals_job_fetch copies request i's
 * outputs while the rest of the job keeps running. */
int ttals_job_poll_each(ttals_job* job, int32_t* done);
int ttals_job_fetch(ttals_job* job, int32_t index);
/* Request `index`'s own statistics once fetched: out[0] its worst final
 * relative residual over its local solves (linear systems: FP64 residual of
 * the local system; eigenproblems: Ritz residual relative to the projected
 * operator's norm), out[1] local solves, out[2] Krylov iterations, out[3]
 * refinement cycles (SLE) or Lanczos restarts (EVP); min(cap, 4) values.
 * No reference counterpart. */
int ttals_job_report(ttals_job* job, int32_t index, double* out, int32_t cap);
int ttals_job_finish(ttals_job* job, ttals_stats* stats);
/* Device bytes a batch would reserve (admission control). */
int ttals_batch_bytes(ttals_ctx* ctx, int32_t count, const ttals_request* reqs, int64_t* bytes);

/* scikit_tt/solvers/evp.py:17 `als(operator, initial_guess, previous, shift,
 * operator_gevp=None, number_ev, repeats, conv_eps, solver, sigma, real)` for
 * symmetric operators (operator_gevp = identity; a symmetric positive
 * definite operator_gevp goes through ttals_solve_batch, TTALS_REQ_GEVP).
 * out_vals[number_ev]; out_data as for ttals_sle_als (for number_ev > 1 core
 * 0 carries a trailing axis of length number_ev, the 5-D core of
 * evp.py:492-493).  *iterations as evp.py:177. */
int ttals_evp_als(ttals_ctx* ctx, const ttals_tt* op, const ttals_tt* x0, int32_t n_previous,
                  const ttals_tt* previous, double shift, int32_t number_ev, int32_t repeats,
                  double conv_eps, int32_t solver, double sigma, int32_t precision, double tol,
                  double* out_vals, double* out_data, int32_t out_on_device, int64_t* out_ranks,
                  int32_t* iterations, ttals_stats* stats);

/* Time-dependent variational principle, scikit_tt/solvers/ode.py:1188
 * `tdvp1site` (kind 1), ode.py:1290 `tdvp2site` (kind 2) and the adaptive
 * one-/two-site mix of ode.py:1076 `tdvp` (kind 0, exact local exponentials).
 * Each step is x <- exp(tau H) x with REAL tau = -i * step_size (imaginary-time
 * steps; the caller refuses complex exponents).  krylov_dim > 1: the local
 * Krylov method of ode.py:1689 with that dimension where the reference uses it
 * (local_solver 'krylov'); 0: converged Krylov exponentials with relative
 * tolerance tol (<= 0: 1e-15) in place of scipy's expm_multiply.  threshold /
 * max_rank (<= 0: unbounded) truncate the two-site SVDs; normalize 0/1/2 scales
 * each step's state to unit 1- or 2-norm.  out receives the states after each
 * of the `steps` steps back to back (capacity: steps * sum_i c_i n_i c_{i+1}
 * doubles, c the initial ranks for kind 1, else min(prod left dims, prod
 * right dims, max_rank) but at least the initial rank); out_ranks[steps*(d+1)]. */
int ttals_tdvp(ttals_ctx* ctx, const ttals_tt* op, const ttals_tt* x0, int32_t kind, double tau, int32_t steps,
               int32_t krylov_dim, double threshold, int64_t max_rank, int32_t normalize, double tol,
               double* out, int64_t out_capacity, int32_t out_on_device, int64_t* out_ranks,
               ttals_stats* stats);

/* Alternating ridge regression, scikit_tt/data_driven/regression.py:15 `arr`:
 * one regression per output row.  theta: the basis functions of every mode
 * evaluated on the data, mode i an (basis_sizes[i] x samples) row-major block,
 * blocks back to back (regression.py:323-326); y: outputs x samples row-major;
 * initial_guesses: one TT per output (row dims = basis sizes).  Each local
 * step is the least-squares fit of lstsq(..., cond=rcond, lapack_driver=
 * 'gelss') (regression.py:487) followed by the QR/RQ re-gauging.  out: the
 * fitted trains back to back (capacity: the sum of the initial core sizes);
 * out_ranks[outputs * (order + 1)].  Host buffers. */
int ttals_arr(ttals_ctx* ctx, int32_t order, const int64_t* basis_sizes, int64_t samples, const double* theta,
              int32_t outputs, const double* y, const ttals_tt* initial_guesses, int32_t repeats, double rcond,
              double* out, int64_t out_capacity, int64_t* out_ranks, ttals_stats* stats);

/* scikit_tt/tensor_train.py:422-501 (`__matmul__` / `dot`): core-wise
 * product of two trains; out has ranks a.ranks[i] * b.ranks[i]. */
int ttals_tt_matmul(ttals_ctx* ctx, const ttals_tt* a, const ttals_tt* b, double* out_data,
                    int32_t out_on_device);

/* scikit_tt/tensor_train.py:1092-1310 (`ortho_left` / `ortho_right` without
 * truncation): Householder QR (left, direction 0) or RQ (right, direction 1)
 * sweep over cores [first, last]; out_ranks receives the new ranks. */
int ttals_tt_ortho(ttals_ctx* ctx, const ttals_tt* t, int32_t direction, int32_t first, int32_t last,
                   double* out_data, int32_t out_on_device, int64_t* out_ranks);

/* scikit_tt/tensor_train.py:1150-1181 and 1262-1296 (`ortho_left` /
 * `ortho_right` with `threshold` / `max_rank`): per core a one-sided Jacobi
 * SVD; singular values with sigma_i / sigma_0 <= threshold are dropped (none
 * when threshold == 0), then at most max_ranks[i + 1] (left) or max_ranks[i]
 * (right) are kept (max_ranks may be NULL; entries <= 0 mean no cap); S V^T
 * (left) or U S (right) moves into the neighbouring core. */
int ttals_tt_ortho_trunc(ttals_ctx* ctx, const ttals_tt* t, int32_t direction, int32_t first, int32_t last,
                         double threshold, const int64_t* max_ranks, double* out_data, int32_t out_on_device,
                         int64_t* out_ranks);

/* scikit_tt/tensor_train.py:1334-1430 (`norm(p=2)`): Euclidean/Frobenius
 * norm, computed by a QR sweep with the scale carried as a logarithm. */
int ttals_tt_norm(ttals_ctx* ctx, const ttals_tt* t, double* out_norm);

/* scikit_tt/solvers/sle.py:194-219 `__construct_stack_left_op` (left=1) and
 * sle.py:250-276 `__construct_stack_right_op` (left=0): one interface stack
 * from its neighbour `stack` (a, R, a) [left] or (s, R', s) [right], solution
 * core x (r0, n, r1) and operator core op (R, n, n, R'). */
int ttals_stack_op(ttals_ctx* ctx, int32_t left, const double* stack, const double* x,
                   const double* op, int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1,
                   double* out, int32_t on_device);

/* Allocation-free ttals_stack_op, for callers that cannot allocate device
 * memory (a process whose device memory is pre-reserved by its own pool, a
 * serving loop that must avoid the synchronisation of cudaMalloc/cudaFree, a
 * foreign host that only hands over buffers it owns).  No counterpart in the
 * reference.  All pointers must be device (or managed) memory of the
 * context's device, else TTALS_ERR_ARG before anything is enqueued; the work
 * is enqueued on the context's stream and the call returns without waiting.
 * The intermediates live in a 16 MiB static device array (2 * max(R0,R1) *
 * max(r0,r1)^2 * n doubles must fit, else TTALS_ERR_ARG).  The first call on
 * a device looks up the array's address (cudaGetSymbolAddress); make that
 * first call before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race. */
int ttals_stack_op_noalloc(ttals_ctx* ctx, int32_t left, const double* stack, const double* x,
                           const double* op, int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1,
                           double* out);

/* Diagnostic: y -> M y for the local operator in FP32 as the mixed-precision
 * inner solver computes it (tensor cores, 3xTF32), host pointers, one CTA.
 * No reference counterpart; used to test the tensor-core path directly. */
int ttals_apply_f32(ttals_ctx* ctx, const float* L, const float* A, const float* Rt, const float* y, int64_t r0,
                    int64_t n, int64_t r1, int64_t R0, int64_t R1, float* out);

/* Diagnostic: y -> M y in FP64 accuracy with the products on the BF16 tensor
 * cores (6-slice Ozaki splitting, FP32 accumulation, FP64 recombination), as
 * the mixed-precision path computes its stacks and refinement residuals.
 * Host pointers, one CTA.  No reference counterpart. */
/* Diagnostic: D = A * Bt^T on the fifth-generation tensor cores (one
 * tcgen05.mma tile of M = 128 rows: operands staged in shared memory, FP32
 * accumulator in tensor memory), kind 0 BF16 or 1 TF32 inputs; A is 128 x K,
 * Bt is N x K, out is 128 x N, all row-major host arrays.  No reference
 * counterpart; pins the tensor-core encodings the batch kernel uses. */
int ttals_umma_selftest(ttals_ctx* ctx, int32_t kind, int32_t N, int32_t K, const float* A, const float* Bt,
                        float* out);

int ttals_apply_f64emu(ttals_ctx* ctx, const double* L, const double* A, const double* Rt, const double* y,
                       int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1, double* out);

/* scikit_tt/solvers/sle.py:308-347 `__construct_micro_matrix_als`: dense
 * local operator (r0*n*r1)^2 from stacks L (r0, R0, r0), Rt (r1, R1, r1) and
 * operator core op (R0, n, n, R1). */
int ttals_micro_matrix(ttals_ctx* ctx, const double* L, const double* op, const double* Rt,
                       int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1, double* out,
                       int32_t on_device);

#ifdef __cplusplus
}
#endif

#endif /* TTALS_H_ */
