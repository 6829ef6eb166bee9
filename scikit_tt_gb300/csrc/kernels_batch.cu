// Batched ALS: one CTA runs one complete ALS solve.
//
// Independent instances (uneven order d, mode sizes and ranks) are taken from
// a device work counter by persistent CTAs; each CTA runs the whole program of
// scikit_tt/solvers/sle.py:10-95 (or evp.py:17-179) for its instance --
// right-orthonormalisation of the guess, initial right stacks, forward and
// backward half-sweeps with matrix-free local solves and QR/RQ re-gauging --
// with nothing but CTA barriers.  No grid-wide synchronisation exists, so the
// GPU fills with instances and FP64 work runs at the device's FP64 rate.
//
// Local solves: GMRES with FP64 residual refinement (inner Krylov in FP32 for
// PREC_MIXED, FP64 otherwise) and, for eigenproblems, Lanczos with full
// reorthogonalisation.  Contractions use the descriptors of ttals_desc.cuh.
#include <float.h>

#include <type_traits>

#include "ttals_batch.h"
#include "ttals_desc.cuh"
#include "ttals_internal.h"
#include "ttals_qr.cuh"
#include "ttals_tc.cuh"
#include "ttals_ozaki.cuh"
#include "ttals_tc_gemm.cuh"
#include "ttals_tri.cuh"

namespace ttals {

constexpr int kMaxOrderB = 256;
// Lanczos restarts per local eigensolve (64-vector basis, restarted from the
// Ritz vector): most sites converge within a few.  A site whose wanted
// eigenvalue is nearly degenerate with the next one (the ferromagnetic Ising
// chain, g ~ 0.57 at d = 42) stagnates near 1e-7 whatever the budget: a larger
// one only costs time there
constexpr int kBatchEvpRestarts = 40;
constexpr int kBatchThreads = 128;
// five CTAs per SM (102 registers a thread): FP32 and FP64 phases of different
// instances overlap, and the memory-latency-bound loops get more warps to hide
// latency behind (measured: +4 % over four CTAs per SM, with 5 x SMs requests)
constexpr int kBatchMinBlocks = 5;
// tensor-core variant: a kernel with tcgen05 instructions runs one CTA per
// SM, which then owns the whole SM.  It runs two solves side by side, one per
// 256-thread group (each with half of the TMEM columns, its own operand tiles
// and named barriers), so that one solve's latency-bound phases (Krylov
// vector loops, QR, waits on MMA completion) overlap the other's products.
constexpr int kBatchThreadsTc = kGroupThreads * kGroups<true>;
constexpr int kBatchMinBlocksTc = 1;

// ---------------------------------------------------------------------------
// CTA primitives
// ---------------------------------------------------------------------------

// Inlined body (used inside the Krylov loops); `c` must not alias C.
// TC: the kernel holds tensor memory and uses tcgen05.  A kernel that contains
// any tcgen05 instruction runs one CTA per SM, so the paths without it are
// separate instantiations (TC = false) free of tcgen05 code.
// TC also selects the two-group form (every CTA routine below runs on the
// calling group: gtid / gsize / gsync of ttals_device.cuh).
template <typename T, bool TC = false, bool G = TC>
__device__ __forceinline__ void cta_contract_body(const Contraction& c, const T* A, const T* B, T* C,
                                                  int* ktab = nullptr, TcState* tc = nullptr) {
  if constexpr (std::is_same<T, float>::value) {
    // FP32 (inner Krylov) contractions go to the tensor cores when GEMM-shaped:
    // tcgen05 (3xTF32, operands staged in shared memory, TMEM accumulator)
    // when the CTA holds tensor memory, warp-level mma.sync otherwise
    if constexpr (TC) {
      if (tc && ktab) {
        const bool done = cta_gemm_tf32_tc<G>(c, A, B, C, ktab, *tc);
        if (gtid<G>() == 0) {
          if (done)
            ++tc->gemms;
          else
            ++tc->fallbacks;
        }
        if (done) return;
      }
    }
    if (ktab && cta_gemm_tf32x3<G>(c, A, B, C, ktab)) return;
  }
  constexpr int VW = DefaultVW<T>::value;
  if (contract_vec_ok<T, VW>(c, B, C)) {
    for (int64_t e = (int64_t)gtid<G>() * VW; e < c.total; e += (int64_t)gsize<G>() * VW)
      contract_vec_elem<T, VW>(c, A, B, C, e);
  } else {
    for (int64_t e = gtid<G>(); e < c.total; e += gsize<G>()) {
      int64_t ao, bo, co;
      contract_offsets(c, e, ao, bo, co);
      C[co] = contract_sum(c, A, B, ao, bo);
    }
  }
  gsync<G>();
}

// FP64 contraction; with `oz` set, GEMM-shaped ones run as emulated FP64 on the
// BF16 tensor cores (ttals_ozaki.cuh), the rest natively.  A contraction over
// fewer than kOzMinK elements stays native: measured on a batch of 32 Ising
// eigenproblems (whose middle contraction has K = 6) 16 % faster than
// emulating it, and no change on the SLE batches.
constexpr int kOzMinK = 16;
template <bool TC, bool G = TC>
__device__ __noinline__ void cta_contract_f64(const Contraction& cref, const double* A, const double* B, double* C,
                                              const OzScratch* oz) {
  __shared__ Contraction sc_g[kGroups<G>];
  Contraction& sc = sc_g[gidx<G>()];
  if (gtid<G>() == 0) sc = cref;
  gsync<G>();
  if (sc.ktotal < kOzMinK) oz = nullptr;
  if constexpr (TC) {
    if (oz && oz->tc) {
      const bool done = cta_gemm_oz_tc<G>(sc, A, B, C, *oz, oz->ktab, *oz->tc);
      if (gtid<G>() == 0) {
        if (done)
          ++oz->tc->gemms;
        else
          ++oz->tc->fallbacks;
      }
      if (done) return;
    }
  } else {
    if (oz && cta_gemm_ozaki(sc, A, B, C, *oz, oz->ktab)) return;
  }
  cta_contract_body<double, TC, G>(sc, A, B, C);
}

// Out-of-line version for the per-site bookkeeping (stacks, pushes): keeps the
// register pressure of the instance driver low.  The descriptor is copied to
// shared memory so that stores to C cannot alias it.
template <typename T, bool G = false>
__device__ __noinline__ void cta_contract(const Contraction& cref, const T* A, const T* B, T* C) {
  __shared__ Contraction sc_g[kGroups<G>];
  Contraction& sc = sc_g[gidx<G>()];
  if (gtid<G>() == 0) sc = cref;
  gsync<G>();
  cta_contract_body<T, G>(sc, A, B, C);
}

// Out-of-line FP32 contraction of the inner Krylov apply: one copy of the
// tensor-core and fallback paths instead of three inlined into the GMRES loop
// (which otherwise spills).
template <bool TC, bool G = TC>
__device__ __noinline__ void cta_contract_f32(const Contraction& cref, const float* A, const float* B, float* C,
                                              int* ktab, TcState* tc) {
  __shared__ Contraction sc_g[kGroups<G>];
  Contraction& sc = sc_g[gidx<G>()];
  if (gtid<G>() == 0) sc = cref;
  gsync<G>();
  cta_contract_body<float, TC, G>(sc, A, B, C, ktab, tc);
}

template <bool G = false>
__device__ __forceinline__ void cta_fill(double* p, int64_t n, double v) {
  for (int64_t i = gtid<G>(); i < n; i += gsize<G>()) p[i] = v;
  gsync<G>();
}
template <bool G = false>
__device__ __forceinline__ void cta_copy(double* d, const double* s, int64_t n) {
  for (int64_t i = gtid<G>(); i < n; i += gsize<G>()) d[i] = s[i];
  gsync<G>();
}
template <bool G = false>
__device__ __forceinline__ void cta_to_float(float* d, const double* s, int64_t n) {
  for (int64_t i = gtid<G>(); i < n; i += gsize<G>()) d[i] = (float)s[i];
  gsync<G>();
}

// sum over the CTA (the group), returned to every thread
template <bool G = false>
__device__ __forceinline__ double cta_sum(double v) {
  __shared__ double red_g[kGroups<G>][32];
  double* red = red_g[gidx<G>()];
  const int lane = gtid<G>() & 31, warp = gtid<G>() >> 5, nw = gsize<G>() >> 5;
  v = warp_sum(v);
  if (lane == 0) red[warp] = v;
  gsync<G>();
  double s = 0.0;
  for (int w = 0; w < nw; ++w) s += red[w];
  gsync<G>();
  return s;
}

// out[kk] = <X_kk, w> for kk < nvec (X_kk = V + kk*N), out[nvec] = <w, w>
// Dots accumulate in the vectors' own precision (FP32 for the inner solver:
// its Gram-Schmidt only needs inner-solver accuracy, and FP64 arithmetic is
// 57x slower on this part); lane partial sums keep the rounding error ~sqrt(N).
template <typename T, bool G = false>
__device__ __forceinline__ void cta_dots(const T* V, int64_t N, int nvec, const T* w, double* out) {
  const int lane = gtid<G>() & 31, warp = gtid<G>() >> 5, nw = gsize<G>() >> 5;
  for (int kk = warp; kk <= nvec; kk += nw) {
    const T* xv = (kk < nvec) ? V + (int64_t)kk * N : w;
    T s0 = T(0), s1 = T(0);
    int64_t e = lane;
    for (; e + 32 < N; e += 64) {
      s0 += xv[e] * w[e];
      s1 += xv[e + 32] * w[e + 32];
    }
    if (e < N) s0 += xv[e] * w[e];
    const T st = warp_sum(s0 + s1);
    if (lane == 0) out[kk] = (double)st;
  }
  gsync<G>();
}

// The same with every thread of the CTA: each thread keeps a partial sum per
// vector over its own elements (four loads in flight), reduced per warp and
// then over warps.  For the one-CTA-per-SM tensor-core kernel, where no
// sibling CTA hides memory latency; nvec <= kWideDotsMax.
constexpr int kWideDotsMax = 64;
template <typename T, bool G = false>
__device__ __noinline__ void cta_dots_wide(const T* V, int64_t N, int nvec, const T* w, double* out) {
  constexpr int kWarps = G ? kGroupThreads / 32 : 32;
  __shared__ double part_g[kGroups<G>][kWarps][kWideDotsMax + 1];
  double(*part)[kWideDotsMax + 1] = part_g[gidx<G>()];
  const int tid = gtid<G>(), nt = gsize<G>(), lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int kk = 0; kk <= nvec; ++kk) {
    const T* xv = (kk < nvec) ? V + (int64_t)kk * N : w;
    T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
    int64_t e = tid;
    for (; e + 3 * (int64_t)nt < N; e += 4 * (int64_t)nt) {
      s0 += xv[e] * w[e];
      s1 += xv[e + nt] * w[e + nt];
      s2 += xv[e + 2 * nt] * w[e + 2 * nt];
      s3 += xv[e + 3 * nt] * w[e + 3 * nt];
    }
    for (; e < N; e += nt) s0 += xv[e] * w[e];
    // FP32 vectors reduce in FP32 within the warp (no per-lane conversions
    // to FP64, whose pipe runs two FMAs per clock per SM); the warps' sums
    // are added in FP64
    T sd = (s0 + s1) + (s2 + s3);
    sd = warp_sum(sd);
    if (lane == 0) part[warp][kk] = (double)sd;
  }
  gsync<G>();
  for (int kk = tid; kk <= nvec; kk += nt) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += part[q][kk];
    out[kk] = t;
  }
  gsync<G>();
}

// y -> out = M y (three contraction phases through T1, T2)
template <typename T, bool TC = false, bool G = TC>
__device__ __forceinline__ void cta_apply(const Contraction& p1, const Contraction& p2, const Contraction& p3,
                                          const T* L, const T* A, const T* R, const T* y, T* T1, T* T2, T* out,
                                          int* ktab = nullptr, TcState* tc = nullptr) {
  if constexpr (std::is_same<T, float>::value) {
    cta_contract_f32<TC, G>(p1, L, y, T1, ktab, tc);
    cta_contract_f32<TC, G>(p2, T1, A, T2, ktab, tc);
    cta_contract_f32<TC, G>(p3, T2, R, out, ktab, tc);
  } else {
    cta_contract_body<T, TC, G>(p1, L, y, T1, ktab);
    cta_contract_body<T, TC, G>(p2, T1, A, T2, ktab);
    cta_contract_body<T, TC, G>(p3, T2, R, out, ktab);
  }
}

// ---------------------------------------------------------------------------
// CTA GMRES with FP64 residual refinement (see gmres_ir_kernel for the grid version)
// ---------------------------------------------------------------------------

struct CtaSolveStats {
  double rel;
  int cycles, inner, status;
};

template <typename TI, bool TC, bool G = TC>
__device__ __noinline__ CtaSolveStats cta_gmres_ir(const Contraction& p1, const Contraction& p2, const Contraction& p3,
                                      const double* L64, const double* A64, const double* R64, double* T1_64,
                                      double* T2_64, const TI* Li, const TI* Ai, const TI* Ri, TI* T1i, TI* T2i,
                                      const double* f, double* x, double* r, TI* V, TI* w, int64_t N, int m,
                                      int max_cycles, double tol, double inner_floor, double* sm,
                                      const OzScratch* oz, long long* cyc_res, long long* cyc_inner,
                                      long long* cyc_apply) {
  double* H = sm;                // (m+1) x m
  double* cs = H + (m + 1) * m;  // m
  double* sn = cs + m;           // m
  double* gv = sn + m;           // m+1
  double* yv = gv + m + 1;       // m
  double* h1 = yv + m;           // m+2
  double* h2 = h1 + m + 2;       // m+2
  __shared__ double s_res_g[kGroups<G>];
  __shared__ int s_flag_g[kGroups<G>];
  __shared__ float s_cf_g[kGroups<G>][kWideDotsMax + 2];  // Gram-Schmidt / correction coefficients in TI (TC path)
  double& s_res = s_res_g[gidx<G>()];
  int& s_flag = s_flag_g[gidx<G>()];
  float* s_cf = s_cf_g[gidx<G>()];
  const int tid = gtid<G>(), nt = gsize<G>();
  CtaSolveStats out{1.0, 0, 0, ST_OK};
  // the tensor-core kernel runs one CTA per SM: its vector loops use every
  // thread, keep several loads in flight and avoid per-element FP64 work
  constexpr bool kWide = TC && std::is_same<TI, float>::value;
  auto dots = [&](int nv, const TI* wv, double* o) {
    if constexpr (kWide)
      cta_dots_wide<TI, G>(V, N, nv, wv, o);
    else
      cta_dots<TI, G>(V, N, nv, wv, o);
  };

  double fs = 0.0;
  for (int64_t e = tid; e < N; e += nt) fs += f[e] * f[e];
  const double fnorm = sqrt(cta_sum<G>(fs));
  if (!(fnorm > 0.0)) {
    for (int64_t e = tid; e < N; e += nt) x[e] = 0.0;
    gsync<G>();
    out.rel = 0.0;
    if (!(fnorm == 0.0)) out.status = ST_NONFINITE;
    return out;
  }
  for (int cyc = 0; cyc < max_cycles; ++cyc) {
    const long long c0 = clock64();
    double rs = 0.0;
    if (oz) {
      // FP64-accurate residual with the products on the BF16 tensor cores
      cta_contract_f64<TC, G>(p1, L64, (const double*)x, T1_64, oz);
      cta_contract_f64<TC, G>(p2, (const double*)T1_64, A64, T2_64, oz);
      cta_contract_f64<TC, G>(p3, (const double*)T2_64, R64, r, oz);
      for (int64_t e = tid; e < N; e += nt) {
        const double re = f[e] - r[e];
        r[e] = re;
        rs += re * re;
      }
    } else {
      cta_contract_body<double, TC, G>(p1, L64, (const double*)x, T1_64);
      cta_contract_body<double, TC, G>(p2, (const double*)T1_64, A64, T2_64);
      for (int64_t e = tid; e < N; e += nt) {
        int64_t ao, bo, co;
        contract_offsets(p3, e, ao, bo, co);
        const double re = f[e] - contract_sum(p3, (const double*)T2_64, R64, ao, bo);
        r[e] = re;
        rs += re * re;
      }
    }
    const double rho = sqrt(cta_sum<G>(rs));
    *cyc_res += clock64() - c0;
    const long long c1 = clock64();
    out.rel = rho / fnorm;
    out.cycles = cyc + 1;
    if (!isfinite(out.rel)) {
      out.status = ST_NONFINITE;
      return out;
    }
    if (out.rel <= tol) break;
    const double target = fmax(tol / out.rel, inner_floor);
    const double irho = 1.0 / rho;
    for (int64_t e = tid; e < N; e += nt) V[e] = (TI)(r[e] * irho);
    if (tid == 0) {
      gv[0] = 1.0;
      for (int i = 1; i <= m; ++i) gv[i] = 0.0;
    }
    gsync<G>();
    int jj = 0;
    for (int j = 0; j < m; ++j) {
      const long long ca0 = clock64();
      cta_apply<TI, TC, G>(p1, p2, p3, Li, Ai, Ri, V + (int64_t)j * N, T1i, T2i, w, oz ? oz->ktab : nullptr,
                        oz ? oz->tc : nullptr);
      *cyc_apply += clock64() - ca0;
      dots(j + 1, w, h1);
      // Classical Gram-Schmidt with selective reorthogonalisation (FP32 inner
      // solves): one projection suffices when it keeps at least 1/sqrt(2) of the
      // norm ("twice is enough" criterion); then the projection and the
      // normalisation are one pass over the basis.  The FP64 solver always
      // projects twice.
      double wn2 = h1[j + 1], hn2 = wn2;
      for (int q = 0; q <= j; ++q) hn2 -= h1[q] * h1[q];
      const bool single = sizeof(TI) == 4 && hn2 >= 0.5 * wn2;
      double hn;
      if (single) {
        if (tid == 0)
          for (int q = 0; q <= j + 1; ++q) h2[q] = 0.0;
        hn = sqrt(fmax(hn2, 0.0));
        if (hn > 0.0) {
          const TI inv = (TI)(1.0 / hn);
          TI* vn = V + (int64_t)(j + 1) * N;
          if constexpr (kWide) {
            for (int q = tid; q <= j; q += nt) s_cf[q] = (float)h1[q];
            gsync<G>();
            for (int64_t e = tid; e < N; e += nt) {
              TI acc = w[e];
#pragma unroll 4
              for (int q = 0; q <= j; ++q) acc -= s_cf[q] * V[(int64_t)q * N + e];
              vn[e] = acc * inv;
            }
          } else {
            for (int64_t e = tid; e < N; e += nt) {
              TI acc = w[e];
              for (int q = 0; q <= j; ++q) acc -= (TI)h1[q] * V[(int64_t)q * N + e];
              vn[e] = acc * inv;
            }
          }
        }
      } else {
        for (int64_t e = tid; e < N; e += nt) {
          TI acc = w[e];
          for (int q = 0; q <= j; ++q) acc -= (TI)h1[q] * V[(int64_t)q * N + e];
          w[e] = acc;
        }
        gsync<G>();
        dots(j + 1, w, h2);
        hn2 = h2[j + 1];
        for (int q = 0; q <= j; ++q) hn2 -= h2[q] * h2[q];
        hn = sqrt(fmax(hn2, 0.0));
        if (hn > 0.0) {
          const TI inv = (TI)(1.0 / hn);
          TI* vn = V + (int64_t)(j + 1) * N;
          for (int64_t e = tid; e < N; e += nt) {
            TI acc = w[e];
            for (int q = 0; q <= j; ++q) acc -= (TI)h2[q] * V[(int64_t)q * N + e];
            vn[e] = acc * inv;
          }
        }
      }
      if (tid == 0) {
        double* col = H + (int64_t)j * (m + 1);
        for (int i = 0; i <= j; ++i) col[i] = h1[i] + h2[i];
        col[j + 1] = hn;
        for (int i = 0; i < j; ++i) {
          const double t = cs[i] * col[i] + sn[i] * col[i + 1];
          col[i + 1] = -sn[i] * col[i] + cs[i] * col[i + 1];
          col[i] = t;
        }
        const double a = col[j], b = col[j + 1];
        double c = 1.0, sg = 0.0, rr = a;
        if (b != 0.0) {
          rr = hypot(a, b);
          c = a / rr;
          sg = b / rr;
        }
        cs[j] = c;
        sn[j] = sg;
        col[j] = rr;
        col[j + 1] = 0.0;
        gv[j + 1] = -sg * gv[j];
        gv[j] = c * gv[j];
        s_res = fabs(gv[j + 1]);
        s_flag = (hn <= 1e-300) ? 1 : 0;
      }
      gsync<G>();
      jj = j + 1;
      ++out.inner;
      if (s_res <= target || s_flag) break;
    }
    if (tid == 0) {
      int bad = 0;
      for (int i = jj - 1; i >= 0; --i) {
        double acc = gv[i];
        for (int l = i + 1; l < jj; ++l) acc -= H[(int64_t)l * (m + 1) + i] * yv[l];
        const double dg = H[(int64_t)i * (m + 1) + i];
        if (dg == 0.0) {
          bad = 1;
          yv[i] = 0.0;
        } else {
          yv[i] = acc / dg;
        }
      }
      s_flag = bad;
    }
    gsync<G>();
    if (s_flag) {
      out.status = ST_SINGULAR;
      return out;
    }
    if constexpr (kWide) {
      // the correction V y is FP32-accurate by construction: sum it in FP32,
      // one FP64 FMA per element adds it to the FP64 solution
      for (int q = tid; q < jj; q += nt) s_cf[q] = (float)yv[q];
      gsync<G>();
      for (int64_t e = tid; e < N; e += nt) {
        float acc = 0.f;
#pragma unroll 4
        for (int q = 0; q < jj; ++q) acc += s_cf[q] * V[(int64_t)q * N + e];
        x[e] += rho * (double)acc;
      }
    } else {
      for (int64_t e = tid; e < N; e += nt) {
        double acc = 0.0;
        for (int q = 0; q < jj; ++q) acc += yv[q] * (double)V[(int64_t)q * N + e];
        x[e] += rho * acc;
      }
    }
    gsync<G>();
    *cyc_inner += clock64() - c1;
  }
  return out;
}

// ---------------------------------------------------------------------------
// CTA Lanczos (FP64, one eigenpair) for the symmetric local eigenproblem
// (see lanczos_kernel for the grid version and the selection rules)
// ---------------------------------------------------------------------------

// Symmetric eigen-decomposition of H (n x n, leading dimension ld, n <= 64)
// by the group: cyclic Jacobi with the round-robin parallel ordering (n/2
// disjoint rotations per round, each applied to the columns of H and Z, then
// to the rows of H), until the off-diagonal mass is below 1e-32 of the total
// (at most 30 sweeps).  On return H's diagonal holds the eigenvalues and Z's
// columns the eigenvectors.
constexpr int kSymEigMax = 64;
template <bool G>
__device__ __noinline__ void cta_sym_eig(double* H, double* Z, int n, int ld) {
  __shared__ int ra_g[kGroups<G>][kSymEigMax / 2], rb_g[kGroups<G>][kSymEigMax / 2];
  __shared__ double rc_g[kGroups<G>][kSymEigMax / 2], rs_g[kGroups<G>][kSymEigMax / 2];
  int* ra = ra_g[gidx<G>()];
  int* rb = rb_g[gidx<G>()];
  double* rc = rc_g[gidx<G>()];
  double* rs = rs_g[gidx<G>()];
  const int tid = gtid<G>(), nt = gsize<G>();
  const int npl = n + (n & 1), npairs = npl / 2;
  for (int idx = tid; idx < n * n; idx += nt) {
    const int r = idx / n, c = idx - r * n;
    Z[r * ld + c] = r == c ? 1.0 : 0.0;
  }
  gsync<G>();
  if (n < 2) return;
  for (int sweep = 0; sweep < 30; ++sweep) {
    double so = 0.0, st = 0.0;
    for (int idx = tid; idx < n * n; idx += nt) {
      const int r = idx / n, c = idx - r * n;
      const double v = H[r * ld + c];
      st += v * v;
      if (r < c) so += v * v;
    }
    so = cta_sum<G>(so);
    st = cta_sum<G>(st);
    if (!(so > 1e-32 * st)) break;
    for (int round = 0; round < npl - 1; ++round) {
      if (tid < npairs) {
        const int pk = tid, qk = npl - 1 - tid;
        int a = pk == 0 ? 0 : 1 + (pk - 1 + round) % (npl - 1);
        int b = 1 + (qk - 1 + round) % (npl - 1);
        if (a > b) {
          const int t = a;
          a = b;
          b = t;
        }
        double c = 1.0, sn = 0.0;
        if (b < n) {
          const double apq = H[a * ld + b];
          if (fabs(apq) > 1e-300) {
            const double theta = (H[b * ld + b] - H[a * ld + a]) / (2.0 * apq);
            const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
            c = 1.0 / sqrt(fma(t, t, 1.0));
            sn = t * c;
          }
        }
        ra[tid] = (b < n && sn != 0.0) ? a : -1;
        rb[tid] = b;
        rc[tid] = c;
        rs[tid] = sn;
      }
      gsync<G>();
      for (int idx = tid; idx < npairs * n; idx += nt) {
        const int k = idx / n, i = idx - k * n;
        const int a = ra[k];
        if (a < 0) continue;
        const int b = rb[k];
        const double c = rc[k], sn = rs[k];
        const double ha = H[i * ld + a], hb = H[i * ld + b];
        H[i * ld + a] = c * ha - sn * hb;
        H[i * ld + b] = sn * ha + c * hb;
        const double za = Z[i * ld + a], zb = Z[i * ld + b];
        Z[i * ld + a] = c * za - sn * zb;
        Z[i * ld + b] = sn * za + c * zb;
      }
      gsync<G>();
      for (int idx = tid; idx < npairs * n; idx += nt) {
        const int k = idx / n, i = idx - k * n;
        const int a = ra[k];
        if (a < 0) continue;
        const int b = rb[k];
        const double c = rc[k], sn = rs[k];
        const double ha = H[a * ld + i], hb = H[b * ld + i];
        H[a * ld + i] = c * ha - sn * hb;
        H[b * ld + i] = sn * ha + c * hb;
      }
      gsync<G>();
    }
  }
}

// Ritz vectors kept by a thick restart of the CTA Lanczos, and the restarts
// from a single Ritz vector tried before the thick ones
constexpr int kLanczosKeep = 8;
constexpr int kPlainRestarts = 3;

struct CtaEigStats {
  double theta, res;
  int its, restarts, status;
};

// TI: arithmetic of the operator, basis and products (double, or float for
// the first stage of the mixed-precision eigensolve).  x (in: start vector,
// out: Ritz vector) and all scalars stay FP64.
template <typename TI, bool TC = false, bool G = TC>
__device__ __noinline__ CtaEigStats cta_lanczos(const Contraction& p1, const Contraction& p2, const Contraction& p3,
                                               const TI* L, const TI* A, const TI* R, TI* T1, TI* T2, double* x,
                                               TI* V, TI* w, int64_t N, int m, int mode, double sigma,
                                               int max_restarts, double tol, double* sm,
                                               const OzScratch* oz = nullptr, double* dense = nullptr) {
  double* al = sm;
  double* be = al + m;
  double* h1 = be + m;
  double* h2 = h1 + m + 2;
  double* z = h2 + m + 2;
  double* twk = z + m;
  int* piv = (int*)(twk + 5 * m + 8);
  __shared__ double s_theta_g[kGroups<G>], s_res_g[kGroups<G>];
  __shared__ int s_conv_g[kGroups<G>];
  double& s_theta = s_theta_g[gidx<G>()];
  double& s_res = s_res_g[gidx<G>()];
  int& s_conv = s_conv_g[gidx<G>()];
  const int tid = gtid<G>(), nt = gsize<G>(), lane = tid & 31, warp = tid >> 5;
  CtaEigStats out{0.0, 0.0, 0, 0, ST_OK};
  if (tid == 0) {
    s_conv = 0;
    s_theta = 0.0;
    s_res = 0.0;
  }
  double xs = 0.0;
  for (int64_t e = tid; e < N; e += nt) xs += x[e] * x[e];
  const double xn = sqrt(cta_sum<G>(xs));
  const bool ok = xn > 0.0 && isfinite(xn);
  for (int64_t e = tid; e < N; e += nt) V[e] = (TI)(ok ? x[e] / xn : 1.0 / sqrt((double)N));
  gsync<G>();
  const int mm = (int)(N < m ? N : m);
  // thick restarts (after a first cycle without convergence): kk Ritz vectors
  // kept in V[0, kk), their values th and couplings bb to V[kk]
  __shared__ double th_g[kGroups<G>][kLanczosKeep], bb_g[kGroups<G>][kLanczosKeep];
  __shared__ int sel_g[kGroups<G>][kLanczosKeep];
  __shared__ int s_keep_g[kGroups<G>];
  double* th = th_g[gidx<G>()];
  double* bb = bb_g[gidx<G>()];
  int* selk = sel_g[gidx<G>()];
  int& s_keep = s_keep_g[gidx<G>()];
  const bool can_thick = dense != nullptr && mm > kLanczosKeep + 1;
  bool thick = false;
  int kk = 0;
  for (;;) {
    int nT = kk;
    for (int j = kk; j < mm; ++j) {
      if constexpr (std::is_same<TI, double>::value) {
        if (oz) {
          // FP64-accurate products on the tensor cores (emulated FP64)
          cta_contract_f64<TC, G>(p1, L, V + (int64_t)j * N, T1, oz);
          cta_contract_f64<TC, G>(p2, T1, A, T2, oz);
          cta_contract_f64<TC, G>(p3, T2, R, w, oz);
        } else {
          cta_apply<TI, G>(p1, p2, p3, L, A, R, V + (int64_t)j * N, T1, T2, w);
        }
      } else {
        cta_apply<TI, G>(p1, p2, p3, L, A, R, V + (int64_t)j * N, T1, T2, w);
      }
      cta_dots<TI, G>(V, N, j + 1, w, h1);
      for (int64_t e = tid; e < N; e += nt) {
        double acc = (double)w[e];
        for (int q = 0; q <= j; ++q) acc -= h1[q] * (double)V[(int64_t)q * N + e];
        w[e] = (TI)acc;
      }
      gsync<G>();
      cta_dots<TI, G>(V, N, j + 1, w, h2);
      double b2 = h2[j + 1];
      for (int q = 0; q <= j; ++q) b2 -= h2[q] * h2[q];
      const double bj = sqrt(fmax(b2, 0.0));
      if (tid == 0) {
        al[j] = h1[j] + h2[j];
        be[j] = bj;
      }
      if (bj > 0.0 && (j + 1 < mm || can_thick)) {
        TI* vn = V + (int64_t)(j + 1) * N;
        const double inv = 1.0 / bj;
        for (int64_t e = tid; e < N; e += nt) {
          double acc = (double)w[e];
          for (int q = 0; q <= j; ++q) acc -= h2[q] * (double)V[(int64_t)q * N + e];
          vn[e] = (TI)(acc * inv);
        }
      }
      gsync<G>();
      ++out.its;
      nT = j + 1;
      double tnorm = 0.0;
      for (int i = kk; i < nT; ++i)
        tnorm = fmax(tnorm, fabs(al[i]) + fabs(be[i]) + (i > kk ? fabs(be[i - 1]) : 0.0));
      const bool breakdown = !(bj > 1e-14 * fmax(tnorm, 1e-300));
      if (thick) {
        if (breakdown) break;
        continue;
      }
      if ((nT % 4) == 0 || nT == mm || breakdown) {
        if (warp == 0) {
          double lo = 1e300, hi = -1e300;
          for (int i = 0; i < nT; ++i) {
            const double rad = (i > 0 ? fabs(be[i - 1]) : 0.0) + (i < nT - 1 ? fabs(be[i]) : 0.0);
            lo = fmin(lo, al[i] - rad);
            hi = fmax(hi, al[i] + rad);
          }
          const double pivmin = 1e-300 + DBL_MIN * fmax(1.0, tnorm * tnorm);
          lo -= 1e-12 * fmax(1.0, tnorm);
          hi += 1e-12 * fmax(1.0, tnorm);
          int sel;
          if (mode == 0) {
            sel = nT - 1;
          } else if (mode == 2) {
            sel = 0;
          } else {
            const int below = sturm_count(al, be, nT, sigma, pivmin);
            const double vdn = below > 0 ? tri_eigval(al, be, nT, below - 1, lo, hi, pivmin) : 0.0;
            const double vup = below < nT ? tri_eigval(al, be, nT, below, lo, hi, pivmin) : 0.0;
            sel = (below > 0 && (below >= nT || fabs(vdn - sigma) <= fabs(vup - sigma))) ? below - 1 : below;
          }
          const double th = tri_eigval(al, be, nT, sel, lo, hi, pivmin);
          if (lane == 0) {
            tri_eigvec(al, be, nT, th, fmax(tnorm, 1e-300), z, twk, piv);
            s_theta = th;
            s_res = bj * fabs(z[nT - 1]) / fmax(tnorm, 1e-300);
            s_conv = (s_res <= tol) || breakdown;
          }
        }
        gsync<G>();
        if (s_conv || nT == mm) break;
      } else if (breakdown) {
        break;
      }
    }
    if (!thick) {
      if (s_conv || out.restarts >= max_restarts || !can_thick || nT < mm || out.restarts < kPlainRestarts) {
        // Ritz vector of the tridiagonal matrix
        for (int64_t e = tid; e < N; e += nt) {
          double acc = 0.0;
          for (int l = 0; l < nT; ++l) acc += z[l] * (double)V[(int64_t)l * N + e];
          x[e] = acc;
        }
        gsync<G>();
        if (s_conv || out.restarts >= max_restarts || nT < mm) break;
        // restart from the Ritz vector (bases too small for thick restarts,
        // and the first restarts: most slow local solves converge within a
        // few of them, checked every four steps)
        ++out.restarts;
        double s2 = 0.0;
        for (int64_t e = tid; e < N; e += nt) s2 += x[e] * x[e];
        const double nrm = sqrt(cta_sum<G>(s2));
        for (int64_t e = tid; e < N; e += nt) V[e] = (TI)(nrm > 0.0 ? x[e] / nrm : 1.0 / sqrt((double)N));
        gsync<G>();
        continue;
      }
      thick = true;  // still not converged: thick restarts from here on
    }
    // Projected matrix of the cycle: kept Ritz values on the diagonal, their
    // couplings to V[kk] (arrow), the cycle's tridiagonal part; its
    // eigen-decomposition (Jacobi) gives the Ritz pairs of the whole basis.
    double* H = dense;
    double* Z = dense + (int64_t)m * m;
    for (int idx = tid; idx < nT * nT; idx += nt) {
      const int r = idx / nT, c = idx - r * nT;
      double v = 0.0;
      if (r == c) v = r < kk ? th[r] : al[r];
      else if (r < kk && c == kk) v = bb[r];
      else if (c < kk && r == kk) v = bb[c];
      else if (r >= kk && c >= kk && (r == c + 1 || c == r + 1)) v = be[r < c ? r : c];
      H[r * m + c] = v;
    }
    gsync<G>();
    cta_sym_eig<G>(H, Z, nT, m);
    const double blast = be[nT - 1];
    if (tid == 0) {
      // wanted pair and the kLanczosKeep best by the selection rule
      double tn = 0.0;
      for (int i = 0; i < nT; ++i) tn = fmax(tn, fabs(H[i * m + i]));
      const int kkeep = nT - 1 < kLanczosKeep ? nT - 1 : kLanczosKeep;
      for (int q = 0; q < kkeep; ++q) {
        int best = -1;
        double bkey = 0.0;
        for (int i = 0; i < nT; ++i) {
          bool used = false;
          for (int u = 0; u < q; ++u) used |= selk[u] == i;
          if (used) continue;
          const double t = H[i * m + i];
          const double key = mode == 0 ? -t : (mode == 2 ? t : fabs(t - sigma));
          if (best < 0 || key < bkey) {
            best = i;
            bkey = key;
          }
        }
        selk[q] = best;
      }
      s_keep = kkeep;
      s_theta = H[selk[0] * m + selk[0]];
      s_res = fabs(blast * Z[(nT - 1) * m + selk[0]]) / fmax(tn, 1e-300);
      s_conv = s_res <= tol;
    }
    gsync<G>();
    if (s_conv || out.restarts >= max_restarts || nT < mm) {
      const int w0 = selk[0];
      for (int64_t e = tid; e < N; e += nt) {
        double acc = 0.0;
        for (int l = 0; l < nT; ++l) acc += Z[l * m + w0] * (double)V[(int64_t)l * N + e];
        x[e] = acc;
      }
      gsync<G>();
      break;
    }
    ++out.restarts;
    // new basis: V[0, k) = V Z[:, sel] (element by element, so in place), V[k] = V[nT]
    const int k = s_keep;
    for (int64_t e = tid; e < N; e += nt) {
      double acc[kLanczosKeep];
#pragma unroll
      for (int i = 0; i < kLanczosKeep; ++i) acc[i] = 0.0;
      for (int l = 0; l < nT; ++l) {
        const double v = (double)V[(int64_t)l * N + e];
#pragma unroll
        for (int i = 0; i < kLanczosKeep; ++i)
          if (i < k) acc[i] += Z[l * m + selk[i]] * v;
      }
      const TI cont = V[(int64_t)nT * N + e];
#pragma unroll
      for (int i = 0; i < kLanczosKeep; ++i)
        if (i < k) V[(int64_t)i * N + e] = (TI)acc[i];
      V[(int64_t)k * N + e] = cont;
    }
    if (tid < k) {
      th[tid] = H[selk[tid] * m + selk[tid]];
      bb[tid] = blast * Z[(nT - 1) * m + selk[tid]];
    }
    gsync<G>();
    kk = k;
  }
  out.theta = s_theta;
  out.res = s_res;
  if (!s_conv) out.status = ST_OK;  // not converged within the restart budget: reported through res
  return out;
}

// ---------------------------------------------------------------------------
// CTA Lanczos for the generalised symmetric-definite local problem
// A x = lambda B x (evp.py:418-439 with micro_op_gevp): Lanczos on B^{-1} A,
// which is self-adjoint in the B inner product, with B-orthonormal basis V
// (and its images BV = B V kept beside it), two B-orthogonalisation passes,
// and each B^{-1} applied by an FP64 GMRES solve with the mass operator's
// local operator (stacks LB, RB).  The tridiagonal matrix and the selection
// rules are those of cta_lanczos.  The returned vector is normalised as the
// reference's local solver returns it: x^T B x = 1 for 'eigh' (mode 0,
// scipy.linalg.eigh with b), |x| = 1 otherwise (scipy.linalg.eig with b).
// ---------------------------------------------------------------------------

template <bool TC, bool G = TC>
__device__ __noinline__ CtaEigStats cta_glanczos(const Contraction& p1, const Contraction& p2, const Contraction& p3,
                                                const Contraction& q1, const Contraction& q2, const Contraction& q3,
                                                const double* L, const double* A, const double* R,
                                                const double* LB, const double* B, const double* RB, double* T1,
                                                double* T2, double* x, double* V, double* BV, double* w, double* y,
                                                double* gV, double* gr, double* gw, int64_t N, int m, int mg,
                                                int mode, double sigma, int max_restarts, double tol, double* sm,
                                                double* smg, const OzScratch* oz, int64_t* inner_its) {
  double* al = sm;
  double* be = al + m;
  double* h1 = be + m;
  double* h2 = h1 + m + 2;
  double* z = h2 + m + 2;
  double* twk = z + m;
  int* piv = (int*)(twk + 5 * m + 8);
  __shared__ double s_theta_g[kGroups<G>], s_res_g[kGroups<G>];
  __shared__ int s_conv_g[kGroups<G>];
  double& s_theta = s_theta_g[gidx<G>()];
  double& s_res = s_res_g[gidx<G>()];
  int& s_conv = s_conv_g[gidx<G>()];
  const int tid = gtid<G>(), nt = gsize<G>(), lane = tid & 31, warp = tid >> 5;
  CtaEigStats out{0.0, 0.0, 0, 0, ST_OK};
  auto applyA = [&](const double* src, double* dst) {
    cta_contract_f64<TC, G>(p1, L, src, T1, oz);
    cta_contract_f64<TC, G>(p2, T1, A, T2, oz);
    cta_contract_f64<TC, G>(p3, T2, R, dst, oz);
  };
  auto applyB = [&](const double* src, double* dst) {
    cta_contract_f64<TC, G>(q1, LB, src, T1, oz);
    cta_contract_f64<TC, G>(q2, T1, B, T2, oz);
    cta_contract_f64<TC, G>(q3, T2, RB, dst, oz);
  };
  // B-normalise v (its image Bv computed into bv); false if v^T B v is not positive
  auto bnormalise = [&](double* v, double* bv) {
    applyB(v, bv);
    double sb = 0.0;
    for (int64_t e = tid; e < N; e += nt) sb += v[e] * bv[e];
    const double nb2 = cta_sum<G>(sb);
    if (!(nb2 > 0.0) || !isfinite(nb2)) return false;
    const double inv = 1.0 / sqrt(nb2);
    for (int64_t e = tid; e < N; e += nt) {
      v[e] *= inv;
      bv[e] *= inv;
    }
    gsync<G>();
    return true;
  };
  if (tid == 0) {
    s_conv = 0;
    s_theta = 0.0;
    s_res = 0.0;
  }
  for (int64_t e = tid; e < N; e += nt) V[e] = x[e];
  gsync<G>();
  if (!bnormalise(V, BV)) {
    for (int64_t e = tid; e < N; e += nt) V[e] = 1.0;
    gsync<G>();
    if (!bnormalise(V, BV)) {
      out.status = ST_SINGULAR;  // the mass operator is not positive definite
      return out;
    }
  }
  const int mm = (int)(N < m ? N : m);
  for (;;) {
    int nT = 0;
    for (int j = 0; j < mm; ++j) {
      applyA(V + (int64_t)j * N, w);
      // y = B^{-1} w (zero start), FP64 to 1e-13
      for (int64_t e = tid; e < N; e += nt) y[e] = 0.0;
      gsync<G>();
      long long c0 = 0, c1 = 0, c2 = 0;
      const CtaSolveStats gs = cta_gmres_ir<double, TC, G>(q1, q2, q3, LB, B, RB, T1, T2, LB, B, RB, T1, T2, w, y, gr, gV,
                                                       gw, N, (int)(N < mg ? N : mg), 60, 1e-13, 0.0, smg, nullptr,
                                                       &c0, &c1, &c2);
      *inner_its += gs.inner;
      if (gs.status != ST_OK) {
        out.status = gs.status;
        return out;
      }
      // two B-orthogonalisation passes: <v_q, y>_B = (B v_q)^T y
      cta_dots<double, G>(BV, N, j + 1, y, h1);
      for (int64_t e = tid; e < N; e += nt) {
        double acc = y[e];
        for (int q = 0; q <= j; ++q) acc -= h1[q] * V[(int64_t)q * N + e];
        y[e] = acc;
      }
      gsync<G>();
      cta_dots<double, G>(BV, N, j + 1, y, h2);
      for (int64_t e = tid; e < N; e += nt) {
        double acc = y[e];
        for (int q = 0; q <= j; ++q) acc -= h2[q] * V[(int64_t)q * N + e];
        y[e] = acc;
      }
      gsync<G>();
      applyB(y, gw);  // B y
      double sb = 0.0;
      for (int64_t e = tid; e < N; e += nt) sb += y[e] * gw[e];
      const double bj = sqrt(fmax(cta_sum<G>(sb), 0.0));
      if (tid == 0) {
        al[j] = h1[j] + h2[j];
        be[j] = bj;
      }
      if (bj > 0.0 && j + 1 < mm) {
        double* vn = V + (int64_t)(j + 1) * N;
        double* bvn = BV + (int64_t)(j + 1) * N;
        const double inv = 1.0 / bj;
        for (int64_t e = tid; e < N; e += nt) {
          vn[e] = y[e] * inv;
          bvn[e] = gw[e] * inv;
        }
      }
      gsync<G>();
      ++out.its;
      nT = j + 1;
      double tnorm = 0.0;
      for (int i = 0; i < nT; ++i)
        tnorm = fmax(tnorm, fabs(al[i]) + fabs(be[i]) + (i > 0 ? fabs(be[i - 1]) : 0.0));
      const bool breakdown = !(bj > 1e-14 * fmax(tnorm, 1e-300));
      if ((nT % 4) == 0 || nT == mm || breakdown) {
        if (warp == 0) {
          double lo = 1e300, hi = -1e300;
          for (int i = 0; i < nT; ++i) {
            const double rad = (i > 0 ? fabs(be[i - 1]) : 0.0) + (i < nT - 1 ? fabs(be[i]) : 0.0);
            lo = fmin(lo, al[i] - rad);
            hi = fmax(hi, al[i] + rad);
          }
          const double pivmin = 1e-300 + DBL_MIN * fmax(1.0, tnorm * tnorm);
          lo -= 1e-12 * fmax(1.0, tnorm);
          hi += 1e-12 * fmax(1.0, tnorm);
          int sel;
          if (mode == 0) {
            sel = nT - 1;
          } else if (mode == 2) {
            sel = 0;
          } else {
            const int below = sturm_count(al, be, nT, sigma, pivmin);
            const double vdn = below > 0 ? tri_eigval(al, be, nT, below - 1, lo, hi, pivmin) : 0.0;
            const double vup = below < nT ? tri_eigval(al, be, nT, below, lo, hi, pivmin) : 0.0;
            sel = (below > 0 && (below >= nT || fabs(vdn - sigma) <= fabs(vup - sigma))) ? below - 1 : below;
          }
          const double th = tri_eigval(al, be, nT, sel, lo, hi, pivmin);
          if (lane == 0) {
            tri_eigvec(al, be, nT, th, fmax(tnorm, 1e-300), z, twk, piv);
            s_theta = th;
            s_res = bj * fabs(z[nT - 1]) / fmax(tnorm, 1e-300);
            s_conv = (s_res <= tol) || breakdown;
          }
        }
        gsync<G>();
        if (s_conv || nT == mm) break;
      } else if (breakdown) {
        break;
      }
    }
    // Ritz vector x = V z and its image B x = BV z (into w)
    for (int64_t e = tid; e < N; e += nt) {
      double acc = 0.0, bacc = 0.0;
      for (int l = 0; l < nT; ++l) {
        acc += z[l] * V[(int64_t)l * N + e];
        bacc += z[l] * BV[(int64_t)l * N + e];
      }
      x[e] = acc;
      w[e] = bacc;
    }
    gsync<G>();
    if (s_conv || out.restarts >= max_restarts) break;
    ++out.restarts;
    for (int64_t e = tid; e < N; e += nt) V[e] = x[e];
    gsync<G>();
    if (!bnormalise(V, BV)) {
      out.status = ST_SINGULAR;
      return out;
    }
  }
  // the reference's normalisation of the local eigenvector
  double s2 = 0.0;
  for (int64_t e = tid; e < N; e += nt) s2 += mode == 0 ? x[e] * w[e] : x[e] * x[e];
  const double nrm2 = cta_sum<G>(s2);
  if (nrm2 > 0.0 && isfinite(nrm2)) {
    const double inv = 1.0 / sqrt(nrm2);
    for (int64_t e = tid; e < N; e += nt) x[e] *= inv;
  }
  gsync<G>();
  out.theta = s_theta;
  out.res = s_res;
  return out;
}

// QR of a core; with a shared-memory region (the group's tensor-core tiles,
// idle between GEMMs) large enough for the matrix, in shared memory.
template <bool G = false, bool SH = G>
__device__ __noinline__ void cta_qr(const QrArgs& q, unsigned char* shm = nullptr, int64_t shm_doubles = 0) {
  if constexpr (SH) {  // only the tensor-core kernels have such a region
    const int64_t k = q.rows < q.cols ? q.rows : q.cols;
    if (shm && q.rows * q.cols <= shm_doubles && k <= kQrSharedMaxK) {
      cta_householder_qr_shared<G>(q, reinterpret_cast<double*>(shm));
      return;
    }
  }
  cta_householder_qr<G>(q);
}

// Make this request's outputs visible to the host and to copy engines, then
// raise its completion flag (host-mapped memory).
template <bool G = false>
__device__ __forceinline__ void signal_done(int* flag) {
  gsync<G>();
  if (gtid<G>() == 0 && flag) {
    __threadfence_system();
    asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(flag), "r"(1) : "memory");
  }
  gsync<G>();
}

// ---------------------------------------------------------------------------
// one instance
// ---------------------------------------------------------------------------

__host__ __device__ size_t batch_smem_scalar_bytes(int m, int m_evp, int gevp);
__host__ __device__ inline size_t batch_lanczos_doubles(int m_evp) {
  return (size_t)10 * m_evp + 12 + m_evp / 2 + 1;  // Lanczos arrays + pivots
}

struct Scratch {
  double *T1, *T2, *U, *f, *r, *w, *V, *rbuf, *qwork, *tmp0, *tmp1;
  float *Vf, *wf, *T1f, *T2f, *Lf, *Rf, *Af;
  // generalised eigenproblems: B-images of the Lanczos basis, the inner
  // GMRES basis and vectors (sized only when the batch holds such a request)
  double *BV, *gV, *gy, *gr, *gw;
  OzScratch oz;
};

__device__ Scratch scratch_of(const BatchArgs& a, int slot) {
  char* base = a.scratch + (int64_t)slot * a.scratch_stride;
  const BatchSizes& z = a.sizes;
  Scratch s;
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    char* p = base + off;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  s.T1 = (double*)take(8 * z.T);
  s.T2 = (double*)take(8 * z.T);
  s.U = (double*)take(8 * z.U);
  s.f = (double*)take(8 * z.N);
  s.r = (double*)take(8 * z.N);
  s.w = (double*)take(8 * z.N);
  const int mv = a.m > a.m_evp ? a.m : a.m_evp;
  s.V = (double*)take(8 * (int64_t)(mv + 1) * z.N);
  s.rbuf = (double*)take(8 * z.R);
  s.qwork = (double*)take(8 * z.Q);
  s.tmp0 = (double*)take(8 * z.core);
  s.tmp1 = (double*)take(8 * z.core);
  s.Vf = (float*)take(4 * (int64_t)(mv + 1) * z.N);
  s.wf = (float*)take(4 * z.N);
  s.T1f = (float*)take(4 * z.T);
  s.T2f = (float*)take(4 * z.T);
  s.Lf = (float*)take(4 * z.stack);
  s.Rf = (float*)take(4 * z.stack);
  s.Af = (float*)take(4 * z.opcore);
  s.BV = (double*)take(8 * (int64_t)(a.m_evp + 1) * z.Ng);
  s.gV = (double*)take(8 * (int64_t)(a.m + 1) * z.Ng);
  s.gy = (double*)take(8 * z.Ng);
  s.gr = (double*)take(8 * z.Ng);
  s.gw = (double*)take(8 * z.Ng);
  s.oz.as = (uint16_t*)take(2 * z.oz_a);
  s.oz.bs = (uint16_t*)take(2 * z.oz_b);
  s.oz.rexp = (int*)take(4 * z.oz_r);
  s.oz.cexp = (int*)take(4 * z.oz_c);
  s.oz.ktab = nullptr;  // set by the kernel: a shared-memory table
  s.oz.cap_a = z.oz_a;
  s.oz.cap_b = z.oz_b;
  s.oz.cap_r = z.oz_r;
  s.oz.cap_c = z.oz_c;
  return s;
}

template <bool TC, bool G = TC>
__device__ __noinline__ void batch_solve(const BatchArgs& a, int j, const Scratch& S, double* sm) {
  const BatchInst& I = a.inst[j];
  const int d = I.d;
  const int64_t* M = a.meta + I.meta_off;
  const int64_t* n = M;
  const int64_t* R = n + d;
  const int64_t* rb = R + d + 1;
  const int64_t* rx0 = rb + d + 1;
  const int64_t* cap = rx0 + d + 1;
  const int64_t* op_off = cap + d + 1;
  const int64_t* rhs_off = op_off + d;
  const int64_t* x0_off = rhs_off + d;
  const int64_t* X_off = x0_off + d;
  const int64_t* L_off = X_off + d;
  const int64_t* Rt_off = L_off + d;
  const int64_t* Lb_off = Rt_off + d;
  const int64_t* Rb_off = Lb_off + d;
  __shared__ int64_t r_g[kGroups<G>][kMaxOrderB + 1];
  int64_t* r = r_g[gidx<G>()];
  const int tid = gtid<G>();
  for (int i = tid; i <= d; i += gsize<G>()) r[i] = cap[i];
  gsync<G>();
  // the group's tensor-core tiles hold the QR factorisations between GEMMs;
  // in mixed precision the gauge pushes run as emulated FP64 on tcgen05 (on
  // the warp-MMA kernel they stay native)
  unsigned char* qsh = S.oz.tc ? S.oz.tc->tiles : nullptr;
  constexpr int64_t qcap = TcCfg<G>::kSmemBytes / 8;
  const OzScratch* ozp = (TC && a.prec == 1) ? &S.oz : nullptr;
  auto X = [&](int i) { return I.X + X_off[i]; };
  auto L = [&](int i) { return I.L + L_off[i]; };
  auto Rt = [&](int i) { return I.Rt + Rt_off[i]; };
  auto Lb = [&](int i) { return I.Lb + Lb_off[i]; };
  auto Rb = [&](int i) { return I.Rb + Rb_off[i]; };
  auto A = [&](int i) { return I.op + op_off[i]; };
  auto B = [&](int i) { return I.rhs + rhs_off[i]; };

  double maxres = 0.0, fl64 = 0.0, fl32 = 0.0;
  int64_t nsolve = 0, nits = 0, ncyc = 0;
  int status = ST_OK;
  // tensor-core counters of the CTA when this request started (thread 0 keeps them)
  long long inner_apply = 0;  // cycles of the inner solves spent in local-operator applications
  const unsigned long long tc0 = S.oz.tc ? S.oz.tc->gemms : 0ull, fb0 = S.oz.tc ? S.oz.tc->fallbacks : 0ull;
  long long ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long long t_start = clock64();
  long long tp = t_start;
  auto lap = [&](int k) {
    const long long now = clock64();
    ph[k] += now - tp;
    tp = now;
  };
  // algorithmic flops of one local-operator application / stack update
  auto apply_fl = [&](double aa, double nn, double ss, double r0, double r1) {
    return 2 * aa * aa * r0 * nn * ss + 2 * aa * ss * nn * nn * r0 * r1 + 2 * aa * nn * ss * ss * r1;
  };
  auto qr_fl = [&](double rows, double cols) {
    const double k = rows < cols ? rows : cols;
    return 2 * rows * cols * cols + 2 * rows * k * k;
  };

  // right-orthonormalise the guess (Householder RQ, R normalised and pushed left)
  {
    const double* cur = I.x0 + x0_off[d - 1];
    int64_t cur_left = rx0[d - 1], cur_right = 1;
    for (int i = d - 1; i >= 1; --i) {
      const int64_t ns = n[i] * cur_right, k = cur_left < ns ? cur_left : ns;
      QrArgs q{cur, 1, ns, X(i), 1, ns, S.rbuf, 1, k, ns, cur_left, 1, nullptr, S.qwork};
      cta_qr<G, TC>(q, qsh, qcap);
      const int64_t p = rx0[i - 1] * n[i - 1];
      double* outb = (i & 1) ? S.tmp1 : S.tmp0;
      cta_contract_f64<TC, G>(desc_push_right(p, cur_left, k), I.x0 + x0_off[i - 1], S.rbuf, outb, ozp);
      cur = outb;
      cur_left = rx0[i - 1];
      cur_right = k;
    }
    cta_copy<G>(X(0), cur, n[0] * cur_right);
  }
  lap(0);

  auto right = [&](int i) {
    if (i == d - 1) {
      if (tid == 0) {
        Rt(i)[0] = 1.0;
        Rb(i)[0] = 1.0;
      }
      gsync<G>();
      return;
    }
    const int64_t aa = r[i + 1], nn = n[i + 1], ss = r[i + 2];
    Contraction q1, q2, q3;
    desc_right(aa, nn, ss, R[i + 1], R[i + 2], &q1, &q2, &q3);
    const OzScratch* oz = a.prec == 1 ? &S.oz : nullptr;
    cta_contract_f64<TC, G>(q1, (const double*)Rt(i + 1), (const double*)X(i + 1), S.T1, oz);
    cta_contract_f64<TC, G>(q2, (const double*)S.T1, A(i + 1), S.T2, oz);
    cta_contract_f64<TC, G>(q3, (const double*)X(i + 1), (const double*)S.T2, Rt(i), oz);
    fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)R[i + 1], (double)R[i + 2]);
    cta_contract<double, G>(desc_vec_u_right(aa, nn, ss, rb[i + 2]), (const double*)X(i + 1), (const double*)Rb(i + 1), S.U);
    cta_contract<double, G>(desc_vec_right(aa, nn, rb[i + 1], rb[i + 2]), B(i + 1), (const double*)S.U, Rb(i));
    lap(1);
  };
  auto left = [&](int i) {
    if (i == 0) {
      if (tid == 0) {
        L(i)[0] = 1.0;
        Lb(i)[0] = 1.0;
      }
      gsync<G>();
      return;
    }
    const int64_t aa = r[i - 1], nn = n[i - 1], ss = r[i];
    Contraction p1, p2, p3;
    desc_apply(aa, nn, ss, R[i - 1], R[i], &p1, &p2, &p3);
    const OzScratch* oz = a.prec == 1 ? &S.oz : nullptr;
    cta_contract_f64<TC, G>(p1, (const double*)L(i - 1), (const double*)X(i - 1), S.T1, oz);
    cta_contract_f64<TC, G>(p2, (const double*)S.T1, A(i - 1), S.T2, oz);
    cta_contract_f64<TC, G>(desc_left_p3(aa, nn, ss, R[i]), (const double*)S.T2, (const double*)X(i - 1), L(i), oz);
    fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)R[i - 1], (double)R[i]);
    cta_contract<double, G>(desc_vec_u_left(aa, nn, rb[i - 1], rb[i]), (const double*)Lb(i - 1), B(i - 1), S.U);
    cta_contract<double, G>(desc_vec_left(aa, nn, ss, rb[i]), (const double*)S.U, (const double*)X(i - 1), Lb(i));
    lap(1);
  };
  auto solve = [&](int i) {
    const int64_t aa = r[i], nn = n[i], ss = r[i + 1], N = aa * nn * ss;
    cta_contract<double, G>(desc_vec_u_left(aa, nn, rb[i], rb[i + 1]), (const double*)Lb(i), B(i), S.U);
    cta_contract<double, G>(desc_micro_f(aa, nn, ss, rb[i + 1]), (const double*)S.U, (const double*)Rb(i), S.f);
    Contraction p1, p2, p3;
    desc_apply(aa, nn, ss, R[i], R[i + 1], &p1, &p2, &p3);
    const int m = (int)(N < a.m ? N : a.m);
    CtaSolveStats st;
    lap(2);
    long long cr = 0, ci = 0, capp = 0;
    if (a.prec == 1) {
      cta_to_float<G>(S.Lf, L(i), aa * R[i] * aa);
      cta_to_float<G>(S.Rf, Rt(i), ss * R[i + 1] * ss);
      cta_to_float<G>(S.Af, A(i), R[i] * nn * nn * R[i + 1]);
      st = cta_gmres_ir<float, TC, G>(p1, p2, p3, L(i), A(i), Rt(i), S.T1, S.T2, S.Lf, S.Af, S.Rf, S.T1f, S.T2f, S.f, X(i),
                               S.r, S.Vf, S.wf, N, m, 30, a.tol, 1e-5, sm, &S.oz, &cr, &ci, &capp);
    } else {
      st = cta_gmres_ir<double, TC, G>(p1, p2, p3, L(i), A(i), Rt(i), S.T1, S.T2, L(i), A(i), Rt(i), S.T1, S.T2, S.f, X(i),
                                S.r, S.V, S.w, N, m, 60, a.tol, 0.0, sm, nullptr, &cr, &ci, &capp);
    }
    ph[3] += cr;
    ph[4] += ci;
    inner_apply += capp;
    tp = clock64();
    ++nsolve;
    nits += st.inner;
    ncyc += st.cycles;
    {
      const double fa = apply_fl((double)aa, (double)nn, (double)ss, (double)R[i], (double)R[i + 1]) + 2.0 * N;
      const double per = st.cycles > 0 ? (double)st.inner / st.cycles : (double)st.inner;
      const double inner = st.inner * fa + st.cycles * 8.0 * (double)N * per * (per + 1) / 2.0;
      fl64 += st.cycles * fa;
      if (a.prec == 1)
        fl32 += inner;
      else
        fl64 += inner;
    }
    maxres = fmax(maxres, st.rel);
    if (st.status != ST_OK && status == ST_OK) status = st.status;
  };

  for (int i = d - 1; i >= 0; --i) right(i);
  for (int sweep = 0; sweep < I.repeats && status == ST_OK; ++sweep) {
    for (int i = 0; i < d; ++i) {
      left(i);
      if (i < d - 1) {
        solve(i);
        const int64_t aa = r[i], nn = n[i], ss = r[i + 1], k = aa * nn < ss ? aa * nn : ss;
        QrArgs q{X(i), ss, 1, X(i), k, 1, S.rbuf, ss, 1, aa * nn, ss, 0, nullptr, S.qwork};
        cta_qr<G, TC>(q, qsh, qcap);
        fl64 += qr_fl((double)(aa * nn), (double)ss);
        const int64_t qq = n[i + 1] * r[i + 2];
        cta_contract_f64<TC, G>(desc_push_left(k, ss, qq), (const double*)S.rbuf, (const double*)X(i + 1), S.tmp0, ozp);
        cta_copy<G>(X(i + 1), S.tmp0, k * qq);
        if (tid == 0) r[i + 1] = k;
        gsync<G>();
        lap(5);
      }
    }
    for (int i = d - 1; i >= 0; --i) {
      right(i);
      solve(i);
      if (i > 0) {
        const int64_t aa = r[i], nn = n[i], ss = r[i + 1], ns = nn * ss, k = aa < ns ? aa : ns;
        QrArgs q{X(i), 1, ns, X(i), 1, ns, S.rbuf, 1, k, ns, aa, 0, nullptr, S.qwork};
        cta_qr<G, TC>(q, qsh, qcap);
        fl64 += qr_fl((double)ns, (double)aa);
        const int64_t p = r[i - 1] * n[i - 1];
        cta_contract_f64<TC, G>(desc_push_right(p, aa, k), (const double*)X(i - 1), (const double*)S.rbuf, S.tmp0, ozp);
        cta_copy<G>(X(i - 1), S.tmp0, p * k);
        if (tid == 0) r[i] = k;
        gsync<G>();
        lap(5);
      }
    }
  }
  // pack the final cores contiguously
  int64_t off = 0;
  for (int i = 0; i < d; ++i) {
    const int64_t cnt = r[i] * n[i] * r[i + 1];
    for (int64_t e = tid; e < cnt; e += gsize<G>()) I.out[off + e] = X(i)[e];
    off += cnt;
  }
  if (tid == 0) {
    I.report[0] = maxres;
    I.report[1] = (double)nsolve;
    I.report[2] = (double)nits;
    I.report[3] = (double)ncyc;
    I.report[4] = (double)status;
    I.report[5] = fl64;
    I.report[6] = fl32;
    I.report[7] = 0.0;
    for (int i = 0; i <= d; ++i) I.report[8 + i] = (double)r[i];
    I.report[9 + d] = (double)I.repeats;
    ph[7] = clock64() - t_start;
    for (int k = 0; k < 8; ++k) I.report[10 + d + k] = (double)ph[k];
    I.report[18 + d] = S.oz.tc ? (double)(S.oz.tc->gemms - tc0) : 0.0;
    I.report[19 + d] = S.oz.tc ? (double)(S.oz.tc->fallbacks - fb0) : 0.0;
    I.report[20 + d] = (double)inner_apply;
  }
  signal_done<G>(I.done);
}

// ---------------------------------------------------------------------------
// one eigenproblem instance (evp.py:17-179, symmetric, number_ev == 1)
// ---------------------------------------------------------------------------

template <bool TC = false, bool G = TC>
__device__ __noinline__ void batch_evp(const BatchArgs& a, int j, const Scratch& S, double* sm) {
  const BatchInst& I = a.inst[j];
  const int d = I.d;
  const int64_t* M = a.meta + I.meta_off;
  const int64_t* n = M;
  const int64_t* R = n + d;
  const int64_t* rb = R + d + 1;  // generalised problems: ranks of operator_gevp
  const int64_t* rx0 = rb + d + 1;
  const int64_t* cap = rx0 + d + 1;
  const int64_t* op_off = cap + d + 1;
  const int64_t* rhs_off = op_off + d;  // ... its cores
  const int64_t* x0_off = op_off + 2 * d;
  const int64_t* X_off = x0_off + d;
  const int64_t* L_off = X_off + d;
  const int64_t* Rt_off = L_off + d;
  const int64_t* Lb_off = Rt_off + d;   // ... and its stacks
  const int64_t* Rb_off = Lb_off + d;
  const bool gevp = I.kind == 2;
  __shared__ int64_t r_g[kGroups<G>][kMaxOrderB + 1];
  __shared__ int64_t ropt_g[kGroups<G>][kMaxOrderB + 1];
  int64_t* r = r_g[gidx<G>()];
  int64_t* ropt = ropt_g[gidx<G>()];
  const int tid = gtid<G>();
  for (int i = tid; i <= d; i += gsize<G>()) r[i] = cap[i];
  gsync<G>();
  auto X = [&](int i) { return I.X + X_off[i]; };
  auto Xo = [&](int i) { return I.Xopt + X_off[i]; };
  const OzScratch* oz = a.prec == 1 ? &S.oz : nullptr;
  unsigned char* qsh = S.oz.tc ? S.oz.tc->tiles : nullptr;
  constexpr int64_t qcap = TcCfg<G>::kSmemBytes / 8;
  auto L = [&](int i) { return I.L + L_off[i]; };
  auto Rt = [&](int i) { return I.Rt + Rt_off[i]; };
  auto A = [&](int i) { return I.op + op_off[i]; };
  auto Bg = [&](int i) { return I.rhs + rhs_off[i]; };
  auto LB = [&](int i) { return I.Lb + Lb_off[i]; };
  auto RB = [&](int i) { return I.Rb + Rb_off[i]; };
  int64_t ginner = 0;  // inner mass-operator GMRES iterations
  double fl64 = 0.0, fl32 = 0.0, maxres = 0.0, theta = 0.0;
  int64_t nsolve = 0, nits = 0, nrst = 0;
  int evp_status = ST_OK;
  auto apply_fl = [&](double aa, double nn, double ss, double r0, double r1) {
    return 2 * aa * aa * r0 * nn * ss + 2 * aa * ss * nn * nn * r0 * r1 + 2 * aa * nn * ss * ss * r1;
  };
  {
    const double* cur = I.x0 + x0_off[d - 1];
    int64_t cur_left = rx0[d - 1], cur_right = 1;
    for (int i = d - 1; i >= 1; --i) {
      const int64_t ns = n[i] * cur_right, k = cur_left < ns ? cur_left : ns;
      QrArgs q{cur, 1, ns, X(i), 1, ns, S.rbuf, 1, k, ns, cur_left, 1, nullptr, S.qwork};
      cta_qr<G, TC>(q, qsh, qcap);
      const int64_t p = rx0[i - 1] * n[i - 1];
      double* outb = (i & 1) ? S.tmp1 : S.tmp0;
      cta_contract<double, G>(desc_push_right(p, cur_left, k), I.x0 + x0_off[i - 1], S.rbuf, outb);
      cur = outb;
      cur_left = rx0[i - 1];
      cur_right = k;
    }
    cta_copy<G>(X(0), cur, n[0] * cur_right);
  }
  auto right = [&](int i) {
    if (i == d - 1) {
      if (tid == 0) {
        Rt(i)[0] = 1.0;
        if (gevp) RB(i)[0] = 1.0;
      }
      gsync<G>();
      return;
    }
    const int64_t aa = r[i + 1], nn = n[i + 1], ss = r[i + 2];
    Contraction q1, q2, q3;
    desc_right(aa, nn, ss, R[i + 1], R[i + 2], &q1, &q2, &q3);
    cta_contract_f64<TC, G>(q1, (const double*)Rt(i + 1), (const double*)X(i + 1), S.T1, oz);
    cta_contract_f64<TC, G>(q2, (const double*)S.T1, A(i + 1), S.T2, oz);
    cta_contract_f64<TC, G>(q3, (const double*)X(i + 1), (const double*)S.T2, Rt(i), oz);
    fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)R[i + 1], (double)R[i + 2]);
    if (gevp) {  // evp.py:314-329
      desc_right(aa, nn, ss, rb[i + 1], rb[i + 2], &q1, &q2, &q3);
      cta_contract_f64<TC, G>(q1, (const double*)RB(i + 1), (const double*)X(i + 1), S.T1, oz);
      cta_contract_f64<TC, G>(q2, (const double*)S.T1, Bg(i + 1), S.T2, oz);
      cta_contract_f64<TC, G>(q3, (const double*)X(i + 1), (const double*)S.T2, RB(i), oz);
      fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)rb[i + 1], (double)rb[i + 2]);
    }
  };
  auto left = [&](int i) {
    if (i == 0) {
      if (tid == 0) {
        L(i)[0] = 1.0;
        if (gevp) LB(i)[0] = 1.0;
      }
      gsync<G>();
      return;
    }
    const int64_t aa = r[i - 1], nn = n[i - 1], ss = r[i];
    Contraction p1, p2, p3;
    desc_apply(aa, nn, ss, R[i - 1], R[i], &p1, &p2, &p3);
    cta_contract_f64<TC, G>(p1, (const double*)L(i - 1), (const double*)X(i - 1), S.T1, oz);
    cta_contract_f64<TC, G>(p2, (const double*)S.T1, A(i - 1), S.T2, oz);
    cta_contract_f64<TC, G>(desc_left_p3(aa, nn, ss, R[i]), (const double*)S.T2, (const double*)X(i - 1), L(i), oz);
    fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)R[i - 1], (double)R[i]);
    if (gevp) {  // evp.py:272-287
      desc_apply(aa, nn, ss, rb[i - 1], rb[i], &p1, &p2, &p3);
      cta_contract_f64<TC, G>(p1, (const double*)LB(i - 1), (const double*)X(i - 1), S.T1, oz);
      cta_contract_f64<TC, G>(p2, (const double*)S.T1, Bg(i - 1), S.T2, oz);
      cta_contract_f64<TC, G>(desc_left_p3(aa, nn, ss, rb[i]), (const double*)S.T2, (const double*)X(i - 1), LB(i), oz);
      fl64 += apply_fl((double)aa, (double)nn, (double)ss, (double)rb[i - 1], (double)rb[i]);
    }
  };
  auto solve = [&](int i) {
    const int64_t aa = r[i], nn = n[i], ss = r[i + 1], N = aa * nn * ss;
    Contraction p1, p2, p3;
    desc_apply(aa, nn, ss, R[i], R[i + 1], &p1, &p2, &p3);
    const int m = (int)(N < a.m_evp ? N : a.m_evp);
    const double fa = apply_fl((double)aa, (double)nn, (double)ss, (double)R[i], (double)R[i + 1]);
    // Eigen solves stay FP64-accurate in both precision modes: warm-started
    // from the previous sweep's core, FP64 Lanczos converges in ~12 steps per
    // site, and an FP32 Lanczos pre-stage (then FP64 polish) measured 2.8x
    // slower.  In mixed precision their products (and the stacks) run as
    // emulated FP64 on the tensor cores.
    CtaEigStats st;
    if (gevp) {
      Contraction g1, g2, g3;
      desc_apply(aa, nn, ss, rb[i], rb[i + 1], &g1, &g2, &g3);
      st = cta_glanczos<TC, G>(p1, p2, p3, g1, g2, g3, L(i), A(i), Rt(i), LB(i), Bg(i), RB(i), S.T1, S.T2, X(i), S.V,
                           S.BV, S.w, S.gy, S.gV, S.gr, S.gw, N, m, a.m, I.mode, I.sigma, kBatchEvpRestarts,
                           a.tol_evp, sm, sm + batch_lanczos_doubles(a.m_evp), oz, &ginner);
      if (st.status != ST_OK && evp_status == ST_OK) evp_status = st.status;
    } else {
      // thick restarts use the group's idle tile memory (tensor-core kernel) or
      // the QR work area for the projected matrix and its eigenvectors
      st = cta_lanczos<double, TC, G>(p1, p2, p3, L(i), A(i), Rt(i), S.T1, S.T2, X(i), S.V, S.w, N, m, I.mode, I.sigma,
                                  kBatchEvpRestarts, a.tol_evp, sm, oz, qsh ? (double*)qsh : S.qwork);
    }
    theta = st.theta;
    nits += st.its;
    nrst += st.restarts;
    maxres = fmax(maxres, st.res);
    fl64 += st.its * (fa + 8.0 * (double)N * (m + 1) / 2.0);
    ++nsolve;
  };
  for (int i = d - 1; i >= 0; --i) right(i);
  double hist[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
  int nh = 1;  // the reference starts its history with one row of inf (evp.py:110)
  double val_opt = INFINITY;
  int it = 1;
  bool conv = false, have_opt = false;
  while (it <= I.repeats && !conv && evp_status == ST_OK) {
    for (int i = 0; i < d; ++i) {
      left(i);
      if (i < d - 1) {
        solve(i);
        const int64_t aa = r[i], nn = n[i], ss = r[i + 1], k = aa * nn < ss ? aa * nn : ss;
        QrArgs q{X(i), ss, 1, X(i), k, 1, S.rbuf, ss, 1, aa * nn, ss, 0, nullptr, S.qwork};
        cta_qr<G, TC>(q, qsh, qcap);
        const int64_t qq = n[i + 1] * r[i + 2];
        cta_contract<double, G>(desc_push_left(k, ss, qq), (const double*)S.rbuf, (const double*)X(i + 1), S.tmp0);
        cta_copy<G>(X(i + 1), S.tmp0, k * qq);
        if (tid == 0) r[i + 1] = k;
        gsync<G>();
      }
    }
    for (int i = d - 1; i >= 0; --i) {
      right(i);
      solve(i);
      if (i > 0) {
        const int64_t aa = r[i], nn = n[i], ss = r[i + 1], ns = nn * ss, k = aa < ns ? aa : ns;
        QrArgs q{X(i), 1, ns, X(i), 1, ns, S.rbuf, 1, k, ns, aa, 0, nullptr, S.qwork};
        cta_qr<G, TC>(q, qsh, qcap);
        const int64_t p = r[i - 1] * n[i - 1];
        cta_contract<double, G>(desc_push_right(p, aa, k), (const double*)X(i - 1), (const double*)S.rbuf, S.tmp0);
        cta_copy<G>(X(i - 1), S.tmp0, p * k);
        if (tid == 0) r[i] = k;
        gsync<G>();
      }
    }
    ++it;
    const double lam = theta;
    if (fabs(lam - I.sigma) < fabs(val_opt - I.sigma)) {
      val_opt = lam;
      have_opt = true;
      for (int i = 0; i < d; ++i) cta_copy<G>(Xo(i), X(i), r[i] * n[i] * r[i + 1]);
      for (int i = tid; i <= d; i += gsize<G>()) ropt[i] = r[i];
      gsync<G>();
    }
    double diff = 0.0;
    const int nl = nh < 3 ? nh : 3;
    for (int q = nh - nl; q < nh; ++q) diff = fmax(diff, fabs(hist[q % 4] - lam));
    if (diff < I.conv_eps) conv = true;
    hist[nh % 4] = lam;
    ++nh;
  }
  // pack the best sweep's cores
  int64_t off = 0;
  for (int i = 0; i < d; ++i) {
    const int64_t cnt = have_opt ? ropt[i] * n[i] * ropt[i + 1] : 0;
    for (int64_t e = tid; e < cnt; e += gsize<G>()) I.out[off + e] = Xo(i)[e];
    off += cnt;
  }
  if (tid == 0) {
    I.report[0] = maxres;
    I.report[1] = (double)nsolve;
    I.report[2] = (double)(nits + ginner);
    I.report[3] = (double)nrst;
    I.report[4] = (double)evp_status;
    I.report[5] = fl64;
    I.report[6] = fl32;
    I.report[7] = val_opt;
    for (int i = 0; i <= d; ++i) I.report[8 + i] = have_opt ? (double)ropt[i] : 0.0;
    I.report[9 + d] = (double)(it - 1);
    for (int k = 0; k < 8; ++k) I.report[10 + d + k] = 0.0;
    I.report[18 + d] = 0.0;
    I.report[19 + d] = 0.0;
    I.report[20 + d] = 0.0;
  }
  signal_done<G>(I.done);
}

// Take the CTA's tensor memory (all threads of the CTA): warp 0 allocates the
// SM's 512 columns once, each of the `groups` groups gets `cols` of them and
// its own completion barrier and operand tiles (tiles + g * tile_stride).
__device__ __forceinline__ void tc_begin(TcState* tc, int groups, uint32_t cols, unsigned char* tiles,
                                         size_t tile_stride) {
  __shared__ uint32_t s_tmem;
  if ((threadIdx.x >> 5) == 0) umma::tmem_alloc(&s_tmem, kTcCtaTmemCols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (threadIdx.x < (unsigned)groups) {
    TcState& t = tc[threadIdx.x];
    t.tmem = s_tmem + cols * threadIdx.x;  // column offset in the low half
    t.tiles = tiles + tile_stride * threadIdx.x;
    t.phase = 0;
    t.status = ST_OK;
    t.gemms = 0;
    t.fallbacks = 0;
    umma::mbar_init(&t.bar, 1);
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
}

// Hand the tensor memory back (all threads of the CTA, after every group is
// done).  A completion wait that gave up leaves MMAs possibly in flight: wait
// for them once more (bounded) first.
__device__ __forceinline__ void tc_end(TcState* tc, int groups) {
  if (threadIdx.x < (unsigned)groups && tc[threadIdx.x].status != ST_OK)
    umma::mbar_wait(&tc[threadIdx.x].bar, tc[threadIdx.x].phase);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if ((threadIdx.x >> 5) == 0) umma::tmem_dealloc(tc[0].tmem, kTcCtaTmemCols);
}

__host__ __device__ inline size_t tc_tiles_offset(size_t before) { return (before + 1023) / 1024 * 1024; }

// Dynamic shared memory of one group: GMRES / Lanczos scalars, the
// contraction-offset table, and (tensor-core variants) the operand tiles.
// use_tc: 0 no tensor memory, 1 two solves per CTA, 2 one solve per CTA.
__host__ __device__ size_t batch_group_smem_bytes(int m, int m_evp, int use_tc, int gevp) {
  const size_t base = batch_smem_scalar_bytes(m, m_evp, gevp) + sizeof(int) * 2 * kTcMaxK;
  if (use_tc == 1) return tc_tiles_offset(base) + TcCfg<true>::kSmemBytes;
  if (use_tc == 2) return tc_tiles_offset(base) + TcCfg<false>::kSmemBytes;
  return base;
}

// The persistent loop of both kernel variants.  Each group (the whole CTA, or
// each of the tensor-core kernel's two) takes requests from the work counter
// and solves them with its own scratch slot and shared-memory region.  With
// UseTc the CTA holds all TMEM columns for its whole life (allocated here,
// released on the way out whatever happened); its GEMM-shaped FP32 and
// emulated-FP64 contractions then run on tcgen05.
template <bool UseTc, bool G = UseTc>
__device__ __forceinline__ void batch_kernel_body(const BatchArgs& a) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  constexpr int NG = kGroups<G>;
  __shared__ int s_j[NG];
  __shared__ TcState s_tc[NG];
  const int g = gidx<G>();
  const int gevp = a.sizes.Ng > 0 ? 1 : 0;
  const size_t gbytes = batch_group_smem_bytes(a.m, a.m_evp, UseTc ? (G ? 1 : 2) : 0, gevp);
  unsigned char* mine = smraw + gbytes * g;
  double* sm = reinterpret_cast<double*>(mine);
  Scratch S = scratch_of(a, (int)blockIdx.x * NG + g);
  const size_t scal = batch_smem_scalar_bytes(a.m, a.m_evp, gevp);
  S.oz.ktab = reinterpret_cast<int*>(mine + scal);
  if constexpr (UseTc) {
    tc_begin(s_tc, NG, TcCfg<G>::kTmemCols, smraw + tc_tiles_offset(scal + sizeof(int) * 2 * kTcMaxK), gbytes);
    S.oz.tc = &s_tc[g];
  }
  bool first = true;
  for (;;) {
    if (gtid<G>() == 0) {
      // every group's first request is fixed: requests 0 .. grid-1 (the
      // largest, in the host's order) go to distinct CTAs, the next grid pair
      // with them in reverse order (largest with smallest); later ones come
      // from the work counter
      const int grid = (int)gridDim.x, b = (int)blockIdx.x;
      s_j[g] = first ? ((g & 1) ? (g + 1) * grid - 1 - b : g * grid + b) : NG * grid + atomicAdd(a.next, 1);
    }
    first = false;
    gsync<G>();
    const int j = s_j[g];
    gsync<G>();
    if (j >= a.count) break;
    if (a.inst[j].kind != 0)
      batch_evp<UseTc, G>(a, j, S, sm);
    else
      batch_solve<UseTc, G>(a, j, S, sm);
  }
  if constexpr (UseTc) tc_end(s_tc, NG);
}

// plain FP64 (and mixed without tensor memory): 128 threads, five CTAs per SM
__global__ void __launch_bounds__(kBatchThreads, kBatchMinBlocks) batch_sle_kernel(BatchArgs a) {
  batch_kernel_body<false>(a);
}

// mixed precision on tcgen05: one CTA per SM holding all of its tensor memory,
// two solves side by side (one per 256-thread group)
__global__ void __launch_bounds__(kBatchThreadsTc, kBatchMinBlocksTc) batch_sle_tc_kernel(BatchArgs a) {
  batch_kernel_body<true, true>(a);
}

// the same with one solve on all 512 threads: faster per solve, for batches
// with fewer requests than two per SM
__global__ void __launch_bounds__(kTcCtaThreads, kBatchMinBlocksTc) batch_sle_tc1_kernel(BatchArgs a) {
  batch_kernel_body<true, false>(a);
}

void oz_need_site(BatchSizes& z, int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1) {
  Contraction cs[7];
  desc_apply(a, n, s, R0, R1, &cs[0], &cs[1], &cs[2]);
  cs[3] = desc_left_p3(a, n, s, R1);
  desc_right(a, n, s, R0, R1, &cs[4], &cs[5], &cs[6]);
  for (const Contraction& c : cs) {
    GemmAxes rows, cols;
    if (!gemm_split(c, rows, cols)) continue;
    const int64_t Kp = (c.ktotal + 15) / 16 * 16;
    z.oz_a = std::max<int64_t>(z.oz_a, (int64_t)kOzSlices * rows.total * Kp);
    z.oz_b = std::max<int64_t>(z.oz_b, (int64_t)kOzSlices * cols.total * Kp);
    z.oz_r = std::max<int64_t>(z.oz_r, rows.total);
    z.oz_c = std::max<int64_t>(z.oz_c, cols.total);
  }
}

// Diagnostic: one CTA applies the local operator with emulated FP64 (Ozaki) products.
__global__ void __launch_bounds__(kBatchThreads) apply_f64emu_kernel(Contraction p1, Contraction p2, Contraction p3,
                                                                     const double* L, const double* A,
                                                                     const double* R, const double* y, double* T1,
                                                                     double* T2, double* out, OzScratch oz) {
  cta_contract_f64<false>(p1, L, y, T1, &oz);
  cta_contract_f64<false>(p2, T1, A, T2, &oz);
  cta_contract_f64<false>(p3, T2, R, out, &oz);
}

// The same on tcgen05 (one 256-thread group, the batch kernel's tensor-core GEMMs).
__global__ void __launch_bounds__(kGroupThreads) apply_f64emu_tc_kernel(Contraction p1, Contraction p2,
                                                                          Contraction p3, const double* L,
                                                                          const double* A, const double* R,
                                                                          const double* y, double* T1, double* T2,
                                                                          double* out, OzScratch oz) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ TcState s_tc;
  oz.ktab = reinterpret_cast<int*>(smraw);
  tc_begin(&s_tc, 1, TcCfg<true>::kTmemCols, smraw + tc_tiles_offset(sizeof(int) * 2 * kTcMaxK), 0);
  oz.tc = &s_tc;
  cta_contract_f64<true>(p1, L, y, T1, &oz);
  cta_contract_f64<true>(p2, T1, A, T2, &oz);
  cta_contract_f64<true>(p3, T2, R, out, &oz);
  tc_end(&s_tc, 1);
}

size_t apply_f64emu_scratch_bytes(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1) {
  BatchSizes z{};
  oz_need_site(z, a, n, s, R0, R1);
  return (size_t)(2 * z.oz_a + 2 * z.oz_b + 4 * z.oz_r + 4 * z.oz_c + 4 * 2 * kTcMaxK + 5 * 256);
}

cudaError_t launch_apply_f64emu(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1, const double* L,
                                const double* A, const double* R, const double* y, double* T1, double* T2,
                                double* out, char* ozmem, size_t ozbytes, int use_tc, cudaStream_t st) {
  BatchSizes z{};
  oz_need_site(z, a, n, s, R0, R1);
  auto rnd = [](int64_t b) { return (b + 255) / 256 * 256; };
  OzScratch oz;
  char* p = ozmem;
  oz.as = (uint16_t*)p;
  p += rnd(2 * z.oz_a);
  oz.bs = (uint16_t*)p;
  p += rnd(2 * z.oz_b);
  oz.rexp = (int*)p;
  p += rnd(4 * z.oz_r);
  oz.cexp = (int*)p;
  p += rnd(4 * z.oz_c);
  oz.ktab = (int*)p;
  p += rnd(4 * 2 * kTcMaxK);
  if ((size_t)(p - ozmem) > ozbytes) return cudaErrorInvalidValue;
  oz.cap_a = z.oz_a;
  oz.cap_b = z.oz_b;
  oz.cap_r = z.oz_r;
  oz.cap_c = z.oz_c;
  Contraction p1, p2, p3;
  desc_apply(a, n, s, R0, R1, &p1, &p2, &p3);
  if (use_tc) {
    const size_t smem = tc_tiles_offset(sizeof(int) * 2 * kTcMaxK) + TcCfg<true>::kSmemBytes;
    cudaError_t e = cudaFuncSetAttribute(apply_f64emu_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    apply_f64emu_tc_kernel<<<1, kGroupThreads, smem, st>>>(p1, p2, p3, L, A, R, y, T1, T2, out, oz);
  } else {
    apply_f64emu_kernel<<<1, kBatchThreads, 0, st>>>(p1, p2, p3, L, A, R, y, T1, T2, out, oz);
  }
  ++launch_counter();
  return cudaGetLastError();
}

// Diagnostic: one CTA applies the FP32 local operator (tensor-core path).
__global__ void __launch_bounds__(kBatchThreads) apply_f32_kernel(Contraction p1, Contraction p2, Contraction p3,
                                                                  const float* L, const float* A, const float* R,
                                                                  const float* y, float* T1, float* T2, float* out,
                                                                  int* ktab) {
  cta_apply<float>(p1, p2, p3, L, A, R, y, T1, T2, out, ktab);
}

// The same on tcgen05 (3xTF32, one 256-thread group).
__global__ void __launch_bounds__(kGroupThreads) apply_f32_tc_kernel(Contraction p1, Contraction p2, Contraction p3,
                                                                       const float* L, const float* A, const float* R,
                                                                       const float* y, float* T1, float* T2,
                                                                       float* out) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ TcState s_tc;
  int* ktab = reinterpret_cast<int*>(smraw);
  tc_begin(&s_tc, 1, TcCfg<true>::kTmemCols, smraw + tc_tiles_offset(sizeof(int) * 2 * kTcMaxK), 0);
  cta_apply<float, true>(p1, p2, p3, L, A, R, y, T1, T2, out, ktab, &s_tc);
  tc_end(&s_tc, 1);
}

cudaError_t launch_apply_f32(int64_t a, int64_t n, int64_t s, int64_t R0, int64_t R1, const float* L, const float* A,
                             const float* R, const float* y, float* T1, float* T2, float* out, int* ktab, int use_tc,
                             cudaStream_t st) {
  Contraction p1, p2, p3;
  desc_apply(a, n, s, R0, R1, &p1, &p2, &p3);
  if (use_tc) {
    const size_t smem = tc_tiles_offset(sizeof(int) * 2 * kTcMaxK) + TcCfg<true>::kSmemBytes;
    cudaError_t e = cudaFuncSetAttribute(apply_f32_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    apply_f32_tc_kernel<<<1, kGroupThreads, smem, st>>>(p1, p2, p3, L, A, R, y, T1, T2, out);
  } else {
    apply_f32_kernel<<<1, kBatchThreads, 0, st>>>(p1, p2, p3, L, A, R, y, T1, T2, out, ktab);
  }
  ++launch_counter();
  return cudaGetLastError();
}

// dynamic shared memory: the GMRES / Lanczos scalars, then one contraction-offset
// table shared by the FP32 tensor-core apply and the emulated-FP64 contractions
// (never used at the same time); the rest of the SM's 256 KB stays L1
// (gevp: the Lanczos arrays and, after them, those of the inner GMRES solves
// with the mass operator, both live at once)
__host__ __device__ size_t batch_smem_scalar_bytes(int m, int m_evp, int gevp) {
  const size_t g = (size_t)(m + 1) * m + 2 * m + (m + 1) + m + 2 * (m + 2);
  const size_t e = batch_lanczos_doubles(m_evp);
  return sizeof(double) * (gevp ? g + e : (g > e ? g : e));
}

size_t batch_smem_bytes(int m, int m_evp, int use_tc, int gevp) {
  return batch_group_smem_bytes(m, m_evp, use_tc, gevp) * batch_solves_per_cta(use_tc);
}

int batch_solves_per_cta(int use_tc) { return use_tc == 1 ? kGroups<true> : 1; }

static const void* batch_kernel_fn(int use_tc) {
  if (use_tc == 1) return (const void*)batch_sle_tc_kernel;
  if (use_tc == 2) return (const void*)batch_sle_tc1_kernel;
  return (const void*)batch_sle_kernel;
}

int64_t batch_scratch_stride(const BatchSizes& z, int mg, int m_evp) {
  const int m = mg > m_evp ? mg : m_evp;
  auto r = [](int64_t b) { return (b + 255) / 256 * 256; };
  return r(8 * z.T) * 2 + r(8 * z.U) + r(8 * z.N) * 3 + r(8 * (int64_t)(m + 1) * z.N) + r(8 * z.R) + r(8 * z.Q) +
         r(8 * z.core) * 2 + r(4 * (int64_t)(m + 1) * z.N) + r(4 * z.N) + r(4 * z.T) * 2 + r(4 * z.stack) * 2 +
         r(4 * z.opcore) + r(8 * (int64_t)(m_evp + 1) * z.Ng) + r(8 * (int64_t)(mg + 1) * z.Ng) + r(8 * z.Ng) * 3 +
         r(2 * z.oz_a) + r(2 * z.oz_b) + r(4 * z.oz_r) + r(4 * z.oz_c);
}

int batch_threads(int use_tc) { return use_tc == 1 ? kBatchThreadsTc : (use_tc == 2 ? kTcCtaThreads : kBatchThreads); }

// Resident CTAs per SM of the kernel variant; *err (if given) receives the
// first CUDA error of the query (the result is then 1).
int batch_blocks_per_sm(int m, int m_evp, int use_tc, cudaError_t* err, int gevp) {
  const size_t smem = batch_smem_bytes(m, m_evp, use_tc, gevp);
  const void* fn = batch_kernel_fn(use_tc);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int occ = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, batch_threads(use_tc), smem);
  if (err) *err = e;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  if (occ < 1) occ = 1;
  // a resident tensor-core CTA holds all of the SM's 512 TMEM columns
  if (use_tc && occ > (int)(512 / kTcCtaTmemCols)) occ = (int)(512 / kTcCtaTmemCols);
  return occ;
}

cudaError_t launch_batch_sle(const BatchArgs& a, int grid, cudaStream_t st) {
  const size_t smem = batch_smem_bytes(a.m, a.m_evp, a.use_tc, a.sizes.Ng > 0 ? 1 : 0);
  const void* fn = batch_kernel_fn(a.use_tc);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (a.use_tc == 1)
    batch_sle_tc_kernel<<<grid, kBatchThreadsTc, smem, st>>>(a);
  else if (a.use_tc == 2)
    batch_sle_tc1_kernel<<<grid, kTcCtaThreads, smem, st>>>(a);
  else
    batch_sle_kernel<<<grid, kBatchThreads, smem, st>>>(a);
  ++launch_counter();
  return cudaGetLastError();
}

}  // namespace ttals
