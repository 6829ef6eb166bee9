// Persistent, grid-cooperative Krylov solvers for the ALS local problems.
//
// The local operator M (the micro matrix of scikit_tt/solvers/sle.py:308-347,
// N = r_i n_i r_{i+1}) is never assembled: every Krylov step applies it as the
// three contractions L -> A -> Rt (O(n R r^3) instead of O(N^2) per product).
//
// gmres_ir_kernel<TI>: restarted GMRES with an FP64 outer residual.
//   Each cycle evaluates r = f - M x in FP64, then runs one GMRES(m) cycle in
//   precision TI on M d = r / |r| (classical Gram-Schmidt, applied twice) and
//   updates x += |r| d in FP64.  TI = double is the plain FP64 solver (the
//   cycles are ordinary restarts); TI = float is GMRES-based iterative
//   refinement: FP32 Krylov work, FP64 residual and solution.
//   Replaces np.linalg.solve / lu_factor+lu_solve of sle.py:505-509.
//
// lanczos_kernel: Lanczos with full reorthogonalisation (CGS2) for the
//   symmetric local eigenproblem of scikit_tt/solvers/evp.py:386-443; Ritz
//   values from the tridiagonal matrix by Sturm-count multisection, Ritz
//   vectors by inverse iteration; selection "largest k" (eigh),
//   "closest to sigma" (eig/eigs) or "smallest".  Deflation by previous
//   eigentensors (evp.py:376-381) is applied matrix-free: M += shift t t^T.
//   With nonsym set the same kernel runs Arnoldi: the full Hessenberg
//   projection is kept, Ritz values come from the Francis QR iteration
//   (ttals_hess.cuh) and are ranked by their complex distance to sigma, Ritz
//   vectors by inverse iteration on H - theta I.  A wanted Ritz value with a
//   nonzero imaginary part ends the solve with ST_UNSUPPORTED (the real-valued
//   cores cannot hold a complex eigenvector).
//
// expm_kernel: x <- exp(tau M) x for real tau, the local time step of the
//   TDVP integrators (ode.py:1398-1616).  Two modes: "literal" runs the
//   fixed-dimension recurrence of local_krylov (ode.py:1689-1758) exactly as
//   written there (unnormalised start vector, three-term recurrence without
//   reorthogonalisation, c = exp(tau T) e_1, x = sum_j c_j v_j); the other
//   replaces scipy's expm_multiply: Lanczos with full reorthogonalisation on
//   x / |x|, grown until the a-posteriori error beta_k |e_k^T exp(h T) e_1| is
//   below tol |exp(h T) e_1|, with the step split into substeps h <= tau when
//   the basis cap is reached first.
//
// One CTA per SM, co-resident (cooperative launch).  Vector work uses a fixed
// chunk of elements per CTA; every scalar (dot, norm, Givens rotation, Ritz
// value) is reduced identically in every CTA, so control flow is uniform.
#include <float.h>

#include <algorithm>

#include "ttals_expm.cuh"
#include "ttals_hess.cuh"
#include "ttals_internal.h"
#include "ttals_tri.cuh"

namespace ttals {

constexpr int kKThreads = 512;

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

template <typename TI>
struct GmresK {
  Contraction p1, p2, p3;
  int N;
  const double *L64, *A64, *R64;
  double *T1_64, *T2_64;
  const TI *Li, *Ai, *Ri;
  TI *T1i, *T2i;
  const double* f;
  double* x;
  double* r;
  TI* V;
  TI* w;
  double* partials;
  int m, max_cycles;
  double tol, inner_floor;
  unsigned* bar;
  int* status;
  double* report;
};

// Phases 1 and 2 of y -> M y over the whole grid (output T2 complete on return).
template <typename T>
__device__ __forceinline__ bool apply12(const Contraction& p1, const Contraction& p2, const T* L, const T* A,
                                        const T* y, T* T1, T* T2, const GridBarrier& bar, int* st) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t G = (int64_t)gridDim.x * blockDim.x;
  contract_range(p1, L, y, T1, T(1), T(0), g, G);
  if (!grid_sync(bar, st)) return false;
  contract_range(p2, T1, A, T2, T(1), T(0), g, G);
  return grid_sync(bar, st);
}

// Phase 3 for one element of the (dense) output vector.
template <typename T>
__device__ __forceinline__ T apply3(const Contraction& p3, const T* T2, const T* R, int64_t e) {
  int64_t ao, bo, co;
  contract_offsets(p3, e, ao, bo, co);
  return contract_sum(p3, T2, R, ao, bo);
}

// partial[kk] = sum_{e in chunk} X_kk[e] w[e] for kk < nvec (X_kk = V_kk),
// partial[nvec] = sum w[e]^2.
template <typename T>
__device__ __forceinline__ void chunk_dots(const T* V, int64_t N, int nvec, const T* w, int e0, int e1,
                                           double* partial) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int kk = warp; kk <= nvec; kk += nw) {
    const T* xv = (kk < nvec) ? V + (int64_t)kk * N : w;
    double s = 0.0;
    for (int e = e0 + lane; e < e1; e += 32) s += (double)xv[e] * (double)w[e];
    s = warp_sum(s);
    if (lane == 0) partial[kk] = s;
  }
}

// Block sum of one value per thread, written by thread 0 to *dst.
__device__ __forceinline__ void block_partial(double v, double* dst) {
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nw; ++i) s += red[i];
    *dst = s;
  }
  __syncthreads();
}

template <typename TI>
__global__ void __launch_bounds__(kKThreads, 1) gmres_ir_kernel(GmresK<TI> k) {
  extern __shared__ double sm[];
  const int m = k.m;
  double* H = sm;  // (m+1) x m, column-major
  double* cs = H + (m + 1) * m;
  double* sn = cs + m;
  double* gv = sn + m;     // m + 1
  double* yv = gv + m + 1; // m
  double* h1 = yv + m;     // m + 2
  double* h2 = h1 + m + 2; // m + 2
  __shared__ double s_scal[4];
  __shared__ int s_flag;

  const GridBarrier bar{k.bar, k.bar + 1};
  const int tid = threadIdx.x, nt = blockDim.x;
  const int64_t N = k.N;
  const int chunk = (int)((N + gridDim.x - 1) / gridDim.x);
  const int e0 = (int)imin64(N, (int64_t)blockIdx.x * chunk);
  const int e1 = (int)imin64(N, (int64_t)e0 + chunk);
  const int ps = m + 2;
  int rb = 0;
  auto prow = [&](int buf) { return k.partials + ((int64_t)buf * gridDim.x + blockIdx.x) * ps; };
  auto pbuf = [&](int buf) { return k.partials + (int64_t)buf * gridDim.x * ps; };

  // ||f||
  {
    double s = 0.0;
    for (int e = e0 + tid; e < e1; e += nt) s += k.f[e] * k.f[e];
    block_partial(s, prow(rb));
    if (!grid_sync(bar, k.status)) return;
    reduce_partials(pbuf(rb), ps, 1, h1);
    rb ^= 1;
  }
  const double fnorm = sqrt(h1[0]);
  if (!(fnorm > 0.0)) {
    for (int e = e0 + tid; e < e1; e += nt) k.x[e] = 0.0;
    if (blockIdx.x == 0 && tid == 0) {
      k.report[0] = 0.0; k.report[1] = 0; k.report[2] = 0;
      if (!(fnorm == 0.0)) atomicCAS(k.status, ST_OK, ST_NONFINITE);
    }
    return;
  }

  double rel = 1.0;
  int cycles = 0, inner = 0;
  for (int cyc = 0; cyc < k.max_cycles; ++cyc) {
    // FP64 residual r = f - M x
    if (!apply12<double>(k.p1, k.p2, k.L64, k.A64, k.x, k.T1_64, k.T2_64, bar, k.status)) return;
    double s = 0.0;
    for (int e = e0 + tid; e < e1; e += nt) {
      const double re = k.f[e] - apply3<double>(k.p3, k.T2_64, k.R64, e);
      k.r[e] = re;
      s += re * re;
    }
    block_partial(s, prow(rb));
    if (!grid_sync(bar, k.status)) return;
    reduce_partials(pbuf(rb), ps, 1, h1);
    rb ^= 1;
    const double rho = sqrt(h1[0]);
    rel = rho / fnorm;
    cycles = cyc + 1;
    if (!isfinite(rel)) {
      if (tid == 0) atomicCAS(k.status, ST_OK, ST_NONFINITE);
      break;
    }
    if (rel <= k.tol) break;

    // one inner GMRES(m) cycle in TI on M d = r / rho
    const double target = fmax(k.tol / rel, k.inner_floor);
    for (int e = e0 + tid; e < e1; e += nt) k.V[e] = (TI)(k.r[e] / rho);
    if (tid == 0) {
      gv[0] = 1.0;
      for (int i = 1; i <= m; ++i) gv[i] = 0.0;
    }
    if (!grid_sync(bar, k.status)) return;
    int jj = 0;
    for (int j = 0; j < m; ++j) {
      const TI* vj = k.V + (int64_t)j * N;
      if (!apply12<TI>(k.p1, k.p2, k.Li, k.Ai, vj, k.T1i, k.T2i, bar, k.status)) return;
      for (int e = e0 + tid; e < e1; e += nt) k.w[e] = apply3<TI>(k.p3, k.T2i, k.Ri, e);
      __syncthreads();
      chunk_dots<TI>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
      if (!grid_sync(bar, k.status)) return;
      reduce_partials(pbuf(rb), ps, j + 2, h1);
      rb ^= 1;
      for (int e = e0 + tid; e < e1; e += nt) {
        double acc = (double)k.w[e];
        for (int q = 0; q <= j; ++q) acc -= h1[q] * (double)k.V[(int64_t)q * N + e];
        k.w[e] = (TI)acc;
      }
      __syncthreads();
      chunk_dots<TI>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
      if (!grid_sync(bar, k.status)) return;
      reduce_partials(pbuf(rb), ps, j + 2, h2);
      rb ^= 1;
      double hn2 = h2[j + 1];
      for (int q = 0; q <= j; ++q) hn2 -= h2[q] * h2[q];
      const double hn = sqrt(fmax(hn2, 0.0));
      if (hn > 0.0) {
        const double inv = 1.0 / hn;
        TI* vn = k.V + (int64_t)(j + 1) * N;
        for (int e = e0 + tid; e < e1; e += nt) {
          double acc = (double)k.w[e];
          for (int q = 0; q <= j; ++q) acc -= h2[q] * (double)k.V[(int64_t)q * N + e];
          vn[e] = (TI)(acc * inv);
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
        cs[j] = c; sn[j] = sg;
        col[j] = rr; col[j + 1] = 0.0;
        gv[j + 1] = -sg * gv[j];
        gv[j] = c * gv[j];
        s_scal[0] = fabs(gv[j + 1]);
        s_flag = (hn <= 1e-300) ? 1 : 0;
      }
      __syncthreads();
      jj = j + 1;
      ++inner;
      if (s_scal[0] <= target || s_flag) break;
      if (!grid_sync(bar, k.status)) return;  // V_{j+1} complete
    }
    // y = H(0:jj, 0:jj)^{-1} g
    if (tid == 0) {
      int bad = 0;
      for (int i = jj - 1; i >= 0; --i) {
        double acc = gv[i];
        for (int l = i + 1; l < jj; ++l) acc -= H[(int64_t)l * (m + 1) + i] * yv[l];
        const double dgl = H[(int64_t)i * (m + 1) + i];
        if (dgl == 0.0) { bad = 1; yv[i] = 0.0; } else yv[i] = acc / dgl;
      }
      s_flag = bad;
    }
    __syncthreads();
    if (s_flag) {
      if (tid == 0) atomicCAS(k.status, ST_OK, ST_SINGULAR);
      break;
    }
    for (int e = e0 + tid; e < e1; e += nt) {
      double acc = 0.0;
      for (int q = 0; q < jj; ++q) acc += yv[q] * (double)k.V[(int64_t)q * N + e];
      k.x[e] += rho * acc;
    }
    if (!grid_sync(bar, k.status)) return;  // x complete before the next residual
  }
  if (blockIdx.x == 0 && tid == 0) {
    k.report[0] = rel;
    k.report[1] = cycles;
    k.report[2] = inner;
  }
}

size_t gmres_partials_doubles(int m, int num_sms) { return (size_t)2 * num_sms * (m + 2); }

static size_t gmres_smem_bytes(int m) {
  return sizeof(double) * ((size_t)(m + 1) * m + 2 * m + (m + 1) + m + 2 * (m + 2));
}

cudaError_t launch_gmres(const GmresLaunch& g, int num_sms, cudaStream_t st) {
  Contraction p1, p2, p3;
  local_apply_descs(g.sh, &p1, &p2, &p3);
  const size_t smem = gmres_smem_bytes(g.m);
  dim3 grid(num_sms), block(kKThreads);
  if (g.precision == 0) {
    GmresK<double> k{p1, p2, p3, (int)g.sh.N(), g.L64, g.A64, g.R64, g.T1_64, g.T2_64,
                     (const double*)g.Li, (const double*)g.Ai, (const double*)g.Ri, (double*)g.T1i,
                     (double*)g.T2i, g.f, g.x, g.r, (double*)g.V, (double*)g.w, g.partials, g.m,
                     g.max_cycles, g.tol, g.inner_floor, g.bar, g.status, g.report};
    cudaError_t e = cudaFuncSetAttribute(gmres_ir_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    void* args[] = {&k};
    ++launch_counter();
    return cudaLaunchCooperativeKernel((const void*)gmres_ir_kernel<double>, grid, block, args, smem, st);
  }
  GmresK<float> k{p1, p2, p3, (int)g.sh.N(), g.L64, g.A64, g.R64, g.T1_64, g.T2_64,
                  (const float*)g.Li, (const float*)g.Ai, (const float*)g.Ri, (float*)g.T1i,
                  (float*)g.T2i, g.f, g.x, g.r, (float*)g.V, (float*)g.w, g.partials, g.m,
                  g.max_cycles, g.tol, g.inner_floor, g.bar, g.status, g.report};
  cudaError_t e = cudaFuncSetAttribute(gmres_ir_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {&k};
  ++launch_counter();
  return cudaLaunchCooperativeKernel((const void*)gmres_ir_kernel<float>, grid, block, args, smem, st);
}

struct LanczosK {
  Contraction p1, p2, p3;
  int N;
  const double *L, *A, *R;
  double *T1, *T2;
  int nprev;
  const double* prevt;
  double shift;
  double* x;
  double* vals;
  double* V;
  double* w;
  double* partials;
  int m, k, mode, nonsym;
  double sigma;
  int max_restarts;
  double tol;
  unsigned* bar;
  int* status;
  double* report;
};

constexpr int kMaxEv = 8;

// smem: al m, be m, h1 (m+2), h2 (m+2), svec m*kMaxEv, tri work 6m, piv m (ints);
// Arnoldi adds H (m+1) x m, its work copy m x m, wr m, wi m
size_t lanczos_smem_bytes(int m, int nonsym) {
  size_t b = sizeof(double) * ((size_t)2 * m + 2 * (m + 2) + (size_t)m * kMaxEv + 6 * (size_t)m + 8) +
             sizeof(int) * (size_t)((m + 3) & ~1);
  if (nonsym) b += sizeof(double) * ((size_t)(m + 1) * m + (size_t)m * m + 2 * (size_t)m);
  return b;
}
size_t lanczos_partials_doubles(int m, int num_sms) { return (size_t)2 * num_sms * (m + 2 + 8); }

__global__ void __launch_bounds__(kKThreads, 1) lanczos_kernel(LanczosK k) {
  extern __shared__ double sm[];
  const int m = k.m;
  double* al = sm;
  double* be = al + m;
  double* h1 = be + m;
  double* h2 = h1 + m + 2;
  double* svec = h2 + m + 2;       // m x kMaxEv, column c at svec + c*m
  double* twk = svec + m * kMaxEv; // 5m tri work + m z
  int* piv = (int*)(twk + 6 * m + 8);
  // Arnoldi: H row-major (m+1) x m (leading dimension m), work copy, Ritz values
  double* Hs = (double*)(piv + ((m + 3) & ~1));  // even int count keeps 8-byte alignment
  double* Hw = Hs + (m + 1) * m;
  double* wr = Hw + m * m;
  double* wi = wr + m;
  __shared__ double s_theta[kMaxEv];
  __shared__ double s_res;
  __shared__ int s_conv, s_cplx;

  const GridBarrier bar{k.bar, k.bar + 1};
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int64_t N = k.N;
  const int chunk = (int)((N + gridDim.x - 1) / gridDim.x);
  const int e0 = (int)imin64(N, (int64_t)blockIdx.x * chunk);
  const int e1 = (int)imin64(N, (int64_t)e0 + chunk);
  const int ps = m + 2 + 8;
  int rb = 0;
  auto prow = [&](int buf) { return k.partials + ((int64_t)buf * gridDim.x + blockIdx.x) * ps; };
  auto pbuf = [&](int buf) { return k.partials + (int64_t)buf * gridDim.x * ps; };
  const int kev = k.k;
  if (tid == 0) {
    s_cplx = 0;
    s_conv = 0;
    s_res = 0.0;
  }

  // V_0 = x / |x| + eps z / |z| (normalised), z a fixed pseudo-random vector.
  // With several wanted eigenpairs, a start vector inside one symmetry sector
  // of the local operator would keep the whole Krylov space there and miss the
  // wanted eigenvalues of the other sectors: eps = 0.01.  A single eigenpair
  // keeps the pure warm start (eps = 0), whose residual is already small.
  {
    auto noise = [](int e) {
      uint32_t hsh = (uint32_t)e * 2654435761u ^ 0x9e3779b9u;
      hsh ^= hsh >> 15;
      hsh *= 2246822519u;
      hsh ^= hsh >> 13;
      return (double)(hsh & 0xffffff) / 8388608.0 - 1.0;
    };
    double sxx = 0.0, szz = 0.0, sxz = 0.0;
    for (int e = e0 + tid; e < e1; e += nt) {
      const double z = noise(e);
      sxx += k.x[e] * k.x[e];
      szz += z * z;
      sxz += k.x[e] * z;
    }
    block_partial(sxx, prow(rb));
    block_partial(szz, prow(rb) + 1);
    block_partial(sxz, prow(rb) + 2);
    if (!grid_sync(bar, k.status)) return;
    reduce_partials(pbuf(rb), ps, 3, h1);
    rb ^= 1;
    const double nx = sqrt(h1[0]), nz = sqrt(h1[1]);
    const bool ok = nx > 0.0 && isfinite(nx);
    const double eps = kev > 1 ? 0.01 : 0.0;
    const double ax = ok ? 1.0 / nx : 0.0, az = eps / nz;
    const double nv = sqrt(fmax((ok ? 1.0 : 0.0) + eps * eps + 2.0 * ax * az * h1[2], 1e-300));
    for (int e = e0 + tid; e < e1; e += nt) k.V[e] = (ax * k.x[e] + az * noise(e)) / nv;
    if (!grid_sync(bar, k.status)) return;
  }

  int total_it = 0, restarts = 0;
  double last_res = 0.0;
  const int mm = (int)imin64((int64_t)m, N);
  for (;;) {
    int nT = 0;
    for (int j = 0; j < mm; ++j) {
      const double* vj = k.V + (int64_t)j * N;
      // deflation dots t_p . v_j over this chunk (reduced after the P1 barrier)
      if (k.nprev > 0) {
        for (int p = warp; p < k.nprev; p += (nt >> 5)) {
          const double* tp = k.prevt + (int64_t)p * N;
          double s = 0.0;
          for (int e = e0 + lane; e < e1; e += 32) s += tp[e] * vj[e];
          s = warp_sum(s);
          if (lane == 0) prow(rb)[p] = s;
        }
      }
      if (!apply12<double>(k.p1, k.p2, k.L, k.A, vj, k.T1, k.T2, bar, k.status)) return;
      if (k.nprev > 0) {
        reduce_partials(pbuf(rb), ps, k.nprev, h2);
        rb ^= 1;
      }
      for (int e = e0 + tid; e < e1; e += nt) {
        double v = apply3<double>(k.p3, k.T2, k.R, e);
        for (int p = 0; p < k.nprev; ++p) v += k.shift * h2[p] * k.prevt[(int64_t)p * N + e];
        k.w[e] = v;
      }
      __syncthreads();
      chunk_dots<double>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
      if (!grid_sync(bar, k.status)) return;
      reduce_partials(pbuf(rb), ps, j + 2, h1);
      rb ^= 1;
      for (int e = e0 + tid; e < e1; e += nt) {
        double acc = k.w[e];
        for (int q = 0; q <= j; ++q) acc -= h1[q] * k.V[(int64_t)q * N + e];
        k.w[e] = acc;
      }
      __syncthreads();
      chunk_dots<double>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
      if (!grid_sync(bar, k.status)) return;
      reduce_partials(pbuf(rb), ps, j + 2, h2);
      rb ^= 1;
      double b2 = h2[j + 1];
      for (int q = 0; q <= j; ++q) b2 -= h2[q] * h2[q];
      const double bj = sqrt(fmax(b2, 0.0));
      const double alj = h1[j] + h2[j];
      double tnorm = 0.0;
      for (int i = 0; i <= j; ++i)
        tnorm = fmax(tnorm, fabs(i == j ? alj : al[i]) + fabs(i == j ? bj : be[i]) + (i > 0 ? fabs(be[i - 1]) : 0.0));
      // Breakdown: the basis spans an invariant subspace.  Unless the basis is
      // full, continue from a fresh direction orthogonal to it (zero coupling in
      // T / H), so that eigenvalues outside the subspace -- other symmetry
      // sectors, further copies of a multiple eigenvalue -- stay reachable.
      const bool breakdown = !(bj > 1e-14 * fmax(tnorm, 1e-300));
      const bool fresh = breakdown && j + 1 < mm;
      __syncthreads();
      if (tid == 0) {
        al[j] = alj;
        be[j] = fresh ? 0.0 : bj;
        if (k.nonsym) {
          for (int q = 0; q <= j; ++q) Hs[q * m + j] = h1[q] + h2[q];
          Hs[(j + 1) * m + j] = fresh ? 0.0 : bj;
        }
      }
      if (!breakdown && j + 1 < mm) {
        double* vn = k.V + (int64_t)(j + 1) * N;
        const double inv = 1.0 / bj;
        for (int e = e0 + tid; e < e1; e += nt) {
          double acc = k.w[e];
          for (int q = 0; q <= j; ++q) acc -= h2[q] * k.V[(int64_t)q * N + e];
          vn[e] = acc * inv;
        }
      }
      __syncthreads();
      if (fresh) {
        // deterministic pseudo-random direction, two classical Gram-Schmidt passes
        for (int e = e0 + tid; e < e1; e += nt) {
          uint32_t hsh = (uint32_t)e * 2654435761u ^ (uint32_t)(j + 1) * 40503u ^ (uint32_t)restarts * 97u;
          hsh ^= hsh >> 15;
          hsh *= 2246822519u;
          hsh ^= hsh >> 13;
          k.w[e] = (double)(hsh & 0xffffff) / 8388608.0 - 1.0;
        }
        __syncthreads();
        double nb2 = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
          chunk_dots<double>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
          if (!grid_sync(bar, k.status)) return;
          reduce_partials(pbuf(rb), ps, j + 2, h2);
          rb ^= 1;
          nb2 = h2[j + 1];
          for (int q = 0; q <= j; ++q) nb2 -= h2[q] * h2[q];
          for (int e = e0 + tid; e < e1; e += nt) {
            double acc = k.w[e];
            for (int q = 0; q <= j; ++q) acc -= h2[q] * k.V[(int64_t)q * N + e];
            k.w[e] = acc;
          }
          __syncthreads();
        }
        const double nb = sqrt(fmax(nb2, 0.0));
        double* vn = k.V + (int64_t)(j + 1) * N;
        for (int e = e0 + tid; e < e1; e += nt) vn[e] = nb > 0.0 ? k.w[e] / nb : 0.0;
        __syncthreads();
      }
      ++total_it;
      nT = j + 1;
      const double bres = fresh ? 0.0 : bj;  // norm of the residual direction of the Ritz pairs
      // Rayleigh-Ritz on T_nT every 4 steps or at the end of the basis
      const bool check = !fresh && nT >= kev && ((nT % 4) == 0 || nT == mm);
      if (check && k.nonsym) {
        if (warp == 0) {
          // Ritz values of the nT x nT Hessenberg projection
          for (int i = lane; i < nT; i += 32)
            for (int q = 0; q < nT; ++q) Hw[i * m + q] = (q >= i - 1) ? Hs[i * m + q] : 0.0;
          double hn = 0.0;
          for (int q = lane; q < nT; q += 32) {
            double cs = 0.0;
            for (int i = 0; i <= (q + 1 < nT ? q + 1 : nT - 1); ++i) cs += fabs(Hs[i * m + q]);
            hn = fmax(hn, cs);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) hn = fmax(hn, __shfl_xor_sync(0xffffffffu, hn, o));
          hn = fmax(hn, 1e-300);
          __syncwarp();
          const bool qr_ok = hess_eigvals_warp(Hw, m, nT, wr, wi);
          double resmax = 0.0;
          if (lane == 0) {
            // wanted indices: closest to sigma (complex distance), ascending; mode 3 reversed
            int sel[kMaxEv];
            bool used[64];
            for (int i = 0; i < nT; ++i) used[i] = false;
            for (int c = 0; c < kev; ++c) {
              int best = -1;
              double bd = 0.0;
              for (int i = 0; i < nT; ++i) {
                if (used[i]) continue;
                double dist;
                if (k.mode == 0) dist = -wr[i];
                else if (k.mode == 2) dist = wr[i];
                else dist = hypot(wr[i] - k.sigma, wi[i]);
                if (best < 0 || dist < bd) {
                  best = i;
                  bd = dist;
                }
              }
              sel[c] = best < 0 ? 0 : best;
              if (best >= 0) used[best] = true;
            }
            if (k.mode == 3)
              for (int c = 0; c < kev / 2; ++c) {
                const int t = sel[c];
                sel[c] = sel[kev - 1 - c];
                sel[kev - 1 - c] = t;
              }
            int cplx = 0;
            for (int c = 0; c < kev; ++c) {
              const double th = wr[sel[c]];
              if (fabs(wi[sel[c]]) > 1e-10 * hn) cplx = 1;
              double* z = svec + c * m;
              hess_eigvec(Hs, m, nT, th, hn, z, Hw, piv);
              s_theta[c] = th;
              resmax = fmax(resmax, bres * fabs(z[nT - 1]) / hn);
            }
            s_cplx = cplx;
            s_res = resmax;
            s_conv = qr_ok && !cplx && (resmax <= k.tol);
          }
          __syncwarp();
        }
        __syncthreads();
        last_res = s_res;
        if (s_conv || nT == mm) break;
      } else if (check) {
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
          // choose the wanted indices
          int sel[kMaxEv];
          if (k.mode == 0) {
            for (int c = 0; c < kev; ++c) sel[c] = nT - 1 - c;
          } else if (k.mode == 2) {
            for (int c = 0; c < kev; ++c) sel[c] = c;
          } else {
            // closest to sigma: merge outward from the count below sigma
            const int below = sturm_count(al, be, nT, k.sigma, pivmin);
            int dn = below - 1, up = below;
            double vdn = (dn >= 0) ? tri_eigval(al, be, nT, dn, lo, hi, pivmin) : 0.0;
            double vup = (up < nT) ? tri_eigval(al, be, nT, up, lo, hi, pivmin) : 0.0;
            for (int c = 0; c < kev; ++c) {
              const bool take_dn = (dn >= 0) && (up >= nT || fabs(vdn - k.sigma) <= fabs(vup - k.sigma));
              if (take_dn) {
                sel[c] = dn--;
                if (dn >= 0) vdn = tri_eigval(al, be, nT, dn, lo, hi, pivmin);
              } else {
                sel[c] = up++;
                if (up < nT) vup = tri_eigval(al, be, nT, up, lo, hi, pivmin);
              }
            }
            if (k.mode == 3)
              for (int c = 0; c < kev / 2; ++c) {
                const int t = sel[c];
                sel[c] = sel[kev - 1 - c];
                sel[kev - 1 - c] = t;
              }
          }
          double resmax = 0.0;
          for (int c = 0; c < kev; ++c) {
            const double th = tri_eigval(al, be, nT, sel[c], lo, hi, pivmin);
            double* z = svec + c * m;
            if (lane == 0) {
              tri_eigvec(al, be, nT, th, fmax(tnorm, 1e-300), z, twk, piv);
              // orthogonalise against earlier selected vectors (clustered values)
              for (int q = 0; q < c; ++q) {
                const double* zq = svec + q * m;
                double dt = 0.0;
                for (int i = 0; i < nT; ++i) dt += zq[i] * z[i];
                for (int i = 0; i < nT; ++i) z[i] -= dt * zq[i];
                double nr = 0.0;
                for (int i = 0; i < nT; ++i) nr += z[i] * z[i];
                nr = sqrt(nr);
                if (nr > 0.0)
                  for (int i = 0; i < nT; ++i) z[i] /= nr;
              }
              s_theta[c] = th;
            }
            __syncwarp();
            resmax = fmax(resmax, bres * fabs(z[nT - 1]) / fmax(tnorm, 1e-300));
          }
          if (lane == 0) {
            s_res = resmax;
            s_conv = resmax <= k.tol;
          }
        }
        __syncthreads();
        last_res = s_res;
        if (s_conv || nT == mm) break;
      }
      if (!grid_sync(bar, k.status)) return;  // V_{j+1} complete
    }
    // Ritz vectors X[e*k + c] = sum_l V_l[e] z_c[l]
    for (int e = e0 + tid; e < e1; e += nt) {
      for (int c = 0; c < kev; ++c) {
        const double* z = svec + c * m;
        double acc = 0.0;
        for (int l = 0; l < nT; ++l) acc += z[l] * k.V[(int64_t)l * N + e];
        k.x[(int64_t)e * kev + c] = acc;
      }
    }
    const bool done = s_conv || restarts >= k.max_restarts;
    if (done) break;
    ++restarts;
    // restart from the (sum of the) wanted Ritz vectors
    if (!grid_sync(bar, k.status)) return;
    double s = 0.0;
    for (int e = e0 + tid; e < e1; e += nt) {
      double v = 0.0;
      for (int c = 0; c < kev; ++c) v += k.x[(int64_t)e * kev + c];
      k.w[e] = v;
      s += v * v;
    }
    block_partial(s, prow(rb));
    if (!grid_sync(bar, k.status)) return;
    reduce_partials(pbuf(rb), ps, 1, h1);
    rb ^= 1;
    const double nrm = sqrt(h1[0]);
    for (int e = e0 + tid; e < e1; e += nt) k.V[e] = (nrm > 0.0) ? k.w[e] / nrm : 1.0 / sqrt((double)N);
    if (!grid_sync(bar, k.status)) return;
  }
  if (k.nonsym && s_cplx && blockIdx.x == 0 && tid == 0) atomicExch(k.status, ST_UNSUPPORTED);
  if (blockIdx.x == 0 && tid == 0) {
    for (int c = 0; c < kev; ++c) k.vals[c] = s_theta[c];
    k.report[0] = last_res;
    k.report[1] = restarts;
    k.report[2] = total_it;
    if (!s_conv) k.report[3] = 1.0;
    else k.report[3] = 0.0;
  }
}

cudaError_t launch_lanczos(const LanczosLaunch& l, int num_sms, cudaStream_t st) {
  if (l.k < 1 || l.k > kMaxEv) return cudaErrorInvalidValue;
  Contraction p1, p2, p3;
  local_apply_descs(l.sh, &p1, &p2, &p3);
  if (l.nonsym && l.m > 64) return cudaErrorInvalidValue;
  LanczosK k{p1, p2, p3, (int)l.sh.N(), l.L, l.A, l.R, l.T1, l.T2, l.nprev, l.prevt, l.shift, l.x, l.vals,
             l.V, l.w, l.partials, l.m, l.k, l.mode, l.nonsym, l.sigma, l.max_restarts, l.tol, l.bar, l.status,
             l.report};
  const size_t smem = lanczos_smem_bytes(l.m, l.nonsym);
  cudaError_t e = cudaFuncSetAttribute(lanczos_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {&k};
  ++launch_counter();
  return cudaLaunchCooperativeKernel((const void*)lanczos_kernel, dim3(num_sms), dim3(kKThreads), args, smem, st);
}

// ---------------------------------------------------------------------------
// exponential action
// ---------------------------------------------------------------------------

struct ExpmK {
  Contraction p1, p2, p3;
  int N;
  const double *L, *A, *R;
  double *T1, *T2;
  double* x;
  double* V;
  double* w;
  double* partials;
  int m, literal, max_substeps;
  double tau, tol;
  unsigned* bar;
  int* status;
  double* report;
};

// smem: al m, be m, h1 (m+2), h2 (m+2), c m
size_t expm_smem_bytes(int m) { return sizeof(double) * ((size_t)5 * m + 4); }

__global__ void __launch_bounds__(kKThreads, 1) expm_kernel(ExpmK k) {
  extern __shared__ double sm[];
  const int m = k.m;
  double* al = sm;
  double* be = al + m;
  double* h1 = be + m;
  double* h2 = h1 + m + 2;
  double* cv = h2 + m + 2;
  __shared__ double s_h, s_err;
  __shared__ int s_stop, s_fail;

  const GridBarrier bar{k.bar, k.bar + 1};
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int64_t N = k.N;
  const int chunk = (int)((N + gridDim.x - 1) / gridDim.x);
  const int e0 = (int)imin64(N, (int64_t)blockIdx.x * chunk);
  const int e1 = (int)imin64(N, (int64_t)e0 + chunk);
  const int ps = m + 2;
  int rb = 0;
  auto prow = [&](int buf) { return k.partials + ((int64_t)buf * gridDim.x + blockIdx.x) * ps; };
  auto pbuf = [&](int buf) { return k.partials + (int64_t)buf * gridDim.x * ps; };
  // the literal recurrence runs its m steps even past dimension N (with an
  // unnormalised start vector it does not terminate there)
  const int mm = k.literal ? m : (int)imin64((int64_t)m, N);
  if (tid == 0) {
    s_fail = 0;
    s_err = 0.0;
  }

  // c = exp(h T_nT) e_1 (warp 0) for the largest admissible h <= rem, with the
  // a-posteriori error estimate bres |c_{nT-1}|; returns through s_h / s_err / s_stop
  auto project = [&](int nT, double bres, bool final_check, double rem) {
    if (warp == 0) {
      bool ok = true;
      double h = rem;
      double cn = tri_expv_warp(al, be, nT, h, cv, &ok);
      double err = bres * fabs(cv[nT - 1]);
      bool stop = !ok || k.literal || err <= k.tol * cn;
      if (!stop && final_check) {
        for (int q = 0; q < 60 && ok && err > k.tol * cn; ++q) {
          h *= 0.5;
          cn = tri_expv_warp(al, be, nT, h, cv, &ok);
          err = bres * fabs(cv[nT - 1]);
        }
        stop = true;
      }
      if (lane == 0) {
        if (!ok) s_fail = 1;
        s_stop = stop ? 1 : 0;
        s_h = h;
        s_err = cn > 0.0 ? err / cn : 0.0;
      }
      __syncwarp();
    }
    __syncthreads();
  };

  double rem = k.tau;
  int substeps = 0, total_it = 0, last_nT = 0;
  for (;;) {
    // start vector: x itself (literal) or x / |x|
    double scale = 1.0;
    if (!k.literal) {
      double sxx = 0.0;
      for (int e = e0 + tid; e < e1; e += nt) sxx += k.x[e] * k.x[e];
      block_partial(sxx, prow(rb));
      if (!grid_sync(bar, k.status)) return;
      reduce_partials(pbuf(rb), ps, 1, h1);
      rb ^= 1;
      scale = sqrt(h1[0]);
      if (!(scale > 0.0)) break;  // exp(tau M) 0 = 0
    }
    const double inv0 = 1.0 / scale;
    for (int e = e0 + tid; e < e1; e += nt) k.V[e] = k.x[e] * inv0;
    if (!grid_sync(bar, k.status)) return;

    int nT = 0;
    double trow = 0.0;
    if (tid == 0) s_stop = 0;
    for (int j = 0; j < mm; ++j) {
      const double* vj = k.V + (int64_t)j * N;
      if (!apply12<double>(k.p1, k.p2, k.L, k.A, vj, k.T1, k.T2, bar, k.status)) return;
      for (int e = e0 + tid; e < e1; e += nt) k.w[e] = apply3<double>(k.p3, k.T2, k.R, e);
      __syncthreads();
      double alj, bj;
      if (k.literal) {
        // alpha_j = w . v_j;  w -= alpha_j v_j + beta_{j-1} v_{j-1};  beta_j = |w|
        double s = 0.0;
        for (int e = e0 + tid; e < e1; e += nt) s += k.w[e] * vj[e];
        block_partial(s, prow(rb));
        if (!grid_sync(bar, k.status)) return;
        reduce_partials(pbuf(rb), ps, 1, h1);
        rb ^= 1;
        alj = h1[0];
        const double bprev = j > 0 ? be[j - 1] : 0.0;
        const double* vp = j > 0 ? k.V + (int64_t)(j - 1) * N : vj;
        double s2 = 0.0;
        for (int e = e0 + tid; e < e1; e += nt) {
          const double v = k.w[e] - alj * vj[e] - bprev * vp[e];
          k.w[e] = v;
          s2 += v * v;
        }
        block_partial(s2, prow(rb));
        if (!grid_sync(bar, k.status)) return;
        reduce_partials(pbuf(rb), ps, 1, h2);
        rb ^= 1;
        bj = sqrt(h2[0]);
      } else {
        // classical Gram-Schmidt against the whole basis; a second pass only
        // when the first removed more than half of |w|^2 ("twice is enough":
        // otherwise one pass leaves w orthogonal to working accuracy)
        chunk_dots<double>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
        if (!grid_sync(bar, k.status)) return;
        reduce_partials(pbuf(rb), ps, j + 2, h1);
        rb ^= 1;
        // sums over q by the lanes of each warp (FP64 is scarce: no per-thread loop)
        double sq = 0.0;
        for (int q = lane; q <= j; q += 32) sq += h1[q] * h1[q];
        sq = warp_sum(sq);
        const double wn2 = h1[j + 1], rest = wn2 - sq;
        for (int e = e0 + tid; e < e1; e += nt) {
          double acc = k.w[e];
          for (int q = 0; q <= j; ++q) acc -= h1[q] * k.V[(int64_t)q * N + e];
          k.w[e] = acc;
        }
        alj = h1[j];
        if (rest >= 0.5 * wn2) {
          bj = sqrt(rest);
        } else {
          __syncthreads();
          chunk_dots<double>(k.V, N, j + 1, k.w, e0, e1, prow(rb));
          if (!grid_sync(bar, k.status)) return;
          reduce_partials(pbuf(rb), ps, j + 2, h2);
          rb ^= 1;
          double sq2 = 0.0;
          for (int q = lane; q <= j; q += 32) sq2 += h2[q] * h2[q];
          sq2 = warp_sum(sq2);
          bj = sqrt(fmax(h2[j + 1] - sq2, 0.0));
          alj += h2[j];
          for (int e = e0 + tid; e < e1; e += nt) {
            double acc = k.w[e];
            for (int q = 0; q <= j; ++q) acc -= h2[q] * k.V[(int64_t)q * N + e];
            k.w[e] = acc;
          }
        }
      }
      // |T|_inf: running maximum over the completed rows plus the current row
      if (j > 0) trow = fmax(trow, fabs(al[j - 1]) + fabs(be[j - 1]) + (j > 1 ? fabs(be[j - 2]) : 0.0));
      const double tnorm = fmax(trow, fabs(alj) + fabs(bj) + (j > 0 ? fabs(be[j - 1]) : 0.0));
      // an invariant subspace (or the whole space) makes the projection exact;
      // the literal recurrence stops only where it would divide by zero
      const bool breakdown = k.literal ? !(bj > 0.0)
                                       : (!(bj > 1e-14 * fmax(tnorm, 1e-300)) || j + 1 == (int)N);
      __syncthreads();
      if (tid == 0) {
        al[j] = alj;
        be[j] = bj;
      }
      nT = j + 1;
      ++total_it;
      if (!breakdown && j + 1 < mm) {
        double* vn = k.V + (int64_t)(j + 1) * N;
        const double inv = 1.0 / bj;
        for (int e = e0 + tid; e < e1; e += nt) vn[e] = k.w[e] * inv;
      }
      __syncthreads();
      const bool last = breakdown || nT == mm;
      if (last || !k.literal) {
        project(nT, breakdown ? 0.0 : bj, last, rem);
        if (s_stop) break;
      }
      if (!grid_sync(bar, k.status)) return;  // V_{j+1} complete
    }
    last_nT = nT;
    // x = scale * sum_l c_l V_l
    for (int e = e0 + tid; e < e1; e += nt) {
      double acc = 0.0;
      for (int l = 0; l < nT; ++l) acc += cv[l] * k.V[(int64_t)l * N + e];
      k.x[e] = scale * acc;
    }
    ++substeps;
    if (s_fail) break;
    const double h = s_h;
    rem = (h == rem) ? 0.0 : rem - h;
    if (k.literal || rem == 0.0) break;
    if (substeps >= k.max_substeps) {
      if (blockIdx.x == 0 && tid == 0) atomicCAS(k.status, ST_OK, ST_NOCONV);
      break;
    }
    if (!grid_sync(bar, k.status)) return;
  }
  if (blockIdx.x == 0 && tid == 0) {
    if (s_fail) atomicCAS(k.status, ST_OK, ST_NONFINITE);
    k.report[0] = s_err;
    k.report[1] = substeps;
    k.report[2] = total_it;
    k.report[3] = last_nT;
  }
}

cudaError_t launch_expm(const ExpmLaunch& l, int num_sms, cudaStream_t st) {
  if (l.m < 1 || l.m > 64 || l.max_substeps < 1) return cudaErrorInvalidValue;
  Contraction p1, p2, p3;
  local_apply_descs(l.sh, &p1, &p2, &p3);
  ExpmK k{p1,  p2,         p3,     (int)l.sh.N(), l.L,   l.A,   l.R,      l.T1,     l.T2,     l.x,
          l.V, l.w,        l.partials, l.m,       l.literal, l.max_substeps, l.tau, l.tol, l.bar, l.status,
          l.report};
  const size_t smem = expm_smem_bytes(l.m);
  cudaError_t e = cudaFuncSetAttribute(expm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // TDVP's local problems are small (10^2 - 10^4 unknowns): one CTA per 64
  // unknowns keeps ~2 us of FP64 work per contraction phase and CTA while the
  // grid barrier, whose latency grows with the CTAs arriving, stays short
  const int grid = (int)std::min<int64_t>(num_sms, std::max<int64_t>(1, (l.sh.N() + 63) / 64));
  void* args[] = {&k};
  ++launch_counter();
  return cudaLaunchCooperativeKernel((const void*)expm_kernel, dim3(grid), dim3(kKThreads), args, smem, st);
}

}  // namespace ttals
