// Device-side building blocks of the tensor-train ALS engine (sm_103a).
//
// * Contraction: a strided "one output element per thread" tensor contraction
//   descriptor.  Every contraction of the ALS hot path (interface stacks,
//   local-operator apply, local right-hand side, gauge pushes, operator-core
//   products) is one or a chain of these.
// * GridBarrier: an all-CTA barrier for cooperative (co-resident) launches.
//   Its spin is bounded: after kSpinLimit polls it records a timeout in the
//   solver's status word and returns false, so a broken launch never hangs
//   the device.
// * Deterministic grid reductions: every CTA writes its partial sums, then
//   every CTA re-reduces all partials in the same fixed order, so all CTAs
//   hold bit-identical scalars and take identical branches.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ttals {

// Thread groups of the batch kernels.  The tensor-core variant runs two
// independent solves per CTA, one per group of kGroupThreads threads, each
// with its own named barrier (ids 1 and 2), shared state and tensor memory,
// so that one group's memory round trips overlap the other's work.  Every
// other kernel is one group: the whole CTA (barrier 0).  G = true selects the
// two-group form; code instantiated with G = true never uses a CTA-wide
// barrier.
constexpr int kGroupThreads = 256;
template <bool G>
constexpr int kGroups = G ? 2 : 1;
template <bool G>
__device__ __forceinline__ int gtid() {
  if constexpr (G)
    return (int)(threadIdx.x & (kGroupThreads - 1));
  else
    return (int)threadIdx.x;
}
template <bool G>
__device__ __forceinline__ int gsize() {
  if constexpr (G)
    return kGroupThreads;
  else
    return (int)blockDim.x;
}
template <bool G>
__device__ __forceinline__ int gidx() {
  if constexpr (G)
    return (int)(threadIdx.x / kGroupThreads);
  else
    return 0;
}
template <bool G>
__device__ __forceinline__ void gsync() {
  if constexpr (G)
    asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x / kGroupThreads)), "n"(kGroupThreads) : "memory");
  else
    __syncthreads();
}

constexpr int kMaxOut = 6;
constexpr int kMaxK = 3;

// status codes shared with the host (mirrors include/ttals.h)
enum : int {
  ST_OK = 0,
  ST_ARG = 1,
  ST_CUDA = 2,
  ST_NOMEM = 3,
  ST_SINGULAR = 4,
  ST_NONFINITE = 5,
  ST_TIMEOUT = 6,
  ST_NOCONV = 7,
  ST_UNSUPPORTED = 8,
};

// C[out] = alpha * sum_k A[a_off(out) + a_k(k)] * B[b_off(out) + b_k(k)] + beta * C[out]
// out is the row-major multi-index over out_dim[0..nout-1].  Offsets and
// element counts are 32-bit (every buffer of the path holds < 2^31 elements;
// launchers reject larger contractions).  Output indices are decoded with
// precomputed multiply-shift division (Granlund-Montgomery round-up method):
// for n < 2^31, n / d == (umulhi(n, mag) + n) >> shf.
struct Contraction {
  int nout, nk;
  int out_dim[kMaxOut];
  uint32_t out_mag[kMaxOut];
  int out_shf[kMaxOut];
  int k_dim[kMaxK];
  int a_os[kMaxOut], a_ks[kMaxK];
  int b_os[kMaxOut], b_ks[kMaxK];
  int c_os[kMaxOut];
  int64_t total;   // product of out_dim
  int64_t ktotal;  // product of k_dim
};

__host__ __device__ __forceinline__ void fast_div_params(uint32_t d, uint32_t* mag, int* shf) {
  int l = 0;
  while (l < 31 && (1u << l) < d) ++l;
  *shf = l;
  *mag = (uint32_t)(((uint64_t)1 << 32) * ((uint64_t(1) << l) - d) / d + 1);
}

__host__ __device__ __forceinline__ uint32_t fast_div(uint32_t n, uint32_t mag, int shf) {
#ifdef __CUDA_ARCH__
  const uint32_t t = __umulhi(n, mag);
#else
  const uint32_t t = (uint32_t)(((uint64_t)n * mag) >> 32);
#endif
  return (t + n) >> shf;
}

// Offsets of output element e (row-major over out_dim) in A, B and C.
__host__ __device__ __forceinline__ void contract_offsets(const Contraction& c, int64_t e, int64_t& ao,
                                                          int64_t& bo, int64_t& co) {
  uint32_t rem = (uint32_t)e;
  int a = 0, b = 0, o = 0;
#pragma unroll
  for (int q = kMaxOut - 1; q >= 0; --q) {
    if (q < c.nout) {
      const uint32_t qq = fast_div(rem, c.out_mag[q], c.out_shf[q]);
      const int iq = (int)(rem - qq * (uint32_t)c.out_dim[q]);
      rem = qq;
      a += iq * c.a_os[q];
      b += iq * c.b_os[q];
      o += iq * c.c_os[q];
    }
  }
  ao = a;
  bo = b;
  co = o;
}

// The contraction sum of one output element.  Split into independent
// accumulator chains so consecutive FMAs do not wait on each other.
template <typename T>
__host__ __device__ __forceinline__ T contract_sum(const Contraction& c, const T* __restrict__ A,
                                                   const T* __restrict__ B, int64_t ao, int64_t bo) {
  const T* pa = A + ao;
  const T* pb = B + bo;
  if (c.nk == 1) {
    const int sa = c.a_ks[0], sb = c.b_ks[0], K = c.k_dim[0];
    T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
    int k = 0;
    for (; k + 3 < K; k += 4) {
      a0 += pa[k * sa] * pb[k * sb];
      a1 += pa[(k + 1) * sa] * pb[(k + 1) * sb];
      a2 += pa[(k + 2) * sa] * pb[(k + 2) * sb];
      a3 += pa[(k + 3) * sa] * pb[(k + 3) * sb];
    }
    for (; k < K; ++k) a0 += pa[k * sa] * pb[k * sb];
    return (a0 + a1) + (a2 + a3);
  }
  if (c.nk == 2) {
    const int sa0 = c.a_ks[0], sb0 = c.b_ks[0], sa = c.a_ks[1], sb = c.b_ks[1];
    const int K0 = c.k_dim[0], K1 = c.k_dim[1];
    T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
    int k0 = 0;
    for (; k0 + 1 < K0; k0 += 2) {
      const T* qa = pa + k0 * sa0;
      const T* qb = pb + k0 * sb0;
      const T* ra = qa + sa0;
      const T* rb = qb + sb0;
      int k1 = 0;
      for (; k1 + 1 < K1; k1 += 2) {
        a0 += qa[k1 * sa] * qb[k1 * sb];
        a1 += ra[k1 * sa] * rb[k1 * sb];
        a2 += qa[(k1 + 1) * sa] * qb[(k1 + 1) * sb];
        a3 += ra[(k1 + 1) * sa] * rb[(k1 + 1) * sb];
      }
      if (k1 < K1) {
        a0 += qa[k1 * sa] * qb[k1 * sb];
        a1 += ra[k1 * sa] * rb[k1 * sb];
      }
    }
    if (k0 < K0) {
      const T* qa = pa + k0 * sa0;
      const T* qb = pb + k0 * sb0;
      for (int k1 = 0; k1 < K1; ++k1) a2 += qa[k1 * sa] * qb[k1 * sb];
    }
    return (a0 + a1) + (a2 + a3);
  }
  if (c.nk == 3) {
    const int sa = c.a_ks[2], sb = c.b_ks[2], K2 = c.k_dim[2];
    T a0 = T(0), a1 = T(0);
    for (int k0 = 0; k0 < c.k_dim[0]; ++k0)
      for (int k1 = 0; k1 < c.k_dim[1]; ++k1) {
        const T* qa = pa + k0 * c.a_ks[0] + k1 * c.a_ks[1];
        const T* qb = pb + k0 * c.b_ks[0] + k1 * c.b_ks[1];
        int k2 = 0;
        for (; k2 + 1 < K2; k2 += 2) {
          a0 += qa[k2 * sa] * qb[k2 * sb];
          a1 += qa[(k2 + 1) * sa] * qb[(k2 + 1) * sb];
        }
        if (k2 < K2) a0 += qa[k2 * sa] * qb[k2 * sb];
      }
    return a0 + a1;
  }
  return pa[0] * pb[0];  // nk == 0: elementwise product
}

// ---------------------------------------------------------------------------
// register-tiled variant: VW consecutive outputs along the innermost output axis
// when that axis has stride 0 in A and stride 1 in B and C (true for every
// apply / stack / rhs phase of the path).  One A load and one VW-wide vector B
// load feed VW FMAs.
// ---------------------------------------------------------------------------

template <typename T, int VW>
struct VecOf;
template <>
struct VecOf<float, 4> {
  using type = float4;
};
template <>
struct VecOf<double, 2> {
  using type = double2;
};
template <>
struct VecOf<double, 1> {
  using type = double;
};

template <typename T, int VW>
__host__ __device__ __forceinline__ bool contract_vec_ok(const Contraction& c, const T* B, const T* C) {
  if (VW < 2) return false;
  const int last = c.nout - 1;
  if (c.nout < 1 || c.out_dim[last] % VW != 0) return false;
  if (c.a_os[last] != 0 || c.b_os[last] != 1 || c.c_os[last] != 1) return false;
  for (int q = 0; q < last; ++q)
    if (c.b_os[q] % VW != 0 || c.c_os[q] % VW != 0) return false;
  for (int q = 0; q < c.nk; ++q)
    if (c.b_ks[q] % VW != 0) return false;
  const uintptr_t align = sizeof(T) * VW;
  return ((uintptr_t)B % align == 0) && ((uintptr_t)C % align == 0);
}

// Computes outputs e0 .. e0+VW-1 (e0 a multiple of VW) into C.  The
// contraction axis with the largest extent runs innermost, unrolled by two
// with separate accumulators (2*VW independent FMA chains).
template <typename T, int VW>
__device__ __forceinline__ void contract_vec_elem(const Contraction& c, const T* __restrict__ A,
                                                  const T* __restrict__ B, T* __restrict__ C, int64_t e0) {
  using V = typename VecOf<T, VW>::type;
  int64_t ao, bo, co;
  contract_offsets(c, e0, ao, bo, co);
  int K[3] = {1, 1, 1}, sa[3] = {0, 0, 0}, sb[3] = {0, 0, 0};
  int inner = 0;
  for (int q = 0; q < c.nk; ++q) {
    K[q] = c.k_dim[q];
    sa[q] = c.a_ks[q];
    sb[q] = c.b_ks[q];
    if (K[q] > K[inner]) inner = q;
  }
  const int o0 = inner == 0 ? 1 : 0, o1 = inner == 2 ? 1 : 2;
  const int Ki = K[inner], sai = sa[inner], sbi = sb[inner];
  T acc0[VW], acc1[VW];
#pragma unroll
  for (int v = 0; v < VW; ++v) acc0[v] = acc1[v] = T(0);
  for (int k0 = 0; k0 < K[o0]; ++k0)
    for (int k1 = 0; k1 < K[o1]; ++k1) {
      const T* pa = A + ao + k0 * sa[o0] + k1 * sa[o1];
      const T* pb = B + bo + k0 * sb[o0] + k1 * sb[o1];
      int k = 0;
      for (; k + 1 < Ki; k += 2) {
        const T a0 = pa[k * sai], a1 = pa[(k + 1) * sai];
        const V b0 = *reinterpret_cast<const V*>(pb + k * sbi);
        const V b1 = *reinterpret_cast<const V*>(pb + (k + 1) * sbi);
        const T* x0 = reinterpret_cast<const T*>(&b0);
        const T* x1 = reinterpret_cast<const T*>(&b1);
#pragma unroll
        for (int v = 0; v < VW; ++v) {
          acc0[v] += a0 * x0[v];
          acc1[v] += a1 * x1[v];
        }
      }
      if (k < Ki) {
        const T a0 = pa[k * sai];
        const V b0 = *reinterpret_cast<const V*>(pb + k * sbi);
        const T* x0 = reinterpret_cast<const T*>(&b0);
#pragma unroll
        for (int v = 0; v < VW; ++v) acc0[v] += a0 * x0[v];
      }
    }
  V out;
  T* ov = reinterpret_cast<T*>(&out);
#pragma unroll
  for (int v = 0; v < VW; ++v) ov[v] = acc0[v] + acc1[v];
  *reinterpret_cast<V*>(C + co) = out;
}

template <typename T>
struct DefaultVW;
template <>
struct DefaultVW<float> {
  static constexpr int value = 4;
};
template <>
struct DefaultVW<double> {
  static constexpr int value = 1;  // FP64 is DFMA-bound: keep the scalar 4-chain path
};

template <typename T>
__device__ __forceinline__ void contract_range(const Contraction& c, const T* __restrict__ A,
                                               const T* __restrict__ B, T* __restrict__ C,
                                               T alpha, T beta, int64_t first, int64_t step) {
  constexpr int VW = DefaultVW<T>::value;
  if (alpha == T(1) && beta == T(0) && contract_vec_ok<T, VW>(c, B, C)) {
    for (int64_t e = first * VW; e < c.total; e += step * VW) contract_vec_elem<T, VW>(c, A, B, C, e);
    return;
  }
  for (int64_t e = first; e < c.total; e += step) {
    int64_t ao, bo, co;
    contract_offsets(c, e, ao, bo, co);
    T out = alpha * contract_sum(c, A, B, ao, bo);
    if (beta != T(0)) out += beta * C[co];
    C[co] = out;
  }
}

// ---------------------------------------------------------------------------
// grid barrier with a bounded spin
// ---------------------------------------------------------------------------

constexpr unsigned kSpinLimit = 1u << 24;  // ~1-2 s of polling with nanosleep

struct GridBarrier {
  unsigned* count;  // arrivals in the current generation
  unsigned* gen;    // generation counter
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Polls *p (acquire) until it differs from `old`, at most `limit` times with a
// 64 ns sleep between polls; false when the limit ran out.  Every spin-wait of
// the engine goes through here.
__device__ __forceinline__ bool bounded_wait_change(const unsigned* p, unsigned old, unsigned limit) {
  unsigned spins = 0;
  while (ld_acquire_u32(p) == old) {
    if (++spins > limit) return false;
    __nanosleep(64);
  }
  return true;
}

// Returns false (all threads of the CTA) if the barrier timed out or another
// CTA has already flagged an error in *status.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    unsigned g = ld_acquire_u32(b.gen);
    unsigned arrived = atom_add_acq_rel_u32(b.count, 1u);
    if (arrived == gridDim.x - 1) {
      *b.count = 0u;
      st_release_u32(b.gen, g + 1u);
    } else if (!bounded_wait_change(b.gen, g, kSpinLimit)) {
      atomicCAS(status, ST_OK, ST_TIMEOUT);
      ok = 0;
    }
    if (ok && ld_acquire_s32(status) != ST_OK) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-reduce `nv` per-thread values (vals[0..nv-1]) into out[0..nv-1]
// (valid in every thread afterwards).  scratch: >= (blockDim/32) * nv doubles.
template <int NV>
__device__ __forceinline__ void block_sum_n(double (&vals)[NV], int nv, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < nv; ++k) {
    double v = warp_sum(vals[k]);
    if (lane == 0) scratch[warp * NV + k] = v;
  }
  __syncthreads();
  for (int k = 0; k < nv; ++k) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += scratch[w * NV + k];
    vals[k] = s;
  }
  __syncthreads();
}

// Reduce the per-CTA partials partials[b * stride + k] (b < gridDim.x,
// k < nv) into out[k] in shared memory, identically in every CTA.
__device__ __forceinline__ void reduce_partials(const double* partials, int stride, int nv, double* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = warp; k < nv; k += nw) {
    double s = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(partials + (int64_t)b * stride + k);
    s = warp_sum(s);
    if (lane == 0) out[k] = s;
  }
  __syncthreads();
}

}  // namespace ttals
