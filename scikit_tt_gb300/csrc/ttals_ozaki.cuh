// FP64-accurate contractions on the BF16 tensor cores (Ozaki-style slicing).
//
// The stack updates and FP64 refinement residuals of the mixed-precision path
// are GEMM-shaped contractions C = A B (see ttals_tc.cuh for the split into
// row / column / contraction axes).  FP64 arithmetic runs at 2 FMA/clk/SM on
// this part, BF16 tensor cores at roughly three orders of magnitude more, so
// each FP64 operand is cut into S = 6 slices of 8 bits in fixed point relative
// to its row (A) or column (B) maximum:
//
//   A[i,k] = 2^E_i * sum_p a_p[i,k] 2^{-8(p+1)},   a_p integer in [-255, 255]
//   B[k,j] = 2^F_j * sum_q b_q[k,j] 2^{-8(q+1)}
//
// Every slice is exact in BF16, every slice product (< 2^16) and every sum of
// at most 64 products per level fits FP32's 24-bit significand exactly, so
//
//   C[i,j] = 2^{E_i+F_j} sum_{L=0}^{S-1} 2^{-8(L+2)} sum_{p+q=L} (a_p b_q)[i,j]
//
// is evaluated with warp-level mma.sync m16n8k16 BF16 products (FP32
// accumulate), one FP32 accumulator per level L, flushed every 64 contraction
// steps into a double-float (hi, lo) FP32 pair with error-free TwoSum.  FP64
// arithmetic is rationed on this part, so the only FP64 operation per output is
// the final hi + lo; slicing, exponents and scaling are integer bit work.
// Products with p + q >= S are dropped.  The result is
// accurate to ~2^-47 relative to |A||B| (truncation of the 48-bit slicing),
// which keeps the refinement residual and the stacks of the mixed path far
// below its 1e-10 local tolerance; the plain FP64 path never uses this.
//
// Operands containing NaN/Inf (or contractions that are not GEMM-shaped or
// too long) return false and the caller falls back to native FP64.
#pragma once

#include <cuda_bf16.h>

#include "ttals_tc.cuh"

namespace ttals {

constexpr int kOzSlices = 6;
constexpr int kOzChunk = 64;  // contraction steps per exact FP32 accumulation chunk

__device__ __forceinline__ void mma_bf16_16x8x16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// exponent E with |v| < 2^E for every v whose magnitude bits are <= abits
// (abits = FP64 bits with the sign cleared; integer order = magnitude order)
__device__ __forceinline__ int oz_exponent_bits(uint64_t abits) {
  if (abits == 0) return 0;
  const int ev = (int)(abits >> 52);
  return ev == 0 ? -1022 : ev - 1022;  // |v| = 1.f * 2^(ev-1023) < 2^(ev-1022)
}

// 48-bit fixed-point magnitude of v relative to 2^E (truncated), sign apart
__device__ __forceinline__ uint64_t oz_fixed48(uint64_t bits, int E) {
  const int ev = (int)((bits >> 52) & 0x7ff);
  if (ev == 0) return 0;  // zero or subnormal: below the slicing's resolution
  const uint64_t m = (bits & 0xfffffffffffffull) | (1ull << 52);
  // |v| = m * 2^(ev-1075); |v| * 2^(48-E) = m * 2^(ev-1075+48-E)
  const int sh = ev - 1075 + 48 - E;
  if (sh >= 0) return m << sh;  // sh <= -5 whenever |v| < 2^E; kept for safety
  if (sh <= -64) return 0;
  return m >> (-sh);
}

// BF16 bits of the signed integer slice p (0 = most significant) of a 48-bit
// magnitude.  |slice| <= 255 has at most 8 significant bits, so it is exact in
// BF16: the FP32 value is formed with the 2^23 magic-number trick and its upper
// half taken (no rounding happens).
__device__ __forceinline__ uint32_t oz_slice_bf16(uint64_t mag, uint32_t sign, int p) {
  const uint32_t s = (uint32_t)(mag >> (8 * (kOzSlices - 1 - p))) & 0xffu;
  const float f = __uint_as_float(0x4B000000u | s) - 8388608.0f;
  return (__float_as_uint(f) >> 16) | sign;
}

// FP32 -> FP64 by bit manipulation for zero and normal values (the only ones
// the level sums produce: multiples of 2^-56 below 2^40).
__device__ __forceinline__ double oz_f2d(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0) return 0.0;
  const uint64_t r = ((uint64_t)(b & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                     ((uint64_t)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)r);
}

// v * 2^sh: exponent-field add while the result stays normal, ldexp otherwise.
__device__ __forceinline__ double oz_scale(double v, int sh) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int ev = (int)((b >> 52) & 0x7ff);
  if (ev == 0) return v;
  const int en = ev + sh;
  if (en >= 1 && en <= 2046) return __longlong_as_double((long long)(b + ((uint64_t)(int64_t)sh << 52)));
  return ldexp(v, sh);
}

// Error-free FP32 accumulation: (hi, lo) += x with hi + lo exact up to lo's rounding.
__device__ __forceinline__ void oz_two_sum(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
  hi = s;
  lo = __fadd_rn(lo, err);
}

struct OzScratch {
  uint16_t* as;  // S slices of A, row-major [i][k_pad]   (bf16 bits)
  uint16_t* bs;  // S slices of B, column-major [j][k_pad] (bf16 bits)
  int* rexp;     // E_i
  int* cexp;     // F_j
  int* ktab;     // 2 * kTcMaxK contraction offsets (global: shared memory is left to L1)
  int64_t cap_a, cap_b, cap_r, cap_c;  // capacities (elements)
};

// C = contraction(A, B) with FP64-level accuracy on the BF16 tensor cores,
// executed by the whole CTA.  ktab: 2 * kTcMaxK ints of shared memory.
__device__ __forceinline__ bool cta_gemm_ozaki(const Contraction& c, const double* __restrict__ A,
                                               const double* __restrict__ B, double* __restrict__ C,
                                               const OzScratch& z, int* ktab) {
  GemmAxes rows, cols;
  if (!gemm_split(c, rows, cols)) return false;
  const int M = rows.total, N = cols.total, K = (int)c.ktotal;
  const int Kp = (K + 15) & ~15;
  if ((int64_t)kOzSlices * M * Kp > z.cap_a || (int64_t)kOzSlices * N * Kp > z.cap_b || M > z.cap_r ||
      N > z.cap_c)
    return false;
  __shared__ int s_bad;
  int* koffA = ktab;
  int* koffB = ktab + kTcMaxK;
  if (threadIdx.x == 0) s_bad = 0;
  for (int kk = threadIdx.x; kk < K; kk += blockDim.x) {
    int rem = kk, oa = 0, ob = 0;
    for (int q = c.nk - 1; q >= 0; --q) {
      const int iq = rem % c.k_dim[q];
      rem /= c.k_dim[q];
      oa += iq * c.a_ks[q];
      ob += iq * c.b_ks[q];
    }
    koffA[kk] = oa;
    koffB[kk] = ob;
  }
  __syncthreads();
  // row exponents of A and column exponents of B (one warp per row / column)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < M + N; i += nw) {
    const bool isrow = i < M;
    int op, dummy;
    gemm_axes_offsets(isrow ? rows : cols, isrow ? i : i - M, op, dummy);
    unsigned long long amax = 0;
    for (int kk = lane; kk < K; kk += 32) {
      const double v = isrow ? A[op + koffA[kk]] : B[op + koffB[kk]];
      const unsigned long long ab = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
      amax = ab > amax ? ab : amax;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, amax, o);
      amax = other > amax ? other : amax;
    }
    // NaN / Inf have the all-ones exponent: larger than every finite magnitude
    if (lane == 0 && amax >= 0x7ff0000000000000ull) s_bad = 1;
    if (lane == 0) {
      if (isrow)
        z.rexp[i] = oz_exponent_bits(amax);
      else
        z.cexp[i - M] = oz_exponent_bits(amax);
    }
  }
  __syncthreads();
  if (s_bad) return false;
  // slice A (row-major, k contiguous) and B (column-major, k contiguous), zero-padded to Kp
  const int Kw = Kp >> 1;  // 32-bit words (bf16 pairs) per slice row
  uint32_t* as32w = reinterpret_cast<uint32_t*>(z.as);
  uint32_t* bs32w = reinterpret_cast<uint32_t*>(z.bs);
  for (int side = 0; side < 2; ++side) {
    const GemmAxes& ax = side == 0 ? rows : cols;
    const double* src = side == 0 ? A : B;
    const int* koff = side == 0 ? koffA : koffB;
    const int* ex = side == 0 ? z.rexp : z.cexp;
    uint32_t* dst = side == 0 ? as32w : bs32w;
    const int MN = side == 0 ? M : N;
    for (int64_t e = threadIdx.x; e < (int64_t)MN * Kw; e += blockDim.x) {
      const int i = (int)(e / Kw), kk = 2 * (int)(e - (int64_t)i * Kw);
      int op, dummy;
      gemm_axes_offsets(ax, i, op, dummy);
      const uint64_t b0 = kk < K ? (uint64_t)__double_as_longlong(src[op + koff[kk]]) : 0ull;
      const uint64_t b1 = kk + 1 < K ? (uint64_t)__double_as_longlong(src[op + koff[kk + 1]]) : 0ull;
      const int E = ex[i];
      const uint64_t m0 = oz_fixed48(b0, E), m1 = oz_fixed48(b1, E);
      const uint32_t s0 = (uint32_t)(b0 >> 48) & 0x8000u, s1 = (uint32_t)(b1 >> 48) & 0x8000u;
#pragma unroll
      for (int p = 0; p < kOzSlices; ++p)
        dst[(int64_t)p * MN * Kw + e] = oz_slice_bf16(m0, s0, p) | (oz_slice_bf16(m1, s1, p) << 16);
    }
  }
  __syncthreads();
  const int g = lane >> 2, t = lane & 3;
  const int tilesM = (M + 15) >> 4, tilesN = (N + 7) >> 3;
  const uint32_t* as32 = as32w;
  const uint32_t* bs32 = bs32w;
  for (int tile = warp; tile < tilesM * tilesN; tile += nw) {
    const int tm = tile / tilesN, tn = tile - tm * tilesN;
    const int r0 = tm * 16 + g, r1 = r0 + 8, cb = tn * 8 + g;
    const int rr0 = r0 < M ? r0 : M - 1, rr1 = r1 < M ? r1 : M - 1, ccb = cb < N ? cb : N - 1;
    // running double-float sum of all levels and chunks (FP32 only)
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k0 = 0; k0 < Kp; k0 += kOzChunk) {
      float acc[kOzSlices][4];
#pragma unroll
      for (int L = 0; L < kOzSlices; ++L) acc[L][0] = acc[L][1] = acc[L][2] = acc[L][3] = 0.f;
      const int kend = k0 + kOzChunk < Kp ? k0 + kOzChunk : Kp;
      for (int kk = k0; kk < kend; kk += 16) {
        const int w = (kk >> 1) + t;  // word of columns (kk + 2t, kk + 2t + 1)
        uint32_t af[kOzSlices][4], bf[kOzSlices][2];
#pragma unroll
        for (int p = 0; p < kOzSlices; ++p) {
          const uint32_t* ap = as32 + (int64_t)p * M * Kw;
          const uint32_t* bp = bs32 + (int64_t)p * N * Kw;
          af[p][0] = ap[(int64_t)rr0 * Kw + w];
          af[p][1] = ap[(int64_t)rr1 * Kw + w];
          af[p][2] = ap[(int64_t)rr0 * Kw + w + 4];
          af[p][3] = ap[(int64_t)rr1 * Kw + w + 4];
          bf[p][0] = bp[(int64_t)ccb * Kw + w];
          bf[p][1] = bp[(int64_t)ccb * Kw + w + 4];
        }
#pragma unroll
        for (int p = 0; p < kOzSlices; ++p)
#pragma unroll
          for (int q = 0; q < kOzSlices - p; ++q) mma_bf16_16x8x16(acc[p + q], af[p], bf[q]);
      }
      // level sums are integers below 2^25; scaling by 2^-8(L+2) is exact in FP32
#pragma unroll
      for (int L = 0; L < kOzSlices; ++L) {
        const float sc = __uint_as_float((uint32_t)(127 - 8 * (L + 2)) << 23);
#pragma unroll
        for (int u = 0; u < 4; ++u) oz_two_sum(hi[u], lo[u], __fmul_rn(acc[L][u], sc));
      }
    }
    double out[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) out[u] = oz_f2d(hi[u]) + oz_f2d(lo[u]);
    const int cc0 = tn * 8 + 2 * t, cc1 = cc0 + 1;
    int ccol0 = 0, ccol1 = 0, cr0 = 0, cr1 = 0, dummy;
    if (r0 < M) gemm_axes_offsets(rows, r0, dummy, cr0);
    if (r1 < M) gemm_axes_offsets(rows, r1, dummy, cr1);
    if (cc0 < N) gemm_axes_offsets(cols, cc0, dummy, ccol0);
    if (cc1 < N) gemm_axes_offsets(cols, cc1, dummy, ccol1);
    if (r0 < M && cc0 < N) C[cr0 + ccol0] = oz_scale(out[0], z.rexp[r0] + z.cexp[cc0]);
    if (r0 < M && cc1 < N) C[cr0 + ccol1] = oz_scale(out[1], z.rexp[r0] + z.cexp[cc1]);
    if (r1 < M && cc0 < N) C[cr1 + ccol0] = oz_scale(out[2], z.rexp[r1] + z.cexp[cc0]);
    if (r1 < M && cc1 < N) C[cr1 + ccol1] = oz_scale(out[3], z.rexp[r1] + z.cexp[cc1]);
  }
  __syncthreads();
  return true;
}

}  // namespace ttals
