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
// Slices are stored in mma-fragment order (oz_word_pos), so that one lane
// fetches all six slices of a fragment with three 16-byte loads, and are cut
// with coalesced reads: one thread per row when the operand's rows are
// unit-stride, one warp per row (lanes along the contraction) otherwise.
//
// Operands containing NaN/Inf (or contractions that are not GEMM-shaped or
// too long) return false and the caller falls back to native FP64.
#pragma once

#include <cuda_bf16.h>

#include "ttals_tc.cuh"

namespace ttals {

constexpr int kOzSlices = 6;
constexpr int kOzChunk = 64;  // contraction steps per exact FP32 accumulation chunk
// The fragment-ordered slice layout below (oz_word_pos, the 16-byte slice stores
// and loads) packs 2 words x 6 slices = 12 words = three 16-byte vectors per
// (row, 16-step block, quad lane) chunk; the scratch capacity is kOzSlices
// values per element.  Both must change together.
static_assert(kOzSlices == 6, "the fragment-ordered slice layout is built for exactly 6 slices");

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

struct TcState;  // ttals_tc_gemm.cuh

struct OzScratch {
  uint16_t* as;  // S slices of A, row-major [i][k_pad]   (bf16 bits)
  uint16_t* bs;  // S slices of B, column-major [j][k_pad] (bf16 bits)
  int* rexp;     // E_i
  int* cexp;     // F_j
  int* ktab;     // 2 * kTcMaxK contraction offsets
  int64_t cap_a, cap_b, cap_r, cap_c;  // capacities (elements)
  TcState* tc = nullptr;  // set: GEMM-shaped contractions run on tcgen05 (ttals_tc_gemm.cuh)
};

// C = contraction(A, B) with FP64-level accuracy on the BF16 tensor cores,
// executed by the whole CTA.  ktab: 2 * kTcMaxK ints of shared memory.
//
// Slice layout (both operands): for row i (A) / column j (B), 16-step block kb
// of the contraction and quad lane t, the 12 words [p][h] (slice p, h = 0 for
// k = 16kb + 2t..2t+1, h = 1 for k = 16kb + 2t+8..2t+9) are contiguous, so one
// lane fetches all six slices of its mma fragment with three 128-bit loads.
__device__ __forceinline__ int oz_word_pos(int i, int w, int nkb) {
  const int kb = w >> 3, wl = w & 7;
  return (((i * nkb + kb) << 2) + (wl & 3)) * 12 + (wl >> 2);
}

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
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int Kw = Kp >> 1, nkb = Kp >> 4;
  // exponents and slices, one warp per row (A) / column (B), four in flight
  constexpr int kRows = 4;
  for (int side = 0; side < 2; ++side) {
    const GemmAxes& ax = side == 0 ? rows : cols;
    const double* __restrict__ src = side == 0 ? A : B;
    const int* koff = side == 0 ? koffA : koffB;
    int* ex = side == 0 ? z.rexp : z.cexp;
    uint32_t* dst = reinterpret_cast<uint32_t*>(side == 0 ? z.as : z.bs);
    const int MN = side == 0 ? M : N;
    if (ax.n > 0 && ax.sop[ax.n - 1] == 1 && MN >= (int)blockDim.x) {
      // rows (columns) are unit-stride in the operand and at least one per
      // thread: one thread per row, so that consecutive lanes read consecutive
      // addresses; each thread writes its fragment chunks (12 words) with three
      // 16-byte stores.  Otherwise one warp per row, lanes along the contraction.
      for (int i = threadIdx.x; i < MN; i += blockDim.x) {
        int op, dummy;
        gemm_axes_offsets(ax, i, op, dummy);
        unsigned long long amax = 0;
#pragma unroll 4
        for (int k = 0; k < K; ++k) {
          const unsigned long long b = (unsigned long long)__double_as_longlong(src[op + koff[k]]) & 0x7fffffffffffffffull;
          amax = b > amax ? b : amax;
        }
        if (amax >= 0x7ff0000000000000ull) s_bad = 1;
        const int E = oz_exponent_bits(amax);
        ex[i] = E;
        uint32_t* base = dst + (int64_t)i * nkb * 48;
        for (int kb = 0; kb < nkb; ++kb) {
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            uint32_t wv[12];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const int k0 = 2 * (kb * 8 + t + 4 * h);
              const uint64_t b0 = k0 < K ? (uint64_t)__double_as_longlong(src[op + koff[k0]]) : 0ull;
              const uint64_t b1 = k0 + 1 < K ? (uint64_t)__double_as_longlong(src[op + koff[k0 + 1]]) : 0ull;
              const uint64_t m0 = oz_fixed48(b0, E), m1 = oz_fixed48(b1, E);
              const uint32_t s0 = (uint32_t)(b0 >> 48) & 0x8000u, s1 = (uint32_t)(b1 >> 48) & 0x8000u;
#pragma unroll
              for (int p = 0; p < kOzSlices; ++p) wv[2 * p + h] = oz_slice_bf16(m0, s0, p) | (oz_slice_bf16(m1, s1, p) << 16);
            }
            uint4* q = reinterpret_cast<uint4*>(base + (kb * 4 + t) * 12);
            q[0] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
            q[1] = make_uint4(wv[4], wv[5], wv[6], wv[7]);
            q[2] = make_uint4(wv[8], wv[9], wv[10], wv[11]);
          }
        }
      }
      continue;
    }
    for (int ib = warp * kRows; ib < MN; ib += nw * kRows) {
      int op[kRows];
#pragma unroll
      for (int u = 0; u < kRows; ++u) {
        int dummy;
        op[u] = 0;
        if (ib + u < MN) gemm_axes_offsets(ax, ib + u, op[u], dummy);
      }
      unsigned long long amax[kRows];
#pragma unroll
      for (int u = 0; u < kRows; ++u) amax[u] = 0;
      for (int w = lane; w < Kw; w += 32) {
        const int k0 = 2 * w;
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          if (ib + u < MN) {
            const unsigned long long b0 =
                k0 < K ? (unsigned long long)__double_as_longlong(src[op[u] + koff[k0]]) & 0x7fffffffffffffffull : 0;
            const unsigned long long b1 =
                k0 + 1 < K ? (unsigned long long)__double_as_longlong(src[op[u] + koff[k0 + 1]]) & 0x7fffffffffffffffull
                           : 0;
            const unsigned long long m = b0 > b1 ? b0 : b1;
            amax[u] = m > amax[u] ? m : amax[u];
          }
        }
      }
      int E[kRows];
#pragma unroll
      for (int u = 0; u < kRows; ++u) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const unsigned long long other = __shfl_xor_sync(0xffffffffu, amax[u], o);
          amax[u] = other > amax[u] ? other : amax[u];
        }
        // NaN / Inf have the all-ones exponent: larger than every finite magnitude
        if (amax[u] >= 0x7ff0000000000000ull) s_bad = 1;
        E[u] = oz_exponent_bits(amax[u]);
        if (lane == 0 && ib + u < MN) ex[ib + u] = E[u];
      }
      for (int w = lane; w < Kw; w += 32) {
        const int k0 = 2 * w;
#pragma unroll
        for (int u = 0; u < kRows; ++u) {
          if (ib + u < MN) {
            const uint64_t b0 = k0 < K ? (uint64_t)__double_as_longlong(src[op[u] + koff[k0]]) : 0ull;
            const uint64_t b1 = k0 + 1 < K ? (uint64_t)__double_as_longlong(src[op[u] + koff[k0 + 1]]) : 0ull;
            const uint64_t m0 = oz_fixed48(b0, E[u]), m1 = oz_fixed48(b1, E[u]);
            const uint32_t s0 = (uint32_t)(b0 >> 48) & 0x8000u, s1 = (uint32_t)(b1 >> 48) & 0x8000u;
            uint32_t* d = dst + oz_word_pos(ib + u, w, nkb);
#pragma unroll
            for (int p = 0; p < kOzSlices; ++p) d[2 * p] = oz_slice_bf16(m0, s0, p) | (oz_slice_bf16(m1, s1, p) << 16);
          }
        }
      }
    }
  }
  __syncthreads();
  if (s_bad) return false;
  const int g = lane >> 2, t = lane & 3;
  const int tilesM = (M + 15) >> 4, tilesN = (N + 7) >> 3;
  const uint4* as4 = reinterpret_cast<const uint4*>(z.as);
  const uint4* bs4 = reinterpret_cast<const uint4*>(z.bs);
  for (int tile = warp; tile < tilesM * tilesN; tile += nw) {
    const int tm = tile / tilesN, tn = tile - tm * tilesN;
    const int r0 = tm * 16 + g, r1 = r0 + 8, cb = tn * 8 + g;
    const int rr0 = r0 < M ? r0 : M - 1, rr1 = r1 < M ? r1 : M - 1, ccb = cb < N ? cb : N - 1;
    // running double-float sum of all levels and chunks (FP32 only)
    float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    for (int kb0 = 0; kb0 < nkb; kb0 += kOzChunk / 16) {
      float acc[kOzSlices][4];
#pragma unroll
      for (int L = 0; L < kOzSlices; ++L) acc[L][0] = acc[L][1] = acc[L][2] = acc[L][3] = 0.f;
      const int kbe = kb0 + kOzChunk / 16 < nkb ? kb0 + kOzChunk / 16 : nkb;
      for (int kb = kb0; kb < kbe; ++kb) {
        const uint4* pa0 = as4 + (((int64_t)rr0 * nkb + kb) * 4 + t) * 3;
        const uint4* pa1 = as4 + (((int64_t)rr1 * nkb + kb) * 4 + t) * 3;
        const uint4* pb = bs4 + (((int64_t)ccb * nkb + kb) * 4 + t) * 3;
        uint32_t wa0[12], wa1[12], wb[12];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const uint4 x0 = pa0[q], x1 = pa1[q], y = pb[q];
          wa0[4 * q] = x0.x; wa0[4 * q + 1] = x0.y; wa0[4 * q + 2] = x0.z; wa0[4 * q + 3] = x0.w;
          wa1[4 * q] = x1.x; wa1[4 * q + 1] = x1.y; wa1[4 * q + 2] = x1.z; wa1[4 * q + 3] = x1.w;
          wb[4 * q] = y.x; wb[4 * q + 1] = y.y; wb[4 * q + 2] = y.z; wb[4 * q + 3] = y.w;
        }
        uint32_t af[kOzSlices][4], bf[kOzSlices][2];
#pragma unroll
        for (int p = 0; p < kOzSlices; ++p) {
          af[p][0] = wa0[2 * p];
          af[p][1] = wa1[2 * p];
          af[p][2] = wa0[2 * p + 1];
          af[p][3] = wa1[2 * p + 1];
          bf[p][0] = wb[2 * p];
          bf[p][1] = wb[2 * p + 1];
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
