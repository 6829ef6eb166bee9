// CTA-level GEMM-shaped contractions on the fifth-generation tensor cores.
//
// Two flavours, both staging their operands straight from the strided
// contraction descriptors (ttals_desc.cuh, split into row / column /
// contraction axes by gemm_split) into shared-memory tiles in the canonical
// K-major layout (ttals_umma.cuh), with the accumulators in tensor memory:
//
// * cta_gemm_oz_tc: FP64-accurate C = A B from FP64 operands (emulated FP64,
//   Ozaki-style slicing as in ttals_ozaki.cuh): each row of A (column of B) is
//   scaled by its power-of-two maximum and cut into 6 slices of 8 bits, exact
//   in BF16.  The 21 slice products with p + q < 6 run as tcgen05.mma
//   kind::f16 (M = 128, N = 64, K = 16) into one FP32 accumulator per level
//   L = p + q (6 x 64 TMEM columns).  Level sums are integers; every 64
//   contraction steps they are drained: converted to integers, combined in
//   64-bit fixed point (level L weighted by 2^(8 (5 - L))) and added to a
//   per-thread running sum, which is finally turned into FP64 by bit
//   manipulation with the scale 2^(E_i + F_j - 56) folded into the exponent.
//   No FP64 instruction is executed (FP64 runs at 2 FMA/clk/SM on this part).
// * cta_gemm_tf32_tc: FP32 C = A B from FP32 operands with the 3xTF32 split
//   a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, three tcgen05.mma kind::tf32 into
//   one FP32 accumulator (N up to 256 columns per tile).
//
// One thread issues the MMAs and commits them to an mbarrier; every thread
// waits on it (bounded), then reads its accumulator lane (row) back.
#pragma once

#include "ttals_ozaki.cuh"
#include "ttals_umma.cuh"

namespace ttals {

// A kernel that contains tcgen05 instructions runs one CTA per SM.  That CTA
// either runs two independent solves, one per thread group (G = true:
// kGroupThreads threads, ttals_device.cuh), each holding half of the SM's 512
// TMEM columns and its own operand tiles, or one solve on all of it (G =
// false: the whole 512-thread CTA).  A group drains its accumulators with
// 128-lane sub-groups side by side.  All functions here work on the calling
// group.
constexpr int kTcM = 128;                        // rows per tile (TMEM lanes)
constexpr int kTcKC = 32;                        // contraction elements per staged chunk
constexpr int kTcOzDrain = 2;                    // chunks accumulated in TMEM between drains (64 steps)
constexpr uint32_t kTcCtaTmemCols = 512;         // TMEM columns allocated by the CTA (all of the SM's)
constexpr int kTcCtaThreads = 512;               // threads of a tensor-core CTA

template <bool G>
struct TcCfg {
  static constexpr int kThreads = G ? kGroupThreads : kTcCtaThreads;  // threads of the group
  static constexpr int kSub = kThreads / 128;                          // 128-lane drain sub-groups
  static constexpr int kOzNT = 16 * kSub;       // columns per emulated-FP64 tile: 16 per sub-group
  static constexpr int kF32NT = G ? 128 : 256;  // columns per 3xTF32 tile
  static constexpr uint32_t kTmemCols = G ? 256 : 512;  // TMEM columns of the group
  static constexpr int kTileBytes = G ? 64 * 1024 : 96 * 1024;  // operand tiles of the group
  // per-tile index tables after the tiles: operand offset, output offset and
  // exponent of each row (kTcM) and column (kF32NT) of the current tile
  static constexpr int kTabBytes = 3 * 4 * (kTcM + kF32NT);
  static constexpr int kSmemBytes = kTileBytes + (kTabBytes + 1023) / 1024 * 1024;
  static_assert(kOzSlices * kOzNT <= (int)kTmemCols, "level accumulators must fit the group's TMEM");
  static_assert(kF32NT <= (int)kTmemCols, "3xTF32 accumulator must fit the group's TMEM");
  static_assert(kOzSlices * kTcM * kTcKC * 2 + kOzSlices * kOzNT * kTcKC * 2 <= kTileBytes, "Ozaki tiles");
  static_assert(2 * kTcM * kTcKC * 4 + 2 * kF32NT * kTcKC * 4 <= kTileBytes, "3xTF32 tiles");
};

// Per-group tensor-core state (lives in shared memory).
struct TcState {
  unsigned char* tiles;  // TcCfg::kSmemBytes, 1024-byte aligned: operand tiles, then the index tables
  uint32_t tmem;         // TMEM base of the group's TcCfg::kTmemCols columns
  uint32_t phase;        // parity of the next MMA completion
  int status;            // ST_OK; ST_TIMEOUT once a completion wait gave up (no further MMAs)
  uint64_t bar;          // mbarrier signalled by tcgen05.commit
  unsigned long long gemms;      // contractions completed on the tensor cores
  unsigned long long fallbacks;  // GEMM-shaped contractions that took the SIMT path instead
};

// The index tables of the current tile (shared memory after the operand tiles).
struct TcTables {
  int *rop, *rco, *rex;  // rows: operand offset (-1 beyond the matrix), output offset, exponent
  int *cop, *cco, *cex;  // columns: the same
};
template <bool G>
__device__ __forceinline__ TcTables tc_tables(const TcState& tc) {
  int* t = reinterpret_cast<int*>(tc.tiles + TcCfg<G>::kTileBytes);
  return TcTables{t, t + kTcM, t + 2 * kTcM, t + 3 * kTcM, t + 3 * kTcM + TcCfg<G>::kF32NT, t + 3 * kTcM + 2 * TcCfg<G>::kF32NT};
}

// int64 fixed point v * 2^e -> FP64, by bit manipulation (round to nearest even).
__device__ __forceinline__ double tc_i64_to_f64(long long v, int e) {
  if (v == 0) return 0.0;
  const uint64_t sign = v < 0 ? 0x8000000000000000ull : 0ull;
  const uint64_t m = v < 0 ? (uint64_t)0 - (uint64_t)v : (uint64_t)v;
  const int msb = 63 - __clzll((long long)m);
  uint64_t mant;
  int ex = msb;
  if (msb > 52) {
    const int sh = msb - 52;
    const uint64_t rem = m & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    mant = m >> sh;
    if (rem > half || (rem == half && (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++ex;
      }
    }
  } else {
    mant = m << (52 - msb);
  }
  const int be = ex + e + 1023;
  if (be <= 0 || be >= 2047) {  // subnormal or overflow: rare, let FP64 handle it
    const double dv = sign ? -(double)m : (double)m;
    return ldexp(dv, e);
  }
  return __longlong_as_double((long long)(sign | ((uint64_t)be << 52) | (mant & 0xfffffffffffffull)));
}

// Contraction-offset tables koffA / koffB of c (smem, 2 * kTcMaxK ints).
template <bool G>
__device__ __forceinline__ void tc_k_tables(const Contraction& c, int* ktab) {
  const int K = (int)c.ktotal;
  for (int kk = gtid<G>(); kk < K; kk += gsize<G>()) {
    int rem = kk, oa = 0, ob = 0;
    for (int q = c.nk - 1; q >= 0; --q) {
      const int iq = rem % c.k_dim[q];
      rem /= c.k_dim[q];
      oa += iq * c.a_ks[q];
      ob += iq * c.b_ks[q];
    }
    ktab[kk] = oa;
    ktab[kTcMaxK + kk] = ob;
  }
}

// Decode rows [r0, r0 + cnt) of an axis set once per tile: operand offset
// (-1 for rows >= valid) and output offset.
template <bool G>
__device__ __forceinline__ void tc_axis_table(const GemmAxes& ax, int r0, int cnt, int valid, int* op, int* co) {
  for (int i = gtid<G>(); i < cnt; i += gsize<G>()) {
    int o = -1, c = 0;
    if (r0 + i < valid) gemm_axes_offsets(ax, r0 + i, o, c);
    op[i] = o;
    co[i] = c;
  }
}

// E[i] with |x| < 2^E[i] over the contraction of table row i; flags
// non-finite values.  One warp takes 8 rows at a time with its lanes along
// the contraction (8 independent loads in flight per lane).
template <bool G>
__device__ __forceinline__ void tc_table_exponents(const double* __restrict__ src, const int* koff, int K,
                                                   const int* op, int cnt, int* E, int* bad) {
  constexpr int kRows = 8;
  const int lane = gtid<G>() & 31, warp = gtid<G>() >> 5, nw = gsize<G>() >> 5;
  for (int ib = warp * kRows; ib < cnt; ib += nw * kRows) {
    int o[kRows];
    unsigned long long amax[kRows];
#pragma unroll
    for (int u = 0; u < kRows; ++u) {
      o[u] = ib + u < cnt ? op[ib + u] : -1;
      amax[u] = 0;
    }
    for (int k = lane; k < K; k += 32) {
      const int ko = koff[k];
#pragma unroll
      for (int u = 0; u < kRows; ++u) {
        if (o[u] >= 0) {
          const unsigned long long b =
              (unsigned long long)__double_as_longlong(src[o[u] + ko]) & 0x7fffffffffffffffull;
          amax[u] = b > amax[u] ? b : amax[u];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < kRows; ++u) {
#pragma unroll
      for (int sft = 16; sft > 0; sft >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, amax[u], sft);
        amax[u] = other > amax[u] ? other : amax[u];
      }
      if (lane == 0 && ib + u < cnt) {
        // NaN / Inf have the all-ones exponent: larger than every finite magnitude
        if (amax[u] >= 0x7ff0000000000000ull) *bad = 1;
        E[ib + u] = oz_exponent_bits(amax[u]);
      }
    }
  }
}

// Rows [0, rows) of the tile (operand offsets op, exponents E) x contraction
// [k0, k0 + kTcKC) of an FP64 operand into kOzSlices BF16 slice tiles (tile p
// at base + p * slice_bytes); rows with op < 0 and k >= K are zero.  One work
// item = one row x 8 contraction steps (one 16-byte core-matrix row per slice);
// consecutive threads take consecutive rows.
template <bool G>
__device__ __forceinline__ void tc_oz_stage(const double* __restrict__ src, const int* koff, int K, int k0,
                                            const int* op, const int* E, int rows, unsigned char* base,
                                            uint32_t slice_bytes) {
  constexpr int kbytes = kTcKC * 2;
  const int items = rows * (kTcKC / 8);
  for (int it = gtid<G>(); it < items; it += gsize<G>()) {
    const int cc = it / rows, r = it - cc * rows;
    const int o = op[r];
    uint32_t w[kOzSlices][4];
#pragma unroll
    for (int p = 0; p < kOzSlices; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
    if (o >= 0) {
      const int e = E[r];
      uint64_t b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + cc * 8 + u;
        b[u] = k < K ? (uint64_t)__double_as_longlong(src[o + koff[k]]) : 0ull;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const uint64_t mag = oz_fixed48(b[u], e);
        const uint32_t sg = (uint32_t)(b[u] >> 48) & 0x8000u;
#pragma unroll
        for (int p = 0; p < kOzSlices; ++p) w[p][u >> 1] |= oz_slice_bf16(mag, sg, p) << (16 * (u & 1));
      }
    }
    const uint32_t off = umma::tile_off(r, cc * 8, 2, kbytes);
#pragma unroll
    for (int p = 0; p < kOzSlices; ++p)
      *reinterpret_cast<uint4*>(base + p * slice_bytes + off) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
  }
}

// Completion waits of one GEMM call: every thread tracks the mbarrier phase in
// a register (all threads wait for the same commits in the same order) and
// one barrier per wait publishes whether any thread gave up.
struct TcWaiter {
  uint32_t phase;
  int* fail;  // shared flag, cleared at the start of the call
};
template <bool G>
__device__ __forceinline__ TcWaiter tc_waiter_begin(TcState& tc) {
  __shared__ int s_fail[2];
  int* f = &s_fail[gidx<G>()];
  if (gtid<G>() == 0) *f = 0;
  return TcWaiter{tc.phase, f};
}
// Wait for the MMAs committed last (all threads); false (status set) if the wait gave up.
template <bool G>
__device__ __forceinline__ bool tc_wait(TcState& tc, TcWaiter& w) {
  if (!umma::mbar_wait(&tc.bar, w.phase)) *w.fail = 1;
  w.phase ^= 1u;
  gsync<G>();
  umma::fence_after_sync();
  if (*w.fail) {
    if (gtid<G>() == 0) tc.status = ST_TIMEOUT;
    return false;
  }
  return true;
}
// End of a GEMM call: the parity of the next completion goes back to the state.
template <bool G>
__device__ __forceinline__ void tc_waiter_end(TcState& tc, const TcWaiter& w) {
  gsync<G>();
  if (gtid<G>() == 0) tc.phase = w.phase;
  gsync<G>();
}

// shared-memory operand writes -> visible to the tensor cores; TMEM reads done
template <bool G>
__device__ __forceinline__ void tc_publish() {
  umma::fence_smem_to_async();
  umma::fence_before_sync();
  gsync<G>();
  umma::fence_after_sync();
}

// C = contraction(A, B) with FP64-level accuracy; false when not GEMM-shaped,
// non-finite, or the tensor cores are unusable (the caller then runs the FP64
// SIMT path, which overwrites whatever was written).
template <bool G>
__device__ __forceinline__ bool cta_gemm_oz_tc(const Contraction& c, const double* __restrict__ A,
                                               const double* __restrict__ B, double* __restrict__ C,
                                               const OzScratch& z, int* ktab, TcState& tc) {
  (void)z;
  GemmAxes rows, cols;
  // a group of TcCfg::kThreads threads: kSub 128-thread sub-groups, each draining 16 of the tile's columns
  if (tc.status != ST_OK || !gemm_split(c, rows, cols)) return false;
  const int M = rows.total, N = cols.total, K = (int)c.ktotal;
  __shared__ int s_bad_g[2];
  int& s_bad = s_bad_g[gidx<G>()];
  if (gtid<G>() == 0) s_bad = 0;
  tc_k_tables<G>(c, ktab);
  const int* koffA = ktab;
  const int* koffB = ktab + kTcMaxK;
  const TcTables T = tc_tables<G>(tc);
  constexpr uint32_t a_slice = kTcM * kTcKC * 2, b_slice = TcCfg<G>::kOzNT * kTcKC * 2;
  constexpr uint32_t sbo = (kTcKC * 2 / 16) * 128;
  unsigned char* ta = tc.tiles;
  unsigned char* tb = tc.tiles + kOzSlices * a_slice;
  const int nK = (K + kTcKC - 1) / kTcKC;
  const int nwin = (nK + kTcOzDrain - 1) / kTcOzDrain;
  const int sh = nwin <= 1 ? 0 : 32 - __clz(nwin - 1);  // 2^sh >= windows: the int64 sum cannot overflow
  const int warp = gtid<G>() >> 5, lane = gtid<G>() & 31, q4 = warp & 3;
  const int hh = warp >> 2;  // this thread's 16-column block of the tile
  const int rl = 32 * q4 + lane;  // this thread's row of the tile (TMEM lane)
  TcWaiter wt = tc_waiter_begin<G>(tc);
  const bool one_n = N <= TcCfg<G>::kOzNT;  // column tables and exponents stay valid across row tiles
  for (int m0 = 0; m0 < M; m0 += kTcM) {
    const bool cols_now = one_n && m0 == 0;  // the single column tile, decoded once
    tc_axis_table<G>(rows, m0, kTcM, M, T.rop, T.rco);
    if (cols_now) tc_axis_table<G>(cols, 0, (N + 15) & ~15, N, T.cop, T.cco);
    gsync<G>();
    tc_table_exponents<G>(A, koffA, K, T.rop, kTcM, T.rex, &s_bad);
    if (cols_now) tc_table_exponents<G>(B, koffB, K, T.cop, (N + 15) & ~15, T.cex, &s_bad);
    for (int n0 = 0; n0 < N; n0 += TcCfg<G>::kOzNT) {
      const int ncols = N - n0 < TcCfg<G>::kOzNT ? N - n0 : TcCfg<G>::kOzNT;
      const int ntile = (ncols + 15) & ~15;
      const uint32_t id = umma::idesc(umma::kFmtBF16, kTcM, ntile);
      if (!one_n) {
        gsync<G>();  // the previous tile's store has read the column tables
        tc_axis_table<G>(cols, n0, ntile, N, T.cop, T.cco);
        gsync<G>();
        tc_table_exponents<G>(B, koffB, K, T.cop, ntile, T.cex, &s_bad);
      }
      gsync<G>();
      if (s_bad) {
        tc_waiter_end<G>(tc, wt);
        return false;
      }
      long long acc[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) acc[j] = 0;
      for (int kc = 0; kc < nK; ++kc) {
        if (nK > 1 || n0 == 0) tc_oz_stage<G>(A, koffA, K, kc * kTcKC, T.rop, T.rex, kTcM, ta, a_slice);
        tc_oz_stage<G>(B, koffB, K, kc * kTcKC, T.cop, T.cex, ntile, tb, b_slice);
        tc_publish<G>();
        if (gtid<G>() == 0) {
          const bool wstart = (kc % kTcOzDrain) == 0;
          const uint32_t a0 = umma::smem_u32(ta), b0 = umma::smem_u32(tb);
          uint64_t da[kOzSlices], db[kOzSlices];
#pragma unroll
          for (int p = 0; p < kOzSlices; ++p) {
            da[p] = umma::sdesc(a0 + p * a_slice, 128, sbo);
            db[p] = umma::sdesc(b0 + p * b_slice, 128, sbo);
          }
#pragma unroll
          for (int ks = 0; ks < kTcKC / 16; ++ks)
#pragma unroll
            for (int p = 0; p < kOzSlices; ++p)
#pragma unroll
              for (int q = 0; q < kOzSlices - p; ++q) {
                // the start-address field counts 16-byte units: +16 per 256-byte K step
                const uint32_t acc_in = (wstart && ks == 0 && p == 0) ? 0u : 1u;
                umma::mma_f16(umma::taddr(tc.tmem, 0, (p + q) * TcCfg<G>::kOzNT), da[p] + 16u * ks, db[q] + 16u * ks, id,
                              acc_in);
              }
          umma::commit(&tc.bar);
        }
        if (!tc_wait<G>(tc, wt)) return false;
        if ((kc % kTcOzDrain) == kTcOzDrain - 1 || kc == nK - 1) {
          if (hh * 16 < ntile) {  // warp-uniform
#pragma unroll
            for (int L = 0; L < kOzSlices; ++L) {
              uint32_t v[16];
              umma::ld16(umma::taddr(tc.tmem, 32 * q4, L * TcCfg<G>::kOzNT + hh * 16), v);
              umma::ld_wait();
              const int lsh = 8 * (kOzSlices - 1 - L) - sh;
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                const long long t = (long long)__float2int_rn(__uint_as_float(v[j]));
                acc[j] += lsh >= 0 ? (t << lsh) : (t >> (-lsh));
              }
            }
          }
          umma::fence_before_sync();
        }
      }
      // results of this tile: row m0 + rl, columns n0 + 16 hh + j
      if (T.rop[rl] >= 0 && hh * 16 < ncols) {
        const int cr = T.rco[rl];
        const int er = T.rex[rl] - 8 * (kOzSlices + 1) + sh;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int cl = hh * 16 + j;
          if (cl < ncols) C[cr + T.cco[cl]] = tc_i64_to_f64(acc[j], er + T.cex[cl]);
        }
      }
      gsync<G>();
    }
  }
  tc_waiter_end<G>(tc, wt);
  return true;
}

// Rows [0, rows) of the tile (operand offsets op) x contraction [k0, k0 + kTcKC)
// of an FP32 operand as TF32 head and tail tiles (hi at base, lo at
// base + half_bytes); rows with op < 0 and k >= K are zero.
template <bool G>
__device__ __forceinline__ void tc_tf32_stage(const float* __restrict__ src, const int* koff, int K, int k0,
                                              const int* op, int rows, unsigned char* base, uint32_t half_bytes) {
  constexpr int kbytes = kTcKC * 4;
  const int items = rows * (kTcKC / 4);
  for (int it = gtid<G>(); it < items; it += gsize<G>()) {
    const int cc = it / rows, r = it - cc * rows;
    const int o = op[r];
    uint32_t hi[4] = {0u, 0u, 0u, 0u}, lo[4] = {0u, 0u, 0u, 0u};
    if (o >= 0) {
      float x[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = k0 + cc * 4 + u;
        x[u] = k < K ? src[o + koff[k]] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        hi[u] = tf32_bits(x[u]);
        lo[u] = tf32_bits(x[u] - __uint_as_float(hi[u]));
      }
    }
    const uint32_t off = umma::tile_off(r, cc * 4, 4, kbytes);
    *reinterpret_cast<uint4*>(base + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(base + half_bytes + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
}

// C = contraction(A, B) in FP32 (3xTF32) on the tensor cores; false when not
// GEMM-shaped or the tensor cores are unusable.
template <bool G>
__device__ __forceinline__ bool cta_gemm_tf32_tc(const Contraction& c, const float* __restrict__ A,
                                                 const float* __restrict__ B, float* __restrict__ C, int* ktab,
                                                 TcState& tc) {
  GemmAxes rows, cols;
  if (tc.status != ST_OK || !gemm_split(c, rows, cols)) return false;
  const int M = rows.total, N = cols.total, K = (int)c.ktotal;
  tc_k_tables<G>(c, ktab);
  const int* koffA = ktab;
  const int* koffB = ktab + kTcMaxK;
  const TcTables T = tc_tables<G>(tc);
  constexpr uint32_t a_half = kTcM * kTcKC * 4, b_half = TcCfg<G>::kF32NT * kTcKC * 4;
  constexpr uint32_t sbo = (kTcKC * 4 / 16) * 128;
  unsigned char* ta = tc.tiles;
  unsigned char* tb = tc.tiles + 2 * a_half;
  const int nK = (K + kTcKC - 1) / kTcKC;
  const int warp = gtid<G>() >> 5, lane = gtid<G>() & 31, q4 = warp & 3;
  const int halves = gsize<G>() >> 7, grp = warp >> 2;
  const int rl = 32 * q4 + lane;
  TcWaiter wt = tc_waiter_begin<G>(tc);
  const bool one_n = N <= TcCfg<G>::kF32NT;
  for (int m0 = 0; m0 < M; m0 += kTcM) {
    tc_axis_table<G>(rows, m0, kTcM, M, T.rop, T.rco);
    for (int n0 = 0; n0 < N; n0 += TcCfg<G>::kF32NT) {
      const int ncols = N - n0 < TcCfg<G>::kF32NT ? N - n0 : TcCfg<G>::kF32NT;
      const int ntile = (ncols + 15) & ~15;
      const uint32_t id = umma::idesc(umma::kFmtTF32, kTcM, ntile);
      if (!one_n || m0 == 0) tc_axis_table<G>(cols, n0, ntile, N, T.cop, T.cco);
      gsync<G>();
      for (int kc = 0; kc < nK; ++kc) {
        if (nK > 1 || n0 == 0) tc_tf32_stage<G>(A, koffA, K, kc * kTcKC, T.rop, kTcM, ta, a_half);
        tc_tf32_stage<G>(B, koffB, K, kc * kTcKC, T.cop, ntile, tb, b_half);
        tc_publish<G>();
        if (gtid<G>() == 0) {
          const uint32_t a0 = umma::smem_u32(ta), b0 = umma::smem_u32(tb);
          const uint32_t d = umma::taddr(tc.tmem, 0, 0);
          const uint64_t ah = umma::sdesc(a0, 128, sbo), al = umma::sdesc(a0 + a_half, 128, sbo);
          const uint64_t bh = umma::sdesc(b0, 128, sbo), bl = umma::sdesc(b0 + b_half, 128, sbo);
#pragma unroll
          for (int ks = 0; ks < kTcKC / 8; ++ks) {
            const uint64_t st = 16u * ks;  // start-address field: 256 bytes per K step
            umma::mma_tf32(d, al + st, bh + st, id, (kc == 0 && ks == 0) ? 0u : 1u);
            umma::mma_tf32(d, ah + st, bl + st, id, 1u);
            umma::mma_tf32(d, ah + st, bh + st, id, 1u);
          }
          umma::commit(&tc.bar);
        }
        if (!tc_wait<G>(tc, wt)) return false;
      }
      const bool live = T.rop[rl] >= 0;
      const int cr = T.rco[rl];
      // each 128-thread group drains every other 16-column block
      for (int cb = grp * 16; cb < ntile; cb += 16 * halves) {
        uint32_t v[16];
        umma::ld16(umma::taddr(tc.tmem, 32 * q4, cb), v);
        umma::ld_wait();
        if (live) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int cl = cb + j;
            if (cl < ncols) C[cr + T.cco[cl]] = __uint_as_float(v[j]);
          }
        }
      }
      umma::fence_before_sync();
      gsync<G>();
    }
  }
  tc_waiter_end<G>(tc, wt);
  return true;
}

}  // namespace ttals
