// Tensor-core contraction for the FP32 inner Krylov solves of the batch kernel.
//
// Every phase of the local-operator apply is a GEMM in disguise: each output
// axis is indexed by exactly one operand (stride 0 in the other), so the
// output splits into M axes (rows, from A) and N axes (columns, from B) and the
// contraction axes form K.  cta_gemm_tf32x3 runs such a contraction on the
// tensor cores with warp-level mma.sync m16n8k8 TF32 instructions and the
// three-product split a*b ~ ah*bh + ah*bl + al*bh (each FP32 operand split into
// a TF32 head and a TF32 tail), which keeps the product accurate to about FP32
// (the inner solver needs ~1e-6, FP32 rounding), while the residual and the
// solution stay FP64 in the surrounding refinement loop.
//
// Operands are gathered straight from global memory (L1/L2 resident at these
// sizes) through per-row / per-column offsets and a per-K offset table in
// shared memory; no layout change of the Krylov vectors is needed.
#pragma once

#include "ttals_device.cuh"

namespace ttals {

constexpr int kTcMaxK = 1024;  // largest contraction length handled (offset tables in smem)

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32_16x8x8(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Row / column decomposition of a contraction's output axes.
struct GemmAxes {
  int n;                    // number of axes
  int dim[kMaxOut];
  uint32_t mag[kMaxOut];
  int shf[kMaxOut];
  int sop[kMaxOut];         // stride in the operand (A for rows, B for columns)
  int sc[kMaxOut];          // stride in C
  int total;
};

__host__ __device__ __forceinline__ void gemm_axes_offsets(const GemmAxes& g, int idx, int& op, int& co) {
  uint32_t rem = (uint32_t)idx;
  int o = 0, c = 0;
#pragma unroll
  for (int q = kMaxOut - 1; q >= 0; --q) {
    if (q < g.n) {
      const uint32_t qq = fast_div(rem, g.mag[q], g.shf[q]);
      const int iq = (int)(rem - qq * (uint32_t)g.dim[q]);
      rem = qq;
      o += iq * g.sop[q];
      c += iq * g.sc[q];
    }
  }
  op = o;
  co = c;
}

// Splits `c` into row (A) and column (B) axes; false if some output axis is
// indexed by both operands or the contraction is too long for the tables.
__host__ __device__ __forceinline__ bool gemm_split(const Contraction& c, GemmAxes& rows, GemmAxes& cols) {
  rows.n = cols.n = 0;
  rows.total = cols.total = 1;
  if (c.ktotal > kTcMaxK || c.ktotal < 1) return false;
  for (int q = 0; q < c.nout; ++q) {
    GemmAxes* g;
    int s;
    if (c.b_os[q] == 0) {
      g = &rows;
      s = c.a_os[q];
    } else if (c.a_os[q] == 0) {
      g = &cols;
      s = c.b_os[q];
    } else {
      return false;
    }
    const int k = g->n++;
    g->dim[k] = c.out_dim[q];
    g->mag[k] = c.out_mag[q];
    g->shf[k] = c.out_shf[q];
    g->sop[k] = s;
    g->sc[k] = c.c_os[q];
    g->total *= c.out_dim[q];
  }
  return rows.n > 0 && cols.n > 0;
}

// C = contraction(A, B) on the tensor cores, executed by the whole CTA (G:
// by the calling group of the two-group form, ttals_device.cuh).
// ktab: 2 * kTcMaxK ints of shared memory.  Returns false (nothing done) when
// the contraction is not GEMM-shaped; the caller then uses the SIMT path.
template <bool G = false>
__device__ __forceinline__ bool cta_gemm_tf32x3(const Contraction& c, const float* __restrict__ A,
                                                const float* __restrict__ B, float* __restrict__ C, int* ktab) {
  GemmAxes rows, cols;
  if (!gemm_split(c, rows, cols)) return false;
  const int M = rows.total, N = cols.total, K = (int)c.ktotal;
  int* koffA = ktab;
  int* koffB = ktab + kTcMaxK;
  for (int kk = gtid<G>(); kk < K; kk += gsize<G>()) {
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
  gsync<G>();
  const int lane = gtid<G>() & 31, warp = gtid<G>() >> 5, nw = gsize<G>() >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tilesM = (M + 15) >> 4, tilesN = (N + 7) >> 3;
  for (int tile = warp; tile < tilesM * tilesN; tile += nw) {
    const int tm = tile / tilesN, tn = tile - tm * tilesN;
    const int r0 = tm * 16 + g, r1 = r0 + 8;
    const int cb = tn * 8 + g, cc0 = tn * 8 + 2 * t, cc1 = cc0 + 1;
    const bool v0 = r0 < M, v1 = r1 < M, vb = cb < N;
    int ar0 = 0, ar1 = 0, cr0 = 0, cr1 = 0, bc = 0, ccol0 = 0, ccol1 = 0, dummy;
    if (v0) gemm_axes_offsets(rows, r0, ar0, cr0);
    if (v1) gemm_axes_offsets(rows, r1, ar1, cr1);
    if (vb) gemm_axes_offsets(cols, cb, bc, dummy);
    if (cc0 < N) gemm_axes_offsets(cols, cc0, dummy, ccol0);
    if (cc1 < N) gemm_axes_offsets(cols, cc1, dummy, ccol1);
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int kk = 0; kk < K; kk += 8) {
      const int k0 = kk + t, k1 = k0 + 4;
      const bool vk0 = k0 < K, vk1 = k1 < K;
      const int oa0 = vk0 ? koffA[k0] : 0, oa1 = vk1 ? koffA[k1] : 0;
      const int ob0 = vk0 ? koffB[k0] : 0, ob1 = vk1 ? koffB[k1] : 0;
      const float x0 = (v0 && vk0) ? A[ar0 + oa0] : 0.f;
      const float x1 = (v1 && vk0) ? A[ar1 + oa0] : 0.f;
      const float x2 = (v0 && vk1) ? A[ar0 + oa1] : 0.f;
      const float x3 = (v1 && vk1) ? A[ar1 + oa1] : 0.f;
      const float y0 = (vb && vk0) ? B[bc + ob0] : 0.f;
      const float y1 = (vb && vk1) ? B[bc + ob1] : 0.f;
      uint32_t ah[4], al[4], bh[2], bl[2];
      ah[0] = tf32_bits(x0);
      ah[1] = tf32_bits(x1);
      ah[2] = tf32_bits(x2);
      ah[3] = tf32_bits(x3);
      al[0] = tf32_bits(x0 - __uint_as_float(ah[0]));
      al[1] = tf32_bits(x1 - __uint_as_float(ah[1]));
      al[2] = tf32_bits(x2 - __uint_as_float(ah[2]));
      al[3] = tf32_bits(x3 - __uint_as_float(ah[3]));
      bh[0] = tf32_bits(y0);
      bh[1] = tf32_bits(y1);
      bl[0] = tf32_bits(y0 - __uint_as_float(bh[0]));
      bl[1] = tf32_bits(y1 - __uint_as_float(bh[1]));
      mma_tf32_16x8x8(acc, al, bh);
      mma_tf32_16x8x8(acc, ah, bl);
      mma_tf32_16x8x8(acc, ah, bh);
    }
    if (v0 && cc0 < N) C[cr0 + ccol0] = acc[0];
    if (v0 && cc1 < N) C[cr0 + ccol1] = acc[1];
    if (v1 && cc0 < N) C[cr1 + ccol0] = acc[2];
    if (v1 && cc1 < N) C[cr1 + ccol1] = acc[3];
  }
  gsync<G>();
  return true;
}

}  // namespace ttals
