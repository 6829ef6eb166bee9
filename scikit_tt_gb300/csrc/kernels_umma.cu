// Self-test of the tcgen05 building blocks (ttals_umma.cuh): one CTA computes
// D = A * B^T for an M = 128 row tile with BF16 (kind::f16) or TF32
// (kind::tf32) operands staged in shared memory in the canonical K-major
// layout and the FP32 accumulator in tensor memory.  It pins the descriptor
// and layout encodings against a host reference before the batch kernel
// relies on them.
#include "ttals_batch.h"
#include "ttals_internal.h"
#include "ttals_umma.cuh"

namespace ttals {

namespace {

__device__ __forceinline__ uint16_t bf16_bits_rn(float x) {
  // round to nearest even on the upper 16 bits (finite inputs)
  const uint32_t u = __float_as_uint(x);
  return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}

__device__ __forceinline__ uint32_t tf32_bits_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

}  // namespace

// A: M x K row-major, Bt: N x K row-major (B^T), C: M x N row-major.
// kind 0: BF16 inputs, kind 1: TF32 inputs.  status[0] = ST_OK or ST_TIMEOUT.
__global__ void __launch_bounds__(128) umma_selftest_kernel(int kind, int N, int K, const float* __restrict__ A,
                                                            const float* __restrict__ Bt, float* __restrict__ C,
                                                            int* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tbase;
  constexpr int M = 128;
  const int esz = kind == 0 ? 2 : 4;
  const int kbytes = K * esz;
  unsigned char* ta = smem;
  unsigned char* tb = smem + (size_t)M * kbytes;
  const uint32_t ncols = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) umma::tmem_alloc(&tbase, ncols);
  if (threadIdx.x == 0) umma::mbar_init(&bar, 1);
  for (int idx = threadIdx.x; idx < M * K; idx += blockDim.x) {
    const int r = idx / K, k = idx - r * K;
    const float v = A[idx];
    unsigned char* p = ta + umma::tile_off(r, k, esz, kbytes);
    if (kind == 0)
      *reinterpret_cast<uint16_t*>(p) = bf16_bits_rn(v);
    else
      *reinterpret_cast<uint32_t*>(p) = tf32_bits_rna(v);
  }
  for (int idx = threadIdx.x; idx < N * K; idx += blockDim.x) {
    const int r = idx / K, k = idx - r * K;
    const float v = Bt[idx];
    unsigned char* p = tb + umma::tile_off(r, k, esz, kbytes);
    if (kind == 0)
      *reinterpret_cast<uint16_t*>(p) = bf16_bits_rn(v);
    else
      *reinterpret_cast<uint32_t*>(p) = tf32_bits_rna(v);
  }
  umma::fence_smem_to_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t d = tbase;
  if (threadIdx.x == 0) {
    const uint32_t id = umma::idesc(kind == 0 ? umma::kFmtBF16 : umma::kFmtTF32, M, N);
    const uint32_t sbo = (uint32_t)(kbytes / 16) * 128;
    const uint32_t a0 = umma::smem_u32(ta), b0 = umma::smem_u32(tb);
    for (int ks = 0; ks < kbytes / 32; ++ks) {
      const uint64_t da = umma::sdesc(a0 + 256u * ks, 128, sbo);
      const uint64_t db = umma::sdesc(b0 + 256u * ks, 128, sbo);
      if (kind == 0)
        umma::mma_f16(d, da, db, id, ks > 0 ? 1u : 0u);
      else
        umma::mma_tf32(d, da, db, id, ks > 0 ? 1u : 0u);
    }
    umma::commit(&bar);
  }
  __shared__ int ok;
  if (threadIdx.x == 0) ok = 1;
  __syncthreads();
  if (!umma::mbar_wait(&bar, 0)) ok = 0;
  __syncthreads();
  umma::fence_after_sync();
  if (ok) {
    const int row = warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t v[16];
      umma::ld16(umma::taddr(d, warp * 32, c0), v);
      umma::ld_wait();
      for (int j = 0; j < 16; ++j) C[(size_t)row * N + c0 + j] = __uint_as_float(v[j]);
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_dealloc(d, ncols);
  if (threadIdx.x == 0) status[0] = ok ? ST_OK : ST_TIMEOUT;
}

cudaError_t launch_umma_selftest(int kind, int N, int K, const float* A, const float* Bt, float* C, int* status,
                                 cudaStream_t st) {
  const int esz = kind == 0 ? 2 : 4;
  const size_t smem = (size_t)(128 + N) * K * esz + 1024;
  cudaError_t e = cudaFuncSetAttribute(umma_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  umma_selftest_kernel<<<1, 128, smem, st>>>(kind, N, K, A, Bt, C, status);
  ++launch_counter();
  return cudaGetLastError();
}

}  // namespace ttals
