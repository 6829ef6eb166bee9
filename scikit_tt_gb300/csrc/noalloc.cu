// Allocation-free variant of the interface-stack update (ttals_stack_op).
//
// Some callers of this library cannot allocate device memory: a host process
// whose device memory is entirely pre-reserved by its own pool allocator, a
// serving loop that must not take the device-wide synchronisation cudaMalloc
// and cudaFree imply, or a foreign-language host that only ever hands over
// buffers it already owns.  For them ttals_stack_op_noalloc keeps the two
// contraction intermediates in a fixed file-scope device array instead of the
// context's arena: the caller passes inputs and output, and the call
// allocates nothing (no cudaMalloc, cudaFree or allocating library routine).
//
// The array holds kScratchDoubles doubles (16 MiB) on every device that loads
// the library, for the lifetime of the process.  All calls share it and it
// keeps the last call's contents; both intermediates are fully overwritten
// before they are read, so nothing needs clearing.  Two calls whose work
// overlaps on the GPU (for example on two streams) race on the array.
#include <mutex>
#include <string>

#include "../../include/ttals.h"
#include "ttals_internal.h"

namespace {

constexpr int64_t kScratchDoubles = int64_t(1) << 21;  // 2,097,152 doubles = 16 MiB
static __device__ __align__(256) double g_stack_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current.  In host code the array's name only stands for
// the device symbol; its address must come from cudaGetSymbolAddress.
cudaError_t scratch_on(int device, double** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[device]) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return e;
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_stack_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = p;
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

// True when `p` is memory a kernel on `device` may dereference: device memory
// of that device or managed memory.  Pageable or pinned host memory, memory of
// another device and unknown pointers are refused before anything is enqueued.
// cudaPointerGetAttributes allocates nothing.
bool device_reachable(const void* p, int device) {
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();  // a failed query leaves a (non-sticky) error behind: clear it
    return false;
  }
  if (attr.type == cudaMemoryTypeManaged) return true;
  return attr.type == cudaMemoryTypeDevice && attr.device == device;
}

}  // namespace

extern "C" int ttals_stack_op_noalloc(ttals_ctx* ctx, int32_t left, const double* stack, const double* x,
                                      const double* op, int64_t r0, int64_t n, int64_t r1, int64_t R0, int64_t R1,
                                      double* out) {
  if (!ctx) return TTALS_ERR_ARG;
  if (r0 <= 0 || n <= 0 || r1 <= 0 || R0 <= 0 || R1 <= 0) {
    ttals::ctx_set_error(ctx, "dimensions must be positive");
    return TTALS_ERR_ARG;
  }
  // Each of the two intermediates holds at most max(R) * max(r)^2 * n doubles.
  // The product is formed with overflow checks, so absurd dimensions cannot
  // wrap around and slip under the limit.
  const int64_t rmax = r0 > r1 ? r0 : r1, Rmax = R0 > R1 ? R0 : R1;
  int64_t per = 0;
  const bool wrapped = __builtin_mul_overflow(Rmax, rmax, &per) || __builtin_mul_overflow(per, rmax, &per) ||
                       __builtin_mul_overflow(per, n, &per);
  if (wrapped || per > kScratchDoubles / 2) {
    ttals::ctx_set_error(ctx, "ttals_stack_op_noalloc: the intermediates need " +
                                  (wrapped ? std::string("more than 2^63") : std::to_string(2 * per)) +
                                  " doubles, above the static scratch of " + std::to_string(kScratchDoubles) +
                                  " doubles (16 MiB); use ttals_stack_op");
    return TTALS_ERR_ARG;
  }
  if (!stack || !x || !op || !out) {
    ttals::ctx_set_error(ctx, "ttals_stack_op_noalloc: null pointer");
    return TTALS_ERR_ARG;
  }
  const int device = ttals::ctx_device(ctx);
  const void* ptrs[4] = {stack, x, op, out};
  const char* names[4] = {"stack", "x", "op", "out"};
  for (int k = 0; k < 4; ++k) {
    if (!device_reachable(ptrs[k], device)) {
      ttals::ctx_set_error(ctx, std::string("ttals_stack_op_noalloc: ") + names[k] +
                                    " is not device or managed memory of the context's device "
                                    "(this entry point takes device pointers only; ttals_stack_op takes host arrays)");
      return TTALS_ERR_ARG;
    }
  }
  double* base = nullptr;
  cudaError_t e = scratch_on(device, &base);
  if (e != cudaSuccess) {
    ttals::ctx_set_error(ctx, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                  cudaGetErrorString(e));
    return TTALS_ERR_CUDA;
  }
  return ttals::stack_op_on_stream(ctx, left, stack, x, op, r0, n, r1, R0, R1, base, base + per, out);
}
