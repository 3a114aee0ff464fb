// rk_evolve_noalloc: rk_evolve for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: code that runs inside a CUDA stream
// capture of someone else's graph, plugins hosted by an application that owns every device
// allocation through its own pool, and embedded or real-time hosts that forbid allocation
// after start-up.  rk_evolve needs per-instance scratch (the coefficient and stage arrays),
// the slab offset table and the work-queue counters, which its callers normally allocate.
// This entry point takes the same rk_batch (its slab, slab_off and queue fields are ignored)
// and places all of that scratch in one file-scope device array of RK_NOALLOC_SCRATCH_BYTES
// instead.  Every GPU that loads the library holds that array until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "rk_evolve.cuh"
#include "rk_launch.h"

namespace rk {

// scratch shared by every call: [64 queue counters | slab offsets | slabs]
static __device__ __align__(256) unsigned char g_noalloc_scratch[RK_NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch per device, with the context it was looked up in.
// The host-side symbol is only a stand-in: a kernel handed it would fault or, where the
// GPU can reach host memory, use the wrong memory.
struct NoallocSlot {
  void* ctx;
  void* ptr;
};
static std::mutex g_noalloc_mu;
static NoallocSlot g_noalloc_slot[64];

typedef int (*ctx_get_current_fn)(void**);

// cuCtxGetCurrent from the driver (through the runtime's entry-point query, so the library
// needs no link against libcuda); NULL when the driver does not offer it
static ctx_get_current_fn ctx_get_current() {
  static ctx_get_current_fn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<ctx_get_current_fn>(p);
  }
  return fn;
}

// Offsets of instance i's slab: a uniform stride (the slab of the largest grid), so no
// per-instance sizes are read back from the device.  Also invalidates each instance's
// cached coefficients and saved low state words: the shared array holds whatever the
// previous call left there.
__global__ void noalloc_prepare_kernel(int64_t* slab_off, int64_t n_inst, int64_t stride, rk_inst_state* state) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_inst) return;
  slab_off[i] = i * stride;
  state[i].h_coeff = __longlong_as_double(0x7ff8000000000000ULL);
  state[i].reserved_i = 0;  // nor are the low words of a double-float state kept there
}

}  // namespace rk

using namespace rk;

extern "C" int rk_evolve_noalloc(const rk_batch* b, void* stream) {
  // every argument check of rk_evolve runs before anything is launched, so a rejected call
  // leaves the caller's state records untouched
  if (int e = validate_batch(b, false)) return e;
  if (b->n_inst == 0) return RK_OK;
  const int64_t m_max = (b->nl_kind == RK_NL_UUX) ? b->n_max / 2 + 1 : b->n_max;
  const int blocks = b->coef_blocks > 1 ? b->coef_blocks : 1;
  const int64_t stride = (slab_bytes(b->method, b->precision, b->coef_complex, m_max, blocks) + 255) / 256 * 256;
  // bound the instance count before any product: 256 bytes of counters, 8 bytes of offset
  // and one slab per instance, plus at most 255 bytes of offset-table padding
  const int64_t avail = (int64_t)RK_NOALLOC_SCRATCH_BYTES - 256 - 255;
  if (b->n_inst > avail / (stride + (int64_t)sizeof(int64_t))) {
    set_error("rk_evolve_noalloc: " + std::to_string((long long)b->n_inst) + " instances of n_max " +
              std::to_string(b->n_max) + " need more than the " + std::to_string((long long)RK_NOALLOC_SCRATCH_BYTES) +
              " bytes of scratch this entry point holds; use rk_evolve with caller-allocated scratch");
    return RK_E_SIZE;
  }
  const int64_t off_bytes = (b->n_inst * (int64_t)sizeof(int64_t) + 255) / 256 * 256;
  int dev = 0;
  if (int e = cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) return e;
  if (dev < 0 || dev >= 64) {
    set_error("rk_evolve_noalloc: device index out of range");
    return RK_E_ARG;
  }
  void* base = nullptr;
  {
    // set-up, once per device (and again only if that device's context was replaced, e.g.
    // after cudaDeviceReset), with the device current: the array's device address
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    void* ctx = nullptr;
    if (ctx_get_current_fn f = ctx_get_current()) {
      if (f(&ctx) != 0) ctx = nullptr;
    }
    NoallocSlot& sl = g_noalloc_slot[dev];
    if (!sl.ptr || sl.ctx != ctx) {
      void* p = nullptr;
      if (int e = cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress")) return e;
      sl.ptr = p;
      sl.ctx = ctx;
    }
    base = sl.ptr;
  }
  unsigned char* sc = static_cast<unsigned char*>(base);
  rk_batch b2 = *b;
  // one launch over all instances: the per-size class split would fork onto side streams,
  // which the library creates on first use
  b2.n_classes = 0;
  b2.class_n = nullptr;
  b2.class_start = nullptr;
  b2.class_threads = nullptr;
  b2.class_place = nullptr;
  b2.class_groups = nullptr;
  b2.queue = reinterpret_cast<int32_t*>(sc);  // zeroed by the launch path before each kernel
  int64_t* offs = reinterpret_cast<int64_t*>(sc + 256);
  b2.slab_off = offs;
  b2.slab = sc + 256 + off_bytes;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned nb = (unsigned)((b->n_inst + 255) / 256);
  noalloc_prepare_kernel<<<nb, 256, 0, s>>>(offs, b->n_inst, stride, b->state);
  if (int e = cuda_check(cudaGetLastError(), "noalloc prepare launch")) return e;
  return rk_evolve(&b2, stream);
}
