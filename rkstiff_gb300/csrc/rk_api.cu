// C entry points of librkstiff_gb300 (declared in include/rkstiff_gb300.h).
#include <cuda_runtime.h>
#include <math.h>

#include <string.h>

#include <mutex>
#include <string>
#include <vector>

#include "rk_coeffs.cuh"
#include "rk_evolve.cuh"
#include "rk_launch.h"

namespace rk {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return RK_OK;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return RK_E_CUDA;
}

__global__ void twiddle_kernel(cx<double>* tw64, cx<float>* tw32) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= RK_TW_N) return;
  double s, c;
  // exp(-2 pi i k / N) = cos(pi * 2k/N) - i sin(pi * 2k/N)
  sincospi(2.0 * (double)k / (double)RK_TW_N, &s, &c);
  if (tw64) tw64[k] = cx<double>{c, -s};
  if (tw32) tw32[k] = cx<float>{(float)c, (float)(-s)};
}

// Eight independent FMA chains per thread: sustained FP32 CUDA-core throughput.
__global__ void fp32_probe_kernel(float* out, int iters) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (threadIdx.x + k) * 1e-7f;
  const float b = 0.9999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// ---- side streams and events used to fork per-class launches -------------------------
struct DevicePool {
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
};
static std::mutex g_pool_mu;
static std::vector<DevicePool> g_pools;

static int pool_get(int dev, int need, DevicePool** out) {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if ((int)g_pools.size() <= dev) g_pools.resize(dev + 1);
  DevicePool& p = g_pools[dev];
  while ((int)p.streams.size() < need) {
    cudaStream_t s;
    if (int e = cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "side stream")) return e;
    p.streams.push_back(s);
  }
  while ((int)p.events.size() < need + 1) {
    cudaEvent_t ev;
    if (int e = cuda_check(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "fork event")) return e;
    p.events.push_back(ev);
  }
  *out = &p;
  return RK_OK;
}

static size_t smem_bytes_method(const rk_batch& b, int n, int place) {
  switch (b.method) {
    case RK_IF34: return smem_bytes_IF34(b, n, place);
    case RK_ETD35: return smem_bytes_ETD35(b, n, place);
    case RK_ETD34: return smem_bytes_ETD34(b, n, place);
    case RK_IF45DP: return smem_bytes_IF45DP(b, n, place);
    case RK_ETD4: return smem_bytes_ETD4(b, n, place);
    case RK_ETD5: return smem_bytes_ETD5(b, n, place);
    case RK_IF4: return smem_bytes_IF4(b, n, place);
  }
  return 0;
}

static size_t max_smem_per_block() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
    v = 227 * 1024;
  return (size_t)v;
}

// Placement for a class of grid size n: prefer shared-memory arrays that still leave room
// for two blocks per SM, then any that fits one block, then the global slab.
// A single-step run keeps the coefficients in the global slab (they persist between
// calls); an evolve may rebuild them in shared memory once per launch.
static int auto_place(const rk_batch& b, int n) {
  const size_t tw = (size_t)fpad_size(n) * (b.precision == RK_FP64 ? 16 : 8) +  // compile-time kernels' table
                    (b.mlp != nullptr ? ((RK_MLP_PACK_BYTES + 15) & ~15) : 0);
  const size_t lim1 = max_smem_per_block();
  const size_t lim2 = lim1 / 2 - 1024;
  const bool step = b.run_mode == RK_RUN_STEP;
  for (size_t lim : {lim2, lim1}) {
    if (!step && smem_bytes_method(b, n, RK_PLACE_SMEM_ALL) + tw <= lim) return RK_PLACE_SMEM_ALL;
    if (smem_bytes_method(b, n, RK_PLACE_SMEM_STATE) + tw <= lim) return RK_PLACE_SMEM_STATE;
  }
  return RK_PLACE_GLOBAL;
}

static int auto_threads(int n) {
  int t = n / 8;
  if (t < 64) t = 64;
  if (t > 256) t = 256;
  return t;
}

// groups per block: a block of about 128 threads
static int auto_groups(int threads) { return threads >= 128 ? 1 : 128 / threads; }

static int launch_class(const rk_batch& b, const ClassLaunch& c, cudaStream_t s) {
  const int nn = c.n > 0 ? c.n : b.n_max;
  const size_t tw_bytes = (size_t)fpad_size(nn) * (b.precision == RK_FP64 ? 16 : 8);  // compile-time kernels' table
  // learned-controller launches add a block-wide copy of the inference buffer
  const size_t learned = b.mlp != nullptr ? ((RK_MLP_PACK_BYTES + 15) & ~15) : 0;
  if (smem_bytes_method(b, nn, c.place) * (size_t)c.groups + tw_bytes + learned > max_smem_per_block()) {
    set_error("rk_evolve: placement " + std::to_string(c.place) + " needs more shared memory than a block has");
    return RK_E_SIZE;
  }
  if (b.method == RK_ETD35 && c.n > 0) {
    int e = launch_evolve_etd35_ct(b, c, s);
    if (e != RK_E_UNSUPPORTED) return e;
  }
  switch (b.method) {
    case RK_IF34: return launch_evolve_IF34(b, c, s);
    case RK_ETD35: return launch_evolve_ETD35(b, c, s);
    case RK_ETD34: return launch_evolve_ETD34(b, c, s);
    case RK_IF45DP: return launch_evolve_IF45DP(b, c, s);
    case RK_ETD4: return launch_evolve_ETD4(b, c, s);
    case RK_ETD5: return launch_evolve_ETD5(b, c, s);
    case RK_IF4: return launch_evolve_IF4(b, c, s);
  }
  return RK_E_ARG;
}

static int check_method(int method) {
  if (method < RK_IF34 || method > RK_IF4) {
    set_error("unknown method id " + std::to_string(method));
    return RK_E_ARG;
  }
  return RK_OK;
}

// Argument checks shared by rk_evolve and rk_evolve_noalloc (the latter passes
// need_scratch = false: it supplies slab, slab_off and queue itself).  Nothing is launched
// before these pass.
int validate_batch(const rk_batch* b, bool need_scratch) {
  if (!b) {
    set_error("rk_evolve: null batch");
    return RK_E_ARG;
  }
  if (int e = check_method(b->method)) return e;
  if (b->precision != RK_FP64 && b->precision != RK_FP32) {
    set_error("rk_evolve: precision must be RK_FP64 or RK_FP32");
    return RK_E_ARG;
  }
  if (b->nl_kind < RK_NL_NONE || b->nl_kind > RK_NL_NLS) {
    set_error("rk_evolve: unknown nonlinearity kind");
    return RK_E_ARG;
  }
  if (b->n_inst < 0) {
    set_error("rk_evolve: negative instance count");
    return RK_E_ARG;
  }
  if (b->n_inst == 0) return RK_OK;
  if (!b->n || !b->mode_off || !b->lin_op || !b->u || !b->state || !b->twiddle ||
      (need_scratch && (!b->slab || !b->slab_off || !b->queue))) {
    set_error("rk_evolve: null device pointer");
    return RK_E_ARG;
  }
  if (b->nl_kind == RK_NL_UUX && !b->kx) {
    set_error("rk_evolve: RK_NL_UUX needs kx");
    return RK_E_ARG;
  }
  const int nmax = b->n_max;
  const int limit = b->precision == RK_FP64 ? 4096 : 8192;
  if (nmax < 4 || (nmax & (nmax - 1)) || nmax > limit) {
    set_error("rk_evolve: n_max must be a power of two in [4, " + std::to_string(limit) + "]");
    return RK_E_SIZE;
  }
  if (b->ring_data) {
    const int64_t m_max = b->nl_kind == RK_NL_UUX ? nmax / 2 + 1 : nmax;
    const int64_t need = RK_RING_HEADER + m_max * (b->precision == RK_FP64 ? 16 : 8);
    if (b->ring_slots < 1 || !b->ring_head || !b->ring_tail || b->ring_slot_bytes < need ||
        (b->ring_slot_bytes & 15) || b->ring_timeout_ms < 1) {
      set_error("rk_evolve: the snapshot ring needs >= 1 slot of >= " + std::to_string((long long)need) +
                " bytes (a multiple of 16), head, tail and a positive timeout");
      return RK_E_ARG;
    }
  } else if (b->store_freq > 0 && (b->snap_cap <= 0 || !b->snap_u || !b->snap_t)) {
    set_error("rk_evolve: snapshots requested without a snapshot buffer");
    return RK_E_ARG;
  }
  if (b->etd.contour_points < 2) {
    set_error("rk_evolve: contour_points must be > 1");
    return RK_E_ARG;
  }
  if (b->etd.contour_at_zero) {
    set_error("rk_evolve: contour_at_zero is the matrix-operator form of rk_coeffs, not a diagonal evolve");
    return RK_E_UNSUPPORTED;
  }
  if (b->threads != 0 && b->threads != 32 && b->threads != 64 && b->threads != 128 && b->threads != 256) {
    set_error("rk_evolve: threads must be 0 (auto), 32, 64, 128 or 256");
    return RK_E_ARG;
  }
  if (b->placement < RK_PLACE_AUTO || b->placement > RK_PLACE_SMEM_U) {
    set_error("rk_evolve: unknown placement");
    return RK_E_ARG;
  }
  if (b->coef_blocks < 0 || b->coef_blocks > RK_COEF_BLOCKS_MAX || b->ladder < 0 || b->ladder > 1) {
    set_error("rk_evolve: coef_blocks must be in [0, RK_COEF_BLOCKS_MAX] and ladder 0 or 1");
    return RK_E_ARG;
  }
  return RK_OK;
}

}  // namespace rk

using namespace rk;

extern "C" {

int rk_abi_version(void) { return RK_ABI_VERSION; }

const char* rk_last_error(void) { return g_err.c_str(); }

int rk_fill_twiddles(void* tw64, void* tw32, void* stream) {
  twiddle_kernel<<<(RK_TW_N + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<cx<double>*>(tw64), reinterpret_cast<cx<float>*>(tw32));
  return cuda_check(cudaGetLastError(), "twiddle launch");
}

int64_t rk_slab_bytes(int32_t method, int32_t precision, int32_t coef_complex, int64_t m) {
  if (check_method(method) || m <= 0) return -1;
  return slab_bytes(method, precision, coef_complex, m);
}

int64_t rk_slab_bytes_blocks(int32_t method, int32_t precision, int32_t coef_complex, int64_t m, int32_t blocks) {
  if (check_method(method) || m <= 0 || blocks < 1 || blocks > RK_COEF_BLOCKS_MAX) return -1;
  return slab_bytes(method, precision, coef_complex, m, blocks);
}

int rk_num_coeffs(int32_t method) {
  if (check_method(method)) return RK_E_ARG;
  return num_coeffs(method);
}

int rk_coeffs(int32_t method, int32_t precision, int32_t coef_complex, int64_t m, const double* lin_op, double h,
              const rk_etd_config* etd, void* out, void* stream) {
  if (int e = check_method(method)) return e;
  if (m <= 0 || !lin_op || !out || !etd || (precision != RK_FP64 && precision != RK_FP32)) {
    set_error("rk_coeffs: invalid argument");
    return RK_E_ARG;
  }
  if (etd->contour_points < 2) {
    set_error("rk_coeffs: contour_points must be > 1");
    return RK_E_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  switch (method) {
    case RK_IF34: return launch_coeffs_IF34(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_ETD35: return launch_coeffs_ETD35(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_ETD34: return launch_coeffs_ETD34(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_IF45DP: return launch_coeffs_IF45DP(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_ETD4: return launch_coeffs_ETD4(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_ETD5: return launch_coeffs_ETD5(precision, coef_complex, m, lin_op, h, *etd, out, s);
    case RK_IF4: return launch_coeffs_IF4(precision, coef_complex, m, lin_op, h, *etd, out, s);
  }
  return RK_E_ARG;
}

int rk_ring_create(int64_t slots, int64_t slot_bytes, rk_ring* r) {
  if (!r || slots < 1 || slots > (1 << 24) || slot_bytes < RK_RING_HEADER || (slot_bytes & 15)) {
    set_error("rk_ring_create: slots in [1, 2^24] and slot_bytes >= RK_RING_HEADER, a multiple of 16");
    return RK_E_ARG;
  }
  void* data = nullptr;
  void* ctr = nullptr;
  if (int e = cuda_check(cudaHostAlloc(&data, (size_t)(slots * slot_bytes), cudaHostAllocMapped), "ring alloc"))
    return e;
  if (int e = cuda_check(cudaHostAlloc(&ctr, 64, cudaHostAllocMapped), "ring counters")) {
    cudaFreeHost(data);
    return e;
  }
  memset(data, 0, (size_t)(slots * slot_bytes));
  memset(ctr, 0, 64);
  void* dd = nullptr;
  void* dc = nullptr;
  if (cudaHostGetDevicePointer(&dd, data, 0) != cudaSuccess || cudaHostGetDevicePointer(&dc, ctr, 0) != cudaSuccess ||
      dd != data || dc != ctr) {
    // the pointers are handed to kernels as they are: a platform without unified addressing
    // would need the separate device aliases, which this ring does not keep
    cudaFreeHost(data);
    cudaFreeHost(ctr);
    set_error("rk_ring_create: mapped host memory is not addressable at the same address on the device");
    return RK_E_UNSUPPORTED;
  }
  r->data = data;
  r->head = static_cast<unsigned long long*>(ctr);
  r->tail = reinterpret_cast<int64_t*>(static_cast<char*>(ctr) + 8);
  r->slot_bytes = slot_bytes;
  r->slots = (int32_t)slots;
  r->reserved = 0;
  return RK_OK;
}

int rk_ring_take(rk_ring* r, int64_t k, void* dst, int64_t bytes) {
  if (!r || !r->data || k < 0 || (bytes > 0 && !dst)) {
    set_error("rk_ring_take: invalid argument");
    return RK_E_ARG;
  }
  const int64_t tail = __atomic_load_n(r->tail, __ATOMIC_RELAXED);
  if (k != tail) {
    set_error("rk_ring_take: slots must be taken in order");
    return RK_E_ARG;
  }
  unsigned char* slot = static_cast<unsigned char*>(r->data) + (k % r->slots) * r->slot_bytes;
  // the kernel publishes `ready` after a system-scope fence over the slot's contents: an
  // acquire load orders the copy below after it
  const int64_t ready = __atomic_load_n(reinterpret_cast<int64_t*>(slot), __ATOMIC_ACQUIRE);
  if (ready != k + 1) return 0;
  if (bytes > 0) memcpy(dst, slot, (size_t)(bytes < r->slot_bytes ? bytes : r->slot_bytes));
  __atomic_store_n(r->tail, k + 1, __ATOMIC_RELEASE);
  return 1;
}

int rk_ring_reset(rk_ring* r) {
  if (!r || !r->data) {
    set_error("rk_ring_reset: invalid ring");
    return RK_E_ARG;
  }
  memset(r->data, 0, (size_t)(r->slots * r->slot_bytes));
  __atomic_store_n(r->head, 0ull, __ATOMIC_RELEASE);
  __atomic_store_n(r->tail, (int64_t)0, __ATOMIC_RELEASE);
  return RK_OK;
}

int rk_ring_destroy(rk_ring* r) {
  if (!r) return RK_E_ARG;
  if (r->data) cudaFreeHost(r->data);
  if (r->head) cudaFreeHost(r->head);
  r->data = nullptr;
  r->head = nullptr;
  r->tail = nullptr;
  return RK_OK;
}

int rk_probe_fp32(float* out, int32_t blocks, int32_t threads, int32_t iters, void* stream) {
  if (!out || blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0) {
    set_error("rk_probe_fp32: invalid argument");
    return RK_E_ARG;
  }
  fp32_probe_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters);
  return cuda_check(cudaGetLastError(), "fp32 probe launch");
}

int rk_evolve(const rk_batch* b, void* stream) {
  if (int e = validate_batch(b, true)) return e;
  if (b->n_inst <= 0) return RK_OK;
  const int nmax = b->n_max;
  cudaStream_t s = (cudaStream_t)stream;
  if (b->n_classes <= 0) {
    const int thr = b->threads > 0 ? b->threads : auto_threads(nmax);
    ClassLaunch c{b->order, b->n_inst, 0, b->queue, thr,
                  b->placement == RK_PLACE_AUTO ? auto_place(*b, nmax) : b->placement, 1};
    return launch_class(*b, c, s);
  }
  if (!b->class_n || !b->class_start) {
    set_error("rk_evolve: classes requested without class_n / class_start");
    return RK_E_ARG;
  }
  if (b->class_start[0] != 0 || b->class_start[b->n_classes] != b->n_inst) {
    set_error("rk_evolve: class_start must run from 0 to n_inst");
    return RK_E_ARG;
  }
  std::vector<ClassLaunch> cls;
  for (int c = 0; c < b->n_classes; ++c) {
    const int n = b->class_n[c];
    const int64_t cnt = b->class_start[c + 1] - b->class_start[c];
    if (n < 4 || (n & (n - 1)) || n > nmax || cnt < 0) {
      set_error("rk_evolve: class grid sizes must be powers of two <= n_max");
      return RK_E_SIZE;
    }
    int thr = b->class_threads ? b->class_threads[c] : (b->threads > 0 ? b->threads : auto_threads(n));
    if (thr != 32 && thr != 64 && thr != 128 && thr != 256) {
      set_error("rk_evolve: class thread counts must be 32, 64, 128 or 256");
      return RK_E_ARG;
    }
    int grp = b->class_groups ? b->class_groups[c] : auto_groups(thr);
    if (grp < 1 || thr * grp > 512 || (thr > 32 && grp > 15)) {
      set_error("rk_evolve: class groups must be >= 1 with threads * groups <= 512");
      return RK_E_ARG;
    }
    int pl = b->class_place ? b->class_place[c] : b->placement;
    if (pl == RK_PLACE_AUTO) pl = auto_place(*b, n);
    if (pl < RK_PLACE_GLOBAL || pl > RK_PLACE_SMEM_U) {
      set_error("rk_evolve: unknown class placement");
      return RK_E_ARG;
    }
    if (cnt > 0) cls.push_back(ClassLaunch{b->order + b->class_start[c], cnt, n, b->queue + c, thr, pl, grp});
  }
  if (cls.size() == 1) return launch_class(*b, cls[0], s);
  int dev = 0;
  cudaGetDevice(&dev);
  DevicePool* pool = nullptr;
  if (int e = pool_get(dev, (int)cls.size(), &pool)) return e;
  if (int e = cuda_check(cudaEventRecord(pool->events[0], s), "fork record")) return e;
  for (size_t c = 0; c < cls.size(); ++c) {
    cudaStream_t sc = pool->streams[c];
    if (int e = cuda_check(cudaStreamWaitEvent(sc, pool->events[0], 0), "fork wait")) return e;
    if (int e = launch_class(*b, cls[c], sc)) return e;
    if (int e = cuda_check(cudaEventRecord(pool->events[c + 1], sc), "join record")) return e;
  }
  for (size_t c = 0; c < cls.size(); ++c)
    if (int e = cuda_check(cudaStreamWaitEvent(s, pool->events[c + 1], 0), "join wait")) return e;
  return RK_OK;
}

}  // extern "C"
