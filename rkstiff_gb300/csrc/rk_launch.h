// Per-method launchers (one translation unit each) used by the C entry points.
#pragma once

#include <cuda_runtime.h>
#include <string>

#include "../../include/rkstiff_gb300.h"

namespace rk {

void set_error(const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

// rk_evolve's argument checks (rk_api.cu); need_scratch = false skips slab, slab_off, queue
int validate_batch(const rk_batch* b, bool need_scratch);

// One launch of the evolve kernel over `count` items of `order`, all of grid size n
// (n = 0: mixed sizes up to b.n_max, runtime-size kernel).
struct ClassLaunch {
  const int32_t* order;
  int64_t count;
  int32_t n;       // class grid size, 0 for mixed
  int32_t* queue;  // work counter (zeroed by the launcher)
  int threads;     // threads per instance group (32, 64, 128 or 256)
  int place;       // RK_PLACE_GLOBAL / SMEM_STATE / SMEM_ALL (resolved, not AUTO)
  int groups;      // instance groups per block (threads * groups <= 256)
};

// Shared-memory bytes a class launch needs, or 0 when the placement does not fit.
size_t class_smem_bytes(const rk_batch& b, int n, int place);

#define RK_DECLARE_METHOD(NAME)                                                                   \
  int launch_evolve_##NAME(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);              \
  size_t smem_bytes_##NAME(const rk_batch& b, int n, int place);                                  \
  int launch_coeffs_##NAME(int precision, int coef_complex, int64_t m, const double* lin, double h, \
                           const rk_etd_config& etd, void* out, cudaStream_t s);

RK_DECLARE_METHOD(IF34)
RK_DECLARE_METHOD(ETD35)
RK_DECLARE_METHOD(ETD34)
RK_DECLARE_METHOD(IF45DP)
RK_DECLARE_METHOD(ETD4)
RK_DECLARE_METHOD(ETD5)
RK_DECLARE_METHOD(IF4)

// Tensor map of a rows x inner FP32 row-major array for TMA 2-D tile loads: box of 32
// (inner) x box_rows, 128-byte swizzle (rk_dense.cu); `map` is a CUtensorMap.
int make_tmap_f32_sw128(void* map, const void* base, int64_t inner, int64_t rows, int box_rows);

// compile-time-size ETD35 kernels for real operators (rk_m_etd35_ct.cu); returns
// RK_E_UNSUPPORTED when no specialisation exists for (precision, n)
int launch_evolve_etd35_ct(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);

}  // namespace rk
