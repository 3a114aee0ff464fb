// Per-method launchers (one translation unit each) used by the C entry points.
#pragma once

#include <cuda_runtime.h>
#include <string>

#include "../../include/rkstiff_gb300.h"

namespace rk {

void set_error(const std::string& msg);
int cuda_check(cudaError_t e, const char* what);

#define RK_DECLARE_METHOD(NAME)                                                      \
  int launch_evolve_##NAME(const rk_batch& b, cudaStream_t s);                       \
  int launch_coeffs_##NAME(int precision, int coef_complex, int64_t m, const double* lin, double h, \
                           const rk_etd_config& etd, void* out, cudaStream_t s);

RK_DECLARE_METHOD(IF34)
RK_DECLARE_METHOD(ETD35)
RK_DECLARE_METHOD(ETD34)
RK_DECLARE_METHOD(IF45DP)
RK_DECLARE_METHOD(ETD4)
RK_DECLARE_METHOD(ETD5)
RK_DECLARE_METHOD(IF4)

}  // namespace rk
