// Building blocks of the stepping loop for a user-supplied nonlinearity (a device-side torch
// callable, evaluated between these kernels): the stage linear combinations of the
// _update_stages methods (e.g. rkstiff/etd35.py:320-345) as one fused pass each, and the
// embedded error test of rkstiff/solveras.py:412-455 reduced on the device.
#include <cuda_runtime.h>

#include <cmath>

#include "rk_common.cuh"
#include "rk_launch.h"

namespace rk {
namespace callable {

constexpr int MAX_TERMS = 8;

struct CombineArgs {
  rk_term t[MAX_TERMS];
  int n;
  int64_t m;
  void* out;
};

// out[j] = sum_i w_i * (c_i[j] * v_i[j])   (c_i absent: w_i * v_i[j])
template <class T, bool CCPLX>
__global__ void combine_kernel(CombineArgs a) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < a.m; j += stride) {
    cx<T> acc{T(0), T(0)};
    for (int i = 0; i < a.n; ++i) {
      cx<T> term = static_cast<const cx<T>*>(a.t[i].v)[j];
      if (a.t[i].coef) {
        if constexpr (CCPLX) term = static_cast<const cx<T>*>(a.t[i].coef)[j] * term;
        else term = static_cast<const T*>(a.t[i].coef)[j] * term;
      }
      acc = acc + (T)a.t[i].w * term;
    }
    static_cast<cx<T>*>(a.out)[j] = acc;
  }
}

// s = safety (eps |u[mask]| / |err[mask]|)^(1/q), mask |u| / max|u| > adapt_cutoff; FP64,
// NaN anywhere in |u| gives an empty mask and s = NaN, as NumPy does.  One block.
template <class T>
__global__ void error_s_kernel(const cx<T>* u, const cx<T>* e, int64_t m, rk_controller ctl, int q, double* s_out) {
  __shared__ double red[64];
  double mx = 0.0;
  int nan = 0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    const double a = hypot((double)u[j].x, (double)u[j].y);
    if (a != a) nan = 1;
    else mx = fmax(mx, a);
  }
  Group g{(int)threadIdx.x, (int)blockDim.x, 0};
  mx = group_max_nan(g, red, nan ? nan_d() : mx);
  double su = 0.0, se = 0.0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    const double a = hypot((double)u[j].x, (double)u[j].y);
    if (a / mx > ctl.adapt_cutoff) {
      su += (double)u[j].x * (double)u[j].x + (double)u[j].y * (double)u[j].y;
      se += (double)e[j].x * (double)e[j].x + (double)e[j].y * (double)e[j].y;
    }
  }
  group_sum2(g, red, su, se);
  if (threadIdx.x == 0) {
    const double tol = ctl.epsilon * sqrt(su);
    *s_out = ctl.safety_f * pow(tol / sqrt(se), 1.0 / q);
  }
}

// y = M x for a dense n x n complex matrix (row-major): one warp per row, lanes striding the
// row (coalesced), warp-shuffle sum.  The basis changes S v and S^-1 N of the eigenbasis
// stepping of a dense lin_op (the S.dot / Sinv.dot of etd35.py:377-495, if34.py:137-199)
template <class T>
__global__ void cgemv_kernel(const cx<T>* M, const cx<T>* x, cx<T>* y, int64_t n) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const cx<T>* r = M + row * n;
  T ax = T(0), ay = T(0);
  for (int64_t j = lane; j < n; j += 32) {
    const cx<T> a = r[j], b = x[j];
    ax += a.x * b.x - a.y * b.y;
    ay += a.x * b.y + a.y * b.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o);
    ay += __shfl_xor_sync(0xffffffffu, ay, o);
  }
  if (lane == 0) y[row] = cx<T>{ax, ay};
}

}  // namespace callable
}  // namespace rk

using namespace rk;
using namespace rk::callable;

extern "C" int rk_combine(int32_t precision, int32_t coef_complex, int64_t m, const rk_term* terms, int32_t nterms,
                          void* out, void* stream) {
  if (!terms || !out || m < 0 || nterms < 1 || nterms > MAX_TERMS || (precision != RK_FP64 && precision != RK_FP32)) {
    set_error("rk_combine: invalid argument (1..8 terms)");
    return RK_E_ARG;
  }
  if (m == 0) return RK_OK;
  CombineArgs a;
  for (int i = 0; i < nterms; ++i) {
    if (!terms[i].v) {
      set_error("rk_combine: a term without a vector");
      return RK_E_ARG;
    }
    a.t[i] = terms[i];
  }
  a.n = nterms;
  a.m = m;
  a.out = out;
  const int threads = 256;
  const int64_t want = (m + threads - 1) / threads;
  const unsigned blocks = (unsigned)(want < 4096 ? want : 4096);
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == RK_FP64) {
    if (coef_complex) combine_kernel<double, true><<<blocks, threads, 0, s>>>(a);
    else combine_kernel<double, false><<<blocks, threads, 0, s>>>(a);
  } else {
    if (coef_complex) combine_kernel<float, true><<<blocks, threads, 0, s>>>(a);
    else combine_kernel<float, false><<<blocks, threads, 0, s>>>(a);
  }
  return cuda_check(cudaGetLastError(), "rk_combine launch");
}

extern "C" int rk_error_s(int32_t precision, int64_t m, const void* unew, const void* err, const rk_controller* ctl,
                          int32_t q, double* s_out, void* stream) {
  if (!unew || !err || !ctl || !s_out || m <= 0 || q < 1 || (precision != RK_FP64 && precision != RK_FP32)) {
    set_error("rk_error_s: invalid argument");
    return RK_E_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == RK_FP64)
    error_s_kernel<double><<<1, 1024, 0, s>>>(static_cast<const cx<double>*>(unew), static_cast<const cx<double>*>(err),
                                              m, *ctl, q, s_out);
  else
    error_s_kernel<float><<<1, 1024, 0, s>>>(static_cast<const cx<float>*>(unew), static_cast<const cx<float>*>(err), m,
                                             *ctl, q, s_out);
  return cuda_check(cudaGetLastError(), "rk_error_s launch");
}

extern "C" int rk_cgemv(int32_t precision, int64_t n, const void* M, const void* x, void* y, void* stream) {
  if (!M || !x || !y || n <= 0 || x == y || (precision != RK_FP64 && precision != RK_FP32)) {
    set_error("rk_cgemv: invalid argument (y must not alias x)");
    return RK_E_ARG;
  }
  const int rows_per_block = 8;
  const unsigned blocks = (unsigned)((n + rows_per_block - 1) / rows_per_block);
  cudaStream_t s = (cudaStream_t)stream;
  if (precision == RK_FP64)
    cgemv_kernel<double><<<blocks, 32 * rows_per_block, 0, s>>>(
        static_cast<const cx<double>*>(M), static_cast<const cx<double>*>(x), static_cast<cx<double>*>(y), n);
  else
    cgemv_kernel<float><<<blocks, 32 * rows_per_block, 0, s>>>(
        static_cast<const cx<float>*>(M), static_cast<const cx<float>*>(x), static_cast<cx<float>*>(y), n);
  return cuda_check(cudaGetLastError(), "rk_cgemv launch");
}
