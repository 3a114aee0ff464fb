// Launcher bodies for one method; included by rk_m_<method>.cu with RK_METHOD_ID and
// RK_METHOD_NAME defined.
#pragma once

#include "rk_evolve.cuh"
#include "rk_launch.h"

namespace rk {

template <class T, class CT, class S, int M>
static int launch_evolve_t(const rk_batch& b, cudaStream_t st) {
  const int nfft = b.n_max;
  const size_t sm = evolve_smem<T>(nfft);
  auto kern = evolve_kernel<T, CT, S, M>;
  if (int e = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                         "cudaFuncSetAttribute(evolve smem)"))
    return e;
  const int threads = b.threads > 0 ? b.threads : 256;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (int e = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, sm), "occupancy"))
    return e;
  if (occ < 1) {
    set_error("evolve kernel does not fit on an SM (shared memory " + std::to_string(sm) + " bytes)");
    return RK_E_SIZE;
  }
  long grid = (long)nsm * occ;
  if ((long)b.n_inst < grid) grid = (long)b.n_inst;
  if (int e = cuda_check(cudaMemsetAsync(b.queue, 0, sizeof(int32_t), st), "queue reset")) return e;
  kern<<<(unsigned)grid, threads, sm, st>>>(b, nfft);
  return cuda_check(cudaGetLastError(), "evolve launch");
}

template <int M>
static int launch_evolve_m(const rk_batch& b, cudaStream_t st) {
  if (b.precision == RK_FP64) {
    if (b.coef_complex) return launch_evolve_t<double, cx<double>, cx<double>, M>(b, st);
    return launch_evolve_t<double, double, double, M>(b, st);
  }
  if (b.coef_complex) return launch_evolve_t<float, cx<float>, cx<double>, M>(b, st);
  return launch_evolve_t<float, float, double, M>(b, st);
}

template <class T, class CT, class S, int M>
static int launch_coeffs_t(int64_t m, const double* lin, double h, const rk_etd_config& etd, void* out,
                           cudaStream_t st) {
  const int threads = 256;
  const unsigned blocks = (unsigned)((m + threads - 1) / threads);
  coeff_kernel<T, CT, S, M><<<blocks, threads, 0, st>>>((int)m, lin, h, etd, reinterpret_cast<CT*>(out));
  return cuda_check(cudaGetLastError(), "coefficient launch");
}

template <int M>
static int launch_coeffs_m(int precision, int coef_complex, int64_t m, const double* lin, double h,
                           const rk_etd_config& etd, void* out, cudaStream_t st) {
  if (precision == RK_FP64) {
    if (coef_complex) return launch_coeffs_t<double, cx<double>, cx<double>, M>(m, lin, h, etd, out, st);
    return launch_coeffs_t<double, double, double, M>(m, lin, h, etd, out, st);
  }
  if (coef_complex) return launch_coeffs_t<float, cx<float>, cx<double>, M>(m, lin, h, etd, out, st);
  return launch_coeffs_t<float, float, double, M>(m, lin, h, etd, out, st);
}

}  // namespace rk

#define RK_CAT2(a, b) a##b
#define RK_CAT(a, b) RK_CAT2(a, b)

namespace rk {
int RK_CAT(launch_evolve_, RK_METHOD_NAME)(const rk_batch& b, cudaStream_t s) {
  return launch_evolve_m<RK_METHOD_ID>(b, s);
}
int RK_CAT(launch_coeffs_, RK_METHOD_NAME)(int precision, int coef_complex, int64_t m, const double* lin, double h,
                                           const rk_etd_config& etd, void* out, cudaStream_t s) {
  return launch_coeffs_m<RK_METHOD_ID>(precision, coef_complex, m, lin, h, etd, out, s);
}
}  // namespace rk
