// Launcher bodies for one method; included by rk_m_<method>.cu with RK_METHOD_ID and
// RK_METHOD_NAME defined.
#pragma once

#include "rk_evolve.cuh"
#include "rk_launch.h"

namespace rk {

template <class T, class CT, class S, int M, int LOGN, int PLACE>
static int launch_evolve_v(const rk_batch& b, const ClassLaunch& c, cudaStream_t st) {
  const int nfft = c.n > 0 ? c.n : b.n_max;
  const int64_t m = (b.nl_kind == RK_NL_UUX) ? nfft / 2 + 1 : nfft;
  const size_t group_smem = (evolve_smem<T>(nfft) + smem_slab_bytes<T, CT, M>(PLACE, m) + 15) & ~size_t(15);
  const size_t sm = block_extra_offset<T, LOGN>(c.groups, (int)group_smem) +
                   (b.mlp != nullptr ? learned_extra_bytes() : 0);
  const int block = c.threads * c.groups;
  auto kern = evolve_kernel<T, CT, S, M, LOGN, PLACE>;
  if (int e = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                         "cudaFuncSetAttribute(evolve smem)"))
    return e;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (int e = cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, sm), "occupancy"))
    return e;
  if (occ < 1) {
    set_error("evolve kernel does not fit on an SM (shared memory " + std::to_string(sm) + " bytes, " +
              std::to_string(block) + " threads)");
    return RK_E_SIZE;
  }
  // enough groups to cover the class, at most a full residency of the device
  long need = (long)((c.count + c.groups - 1) / c.groups);
  long grid = (long)nsm * occ;
  if (need < grid) grid = need;
  if (int e = cuda_check(cudaMemsetAsync(c.queue, 0, sizeof(int32_t), st), "queue reset")) return e;
  kern<<<(unsigned)grid, block, sm, st>>>(b, c.order, c.count, c.queue, nfft, c.threads, (int)group_smem);
  return cuda_check(cudaGetLastError(), "evolve launch");
}

template <class T, class CT, class S, int M, int LOGN>
static int launch_evolve_p(const rk_batch& b, const ClassLaunch& c, cudaStream_t st) {
  switch (c.place) {
    case RK_PLACE_GLOBAL: return launch_evolve_v<T, CT, S, M, LOGN, PL_GLOBAL>(b, c, st);
    case RK_PLACE_SMEM_STATE: return launch_evolve_v<T, CT, S, M, LOGN, PL_SMEM_STATE>(b, c, st);
    case RK_PLACE_SMEM_ALL: return launch_evolve_v<T, CT, S, M, LOGN, PL_SMEM_ALL>(b, c, st);
    case RK_PLACE_SMEM_U:
      set_error("placement RK_PLACE_SMEM_U is served by the compile-time ETD35 kernels (real operator, u*ux, "
                "n = 256 .. 2048) only");
      return RK_E_UNSUPPORTED;
  }
  set_error("unknown placement");
  return RK_E_ARG;
}

// shared memory of one instance group (the block holds `groups` of them)
template <class T, class CT>
static size_t smem_bytes_t(const rk_batch& b, int M, int n, int place) {
  const int64_t m = (b.nl_kind == RK_NL_UUX) ? n / 2 + 1 : n;
  size_t sm = evolve_smem<T>(n);
  switch (M) {
    case RK_ETD35: sm += smem_slab_bytes<T, CT, RK_ETD35>(place, m); break;
    case RK_ETD5: sm += smem_slab_bytes<T, CT, RK_ETD5>(place, m); break;
    case RK_ETD34: sm += smem_slab_bytes<T, CT, RK_ETD34>(place, m); break;
    case RK_ETD4: sm += smem_slab_bytes<T, CT, RK_ETD4>(place, m); break;
    case RK_IF34: sm += smem_slab_bytes<T, CT, RK_IF34>(place, m); break;
    case RK_IF4: sm += smem_slab_bytes<T, CT, RK_IF4>(place, m); break;
    case RK_IF45DP: sm += smem_slab_bytes<T, CT, RK_IF45DP>(place, m); break;
  }
  return (sm + 15) & ~size_t(15);
}

template <int M>
static size_t smem_bytes_m(const rk_batch& b, int n, int place) {
  if (b.precision == RK_FP64)
    return b.coef_complex ? smem_bytes_t<double, cx<double>>(b, M, n, place) : smem_bytes_t<double, double>(b, M, n, place);
  return b.coef_complex ? smem_bytes_t<float, cx<float>>(b, M, n, place) : smem_bytes_t<float, float>(b, M, n, place);
}

template <int M>
static int launch_evolve_m(const rk_batch& b, const ClassLaunch& c, cudaStream_t st) {
  if (b.precision == RK_FP64) {
    if (b.coef_complex) return launch_evolve_p<double, cx<double>, cx<double>, M, 0>(b, c, st);
    return launch_evolve_p<double, double, double, M, 0>(b, c, st);
  }
  if (b.coef_complex) return launch_evolve_p<float, cx<float>, cx<double>, M, 0>(b, c, st);
  return launch_evolve_p<float, float, double, M, 0>(b, c, st);
}

template <class T, class CT, class S, int M>
static int launch_coeffs_t(int64_t m, const double* lin, double h, const rk_etd_config& etd, void* out,
                           cudaStream_t st) {
  if (etd.contour_at_zero && is_etd(M)) {
    const unsigned blocks = (unsigned)((m * 32 + 255) / 256);  // a warp per mode
    coeff_zero_contour_kernel<CT, S, M><<<blocks, 256, 0, st>>>((int)m, lin, h, etd, reinterpret_cast<CT*>(out));
    return cuda_check(cudaGetLastError(), "coefficient launch");
  }
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

#ifdef RK_METHOD_ID
#define RK_CAT2(a, b) a##b
#define RK_CAT(a, b) RK_CAT2(a, b)

namespace rk {
int RK_CAT(launch_evolve_, RK_METHOD_NAME)(const rk_batch& b, const ClassLaunch& c, cudaStream_t s) {
  return launch_evolve_m<RK_METHOD_ID>(b, c, s);
}
size_t RK_CAT(smem_bytes_, RK_METHOD_NAME)(const rk_batch& b, int n, int place) {
  return smem_bytes_m<RK_METHOD_ID>(b, n, place);
}
int RK_CAT(launch_coeffs_, RK_METHOD_NAME)(int precision, int coef_complex, int64_t m, const double* lin, double h,
                                           const rk_etd_config& etd, void* out, cudaStream_t s) {
  return launch_coeffs_m<RK_METHOD_ID>(precision, coef_complex, m, lin, h, etd, out, s);
}
}  // namespace rk
#endif
