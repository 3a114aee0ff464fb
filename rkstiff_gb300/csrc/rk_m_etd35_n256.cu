// ETD35 with a real operator at the compile-time grid size n = 256 (FP32 and FP64):
// one of the batched-ensemble configurations.
#include "rk_launch_impl.cuh"

namespace rk {

template <class T>
static int ct_256(const rk_batch& b, const ClassLaunch& c, cudaStream_t s) {
  switch (c.place) {
    case RK_PLACE_GLOBAL: return launch_evolve_v<T, T, double, RK_ETD35, 8, PL_GLOBAL>(b, c, s);
    case RK_PLACE_SMEM_STATE: return launch_evolve_v<T, T, double, RK_ETD35, 8, PL_SMEM_STATE>(b, c, s);
    case RK_PLACE_SMEM_ALL: return launch_evolve_v<T, T, double, RK_ETD35, 8, PL_SMEM_ALL>(b, c, s);
    case RK_PLACE_SMEM_U: return launch_evolve_v<T, T, double, RK_ETD35, 8, PL_SMEM_U>(b, c, s);
  }
  return RK_E_UNSUPPORTED;
}

int launch_evolve_etd35_n256(const rk_batch& b, const ClassLaunch& c, cudaStream_t s) {
  return b.precision == RK_FP64 ? ct_256<double>(b, c, s) : ct_256<float>(b, c, s);
}

}  // namespace rk
