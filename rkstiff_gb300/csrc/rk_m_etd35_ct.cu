// Dispatch to the compile-time-size ETD35 kernels (real operator, the u*ux nonlinearity,
// n = 256..2048).
#include "rk_launch.h"

namespace rk {

int launch_evolve_etd35_n256(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);
int launch_evolve_etd35_n512(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);
int launch_evolve_etd35_n1024(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);
int launch_evolve_etd35_n2048(const rk_batch& b, const ClassLaunch& c, cudaStream_t s);

int launch_evolve_etd35_ct(const rk_batch& b, const ClassLaunch& c, cudaStream_t s) {
  if (b.coef_complex || c.n <= 0 || b.nl_kind != RK_NL_UUX) return RK_E_UNSUPPORTED;
  switch (c.n) {
    case 256: return launch_evolve_etd35_n256(b, c, s);
    case 512: return launch_evolve_etd35_n512(b, c, s);
    case 1024: return launch_evolve_etd35_n1024(b, c, s);
    case 2048: return launch_evolve_etd35_n2048(b, c, s);
  }
  return RK_E_UNSUPPORTED;
}

}  // namespace rk
