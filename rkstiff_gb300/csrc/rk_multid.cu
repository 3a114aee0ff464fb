// Multi-dimensional NLS nonlinearities of the reference's NLS demo (demos/nls.ipynb) on the
// library's own kernels:
//   * rk_nls_lines: along every line of a 2-D array (rows or columns, any element stride),
//     the inverse FFT, the NLS product i gamma |v|^2 v, or the whole step
//     fft(i gamma |v|^2 v) with v = ifft(x) fused in shared memory; the 2-D NLS
//     N(g) = fft2(i gamma |F|^2 F), F = ifft2(g), is an inverse row transform, the fused
//     step along the columns and a forward row transform (the two axes' transforms
//     commute);
//   * rk_dht: the quasi-discrete Hankel transform over the radial axis, out = Y in * s or
//     Y in / s with the real n x n matrix Y of rkstiff/transforms.py:110-114, as a tiled
//     product (complex columns as pairs of real ones).
// Transforms run the library's Stockham FFT (fft_group, power-of-two lengths up to RK_TW_N)
// on one thread group per line; several groups share a block.
#include <cuda_runtime.h>

#include <string>

#include "rk_fft.cuh"
#include "rk_launch.h"

namespace rk {
namespace md {

enum { LINES_INVERSE = 0, LINES_FORWARD = 1, LINES_NLS = 2 };

// Line l's element j sits at in[l * line_stride + j * elem_stride] (complex T).  INVERSE
// scales by 1/n as numpy.fft.ifft does; NLS forms fft(i gamma |v|^2 v) of v = ifft(x).
template <class T, int MODE>
__global__ void __launch_bounds__(256) lines_kernel(int n, int logn, int64_t lines, int64_t elem_stride,
                                                    int64_t line_stride, T gamma, const cx<T>* in, cx<T>* out,
                                                    const cx<T>* __restrict__ tw,
                                                    int gthreads) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ngroups = blockDim.x / gthreads;
  const int gi = threadIdx.x / gthreads;
  const int64_t line = (int64_t)blockIdx.x * ngroups + gi;
  if (line >= lines) return;  // this group's named barrier is its own
  const Group g{(int)(threadIdx.x % gthreads), gthreads, gthreads == 32 ? -1 : (ngroups == 1 ? 0 : 1 + gi)};
  cx<T>* a = reinterpret_cast<cx<T>*>(smem) + (size_t)gi * 2 * n;
  cx<T>* b = a + n;
  const cx<T>* src = in + line * line_stride;
  for (int j = g.tid; j < n; j += g.nthr) a[j] = src[j * elem_stride];
  g.sync();
  cx<T>* r;
  if (MODE == LINES_FORWARD) {
    r = fft_group<T, false>(g, a, b, logn, tw);
  } else {
    cx<T>* v = fft_group<T, true>(g, a, b, logn, tw);
    const T inv_n = T(1) / T(n);
    if (MODE == LINES_INVERSE) {
      for (int j = g.tid; j < n; j += g.nthr) v[j] = v[j] * inv_n;
      g.sync();
      r = v;
    } else {
      cx<T>* p = v == a ? b : a;
      for (int j = g.tid; j < n; j += g.nthr) {
        const cx<T> f = v[j] * inv_n;
        const T a2 = (f.x * f.x + f.y * f.y) * gamma;
        p[j] = cx<T>{-a2 * f.y, a2 * f.x};
      }
      g.sync();
      r = fft_group<T, false>(g, p, v, logn, tw);
    }
  }
  cx<T>* dst = out + line * line_stride;
  for (int j = g.tid; j < n; j += g.nthr) dst[j * elem_stride] = r[j];
}

// out = i gamma |x|^2 x elementwise (the product alone, for lines of one point)
template <class T>
__global__ void nls_pointwise_kernel(int64_t count, T gamma, const cx<T>* __restrict__ in, cx<T>* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const cx<T> f = in[i];
  const T a2 = (f.x * f.x + f.y * f.y) * gamma;
  out[i] = cx<T>{-a2 * f.y, a2 * f.x};
}

// out[i][c] = (sum_k Y[i][k] in[k][c]) * s (DIVIDE: / s) for an n x n real Y and an n x w
// real in (a complex array of c columns is w = 2c real ones); 16 x 16 tiles
template <class T, bool DIVIDE>
__global__ void dht_kernel(int64_t n, int64_t w, const T* __restrict__ Y, T s, const T* __restrict__ in,
                           T* __restrict__ out) {
  __shared__ T ys[16][17], xs[16][17];
  const int64_t r = (int64_t)blockIdx.y * 16 + threadIdx.y, c = (int64_t)blockIdx.x * 16 + threadIdx.x;
  T acc = T(0);
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    const int64_t ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
    ys[threadIdx.y][threadIdx.x] = (r < n && ka < n) ? Y[r * n + ka] : T(0);
    xs[threadIdx.y][threadIdx.x] = (kb < n && c < w) ? in[kb * w + c] : T(0);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) acc = fma(ys[threadIdx.y][k], xs[k][threadIdx.x], acc);
    __syncthreads();
  }
  if (r < n && c < w) out[r * w + c] = DIVIDE ? acc / s : acc * s;
}

template <class T, int MODE>
static int launch_lines(int n, int logn, int64_t lines, int64_t es, int64_t ls, double gamma, const void* in,
                        void* out, const void* tw, cudaStream_t st) {
  int gth = n / 4;
  gth = gth < 32 ? 32 : (gth > 256 ? 256 : gth);
  const int groups = 256 / gth;
  const size_t sm = (size_t)groups * 2 * n * sizeof(cx<T>);
  auto kern = lines_kernel<T, MODE>;
  if (int e = cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                         "rk_nls_lines smem"))
    return e;
  const unsigned blocks = (unsigned)((lines + groups - 1) / groups);
  kern<<<blocks, gth * groups, sm, st>>>(n, logn, lines, es, ls, T(gamma), static_cast<const cx<T>*>(in),
                                         static_cast<cx<T>*>(out), static_cast<const cx<T>*>(tw), gth);
  return cuda_check(cudaGetLastError(), "rk_nls_lines launch");
}

template <class T>
static int lines_t(int32_t mode, int n, int logn, int64_t lines, int64_t es, int64_t ls, double gamma,
                   const void* in, void* out, const void* tw, cudaStream_t st) {
  if (n == 1) {
    if (mode != LINES_NLS) {
      // a transform of one point is the identity
      if (in == out) return RK_OK;
      for (int64_t l = 0; l < lines; ++l) {
        if (int e = cuda_check(cudaMemcpyAsync(static_cast<cx<T>*>(out) + l * ls, static_cast<const cx<T>*>(in) + l * ls,
                                               sizeof(cx<T>), cudaMemcpyDeviceToDevice, st),
                               "rk_nls_lines copy"))
          return e;
      }
      return RK_OK;
    }
    if (ls != 1) {
      set_error("rk_nls_lines: one-point lines must be contiguous (line_stride 1)");
      return RK_E_ARG;
    }
    nls_pointwise_kernel<T><<<(unsigned)((lines + 255) / 256), 256, 0, st>>>(lines, T(gamma),
                                                                             static_cast<const cx<T>*>(in),
                                                                             static_cast<cx<T>*>(out));
    return cuda_check(cudaGetLastError(), "rk_nls_lines pointwise launch");
  }
  switch (mode) {
    case LINES_INVERSE: return launch_lines<T, LINES_INVERSE>(n, logn, lines, es, ls, gamma, in, out, tw, st);
    case LINES_FORWARD: return launch_lines<T, LINES_FORWARD>(n, logn, lines, es, ls, gamma, in, out, tw, st);
    default: return launch_lines<T, LINES_NLS>(n, logn, lines, es, ls, gamma, in, out, tw, st);
  }
}

}  // namespace md
}  // namespace rk

using namespace rk;
using namespace rk::md;

extern "C" int rk_nls_lines(int32_t precision, int32_t mode, int64_t n, int64_t lines, int64_t elem_stride,
                            int64_t line_stride, double gamma, const void* in, void* out, const void* twiddle,
                            void* stream) {
  if ((precision != RK_FP64 && precision != RK_FP32) || mode < LINES_INVERSE || mode > LINES_NLS || lines < 0 ||
      !in || !out || (n > 1 && !twiddle)) {
    set_error("rk_nls_lines: invalid argument");
    return RK_E_ARG;
  }
  if (n < 1 || (n & (n - 1)) || n > RK_TW_N) {
    set_error("rk_nls_lines: the line length must be a power of two <= RK_TW_N");
    return RK_E_SIZE;
  }
  if (precision == RK_FP64 && 2 * n * 16 > 200 * 1024) {
    set_error("rk_nls_lines: FP64 lines are limited to 4096 points");
    return RK_E_SIZE;
  }
  if (lines == 0) return RK_OK;
  int logn = 0;
  while ((int64_t(1) << logn) < n) ++logn;
  cudaStream_t st = (cudaStream_t)stream;
  return precision == RK_FP64
             ? lines_t<double>(mode, (int)n, logn, lines, elem_stride, line_stride, gamma, in, out, twiddle, st)
             : lines_t<float>(mode, (int)n, logn, lines, elem_stride, line_stride, gamma, in, out, twiddle, st);
}

extern "C" int rk_dht(int32_t precision, int32_t divide, int64_t n, int64_t w, const void* Y, double scale,
                      const void* in, void* out, void* stream) {
  if ((precision != RK_FP64 && precision != RK_FP32) || n < 1 || w < 1 || !Y || !in || !out || in == out) {
    set_error("rk_dht: invalid argument (out must not alias in)");
    return RK_E_ARG;
  }
  const int64_t cols = w;
  const dim3 blk(16, 16), grd((unsigned)((w + 15) / 16), (unsigned)((n + 15) / 16));
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == RK_FP64) {
    const auto* y = static_cast<const double*>(Y);
    const auto* x = static_cast<const double*>(in);
    auto* o = static_cast<double*>(out);
    if (divide) dht_kernel<double, true><<<grd, blk, 0, st>>>(n, cols, y, scale, x, o);
    else dht_kernel<double, false><<<grd, blk, 0, st>>>(n, cols, y, scale, x, o);
  } else {
    const auto* y = static_cast<const float*>(Y);
    const auto* x = static_cast<const float*>(in);
    auto* o = static_cast<float*>(out);
    if (divide) dht_kernel<float, true><<<grd, blk, 0, st>>>(n, cols, y, (float)scale, x, o);
    else dht_kernel<float, false><<<grd, blk, 0, st>>>(n, cols, y, (float)scale, x, o);
  }
  return cuda_check(cudaGetLastError(), "rk_dht launch");
}
