// Device grid and derivative helpers: the Fourier and Chebyshev grids of rkstiff/grids.py
// and the spectral derivatives of rkstiff/derivatives.py, computed on the GPU so that a
// problem's set-up need not leave the device.
//
// Grids follow NumPy's arithmetic step by step (arange fills start + i*delta with
// delta = (start + step) - start; fftfreq / rfftfreq scale integer indices by
// 1 / (n d)); every product and sum is rounded separately (no fused multiply-add), so the
// Fourier grids are bitwise those of the reference.  The derivatives transform one row per
// block with the library's shared-memory Stockham FFT (FP64).
#include <cuda_runtime.h>

#include <string>

#include "rk_fft.cuh"
#include "rk_launch.h"

namespace rk {
namespace grid {

// x_j = a + j*delta, delta = (a + dx) - a (numpy.arange); kx = 2 pi (k / (n dx)) with k the
// rfftfreq (0..n/2) or fftfreq (0..(n-1)/2, -(n/2)..-1) integers (numpy.fft.*freq)
__global__ void fourier_grid_kernel(int real_grid, int64_t n, double a, double dx, double* x, double* kx) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double delta = __dsub_rn(__dadd_rn(a, dx), a);
  if (x && j < n) x[j] = __dadd_rn(a, __dmul_rn((double)j, delta));
  const int64_t m = real_grid ? n / 2 + 1 : n;
  if (kx && j < m) {
    const double val = __ddiv_rn(1.0, __dmul_rn((double)n, dx));
    int64_t k = j;
    if (!real_grid && j >= (n - 1) / 2 + 1) k = j - n;
    kx[j] = __dmul_rn(6.283185307179586, __dmul_rn((double)k, val));
  }
}

// Chebyshev extreme points on [a, b] (numpy.polynomial.chebyshev.chebpts2 mapped as
// a + (b - a)(x + 1)/2) and the first-derivative matrix (Trefethen, Spectral Methods in
// MATLAB, cheb.m): D_ij = c_i/c_j / (x_i - x_j) off the diagonal with
// c = (2, 1, ..., 1, 2) * (-1)^i, the diagonal minus the row sum.
__global__ void cheb_points_kernel(int64_t n, double a, double b, double* x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n) return;
  // numpy.linspace(-pi, 0, n + 1): i * step + start, the last point exactly 0
  const double step = __ddiv_rn(3.141592653589793, (double)n);
  const double t = i == n ? 0.0 : __dadd_rn(__dmul_rn((double)i, step), -3.141592653589793);
  const double c = cos(t);
  x[i] = __dadd_rn(a, __ddiv_rn(__dmul_rn(__dsub_rn(b, a), __dadd_rn(c, 1.0)), 2.0));
}

__device__ __forceinline__ double cheb_c(int64_t i, int64_t n) {
  const double c = (i == 0 || i == n) ? 2.0 : 1.0;
  return (i & 1) ? -c : c;
}

// one block per row: off-diagonal entries, then the diagonal as minus the row sum (summed in
// column order, as numpy's row sum of a small matrix)
__global__ void cheb_matrix_kernel(int64_t n, const double* x, double* D) {
  const int64_t i = blockIdx.x;
  const int64_t N1 = n + 1;
  const double ci = cheb_c(i, n), xi = x[i];
  for (int64_t j = threadIdx.x; j < N1; j += blockDim.x) {
    if (j == i) continue;
    const double q = __ddiv_rn(ci, cheb_c(j, n));
    D[i * N1 + j] = __ddiv_rn(q, __dsub_rn(xi, x[j]));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the diagonal of outer(c, 1/c) / (dX + I) is 1; the trick subtracts the full row sum
    double s = 1.0;
    for (int64_t j = 0; j < N1; ++j)
      if (j != i) s = __dadd_rn(s, D[i * N1 + j]);
    D[i * N1 + i] = __dsub_rn(1.0, s);
  }
}

// (i kx)^p = i^p kx^p, kx^p by repeated products
__device__ __forceinline__ cx<double> ikx_pow(double k, int p) {
  double r = 1.0;
  for (int q = 0; q < p; ++q) r *= k;
  switch (p & 3) {
    case 0: return cx<double>{r, 0.0};
    case 1: return cx<double>{0.0, r};
    case 2: return cx<double>{-r, 0.0};
    default: return cx<double>{0.0, -r};
  }
}

// One row per block: F = fft(u); multiply by (i kx)^p; inverse transform; / n.  REAL: u is
// real, only the n/2 + 1 non-negative modes are scaled and the inverse is Hermitian with the
// imaginary parts of the DC bin (and, n even, the Nyquist bin) dropped -- numpy.fft.irfft's
// convention.  POW2: n a power of two, Stockham FFTs over the RK_TW_N table; otherwise direct
// DFTs over a table of the n roots of unity (any n: the reference's own tests use n = 100
// and 400).
template <bool REAL, bool POW2>
__global__ void __launch_bounds__(256) dx_fourier_kernel(int n, int logn, int order, const double* __restrict__ kx,
                                                         const void* __restrict__ u, void* __restrict__ out,
                                                         const cx<double>* __restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smem[];
  cx<double>* fa = reinterpret_cast<cx<double>*>(smem);
  cx<double>* fb = fa + n;
  cx<double>* fc = fb + n;  // !POW2 only
  const Group g{(int)threadIdx.x, (int)blockDim.x, 0};
  const int64_t row = blockIdx.x;
  if (REAL) {
    const double* ur = static_cast<const double*>(u) + row * n;
    for (int j = g.tid; j < n; j += g.nthr) fa[j] = cx<double>{ur[j], 0.0};
  } else {
    const cx<double>* uc = static_cast<const cx<double>*>(u) + row * n;
    for (int j = g.tid; j < n; j += g.nthr) fa[j] = uc[j];
  }
  if (!POW2) {
    // w[k] = exp(-2 pi i k / n)
    for (int k = g.tid; k < n; k += g.nthr) {
      double sn, cs;
      sincospi(2.0 * (double)k / (double)n, &sn, &cs);
      fb[k] = cx<double>{cs, -sn};
    }
  }
  g.sync();
  cx<double>* F;
  if (POW2) {
    F = fft_group<double, false>(g, fa, fb, logn, tw);
  } else {
    for (int k = g.tid; k < n; k += g.nthr) {
      cx<double> acc{0.0, 0.0};
      int idx = 0;
      for (int j = 0; j < n; ++j) {
        acc = acc + fa[j] * fb[idx];
        idx += k;
        if (idx >= n) idx -= n;
      }
      fc[k] = acc;
    }
    g.sync();
    F = fc;
  }
  cx<double>* Z = POW2 ? (F == fa ? fb : fa) : fa;
  const int M = n / 2;
  if (REAL) {
    for (int k = g.tid; k <= M; k += g.nthr) {
      cx<double> c = F[k] * ikx_pow(kx[k], order);
      if (k == 0 || (k == M && (n & 1) == 0)) c.y = 0.0;
      Z[k] = c;
      if (k > 0 && n - k > M) Z[n - k] = conj(c);
    }
  } else {
    for (int k = g.tid; k < n; k += g.nthr) Z[k] = F[k] * ikx_pow(kx[k], order);
  }
  g.sync();
  const double inv = 1.0 / (double)n;
  if (POW2) {
    cx<double>* G = fft_group<double, true>(g, Z, F, logn, tw);
    if (REAL) {
      double* o = static_cast<double*>(out) + row * n;
      for (int j = g.tid; j < n; j += g.nthr) o[j] = G[j].x * inv;
    } else {
      cx<double>* o = static_cast<cx<double>*>(out) + row * n;
      for (int j = g.tid; j < n; j += g.nthr) o[j] = G[j] * inv;
    }
  } else {
    for (int j = g.tid; j < n; j += g.nthr) {
      cx<double> acc{0.0, 0.0};
      int idx = 0;
      for (int k = 0; k < n; ++k) {
        acc = acc + Z[k] * conj(fb[idx]);
        idx += j;
        if (idx >= n) idx -= n;
      }
      if (REAL) static_cast<double*>(out)[row * n + j] = acc.x * inv;
      else static_cast<cx<double>*>(out)[row * n + j] = acc * inv;
    }
  }
}

template <bool REAL, bool POW2>
static int launch_dx(int n, int logn, int order, int64_t rows, const double* kx, const void* u, void* out,
                     const cx<double>* tw, cudaStream_t s) {
  const size_t sm = (POW2 ? 2 : 3) * (size_t)n * sizeof(cx<double>);
  if (int e = cuda_check(cudaFuncSetAttribute(dx_fourier_kernel<REAL, POW2>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
                         "rk_dx_fourier smem"))
    return e;
  dx_fourier_kernel<REAL, POW2><<<(unsigned)rows, 256, sm, s>>>(n, logn, order, kx, u, out, tw);
  return cuda_check(cudaGetLastError(), "rk_dx_fourier launch");
}

// C = A B for n x n row-major FP64 matrices, B with `cols` columns (ld = cols); 16 x 16 tiles
__global__ void dgemm_kernel(int64_t n, int64_t cols, const double* __restrict__ A, const double* __restrict__ B,
                             double* __restrict__ C) {
  __shared__ double as[16][17], bs[16][17];
  const int64_t r = (int64_t)blockIdx.y * 16 + threadIdx.y, c = (int64_t)blockIdx.x * 16 + threadIdx.x;
  double acc = 0.0;
  for (int64_t k0 = 0; k0 < n; k0 += 16) {
    const int64_t ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
    as[threadIdx.y][threadIdx.x] = (r < n && ka < n) ? A[r * n + ka] : 0.0;
    bs[threadIdx.y][threadIdx.x] = (kb < n && c < cols) ? B[kb * cols + c] : 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) acc = fma(as[threadIdx.y][k], bs[k][threadIdx.x], acc);
    __syncthreads();
  }
  if (r < n && c < cols) C[r * cols + c] = acc;
}

static int gemm(int64_t n, int64_t cols, const double* A, const double* B, double* C, cudaStream_t s) {
  const dim3 blk(16, 16), grd((unsigned)((cols + 15) / 16), (unsigned)((n + 15) / 16));
  dgemm_kernel<<<grd, blk, 0, s>>>(n, cols, A, B, C);
  return cuda_check(cudaGetLastError(), "dx_cheb product launch");
}

}  // namespace grid
}  // namespace rk

using namespace rk;
using namespace rk::grid;

extern "C" int rk_fourier_grid(int32_t real_grid, int64_t n, double a, double dx, double* x, double* kx,
                               void* stream) {
  if (n < 4 || (n & 1) || (!x && !kx)) {
    set_error("rk_fourier_grid: n must be an even integer greater than 2 and an output given");
    return RK_E_ARG;
  }
  const unsigned blocks = (unsigned)((n + 255) / 256);
  fourier_grid_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(real_grid ? 1 : 0, n, a, dx, x, kx);
  return cuda_check(cudaGetLastError(), "rk_fourier_grid launch");
}

extern "C" int rk_cheb_grid(int64_t n, double a, double b, double* x, double* D, void* stream) {
  if (n < 2 || n > 65535 || !x) {
    set_error("rk_cheb_grid: n must be in [2, 65535] and x given");
    return RK_E_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cheb_points_kernel<<<(unsigned)((n + 256) / 256), 256, 0, s>>>(n, a, b, x);
  if (int e = cuda_check(cudaGetLastError(), "rk_cheb_grid launch")) return e;
  if (!D) return RK_OK;
  cheb_matrix_kernel<<<(unsigned)(n + 1), 128, 0, s>>>(n, x, D);
  return cuda_check(cudaGetLastError(), "rk_cheb_grid matrix launch");
}

extern "C" int rk_dx_fourier(int32_t real_grid, int32_t order, int64_t n, int64_t rows, const double* kx,
                             const void* u, void* out, const void* twiddle64, void* stream) {
  if (order < 0 || rows < 0 || !kx || !u || !out || !twiddle64) {
    set_error("rk_dx_fourier: invalid argument");
    return RK_E_ARG;
  }
  if (n < 2 || n > 4096) {
    set_error("rk_dx_fourier: n must be in [2, 4096]");
    return RK_E_SIZE;
  }
  if (rows == 0) return RK_OK;
  const bool pow2 = (n & (n - 1)) == 0 && n >= 4;
  int logn = 0;
  while ((1 << logn) < n) ++logn;
  cudaStream_t s = (cudaStream_t)stream;
  const auto* tw = static_cast<const cx<double>*>(twiddle64);
  const int ni = (int)n;
  if (real_grid)
    return pow2 ? launch_dx<true, true>(ni, logn, order, rows, kx, u, out, tw, s)
                : launch_dx<true, false>(ni, logn, order, rows, kx, u, out, tw, s);
  return pow2 ? launch_dx<false, true>(ni, logn, order, rows, kx, u, out, tw, s)
              : launch_dx<false, false>(ni, logn, order, rows, kx, u, out, tw, s);
}

extern "C" int64_t rk_dx_cheb_work_bytes(int64_t n) { return n > 0 ? 2 * n * n * (int64_t)sizeof(double) : 0; }

extern "C" int rk_dx_cheb(int32_t order, int64_t n, int64_t cols, const double* D, const double* u, double* out,
                          void* work, void* stream) {
  if (order < 1 || n < 1 || cols < 1 || !D || !u || !out || (order > 1 && !work)) {
    set_error("rk_dx_cheb: invalid argument");
    return RK_E_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (order == 1) return gemm(n, cols, D, u, out, s);
  // D^order by repeated products left to right (D D, then (D D) D, ...), then times u
  double* P = static_cast<double*>(work);
  double* Q = P + n * n;
  if (int e = gemm(n, n, D, D, P, s)) return e;
  for (int q = 3; q <= order; ++q) {
    if (int e = gemm(n, n, P, D, Q, s)) return e;
    double* t = P;
    P = Q;
    Q = t;
  }
  return gemm(n, cols, P, u, out, s);
}
