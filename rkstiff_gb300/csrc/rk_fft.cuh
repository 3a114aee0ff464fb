// Shared-memory Stockham FFT executed cooperatively by one thread group.
//
// Radix-4 passes (plus one radix-2 pass when log2(N) is odd) in the autosort
// formulation: pass p (sub-transform length Ls before the pass) maps butterfly i to
// inputs x[i + r*N/R] and outputs y[(i - i%Ls)*R + i%Ls + r*Ls].  Twiddles come from a
// table tw[k] = exp(-2*pi*i*k/RK_TW_N) (FP64-accurate, stored in the working precision).
#pragma once

#include "rk_common.cuh"

namespace rk {

// forward: sign = -1 (exp(-2 pi i jk/N)); inverse: sign = +1 (unnormalised).
template <class T, bool INV>
RK_DEV cx<T> twiddle(const cx<T>* __restrict__ tw, int idx) {
  cx<T> w = tw[idx];
  return INV ? conj(w) : w;
}

template <class T, bool INV>
RK_DEV void dft4(cx<T>& a0, cx<T>& a1, cx<T>& a2, cx<T>& a3) {
  cx<T> s02 = a0 + a2, d02 = a0 - a2;
  cx<T> s13 = a1 + a3, d13 = a1 - a3;
  // forward: X1 = d02 - i d13, X3 = d02 + i d13; inverse flips the sign of i
  cx<T> t = INV ? mul_i(d13) : mul_mi(d13);
  a0 = s02 + s13;
  a2 = s02 - s13;
  a1 = d02 + t;
  a3 = d02 - t;
}

// In-place-by-ping-pong FFT of length N = 2^logn held in `a`; `b` is scratch of the same
// size.  Returns the buffer that holds the result (a or b).  All group threads must call.
template <class T, bool INV>
RK_DEV cx<T>* fft_group(const Group& g, cx<T>* __restrict__ a, cx<T>* __restrict__ b, int logn,
                        const cx<T>* __restrict__ tw) {
  const int N = 1 << logn;
  cx<T>* x = a;
  cx<T>* y = b;
  int Ls = 1;
  int lgLs = 0;
  if (logn & 1) {
    // radix-2 first pass (Ls = 1: no twiddles)
    const int half = N >> 1;
    for (int i = g.tid; i < half; i += g.nthr) {
      cx<T> u0 = x[i], u1 = x[i + half];
      y[2 * i] = u0 + u1;
      y[2 * i + 1] = u0 - u1;
    }
    g.sync();
    cx<T>* t = x; x = y; y = t;
    Ls = 2;
    lgLs = 1;
  }
  const int quarter = N >> 2;
  // table stride for exp(-2 pi i r k / (4 Ls)): RK_TW_N / (4 Ls)
  while (Ls < N) {
    const int tstride = RK_TW_N >> (lgLs + 2);
    for (int i = g.tid; i < quarter; i += g.nthr) {
      const int k = i & (Ls - 1);
      cx<T> u0 = x[i];
      cx<T> u1 = x[i + quarter];
      cx<T> u2 = x[i + 2 * quarter];
      cx<T> u3 = x[i + 3 * quarter];
      if (Ls > 1) {
        u1 = u1 * twiddle<T, INV>(tw, k * tstride);
        u2 = u2 * twiddle<T, INV>(tw, 2 * k * tstride);
        u3 = u3 * twiddle<T, INV>(tw, 3 * k * tstride);
      }
      dft4<T, INV>(u0, u1, u2, u3);
      const int j = ((i - k) << 2) + k;
      y[j] = u0;
      y[j + Ls] = u1;
      y[j + 2 * Ls] = u2;
      y[j + 3 * Ls] = u3;
    }
    g.sync();
    cx<T>* t = x; x = y; y = t;
    Ls <<= 2;
    lgLs += 2;
  }
  return x;
}

}  // namespace rk
