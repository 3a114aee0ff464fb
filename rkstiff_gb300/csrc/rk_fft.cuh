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

namespace rk {

// ---------------------------------------------------------------------------------
// Compile-time-size FFT: Stockham passes of radix 16/8/4/2 with the butterfly held in
// registers.  LOGN = sum of the pass radices' log2; one barrier per pass.
// ---------------------------------------------------------------------------------

// multiply by W_16^e = exp(-+2 pi i e/16) with e a compile-time constant
template <class T, bool INV, int E>
RK_DEV cx<T> mul_w16(cx<T> v) {
  constexpr int e = E & 15;
  if constexpr (e == 0) return v;
  else if constexpr (e == 4) return INV ? mul_i(v) : mul_mi(v);
  else if constexpr (e == 8) return -v;
  else if constexpr (e == 12) return INV ? mul_mi(v) : mul_i(v);
  else {
    // W = cos(2 pi e/16) -/+ i sin(2 pi e/16); sin(2 pi e/16) = cos(2 pi (e - 4)/16)
    constexpr double c = e == 1 ? 0.9238795325112867 : e == 2 ? 0.7071067811865476 : e == 3 ? 0.3826834323650898
                       : e == 5 ? -0.3826834323650898 : e == 6 ? -0.7071067811865476 : e == 7 ? -0.9238795325112867
                       : e == 9 ? -0.9238795325112867 : e == 10 ? -0.7071067811865476 : e == 11 ? -0.3826834323650898
                       : e == 13 ? 0.3826834323650898 : e == 14 ? 0.7071067811865476 : 0.9238795325112867;
    constexpr double s = e == 1 ? 0.3826834323650898 : e == 2 ? 0.7071067811865476 : e == 3 ? 0.9238795325112867
                       : e == 5 ? 0.9238795325112867 : e == 6 ? 0.7071067811865476 : e == 7 ? 0.3826834323650898
                       : e == 9 ? -0.3826834323650898 : e == 10 ? -0.7071067811865476 : e == 11 ? -0.9238795325112867
                       : e == 13 ? -0.9238795325112867 : e == 14 ? -0.7071067811865476 : -0.3826834323650898;
    const T cc = T(c), ss = INV ? T(s) : T(-s);
    return cx<T>{v.x * cc - v.y * ss, v.x * ss + v.y * cc};
  }
}

// Padded shared-memory index of complex element c: one spare slot per 16 elements, so a
// pass that stores at a stride of 16 elements spreads over the banks.
RK_HD constexpr int fpad(int c) { return c + (c >> 4); }
// complex slots a padded buffer of n elements occupies
RK_HD constexpr int fpad_size(int n) { return n + (n >> 4); }

template <class T, bool INV>
RK_DEV void dft2(cx<T>& a, cx<T>& b) {
  cx<T> t = a - b;
  a = a + b;
  b = t;
}

// In-register DFT of size R in natural order: v[k] <- sum_j v[j] W_R^{jk}.
template <class T, int R, bool INV>
RK_DEV void dft_reg(cx<T>* v) {
  if constexpr (R == 2) {
    dft2<T, INV>(v[0], v[1]);
  } else if constexpr (R == 4) {
    dft4<T, INV>(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    // 8 = 2 x 4: inner 4-point DFTs over the even/odd halves, twiddle, 2-point combine
    cx<T> e[4] = {v[0], v[2], v[4], v[6]};
    cx<T> o[4] = {v[1], v[3], v[5], v[7]};
    dft4<T, INV>(e[0], e[1], e[2], e[3]);
    dft4<T, INV>(o[0], o[1], o[2], o[3]);
    o[1] = mul_w16<T, INV, 2>(o[1]);
    o[2] = mul_w16<T, INV, 4>(o[2]);
    o[3] = mul_w16<T, INV, 6>(o[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = e[k] + o[k];
      v[k + 4] = e[k] - o[k];
    }
  } else {
    static_assert(R == 16, "radix must be 2, 4, 8 or 16");
    // 16 = 4 x 4: y[k1][n2] = DFT4 over n1 of x[4 n1 + n2]; twiddle W16^{n2 k1};
    // X[k1 + 4 k2] = DFT4 over n2 of y[k1][n2]
    cx<T> w[16];
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
      cx<T> a0 = v[n2], a1 = v[4 + n2], a2 = v[8 + n2], a3 = v[12 + n2];
      dft4<T, INV>(a0, a1, a2, a3);
      w[0 * 4 + n2] = a0;
      w[1 * 4 + n2] = a1;
      w[2 * 4 + n2] = a2;
      w[3 * 4 + n2] = a3;
    }
    w[5] = mul_w16<T, INV, 1>(w[5]);
    w[6] = mul_w16<T, INV, 2>(w[6]);
    w[7] = mul_w16<T, INV, 3>(w[7]);
    w[9] = mul_w16<T, INV, 2>(w[9]);
    w[10] = mul_w16<T, INV, 4>(w[10]);
    w[11] = mul_w16<T, INV, 6>(w[11]);
    w[13] = mul_w16<T, INV, 3>(w[13]);
    w[14] = mul_w16<T, INV, 6>(w[14]);
    w[15] = mul_w16<T, INV, 9>(w[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      cx<T> a0 = w[4 * k1], a1 = w[4 * k1 + 1], a2 = w[4 * k1 + 2], a3 = w[4 * k1 + 3];
      dft4<T, INV>(a0, a1, a2, a3);
      v[k1] = a0;
      v[k1 + 4] = a1;
      v[k1 + 8] = a2;
      v[k1 + 12] = a3;
    }
  }
}

// radix of pass p for a size-2^LOGN transform: 16 while >= 4 bits remain, then the rest,
// preferring 8+8 over 16+4 / 16+2 splits of the last 6/5 bits; the radix is capped so that
// a pass has at least 32 butterflies (N / R >= 32), which keeps every lane of a one-warp
// group busy on the small transforms (n = 128, 256) instead of half or a quarter of them.
template <int LOGN, int P>
struct PassRadix {
  __host__ __device__ static constexpr int pick(int left) {
    int lg = left >= 4 ? 4 : left;
    if (left == 6 || left == 5) lg = 3;
    if (left == 7) lg = 4;
    const int cap = LOGN - 5 < 1 ? 1 : LOGN - 5;
    return lg > cap ? cap : lg;
  }
  __host__ __device__ static constexpr int used() {
    int left = LOGN, lg = 0;
    for (int q = 0; q <= P; ++q) {
      lg = pick(left);
      left -= lg;
    }
    return lg;
  }
  __host__ __device__ static constexpr int bits_before() {
    int left = LOGN, done = 0;
    for (int q = 0; q < P; ++q) {
      const int lg = pick(left);
      left -= lg;
      done += lg;
    }
    return done;
  }
};

// One Stockham pass of radix R = 2^LGR at sub-length Ls = 2^LGLS over N = 2^LOGN points.
// `store(idx, pidx, value)` receives each output with its unpadded index and its padded
// position fpad(idx).  With power-of-two R, Ls and NB the padded positions of a butterfly's
// inputs i + r NB and outputs j + r Ls are its base position plus compile-time offsets
// (fpad(a + b) = fpad(a) + b + (b >> 4) for these b), so each load and store needs no
// index arithmetic of its own.
template <class T, int LOGN, int LGR, int LGLS, bool INV, int TWLOG, class Store>
RK_DEV void stockham_pass(const Group& g, const cx<T>* __restrict__ x, const cx<T>* __restrict__ tw, Store store) {
  constexpr int N = 1 << LOGN, R = 1 << LGR, Ls = 1 << LGLS, NB = N / R;
  constexpr int TWS = (1 << TWLOG) >> (LGLS + LGR);  // table stride of W_{R Ls}
  for (int i = g.tid; i < NB; i += g.nthr) {
    const int k = i & (Ls - 1);
    const cx<T>* xi = x + fpad(i);
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = xi[r * NB + ((r * NB) >> 4)];
    if constexpr (Ls > 1) {
      // twiddle tables of 2^TWLOG <= 4096 entries live in shared memory at padded
      // positions (strided reads would otherwise fall into a few banks)
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = v[r] * twiddle<T, INV>(tw, fpad(r * k * TWS));
    }
    dft_reg<T, R, INV>(v);
    const int j = ((i - k) << LGR) + k;
    const int pj = fpad(j);
#pragma unroll
    for (int r = 0; r < R; ++r) store(j + r * Ls, pj + r * Ls + ((r * Ls) >> 4), v[r]);
  }
}

template <class T, int LOGN, int P, bool INV, int TWLOG, class FinalStore>
RK_DEV cx<T>* fft_ct_passes(const Group& g, cx<T>* x, cx<T>* y, const cx<T>* tw, FinalStore fin) {
  constexpr int LGR = PassRadix<LOGN, P>::used();
  constexpr int DONE = PassRadix<LOGN, P>::bits_before();
  if constexpr (DONE + LGR == LOGN) {
    // final pass: outputs go to fin(y, index, value); y is the buffer not being read
    stockham_pass<T, LOGN, LGR, DONE, INV, TWLOG>(g, x, tw, [&](int idx, int pidx, cx<T> v) { fin(y, idx, pidx, v); });
    g.sync();
    return y;
  } else {
    stockham_pass<T, LOGN, LGR, DONE, INV, TWLOG>(g, x, tw, [&](int, int pidx, cx<T> v) { y[pidx] = v; });
    g.sync();
    return fft_ct_passes<T, LOGN, P + 1, INV, TWLOG>(g, y, x, tw, fin);
  }
}

// FFT of 2^LOGN points held in `a` at padded positions fpad(i) (`b` is scratch of the same
// size), with `tw` a table of the 2^TWLOG twiddles exp(-2 pi i k/2^TWLOG), TWLOG >= LOGN,
// stored at padded positions fpad(k).
// The final pass hands every output to fin(y, index, padded index, value), where y is the
// buffer that pass does not read and `index` the unpadded output index; returns y.  All group threads
// call.
template <class T, int LOGN, bool INV, int TWLOG, class FinalStore>
RK_DEV cx<T>* fft_ct(const Group& g, cx<T>* a, cx<T>* b, const cx<T>* tw, FinalStore fin) {
  return fft_ct_passes<T, LOGN, 0, INV, TWLOG>(g, a, b, tw, fin);
}

template <class T>
struct StoreY {
  RK_DEV void operator()(cx<T>* y, int, int pidx, cx<T> v) const { y[pidx] = v; }
};

}  // namespace rk
