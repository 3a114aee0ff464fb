// Shared-memory Stockham FFT executed cooperatively by one thread group.
//
// Radix-4 passes (plus one radix-2 pass when log2(N) is odd) in the autosort
// formulation: pass p (sub-transform length Ls before the pass) maps butterfly i to
// inputs x[i + r*N/R] and outputs y[(i - i%Ls)*R + i%Ls + r*Ls].  Twiddles come from a
// table tw[k] = exp(-2*pi*i*k/RK_TW_N) (FP64-accurate, stored in the working precision).
#pragma once

#include <utility>

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

// Per grid size n = 2^logn of a u*ux kernel: whether the packing is fused with the inverse
// transform's first pass and the split with the forward transform's last pass
// (pack_first_pass, fwd_last_split; both exchange values between lane pairs by shuffles
// instead of a pass through shared memory), and with it the pass plans.  Chosen by timing
// each grid-size class of the KS ensemble workload (about 1000 instances, ETD35 FP32, tf =
// 100) on a GB300, ms per class at its best launch shape:
//   n = 2048  fused,   inverse 8.8.8.4, forward 8.8.8.2   102.1   (unfused 16.16.8 / 16.8.8:
//             107.5; unfused 8.8.8.4: 112.5; fused 8.16.16 / 8.16.8: 107.1)
//   n = 1024  fused,   inverse 8.16.8,  forward 8.8.8      55.5   (unfused, 16.8.8 / 16.8.4: 57.2;
//             fused 8.8.8.2: 55.5)
//   n = 512   unfused, inverse 16.8.4,  forward 8.8.4      31.0   (fused, 8.8.8 / 8.8.4: 33.2)
//   n = 256   fused,   inverse 8.8.4,   forward 4.4.4.2    18.3   (unfused: 20.1)
// A fused pass runs one lane per butterfly and evaluates several modes per lane; where that
// leaves lanes of the group idle (n = 512 with 128-thread groups) the unfused form is
// faster.  At n = 2048 radix-8 passes keep every lane of a 128- or 256-thread group busy
// (a radix-16 pass has 128 butterflies) and need fewer registers, which pays for the fourth
// pass only together with the fused first and last passes.
__host__ __device__ constexpr bool uux_fused(int logn) { return logn == 8 || logn == 10 || logn == 11; }

// log2 of the radix of pass p of a size-2^logn transform (fwd: the forward n/2-point
// transform of a kernel of 2n points): 16 while >= 4 bits remain, preferring 8+8 over 16+4 /
// 16+2 splits of the last 6/5 bits; at most 8 for the first pass of a fused kernel's
// transforms (the paired first pass holds two columns' worth of values per lane pair); every
// radix is capped so that a pass has at least 32 butterflies (N / R >= 32), which keeps
// every lane of a one-warp group busy on the small transforms (n = 128, 256) instead of half
// or a quarter of them.
__host__ __device__ constexpr int pass_pick(int logn, int p, int left, bool fwd) {
  int lg = left >= 4 ? 4 : left;
  if (left == 6 || left == 5) lg = 3;
  if (left == 7) lg = 4;
  if (p == 0 && lg > 3 && uux_fused(fwd ? logn + 1 : logn)) lg = 3;
  if ((fwd ? logn + 1 : logn) == 11 && lg > 3) lg = 3;  // n = 2048: radix-8 passes only
  const int cap = logn - 5 < 1 ? 1 : logn - 5;
  return lg > cap ? cap : lg;
}

template <int LOGN, int P, bool FWD = false>
struct PassRadix {
  __host__ __device__ static constexpr int used() {
    int left = LOGN, lg = 0;
    for (int q = 0; q <= P; ++q) {
      lg = pass_pick(LOGN, q, left, FWD);
      left -= lg;
    }
    return lg;
  }
  __host__ __device__ static constexpr int bits_before() {
    int left = LOGN, done = 0;
    for (int q = 0; q < P; ++q) {
      const int lg = pass_pick(LOGN, q, left, FWD);
      left -= lg;
      done += lg;
    }
    return done;
  }
};

template <class T>
struct StoreY {
  RK_DEV void operator()(cx<T>* y, int, int pidx, cx<T> v) const { y[pidx] = v; }
};

}  // namespace rk

namespace rk {

// ---------------------------------------------------------------------------------
// Twiddle rows.  The compile-time u*ux transforms read their twiddles from one table per
// block: for every pass p (radix R, sub-length Ls > 1) of the 2^LOGN-point transform the rows
// T_p[(r - 1) Ls + k] = W_{R Ls}^{r k} (r = 1..R-1, k < Ls).  A pass reads T_p + k at the
// compile-time offsets (r - 1) Ls: consecutive lanes (consecutive k) hit consecutive
// entries, no bank conflicts and no per-twiddle index arithmetic.  The forward transform of
// 2^(LOGN-1) points needs W_{Rf Lsf}^{r k} = W_{Ri Lsi}^{(alpha r)(beta k)} with alpha beta
// = Ri Lsi / (Rf Lsf): a compile-time map onto a pass of the table (smallest beta, so the
// reads stay contiguous where they can).  The split formula's W_n^k, k < n/2, is row 1 of the
// last pass (W_n^s, s < Ls_last) times W_R^q, q = k / Ls_last (q < 4).  The table holds the
// values of the global table (same angles, same rounding), so the transforms are bitwise
// those of the full padded table it replaces, and it is smaller (n (R_last - 1)/R_last + a
// few entries against n + n/16).
// ---------------------------------------------------------------------------------
template <int LOGN, int P, bool FWD = false>
struct PassInfo {
  static constexpr int LGR = PassRadix<LOGN, P, FWD>::used();
  static constexpr int DONE = PassRadix<LOGN, P, FWD>::bits_before();
  static constexpr int R = 1 << LGR, Ls = 1 << DONE;
  static constexpr bool last = DONE + LGR == LOGN;
  static constexpr int rows = DONE > 0 ? (R - 1) * Ls : 0;  // table entries of this pass
};

__host__ __device__ constexpr int fft_passes(int logn, bool fwd = false) {
  int left = logn, p = 0;
  while (left > 0) {
    left -= pass_pick(logn, p, left, fwd);
    ++p;
  }
  return p;
}

// table offset of pass P's rows, and the table's size
template <int LOGN, int P>
__host__ __device__ constexpr int rows_offset() {
  if constexpr (P == 0) return 0;
  else return rows_offset<LOGN, P - 1>() + PassInfo<LOGN, P - 1>::rows;
}
template <int LOGN>
__host__ __device__ constexpr int twiddle_rows() {
  if constexpr (LOGN <= 0) return 0;  // runtime-size kernels keep no rows
  else return rows_offset<LOGN, fft_passes(LOGN) - 1>() + PassInfo<LOGN, fft_passes(LOGN) - 1>::rows;
}

// fill the rows of the 2^LOGN-point transform from the global table of RK_TW_N twiddles
template <class T, int LOGN, int P = 0>
RK_DEV void fill_twiddle_rows(cx<T>* tab, const cx<T>* __restrict__ tw, int tid, int nthr) {
  using I = PassInfo<LOGN, P>;
  if constexpr (I::rows > 0) {
    cx<T>* t = tab + rows_offset<LOGN, P>();
    for (int e = tid; e < I::rows; e += nthr) {
      const int r = e / I::Ls + 1, k = e % I::Ls;
      t[e] = tw[(r * k) * (RK_TW_N / (I::R * I::Ls))];
    }
  }
  if constexpr (!I::last) fill_twiddle_rows<T, LOGN, P + 1>(tab, tw, tid, nthr);
}

// map of forward pass PF of the 2^(LOGN-1) transform onto the rows: PI * 10000 + alpha * 100
// + beta, -1 if no pass serves it
template <int LOGN, int PF, int PI = 1>
__host__ __device__ constexpr int fwd_row_map() {
  using F = PassInfo<LOGN - 1, PF, true>;
  if constexpr (PI >= fft_passes(LOGN)) {
    return -1;
  } else {
    using I = PassInfo<LOGN, PI>;
    int best = -1;
    if (I::Ls > 1 && (I::R * I::Ls) % (F::R * F::Ls) == 0) {
      const int a = (I::R * I::Ls) / (F::R * F::Ls);
      for (int beta = 1; beta <= a; beta *= 2) {
        const int alpha = a / beta;
        if (alpha * (F::R - 1) <= I::R - 1 && beta * (F::Ls - 1) <= I::Ls - 1) {
          best = PI * 10000 + alpha * 100 + beta;
          break;
        }
      }
    }
    const int rest = fwd_row_map<LOGN, PF, PI + 1>();
    if (best < 0) return rest;
    if (rest < 0) return best;
    return (best % 100) <= (rest % 100) ? best : rest;
  }
}

// The R - 1 twiddles t_r = W^{r k} (r = 1..R-1) of one butterfly, t_r at tk[(ALPHA r - 1) LSI].
// FP64 reads every one.  FP32 reads t_1..t_3 and t_4, t_8, t_12 and forms the others as one
// product t_{4a + b} = t_{4a} t_b (b = 1..3): 6 shared-memory reads instead of 15 for radix
// 16, 4 instead of 7 for radix 8, each product within ~1.5 FP32 ulps of the table value.
// The reads were a fifth of the transforms' shared-memory wavefronts.
template <class T, int R, bool INV, int ALPHA, int LSI>
RK_DEV void load_twiddles(const cx<T>* __restrict__ tk, cx<T>* t) {
  if constexpr (sizeof(T) == sizeof(double) || R <= 4) {
#pragma unroll
    for (int r = 1; r < R; ++r) t[r] = twiddle<T, INV>(tk, (ALPHA * r - 1) * LSI);
  } else {
#pragma unroll
    for (int r = 1; r < 4; ++r) t[r] = twiddle<T, INV>(tk, (ALPHA * r - 1) * LSI);
#pragma unroll
    for (int a = 4; a < R; a += 4) {
      t[a] = twiddle<T, INV>(tk, (ALPHA * a - 1) * LSI);
#pragma unroll
      for (int b = 1; b < 4; ++b) t[a + b] = t[a] * t[b];
    }
  }
}

// One Stockham pass (as stockham_pass) with its twiddles W^{r k} at rows[(ALPHA r - 1) LSI +
// BETA k]
template <class T, int LOGN, int LGR, int LGLS, bool INV, int ALPHA, int BETA, int LSI, class Store>
RK_DEV void stockham_pass_rows(const Group& g, const cx<T>* __restrict__ x, const cx<T>* __restrict__ rows,
                               Store store) {
  constexpr int N = 1 << LOGN, R = 1 << LGR, Ls = 1 << LGLS, NB = N / R;
  for (int i = g.tid; i < NB; i += g.nthr) {
    const int k = i & (Ls - 1);
    const cx<T>* xi = x + fpad(i);
    cx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = xi[r * NB + ((r * NB) >> 4)];
    if constexpr (Ls > 1) {
      cx<T> t[R];
      load_twiddles<T, R, INV, ALPHA, LSI>(rows + BETA * k, t);
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = v[r] * t[r];
    }
    dft_reg<T, R, INV>(v);
    const int j = ((i - k) << LGR) + k;
    const int pj = fpad(j);
#pragma unroll
    for (int r = 0; r < R; ++r) store(j + r * Ls, pj + r * Ls + ((r * Ls) >> 4), v[r]);
  }
}

// the 2^LOGN-point transform (sign INV) through its own rows
template <class T, int LOGN, int P, bool INV, class FinalStore>
RK_DEV cx<T>* fft_rows(const Group& g, cx<T>* x, cx<T>* y, const cx<T>* tab, FinalStore fin) {
  using I = PassInfo<LOGN, P>;
  const cx<T>* rows = tab + rows_offset<LOGN, P>();
  if constexpr (I::last) {
    stockham_pass_rows<T, LOGN, I::LGR, I::DONE, INV, 1, 1, I::Ls>(
        g, x, rows, [&](int idx, int pidx, cx<T> v) { fin(y, idx, pidx, v); });
    g.sync();
    return y;
  } else {
    stockham_pass_rows<T, LOGN, I::LGR, I::DONE, INV, 1, 1, I::Ls>(g, x, rows,
                                                                   [&](int, int pidx, cx<T> v) { y[pidx] = v; });
    g.sync();
    return fft_rows<T, LOGN, P + 1, INV>(g, y, x, tab, fin);
  }
}

// Which rows serve forward pass P of the 2^(LOGN-1)-point transform: (pass of the rows,
// ALPHA, BETA) packed as fwd_row_map returns them; the first pass has no twiddles.
template <int LOGN, int P>
__host__ __device__ constexpr int fwd_map() {
  return PassInfo<LOGN - 1, P, true>::Ls > 1 ? fwd_row_map<LOGN, P>() : 10101;
}

// Forward 2^(LOGN-1)-point transform through the rows of the 2^LOGN-point one, every pass
// but the last; returns the buffer that holds the last pass's input.
template <class T, int LOGN, int P>
RK_DEV cx<T>* fft_half_rows_to_last(const Group& g, cx<T>* x, cx<T>* y, const cx<T>* tab) {
  using F = PassInfo<LOGN - 1, P, true>;
  if constexpr (F::last) {
    return x;
  } else {
    constexpr int MAP = fwd_map<LOGN, P>();
    static_assert(MAP >= 0, "no pass of the twiddle rows serves this forward pass");
    constexpr int PI = MAP / 10000, ALPHA = (MAP / 100) % 100, BETA = MAP % 100;
    const cx<T>* rows = tab + rows_offset<LOGN, PI>();
    stockham_pass_rows<T, LOGN - 1, F::LGR, F::DONE, false, ALPHA, BETA, PassInfo<LOGN, PI>::Ls>(
        g, x, rows, [&](int, int pidx, cx<T> v) { y[pidx] = v; });
    g.sync();
    return fft_half_rows_to_last<T, LOGN, P + 1>(g, y, x, tab);
  }
}

// value of a complex pair from the partner lane of paired_column (lane index ^ 16)
template <class T>
RK_DEV cx<T> shfl_pair(cx<T> v) {
  return cx<T>{__shfl_xor_sync(0xffffffffu, v.x, 16), __shfl_xor_sync(0xffffffffu, v.y, 16)};
}

// Paired columns of a pass with NB butterflies (NB a multiple of 32).  Iteration tt of a loop
// over tt < NB: in each warp, lane l < 16 takes the column q = 16 w + l (w: the warp's 32-wide
// slice of tt, pair_unit) and lane l + 16 its mirror NB - q (q = 0: 0 and NB/2), the two
// columns whose values are each other's mirror images in a Hermitian-symmetric spectrum.  All
// lanes of a warp run the same iterations, so shfl_pair is safe inside the loop.  Pairing
// across half-warps, not adjacent lanes, puts each half-warp on 16 consecutive columns: the
// fused passes' stride-R stores and loads of shared memory then meet fewer bank conflicts
// (3-4% of the n = 2048, 1024 and 256 class kernels' time).
RK_DEV int pair_unit(int tt) { return ((tt >> 5) << 4) + (tt & 15); }
RK_DEV int paired_column(int tt, int nb) {
  const int unit = pair_unit(tt);
  return (tt & 16) == 0 ? unit : (unit == 0 ? nb / 2 : nb - unit);
}

// compile-time loop: f(std::integral_constant<int, r>) for r = 0 .. N-1
template <int N, class F, int... R>
RK_DEV void static_for_impl(F&& f, std::integer_sequence<int, R...>) {
  (f(std::integral_constant<int, R>{}), ...);
}
template <int N, class F>
RK_DEV void static_for(F&& f) {
  static_for_impl<N>(f, std::make_integer_sequence<int, N>{});
}

// v W_R^q, q < 4, R the radix of the last pass (4 or 8)
template <class T, int R>
RK_DEV cx<T> mul_wr(cx<T> v, int q) {
  static_assert(R == 4 || R == 8 || R == 16, "split twiddles need a last pass of radix 4, 8 or 16");
  if constexpr (R == 16) {
    return q == 0 ? v : q == 1 ? mul_w16<T, false, 1>(v) : q == 2 ? mul_w16<T, false, 2>(v) : mul_w16<T, false, 3>(v);
  } else if constexpr (R == 4) {
    return q == 0 ? v : mul_mi(v);
  } else {
    const T h = T(0.7071067811865476);
    if (q == 0) return v;
    if (q == 2) return mul_mi(v);
    return v * (q == 1 ? cx<T>{h, -h} : cx<T>{-h, -h});
  }
}

}  // namespace rk
