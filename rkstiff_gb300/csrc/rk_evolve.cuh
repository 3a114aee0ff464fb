// Persistent evolve kernel: one thread group per instance runs the reference's evolve
// loop (rkstiff/solveras.py:556-650 or solvercs.py:191-279) entirely on the device.
//
// Per attempt: coefficients when h changed (FP64, rkstiff/etd35.py:842-855), the stage
// program of the method with the built-in nonlinearity evaluated by in-shared-memory
// FFTs, the masked error norm accumulated in FP64 (solveras.py:451-455), and the
// accept/reject rule (solveras.py:384-410, 457-554).
#pragma once

#include <type_traits>

#include "rk_coeffs.cuh"
#include "rk_dd.cuh"
#include "rk_common.cuh"
#include "rk_fft.cuh"
#include "rk_mlp.cuh"

namespace rk {

// ---------------------------------------------------------------------------------
// method traits: NN stage arrays N1..NN, NC coefficient arrays, order q
// ---------------------------------------------------------------------------------
template <int M> struct Traits;
template <> struct Traits<RK_ETD35> { enum { NN = 6, NC = C35_N, Q = 4, ADAPT = 1, FSAL = 0 }; };
template <> struct Traits<RK_ETD5> { enum { NN = 6, NC = C35_N, Q = 0, ADAPT = 0, FSAL = 0 }; };
template <> struct Traits<RK_ETD34> { enum { NN = 5, NC = C34_N, Q = 4, ADAPT = 1, FSAL = 1 }; };
template <> struct Traits<RK_ETD4> { enum { NN = 4, NC = C34_N, Q = 0, ADAPT = 0, FSAL = 0 }; };
template <> struct Traits<RK_IF34> { enum { NN = 5, NC = CIF_N, Q = 4, ADAPT = 1, FSAL = 1 }; };
template <> struct Traits<RK_IF4> { enum { NN = 4, NC = CIF_N, Q = 0, ADAPT = 0, FSAL = 0 }; };
template <> struct Traits<RK_IF45DP> { enum { NN = 7, NC = CDP_N, Q = 5, ADAPT = 1, FSAL = 1 }; };

RK_HD int64_t round_up4(int64_t m) { return (m + 3) & ~int64_t(3); }

RK_HD int traits_nn(int method) {
  switch (method) {
    case RK_ETD35: case RK_ETD5: return 6;
    case RK_ETD34: case RK_IF34: return 5;
    case RK_ETD4: case RK_IF4: return 4;
    case RK_IF45DP: return 7;
  }
  return 0;
}

// ETD35 / ETD5 write the new state into N2's array: neither the new state nor the error
// combination reads N2 (etd35.py:337-344, etd5.py:248-252; a72 = 0), so the method needs one
// state vector fewer -- 7 complex vectors u, N1..N6 instead of 8
RK_HD constexpr bool unew_in_n2(int method) { return method == RK_ETD35 || method == RK_ETD5; }

// complex vectors of an instance's scratch
RK_HD int traits_nv(int method) { return traits_nn(method) + (unew_in_n2(method) ? 1 : 2); }

// bytes of an instance's scratch: u, unew, N1..NN (complex T), the coefficient block and,
// in FP32, a working-precision copy of the wavenumbers (read once per nonlinear evaluation
// per mode; converting the FP64 input there would put a conversion per mode on the FP64 pipe)
// bytes after the coefficient blocks: their h tags (RK_COEF_BLOCKS_MAX doubles) and the
// index of the block the next miss replaces
constexpr int64_t RK_TAG_BYTES = 8 * (RK_COEF_BLOCKS_MAX + 4);

// FP32 ETD35 / ETD5 carry the state in double-float: two more complex
// vectors after the stage vectors (the low FP32 words of u and of the new state) and one more
// array in each coefficient block (the low word of E = e^z of the final combination).  The
// stages and transforms stay FP32; only unew = E u + S is formed in double-float.
RK_HD constexpr bool df_state(int method, int precision, int coef_complex) {
  return precision == RK_FP32 && unew_in_n2(method) && coef_complex >= 0;
}
// complex vectors and coefficient arrays (per block) of an instance's slab
RK_HD int slab_nv(int method, int precision, int coef_complex) {
  return traits_nv(method) + (df_state(method, precision, coef_complex) ? 2 : 0);
}
RK_HD int slab_nc(int method, int precision, int coef_complex) {
  return num_coeffs(method) + (df_state(method, precision, coef_complex) ? 1 : 0);
}

RK_HD int64_t slab_bytes(int method, int precision, int coef_complex, int64_t m, int blocks = 1) {
  const int64_t mp = round_up4(m);
  const int64_t ts = precision == RK_FP64 ? 8 : 4;
  const int64_t vec = 2 * ts * mp;
  const int64_t coef = (coef_complex ? 2 : 1) * ts * mp;
  const int64_t kxw = precision == RK_FP64 ? 0 : ts * mp;
  const int64_t nc = slab_nc(method, precision, coef_complex);
  // with several coefficient blocks: the extra blocks, then their h tags
  const int64_t extra = blocks > 1 ? (blocks - 1) * nc * coef + RK_TAG_BYTES : 0;
  return slab_nv(method, precision, coef_complex) * vec + nc * coef + kxw + extra;
}

// the same counts at compile time for a kernel instantiation
template <class T, class CT, int METHOD>
struct SlabShape {
  static constexpr bool DF = sizeof(T) == sizeof(float) && unew_in_n2(METHOD);
  static constexpr int NV = Traits<METHOD>::NN + (unew_in_n2(METHOD) ? 1 : 2);  // state vectors
  static constexpr int NVS = NV + (DF ? 2 : 0);                                // with the low words
  static constexpr int NCX = Traits<METHOD>::NC + (DF ? 1 : 0);                // arrays per block
};

// 2^(r/16), r = 0..15: the rungs of the learned controller's step-size ladder within an octave
__constant__ const double k_ladder[16] = {
    1.0, 1.0442737824274138, 1.0905077326652577, 1.1387886347566916, 1.189207115002721, 1.241857812073484,
    1.2968395546510096, 1.3542555469368927, 1.4142135623730951, 1.4768261459394993, 1.5422108254079407,
    1.6104903319492543, 1.681792830507429, 1.7562521603732995, 1.8340080864093424, 1.9152065613971474};

RK_DEV double ladder_rung(double h0, int k) { return h0 * k_ladder[k & 15] * ldexp(1.0, k >> 4); }

// the rung h0 * 2^(k/16) (k an integer) nearest to h, or (floor) the largest not above h;
// the rung is picked in FP32, the floor checked in FP64
static __device__ __noinline__ double ladder_step(double h, double h0, bool floor_) {
  const float l = 16.f * log2f((float)(h / h0));
  int k = floor_ ? (int)floorf(l + 1e-3f) : (int)rintf(l);
  double v = ladder_rung(h0, k);
  if (floor_ && v > h) v = ladder_rung(h0, --k);
  return v;
}

// FP32 controller constants, formed once per instance run so that no attempt needs FP64
// arithmetic for them: cutoff^2 for the mask, log2(epsilon^2), safety
struct CtlF {
  float cut2, log2_eps2, safety;
};
RK_DEV CtlF make_ctlf(const rk_controller& c) {
  return CtlF{(float)(c.adapt_cutoff * c.adapt_cutoff), (float)(2.0 * log2(c.epsilon)), (float)c.safety_f};
}

// ---------------------------------------------------------------------------------
// per-instance working context
// ---------------------------------------------------------------------------------
// LOGN > 0: the grid size is the compile-time constant 2^LOGN (register-radix FFTs);
// LOGN == 0: runtime size (radix-4 FFTs).
template <class T, class CT, int LOGN = 0>
struct Ctx {
  Group g;
  int n, logn, m, mp, nl_kind;
  T nl_c;
  const T* kx;  // wavenumbers in the working precision (u*ux only)
  const cx<double>* lin;
  cx<T>* u;
  cx<T>* unew;
  cx<T>* N[8];
  CT* C;
  cx<T>* fa;
  cx<T>* fb;
  double* red;
  const cx<T>* tw;   // global table of RK_TW_N twiddles
  const cx<T>* tws;  // compile-time path: the block's twiddle rows in shared memory
  CtlF cf;           // FP32 controller constants (FP32 working precision)
  cx<T>* ulo;        // double-float state (df_state): low words of u and of the new state,
  cx<T>* unlo;       // null otherwise; the low word of E = e^z is coefficient C35_N
  bool want_tail;    // the attempt's pass over unew also forms the tail-energy fraction
  mutable float tail_frac;  // that fraction (-1: not formed by the attempt)
  RK_DEV CT c(int idx, int j) const { return C[idx * mp + j]; }
};

// ---------------------------------------------------------------------------------
// built-in nonlinearities: out[j] = N(k)[j] with k[j] = kf(j)
// ---------------------------------------------------------------------------------
// The u*ux packing fused with the first pass (radix R0, no twiddles) of the inverse
// n-point transform.  The packed spectrum is Z = A + iB with A = k/n and B = i kx k/n the
// Hermitian spectra of u and u_x: Z[j] = (A.x - B.y, A.y + B.x) and Z[n-j] = (A.x + B.y, B.x -
// A.y) for 0 < j < n/2, the imaginary parts of A and B dropped at j = 0 and n/2 (as numpy's
// irfft drops them).  Butterfly c of the pass needs Z[c + r NB0], r < R0: the rows r < R0/2
// are modes of column c, the others mirror images of the modes of column NB0 - c.  Two
// partner lanes hold the columns c and NB0 - c (paired_column), so each lane evaluates kf
// for the R0/2 modes of its own column and swaps the mirror images with its partner by
// shuffles; columns 0 and NB0/2 mirror themselves (column 0 also takes the Nyquist mode
// n/2).  Every mode is evaluated once, and the packed spectrum never goes through shared
// memory.
template <class T, int LOGN, class KF>
RK_DEV void pack_first_pass(const Group& g, KF kf, const T* __restrict__ kx, cx<T>* __restrict__ y, T inv_n) {
  using P0 = PassInfo<LOGN, 0>;
  constexpr int n = 1 << LOGN, M = n / 2, R0 = P0::R, NB0 = n / R0, H = R0 / 2;
  static_assert(P0::DONE == 0 && R0 >= 2 && NB0 % 32 == 0, "paired first pass: whole warps of butterflies");
  auto packed = [&](int j, cx<T>& own, cx<T>& mirror) {
    const cx<T> kv = kf(j);
    const T kxv = kx[j];
    cx<T> A = kv * inv_n;
    cx<T> B = mul_i(kv) * (kxv * inv_n);
    if (j == 0 || j == M) {
      A.y = T(0);
      B.y = T(0);
    }
    own = cx<T>{A.x - B.y, A.y + B.x};
    mirror = cx<T>{A.x + B.y, B.x - A.y};
  };
  for (int tt = g.tid; tt < NB0; tt += g.nthr) {
    const int c = paired_column(tt, NB0);
    const bool self = pair_unit(tt) == 0;  // columns 0 and NB0/2: their own mirror images
    const bool col0 = c == 0;
    cx<T> v[R0], mir[H], nyq{T(0), T(0)}, unused;
#pragma unroll
    for (int r = 0; r < H; ++r) packed(c + r * NB0, v[r], mir[r]);
    if (col0) packed(M, nyq, unused);
    cx<T> p[H];
#pragma unroll
    for (int r = 0; r < H; ++r) p[r] = shfl_pair(mir[r]);
    // rows s >= H: Z[c + s NB0] = mirror image of mode (NB0 - c) + (R0 - 1 - s) NB0, which is
    // the partner's mode at row R0-1-s; for column 0 mode (R0 - s) NB0 (row H: the Nyquist
    // mode itself), for column NB0/2 its own mode at row R0-1-s
#pragma unroll
    for (int s = H; s < R0; ++s) {
      const cx<T> d = (s == H) ? nyq : mir[(R0 - s) % H];
      v[s] = !self ? p[R0 - 1 - s] : (col0 ? d : mir[R0 - 1 - s]);
    }
    dft_reg<T, R0, true>(v);
#pragma unroll
    for (int r = 0; r < R0; ++r) y[fpad(c * R0 + r)] = v[r];
  }
}

// Last pass of the forward n/2-point transform fused with the rfft split.  Butterfly k (k <
// NB, the pass's sub-length) produces F[k + r NB], r < Rf; rfft mode k' = k + r NB needs F[k']
// and conj(F[n/2 - k']), and n/2 - k' = (NB - k) + (Rf - 1 - r) NB is an output of butterfly
// NB - k: with the butterflies paired over partner lanes (paired_column) the partner's outputs
// arrive by shuffles, and each lane writes the Rf modes of its butterfly (butterfly 0 also
// the Nyquist mode n/2) with no pass through shared memory.
// mode k': out = ((F + conj(Fm))/2 + W_n^k' (-i)(F - conj(Fm))/2) c.  W_n^k': FP32 from row 1
// of the inverse transform's last pass (W_n^k, k < NB) times the constant W_n^(r NB) =
// W_16^(8 r / Rf); FP64 from the global table `tw`.
template <class T, int LOGN>
RK_DEV void fwd_last_split(const Group& g, const cx<T>* __restrict__ x, const cx<T>* __restrict__ tab,
                           const cx<T>* __restrict__ tw, T c, cx<T>* __restrict__ out) {
  constexpr int PF = fft_passes(LOGN - 1, true) - 1;
  using F = PassInfo<LOGN - 1, PF, true>;
  constexpr int Rf = F::R, NB = F::Ls, M = 1 << (LOGN - 1);
  static_assert(F::last && F::DONE > 0 && NB * Rf == M, "last forward pass");
  static_assert(NB % 32 == 0, "paired butterflies: whole warps");
  static_assert(Rf <= 8, "W_n^(r NB) = W_16^(8 r / Rf) needs Rf <= 8");
  constexpr int MAP = fwd_map<LOGN, PF>();
  static_assert(MAP >= 0, "no pass of the twiddle rows serves the last forward pass");
  constexpr int PI = MAP / 10000, ALPHA = (MAP / 100) % 100, BETA = MAP % 100;
  const cx<T>* rows = tab + rows_offset<LOGN, PI>();
  constexpr int PL = fft_passes(LOGN) - 1;
  static_assert(NB <= PassInfo<LOGN, PL>::Ls, "W_n^k, k < NB, from row 1 of the last inverse pass");
  const cx<T>* row1 = tab + rows_offset<LOGN, PL>();
  constexpr int TWS = RK_TW_N >> LOGN;
  auto mode = [&](int k, cx<T> Fk, cx<T> Fm, cx<T> wk) {
    const cx<T> Fe = (Fk + Fm) * T(0.5);
    const cx<T> Fo = mul_mi(Fk - Fm) * T(0.5);
    out[k] = (Fe + wk * Fo) * c;
  };
  for (int tt = g.tid; tt < NB; tt += g.nthr) {
    const int k = paired_column(tt, NB);
    const bool self = pair_unit(tt) == 0;
    const bool col0 = k == 0;
    const cx<T>* xi = x + fpad(k);
    cx<T> v[Rf];
#pragma unroll
    for (int r = 0; r < Rf; ++r) v[r] = xi[r * NB + ((r * NB) >> 4)];
    {
      cx<T> t[Rf];
      load_twiddles<T, Rf, false, ALPHA, PassInfo<LOGN, PI>::Ls>(rows + BETA * k, t);
#pragma unroll
      for (int r = 1; r < Rf; ++r) v[r] = v[r] * t[r];
    }
    dft_reg<T, Rf, false>(v);
    cx<T> p[Rf];
#pragma unroll
    for (int r = 0; r < Rf; ++r) p[r] = shfl_pair(v[r]);
    cx<T> wk{T(1), T(0)};
    if constexpr (sizeof(T) == sizeof(float)) wk = row1[k];
    static_for<Rf>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      // F[n/2 - k']: the partner's row Rf-1-r; butterfly 0: its own row (Rf - r) % Rf;
      // butterfly NB/2: its own row Rf-1-r
      const cx<T> fm = !self ? p[Rf - 1 - r] : (col0 ? v[(Rf - r) % Rf] : v[Rf - 1 - r]);
      cx<T> w;
      if constexpr (sizeof(T) == sizeof(double)) w = tw[(k + r * NB) * TWS];
      else w = mul_w16<T, false, (8 * r) / Rf>(wk);
      mode(k + r * NB, v[r], conj(fm), w);
    });
    if (col0) mode(M, v[0], conj(v[0]), cx<T>{T(-1), T(0)});
  }
  g.sync();
}

// Transform part of the u*ux nonlinearity for a compile-time grid size, kept out of line so
// that its fully unrolled passes exist once per kernel rather than once per stage.
//
// On entry fb holds the output of the inverse transform's first pass (pack_first_pass).  The
// remaining inverse passes run, the last one writing the real product u*ux; the forward
// transform of n/2 points reads it as complex pairs (real t at 2*fpad(t/2) + t%2); its last
// pass is fused with the split into the n/2+1 rfft modes times c (fwd_last_split), which
// writes out[0 .. n/2].
// The FFT buffers and the twiddle rows (fill_twiddle_rows) arrive as byte offsets into the
// kernel's dynamic shared memory and are rebuilt from it here, so that the compiler knows
// they address shared memory inside this out-of-line function (pointer arguments would be
// generic).
template <class T, int LOGN>
__device__ __noinline__ void uux_core(Group g, uint32_t fa_off, uint32_t fb_off, uint32_t tws_off,
                                      const cx<T>* __restrict__ tw, T c, cx<T>* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  cx<T>* fa = reinterpret_cast<cx<T>*>(smem + fa_off);
  cx<T>* fb = reinterpret_cast<cx<T>*>(smem + fb_off);
  const cx<T>* tab = reinterpret_cast<const cx<T>*>(smem + tws_off);
  constexpr bool FUSED = uux_fused(LOGN);
  auto prod = [](cx<T>* y, int idx, int, cx<T> v) {
    reinterpret_cast<T*>(y)[2 * fpad(idx >> 1) + (idx & 1)] = v.x * v.y;
  };
  // fused: pass 0 ran in pack_first_pass (output in fb); unfused: the packed spectrum is in fa
  cx<T>* w = FUSED ? fft_rows<T, LOGN, 1, true>(g, fb, fa, tab, prod) : fft_rows<T, LOGN, 0, true>(g, fa, fb, tab, prod);
  cx<T>* other = (w == fa) ? fb : fa;
  const cx<T>* x = fft_half_rows_to_last<T, LOGN, 0>(g, w, other, tab);
  if constexpr (FUSED) {
    fwd_last_split<T, LOGN>(g, x, tab, tw, c, out);
  } else {
    // last forward pass into the other buffer, then the split: rfft mode k from F[k] and
    // conj(F[M - k]); the modes k and M - k read the same two values, so one thread forms
    // both (units q = 0 .. M/2 - 1: modes q and M - q; unit 0 also the self-paired mode M/2),
    // with W_n^(M - q) = -conj(W_n^q) in FP32.  M/2 units divide evenly over any group of up
    // to M/2 threads.
    constexpr int M = 1 << (LOGN - 1);
    constexpr int PF = fft_passes(LOGN - 1, true) - 1;
    using F = PassInfo<LOGN - 1, PF, true>;
    constexpr int MAP = fwd_map<LOGN, PF>();
    constexpr int PI = MAP / 10000, ALPHA = (MAP / 100) % 100, BETA = MAP % 100;
    cx<T>* Fb = (x == fa) ? fb : fa;
    stockham_pass_rows<T, LOGN - 1, F::LGR, F::DONE, false, ALPHA, BETA, PassInfo<LOGN, PI>::Ls>(
        g, x, tab + rows_offset<LOGN, PI>(), [&](int, int pidx, cx<T> v) { Fb[pidx] = v; });
    g.sync();
    constexpr int PL = fft_passes(LOGN) - 1;
    using L = PassInfo<LOGN, PL>;
    const cx<T>* row1 = tab + rows_offset<LOGN, PL>();  // W_n^s, s < L::Ls
    auto mode = [&](int k, cx<T> Fk, cx<T> Fm, cx<T> wk) {
      const cx<T> Fe = (Fk + Fm) * T(0.5);
      const cx<T> Fo = mul_mi(Fk - Fm) * T(0.5);
      out[k] = (Fe + wk * Fo) * c;
    };
    for (int q = g.tid; q < M / 2; q += g.nthr) {
      const cx<T> a = Fb[fpad(q)];
      const cx<T> b = Fb[fpad(q == 0 ? 0 : M - q)];
      cx<T> wq, wm;
      if constexpr (sizeof(T) == sizeof(double)) {
        wq = tw[q * (RK_TW_N >> LOGN)];
        wm = q == 0 ? cx<T>{T(-1), T(0)} : tw[(M - q) * (RK_TW_N >> LOGN)];
      } else {
        wq = mul_wr<T, L::R>(row1[q & (L::Ls - 1)], q / L::Ls);
        wm = cx<T>{-wq.x, wq.y};
      }
      mode(q, a, conj(b), wq);
      mode(q == 0 ? M : M - q, b, conj(a), wm);
      if (q == 0) {
        const cx<T> h = Fb[fpad(M / 2)];
        cx<T> wh{T(0), T(-1)};  // W_n^(n/4) = -i
        if constexpr (sizeof(T) == sizeof(double)) wh = tw[(M / 2) * (RK_TW_N >> LOGN)];
        mode(M / 2, h, conj(h), wh);
      }
    }
    g.sync();
  }
}

template <class T, class CT, int LOGN, class KF>
RK_DEV void nl_eval(const Ctx<T, CT, LOGN>& x, KF kf, cx<T>* __restrict__ out) {
  const Group& g = x.g;
  // FFT-buffer index: padded for the compile-time transforms
  auto P = [](int c) { return LOGN > 0 ? fpad(c) : c; };
  // the compile-time-size kernels serve u*ux only (rk_m_etd35_ct.cu dispatches nothing else
  // to them), so they carry no other nonlinearity's code
  if (LOGN > 0 || x.nl_kind == RK_NL_UUX) {
    // u = irfft(k), ux = irfft(i kx k) packed as one complex inverse FFT of length n:
    // Z = A + iB with A, B the Hermitian spectra; numpy's irfft drops the imaginary
    // parts of the DC and Nyquist bins, so they are dropped here too.
    const int n = LOGN > 0 ? (1 << LOGN) : x.n, M = n >> 1;
    const T inv_n = T(1) / T(n);
    if constexpr (LOGN > 0) {
      extern __shared__ __align__(16) unsigned char smem[];
      auto off = [](const void* q) {
        return (uint32_t)(reinterpret_cast<const unsigned char*>(q) - smem);
      };
if constexpr (uux_fused(LOGN)) {
        pack_first_pass<T, LOGN>(g, kf, x.kx, x.fb, inv_n);
      } else {
        cx<T>* Z = x.fa;
        auto pack = [&](int j, cx<T> kv, T kxv) {
          cx<T> A = kv * inv_n;
          cx<T> B = mul_i(kv) * (kxv * inv_n);
          if (j == 0 || j == M) {
            A.y = T(0);
            B.y = T(0);
          }
          Z[fpad(j)] = cx<T>{A.x - B.y, A.y + B.x};
          if (j > 0 && j < M) Z[fpad(n - j)] = cx<T>{A.x + B.y, B.x - A.y};
        };
        // modes 0 .. M-1 over the group, the Nyquist mode M with mode 0: for a group of up to
        // M threads M is a multiple of its size, so no thread runs an extra iteration for it
        for (int j = g.tid; j < M; j += g.nthr) {
          const cx<T> kv = kf(j);
          const T kxv = x.kx[j];
          if (j == 0) pack(M, kf(M), x.kx[M]);
          pack(j, kv, kxv);
        }
      }
      g.sync();
      uux_core<T, LOGN>(g, off(x.fa), off(x.fb), off(x.tws), sizeof(T) == sizeof(double) ? x.tw : nullptr,
                        x.nl_c, out);
      return;
    }
    cx<T>* Z = x.fa;
    auto pack = [&](int j, cx<T> kv, T kxv) {
      cx<T> A = kv * inv_n;
      cx<T> B = mul_i(kv) * (kxv * inv_n);
      if (j == 0 || j == M) {
        A.y = T(0);
        B.y = T(0);
      }
      Z[P(j)] = cx<T>{A.x - B.y, A.y + B.x};
      if (j > 0 && j < M) Z[P(n - j)] = cx<T>{A.x + B.y, B.x - A.y};
    };
    // modes 0 .. M-1 over the group, the Nyquist mode M with mode 0: for a group of up to M
    // threads M is a multiple of its size, so no thread runs an extra iteration for one mode
    for (int j = g.tid; j < M; j += g.nthr) {
      const cx<T> kv = kf(j);
      const T kxv = x.kx[j];
      if (j == 0) pack(M, kf(M), x.kx[M]);
      pack(j, kv, kxv);
    }
    g.sync();
    cx<T>* F;
    {
      cx<T>* z = fft_group<T, true>(g, x.fa, x.fb, x.logn, x.tw);
      cx<T>* other = (z == x.fa) ? x.fb : x.fa;
      T* w = reinterpret_cast<T*>(other);
      for (int t = g.tid; t < n; t += g.nthr) {
        cx<T> v = z[t];
        w[t] = v.x * v.y;
      }
      g.sync();
      F = fft_group<T, false>(g, other, z, x.logn - 1, x.tw);
    }
    // rfft of the real product from the length-n/2 transform (split formula), with
    // exp(-2 pi i k/n) from the global table (runtime-size path; the compile-time path
    // returned above)
    const cx<T>* twu = x.tw;
    const int tws = RK_TW_N >> x.logn;
    for (int k = g.tid; k <= M; k += g.nthr) {
      cx<T> Fk = F[P(k == M ? 0 : k)];
      cx<T> Fm = conj(F[P(k == 0 ? 0 : M - k)]);
      cx<T> Fe = (Fk + Fm) * T(0.5);
      cx<T> Fo = mul_mi(Fk - Fm) * T(0.5);
      out[k] = (Fe + (k == M ? cx<T>{T(-1), T(0)} : twu[k * tws]) * Fo) * x.nl_c;
    }
    g.sync();
  } else if constexpr (LOGN > 0) {
    // not reached
  } else if (x.nl_kind == RK_NL_NLS) {
    // v = ifft(k); N = fft(i c |v|^2 v)
    const int n = LOGN > 0 ? (1 << LOGN) : x.n;
    const T inv_n = T(1) / T(n);
    constexpr int PK = 1;
    for (int j0 = g.tid; j0 < n; j0 += PK * g.nthr) {
      cx<T> kv[PK];
#pragma unroll
      for (int q = 0; q < PK; ++q) {
        const int j = j0 + q * g.nthr;
        kv[q] = j < n ? kf(j) : cx<T>{T(0), T(0)};
      }
#pragma unroll
      for (int q = 0; q < PK; ++q) {
        const int j = j0 + q * g.nthr;
        if (j < n) x.fa[P(j)] = kv[q] * inv_n;
      }
    }
    g.sync();
    const T c = x.nl_c;
    {
      cx<T>* z = fft_group<T, true>(g, x.fa, x.fb, x.logn, x.tw);
      cx<T>* other = (z == x.fa) ? x.fb : x.fa;
      for (int t = g.tid; t < n; t += g.nthr) {
        cx<T> v = z[t];
        T a2 = (v.x * v.x + v.y * v.y) * c;
        other[t] = cx<T>{-a2 * v.y, a2 * v.x};
      }
      g.sync();
      cx<T>* F = fft_group<T, false>(g, other, z, x.logn, x.tw);
      for (int k = g.tid; k < n; k += g.nthr) out[k] = F[k];
      g.sync();
    }
  } else {
    for (int k = g.tid; k < x.m; k += g.nthr) out[k] = cx<T>{T(0), T(0)};
    g.sync();
  }
}

// ---------------------------------------------------------------------------------
// coefficients at step h (FP64 math), stored in the working precision
// ---------------------------------------------------------------------------------
template <class T> RK_DEV void store_c(T& d, double v) { d = T(v); }
template <class T> RK_DEV void store_c(cx<T>& d, cx<double> v) { d = cx<T>{T(v.x), T(v.y)}; }
// the low word of v after store_c (the double-float state's E_lo)
RK_DEV void store_lo(float& d, double v) { d = (float)(v - (double)(float)v); }
RK_DEV void store_lo(cx<float>& d, cx<double> v) {
  d = cx<float>{(float)(v.x - (double)(float)v.x), (float)(v.y - (double)(float)v.y)};
}
template <class T, class V> RK_DEV void store_lo(T&, V) {}

template <class S> RK_DEV S load_z(const cx<double>* lin, int j, double h);
template <> RK_DEV double load_z<double>(const cx<double>* lin, int j, double h) { return h * lin[j].x; }
template <> RK_DEV cx<double> load_z<cx<double>>(const cx<double>* lin, int j, double h) {
  cx<double> L = lin[j];
  return cx<double>{h * L.x, h * L.y};
}

// FP32 ETD35 / ETD5 coefficients of one real mode into the block.  With the double-float
// state (elo set) only e^(z/4) of the four exponentials is stored: the stage code forms
// e^(z/2) = e14 e14, e^(3z/4) = e^(z/2) e14 and e^z = e^(z/2) e^(z/2) by rounded FP32
// products (e12 / e34 / e1 in attempt_etd35_family), and the low word of e^z is taken
// against that product (e_hi + e_lo = e^z as the rebuild formed it, e_hi = of[C35_E]), so
// the new state keeps its accuracy.  Three fewer arrays per instance pass through the stage
// loops and the L2.
template <int METHOD>
RK_DEV void put_coeffs_f32(float* __restrict__ C, int mp, int j, const float* of, float* __restrict__ elo,
                           float e_lo) {
  constexpr int NC = Traits<METHOD>::NC;
  if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5) {
    if (elo) {
      const float e12 = __fmul_rn(of[C35_E14], of[C35_E14]);
      elo[j] = (of[C35_E] - __fmul_rn(e12, e12)) + e_lo;
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c != C35_E12 && c != C35_E34 && c != C35_E) C[c * mp + j] = of[c];
      return;
    }
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) C[c * mp + j] = of[c];
}

// Coefficients of one instance at step h into C (array c at C + c*mp).  S is double for
// a real operator (CT real) and cx<double> for a complex one.  FAST selects the
// reduced-cost psi evaluation for real modes (coefficients stored in FP32).  Kept out of
// line: it runs on a small fraction of attempts and would otherwise inflate the
// register budget of the stage loop.
template <class CT, class S, int METHOD, bool FAST>
__device__ __noinline__ void compute_coeffs_impl(Group g, int m, int mp, const cx<double>* __restrict__ lin,
                                                 CT* __restrict__ C, double h, EtdCfg ec,
                                                 CT* __restrict__ elo = nullptr) {
  constexpr int NC = Traits<METHOD>::NC;
  if (!is_etd(METHOD)) {
    for (int j = g.tid; j < m; j += g.nthr) {
      S z = load_z<S>(lin, j, h);
      S o[NC];
      if_coeffs<S>(METHOD, z, h, o);
#pragma unroll
      for (int c = 0; c < NC; ++c) store_c(C[c * mp + j], o[c]);
    }
    g.sync();
    return;
  }
  constexpr int NP = (METHOD == RK_ETD35 || METHOD == RK_ETD5) ? RK_PSI35_N : RK_PSI34_N;
  // pass 1: thread per mode, direct formula for |z| >= modecutoff; with FAST the small
  // modes are evaluated here too, by the Taylor series of psi_k (see taylor_psi)
  for (int j = g.tid; j < m; j += g.nthr) {
    S z = load_z<S>(lin, j, h);
    const bool small = sabs(z) < ec.cutoff;
    if (small && !FAST) continue;
    S P[NP];
    S o[NC];
    if constexpr (FAST) {
      if (small) {
        if constexpr (sizeof(S) == sizeof(double) && sizeof(CT) == sizeof(float)) {
          // each combination's own Taylor series in FP32 (series_coeffs_f32): the FP64
          // series would hold the whole warp on the 1/64-rate FP64 pipe for one small mode
          float of[NC], el = 0.f;
          series_coeffs_f32<METHOD>(sre(z), h, of, nullptr, &el);
          put_coeffs_f32<METHOD>(C, mp, j, of, elo, el);
        } else {
          S E[4];
          taylor_psi<S>(METHOD, z, h, E, P);
          etd_from_psi_e<S>(METHOD, E, P, o);
#pragma unroll
          for (int c = 0; c < NC; ++c) store_c(C[c * mp + j], o[c]);
          if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5)
            if (elo) store_lo(elo[j], o[C35_E]);
        }
        continue;
      }
    }
    if constexpr (FAST && sizeof(S) == sizeof(double) && sizeof(CT) == sizeof(float)) {
      const double zr = sre(z);
      if (zr < -(double)STIFF_Z) {
        // stiff: FP32 arithmetic in a form without cancellation (a few FP32 ulps)
        float of[NC];
        stiff_coeffs_f32<METHOD>(zr, h, of);
        put_coeffs_f32<METHOD>(C, mp, j, of, elo, 0.f);  // e^z < e^-32: no low word of its own
        continue;
      }
      if (zr <= 80.0) {
        // FP32 series / stiff forms per combination (series_coeffs_f32)
        float of[NC], el = 0.f;
        series_coeffs_f32<METHOD>(zr, h, of, nullptr, &el);
        put_coeffs_f32<METHOD>(C, mp, j, of, elo, el);
        continue;
      }
      double E[4];
      fast_real_psi(METHOD, zr, h, E, reinterpret_cast<double*>(P));
      etd_from_psi_e<double>(METHOD, E, reinterpret_cast<double*>(P), reinterpret_cast<double*>(o));
      const double* od = reinterpret_cast<const double*>(o);
      float of[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) of[c] = (float)od[c];
      float el = 0.f;
      if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5) el = (float)(od[C35_E] - (double)of[C35_E]);
      put_coeffs_f32<METHOD>(C, mp, j, of, elo, el);
      continue;
    } else if constexpr (FAST && sizeof(S) == sizeof(double)) {
      double E[4];
      fast_real_psi(METHOD, sre(z), h, E, reinterpret_cast<double*>(P));
      etd_from_psi_e<double>(METHOD, E, reinterpret_cast<double*>(P), reinterpret_cast<double*>(o));
    } else {
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        int order;
        double num, den;
        psi_slot(METHOD, k, order, num, den);
        P[k] = direct_hpsi(z, h, order, num, den);
      }
      etd_from_psi<S>(METHOD, z, P, o);
    }
    // (the FP32 real-operator branch above stores its modes itself)
    if constexpr (!(FAST && sizeof(S) == sizeof(double) && sizeof(CT) == sizeof(float))) {
#pragma unroll
      for (int c = 0; c < NC; ++c) store_c(C[c * mp + j], o[c]);
      if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5)
        if (elo) store_lo(elo[j], o[C35_E]);
    }
  }
  if constexpr (FAST) {
    g.sync();
    return;
  }
  // pass 2: warp per small mode, lanes over the contour nodes (rkstiff/etd35.py:257-288)
  const int lane = g.tid & 31, warp = g.tid >> 5, nwarp = g.nthr >> 5;
  for (int j = warp; j < m; j += nwarp) {
    S z = load_z<S>(lin, j, h);
    if (!(sabs(z) < ec.cutoff)) continue;
    cx<double> zc = to_cx(z);
    cx<double> acc[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) acc[k] = cx<double>{0.0, 0.0};
    for (int q = lane; q < ec.np; q += 32) {
      const cx<double> Z = zc + contour_node(ec, q);
      if constexpr (FAST) {
        contour_terms_fast(METHOD, Z, acc);
      } else {
#pragma unroll
        for (int k = 0; k < NP; ++k) {
          int order;
          double num, den;
          psi_slot(METHOD, k, order, num, den);
          acc[k] = acc[k] + contour_term_at(Z, order, num, den);
        }
      }
    }
    S P[NP];
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      double re = warp_sum(acc[k].x), im = warp_sum(acc[k].y);
      P[k] = from_cx<S>(rdiv(h * cx<double>{re, im}, (double)ec.np));
    }
    if (lane == 0) {
      S o[NC];
      etd_from_psi<S>(METHOD, z, P, o);
#pragma unroll
      for (int c = 0; c < NC; ++c) store_c(C[c * mp + j], o[c]);
    }
  }
  g.sync();
}

template <class T, class CT, class S, int METHOD, int LOGN>
RK_DEV void compute_coeffs(const Ctx<T, CT, LOGN>& x, double h, const EtdCfg& ec) {
  CT* elo = nullptr;
  if constexpr (SlabShape<T, CT, METHOD>::DF) elo = x.C + Traits<METHOD>::NC * x.mp;
  compute_coeffs_impl<CT, S, METHOD, sizeof(T) == sizeof(float)>(x.g, x.m, x.mp, x.lin, x.C, h, ec, elo);
}

// ---------------------------------------------------------------------------------
// new state + controller factor s (FP64 masked norms)
// ---------------------------------------------------------------------------------
template <class T> RK_DEV double cabs_d(cx<T> v) { return hypot((double)v.x, (double)v.y); }

// New state into unew; returns the group-wide max of |unew| (FP64 working precision)
// or of |unew|^2 (FP32 working precision), NaN if any entry is NaN.
template <class T, class CT, int LOGN, class KF>
RK_DEV double write_unew(const Ctx<T, CT, LOGN>& x, KF kf) {
  bool nan = false;
  if constexpr (sizeof(T) == sizeof(double)) {
    double mx = 0.0;
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
      cx<T> v = kf(j);
      x.unew[j] = v;
      double a = cabs_d(v);
      if (a != a) nan = true;
      else mx = fmax(mx, a);
    }
    return group_max_nan(x.g, x.red, nan ? nan_d() : mx);
  } else {
    float mx = 0.f;
    constexpr int PK = 1;
    for (int j0 = x.g.tid; j0 < x.m; j0 += PK * x.g.nthr) {
      cx<T> v[PK];
#pragma unroll
      for (int q = 0; q < PK; ++q) {
        const int j = j0 + q * x.g.nthr;
        v[q] = j < x.m ? kf(j) : cx<T>{T(0), T(0)};
      }
#pragma unroll
      for (int q = 0; q < PK; ++q) {
        const int j = j0 + q * x.g.nthr;
        if (j >= x.m) break;
        x.unew[j] = v[q];
        float a2 = v[q].x * v[q].x + v[q].y * v[q].y;
        if (a2 != a2) nan = true;
        else mx = fmaxf(mx, a2);
      }
    }
    return (double)group_max_nan_f(x.g, x.red, mx, nan);
  }
}

// s from the masked sums su = sum |u|^2, se = sum |err|^2 in FP32 working precision:
// (eps |u| / |err|)^(1/q) = ratio^(1/(2q)) with ratio = eps^2 su / se formed in FP64; the
// fractional power runs in FP32 (FP64 pow is a long dependent chain on this GPU).  Edge
// values keep the reference's outcome: 0/0 -> NaN and x/0 -> inf (both rejected), a finite
// ratio beyond FP32 range stays finite (accepted).  The one exception: an error vector that
// is exactly zero in FP32 while |u| > 0 lies below FP32 resolution (an FP64 error of the same
// attempt is small but not zero), so the attempt takes the largest growth, MAX_S = 4,
// instead of the rejection that x/0 = inf would give.
RK_DEV double s_from_sums_f32(double su, double se, const rk_controller& ctl, int q) {
  if (se == 0.0 && su > 0.0 && !isinf(su)) return 4.0;
  const double ratio = (ctl.epsilon * ctl.epsilon * su) / se;
  if (ratio != ratio || isinf(ratio)) return ctl.safety_f * ratio;
  const float rf = (float)fmin(ratio, 1e30);
  return ctl.safety_f * (double)exp2f(log2f(rf) * (0.5f / (float)q));
}

// The same s from double-float sums with FP32 instructions only: log2 of the ratio as
// log2(eps^2) + log2(su) - log2(se) (the pairs' high words carry the sums to FP32
// precision, which bounds s's precision anyway), clamped where the ratio passes 1e30, and
// the edge values of s_from_sums_f32: 0/0 and x/0 = inf reject (x/0 with |u| > 0 finite
// takes MAX_S = 4, see above), a zero |u| gives s = 0.  log2_eps2 = log2(epsilon^2).
RK_DEV double s_from_sums_f32_fast(df su, df se, float log2_eps2, float safety, int q) {
  const float u = su.hi + su.lo, e = se.hi + se.lo;
  const double inf = __longlong_as_double(0x7ff0000000000000ULL);
  if (u != u || e != e) return nan_d();
  if (e == 0.f) {
    if (u > 0.f && !isinf(u)) return 4.0;  // below FP32 resolution, see above
    return u == 0.f ? nan_d() : inf;      // 0/0, inf/0
  }
  if (isinf(u)) return isinf(e) ? nan_d() : inf;
  if (u == 0.f || isinf(e)) return 0.0;
  const float l = fminf(log2_eps2 + (log2f(u) - log2f(e)), 99.65784f);  // log2(1e30)
  return (double)(safety * exp2f(l * (0.5f / (float)q)));
}

// s = safety (eps |unew[mask]| / |err[mask]|)^(1/q), mask = |unew| / max|unew| > cutoff
// (rkstiff/solveras.py:451-455).  The sums of squares are accumulated in FP64.  In FP32
// working precision the mask is evaluated on squared magnitudes, |u|^2 > cutoff^2 max|u|^2,
// which needs no square root or division per mode.
template <class T, class CT, int LOGN, class EF>
RK_DEV double controller_s(const Ctx<T, CT, LOGN>& x, double maxu, EF ef, const rk_controller& ctl, int q) {
  double su = 0.0, se = 0.0;
  if constexpr (sizeof(T) == sizeof(double)) {
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
      cx<T> v = x.unew[j];
      double a = cabs_d(v);
      if (a / maxu > ctl.adapt_cutoff) {
        su += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        cx<T> e = ef(j);
        se += (double)e.x * (double)e.x + (double)e.y * (double)e.y;
      }
    }
  } else {
    // maxu holds max |unew|^2 here; NaN keeps every comparison false, as in the reference.
    // The sums are carried in double-float (FP32 pairs with error-free addition, a
    // 48-bit significand) and formed as FP64 once per group.
    const float thr = (float)(ctl.adapt_cutoff * ctl.adapt_cutoff * maxu);
    df au{0.f, 0.f}, ae{0.f, 0.f};
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
      cx<T> v = x.unew[j];
      float a2 = v.x * v.x + v.y * v.y;
      if (a2 > thr) {
        au = df_add(au, a2);
        cx<T> e = ef(j);
        ae = df_add(ae, e.x * e.x + e.y * e.y);
      }
    }
    group_sum2_df(x.g, x.red, au, ae, su, se);
  }
  if constexpr (sizeof(T) == sizeof(double)) {
    group_sum2(x.g, x.red, su, se);
    double tol = ctl.epsilon * sqrt(su);
    return ctl.safety_f * pow(tol / sqrt(se), 1.0 / q);
  } else {
    return s_from_sums_f32(su, se, ctl, q);
  }
}

// the new state of one mode as a double-float pair (high and low FP32 words)
template <class T>
struct HiLo {
  cx<T> hi, lo;
};

// ETD35 in FP32 working precision: unew and |err|^2 in one pass over the modes (the error
// combination reads the same stage vectors as unew), |unew|^2 and |err|^2 of each mode
// parked in the FFT buffer (free between attempts) until the group maximum of |unew|^2 is
// known; then the masked sums from those two floats per mode.  Same values as write_unew
// followed by controller_s, without the second pass over the stage vectors.
template <class T, class CT, int LOGN, class KF, class EF>
RK_DEV double unew_and_s_f32(const Ctx<T, CT, LOGN>& x, KF kf, EF ef, const CtlF& cf, int q) {
  float* park = reinterpret_cast<float*>(x.fa);  // [2 m] floats: the buffer holds >= n complex
  x.g.sync();  // the last transform has released the buffer
  float mx = 0.f;
  bool nan = false;
  auto one = [&](int j) {
    const auto r = kf(j);
    const cx<T> e = ef(j);
    // stores after both combinations have read the stage vectors (a store before them could
    // alias those arrays as far as the compiler knows, and make it load them again)
    cx<T> v;
    if constexpr (std::is_same<typename std::decay<decltype(r)>::type, HiLo<T>>::value) {
      v = r.hi;
      x.unlo[j] = r.lo;
    } else {
      v = r;
    }
    x.unew[j] = v;
    const float a2 = v.x * v.x + v.y * v.y;
    if (a2 != a2) nan = true;
    else mx = fmaxf(mx, a2);
    park[2 * j] = a2;
    park[2 * j + 1] = e.x * e.x + e.y * e.y;
  };
  // an odd mode count (a real grid's n/2 + 1) puts its last mode with mode 0, so that the
  // group's threads run the same number of iterations over these global loads
  const int odd = x.m & 1;
  for (int j = x.g.tid; j < x.m - odd; j += x.g.nthr) {
    if (odd && j == 0) one(x.m - 1);
    one(j);
  }
  const float maxu = group_max_nan_f(x.g, x.red, mx, nan);
  // NaN keeps every comparison false, as in the reference
  const float thr = cf.cut2 * maxu;
  df au{0.f, 0.f}, ae{0.f, 0.f};
  if (x.want_tail) {
    // with the tail-energy fraction of unew (tail_fraction's sums) in the same pass
    const bool full = x.m == x.n;
    const int j0 = full ? (3 * x.n) / 8 : (3 * x.m) / 4;
    const int j1 = full ? (5 * x.n) / 8 : x.m - 1;
    df v[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
      const float a2 = park[2 * j];
      if (a2 > thr) {
        v[0] = df_add(v[0], a2);
        v[1] = df_add(v[1], park[2 * j + 1]);
      }
      v[3] = df_add(v[3], a2);
      if (j >= j0 && j <= j1) v[2] = df_add(v[2], a2);
    }
    group_sum4_dff(x.g, x.red, v);
    const double st = (double)v[2].hi + (double)v[2].lo, sa = (double)v[3].hi + (double)v[3].lo;
    x.tail_frac = sa > 0.0 ? (float)(st / sa) : 0.f;
    return s_from_sums_f32_fast(v[0], v[1], cf.log2_eps2, cf.safety, q);
  }
  for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
    const float a2 = park[2 * j];
    if (a2 > thr) {
      au = df_add(au, a2);
      ae = df_add(ae, park[2 * j + 1]);
    }
  }
  df su, se;
  group_sum2_dff(x.g, x.red, au, ae, su, se);
  return s_from_sums_f32_fast(su, se, cf.log2_eps2, cf.safety, q);
}

// ---------------------------------------------------------------------------------
// stage programs.  Each computes N2.. and unew (and N(unew) where the method needs it)
// and returns s (adaptive) or 0 (constant).  N1 must be valid on entry.
// ---------------------------------------------------------------------------------
template <class T, class CT, int LOGN>
RK_DEV double attempt_etd35_family(const Ctx<T, CT, LOGN>& x, bool adaptive, const rk_controller& ctl, int& nl_count) {
  const cx<T>* u = x.u;
  cx<T>* const* N = x.N;
  // e^(z/2), e^(3z/4), e^z: FP32 with a real operator (the double-float state) keeps only
  // e^(z/4) in the block and forms the others by the rounded products the rebuild took the
  // low word of e^z against (put_coeffs_f32); otherwise loaded
  constexpr bool EPOW = SlabShape<T, CT, RK_ETD35>::DF && sizeof(CT) == sizeof(float);
  auto e12 = [&](int j) -> CT {
    if constexpr (EPOW) return __fmul_rn(x.c(C35_E14, j), x.c(C35_E14, j));
    else return x.c(C35_E12, j);
  };
  auto e34 = [&](int j) -> CT {
    if constexpr (EPOW) {
      const float a = x.c(C35_E14, j);
      return __fmul_rn(__fmul_rn(a, a), a);
    } else {
      return x.c(C35_E34, j);
    }
  };
  auto e1 = [&](int j) -> CT {
    if constexpr (EPOW) {
      const float a = x.c(C35_E14, j), b = __fmul_rn(a, a);
      return __fmul_rn(b, b);
    } else {
      return x.c(C35_E, j);
    }
  };
  // rkstiff/etd35.py:320-345 (ETD5: etd5.py:236-260)
  nl_eval(x, [&](int j) { return cmul(x.c(C35_E14, j), u[j]) + cmul(x.c(C35_A21, j), N[0][j]); }, N[1]);
  nl_eval(x, [&](int j) {
    return (cmul(x.c(C35_E14, j), u[j]) + cmul(x.c(C35_A31, j), N[0][j])) + cmul(x.c(C35_A32, j), N[1][j]);
  }, N[2]);
  nl_eval(x, [&](int j) {
    return (cmul(e12(j), u[j]) + cmul(x.c(C35_A41, j), N[0][j])) + cmul(x.c(C35_A43, j), N[2][j]);
  }, N[3]);
  nl_eval(x, [&](int j) {
    return ((cmul(e34(j), u[j]) + cmul(x.c(C35_A51, j), N[0][j])) + cmul(x.c(C35_A52, j), N[1][j] - N[2][j])) +
           cmul(x.c(C35_A54, j), N[3][j]);
  }, N[4]);
  nl_eval(x, [&](int j) {
    cx<T> t = N[1][j] - (T(3) * N[3][j]) * T(0.5);
    return (((cmul(e1(j), u[j]) + cmul(x.c(C35_A61, j), N[0][j])) + cmul(x.c(C35_A62, j), t)) +
            cmul(x.c(C35_A63, j), N[2][j])) + cmul(x.c(C35_A65, j), N[4][j]);
  }, N[5]);
  nl_count += 5;
  auto k7 = [&](int j) {
    return ((((cmul(e1(j), u[j]) + cmul(x.c(C35_A71, j), N[0][j])) + cmul(x.c(C35_A73, j), N[2][j])) +
             cmul(x.c(C35_A74, j), N[3][j])) + cmul(x.c(C35_A75, j), N[4][j])) + cmul(x.c(C35_A76, j), N[5][j]);
  };
  // Double-float state (x.ulo set: FP32): unew = E u + S with u = u_hi +
  // u_lo and E = E_hi + E_lo, S the FP32 sum of the a7k N_k terms; E_hi u_hi exactly as a
  // product and its rounding error (FMA), the cross terms and the rounding of the sum with S
  // (TwoSum) collected in the low word.  Returns both words (the caller stores them).
  // Rounding u to FP32 on every accepted step, and E to FP32, is what accumulates over a
  // long run; the stage values' FP32 error enters only through h-scaled terms.
  auto k7df = [&](int j) {
    if constexpr (sizeof(T) == sizeof(float) && sizeof(CT) == sizeof(T)) {
      const cx<T> S = (((cmul(x.c(C35_A71, j), N[0][j]) + cmul(x.c(C35_A73, j), N[2][j])) +
                        cmul(x.c(C35_A74, j), N[3][j])) + cmul(x.c(C35_A75, j), N[4][j])) +
                      cmul(x.c(C35_A76, j), N[5][j]);
      const float eh = e1(j), el = x.c(C35_N, j);
      const cx<T> uh = u[j], ul = x.ulo[j];
      auto part = [&](float h, float l, float sv, float& lo_out) {
        const float p = eh * h;
        const float ep = fmaf(eh, h, -p);  // exact: E_hi u_hi = p + ep
        const float corr = fmaf(eh, l, fmaf(el, h, ep));
        const float q = p + sv;  // TwoSum(p, sv)
        const float bb = q - p;
        const float e2 = (p - (q - bb)) + (sv - bb);
        const float lo = e2 + corr;
        const float hi = q + lo;
        lo_out = lo - (hi - q);
        return hi;
      };
      HiLo<T> r;
      r.hi = cx<T>{part(uh.x, ul.x, S.x, r.lo.x), part(uh.y, ul.y, S.y, r.lo.y)};
      return r;
    } else if constexpr (sizeof(T) == sizeof(float)) {
      // complex E (an operator with imaginary parts, e.g. the NLS dispersion): each component
      // of E_hi u_hi is a sum of two products, both taken exactly
      const cx<T> S = (((cmul(x.c(C35_A71, j), N[0][j]) + cmul(x.c(C35_A73, j), N[2][j])) +
                        cmul(x.c(C35_A74, j), N[3][j])) + cmul(x.c(C35_A75, j), N[4][j])) +
                      cmul(x.c(C35_A76, j), N[5][j]);
      const cx<T> eh = x.c(C35_E, j), el = x.c(C35_N, j);
      const cx<T> uh = u[j], ul = x.ulo[j];
      // a1 b1 + a2 b2 + la + sv: the two products and the sums' rounding in the low word
      auto comp = [&](float a1, float b1, float a2, float b2, float la, float sv, float& lo_out) {
        const float p1 = a1 * b1, e1 = fmaf(a1, b1, -p1);
        const float p2 = a2 * b2, e2 = fmaf(a2, b2, -p2);
        const float q = p1 + p2, qb = q - p1, e3 = (p1 - (q - qb)) + (p2 - qb);
        const float r = q + sv, rb = r - q, e4 = (q - (r - rb)) + (sv - rb);
        const float lo = ((e1 + e2) + (e3 + e4)) + la;
        const float hi = r + lo;
        lo_out = lo - (hi - r);
        return hi;
      };
      const float la_re = fmaf(eh.x, ul.x, -eh.y * ul.y) + fmaf(el.x, uh.x, -el.y * uh.y);
      const float la_im = fmaf(eh.x, ul.y, eh.y * ul.x) + fmaf(el.x, uh.y, el.y * uh.x);
      HiLo<T> r;
      r.hi = cx<T>{comp(eh.x, uh.x, -eh.y, uh.y, la_re, S.x, r.lo.x), comp(eh.x, uh.y, eh.y, uh.x, la_im, S.y, r.lo.y)};
      return r;
    } else {
      return HiLo<T>{k7(j), cx<T>{T(0), T(0)}};
    }
  };
  if (!adaptive) {
    // ETD5: unew, then N1 <- N(unew) (FSAL, etd5.py:260)
    if (x.ulo) {
      for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
        const HiLo<T> r = k7df(j);
        x.unew[j] = r.hi;
        x.unlo[j] = r.lo;
      }
    } else {
      for (int j = x.g.tid; j < x.m; j += x.g.nthr) x.unew[j] = k7(j);
    }
    x.g.sync();
    const cx<T>* un = x.unew;
    nl_eval(x, [&](int j) { return un[j]; }, N[0]);
    nl_count += 1;
    return 0.0;
  }
  auto err = [&](int j) {
    cx<T> s = (((-N[0][j] + T(4) * N[2][j]) - T(6) * N[3][j]) + T(4) * N[4][j]) - N[5][j];
    return cmul(x.c(C35_A75, j), s);
  };
  if constexpr (sizeof(T) == sizeof(float)) {
    if (x.ulo) return unew_and_s_f32(x, k7df, err, x.cf, 4);
    return unew_and_s_f32(x, k7, err, x.cf, 4);
  } else {
    double mx = write_unew(x, k7);
    return controller_s(x, mx, err, ctl, 4);
  }
}

template <class T, class CT, int LOGN>
RK_DEV double attempt_etd34_family(const Ctx<T, CT, LOGN>& x, bool adaptive, const rk_controller& ctl, int& nl_count) {
  const cx<T>* u = x.u;
  cx<T>* const* N = x.N;
  // rkstiff/etd34.py:182-190 (ETD4: etd4.py:167-174)
  nl_eval(x, [&](int j) { return cmul(x.c(C34_E2, j), u[j]) + cmul(x.c(C34_A21, j), N[0][j]); }, N[1]);
  nl_eval(x, [&](int j) {
    return (cmul(x.c(C34_E2, j), u[j]) + cmul(x.c(C34_A31, j), N[0][j])) + cmul(x.c(C34_A32, j), N[1][j]);
  }, N[2]);
  nl_eval(x, [&](int j) {
    return (cmul(x.c(C34_E, j), u[j]) + cmul(x.c(C34_A41, j), N[0][j])) + cmul(x.c(C34_A43, j), N[2][j]);
  }, N[3]);
  nl_count += 3;
  auto k5 = [&](int j) {
    return ((cmul(x.c(C34_E, j), u[j]) + cmul(x.c(C34_A51, j), N[0][j])) + cmul(x.c(C34_A52, j), N[1][j] + N[2][j])) +
           cmul(x.c(C34_A54, j), N[3][j]);
  };
  const cx<T>* un = x.unew;
  if (!adaptive) {
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) x.unew[j] = k5(j);
    x.g.sync();
    nl_eval(x, [&](int j) { return un[j]; }, N[0]);
    nl_count += 1;
    return 0.0;
  }
  double mx = write_unew(x, k5);
  nl_eval(x, [&](int j) { return un[j]; }, N[4]);
  nl_count += 1;
  return controller_s(x, mx, [&](int j) { return cmul(x.c(C34_A54, j), N[3][j] - N[4][j]); }, ctl, 4);
}

template <class T, class CT, int LOGN>
RK_DEV double attempt_if34_family(const Ctx<T, CT, LOGN>& x, double hd, bool adaptive, const rk_controller& ctl,
                                  int& nl_count) {
  const cx<T>* u = x.u;
  cx<T>* const* N = x.N;
  const T h = T(hd);
  const T r6 = T(1.0 / 6.0), r3 = T(1.0 / 3.0);
  // rkstiff/if34.py:120-130 (IF4: if4.py:112-121)
  nl_eval(x, [&](int j) { return cmul(x.c(CIF_E2, j), u[j]) + cmul(h * x.c(CIF_E2, j), N[0][j]) * T(0.5); }, N[1]);
  nl_eval(x, [&](int j) { return cmul(x.c(CIF_E2, j), u[j]) + (h * N[1][j]) * T(0.5); }, N[2]);
  nl_eval(x, [&](int j) { return cmul(x.c(CIF_E, j), u[j]) + cmul(h * x.c(CIF_E2, j), N[2][j]); }, N[3]);
  nl_count += 3;
  auto k5 = [&](int j) {
    cx<T> s = ((cmul(x.c(CIF_E, j), N[0][j]) * r6 + cmul(x.c(CIF_E2, j), N[1][j]) * r3) +
               cmul(x.c(CIF_E2, j), N[2][j]) * r3) + N[3][j] * r6;
    return cmul(x.c(CIF_E, j), u[j]) + h * s;
  };
  const cx<T>* un = x.unew;
  if (!adaptive) {
    for (int j = x.g.tid; j < x.m; j += x.g.nthr) x.unew[j] = k5(j);
    x.g.sync();
    nl_eval(x, [&](int j) { return un[j]; }, N[0]);
    nl_count += 1;
    return 0.0;
  }
  double mx = write_unew(x, k5);
  nl_eval(x, [&](int j) { return un[j]; }, N[4]);
  nl_count += 1;
  return controller_s(x, mx, [&](int j) { return (h * (N[3][j] - N[4][j])) * r6; }, ctl, 4);
}

template <class T, class CT, int LOGN>
RK_DEV double attempt_if45dp(const Ctx<T, CT, LOGN>& x, double hd, const rk_controller& ctl, int& nl_count) {
  const cx<T>* u = x.u;
  cx<T>* const* N = x.N;
  const T a76 = T(dp_a76(hd)), r6 = T(dp_r6(hd)), r7 = T(dp_r7(hd));
  // rkstiff/if45dp.py:140-179
  nl_eval(x, [&](int j) { return cmul(x.c(CDP_E15, j), u[j]) + cmul(x.c(CDP_A21, j), N[0][j]); }, N[1]);
  nl_eval(x, [&](int j) {
    return (cmul(x.c(CDP_E310, j), u[j]) + cmul(x.c(CDP_A31, j), N[0][j])) + cmul(x.c(CDP_A32, j), N[1][j]);
  }, N[2]);
  nl_eval(x, [&](int j) {
    return ((cmul(x.c(CDP_E45, j), u[j]) + cmul(x.c(CDP_A41, j), N[0][j])) + cmul(x.c(CDP_A42, j), N[1][j])) +
           cmul(x.c(CDP_A43, j), N[2][j]);
  }, N[3]);
  nl_eval(x, [&](int j) {
    return (((cmul(x.c(CDP_E89, j), u[j]) + cmul(x.c(CDP_A51, j), N[0][j])) + cmul(x.c(CDP_A52, j), N[1][j])) +
            cmul(x.c(CDP_A53, j), N[2][j])) + cmul(x.c(CDP_A54, j), N[3][j]);
  }, N[4]);
  nl_eval(x, [&](int j) {
    return ((((cmul(x.c(CDP_E, j), u[j]) + cmul(x.c(CDP_A61, j), N[0][j])) + cmul(x.c(CDP_A62, j), N[1][j])) +
             cmul(x.c(CDP_A63, j), N[2][j])) + cmul(x.c(CDP_A64, j), N[3][j])) + cmul(x.c(CDP_A65, j), N[4][j]);
  }, N[5]);
  nl_count += 5;
  auto k7 = [&](int j) {
    return ((((cmul(x.c(CDP_E, j), u[j]) + cmul(x.c(CDP_A71, j), N[0][j])) + cmul(x.c(CDP_A73, j), N[2][j])) +
             cmul(x.c(CDP_A74, j), N[3][j])) + cmul(x.c(CDP_A75, j), N[4][j])) + a76 * N[5][j];
  };
  double mx = write_unew(x, k7);
  const cx<T>* un = x.unew;
  nl_eval(x, [&](int j) { return un[j]; }, N[6]);
  nl_count += 1;
  return controller_s(x, mx, [&](int j) {
    return ((((cmul(x.c(CDP_R1, j), N[0][j]) + cmul(x.c(CDP_R3, j), N[2][j])) + cmul(x.c(CDP_R4, j), N[3][j])) +
             cmul(x.c(CDP_R5, j), N[4][j])) + r6 * N[5][j]) + r7 * N[6][j];
  }, ctl, 5);
}

template <class T, class CT, int METHOD, int LOGN>
RK_DEV double run_attempt(const Ctx<T, CT, LOGN>& x, double h, const rk_controller& ctl, int& nl_count) {
  switch (METHOD) {
    case RK_ETD35: return attempt_etd35_family(x, true, ctl, nl_count);
    case RK_ETD5: return attempt_etd35_family(x, false, ctl, nl_count);
    case RK_ETD34: return attempt_etd34_family(x, true, ctl, nl_count);
    case RK_ETD4: return attempt_etd34_family(x, false, ctl, nl_count);
    case RK_IF34: return attempt_if34_family(x, h, true, ctl, nl_count);
    case RK_IF4: return attempt_if34_family(x, h, false, ctl, nl_count);
    case RK_IF45DP: return attempt_if45dp(x, h, ctl, nl_count);
  }
  return 0.0;
}

// ---------------------------------------------------------------------------------
// step-size rules (rkstiff/solveras.py:492-554); class constants MIN_S, MAX_S, MAX_LOOPS
// ---------------------------------------------------------------------------------
RK_DEV double reject_h(double s, double h, const rk_controller& c) {
  if (isinf(s) || isnan(s)) return 0.25 * h;
  s = fmax(s, 0.25);
  s = fmin(s, c.decr_f);
  return s * h;
}
RK_DEV double accept_h(double s, double h, const rk_controller& c) {
  s = fmin(s, 4.0);
  return s > c.incr_f ? s * h : h;
}

// Fraction of sum |unew|^2 held by the top quarter of the modes (a spectral-resolution
// feature of the learned controller and of the attempt log).
template <class T, class CT, int LOGN>
RK_DEV float tail_fraction(const Ctx<T, CT, LOGN>& x) {
  df tail{0.f, 0.f}, tot{0.f, 0.f};
  // the top quarter of |k|: rfft modes j >= 3m/4; a full fft grid (m = n) has |k| >= 3n/8
  // at indices [3n/8, 5n/8]
  const bool full = x.m == x.n;
  const int j0 = full ? (3 * x.n) / 8 : (3 * x.m) / 4;
  const int j1 = full ? (5 * x.n) / 8 : x.m - 1;
  for (int j = x.g.tid; j < x.m; j += x.g.nthr) {
    const cx<T> v = x.unew[j];
    const float a2 = (float)(v.x * v.x + v.y * v.y);
    tot = df_add(tot, a2);
    if (j >= j0 && j <= j1) tail = df_add(tail, a2);
  }
  double st, sa;
  group_sum2_df(x.g, x.red, tail, tot, st, sa);
  x.g.sync();
  return sa > 0.0 ? (float)(st / sa) : 0.f;
}

RK_DEV float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
RK_DEV float safe_log(double v) { return (v > 0.0 && v < 1e300) ? (float)log(v) : (v > 0.0 ? 690.f : -690.f); }
// log v clamped to [-8, 8] in FP32 (a NaN or non-positive v gives -8): the learned
// controller's log s feature, which needs no FP64 log
RK_DEV float log_clamped8(double v) {
  const float f = (float)v;
  return v > 0.0 ? clampf(__logf(f), -8.f, 8.f) : -8.f;
}

// ---------------------------------------------------------------------------------
// snapshot stream: one slot of the mapped host ring per snapshot
// ---------------------------------------------------------------------------------
RK_DEV uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Writes the instance's state u (m modes) at time t, step `step` into the next ring slot.
// Thread 0 claims the slot and waits (bounded by ring_timeout_ms) until the host has taken
// its previous occupant; the group then writes the states, fences them to the system scope
// and thread 0 publishes the slot (ready = k + 1).  Returns false if the wait ran out (the
// slot stays unpublished).  `red` provides the group's broadcast word.
template <class T>
RK_DEV bool ring_write(const rk_batch& b, int inst, const Group& g, const cx<T>* u, int m, double t, int64_t step,
                       double* red) {
  long long* slot_s = reinterpret_cast<long long*>(red + 65);
  g.sync();  // earlier readers of the broadcast word are done
  if (g.tid == 0) {
    const long long k = (long long)atomicAdd(b.ring_head, 1ull);
    const volatile int64_t* tail = b.ring_tail;
    const uint64_t t0 = global_ns(), lim = (uint64_t)b.ring_timeout_ms * 1000000ull;
    long long res = k;
    while (k - (long long)*tail >= (long long)b.ring_slots) {
      if (global_ns() - t0 > lim) {
        res = -1;
        break;
      }
      __nanosleep(2000);
    }
    *slot_s = res;
  }
  g.sync();
  const long long k = *slot_s;
  if (k < 0) return false;
  unsigned char* slot = static_cast<unsigned char*>(b.ring_data) + (k % b.ring_slots) * b.ring_slot_bytes;
  cx<T>* dst = reinterpret_cast<cx<T>*>(slot + RK_RING_HEADER);
  for (int j = g.tid; j < m; j += g.nthr) dst[j] = u[j];
  if (g.tid == 0) {
    int64_t* hdr = reinterpret_cast<int64_t*>(slot);
    hdr[1] = inst;
    reinterpret_cast<double*>(hdr)[2] = t;
    hdr[3] = step;
  }
  __threadfence_system();
  g.sync();
  if (g.tid == 0) {
    __threadfence_system();
    *reinterpret_cast<volatile int64_t*>(slot) = (int64_t)k + 1;
  }
  return true;
}

// ---------------------------------------------------------------------------------
// one instance, start to pause/finish
//
// PLACE selects where the instance's arrays live: PL_GLOBAL (all in the global scratch
// slab), PL_SMEM_STATE (u, unew and the stage arrays in shared memory, coefficients in
// the global slab), PL_SMEM_ALL (everything in shared memory; the coefficients are then
// rebuilt at the start of every launch).
// ---------------------------------------------------------------------------------
enum { PL_GLOBAL = 0, PL_SMEM_STATE = 1, PL_SMEM_ALL = 2, PL_SMEM_U = 3 };

// Coefficient blocks of one instance (rk_batch.coef_blocks = nblk > 1), in its global slab:
// block i at C0 + i * NC * mp, the blocks' h tags and the index of the block the next miss
// replaces after them.  Kept out of line: the learned controller's ladder uses them, the
// plain path does not, and their state would otherwise sit in registers through every
// transform.
// The helpers take the instance's slab pointer and return their results by value: a
// reference to the kernel's rk_batch parameter or to a field of the stepping context would
// give those objects an address, and every later read of them in the stepping loop would then
// come from local memory instead of registers or the parameter bank.
template <class T, class CT, int METHOD>
RK_DEV CT* coef_block0(unsigned char* slab, int mp) {
  constexpr int NVS = SlabShape<T, CT, METHOD>::NVS;
  constexpr int KXW = sizeof(T) == sizeof(float) ? 1 : 0;
  cx<T>* gsl = reinterpret_cast<cx<T>*>(slab);
  return reinterpret_cast<CT*>(reinterpret_cast<T*>(gsl + NVS * mp) + KXW * mp);
}
template <class T, class CT, int METHOD>
RK_DEV double* coef_tags(unsigned char* slab, int m, int nblk) {
  const int64_t bytes = slab_bytes(METHOD, sizeof(T) == 8 ? RK_FP64 : RK_FP32, sizeof(CT) == 2 * sizeof(T), m, nblk);
  return reinterpret_cast<double*>(slab + bytes - RK_TAG_BYTES);
}

template <class CT>
struct CoefPick {
  CT* C;      // the block to use
  double hc;  // coef_block: 1 if the caller rebuilds C, else 0; coef_block_resume: h_coeff
};

// The block whose tag is h (rebuild 0).  Otherwise takes the next block in turn, tags it with
// h (after a barrier: every thread has read the tags before one changes them) and returns it
// with rebuild 1 -- the caller rebuilds that block, and compute_coeffs' closing barrier
// publishes the new tag.
template <class T, class CT, int METHOD>
__device__ __noinline__ CoefPick<CT> coef_block(unsigned char* slab, Group g, int mp, int m, int nblk, double h) {
  double* tags = coef_tags<T, CT, METHOD>(slab, m, nblk);
  CT* const C0 = coef_block0<T, CT, METHOD>(slab, mp);
  const int64_t blk = (int64_t)SlabShape<T, CT, METHOD>::NCX * mp;
  int hit = -1;
  for (int i = 0; i < nblk; ++i)
    if (tags[i] == h) hit = i;
  if (hit >= 0) return CoefPick<CT>{C0 + hit * blk, 0.0};
  long long* next = reinterpret_cast<long long*>(tags + RK_COEF_BLOCKS_MAX);
  const int victim = (int)(*next % nblk);
  g.sync();
  if (g.tid == 0) {
    tags[victim] = h;
    *next = victim + 1;
  }
  return CoefPick<CT>{C0 + victim * blk, 1.0};
}

// At the start of a launch: h_coeff NaN (a fresh record, or a noalloc call) invalidates every
// tag; otherwise the block tagged h_coeff, and if none is, h_coeff is dropped (C unchanged).
template <class T, class CT, int METHOD>
__device__ __noinline__ CoefPick<CT> coef_block_resume(unsigned char* slab, Group g, int mp, int m, int nblk,
                                                       double hc, CT* C) {
  double* tags = coef_tags<T, CT, METHOD>(slab, m, nblk);
  if (hc != hc) {
    g.sync();
    if (g.tid < RK_COEF_BLOCKS_MAX) tags[g.tid] = __longlong_as_double(0x7ff8000000000000ULL);
    if (g.tid == 0) *reinterpret_cast<long long*>(tags + RK_COEF_BLOCKS_MAX) = 0;
    g.sync();
    return CoefPick<CT>{C, hc};
  }
  int found = -1;
  for (int i = 0; i < nblk; ++i)
    if (tags[i] == hc) found = i;
  if (found < 0) return CoefPick<CT>{C, __longlong_as_double(0x7ff8000000000000ULL)};  // rebuild first
  return CoefPick<CT>{coef_block0<T, CT, METHOD>(slab, mp) + found * (int64_t)SlabShape<T, CT, METHOD>::NCX * mp, hc};
}

// u <- unew after an accepted step.  With the new state in N2's array the two arrays swap
// roles: the old u array becomes N2 (and the next new state's home).
template <bool U2, class X>
RK_DEV void accept_swap(X& x) {
  cx_ptr_swap(x.u, U2 ? x.N[1] : x.unew);
  if (U2) x.unew = x.N[1];
  if (x.ulo) cx_ptr_swap(x.ulo, x.unlo);
}

template <class T, class CT, class S, int METHOD, int LOGN, int PLACE>
RK_DEV void run_instance(const rk_batch& b, int inst, const Group& g, cx<T>* fa, cx<T>* fb, double* red,
                         unsigned char* sm_slab, const cx<T>* tws, float* mlp_s, int nfft,
                         const unsigned char* mlpw) {
  using Tr = Traits<METHOD>;
  Ctx<T, CT, LOGN> x;
  x.g = g;
  x.n = LOGN > 0 ? (1 << LOGN) : b.n[inst];
  x.logn = LOGN > 0 ? LOGN : 31 - __clz(x.n);
  x.nl_kind = b.nl_kind;
  x.m = (b.nl_kind == RK_NL_UUX) ? (x.n / 2 + 1) : x.n;
  x.mp = (int)round_up4(x.m);
  x.nl_c = T(b.nl_coef);
  const int64_t mo = b.mode_off[inst];
  x.lin = reinterpret_cast<const cx<double>*>(b.lin_op) + mo;
  cx<T>* gsl = reinterpret_cast<cx<T>*>(reinterpret_cast<char*>(b.slab) + b.slab_off[inst]);
  cx<T>* ssl = PLACE == PL_GLOBAL ? gsl : reinterpret_cast<cx<T>*>(sm_slab);
  constexpr bool U2 = unew_in_n2(METHOD);
  using SS = SlabShape<T, CT, METHOD>;
  constexpr int NV = SS::NV;    // state vectors u, (unew,) N1..NN
  constexpr int NVS = SS::NVS;  // and, with the double-float state, the low words of u and unew
  x.u = ssl;
  for (int i = 0; i < 8; ++i) x.N[i] = (i < Tr::NN) ? ssl + ((U2 ? 1 : 2) + i) * x.mp : nullptr;
  x.unew = U2 ? x.N[1] : ssl + x.mp;
  // the low words of u and unew: in shared memory with everything else under PL_SMEM_ALL
  // (small grids, where shared memory has room), in the global slab otherwise (they cost a
  // resident block of the larger grids' shared-memory placements)
  cx<T>* lsl = PLACE == PL_SMEM_ALL ? ssl : gsl;
  x.ulo = SS::DF ? lsl + NV * x.mp : nullptr;
  x.unlo = SS::DF ? lsl + (NV + 1) * x.mp : nullptr;
  if constexpr (PLACE == PL_SMEM_U) {
    // u and the new-state array (N2's for ETD35 / ETD5) in shared memory: u is read by every
    // stage combination, and the two swap roles on every accepted step; the other stage
    // arrays stay in the global slab (their slots of u and N2 there go unused)
    cx<T>* sm = reinterpret_cast<cx<T>*>(sm_slab);
    for (int i = 0; i < 8; ++i) x.N[i] = (i < Tr::NN) ? gsl + ((U2 ? 1 : 2) + i) * x.mp : nullptr;
    x.u = sm;
    if (U2) x.N[1] = sm + x.mp;
    x.unew = U2 ? x.N[1] : sm + x.mp;
  }
  // global slab: [NVS vectors | FP32 wavenumbers | coefficient block(s) of NCX arrays | tags]
  constexpr int KXW = sizeof(T) == sizeof(float) ? 1 : 0;
  x.C = PLACE == PL_SMEM_ALL ? reinterpret_cast<CT*>(ssl + NVS * x.mp)
                             : reinterpret_cast<CT*>(reinterpret_cast<T*>(gsl + NVS * x.mp) + KXW * x.mp);
  x.fa = fa;
  x.fb = fb;
  x.red = red;
  x.tw = reinterpret_cast<const cx<T>*>(b.twiddle);
  x.tws = tws;
  x.cf = make_ctlf(b.ctl);
  x.want_tail = false;
  x.tail_frac = -1.f;
  const EtdCfg ec{b.etd.modecutoff, b.etd.contour_radius, b.etd.contour_points};
  const rk_controller ctl = b.ctl;

  rk_inst_state st = b.state[inst];
  // only RUNNING instances step; finished or failed ones keep their record untouched
  if (st.status != RK_ST_RUNNING) return;
  {
    // the shared-memory transforms (and the noalloc slabs) are sized for nfft points: an
    // instance of another size is refused rather than stepped out of bounds
    const int ni = b.n[inst];
    const bool bad = LOGN > 0 ? (ni != (1 << LOGN)) : (ni < 4 || (ni & (ni - 1)) != 0 || ni > nfft);
    if (bad) {
      if (g.tid == 0) b.state[inst].status = RK_ST_BAD_SIZE;
      g.sync();
      return;
    }
  }
  x.kx = nullptr;
  if (b.kx) {
    if constexpr (sizeof(T) == sizeof(double)) {
      x.kx = b.kx + mo;
    } else {
      // FP32: a working-precision copy after the coefficient block (shared memory when the
      // stage arrays are there, the global slab otherwise), filled once per launch
      T* kw = (PLACE == PL_GLOBAL || PLACE == PL_SMEM_U) ? reinterpret_cast<T*>(gsl + NVS * x.mp)
            : PLACE == PL_SMEM_STATE ? reinterpret_cast<T*>(ssl + NV * x.mp)
                                     : reinterpret_cast<T*>(x.C + SS::NCX * x.mp);
      const double* kd = b.kx + mo;
      for (int j = g.tid; j < x.m; j += g.nthr) kw[j] = T(kd[j]);
      x.kx = kw;
    }
  }
  cx<T>* uio = reinterpret_cast<cx<T>*>(b.u) + mo;
  for (int j = g.tid; j < x.m; j += g.nthr) x.u[j] = uio[j];
  // Double-float state: u's low words continue from the previous launch of this evolve (it
  // saved them in the slab's first low-word array and set reserved_i), else start at zero (a
  // fresh state, a step() call, a noalloc call); E's low words come with the coefficients.
  if (x.ulo) {
    cx<T>* lo0 = gsl + NV * x.mp;
    const bool keep = b.run_mode == RK_RUN_EVOLVE && st.reserved_i == 1;
    if (!keep) {
      for (int j = g.tid; j < x.m; j += g.nthr) x.ulo[j] = cx<T>{T(0), T(0)};
    } else if (x.ulo != lo0) {
      for (int j = g.tid; j < x.m; j += g.nthr) x.ulo[j] = lo0[j];
    }
  }
  g.sync();

  double t = st.t, tf = st.tf, h = st.h;
  double hc = PLACE == PL_SMEM_ALL ? nan_d() : st.h_coeff;
  // Coefficient blocks (b.coef_blocks > 1): see coef_block / coef_block_resume
  const int nblk =
      (!Tr::ADAPT || PLACE == PL_SMEM_ALL || b.coef_blocks <= 1) ? 1 : min(b.coef_blocks, RK_COEF_BLOCKS_MAX);
  if (nblk > 1) {
    const CoefPick<CT> r =
        coef_block_resume<T, CT, METHOD>(reinterpret_cast<unsigned char*>(gsl), g, x.mp, x.m, nblk, hc, x.C);
    x.C = r.C;
    hc = r.hc;
  }
  // the learned controller's step-size ladder starts at the instance's first step size
  const bool ladder = Tr::ADAPT && b.ladder != 0 && b.mlp != nullptr;
  double h0 = st.reserved_d;
  if (ladder && (st.steps == 0 && st.attempts == 0)) h0 = st.h;
  bool accept = st.accept != 0;
  bool n1_valid = false;
  const bool resumed = st.steps > 0;
  int status = RK_ST_RUNNING;
  int64_t steps_this = 0;
  int snap = 0;
  int64_t attempts = 0, rejects = 0, nl_evals = 0, coeff_updates = 0;
  double s_last = st.s_last, h_used = st.h_used, h_sug = st.h_suggest;

  // learned-controller features and the attempt log
  const bool learned = Tr::ADAPT && b.mlp != nullptr;
  const bool want_tail = learned || b.attempt_log != nullptr;
  x.want_tail = want_tail;
  float s_prev = 0.f, s_prev2 = 0.f, acc_prev = 1.f, tail_prev = -1.f;  // log s history starts neutral
  double h_prev = 0.0;

  if (b.run_mode == RK_RUN_EVOLVE && !(t < tf)) status = RK_ST_DONE;
  while (status == RK_ST_RUNNING) {
    if (Tr::ADAPT) {
      int numloops = 0;
      double hs = h;
      for (;;) {
        if (h != hc) {  // exact compare, as the reference's _update_coeffs
          bool rebuild = true;
          if (nblk > 1) {
            const CoefPick<CT> r = coef_block<T, CT, METHOD>(reinterpret_cast<unsigned char*>(gsl), g, x.mp, x.m, nblk, h);
            x.C = r.C;
            rebuild = r.hc != 0.0;
          }
          if (rebuild) {
            compute_coeffs<T, CT, S, METHOD>(x, h, ec);
            ++coeff_updates;
          }
          hc = h;
        }
        int nlc = 0;
        if (!n1_valid || (METHOD == RK_ETD35 && accept)) {
          const cx<T>* uu = x.u;
          nl_eval(x, [&](int j) { return uu[j]; }, x.N[0]);
          // an FSAL method resuming mid-run re-derives N1 = N(u); it is not a new evaluation
          if (!(resumed && !n1_valid && Tr::FSAL)) ++nlc;
          n1_valid = true;
        }
        x.tail_frac = -1.f;
        double s = run_attempt<T, CT, METHOD>(x, h, ctl, nlc);
        nl_evals += nlc;
        s_last = s;
        const bool ok = !(isinf(s) || isnan(s) || s < 1.0);
        const float tail = !want_tail ? 0.f : (x.tail_frac >= 0.f ? x.tail_frac : tail_fraction(x));
        if (b.attempt_log && g.tid == 0) {
          const int64_t k = st.attempts + attempts;
          if (k < b.log_cap) {
            float* rec = b.attempt_log + ((int64_t)inst * b.log_cap + k) * RK_LOG_FIELDS;
            rec[0] = (float)t;
            rec[1] = (float)h;
            rec[2] = isnan(s) ? -1.f : (isinf(s) || s > 1e30 ? 1e30f : (float)s);
            rec[3] = ok ? 1.f : 0.f;
            rec[4] = tail;
            rec[5] = (float)numloops;
            rec[6] = (float)x.n;
            rec[7] = (float)METHOD;
          }
        }
        ++attempts;
        // log s feeds only the learned controller's features (an FP64 log per attempt
        // would otherwise hold the slow FP64 pipe)
        const float f_s = learned ? log_clamped8(s) : 0.f;
        if (!ok) {
          accept = false;
          ++rejects;
          h_prev = h;
          h = reject_h(s, h, ctl);
          if (ladder) h = ladder_step(h, h0, true);  // a rejection never grows the step
          ++numloops;
          s_prev2 = s_prev;
          s_prev = f_s;
          acc_prev = 0.f;
          tail_prev = tail;
          if (numloops > 50) { status = RK_ST_MAX_LOOPS; break; }
          if (h < ctl.minh) { status = RK_ST_MIN_STEP; break; }
        } else {
          accept = true;
          if (learned) {
            // The MLP estimates a bounded correction y to log s: log s of the next attempt,
            // rescaled to this h, is taken as log s + clamp(y, -1, 1) and the next step is
            // h exp(that) / target.  The error test above still judges every attempt.
            if (g.tid == 0) {
              float* f = mlp_s;
              const float lt = log10f(tail + 1e-30f);
              f[0] = f_s;
              f[1] = s_prev;
              f[2] = s_prev2;
              f[3] = h_prev > 0.0 ? clampf(__logf((float)h / (float)h_prev), -3.f, 3.f) : 0.f;
              f[4] = acc_prev;
              f[5] = fminf((float)numloops, 5.f);
              f[6] = clampf(lt, -30.f, 0.f);
              f[7] = tail_prev >= 0.f ? clampf(lt - log10f(tail_prev + 1e-30f), -10.f, 10.f) : 0.f;
            }
            g.sync();
            const float y = mlp_infer(g, mlpw, mlp_s, mlp_s + MLP_IN);
            const float d = fminf(fmaxf(y, -1.f), 1.f);
            const double fac = (double)fminf(fmaxf(__expf(f_s + d) / b.mlp_target, 0.5f), 4.f);
            hs = (y == y) ? h * fac : accept_h(s, h, ctl);
            if (ladder) hs = ladder_step(hs, h0, false);
          } else {
            hs = accept_h(s, h, ctl);
          }
          h_prev = h;
          s_prev2 = s_prev;
          s_prev = f_s;
          acc_prev = 1.f;
          tail_prev = tail;
          break;
        }
      }
      if (status != RK_ST_RUNNING) break;
      // accepted: u <- unew; FSAL methods carry N(unew) into N1
      accept_swap<U2>(x);
      if (Tr::FSAL) { cx<T>* tmp = x.N[0]; x.N[0] = x.N[Tr::NN - 1]; x.N[Tr::NN - 1] = tmp; }
      t += h;
      h_used = h;
      h_sug = hs;
      h = (t + hs > tf) ? tf - t : hs;
      // A next step that can no longer advance t (or, from the learned rule, below minh)
      // would repeat forever; the reference would loop, this ends the instance instead.
      if (t < tf && (t + h == t || (learned && h < ctl.minh))) status = RK_ST_MIN_STEP;
    } else {
      if (h != hc) {
        compute_coeffs<T, CT, S, METHOD>(x, h, ec);
        hc = h;
        ++coeff_updates;
      }
      int nlc = 0;
      if (!n1_valid) {
        const cx<T>* uu = x.u;
        nl_eval(x, [&](int j) { return uu[j]; }, x.N[0]);
        if (!resumed) ++nlc;
        n1_valid = true;
      }
      run_attempt<T, CT, METHOD>(x, h, ctl, nlc);
      nl_evals += nlc;
      ++attempts;
      accept_swap<U2>(x);
      t += h;
      h_used = h;
    }
    ++st.steps;
    ++steps_this;
    if (status != RK_ST_RUNNING) break;
    bool ring_full = false;
    if (b.store_freq > 0 && (st.steps % b.store_freq) == 0) {
      if (b.ring_data) {
        ring_full = !ring_write<T>(b, inst, g, x.u, x.m, t, st.steps, red);
        if (!ring_full) ++snap;
      } else if (snap < b.snap_cap) {
        cx<T>* su = reinterpret_cast<cx<T>*>(b.snap_u) + (int64_t)b.snap_cap * mo + (int64_t)snap * x.m;
        for (int j = g.tid; j < x.m; j += g.nthr) su[j] = x.u[j];
        if (g.tid == 0) b.snap_t[(int64_t)inst * b.snap_cap + snap] = t;
        ++snap;
      }
    }
    if (ring_full) status = RK_ST_SNAP_FULL;
    else if (b.run_mode == RK_RUN_STEP) status = RK_ST_STEP_DONE;
    else if (!(t < tf)) status = RK_ST_DONE;
    else if (b.store_freq > 0 && !b.ring_data && snap >= b.snap_cap) status = RK_ST_SNAP_FULL;
    else if (steps_this >= b.max_steps) status = RK_ST_ITER_CAP;
  }
  g.sync();
  for (int j = g.tid; j < x.m; j += g.nthr) uio[j] = x.u[j];
  if (x.ulo) {
    // the low words of the final state, where the next launch of this evolve looks for them
    cx<T>* lo0 = gsl + NV * x.mp;
    if (x.ulo != lo0)
      for (int j = g.tid; j < x.m; j += g.nthr) lo0[j] = x.ulo[j];
  }
  if (g.tid == 0) {
    if (x.ulo) st.reserved_i = 1;
    st.t = t;
    st.h = h;
    st.h_coeff = PLACE == PL_SMEM_ALL ? nan_d() : hc;
    if (ladder) st.reserved_d = h0;
    st.h_used = h_used;
    st.h_suggest = h_sug;
    st.s_last = s_last;
    st.status = status;
    st.accept = accept ? 1 : 0;
    st.snap_count = snap;
    st.attempts += attempts;
    st.rejects += rejects;
    st.nl_evals += nl_evals;
    st.coeff_updates += coeff_updates;
    b.state[inst] = st;
  }
  // The swapped u/unew roles mean the first state array may no longer hold u; only the
  // copy in `uio` is authoritative between launches, so nothing else is persisted.
  g.sync();
}

RK_HD constexpr size_t align16(size_t v) { return (v + 15) & ~size_t(15); }
// offset of the block-wide copy of the inference buffer (learned-controller launches) and
// its bytes
template <class T, int LOGN>
RK_HD constexpr size_t block_extra_offset(int ngroups, int group_smem) {
  return (size_t)ngroups * group_smem + (LOGN > 0 ? align16(sizeof(cx<T>) * twiddle_rows<LOGN>()) : 0);
}
RK_HD constexpr size_t learned_extra_bytes() { return align16(RK_MLP_PACK_BYTES); }

// A block holds blockDim.x / gthreads independent groups; each group owns one slice of
// shared memory: [fa | fb] FFT buffers of fpad_size(nfft) points, 64 doubles of reduction
// scratch, the work-item slot, then (PLACE > 0) the instance arrays (group_smem bytes in
// all).  Compile-time-size kernels put the block's twiddle rows (fill_twiddle_rows) after
// the group slices.  A one-warp group synchronises with __syncwarp, a multi-warp group with a
// named barrier (one per group), a block-wide group with __syncthreads.
template <class T, class CT, class S, int METHOD, int LOGN, int PLACE>
__global__ void __launch_bounds__(512, 1) evolve_kernel(const rk_batch b, const int32_t* __restrict__ order,
                                                        int64_t count, int32_t* queue, int nfft, int gthreads,
                                                        int group_smem) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ngroups = blockDim.x / gthreads;
  const int gi = threadIdx.x / gthreads;
  cx<T>* tws = nullptr;
  if constexpr (LOGN > 0) {
    tws = reinterpret_cast<cx<T>*>(smem + (size_t)ngroups * group_smem);
    fill_twiddle_rows<T, LOGN>(tws, reinterpret_cast<const cx<T>*>(b.twiddle), threadIdx.x, blockDim.x);
    __syncthreads();
  }
  // Launches with the learned controller: the inference buffer, copied once per block into
  // shared memory after the group slices and the twiddle rows.  (The coefficient rebuilds,
  // one per attempt under this controller, read the series table from global memory: a
  // shared-memory copy reached through the out-of-line rebuild's pointer argument made each
  // rebuild slower, 12 of 50 ms on 1546 Burgers instances to t = 5.)
  const unsigned char* mlpw = reinterpret_cast<const unsigned char*>(b.mlp);
  if (b.mlp != nullptr) {
    unsigned char* ex = smem + block_extra_offset<T, LOGN>(ngroups, group_smem);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(b.mlp);
    uint32_t* dst = reinterpret_cast<uint32_t*>(ex);
    for (int i = threadIdx.x; i < RK_MLP_PACK_BYTES / 4; i += blockDim.x) dst[i] = src[i];
    mlpw = ex;
    __syncthreads();
  }
  unsigned char* base = smem + (size_t)gi * group_smem;
  cx<T>* fa = reinterpret_cast<cx<T>*>(base);
  cx<T>* fb = fa + fpad_size(nfft);
  double* red = reinterpret_cast<double*>(fb + fpad_size(nfft));
  int* item_s = reinterpret_cast<int*>(red + 64);
  float* mlp_s = reinterpret_cast<float*>(red + 66);
  unsigned char* sm_slab = reinterpret_cast<unsigned char*>(red + 66 + MLP_SCRATCH_FLOATS / 2);
  const Group g{(int)(threadIdx.x % gthreads), gthreads, gthreads == 32 ? -1 : (ngroups == 1 ? 0 : 1 + gi)};
  for (;;) {
    if (g.tid == 0) *item_s = atomicAdd(queue, 1);
    g.sync();
    const int item = *item_s;
    g.sync();
    if (item >= count) break;
    const int inst = order ? order[item] : item;
    run_instance<T, CT, S, METHOD, LOGN, PLACE>(b, inst, g, fa, fb, red, sm_slab, tws, mlp_s, nfft, mlpw);
  }
}

template <class T, class CT, class S, int METHOD>
__global__ void coeff_kernel(int m, const double* lin, double h, rk_etd_config etd, CT* out) {
  // standalone coefficient evaluation for one operator (blocks split the modes)
  const Group g{(int)threadIdx.x, (int)blockDim.x, 0};
  const int per = blockDim.x;
  const int j0 = blockIdx.x * per;
  const EtdCfg ec{etd.modecutoff, etd.contour_radius, etd.contour_points};
  // arrays of length m, shifted so that c*m + j addresses mode j0 + j
  compute_coeffs_impl<CT, S, METHOD, sizeof(T) == sizeof(float)>(g, min(per, m - j0), m,
                                                                reinterpret_cast<const cx<double>*>(lin) + j0,
                                                                out + j0, h, ec);
}

// Coefficients with the reference's matrix-form psi values (rk_etd_config.contour_at_zero):
// for each mode the mean over the zero-centred contour nodes r_q of r_q psi_k(r_q) /
// (r_q - c z), c the scale of the slot -- the reference's non-diagonal psi-matrices
// (etd35.py:602-658) on one eigenvalue.  A warp per mode, lanes over the nodes; its own
// kernel, so that none of its registers weigh on the stepping kernels.
template <class CT, class S, int METHOD>
__global__ void coeff_zero_contour_kernel(int m, const double* lin_, double h, rk_etd_config etd, CT* C) {
  constexpr int NP = (METHOD == RK_ETD35 || METHOD == RK_ETD5) ? RK_PSI35_N : RK_PSI34_N;
  constexpr int NC = Traits<METHOD>::NC;
  const cx<double>* lin = reinterpret_cast<const cx<double>*>(lin_);
  const EtdCfg ec{etd.modecutoff, etd.contour_radius, etd.contour_points};
  const int mp = m;
  const int lane = threadIdx.x & 31;
  const int j = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (j >= m) return;
  S z = load_z<S>(lin, j, h);
  const cx<double> zc = to_cx(z);
  cx<double> acc[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) acc[k] = cx<double>{0.0, 0.0};
  for (int q = lane; q < ec.np; q += 32) {
    const cx<double> r = contour_node(ec, q);
    const cx<double> e = cexp(r);
    const cx<double> p1 = psi1(r, e), p2 = psi2(r, e), p3 = psi3(r, e);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      int order;
      double num, den;
      psi_slot(METHOD, k, order, num, den);
      const cx<double> cz = (num == 1.0 && den == 1.0) ? zc : rdiv(num * zc, den);
      const cx<double> pv = order == 1 ? p1 : (order == 2 ? p2 : p3);
      acc[k] = acc[k] + (r * pv) * crecip(r - cz);
    }
  }
  S P[NP];
#pragma unroll
  for (int k = 0; k < NP; ++k) {
    double re = warp_sum(acc[k].x), im = warp_sum(acc[k].y);
    P[k] = from_cx<S>(rdiv(h * cx<double>{re, im}, (double)ec.np));
  }
  if (lane == 0) {
    S o[NC];
    etd_from_psi<S>(METHOD, z, P, o);
#pragma unroll
    for (int c = 0; c < NC; ++c) store_c(C[c * mp + j], o[c]);
  }
}

// bytes of the per-instance arrays held in shared memory under placement `place`
template <class T, class CT, int METHOD>
inline size_t smem_slab_bytes(int place, int64_t m) {
  const size_t mp = (size_t)round_up4(m);
  size_t bytes = 0;
  using SS = SlabShape<T, CT, METHOD>;
  if (place == PL_SMEM_U) return 2 * mp * sizeof(cx<T>);  // u and the new-state array
  // the state vectors; under PL_SMEM_ALL with the double-float state's low words
  if (place >= PL_SMEM_STATE) bytes += (size_t)(place == PL_SMEM_ALL ? SS::NVS : SS::NV) * mp * sizeof(cx<T>);
  if (place >= PL_SMEM_ALL) bytes += SS::NCX * mp * sizeof(CT);
  if (place >= PL_SMEM_STATE && sizeof(T) == sizeof(float)) bytes += mp * sizeof(T);  // wavenumbers
  return bytes;
}

// smem bytes of the evolve kernel's FFT buffers and scratch for complex FFT length nfft
template <class T> inline size_t evolve_smem(int nfft) {
  return 2 * (size_t)fpad_size(nfft) * sizeof(cx<T>) + (66 + MLP_SCRATCH_FLOATS / 2) * sizeof(double);
}

}  // namespace rk
