// Common device helpers for the rkstiff GB300 stepping kernels: complex arithmetic,
// thread-group barriers and reductions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rkstiff_gb300.h"

#define RK_DEV __device__ __forceinline__
#define RK_HD __host__ __device__ __forceinline__

namespace rk {

// ---------------------------------------------------------------------------------
// complex numbers (interleaved re, im; 8-byte aligned for float, 16-byte for double)
// ---------------------------------------------------------------------------------
template <class T>
struct alignas(2 * sizeof(T)) cx {
  T x, y;
};

template <class T> RK_HD cx<T> mk(T a, T b) { return cx<T>{a, b}; }
template <class T> RK_HD cx<T> operator+(cx<T> a, cx<T> b) { return cx<T>{a.x + b.x, a.y + b.y}; }
template <class T> RK_HD cx<T> operator-(cx<T> a, cx<T> b) { return cx<T>{a.x - b.x, a.y - b.y}; }
template <class T> RK_HD cx<T> operator-(cx<T> a) { return cx<T>{-a.x, -a.y}; }
template <class T> RK_HD cx<T> operator*(cx<T> a, cx<T> b) {
  return cx<T>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class T> RK_HD cx<T> operator*(T s, cx<T> a) { return cx<T>{s * a.x, s * a.y}; }
template <class T> RK_HD cx<T> operator*(cx<T> a, T s) { return cx<T>{a.x * s, a.y * s}; }
template <class T> RK_HD cx<T> operator/(cx<T> a, T s) { return cx<T>{a.x / s, a.y / s}; }
template <class T> RK_HD cx<T> conj(cx<T> a) { return cx<T>{a.x, -a.y}; }
// multiply by +i / -i
template <class T> RK_HD cx<T> mul_i(cx<T> a) { return cx<T>{-a.y, a.x}; }
template <class T> RK_HD cx<T> mul_mi(cx<T> a) { return cx<T>{a.y, -a.x}; }

// coefficient x vector: a real coefficient scales both parts, a complex one multiplies.
template <class T> RK_HD cx<T> cmul(T c, cx<T> v) { return cx<T>{c * v.x, c * v.y}; }
template <class T> RK_HD cx<T> cmul(cx<T> c, cx<T> v) { return c * v; }

// Smith's complex division (the algorithm NumPy uses for complex128 true_divide).
RK_HD cx<double> cdiv(cx<double> a, cx<double> b) {
  double abr = fabs(b.x), abi = fabs(b.y);
  if (abr >= abi) {
    if (abr == 0.0 && abi == 0.0) return cx<double>{a.x / abr, a.y / abi};
    double rat = b.y / b.x;
    double scl = 1.0 / (b.x + b.y * rat);
    return cx<double>{(a.x + a.y * rat) * scl, (a.y - a.x * rat) * scl};
  } else {
    double rat = b.x / b.y;
    double scl = 1.0 / (b.y + b.x * rat);
    return cx<double>{(a.x * rat + a.y) * scl, (a.y * rat - a.x) * scl};
  }
}

RK_DEV cx<double> cexp(cx<double> z) {
  double e = exp(z.x);
  if (z.y == 0.0) return cx<double>{e, 0.0};
  double s, c;
  sincos(z.y, &s, &c);
  return cx<double>{e * c, e * s};
}

template <class T> RK_DEV cx<T> ld(const cx<T>* p, int64_t i) { return p[i]; }
template <class T> RK_DEV void cx_ptr_swap(cx<T>*& a, cx<T>*& b) {
  cx<T>* t = a;
  a = b;
  b = t;
}

// ---------------------------------------------------------------------------------
// Thread groups: `nthr` consecutive threads (a multiple of 32) that own one instance.
// A group that spans the whole CTA uses barrier 0; sub-CTA groups use named barriers.
// ---------------------------------------------------------------------------------
struct Group {
  int tid;    // rank inside the group
  int nthr;   // threads in the group
  int bar;    // 0: the whole block (__syncthreads); > 0: named barrier; < 0: one warp
  RK_DEV void sync() const {
    if (bar == 0) {
      __syncthreads();
    } else if (bar < 0) {
      __syncwarp();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthr) : "memory");
    }
  }
};

// ---------------------------------------------------------------------------------
// double-float sums: (hi, lo) FP32 pairs with error-free addition (Knuth's TwoSum), a
// 48-bit-significand accumulator that needs no FP64 instruction.
// ---------------------------------------------------------------------------------
struct df {
  float hi, lo;
};
RK_DEV df df_add(df a, df b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float err = (a.hi - (s - bb)) + (b.hi - bb);
  const float lo = err + a.lo + b.lo;
  const float hi = s + lo;
  return df{hi, lo - (hi - s)};
}
RK_DEV df df_add(df a, float b) { return df_add(a, df{b, 0.f}); }
RK_DEV df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    df w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = df_add(v, w);
  }
  return v;
}
RK_DEV float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// group-wide double-float sums of two values (FP32 instructions only); the results are
// returned as FP64 (hi + lo)
RK_DEV void group_sum2_df(const Group& g, double* red, df a, df b, double& sa, double& sb) {
  a = warp_sum_df(a);
  b = warp_sum_df(b);
  const int nw = g.nthr >> 5;
  if (nw == 1) {
    sa = (double)a.hi + (double)a.lo;
    sb = (double)b.hi + (double)b.lo;
    return;
  }
  float* rf = reinterpret_cast<float*>(red);
  const int w = g.tid >> 5;
  g.sync();
  if ((g.tid & 31) == 0) {
    rf[4 * w] = a.hi;
    rf[4 * w + 1] = a.lo;
    rf[4 * w + 2] = b.hi;
    rf[4 * w + 3] = b.lo;
  }
  g.sync();
  df ta{0.f, 0.f}, tb{0.f, 0.f};
  for (int i = 0; i < nw; ++i) {
    ta = df_add(ta, df{rf[4 * i], rf[4 * i + 1]});
    tb = df_add(tb, df{rf[4 * i + 2], rf[4 * i + 3]});
  }
  sa = (double)ta.hi + (double)ta.lo;
  sb = (double)tb.hi + (double)tb.lo;
}

// group-wide double-float sums of two values, kept as double-float pairs (no FP64 at all)
RK_DEV void group_sum2_dff(const Group& g, double* red, df a, df b, df& sa, df& sb) {
  a = warp_sum_df(a);
  b = warp_sum_df(b);
  const int nw = g.nthr >> 5;
  if (nw == 1) {
    sa = a;
    sb = b;
    return;
  }
  float* rf = reinterpret_cast<float*>(red);
  const int w = g.tid >> 5;
  g.sync();
  if ((g.tid & 31) == 0) {
    rf[4 * w] = a.hi;
    rf[4 * w + 1] = a.lo;
    rf[4 * w + 2] = b.hi;
    rf[4 * w + 3] = b.lo;
  }
  g.sync();
  df ta{0.f, 0.f}, tb{0.f, 0.f};
  for (int i = 0; i < nw; ++i) {
    ta = df_add(ta, df{rf[4 * i], rf[4 * i + 1]});
    tb = df_add(tb, df{rf[4 * i + 2], rf[4 * i + 3]});
  }
  sa = ta;
  sb = tb;
}

// Group-wide double-float sums of four values (all threads receive them).
RK_DEV void group_sum4_dff(const Group& g, double* red, df* v) {
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = warp_sum_df(v[q]);
  const int nw = g.nthr >> 5;
  if (nw == 1) return;
  float* rf = reinterpret_cast<float*>(red);  // 8 floats per warp, <= 16 warps
  const int w = g.tid >> 5;
  g.sync();
  if ((g.tid & 31) == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      rf[8 * w + 2 * q] = v[q].hi;
      rf[8 * w + 2 * q + 1] = v[q].lo;
    }
  }
  g.sync();
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    df t{0.f, 0.f};
    for (int i = 0; i < nw; ++i) t = df_add(t, df{rf[8 * i + 2 * q], rf[8 * i + 2 * q + 1]});
    v[q] = t;
  }
}

// group-wide max of a non-negative FP32 value; NaN anywhere gives NaN
RK_DEV float group_max_nan_f(const Group& g, double* red, float v, bool nan) {
  v = warp_max_f(nan ? 0.f : v);
  const unsigned anynan = __ballot_sync(0xffffffffu, nan);
  const int nw = g.nthr >> 5;
  if (nw == 1) return anynan ? __int_as_float(0x7fc00000) : v;
  float* rf = reinterpret_cast<float*>(red);
  const int w = g.tid >> 5;
  g.sync();
  if ((g.tid & 31) == 0) {
    rf[2 * w] = v;
    rf[2 * w + 1] = anynan ? 1.f : 0.f;
  }
  g.sync();
  float m = 0.f, f = 0.f;
  for (int i = 0; i < nw; ++i) {
    m = fmaxf(m, rf[2 * i]);
    f = fmaxf(f, rf[2 * i + 1]);
  }
  return f > 0.f ? __int_as_float(0x7fc00000) : m;
}

// Reductions over a group through a small shared scratch (>= 32 doubles per group).
RK_DEV double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
RK_DEV double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Returns the group-wide sum of two values (all threads receive it).  NaN propagates.
RK_DEV void group_sum2(const Group& g, double* red, double& a, double& b) {
  a = warp_sum(a);
  b = warp_sum(b);
  int w = g.tid >> 5, nw = g.nthr >> 5;
  g.sync();  // previous users of `red` are done
  if ((g.tid & 31) == 0) {
    red[2 * w] = a;
    red[2 * w + 1] = b;
  }
  g.sync();
  double sa = 0.0, sb = 0.0;
  for (int i = 0; i < nw; ++i) {
    sa += red[2 * i];
    sb += red[2 * i + 1];
  }
  a = sa;
  b = sb;
}

// Group-wide max that propagates NaN (a NaN anywhere yields NaN, as numpy's max does).
RK_DEV double group_max_nan(const Group& g, double* red, double v) {
  double nanflag = (v != v) ? 1.0 : 0.0;
  v = (v != v) ? 0.0 : v;
  v = warp_max(v);
  nanflag = warp_max(nanflag);
  int w = g.tid >> 5, nw = g.nthr >> 5;
  g.sync();
  if ((g.tid & 31) == 0) {
    red[2 * w] = v;
    red[2 * w + 1] = nanflag;
  }
  g.sync();
  double m = 0.0, f = 0.0;
  for (int i = 0; i < nw; ++i) {
    m = fmax(m, red[2 * i]);
    f = fmax(f, red[2 * i + 1]);
  }
  return f > 0.0 ? __longlong_as_double(0x7ff8000000000000ULL) : m;
}

RK_DEV double nan_d() { return __longlong_as_double(0x7ff8000000000000ULL); }

}  // namespace rk
