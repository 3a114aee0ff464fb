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

// ---------------------------------------------------------------------------------
// Thread groups: `nthr` consecutive threads (a multiple of 32) that own one instance.
// A group that spans the whole CTA uses barrier 0; sub-CTA groups use named barriers.
// ---------------------------------------------------------------------------------
struct Group {
  int tid;    // rank inside the group
  int nthr;   // threads in the group
  int bar;    // hardware barrier id
  RK_DEV void sync() const {
    if (bar == 0) {
      __syncthreads();
    } else {
      asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthr) : "memory");
    }
  }
};

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
