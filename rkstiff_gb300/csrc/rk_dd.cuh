// Double-float ("dd") arithmetic: a value is an unevaluated sum hi + lo of two FP32 numbers
// with |lo| <= ulp(hi)/2, about 48 significant bits, computed on the FP32 pipes (GB300 runs
// FP64 at 1/64 of the FP32 rate).  Error-free transformations: Knuth's TwoSum, the FMA form
// of Dekker's TwoProduct; the reciprocal by one Newton step from the FP32 reciprocal; exp by
// range reduction x = k ln2 + r, r / 16 through a degree-7 Taylor polynomial of e^r - 1 and
// four squarings of (1 + q) kept as q -> 2q + q^2 (so that e^x - 1 keeps its relative
// accuracy for small x).
//
// Used for the ETD psi functions and coefficient combinations of real modes when the
// coefficients are stored in FP32: their results match the FP64 evaluation after rounding
// to FP32 (the combinations cancel by up to ~100x, which FP32 alone would not survive).
#pragma once

#include "rk_coef_series.cuh"
#include "rk_common.cuh"

namespace rk {

struct dd {
  float hi, lo;
};

// compile-time split of a double constant
struct ddc {
  float hi, lo;
  __host__ __device__ constexpr ddc(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
};

RK_DEV dd two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return dd{s, (a - (s - bb)) + (b - bb)};
}
RK_DEV dd quick_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return dd{s, b - (s - a)};
}
RK_DEV dd two_prod(float a, float b) {
  const float p = a * b;
  return dd{p, fmaf(a, b, -p)};
}

RK_DEV dd dd_of(float a) { return dd{a, 0.f}; }
RK_DEV dd dd_of(ddc c) { return dd{c.hi, c.lo}; }

RK_DEV dd operator+(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
RK_DEV dd operator-(dd a) { return dd{-a.hi, -a.lo}; }
RK_DEV dd operator-(dd a, dd b) { return a + (-b); }
RK_DEV dd operator*(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
RK_DEV dd operator*(dd a, float b) {
  dd p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
RK_DEV dd operator*(float b, dd a) { return a * b; }
RK_DEV dd operator*(dd a, ddc c) { return a * dd_of(c); }
// exact scaling by a power of two
RK_DEV dd scale2(dd a, float p2) { return dd{a.hi * p2, a.lo * p2}; }

RK_DEV dd dd_recip(dd b) {
  const float y0 = 1.0f / b.hi;
  const dd e = dd_of(1.f) - b * y0;  // 1 - b y0, small
  return dd_of(y0) + e * y0;
}

// e^x for x.hi in [-87, 80] and em1 = e^x - 1, each to ~2^-46 relative: x = k ln2 + r,
// q = e^(r/16) - 1 by its Taylor polynomial, four squarings q -> 2q + q^2 give e^r - 1; em1
// is q itself when k = 0 (no cancellation for small x) and e - 1 otherwise (|e^x - 1| >
// 0.29 there).  Below -87, e = 0 and em1 = -1 (e^x is below FP32 range).
RK_DEV dd dd_exp(dd xin, dd& em1) {
  // branch-free, so that independent evaluations interleave: clamp, then select
  const bool under = xin.hi < -87.f;
  const dd x = under ? dd{-87.f, 0.f} : xin;
  constexpr ddc LN2(0.6931471805599453);
  const float k = rintf(x.hi * 1.44269504f);
  dd r = x - dd_of(LN2) * k;
  r = scale2(r, 0.0625f);  // |r| <= ln2/32
  // q = e^r - 1 = r (1 + r/2 (1 + r/3 (... (1 + r/7))))
  constexpr ddc I3(1.0 / 3.0), I5(1.0 / 5.0), I6(1.0 / 6.0), I7(1.0 / 7.0);
  dd q = dd_of(1.f) + r * dd_of(I7);
  q = dd_of(1.f) + (r * dd_of(I6)) * q;
  q = dd_of(1.f) + (r * dd_of(I5)) * q;
  q = dd_of(1.f) + scale2(r, 0.25f) * q;
  q = dd_of(1.f) + (r * dd_of(I3)) * q;
  q = dd_of(1.f) + scale2(r, 0.5f) * q;
  q = r * q;
#pragma unroll
  for (int i = 0; i < 4; ++i) q = scale2(q, 2.f) + q * q;
  const dd e1 = dd_of(1.f) + q;
  const int ki = (int)k;
  const dd e{ldexpf(e1.hi, ki), ldexpf(e1.lo, ki)};
  em1 = under ? dd_of(-1.f) : (ki == 0 ? q : e - dd_of(1.f));
  return under ? dd{0.f, 0.f} : e;
}

RK_DEV dd dd_from_double(double v) {
  const float hi = (float)v;
  return dd{hi, (float)(v - (double)hi)};
}

// s1 = (e^x - 1)/x, s2 = (e^x - 1 - x)/x^2, s3 = (e^x - 1 - x - x^2/2)/x^3 by their Taylor
// series (sum x^k / (k + j)!), 16 terms: below 2^-48 relative for |x| <= 1 (ETDConfig caps
// modecutoff at 1).  The inverse factorials 1/(k+3)! as double-float pairs.
RK_DEV void dd_taylor_s123(dd x, dd& s1, dd& s2, dd& s3) {
  constexpr float F[16][2] = {{0x1.5555560000000p-3f, -0x1.5555560000000p-28f},
                              {0x1.5555560000000p-5f, -0x1.5555560000000p-30f},
                              {0x1.1111120000000p-7f, -0x1.ddddde0000000p-32f},
                              {0x1.6c16c20000000p-10f, -0x1.27d27e0000000p-35f},
                              {0x1.a01a020000000p-13f, -0x1.7f97fa0000000p-39f},
                              {0x1.a01a020000000p-16f, -0x1.7f97fa0000000p-42f},
                              {0x1.71de3a0000000p-19f, 0x1.55b1cc0000000p-45f},
                              {0x1.27e4fc0000000p-22f, -0x1.10ec140000000p-47f},
                              {0x1.ae64560000000p-26f, 0x1.fd51380000000p-52f},
                              {0x1.1eed8e0000000p-29f, 0x1.ff1b140000000p-54f},
                              {0x1.6124620000000p-33f, -0x1.8af25e0000000p-58f},
                              {0x1.93974a0000000p-37f, 0x1.180f940000000p-62f},
                              {0x1.ae7f3e0000000p-41f, 0x1.ccee080000000p-67f},
                              {0x1.ae7f3e0000000p-45f, 0x1.ccee080000000p-71f},
                              {0x1.952c780000000p-49f, -0x1.f9ea560000000p-74f},
                              {0x1.6827860000000p-53f, 0x1.dcbecc0000000p-80f}};
  dd acc{F[15][0], F[15][1]};
#pragma unroll
  for (int k = 14; k >= 0; --k) acc = dd{F[k][0], F[k][1]} + x * acc;
  s3 = acc;
  s2 = dd_of(0.5f) + x * s3;
  s1 = dd_of(1.f) + x * s2;
}

// FP32 ETD coefficients of a real mode z = h lambda (z <= 80) in double-float arithmetic,
// h given as a double-float: method ETD35/ETD5 (21 values, layout C35_*) or ETD34/ETD4 (10,
// C34_*).  For |z| >= modecutoff the psi forms are those of fast_real_psi, reassociated so
// that no intermediate leaves FP32 range for |z| up to ~1e18; below it (`small`) the
// psi functions come from their Taylor series, as the FP64 build does.  The combinations
// follow etd_from_psi_e.
RK_DEV void dd_etd_coeffs(int method, double zd, dd h, float* o, bool small = false) {
  const dd z = dd_from_double(zd);
  const dd rz = small ? dd_of(0.f) : dd_recip(z);
  // h psi_1..3 of x = c z from e^x - 1 and r = 1/x (or the series)
  auto psis = [&](dd x, dd em1, dd r, dd* P, bool third) {
    if (small) {
      dd s1, s2, s3;
      dd_taylor_s123(x, s1, s2, s3);
      P[0] = h * s1;
      P[1] = scale2(h, 2.f) * s2;
      if (third) P[2] = (h * 6.f) * s3;
      return;
    }
    const dd d = em1 - x;
    const dd dr = d * r;
    P[0] = h * (em1 * r);
    P[1] = scale2(h, 2.f) * (dr * r);
    if (third) P[2] = (h * 6.f) * (r * (dr * r - dd_of(0.5f)));
  };
  // one exponential: e^(z/4) and m1 = e^(z/4) - 1; the other scales by products, e^(cz)
  // from e1 (relative accuracy for stiff modes) and e^(cz) - 1 from m1 through
  // (1 + m)^2 - 1 = m (m + 2) (relative accuracy for small z)
  dd m1;
  const dd e1 = dd_exp(scale2(z, 0.25f), m1);
  const dd e2 = e1 * e1;
  const dd m2 = m1 * (m1 + dd_of(2.f));
  const dd e4 = e2 * e2;
  const dd m4 = m2 * (m2 + dd_of(2.f));
  if (method == RK_ETD35 || method == RK_ETD5) {
    constexpr ddc F43(4.0 / 3.0);
    const dd z34 = z * 0.75f;
    const dd e3 = e2 * e1;
    const dd m3 = (m1 + m2) + m1 * m2;
    dd P[9];
    psis(scale2(z, 0.25f), m1, scale2(rz, 4.f), P + 0, false);
    psis(scale2(z, 0.5f), m2, scale2(rz, 2.f), P + 2, false);
    psis(z34, m3, rz * dd_of(F43), P + 4, false);
    psis(z, m4, rz, P + 6, true);
    const dd p1_14 = P[0], p2_14 = P[1], p1_12 = P[2], p2_12 = P[3], p1_34 = P[4], p2_34 = P[5];
    const dd p1 = P[6], p2 = P[7], p3 = P[8];
    constexpr ddc R42(1.0 / 42), R7(1.0 / 7), R28(1.0 / 28), R84(1.0 / 84), R2700(1.0 / 2700), R1350(1.0 / 1350),
        R225(1.0 / 225);
    o[C35_E14] = e1.hi;
    o[C35_E12] = e2.hi;
    o[C35_E34] = e3.hi;
    o[C35_E] = e4.hi;
    o[C35_A21] = scale2(p1_14, 0.25f).hi;
    o[C35_A31] = scale2(p1_14 - scale2(p2_14, 0.5f), 0.25f).hi;
    o[C35_A32] = scale2(p2_14, 0.125f).hi;
    o[C35_A41] = scale2(p1_12 - p2_12, 0.5f).hi;
    o[C35_A43] = scale2(p2_12, 0.5f).hi;
    o[C35_A51] = scale2((p1_34 - scale2(p2_34 * 3.f, 0.25f)) * 3.f, 0.25f).hi;
    o[C35_A52] = scale2(p1_34 * -3.f, 0.125f).hi;
    o[C35_A54] = scale2(p2_34 * 9.f, 0.0625f).hi;
    o[C35_A61] = ((p1 * -77.f + p2 * 59.f) * R42).hi;
    o[C35_A62] = ((p1 * 8.f) * R7).hi;
    o[C35_A63] = ((p1 * 111.f - p2 * 87.f) * R28).hi;
    o[C35_A65] = ((p1 * -47.f + p2 * 143.f) * R84).hi;
    o[C35_A71] = (((p1 * 257.f - p2 * 497.f) + p3 * 270.f) * 7.f * R2700).hi;
    o[C35_A73] = (((p1 * 1097.f - p2 * 467.f) - p3 * 150.f) * R1350).hi;
    o[C35_A74] = (scale2((p1 * -49.f + p2 * 199.f) - p3 * 135.f, 2.f) * R225).hi;
    o[C35_A75] = (((p1 * -313.f + p2 * 883.f) - p3 * 90.f) * R1350).hi;
    o[C35_A76] = (((p1 * 509.f - p2 * 2129.f) + p3 * 1830.f) * R2700).hi;
  } else {
    dd P[5];
    psis(scale2(z, 0.5f), m2, scale2(rz, 2.f), P + 0, false);
    psis(z, m4, rz, P + 2, true);
    const dd p1_12 = P[0], p2_12 = P[1], p1 = P[2], p2 = P[3], p3 = P[4];
    constexpr ddc T23(2.0 / 3.0);
    o[C34_E] = e4.hi;
    o[C34_E2] = e2.hi;
    o[C34_A21] = scale2(p1_12, 0.5f).hi;
    o[C34_A31] = scale2(p1_12 - p2_12, 0.5f).hi;
    o[C34_A32] = scale2(p2_12, 0.5f).hi;
    o[C34_A41] = (p1 - p2).hi;
    o[C34_A43] = p2.hi;
    o[C34_A51] = ((p1 - p2 * 1.5f) + p3 * T23).hi;
    o[C34_A52] = (p2 - p3 * T23).hi;
    o[C34_A54] = (scale2(p2, -0.5f) + p3 * T23).hi;
  }
}

// Stiff modes: below z = -STIFF_Z the coefficients are evaluated in FP32 (expf for the
// exponentials) in a form without cancellation, accurate to a few FP32 ulps.
constexpr float STIFF_Z = 32.f;

// (a psi_1 + b psi_2 + g psi_3) / D at the scale x = 1/r (h psi_k as the coefficient
// formulas use them) with e = e^x.  From psi_1 = h r (e - 1), psi_2 = 2 h r^2 (e - 1) - 2 h r
// and psi_3 = 6 h r^3 (e - 1) - 6 h r^2 - 3 h r:
//   h r [ -(a + 2b + 3g) - (2b + 6g) r - 6g r^2 + e (a + 2b r + 6g r^2) ] / D,
// the integer sums exact, so that the leading terms of the combinations (which cancel in
// the psi form, e.g. psi_1 - psi_2 / 2 ~ r^2) never cancel in FP32; |r| <= 1/8 here.
template <int A, int B, int G, int D>
RK_DEV float stiff_comb(float h, float r, float e) {
  constexpr float k1 = -(float)(A + 2 * B + 3 * G) / (float)D, k2 = -(float)(2 * B + 6 * G) / (float)D;
  constexpr float k3 = -(float)(6 * G) / (float)D;
  constexpr float m0 = (float)A / (float)D, m1 = (float)(2 * B) / (float)D, m2 = (float)(6 * G) / (float)D;
  return (h * r) * ((k1 + r * (k2 + r * k3)) + e * (m0 + r * (m1 + r * m2)));
}

// FP32 coefficients of a stiff real mode (z < -STIFF_Z), layouts C35_* (ETD35, ETD5), C34_*
// (ETD34, ETD4) and CIF_* (IF34): the combinations of etd_from_psi_e (etd35.py:157-288,
// etd34.py:107-149, if34.py:109-112) through stiff_comb.  z = zf + zl
// with zf its FP32 rounding: each exponential e^(c z) = e^(c zf) (1 + c zl) and 1/z =
// (1/zf)(1 - zl/zf) to first order in zl (|zl| <= 2^-24 |z|), so that neither takes the
// rounding of z (an error of |c z| 2^-24 relative in e^(c z)).
template <int METHOD>
RK_DEV void stiff_coeffs_f32(double zd, double hd, float* o) {
  const float zf = (float)zd, zl = (float)(zd - (double)zf), h = (float)hd;
  auto ex = [&](float c) {  // e^(c z) for c = 1/4, 1/2, 1 (c zf exact)
    const float e = expf(c * zf);
    return fmaf(e, c * zl, e);
  };
  if constexpr (METHOD == RK_IF34) {
    o[CIF_E] = ex(1.f);
    o[CIF_E2] = ex(0.5f);
  } else {
    const float e2 = ex(0.5f), e4 = ex(1.f);
    float rz = 1.f / zf;
    rz = fmaf(-(zl * rz), rz, rz);
    if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5) {
      const float e1 = ex(0.25f), e3 = e2 * e1, r14 = 4.f * rz, r12 = 2.f * rz, r34 = rz * (4.f / 3.f);
      o[C35_E14] = e1;
      o[C35_E12] = e2;
      o[C35_E34] = e3;
      o[C35_E] = e4;
      o[C35_A21] = stiff_comb<1, 0, 0, 4>(h, r14, e1);
      o[C35_A31] = stiff_comb<2, -1, 0, 8>(h, r14, e1);
      o[C35_A32] = stiff_comb<0, 1, 0, 8>(h, r14, e1);
      o[C35_A41] = stiff_comb<1, -1, 0, 2>(h, r12, e2);
      o[C35_A43] = stiff_comb<0, 1, 0, 2>(h, r12, e2);
      o[C35_A51] = stiff_comb<12, -9, 0, 16>(h, r34, e3);
      o[C35_A52] = stiff_comb<-3, 0, 0, 8>(h, r34, e3);
      o[C35_A54] = stiff_comb<0, 9, 0, 16>(h, r34, e3);
      o[C35_A61] = stiff_comb<-77, 59, 0, 42>(h, rz, e4);
      o[C35_A62] = stiff_comb<8, 0, 0, 7>(h, rz, e4);
      o[C35_A63] = stiff_comb<111, -87, 0, 28>(h, rz, e4);
      o[C35_A65] = stiff_comb<-47, 143, 0, 84>(h, rz, e4);
      o[C35_A71] = stiff_comb<1799, -3479, 1890, 2700>(h, rz, e4);
      o[C35_A73] = stiff_comb<1097, -467, -150, 1350>(h, rz, e4);
      o[C35_A74] = stiff_comb<-98, 398, -270, 225>(h, rz, e4);
      o[C35_A75] = stiff_comb<-313, 883, -90, 1350>(h, rz, e4);
      o[C35_A76] = stiff_comb<509, -2129, 1830, 2700>(h, rz, e4);
    } else {
      const float r12 = 2.f * rz;
      o[C34_E] = e4;
      o[C34_E2] = e2;
      o[C34_A21] = stiff_comb<1, 0, 0, 2>(h, r12, e2);
      o[C34_A31] = stiff_comb<1, -1, 0, 2>(h, r12, e2);
      o[C34_A32] = stiff_comb<0, 1, 0, 2>(h, r12, e2);
      o[C34_A41] = stiff_comb<1, -1, 0, 1>(h, rz, e4);
      o[C34_A43] = stiff_comb<0, 1, 0, 1>(h, rz, e4);
      o[C34_A51] = stiff_comb<6, -9, 4, 6>(h, rz, e4);
      o[C34_A52] = stiff_comb<0, 3, -2, 3>(h, rz, e4);
      o[C34_A54] = stiff_comb<0, -3, 4, 6>(h, rz, e4);
    }
  }
}

// ---------------------------------------------------------------------------------
// FP32 coefficients of a real mode for -STIFF_Z <= z <= 80 without double-float work.
// Each coefficient h c(x), c = (a psi_1 + b psi_2 + g psi_3)/D at its own scale x = s z
// (s = 1/4, 1/2, 3/4, 1), comes from the combination's Taylor series around the nearest
// of x0 = 0, +-2, ..., +-8 (|x - x0| <= 1, 14 terms, tables k_ser_etd35 / k_ser_etd34
// generated in 60-digit arithmetic by gen_coef_series.py) for |x| < 9, and from the stiff
// form above for |x| >= 9.  The series never cancels, so the result is within ~2 FP32
// ulps of the combination's psi-term scale (|a psi_1| + |b psi_2| + |g psi_3|)/D, i.e. a
// few ulps of the value except where a combination crosses zero; x enters as an FP32
// pair (xf, xl) so that its rounding does not reach the result.
// ---------------------------------------------------------------------------------
struct SerScale {
  bool big;  // |x| >= 9: stiff form
  int k;     // series centre index (0, -2, 2, -4, 4, -6, 6, -8, 8)
  float t;   // x - x0
  float e;   // e^x (stiff form)
  float r;   // 1/x (stiff form)
};

RK_DEV SerScale ser_scale(float xf, float xl) {
  SerScale s;
  s.big = fabsf(xf) >= 9.f;
  if (s.big) {
    const float ef = expf(xf);
    s.e = fmaf(ef, xl, ef);
    const float r = 1.f / xf;
    s.r = fmaf(-(xl * r), r, r);
    s.k = 0;
    s.t = 0.f;
  } else {
    int c = 0;
    if (fabsf(xf) >= 1.f) c = max(-8, min(8, 2 * __float2int_rn(0.5f * xf)));
    s.k = c == 0 ? 0 : (c < 0 ? -c - 1 : c);
    s.t = (xf - (float)c) + xl;  // xf - c is exact (|xf - c| <= 1, same binade or below)
    s.e = 0.f;
    s.r = 0.f;
  }
  return s;
}

// SH: the table is a copy in shared memory (plain loads), else the global one (__ldg)
template <int A, int B, int G, int D, bool SH>
RK_DEV float ser_comb(const float* __restrict__ tab, int row, const SerScale& s, float h) {
  if (s.big) return stiff_comb<A, B, G, D>(h, s.r, s.e);
  const float* p = tab + (row * RK_SER_NC + s.k) * RK_SER_NT;
  float acc = SH ? p[RK_SER_NT - 1] : __ldg(p + RK_SER_NT - 1);
#pragma unroll
  for (int j = RK_SER_NT - 2; j >= 0; --j) acc = fmaf(acc, s.t, SH ? p[j] : __ldg(p + j));
  return h * acc;
}

// layouts C35_* (ETD35, ETD5) and C34_* (ETD34, ETD4); z in [-STIFF_Z, 80].  `tab`: a copy
// of the method's table in shared memory (SH) or null (the global table)
template <int METHOD, bool SH = false>
RK_DEV void series_coeffs_f32(double zd, double hd, float* o, const float* tab = nullptr, float* elo = nullptr) {
  const float zf = (float)zd, zl = (float)(zd - (double)zf), h = (float)hd;
  // The exponentials multiply u in every stage, so an error in them accumulates step after
  // step: they are formed in double-float and rounded once (one dd_exp of the smallest
  // fraction of z, the others as its powers), as the double-float coefficient path does.
  dd m1;
  const dd z2{zf, zl};
  const dd e1 = dd_exp(scale2(z2, (METHOD == RK_ETD35 || METHOD == RK_ETD5) ? 0.25f : 0.5f), m1);
  const SerScale S12 = ser_scale(0.5f * zf, 0.5f * zl), S1 = ser_scale(zf, zl);
  if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD5) {
    const float q34 = 0.75f * zf, l34 = fmaf(0.75f, zf, -q34) + 0.75f * zl;  // 3z/4 as a pair
    const SerScale S14 = ser_scale(0.25f * zf, 0.25f * zl), S34 = ser_scale(q34, l34);
    const float* T = SH ? tab : k_ser_etd35;
    const dd e2 = e1 * e1, e3 = e2 * e1, e4 = e2 * e2;
    o[C35_E14] = e1.hi;
    o[C35_E12] = e2.hi;
    o[C35_E34] = e3.hi;
    o[C35_E] = e4.hi;
    if (elo) *elo = e4.lo;  // the low word of e^z, for the double-float state update
    o[C35_A21] = ser_comb<1, 0, 0, 4, SH>(T, 0, S14, h);
    o[C35_A31] = ser_comb<2, -1, 0, 8, SH>(T, 1, S14, h);
    o[C35_A32] = ser_comb<0, 1, 0, 8, SH>(T, 2, S14, h);
    o[C35_A41] = ser_comb<1, -1, 0, 2, SH>(T, 3, S12, h);
    o[C35_A43] = ser_comb<0, 1, 0, 2, SH>(T, 4, S12, h);
    o[C35_A51] = ser_comb<12, -9, 0, 16, SH>(T, 5, S34, h);
    o[C35_A52] = ser_comb<-3, 0, 0, 8, SH>(T, 6, S34, h);
    o[C35_A54] = ser_comb<0, 9, 0, 16, SH>(T, 7, S34, h);
    o[C35_A61] = ser_comb<-77, 59, 0, 42, SH>(T, 8, S1, h);
    o[C35_A62] = ser_comb<8, 0, 0, 7, SH>(T, 9, S1, h);
    o[C35_A63] = ser_comb<111, -87, 0, 28, SH>(T, 10, S1, h);
    o[C35_A65] = ser_comb<-47, 143, 0, 84, SH>(T, 11, S1, h);
    o[C35_A71] = ser_comb<1799, -3479, 1890, 2700, SH>(T, 12, S1, h);
    o[C35_A73] = ser_comb<1097, -467, -150, 1350, SH>(T, 13, S1, h);
    o[C35_A74] = ser_comb<-98, 398, -270, 225, SH>(T, 14, S1, h);
    o[C35_A75] = ser_comb<-313, 883, -90, 1350, SH>(T, 15, S1, h);
    o[C35_A76] = ser_comb<509, -2129, 1830, 2700, SH>(T, 16, S1, h);
  } else {
    const float* T = SH ? tab : k_ser_etd34;
    o[C34_E] = (e1 * e1).hi;
    o[C34_E2] = e1.hi;
    o[C34_A21] = ser_comb<1, 0, 0, 2, SH>(T, 0, S12, h);
    o[C34_A31] = ser_comb<1, -1, 0, 2, SH>(T, 1, S12, h);
    o[C34_A32] = ser_comb<0, 1, 0, 2, SH>(T, 2, S12, h);
    o[C34_A41] = ser_comb<1, -1, 0, 1, SH>(T, 3, S1, h);
    o[C34_A43] = ser_comb<0, 1, 0, 1, SH>(T, 4, S1, h);
    o[C34_A51] = ser_comb<6, -9, 4, 6, SH>(T, 5, S1, h);
    o[C34_A52] = ser_comb<0, 3, -2, 3, SH>(T, 6, S1, h);
    o[C34_A54] = ser_comb<0, -3, 4, 6, SH>(T, 7, S1, h);
  }
}

}  // namespace rk
