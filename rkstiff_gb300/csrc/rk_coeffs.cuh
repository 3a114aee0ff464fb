// FP64 coefficient sets of the seven methods for one mode of a diagonal operator.
//
// Arithmetic follows the NumPy semantics of the reference: the ETD classes cast the
// operator to complex128 (rkstiff/etd35.py:124), so a division by a real constant is a
// complex division, which NumPy performs as a multiplication by the reciprocal (Smith's
// algorithm with a zero imaginary part).  The IF classes keep the operator's dtype
// (rkstiff/if34.py:71, if45dp.py:204), so a real operator divides exactly there.
// Scalar type S is `double` (real operator) or `cx<double>` (complex operator).
#pragma once

#include "rk_common.cuh"

namespace rk {

// ---- scalar helpers ---------------------------------------------------------------
RK_DEV double sre(double a) { return a; }
RK_DEV double sre(cx<double> a) { return a.x; }
RK_DEV double sabs(double a) { return fabs(a); }
RK_DEV double sabs(cx<double> a) { return hypot(a.x, a.y); }
RK_DEV double sexp(double a) { return exp(a); }
RK_DEV cx<double> sexp(cx<double> a) { return cexp(a); }
// complex-semantics division by a real constant: a * (1/d)
RK_DEV double rdiv(double a, double d) { return a * (1.0 / d); }
RK_DEV cx<double> rdiv(cx<double> a, double d) { double s = 1.0 / d; return cx<double>{a.x * s, a.y * s}; }
// complex-semantics division
RK_DEV double sdiv(double a, double b) { return a * (1.0 / b); }
RK_DEV cx<double> sdiv(cx<double> a, cx<double> b) { return cdiv(a, b); }
RK_DEV double ssub1(double a) { return a - 1.0; }
RK_DEV cx<double> ssub1(cx<double> a) { return cx<double>{a.x - 1.0, a.y}; }
template <class S> RK_DEV S smul(double c, S a) { return c * a; }
RK_DEV cx<double> to_cx(double a) { return cx<double>{a, 0.0}; }
RK_DEV cx<double> to_cx(cx<double> a) { return a; }

// psi_1..3 (rkstiff/etd.py:148,165,182); z**2 = z*z, z**3 = z*(z*z) as NumPy computes them
template <class S> RK_DEV S psi1(S z, S e) { return sdiv(ssub1(e), z); }
template <class S> RK_DEV S psi2(S z, S e) { return sdiv(2.0 * (ssub1(e) - z), z * z); }
template <class S> RK_DEV S psi3(S z, S e) {
  S z2 = z * z;
  return sdiv(6.0 * ((ssub1(e) - z) - rdiv(z2, 2.0)), z * z2);
}

struct EtdCfg {
  double cutoff;
  double R;
  int np;
};

// The contour node r_j = R exp(2 pi i (j + 1/2)/Np) (rkstiff/etd35.py:259).
RK_DEV cx<double> contour_node(const EtdCfg& c, int j) {
  double th = (6.283185307179586 * (j + 0.5)) * (1.0 / c.np);
  double s, co;
  sincos(th, &s, &co);
  return cx<double>{c.R * co, c.R * s};
}

template <class S> RK_DEV S from_d(double v);
template <> RK_DEV double from_d<double>(double v) { return v; }
template <> RK_DEV cx<double> from_d<cx<double>>(double v) { return cx<double>{v, 0.0}; }
RK_DEV cx<double> operator+(cx<double> a, double b) { return cx<double>{a.x + b, a.y}; }

template <class S> RK_DEV S from_cx(cx<double> v);
template <> RK_DEV double from_cx<double>(cx<double> v) { return v.x; }
template <> RK_DEV cx<double> from_cx<cx<double>>(cx<double> v) { return v; }

// ---------------------------------------------------------------------------------
// Coefficient layouts (index of each array inside a method's coefficient block)
// ---------------------------------------------------------------------------------
// ETD35 / ETD5: rkstiff/etd35.py:180-237 (the ETD5 b-weights are a71..a76)
enum { C35_E14, C35_E12, C35_E34, C35_E, C35_A21, C35_A31, C35_A32, C35_A41, C35_A43, C35_A51, C35_A52,
       C35_A54, C35_A61, C35_A62, C35_A63, C35_A65, C35_A71, C35_A73, C35_A74, C35_A75, C35_A76, C35_N };
// ETD34 / ETD4: rkstiff/etd34.py:107-149 (ETD4's b1,b2,b4 are a51,a52,a54)
enum { C34_E, C34_E2, C34_A21, C34_A31, C34_A32, C34_A41, C34_A43, C34_A51, C34_A52, C34_A54, C34_N };
// IF34 / IF4: rkstiff/if34.py:91-93
enum { CIF_E, CIF_E2, CIF_N };
// IF45DP: rkstiff/if45dp.py:205-237 (a76, r6, r7 are scalars and not stored)
enum { CDP_E15, CDP_E310, CDP_E45, CDP_E89, CDP_E, CDP_A21, CDP_A31, CDP_A32, CDP_A41, CDP_A42, CDP_A43,
       CDP_A51, CDP_A52, CDP_A53, CDP_A54, CDP_A61, CDP_A62, CDP_A63, CDP_A64, CDP_A65, CDP_A71, CDP_A73,
       CDP_A74, CDP_A75, CDP_R1, CDP_R3, CDP_R4, CDP_R5, CDP_N };

RK_HD int num_coeffs(int method) {
  switch (method) {
    case RK_ETD35: case RK_ETD5: return C35_N;
    case RK_ETD34: case RK_ETD4: return C34_N;
    case RK_IF34: case RK_IF4: return CIF_N;
    case RK_IF45DP: return CDP_N;
  }
  return 0;
}

// ---- ETD families: psi sets and the coefficients built from them ----------------------
// psi slots of the ETD35/ETD5 family: (order, num/den) pairs in this order
#define RK_PSI35_N 9
RK_HD void psi35_slot(int k, int& order, double& num, double& den) {
  const int o[9] = {1, 2, 1, 2, 1, 2, 1, 2, 3};
  const double nu[9] = {1, 1, 1, 1, 3, 3, 1, 1, 1};
  const double de[9] = {4, 4, 2, 2, 4, 4, 1, 1, 1};
  order = o[k]; num = nu[k]; den = de[k];
}
#define RK_PSI34_N 5
RK_HD void psi34_slot(int k, int& order, double& num, double& den) {
  const int o[5] = {1, 2, 1, 2, 3};
  const double nu[5] = {1, 1, 1, 1, 1};
  const double de[5] = {2, 2, 1, 1, 1};
  order = o[k]; num = nu[k]; den = de[k];
}

// rkstiff/etd35.py:180-183 and 220-237 (the large- and small-mode formulas are the same)
template <class S>
RK_DEV void etd35_from_psi(S z, const S* P, S* o) {
  const S p1_14 = P[0], p2_14 = P[1], p1_12 = P[2], p2_12 = P[3], p1_34 = P[4], p2_34 = P[5];
  const S p1 = P[6], p2 = P[7], p3 = P[8];
  o[C35_E14] = sexp(rdiv(z, 4.0));
  o[C35_E12] = sexp(rdiv(z, 2.0));
  o[C35_E34] = sexp(rdiv(3.0 * z, 4.0));
  o[C35_E] = sexp(z);
  o[C35_A21] = rdiv(p1_14, 4.0);
  o[C35_A31] = rdiv(p1_14 - rdiv(p2_14, 2.0), 4.0);
  o[C35_A32] = rdiv(p2_14, 8.0);
  o[C35_A41] = rdiv(p1_12 - p2_12, 2.0);
  o[C35_A43] = rdiv(p2_12, 2.0);
  o[C35_A51] = rdiv(3.0 * (p1_34 - rdiv(3.0 * p2_34, 4.0)), 4.0);
  o[C35_A52] = rdiv(-3.0 * p1_34, 8.0);
  o[C35_A54] = rdiv(9.0 * p2_34, 16.0);
  o[C35_A61] = rdiv(-77.0 * p1 + 59.0 * p2, 42.0);
  o[C35_A62] = rdiv(8.0 * p1, 7.0);
  o[C35_A63] = rdiv(111.0 * p1 - 87.0 * p2, 28.0);
  o[C35_A65] = rdiv(-47.0 * p1 + 143.0 * p2, 84.0);
  o[C35_A71] = rdiv(7.0 * ((257.0 * p1 - 497.0 * p2) + 270.0 * p3), 2700.0);
  o[C35_A73] = rdiv((1097.0 * p1 - 467.0 * p2) - 150.0 * p3, 1350.0);
  o[C35_A74] = rdiv(2.0 * ((-49.0 * p1 + 199.0 * p2) - 135.0 * p3), 225.0);
  o[C35_A75] = rdiv((-313.0 * p1 + 883.0 * p2) - 90.0 * p3, 1350.0);
  o[C35_A76] = rdiv((509.0 * p1 - 2129.0 * p2) + 1830.0 * p3, 2700.0);
}

// rkstiff/etd34.py:107-126 and 142-149
template <class S>
RK_DEV void etd34_from_psi(S z, const S* P, S* o) {
  const S p1_12 = P[0], p2_12 = P[1], p1 = P[2], p2 = P[3], p3 = P[4];
  o[C34_E] = sexp(z);
  o[C34_E2] = sexp(rdiv(z, 2.0));
  o[C34_A21] = 0.5 * p1_12;
  o[C34_A31] = 0.5 * (p1_12 - p2_12);
  o[C34_A32] = 0.5 * p2_12;
  o[C34_A41] = p1 - p2;
  o[C34_A43] = p2;
  o[C34_A51] = (p1 - 1.5 * p2) + (2.0 / 3) * p3;
  o[C34_A52] = p2 - (2.0 / 3) * p3;
  o[C34_A54] = -0.5 * p2 + (2.0 / 3) * p3;
}

RK_HD bool is_etd(int method) {
  return method == RK_ETD35 || method == RK_ETD5 || method == RK_ETD34 || method == RK_ETD4;
}
RK_HD int num_psi(int method) {
  return (method == RK_ETD35 || method == RK_ETD5) ? RK_PSI35_N : RK_PSI34_N;
}
RK_HD void psi_slot(int method, int k, int& order, double& num, double& den) {
  if (method == RK_ETD35 || method == RK_ETD5) psi35_slot(k, order, num, den);
  else psi34_slot(k, order, num, den);
}

// Direct (|z| >= modecutoff) psi values: h * psi_order(num/den * z).
template <class S>
RK_DEV S direct_hpsi(S z, double h, int order, double num, double den) {
  S arg = (num == 1.0 && den == 1.0) ? z : rdiv(num * z, den);
  S e = sexp(arg);
  S p = order == 1 ? psi1(arg, e) : (order == 2 ? psi2(arg, e) : psi3(arg, e));
  return h * p;
}

// psi_order(num/den * Z) at one contour point Z = z + r_q (the summand of the mean)
RK_DEV cx<double> contour_term_at(cx<double> Z, int order, double num, double den) {
  cx<double> arg = (num == 1.0 && den == 1.0) ? Z : rdiv(num * Z, den);
  cx<double> e = cexp(arg);
  return order == 1 ? psi1(arg, e) : (order == 2 ? psi2(arg, e) : psi3(arg, e));
}

// complex reciprocal 1/a (Smith's algorithm)
RK_DEV cx<double> crecip(cx<double> a) { return cdiv(cx<double>{1.0, 0.0}, a); }

// Adds the psi summands of every slot at contour point Z to acc[] with one complex exp
// (e^{Z/4}; the other scales by products) and one reciprocal per scale (coefficients
// stored in FP32).
RK_DEV void contour_terms_fast(int method, cx<double> Z, cx<double>* acc) {
  auto add = [&](cx<double> x, cx<double> e, cx<double>* out, bool third) {
    const cx<double> r = crecip(x);
    const cx<double> em1 = cx<double>{e.x - 1.0, e.y};
    const cx<double> d = em1 - x;
    const cx<double> r2 = r * r;
    out[0] = out[0] + em1 * r;
    out[1] = out[1] + (2.0 * d) * r2;
    if (third) out[2] = out[2] + (6.0 * (d - 0.5 * (x * x))) * (r2 * r);
  };
  const cx<double> e1 = cexp(0.25 * Z);
  const cx<double> e2 = e1 * e1;
  if (method == RK_ETD35 || method == RK_ETD5) {
    add(0.25 * Z, e1, acc + 0, false);
    add(0.5 * Z, e2, acc + 2, false);
    add(0.25 * (3.0 * Z), e2 * e1, acc + 4, false);
    add(Z, e2 * e2, acc + 6, true);
  } else {
    add(0.5 * Z, e2, acc + 0, false);
    add(Z, e2 * e2, acc + 2, true);
  }
}

// Same coefficients with the exponentials E = {e^{z/4}, e^{z/2}, e^{3z/4}, e^z} given
// (ETD34 uses E[1], E[3]).
template <class S>
RK_DEV void etd_from_psi_e(int method, const S* E, const S* P, S* o) {
  if (method == RK_ETD35 || method == RK_ETD5) {
    const S p1_14 = P[0], p2_14 = P[1], p1_12 = P[2], p2_12 = P[3], p1_34 = P[4], p2_34 = P[5];
    const S p1 = P[6], p2 = P[7], p3 = P[8];
    o[C35_E14] = E[0];
    o[C35_E12] = E[1];
    o[C35_E34] = E[2];
    o[C35_E] = E[3];
    o[C35_A21] = rdiv(p1_14, 4.0);
    o[C35_A31] = rdiv(p1_14 - rdiv(p2_14, 2.0), 4.0);
    o[C35_A32] = rdiv(p2_14, 8.0);
    o[C35_A41] = rdiv(p1_12 - p2_12, 2.0);
    o[C35_A43] = rdiv(p2_12, 2.0);
    o[C35_A51] = rdiv(3.0 * (p1_34 - rdiv(3.0 * p2_34, 4.0)), 4.0);
    o[C35_A52] = rdiv(-3.0 * p1_34, 8.0);
    o[C35_A54] = rdiv(9.0 * p2_34, 16.0);
    o[C35_A61] = rdiv(-77.0 * p1 + 59.0 * p2, 42.0);
    o[C35_A62] = rdiv(8.0 * p1, 7.0);
    o[C35_A63] = rdiv(111.0 * p1 - 87.0 * p2, 28.0);
    o[C35_A65] = rdiv(-47.0 * p1 + 143.0 * p2, 84.0);
    o[C35_A71] = rdiv(7.0 * ((257.0 * p1 - 497.0 * p2) + 270.0 * p3), 2700.0);
    o[C35_A73] = rdiv((1097.0 * p1 - 467.0 * p2) - 150.0 * p3, 1350.0);
    o[C35_A74] = rdiv(2.0 * ((-49.0 * p1 + 199.0 * p2) - 135.0 * p3), 225.0);
    o[C35_A75] = rdiv((-313.0 * p1 + 883.0 * p2) - 90.0 * p3, 1350.0);
    o[C35_A76] = rdiv((509.0 * p1 - 2129.0 * p2) + 1830.0 * p3, 2700.0);
  } else {
    const S p1_12 = P[0], p2_12 = P[1], p1 = P[2], p2 = P[3], p3 = P[4];
    o[C34_E] = E[3];
    o[C34_E2] = E[1];
    o[C34_A21] = 0.5 * p1_12;
    o[C34_A31] = 0.5 * (p1_12 - p2_12);
    o[C34_A32] = 0.5 * p2_12;
    o[C34_A41] = p1 - p2;
    o[C34_A43] = p2;
    o[C34_A51] = (p1 - 1.5 * p2) + (2.0 / 3) * p3;
    o[C34_A52] = p2 - (2.0 / 3) * p3;
    o[C34_A54] = -0.5 * p2 + (2.0 / 3) * p3;
  }
}

// Reduced-cost FP64 psi set of a real mode for coefficients stored in FP32: one exp
// (e^{z/4}; the other scales by products) and one reciprocal of z shared by every psi.
// The results differ from the per-scale formulas by a few FP64 ulps, far below FP32
// resolution.  E receives {e^{z/4}, e^{z/2}, e^{3z/4}, e^z}.
RK_DEV void fast_real_psi(int method, double z, double h, double* E, double* P) {
  const double e1 = exp(0.25 * z);
  const double e2 = e1 * e1;
  E[0] = e1;
  E[1] = e2;
  E[2] = e2 * e1;
  E[3] = e2 * e2;
  const double rz = 1.0 / z;
  auto psis = [&](double x, double e, double r, double* out, bool third) {
    const double em1 = e - 1.0;
    const double d = em1 - x;
    out[0] = h * (em1 * r);
    out[1] = h * ((2.0 * d) * (r * r));
    if (third) out[2] = h * ((6.0 * (d - 0.5 * (x * x))) * (r * (r * r)));
  };
  if (method == RK_ETD35 || method == RK_ETD5) {
    psis(0.25 * z, E[0], 4.0 * rz, P + 0, false);
    psis(0.5 * z, E[1], 2.0 * rz, P + 2, false);
    psis(0.25 * (3.0 * z), E[2], rz * (4.0 / 3.0), P + 4, false);
    psis(z, E[3], rz, P + 6, true);
  } else {
    psis(0.5 * z, E[1], 2.0 * rz, P + 0, false);
    psis(z, E[3], rz, P + 2, true);
  }
}

// psi_1..3 of a small argument by their Taylor series, used for coefficients stored in
// FP32 in place of the contour mean (both evaluate the same functions to FP64 accuracy).
// With S_k(x) = sum_{j>=0} x^j/(j+k)!: psi_1 = S_1, psi_2 = 2 S_2, psi_3 = 6 S_3 and
// S_1 = 1 + x S_2, S_2 = 1/2 + x S_3.  S_3 is summed by Horner's rule through j = 21,
// below FP64 resolution for |x| <= 1 (ETDConfig caps modecutoff at 1).
template <class S>
RK_DEV void taylor_s123(S x, S& s1, S& s2, S& s3) {
  // inverse factorials 1/k! for k = 3..24, from the recurrence (no table of constants)
  double inv[22];
  inv[0] = 1.0 / 6.0;
#pragma unroll
  for (int k = 1; k < 22; ++k) inv[k] = inv[k - 1] / (double)(k + 3);
  S acc = from_d<S>(inv[21]);
#pragma unroll
  for (int k = 20; k >= 0; --k) acc = from_d<S>(inv[k]) + x * acc;
  s3 = acc;
  s2 = from_d<S>(0.5) + x * s3;
  s1 = from_d<S>(1.0) + x * s2;
}

// Small-mode psi set (same slots as the direct evaluation) and the exponentials
// E = {e^{z/4}, e^{z/2}, e^{3z/4}, e^z}.
template <class S>
RK_DEV void taylor_psi(int method, S z, double h, S* E, S* P) {
  E[0] = sexp(rdiv(z, 4.0));
  E[1] = sexp(rdiv(z, 2.0));
  E[2] = sexp(rdiv(3.0 * z, 4.0));
  E[3] = sexp(z);
  auto put = [&](S x, S* out, bool third) {
    S s1, s2, s3;
    taylor_s123(x, s1, s2, s3);
    out[0] = h * s1;
    out[1] = h * (2.0 * s2);
    if (third) out[2] = h * (6.0 * s3);
  };
  if (method == RK_ETD35 || method == RK_ETD5) {
    put(rdiv(z, 4.0), P + 0, false);
    put(rdiv(z, 2.0), P + 2, false);
    put(rdiv(3.0 * z, 4.0), P + 4, false);
    put(z, P + 6, true);
  } else {
    put(rdiv(z, 2.0), P + 0, false);
    put(z, P + 2, true);
  }
}

template <class S>
RK_DEV void etd_from_psi(int method, S z, const S* P, S* o) {
  if (method == RK_ETD35 || method == RK_ETD5) etd35_from_psi(z, P, o);
  else etd34_from_psi(z, P, o);
}

// IF methods keep the operator dtype: a real operator divides exactly (TD = true).
template <bool TD> RK_DEV double idiv(double a, double d) { return TD ? a / d : a * (1.0 / d); }
template <bool TD> RK_DEV cx<double> idiv(cx<double> a, double d) { return rdiv(a, d); }

template <class S, bool TD>
RK_DEV void coeffs_if34(S z, double h, S* o) {
  o[CIF_E] = sexp(z);
  o[CIF_E2] = sexp(idiv<TD>(z, 2.0));
}

template <class S, bool TD>
RK_DEV void coeffs_if45dp(S z, double h, S* o) {
  S E15 = sexp(idiv<TD>(z, 5.0)), E310 = sexp(idiv<TD>(3.0 * z, 10.0)), E45 = sexp(idiv<TD>(4.0 * z, 5.0));
  S E89 = sexp(idiv<TD>(8.0 * z, 9.0)), E = sexp(z), E710 = sexp(idiv<TD>(7.0 * z, 10.0));
  S E19 = sexp(idiv<TD>(z, 9.0));
  o[CDP_E15] = E15; o[CDP_E310] = E310; o[CDP_E45] = E45; o[CDP_E89] = E89; o[CDP_E] = E;
  o[CDP_A21] = idiv<TD>(h * E15, 5.0);
  o[CDP_A31] = idiv<TD>((3.0 * h) * E310, 40.0);
  o[CDP_A32] = idiv<TD>((9.0 * h) * sexp(idiv<TD>(z, 10.0)), 40.0);
  o[CDP_A41] = idiv<TD>((44.0 * h) * E45, 45.0);
  o[CDP_A42] = idiv<TD>((-56.0 * h) * sexp(idiv<TD>(3.0 * z, 5.0)), 15.0);
  o[CDP_A43] = idiv<TD>((32.0 * h) * sexp(idiv<TD>(z, 2.0)), 9.0);
  o[CDP_A51] = idiv<TD>((19372.0 * h) * E89, 6561.0);
  o[CDP_A52] = idiv<TD>((-25360.0 * h) * sexp(idiv<TD>(31.0 * z, 45.0)), 2187.0);
  o[CDP_A53] = idiv<TD>((64448.0 * h) * sexp(idiv<TD>(53.0 * z, 90.0)), 6561.0);
  o[CDP_A54] = idiv<TD>((-212.0 * h) * sexp(idiv<TD>(4.0 * z, 45.0)), 729.0);
  o[CDP_A61] = idiv<TD>((9017.0 * h) * E, 3168.0);
  o[CDP_A62] = idiv<TD>((-355.0 * h) * E45, 33.0);
  o[CDP_A63] = idiv<TD>((46732.0 * h) * E710, 5247.0);
  o[CDP_A64] = idiv<TD>((49.0 * h) * E15, 176.0);
  o[CDP_A65] = idiv<TD>((-5103.0 * h) * E19, 18656.0);
  o[CDP_A71] = idiv<TD>((35.0 * h) * E, 384.0);
  o[CDP_A73] = idiv<TD>((500.0 * h) * E710, 1113.0);
  o[CDP_A74] = idiv<TD>((125.0 * h) * E15, 192.0);
  o[CDP_A75] = idiv<TD>((-2187.0 * h) * E19, 6784.0);
  o[CDP_R1] = idiv<TD>((h * 71.0) * E, 57600.0);
  o[CDP_R3] = idiv<TD>((-71.0 * h) * E710, 16695.0);
  o[CDP_R4] = idiv<TD>((17.0 * h) * E15, 1920.0);
  o[CDP_R5] = idiv<TD>((-17253.0 * h) * E19, 339200.0);
}

// IF45DP scalar weights a76, r6, r7 (rkstiff/if45dp.py:231,236,237)
RK_HD double dp_a76(double h) { return 11.0 * h / 84.0; }
RK_HD double dp_r6(double h) { return 22.0 * h / 525.0; }
RK_HD double dp_r7(double h) { return -h / 40.0; }

// IF-family coefficients for mode z into o[] (no psi functions involved).
template <class S>
RK_DEV void if_coeffs(int method, S z, double h, S* o) {
  if (method == RK_IF45DP) coeffs_if45dp<S, true>(z, h, o);
  else coeffs_if34<S, true>(z, h, o);
}

}  // namespace rk
