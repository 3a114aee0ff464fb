"""Generate rk_coef_series.cuh: Taylor tables of the ETD35/ETD34 coefficient combinations.

Each FP32 ETD coefficient of a real mode is h c(x) with x = s z (s = 1/4, 1/2, 3/4 or 1 for
the coefficient's stage fraction) and

    c(x) = (a psi_1(x) + b psi_2(x) + g psi_3(x)) / D,
    psi_1 = (e^x - 1)/x,  psi_2 = 2 (e^x - 1 - x)/x^2,  psi_3 = 6 (e^x - 1 - x - x^2/2)/x^3,

the integers (a, b, g, D) of each combination being those of the methods' coefficient
formulas (ETD35: etd35.py:157-288; ETD34: etd34.py:107-149, as restated in rk_coeffs.cuh).
The combinations cancel (e.g. ETD35 a71 = 7 (257 psi_1 - 497 psi_2 + 270 psi_3)/2700) so
their psi form loses up to ~7 bits in FP32 near x = 0.  Their own Taylor series does not:
around x0 the coefficients c^(j)(x0)/j! are evaluated here in 60-digit arithmetic from the
series of e^x and of 1/x, so a 14-term Horner evaluation in FP32 at |x - x0| <= 1 rounds
to a few FP32 ulps of the combination's scale.  Centres 0, +-2, +-4, +-6, +-8 cover
|x| < 9; beyond, the kernels use the cancellation-free stiff form.

Run: python gen_coef_series.py  (writes rk_coef_series.cuh beside this script; needs mpmath)
"""
import os

import mpmath as mp

mp.mp.dps = 60
NT = 14
CENTERS = (0, -2, 2, -4, 4, -6, 6, -8, 8)

# (name, a, b, g, D); order = the C35_* / C34_* coefficient order after the exponentials
ETD35 = (("A21", 1, 0, 0, 4), ("A31", 2, -1, 0, 8), ("A32", 0, 1, 0, 8), ("A41", 1, -1, 0, 2),
         ("A43", 0, 1, 0, 2), ("A51", 12, -9, 0, 16), ("A52", -3, 0, 0, 8), ("A54", 0, 9, 0, 16),
         ("A61", -77, 59, 0, 42), ("A62", 8, 0, 0, 7), ("A63", 111, -87, 0, 28), ("A65", -47, 143, 0, 84),
         ("A71", 1799, -3479, 1890, 2700), ("A73", 1097, -467, -150, 1350), ("A74", -98, 398, -270, 225),
         ("A75", -313, 883, -90, 1350), ("A76", 509, -2129, 1830, 2700))
ETD34 = (("A21", 1, 0, 0, 2), ("A31", 1, -1, 0, 2), ("A32", 0, 1, 0, 2), ("A41", 1, -1, 0, 1),
         ("A43", 0, 1, 0, 1), ("A51", 6, -9, 4, 6), ("A52", 0, 3, -2, 3), ("A54", 0, -3, 4, 6))


def series(a, b, g, D, x0):
    """c^(j)(x0)/j!, j < NT."""
    N = NT + 8
    if x0 == 0:
        # c(x) = sum_j x^j (a/(j+1)! + 2b/(j+2)! + 6g/(j+3)!) / D
        return [(a / mp.factorial(j + 1) + 2 * b / mp.factorial(j + 2) + 6 * g / mp.factorial(j + 3)) / D
                for j in range(NT)]
    x0 = mp.mpf(x0)
    ex = [mp.e ** x0 / mp.factorial(j) for j in range(N)]           # e^(x0 + t)
    poly = lambda cs: cs + [mp.mpf(0)] * (N - len(cs))

    def mul(p, q):
        return [mp.fsum(p[i] * q[k - i] for i in range(k + 1)) for k in range(N)]
    inv = [(-1) ** j / x0 ** (j + 1) for j in range(N)]                # 1/(x0 + t)
    inv2, inv3 = mul(inv, inv), mul(mul(inv, inv), inv)
    one = poly([mp.mpf(1)])
    xx = poly([x0, mp.mpf(1)])                                          # x0 + t
    xx2 = mul(xx, xx)
    em1 = [ex[k] - one[k] for k in range(N)]
    d2 = [em1[k] - xx[k] for k in range(N)]
    d3 = [d2[k] - xx2[k] / 2 for k in range(N)]
    p1 = mul(em1, inv)
    p2 = [2 * v for v in mul(d2, inv2)]
    p3 = [6 * v for v in mul(d3, inv3)]
    return [(a * p1[j] + b * p2[j] + g * p3[j]) / D for j in range(NT)]


def emit(name, combs):
    rows = []
    for (cname, a, b, g, D) in combs:
        for x0 in CENTERS:
            cs = series(a, b, g, D, x0)
            rows.append("  /* %s x0=%+d */ " % (cname, x0) + ", ".join("%sf" % repr(float(c)) for c in cs))
    return ("static __device__ const float %s[%d] = {\n" % (name, len(combs) * len(CENTERS) * NT)
            + ",\n".join(rows) + "};\n")


def render() -> str:
    return ("// Generated by gen_coef_series.py (Taylor tables of the ETD coefficient combinations,\n"
            "// 60-digit arithmetic); do not edit by hand.\n#pragma once\n\nnamespace rk {\n\n"
            "constexpr int RK_SER_NT = %d;\nconstexpr int RK_SER_NC = %d;  // centres 0, -2, 2, -4, 4, -6, 6, -8, 8\n\n"
            % (NT, len(CENTERS))
            + emit("k_ser_etd35", ETD35) + "\n" + emit("k_ser_etd34", ETD34) + "\n}  // namespace rk\n")


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rk_coef_series.cuh")
    with open(out, "w") as f:
        f.write(render())
    print(out)


if __name__ == "__main__":
    main()
