"""The FP32 Taylor tables of the ETD coefficient combinations (rk_coef_series.cuh): the
committed header is what its generator writes, and an FP32 Horner evaluation of the table
(the kernels' ser_comb, restated with NumPy float32) stays within 3 FP32 ulps of each
combination's psi-term scale against 40-digit values over |x| < 9."""

import os
import re
import sys

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "rkstiff_gb300", "csrc")
sys.path.insert(0, CSRC)
import gen_coef_series as G  # noqa: E402


def _header():
    with open(os.path.join(CSRC, "rk_coef_series.cuh")) as f:
        return f.read()


def test_header_is_generated():
    assert _header() == G.render()


def _table(name, ncomb):
    src = _header()
    body = src[src.index(name):]
    body = re.sub(r"/\*.*?\*/", "", body[body.index("{") + 1: body.index("};")])
    vals = np.array([float(v.strip().rstrip("f")) for v in body.split(",") if v.strip()], dtype=np.float32)
    return vals.reshape(ncomb, len(G.CENTERS), G.NT)


def _ser(tab, row, x):
    f32 = np.float32
    c = 0 if abs(x) < 1 else int(np.clip(2 * np.rint(0.5 * x), -8, 8))
    k = G.CENTERS.index(c)
    t = f32(x - c)
    acc = tab[row, k, G.NT - 1]
    for j in range(G.NT - 2, -1, -1):
        acc = f32(f32(acc * t) + tab[row, k, j])
    return float(acc)


@pytest.mark.parametrize("name,combs", [("k_ser_etd35", G.ETD35), ("k_ser_etd34", G.ETD34)])
def test_fp32_series_accuracy(name, combs):
    mp.mp.dps = 40
    tab = _table(name, len(combs))
    xs = np.concatenate([-np.logspace(-4, np.log10(8.99), 90), np.logspace(-4, np.log10(8.99), 90), [0.0]])
    for row, (cname, a, b, g, D) in enumerate(combs):
        worst = 0.0
        for x in xs:
            xm = mp.mpf(float(x))
            if xm == 0:
                exact, scale = mp.mpf(a + b + g) / D, abs(mp.mpf(a + b + g)) / D
            else:
                e = mp.e ** xm
                p1, p2, p3 = (e - 1) / xm, 2 * (e - 1 - xm) / xm**2, 6 * (e - 1 - xm - xm**2 / 2) / xm**3
                exact = (a * p1 + b * p2 + g * p3) / D
                scale = (abs(a * p1) + abs(b * p2) + abs(g * p3)) / D
            err = abs(_ser(tab, row, float(x)) - float(exact))
            worst = max(worst, err / float(np.spacing(np.float32(float(scale)))))
        assert worst <= 3.0, (name, cname, worst)
