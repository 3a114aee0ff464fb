"""The stiff-mode coefficient forms of the per-instance dense kernel (CPU, no device).

Below z = -32 the kernel evaluates each ETD coefficient (a psi_1 + b psi_2 + g psi_3) / D at
the scale x = c z as

    h r [ -(a + 2b + 3g) - (2b + 6g) r - 6g r^2 + e (a + 2b r + 6g r^2) ] / D,  r = 1/x, e = e^x,

with the integer tuple (a, b, g, D) written into its source.  This test reads those tuples
from the kernel source and checks each line against the oracle's FP64 coefficient formulas
(etd35.py:180-237, etd34.py:107-149): the right scale for r and e on every line, every
a-coefficient covered, and the grouped form equal to the psi form in FP64 (to ~1e-13 |z|
relative, the cancellation the psi form itself carries at large |z|).
"""

import os
import re

import numpy as np
import pytest

from oracle import rk_oracle as O

SRC = os.path.join(os.path.dirname(__file__), "..", "rkstiff_gb300", "csrc", "rk_dd.cuh")
LINE = re.compile(r"o\[(C35|C34)_(\w+)\] = stiff_comb<(-?\d+), (-?\d+), (-?\d+), (\d+)>\(h, (\w+), (\w+)\);")
R_SCALE = {"r14": 0.25, "r12": 0.5, "r34": 0.75, "rz": 1.0}
E_SCALE = {"e1": 0.25, "e2": 0.5, "e3": 0.75, "e4": 1.0}


def stiff_lines():
    with open(SRC) as f:
        text = f.read()
    out = {"C35": {}, "C34": {}}
    for m in LINE.finditer(text):
        fam, name, a, b, g, d, rt, et = m.groups()
        out[fam][name.lower()] = (int(a), int(b), int(g), int(d), rt, et)
    return out


def grouped(a, b, g, d, h, x):
    r = 1.0 / x
    e = np.exp(x)
    return h * r * ((-(a + 2 * b + 3 * g) - (2 * b + 6 * g) * r - 6 * g * r * r) + e * (a + 2 * b * r + 6 * g * r * r)) / d


@pytest.mark.parametrize("method,fam,count", [("ETD35", "C35", 17), ("ETD34", "C34", 8)])
def test_stiff_grouping_matches_psi_formulas(method, fam, count):
    lines = stiff_lines()[fam]
    assert len(lines) == count, sorted(lines)
    h = 0.37
    z = -np.logspace(np.log10(32.0), 5, 200)
    ref = O.diag_coeffs(method, (z / h).astype(np.complex128), h)  # the oracle forms z = h lin
    for name, (a, b, g, d, rt, et) in lines.items():
        assert R_SCALE[rt] == E_SCALE[et], (name, rt, et)
        got = grouped(a, b, g, d, h, R_SCALE[rt] * z)
        want = ref[name].real
        rel = np.abs(got - want) / np.abs(want)
        assert np.all(rel <= 1e-13 * np.maximum(1.0, np.abs(z))), (name, float(rel.max()))
