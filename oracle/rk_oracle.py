"""NumPy FP64 restatement of rkstiff's time-stepping path (CPU oracle; test infrastructure).

Every function names the reference lines it follows (paths are relative to the
whalenpt/rkstiff project root).  The restatement is organised differently from the
reference -- coefficient sets are dictionaries, the stage programs are plain functions
parameterised by a ``mul`` (elementwise product for a diagonal operator, matrix product
for a dense one) -- but it performs the same arithmetic in the same order wherever the
order changes FP64 results.

Parity pin: ``tests/test_oracle_golden.py`` checks this module against vectors written by
the reference itself (``tests/golden/make_golden.py``).
"""

from __future__ import annotations

import math
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import scipy.linalg

Array = np.ndarray

ADAPTIVE_METHODS = ("IF34", "ETD35", "ETD34", "IF45DP")
CONSTANT_METHODS = ("ETD4", "ETD5", "IF4")
METHODS = ADAPTIVE_METHODS + CONSTANT_METHODS

# solveras.py:255-257
MAX_LOOPS = 50
MAX_S = 4.0
MIN_S = 0.25


class MaxLoopsExceeded(RuntimeError):
    """solveras.py:249 -- too many retries inside one adaptive step."""


class MinimumStepReached(RuntimeError):
    """solveras.py:252 -- the step size fell below ``minh``."""


class SolverConfig:
    """Adaptive controller settings with the reference defaults (solveras.py:71-94)."""

    def __init__(self, epsilon=1e-4, incr_f=1.25, decr_f=0.85, safety_f=0.8, adapt_cutoff=0.01, minh=1e-16):
        self.epsilon = float(epsilon)
        self.incr_f = float(incr_f)
        self.decr_f = float(decr_f)
        self.safety_f = float(safety_f)
        self.adapt_cutoff = float(adapt_cutoff)
        self.minh = float(minh)


class ETDConfig:
    """psi-function evaluation settings with the reference defaults (etd.py:81-87)."""

    def __init__(self, modecutoff=0.01, contour_points=32, contour_radius=1.0):
        self.modecutoff = modecutoff
        self.contour_points = contour_points
        self.contour_radius = contour_radius


# ----------------------------------------------------------------------------------
# psi functions (etd.py:134-182)
# ----------------------------------------------------------------------------------
def psi1(z):
    """(e^z - 1)/z, etd.py:148."""
    return (np.exp(z) - 1) / z


def psi2(z):
    """2 (e^z - 1 - z)/z^2, etd.py:165."""
    return 2 * (np.exp(z) - 1 - z) / z**2


def psi3(z):
    """6 (e^z - 1 - z - z^2/2)/z^3, etd.py:182."""
    return 6 * (np.exp(z) - 1 - z - z**2 / 2) / z**3


_PSI = {1: psi1, 2: psi2, 3: psi3}


def _contour_nodes(cfg: ETDConfig) -> Array:
    """R exp(2 pi i (j + 1/2)/Np), etd35.py:259 / etd4.py:120-122."""
    npts = cfg.contour_points
    return cfg.contour_radius * np.exp(2j * np.pi * np.arange(0.5, npts) / npts)


def _h_psi(z: Array, h: float, cfg: ETDConfig, order: int, num: int, den: int) -> Array:
    """h * psi_order(num/den * z), direct for |z| >= modecutoff, contour mean below.

    Direct branch: etd35.py:212-215 (h * psi(zb/4) etc.).  Contour branch: the mean of
    psi over ``Z = z + r_j`` scaled by the same factor, etd35.py:257-264 and
    etd4.py:119-130.  The mask is taken on the unscaled z (etd35.py:185).
    """
    fn = _PSI[order]
    out = np.zeros(z.shape, dtype=np.complex128)
    small = np.abs(z) < cfg.modecutoff
    big = ~small
    if np.any(big):
        zb = z[big]
        arg = zb if (num == 1 and den == 1) else (num * zb / den)
        out[big] = h * fn(arg)
    if np.any(small):
        r = _contour_nodes(cfg)
        rr, zz = np.meshgrid(r, z[small])
        Z = zz + rr
        arg = Z if (num == 1 and den == 1) else (num * Z / den)
        out[small] = h * np.sum(fn(arg), axis=1) / cfg.contour_points
    return out


# ----------------------------------------------------------------------------------
# Coefficient sets for diagonal operators
# ----------------------------------------------------------------------------------
def _coeffs_etd35_family(z: Array, h: float, cfg: ETDConfig) -> Dict[str, Array]:
    """ETD35 / ETD5 coefficients, etd35.py:180-237 (identical formulas in etd5.py:131-203)."""
    p1_14 = _h_psi(z, h, cfg, 1, 1, 4)
    p2_14 = _h_psi(z, h, cfg, 2, 1, 4)
    p1_12 = _h_psi(z, h, cfg, 1, 1, 2)
    p2_12 = _h_psi(z, h, cfg, 2, 1, 2)
    p1_34 = _h_psi(z, h, cfg, 1, 3, 4)
    p2_34 = _h_psi(z, h, cfg, 2, 3, 4)
    p1 = _h_psi(z, h, cfg, 1, 1, 1)
    p2 = _h_psi(z, h, cfg, 2, 1, 1)
    p3 = _h_psi(z, h, cfg, 3, 1, 1)
    c = {
        "E14": np.exp(z / 4.0),
        "E12": np.exp(z / 2.0),
        "E34": np.exp(3.0 * z / 4.0),
        "E": np.exp(z),
        "a21": p1_14 / 4.0,
        "a31": (p1_14 - p2_14 / 2.0) / 4.0,
        "a32": p2_14 / 8.0,
        "a41": (p1_12 - p2_12) / 2.0,
        "a43": p2_12 / 2.0,
        "a51": 3.0 * (p1_34 - 3.0 * p2_34 / 4.0) / 4.0,
        "a52": -3 * p1_34 / 8.0,
        "a54": 9 * p2_34 / 16.0,
        "a61": (-77 * p1 + 59 * p2) / 42.0,
        "a62": 8 * p1 / 7.0,
        "a63": (111 * p1 - 87 * p2) / 28.0,
        "a65": (-47 * p1 + 143 * p2) / 84.0,
        "a71": 7 * (257 * p1 - 497 * p2 + 270 * p3) / 2700,
        "a73": (1097 * p1 - 467 * p2 - 150 * p3) / 1350,
        "a74": 2 * (-49 * p1 + 199 * p2 - 135 * p3) / 225,
        "a75": (-313 * p1 + 883 * p2 - 90 * p3) / 1350,
        "a76": (509 * p1 - 2129 * p2 + 1830 * p3) / 2700,
    }
    return c


def _coeffs_etd34_family(z: Array, h: float, cfg: ETDConfig) -> Dict[str, Array]:
    """ETD34 / ETD4 coefficients, etd34.py:107-149 (same formulas as etd4.py:97-139)."""
    p1_12 = _h_psi(z, h, cfg, 1, 1, 2)
    p2_12 = _h_psi(z, h, cfg, 2, 1, 2)
    p1 = _h_psi(z, h, cfg, 1, 1, 1)
    p2 = _h_psi(z, h, cfg, 2, 1, 1)
    p3 = _h_psi(z, h, cfg, 3, 1, 1)
    return {
        "E": np.exp(z),
        "E2": np.exp(z / 2),
        "a21": 0.5 * p1_12,
        "a31": 0.5 * (p1_12 - p2_12),
        "a32": 0.5 * p2_12,
        "a41": p1 - p2,
        "a43": p2,
        "a51": p1 - (3.0 / 2) * p2 + (2.0 / 3) * p3,
        "a52": p2 - (2.0 / 3) * p3,
        "a54": -(1.0 / 2) * p2 + (2.0 / 3) * p3,
    }


def _coeffs_if34_family(z: Array, h: float, cfg: Optional[ETDConfig]) -> Dict[str, Array]:
    """IF34 / IF4 exponentials, if34.py:91-93 and if4.py:81-83."""
    return {"E": np.exp(z), "E2": np.exp(z / 2)}


def _coeffs_if45dp(z: Array, h: float, cfg: Optional[ETDConfig]) -> Dict[str, Array]:
    """IF45DP Dormand-Prince integrating-factor weights, if45dp.py:204-237."""
    E15 = np.exp(z / 5)
    E310 = np.exp(3 * z / 10)
    E45 = np.exp(4 * z / 5)
    E89 = np.exp(8 * z / 9)
    E = np.exp(z)
    E710 = np.exp(7 * z / 10)
    E19 = np.exp(z / 9)
    return {
        "E15": E15, "E310": E310, "E45": E45, "E89": E89, "E": E,
        "a21": h * E15 / 5.0,
        "a31": 3 * h * E310 / 40.0,
        "a32": 9 * h * np.exp(z / 10) / 40.0,
        "a41": 44 * h * E45 / 45.0,
        "a42": -56 * h * np.exp(3 * z / 5) / 15.0,
        "a43": 32 * h * np.exp(z / 2) / 9.0,
        "a51": 19372 * h * E89 / 6561.0,
        "a52": -25360 * h * np.exp(31 * z / 45) / 2187.0,
        "a53": 64448.0 * h * np.exp(53 * z / 90) / 6561.0,
        "a54": -212 * h * np.exp(4 * z / 45) / 729.0,
        "a61": 9017 * h * E / 3168.0,
        "a62": -355 * h * E45 / 33.0,
        "a63": 46732 * h * E710 / 5247.0,
        "a64": 49 * h * E15 / 176.0,
        "a65": -5103 * h * E19 / 18656.0,
        "a71": 35 * h * E / 384.0,
        "a73": 500 * h * E710 / 1113.0,
        "a75": -2187 * h * E19 / 6784.0,
        "a74": 125 * h * E15 / 192.0,
        "a76": 11 * h / 84.0,
        "r1": h * 71 * E / 57600.0,
        "r3": -71 * h * E710 / 16695.0,
        "r4": 17 * h * E15 / 1920.0,
        "r5": -17253 * h * E19 / 339200.0,
        "r6": 22 * h / 525.0,
        "r7": -h / 40.0,
    }


_COEFF_FN = {
    "ETD35": _coeffs_etd35_family,
    "ETD5": _coeffs_etd35_family,
    "ETD34": _coeffs_etd34_family,
    "ETD4": _coeffs_etd34_family,
    "IF34": _coeffs_if34_family,
    "IF4": _coeffs_if34_family,
    "IF45DP": _coeffs_if45dp,
}

_IS_ETD = {"ETD35": True, "ETD5": True, "ETD34": True, "ETD4": True, "IF34": False, "IF4": False, "IF45DP": False}


def diag_coeffs(method: str, lin_op: Array, h: float, cfg: Optional[ETDConfig] = None) -> Dict[str, Array]:
    """Coefficient set of ``method`` for a diagonal operator at step ``h``.

    ETD classes cast the operator to complex128 before forming z = h L (etd35.py:124,
    etd34.py:63, etd4.py:76, etd5.py:89); the IF classes keep its dtype (if34.py:71,
    if4.py:64, if45dp.py:204).
    """
    cfg = cfg or ETDConfig()
    lin = lin_op.astype(np.complex128, copy=False) if _IS_ETD[method] else lin_op
    z = h * lin
    return _COEFF_FN[method](z, h, cfg)


# ----------------------------------------------------------------------------------
# Dense coefficient sets (non-diagonal operators)
# ----------------------------------------------------------------------------------
def _dense_contour_psis(z: Array, cfg: ETDConfig, scales: Tuple[Tuple[int, int], ...], orders) -> Dict:
    """Matrix psi via the contour mean sum_j r_j psi_k(r_j) (r_j I - s Z)^{-1} / Np.

    etd35.py:619-640 (and etd34.py:369-383): the Cauchy integral centred at 0 with
    radius R, one resolvent per node and scale.
    """
    n = z.shape[0]
    out = {}
    for (num, den) in scales:
        for k in orders[(num, den)]:
            out[(k, num, den)] = np.zeros((n, n), dtype=np.complex128)
    for point in _contour_nodes(cfg):
        for (num, den) in scales:
            zs = z if (num == 1 and den == 1) else (num * z / den)
            Q = np.linalg.inv(point * np.eye(n) - zs)
            for k in orders[(num, den)]:
                out[(k, num, den)] += point * _PSI[k](point) * Q / cfg.contour_points
    return out


def dense_coeffs_eig(method: str, lin_op: Array, h: float, cfg: Optional[ETDConfig] = None) -> Dict[str, Array]:
    """The coefficient matrices of a non-diagonal solver formed through the eigenbasis,
    M = S diag(c(h lambda)) S^-1 with the diagonal coefficient functions c (diag_coeffs);
    real when lin_op and its spectrum are real.  Same matrices as dense_coeffs (etd35.py:
    602-658) wherever the reference's contour mean converges, which it does not for
    eigenvalues of h lin_op far outside the contour radius; the dense tensor-core path forms
    its matrices this way."""
    w, S = np.linalg.eig(lin_op)
    Sinv = np.linalg.inv(S)
    C = diag_coeffs(method, w, h, cfg)
    real = not np.iscomplexobj(lin_op) and np.max(np.abs(np.imag(w))) == 0.0
    out = {}
    for k, c in C.items():
        M = (S * c[None, :]) @ Sinv
        out[k] = M.real if real else M
    return out


def dense_coeffs(method: str, lin_op: Array, h: float, cfg: Optional[ETDConfig] = None) -> Dict[str, Array]:
    """Coefficient matrices of a non-diagonal solver (etd35.py:602-658, etd34.py:356-392,
    if34.py:225-229, etd4.py:235-271, if4.py:152-164)."""
    cfg = cfg or ETDConfig()
    if method in ("IF34", "IF4"):
        z = h * lin_op
        return {"E": scipy.linalg.expm(z), "E2": scipy.linalg.expm(z / 2)}
    z = h * lin_op.astype(np.complex128, copy=False)
    if method in ("ETD35", "ETD5"):
        P = _dense_contour_psis(
            z, cfg, ((1, 4), (1, 2), (3, 4), (1, 1)),
            {(1, 4): (1, 2), (1, 2): (1, 2), (3, 4): (1, 2), (1, 1): (1, 2, 3)},
        )
        p1_14, p2_14 = P[(1, 1, 4)], P[(2, 1, 4)]
        p1_12, p2_12 = P[(1, 1, 2)], P[(2, 1, 2)]
        p1_34, p2_34 = P[(1, 3, 4)], P[(2, 3, 4)]
        p1, p2, p3 = P[(1, 1, 1)], P[(2, 1, 1)], P[(3, 1, 1)]
        return {
            "E14": scipy.linalg.expm(z / 4.0),
            "E12": scipy.linalg.expm(z / 2.0),
            "E34": scipy.linalg.expm(3.0 * z / 4.0),
            "E": scipy.linalg.expm(z),
            "a21": h * p1_14 / 4.0,
            "a31": h * (p1_14 - p2_14 / 2.0) / 4.0,
            "a32": h * p2_14 / 8.0,
            "a41": h * (p1_12 - p2_12) / 2.0,
            "a43": h * p2_12 / 2.0,
            "a51": h * 3.0 * (p1_34 - 3.0 * p2_34 / 4.0) / 4.0,
            "a52": -3 * h * p1_34 / 8.0,
            "a54": h * 9 * p2_34 / 16.0,
            "a61": h * (-77 * p1 + 59 * p2) / 42.0,
            "a62": h * 8 * p1 / 7.0,
            "a63": h * (111 * p1 - 87 * p2) / 28.0,
            "a65": h * (-47 * p1 + 143 * p2) / 84.0,
            "a71": h * 7 * (257 * p1 - 497 * p2 + 270 * p3) / 2700,
            "a73": h * (1097 * p1 - 467 * p2 - 150 * p3) / 1350,
            "a74": h * 2 * (-49 * p1 + 199 * p2 - 135 * p3) / 225,
            "a75": h * (-313 * p1 + 883 * p2 - 90 * p3) / 1350,
            "a76": h * (509 * p1 - 2129 * p2 + 1830 * p3) / 2700,
        }
    if method in ("ETD34", "ETD4"):
        P = _dense_contour_psis(z, cfg, ((1, 1), (1, 2)), {(1, 1): (1, 2, 3), (1, 2): (1, 2)})
        p1_12, p2_12 = P[(1, 1, 2)], P[(2, 1, 2)]
        p1, p2, p3 = P[(1, 1, 1)], P[(2, 1, 1)], P[(3, 1, 1)]
        return {
            "E": scipy.linalg.expm(z),
            "E2": scipy.linalg.expm(z / 2),
            "a21": 0.5 * h * p1_12,
            "a31": 0.5 * h * (p1_12 - p2_12),
            "a32": 0.5 * h * p2_12,
            "a41": h * (p1 - p2),
            "a43": h * p2,
            "a51": h * (p1 - (3.0 / 2) * p2 + (2.0 / 3) * p3),
            "a52": h * (p2 - (2.0 / 3) * p3),
            "a54": h * (-(1.0 / 2) * p2 + (2.0 / 3) * p3),
        }
    raise ValueError(f"no dense form for {method}")


# ----------------------------------------------------------------------------------
# Stage programs.  ``mul(c, v)`` is c*v (diagonal) or c.dot(v) (dense); ``N`` is the
# nonlinear map in the working basis.  Each returns (unew, err, N_last) where N_last is
# the last stage's nonlinear value (FSAL carry) or None.
# ----------------------------------------------------------------------------------
def _stages_etd35(u, N1, C, N, mul):
    """etd35.py:320-345 (diagonal) / etd35.py:690-719 (dense)."""
    k = mul(C["E14"], u) + mul(C["a21"], N1)
    N2 = N(k)
    k = mul(C["E14"], u) + mul(C["a31"], N1) + mul(C["a32"], N2)
    N3 = N(k)
    k = mul(C["E12"], u) + mul(C["a41"], N1) + mul(C["a43"], N3)
    N4 = N(k)
    k = mul(C["E34"], u) + mul(C["a51"], N1) + mul(C["a52"], N2 - N3) + mul(C["a54"], N4)
    N5 = N(k)
    k = mul(C["E"], u) + mul(C["a61"], N1) + mul(C["a62"], N2 - 3 * N4 / 2.0) + mul(C["a63"], N3) + mul(C["a65"], N5)
    N6 = N(k)
    k = (
        mul(C["E"], u) + mul(C["a71"], N1) + mul(C["a73"], N3) + mul(C["a74"], N4)
        + mul(C["a75"], N5) + mul(C["a76"], N6)
    )
    err = mul(C["a75"], -N1 + 4 * N3 - 6 * N4 + 4 * N5 - N6)
    return k, err, None


def _stages_etd34(u, N1, C, N, mul):
    """etd34.py:182-190 (diagonal) / etd34.py:425-435 (dense)."""
    k = mul(C["E2"], u) + mul(C["a21"], N1)
    N2 = N(k)
    k = mul(C["E2"], u) + mul(C["a31"], N1) + mul(C["a32"], N2)
    N3 = N(k)
    k = mul(C["E"], u) + mul(C["a41"], N1) + mul(C["a43"], N3)
    N4 = N(k)
    k = mul(C["E"], u) + mul(C["a51"], N1) + mul(C["a52"], N2 + N3) + mul(C["a54"], N4)
    N5 = N(k)
    err = mul(C["a54"], N4 - N5)
    return k, err, N5


def _stages_if34(u, N1, C, N, mul, h):
    """if34.py:120-130 (diagonal) / if34.py:240-253 (dense)."""
    if mul is _dmul:
        k = C["E2"] * u + h * C["E2"] * N1 / 2.0
        N2 = N(k)
        k = C["E2"] * u + h * N2 / 2.0
        N3 = N(k)
        k = C["E"] * u + h * C["E2"] * N3
        N4 = N(k)
        k = C["E"] * u + h * (C["E"] * N1 / 6.0 + C["E2"] * N2 / 3.0 + C["E2"] * N3 / 3.0 + N4 / 6.0)
    else:
        k = C["E2"].dot(u) + h * C["E2"].dot(N1 / 2.0)
        N2 = N(k)
        k = C["E2"].dot(u) + h * N2 / 2.0
        N3 = N(k)
        k = C["E"].dot(u) + h * C["E2"].dot(N3)
        N4 = N(k)
        k = C["E"].dot(u) + h * (C["E"].dot(N1 / 6.0) + C["E2"].dot(N2 / 3.0) + C["E2"].dot(N3 / 3.0) + N4 / 6.0)
    N5 = N(k)
    err = h * (N4 - N5) / 6.0
    return k, err, N5


def _stages_if45dp(u, N1, C, N, mul):
    """if45dp.py:140-179 (diagonal only)."""
    k = C["E15"] * u + C["a21"] * N1
    N2 = N(k)
    k = C["E310"] * u + C["a31"] * N1 + C["a32"] * N2
    N3 = N(k)
    k = C["E45"] * u + C["a41"] * N1 + C["a42"] * N2 + C["a43"] * N3
    N4 = N(k)
    k = C["E89"] * u + C["a51"] * N1 + C["a52"] * N2 + C["a53"] * N3 + C["a54"] * N4
    N5 = N(k)
    k = C["E"] * u + C["a61"] * N1 + C["a62"] * N2 + C["a63"] * N3 + C["a64"] * N4 + C["a65"] * N5
    N6 = N(k)
    k = C["E"] * u + C["a71"] * N1 + C["a73"] * N3 + C["a74"] * N4 + C["a75"] * N5 + C["a76"] * N6
    N7 = N(k)
    err = C["r1"] * N1 + C["r3"] * N3 + C["r4"] * N4 + C["r5"] * N5 + C["r6"] * N6 + C["r7"] * N7
    return k, err, N7


def _stages_etd4(u, N1, C, N, mul):
    """etd4.py:167-174 (diagonal) / etd4.py:298-307 (dense); FSAL N1 <- N(unew)."""
    k = mul(C["E2"], u) + mul(C["a21"], N1)
    N2 = N(k)
    k = mul(C["E2"], u) + mul(C["a31"], N1) + mul(C["a32"], N2)
    N3 = N(k)
    k = mul(C["E"], u) + mul(C["a41"], N1) + mul(C["a43"], N3)
    N4 = N(k)
    k = mul(C["E"], u) + mul(C["a51"], N1) + mul(C["a52"], N2 + N3) + mul(C["a54"], N4)
    return k, None, N(k)


def _stages_etd5(u, N1, C, N, mul):
    """etd5.py:236-260; the b-weights are the ETD35 a7j coefficients."""
    k = mul(C["E14"], u) + mul(C["a21"], N1)
    N2 = N(k)
    k = mul(C["E14"], u) + mul(C["a31"], N1) + mul(C["a32"], N2)
    N3 = N(k)
    k = mul(C["E12"], u) + mul(C["a41"], N1) + mul(C["a43"], N3)
    N4 = N(k)
    k = mul(C["E34"], u) + mul(C["a51"], N1) + mul(C["a52"], N2 - N3) + mul(C["a54"], N4)
    N5 = N(k)
    k = mul(C["E"], u) + mul(C["a61"], N1) + mul(C["a62"], N2 - 3 * N4 / 2.0) + mul(C["a63"], N3) + mul(C["a65"], N5)
    N6 = N(k)
    k = (
        mul(C["E"], u) + mul(C["a71"], N1) + mul(C["a73"], N3) + mul(C["a74"], N4)
        + mul(C["a75"], N5) + mul(C["a76"], N6)
    )
    return k, None, N(k)


def _stages_if4(u, N1, C, N, mul, h):
    """if4.py:112-121 (diagonal) / if4.py:186-198 (dense)."""
    k, _, Nl = _stages_if34(u, N1, C, N, mul, h)
    return k, None, Nl


def _dmul(c, v):
    return c * v


def _mmul(c, v):
    return c.dot(v)


# method order used by the adaptive controller, solveras.py:454 via _q()
Q_ORDER = {"IF34": 4, "ETD35": 4, "ETD34": 4, "IF45DP": 5}


# ----------------------------------------------------------------------------------
# Controller (solveras.py:412-554)
# ----------------------------------------------------------------------------------
def compute_s(u: Array, err: Array, cfg: SolverConfig, q: int) -> float:
    """solveras.py:451-455: masked L2 norms, s = safety (eps |u| / |err|)^(1/q)."""
    magu = np.abs(u)
    with np.errstate(divide="ignore", invalid="ignore"):
        idx = magu / magu.max() > cfg.adapt_cutoff
        tol = cfg.epsilon * np.linalg.norm(u[idx])
        s = cfg.safety_f * np.power(tol / np.linalg.norm(err[idx]), 1.0 / q)
    return float(s)


def reject_step_size(s: float, h: float, cfg: SolverConfig) -> float:
    """solveras.py:492-506."""
    if math.isinf(s) or math.isnan(s):
        return MIN_S * h
    s = max(s, MIN_S)
    s = min(s, cfg.decr_f)
    return s * h


def accept_step_size(s: float, h: float, cfg: SolverConfig) -> float:
    """solveras.py:543-554."""
    s = min(s, MAX_S)
    if s > cfg.incr_f:
        return s * h
    return h


# ----------------------------------------------------------------------------------
# Solver driver
# ----------------------------------------------------------------------------------
class OracleSolver:
    """One rkstiff solver object restated: method + operator + nonlinear map + state.

    ``diagonalize`` selects the eigenbasis form (etd35.py:348-495, etd34.py:194-304,
    if34.py:137-196) for a 2-D operator; otherwise a 2-D operator uses the dense form, whose
    coefficient matrices come from the reference's contour mean (``dense_psi="contour"``) or
    from the eigenbasis (``dense_psi="eig"``, see dense_coeffs_eig).
    ``log`` collects one record per attempt: (t, h, s, accepted).
    """

    def __init__(self, method: str, lin_op: Array, nl_func: Callable[[Array], Array],
                 config: Optional[SolverConfig] = None, etd_config: Optional[ETDConfig] = None,
                 diagonalize: bool = False, dense_psi: str = "contour"):
        if method not in METHODS:
            raise ValueError(method)
        if dense_psi not in ("contour", "eig"):
            raise ValueError(dense_psi)
        self.dense_psi = dense_psi
        self.method = method
        self.lin_op = lin_op
        self.nl_func = nl_func
        self.config = config or SolverConfig()
        self.etd_config = etd_config or ETDConfig()
        self.diag = lin_op.ndim == 1
        # only ETD35, ETD34 and IF34 have an eigenbasis form (etd35.py:826, etd34.py:551, if34.py:302)
        self.diagonalize = bool(diagonalize) and not self.diag and method in ("ETD35", "ETD34", "IF34")
        if method == "IF45DP" and not self.diag:
            raise ValueError("IF45DP only handles 1D linear operators")  # if45dp.py:69-70
        if self.diagonalize:
            self._eig, self._S = np.linalg.eig(lin_op)
            self._Sinv = np.linalg.inv(self._S)
        self.t: List[float] = []
        self.u: List[Array] = []
        self.log: List[Tuple[float, float, float, bool]] = []
        self.nl_evals = 0
        self.attempts = 0
        self.coeff_updates = 0
        self.reset()

    # -- state -------------------------------------------------------------------
    def reset(self):
        """solveras.py:306-312 / solvercs.py:125-130 plus the per-class _reset."""
        self.t, self.u = [], []
        self._accept = False
        self._h_coeff = None
        self._n1 = None
        self._v = None
        self._tc = 0.0

    @property
    def adaptive(self) -> bool:
        return self.method in ADAPTIVE_METHODS

    def _N(self, v):
        self.nl_evals += 1
        return self.nl_func(v)

    def _coeffs(self, h):
        if h == self._h_coeff:  # exact compare, etd35.py:851
            return
        self._h_coeff = h
        self.coeff_updates += 1
        if self.diag:
            self._C = diag_coeffs(self.method, self.lin_op, h, self.etd_config)
        elif self.diagonalize:
            self._C = diag_coeffs(self.method, self._eig, h, self.etd_config)
        elif self.dense_psi == "eig":
            self._C = dense_coeffs_eig(self.method, self.lin_op, h, self.etd_config)
        else:
            self._C = dense_coeffs(self.method, self.lin_op, h, self.etd_config)

    def _update_stages(self, u, h):
        """One attempt: coefficients on h change, N1 bookkeeping, the stage program."""
        self._coeffs(h)
        self.attempts += 1
        m = self.method
        if self.diagonalize:
            S, Sinv = self._S, self._Sinv

            def Nb(k):
                return Sinv.dot(self._N(S.dot(k)))

            def first(x):
                self._v = Sinv.dot(x)
                return Sinv.dot(self._N(x))
            mul = _dmul
        else:
            Nb = self._N

            def first(x):
                return self._N(x)
            mul = _dmul if self.diag else _mmul

        # N1 bookkeeping: etd35.py:874-878 + 317-318 (recompute on accept);
        # if34.py:330-334 + 117-118 and etd34.py:605-609 + 179-180 (FSAL copy);
        # if45dp.py:134-138; etd4.py:418-422, etd5.py, if4.py:271-275 (N1 set at step end).
        if m == "ETD35":
            if self._n1 is None:
                self._n1 = first(u)
            elif self._accept:
                self._n1 = first(u)
        else:
            if self._n1 is None:
                self._n1 = first(u)
            elif self._accept and m in ("IF34", "ETD34", "IF45DP"):
                self._n1 = self._carry
                if self.diagonalize:
                    self._v = Sinv.dot(u)
        base = self._v if self.diagonalize else u
        C = self._C
        if m == "ETD35":
            k, err, carry = _stages_etd35(base, self._n1, C, Nb, mul)
        elif m == "ETD34":
            k, err, carry = _stages_etd34(base, self._n1, C, Nb, mul)
        elif m == "IF34":
            k, err, carry = _stages_if34(base, self._n1, C, Nb, mul, h)
        elif m == "IF45DP":
            k, err, carry = _stages_if45dp(base, self._n1, C, Nb, mul)
        elif m == "ETD4":
            k, err, carry = _stages_etd4(base, self._n1, C, Nb, mul)
        elif m == "ETD5":
            k, err, carry = _stages_etd5(base, self._n1, C, Nb, mul)
        else:
            k, err, carry = _stages_if4(base, self._n1, C, Nb, mul, h)
        if m in CONSTANT_METHODS:
            self._n1 = carry  # FSAL at the end of every constant step
        else:
            self._carry = carry
        unew = S.dot(k) if self.diagonalize else k
        return unew, err

    # -- adaptive ------------------------------------------------------------------
    def step(self, u: Array, h_suggest: float):
        """solveras.py:379-410 (adaptive) or solvercs.py:184-186 (constant)."""
        if not self.adaptive:
            assert h_suggest >= 0.0
            unew, _ = self._update_stages(u, h_suggest)
            return unew
        h = h_suggest
        assert h >= 0.0
        numloops = 0
        q = Q_ORDER[self.method]
        while True:
            unew, err = self._update_stages(u, h)
            s = compute_s(unew, err, self.config, q)
            if math.isinf(s) or math.isnan(s) or s < 1.0:
                self.log.append((self._tc, h, s, False))
                self._accept = False
                h = reject_step_size(s, h, self.config)
            else:
                self.log.append((self._tc, h, s, True))
                self._accept = True
                return unew, h, accept_step_size(s, h, self.config)
            numloops += 1
            if numloops > MAX_LOOPS:
                raise MaxLoopsExceeded("adaptive step made too many attempts")
            if h < self.config.minh:
                raise MinimumStepReached("adaptive step reached minimum step size")

    def evolve(self, u: Array, t0: float, tf: float, h_init: Optional[float] = None,
               store_data: bool = True, store_freq: int = 1) -> Array:
        """solveras.py:605-650 (adaptive) or solvercs.py:243-279 (constant)."""
        self.reset()
        self._tc = t0
        if store_data:
            self.t.append(t0)
            self.u.append(u)
        if not self.adaptive:
            h = h_init
            if self._tc + h > tf:
                raise ValueError("Step size h must be <= (tf - t0); reduce h or extend tf.")
            step_count = 0
            while self._tc < tf:
                u = self.step(u, h)
                self._tc += h
                step_count += 1
                if store_data and step_count % store_freq == 0:
                    self.t.append(self._tc)
                    self.u.append(u)
            return u
        if h_init is None:
            h_init = (tf - t0) / 100.0
        h = h_init
        if self._tc + h > tf:
            h = tf - self._tc
        step_count = 0
        while self._tc < tf:
            u, h, h_suggest = self.step(u, h)
            self._tc += h
            step_count += 1
            if self._tc + h_suggest > tf:
                h = tf - self._tc
            else:
                h = h_suggest
            if store_data and step_count % store_freq == 0:
                self.t.append(self._tc)
                self.u.append(u)
        return u
