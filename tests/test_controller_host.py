"""Learned step-size controller, host side: the NumPy FP64 MLP oracle against finite
differences, the feature/target extraction on a hand-made attempt log, and the shipped
parameter file."""

import math
import os

import numpy as np
import pytest

from oracle import mlp as MO
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import controller as C


def _params(rng):
    IN, H = MO.IN, MO.H
    return np.concatenate([rng.standard_normal(H * IN) / np.sqrt(IN), 0.1 * rng.standard_normal(H),
                           rng.standard_normal(H * H) / np.sqrt(H), 0.1 * rng.standard_normal(H),
                           rng.standard_normal(H) / np.sqrt(H), [0.3]])


def test_layout_matches_header():
    assert MO.IN == nat.RK_MLP_IN and MO.H == nat.RK_MLP_H
    assert MO.IN * MO.H + MO.H + MO.H * MO.H + MO.H + MO.H + 1 == nat.RK_MLP_NPARAM


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(rng)
    X = rng.standard_normal((37, MO.IN))
    T = rng.standard_normal(37) * 0.1
    loss, g = MO.loss_and_grad(p, X, T, 37.0)
    idx = rng.choice(p.size, 60, replace=False).tolist() + [p.size - 1]  # include b3
    for i in idx:
        d = np.zeros_like(p)
        d[i] = 1e-6
        fd = (MO.loss_and_grad(p + d, X, T, 37.0)[0] - MO.loss_and_grad(p - d, X, T, 37.0)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-7 + 1e-6 * abs(fd), (i, fd, g[i])


def _record(t, h, s, ok, tail, loops):
    return [t, h, s, 1.0 if ok else 0.0, tail, loops, 512, nat.RK_ETD35]


def test_features_targets_on_a_hand_made_log():
    # attempt 0 accepted, 1 rejected, 2 accepted (after one retry), 3 accepted
    rec = np.array([_record(0.0, 0.1, 1.5, True, 1e-12, 0),
                    _record(0.1, 0.15, 0.6, False, 1e-11, 0),
                    _record(0.1, 0.09, 1.2, True, 1e-11, 1),
                    _record(0.19, 0.09, 1.1, True, 2e-11, 0)], dtype=np.float32)
    log = rec[None]
    X, T = C.features_targets(log, np.array([4]))
    assert X.shape == (2, nat.RK_MLP_IN) and T.shape == (2,)  # attempts 0 and 2; 3 has no successor
    ls = [math.log(v) for v in (1.5, 0.6, 1.2, 1.1)]
    # sample from attempt 0: no history yet
    np.testing.assert_allclose(X[0], [ls[0], 0, 0, 0, 1, 0, math.log10(1e-12 + 1e-30), 0], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(T[0], ls[1] + math.log(0.15 / 0.1) - ls[0], rtol=1e-5)
    # sample from attempt 2: previous attempt rejected, one retry, ratio to the rejected h
    f2 = [ls[2], ls[1], ls[0], math.log(0.09 / 0.15), 0, 1, math.log10(1e-11), 0.0]
    np.testing.assert_allclose(X[1], f2, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(T[1], ls[3] + math.log(0.09 / 0.09) - ls[2], rtol=1e-5)


def test_features_skip_non_finite_successors_and_clip_targets():
    rec = np.array([_record(0.0, 0.1, 1.3, True, 0.0, 0),
                    _record(0.1, 0.1, -1.0, False, 0.0, 0),       # NaN s: no sample from attempt 0
                    _record(0.1, 0.025, 50.0, True, 0.0, 1),
                    _record(0.125, 0.1, 1e30, True, 0.0, 0),      # inf s: no sample from attempt 2
                    _record(0.225, 0.1, 1.01, True, 0.0, 0),
                    _record(0.325, 0.1, 1e-6, False, 0.0, 0)], dtype=np.float32)
    X, T = C.features_targets(rec[None], np.array([6]))
    assert X.shape[0] == 2  # from attempts 3 and 4
    assert np.all(np.abs(T) <= 1.0) and T[1] == -1.0  # a big drop is clipped
    assert X[0][0] == 8.0  # log s of an infinite s is clamped to 8


def test_shipped_controller_file():
    assert os.path.exists(C.PRETRAINED)
    with np.load(C.PRETRAINED) as z:
        assert z["params"].shape == (nat.RK_MLP_NPARAM,) and z["params"].dtype == np.float32
        assert z["mu"].shape == (nat.RK_MLP_IN,) and np.all(z["sd"] > 0)
        assert np.all(np.isfinite(z["params"]))
        assert 1.0 < float(z["target"]) < 1.3
