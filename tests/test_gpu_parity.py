"""GPU parity: the CUDA path (through the C ABI) against the reference's golden vectors
and the CPU oracle.

Tolerances (relative L2 unless noted):
  * FP64 coefficient arrays vs the reference: 1e-13 (different exp/sincos/FMA rounding)
  * FP64 fixed-step ETD4/IF4/ETD5 final states vs the reference: 1e-12
  * FP64 adaptive runs vs the reference: identical number of attempts (the same
    accept/reject sequence), snapshot times 1e-10 (h = s*h carries ~1e-16 rounding of
    the norm's summation order each step), final states 1e-8 (chaotic KS amplifies it)
  * FP32 runs vs the FP64 oracle: one step 1e-6, short trajectories 1e-4
"""

import ctypes

import numpy as np
import pytest
import torch

import problems as P
import rkstiff_gb300 as rk
from oracle import rk_oracle as O
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rel_max(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def device_coeffs(method, lin, h, precision, etd=None):
    lib = nat.load()
    etd = etd or O.ETDConfig()
    cfg = nat.RkEtdConfig(modecutoff=etd.modecutoff, contour_radius=etd.contour_radius,
                          contour_points=etd.contour_points)
    m = lin.shape[0]
    cplx = 1 if np.iscomplexobj(lin) else 0
    nc = lib.rk_num_coeffs(nat.METHOD_IDS[method])
    lin_d = torch.from_numpy(lin.astype(np.complex128)).cuda()
    if precision == nat.RK_FP64:
        dt = torch.complex128 if cplx else torch.float64
    else:
        dt = torch.complex64 if cplx else torch.float32
    out = torch.zeros(nc * m, dtype=dt, device="cuda")
    nat.check(lib.rk_coeffs(nat.METHOD_IDS[method], precision, cplx, m, lin_d.data_ptr(), h, ctypes.byref(cfg),
                            out.data_ptr(), torch.cuda.current_stream().cuda_stream), "rk_coeffs")
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.complex128).reshape(nc, m)


ETD35_ORDER = ["E14", "E12", "E34", "E", "a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54", "a61", "a62",
               "a63", "a65", "a71", "a73", "a74", "a75", "a76"]
ETD34_ORDER = ["E", "E2", "a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54"]
IF45_ORDER = ["E15", "E310", "E45", "E89", "E", "a21", "a31", "a32", "a41", "a42", "a43", "a51", "a52", "a53", "a54",
              "a61", "a62", "a63", "a64", "a65", "a71", "a73", "a74", "a75", "r1", "r3", "r4", "r5"]


@pytest.mark.parametrize("tag", ["ks", "nls"])
@pytest.mark.parametrize("h", [0.05, 0.3])
@pytest.mark.parametrize("method,order", [("ETD35", ETD35_ORDER), ("ETD5", ETD35_ORDER), ("ETD34", ETD34_ORDER),
                                          ("ETD4", ETD34_ORDER), ("IF34", ["E", "E2"]), ("IF4", ["E", "E2"]),
                                          ("IF45DP", IF45_ORDER)])
def test_coefficients_fp64_match_reference(golden, tag, h, method, order):
    g = golden("coeffs")
    lin = g[f"coef_{tag}_lin"]
    got = device_coeffs(method, lin, h, nat.RK_FP64)
    ref = O.diag_coeffs(method, lin, h)
    for i, name in enumerate(order):
        r = ref[name]
        if r.ndim == 0:
            continue
        err = np.max(np.abs(got[i] - r)) / max(np.max(np.abs(r)), 1e-300)
        assert err < 1e-13, (method, name, err)


@pytest.mark.parametrize("method", ["ETD35", "ETD34"])
def test_coefficients_fp32_and_etdconfig(golden, method):
    g = golden("coeffs")
    lin = g["coef_ks_lin"]
    order = ETD35_ORDER if method == "ETD35" else ETD34_ORDER
    got = device_coeffs(method, lin, 0.3, nat.RK_FP32)
    ref = O.diag_coeffs(method, lin, 0.3)
    for i, name in enumerate(order):
        assert rel_max(got[i], ref[name]) < 1e-6, name
    cfg = O.ETDConfig(modecutoff=0.5, contour_points=16, contour_radius=2.0)
    got = device_coeffs("ETD35", lin, 0.1, nat.RK_FP64, cfg)
    for name in ("a21", "a54", "a61", "a71", "a75", "a76"):
        assert rel_max(got[ETD35_ORDER.index(name)], g[f"coef_ETD35cfg2_{name}"]) < 1e-13, name


# ------------------------------------------------------------------------------------
# fixed step: the <= 1e-12 FP64 parity target
# ------------------------------------------------------------------------------------
@pytest.mark.parametrize("method", ["ETD4", "ETD5", "IF4"])
def test_fixed_step_kdv_fp64(golden, method):
    g = golden("fixed_step")
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, nl = models.kdv_ops(kx)
    cls = getattr(rk, method)
    s = cls(lin, nl)
    uf = s.evolve(g["kdv_u0"], 0.0, 0.025 * 200, 0.025, store_data=False)
    assert rel(uf, g[f"kdv_{method}_final"]) < 1e-12
    s = cls(lin, nl)
    s.evolve(g["kdv_u0"], 0.0, 0.5, 0.025, store_data=True, store_freq=4)
    np.testing.assert_allclose(s.t, g[f"kdv_{method}_snap_t"], rtol=0, atol=1e-15)
    for a, b in zip(s.u, g[f"kdv_{method}_snap_u"]):
        assert rel(a, b) < 1e-12


@pytest.mark.parametrize("method", ["ETD4", "IF4", "ETD5"])
def test_fixed_step_ks_fp64(golden, method):
    g = golden("fixed_step")
    x, kx = rk.grids.construct_x_kx_rfft(128, 0.0, 32 * np.pi)
    lin, nl = models.ks_ops(kx)
    uf = getattr(rk, method)(lin, nl).evolve(g["ks128_u0"], 0.0, 10.0, 0.02, store_data=False)
    assert rel(uf, g[f"ks128_{method}_final"]) < 1e-12


def test_fixed_step_step_api_and_fsal():
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, nl = models.kdv_ops(kx)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0))
    s = rk.ETD4(lin, nl)
    o = O.OracleSolver("ETD4", lin, nl)
    u, uo = u0.copy(), u0.copy()
    for _ in range(20):
        u = s.step(u, 0.025)
        uo = o.step(uo, 0.025)
    assert rel(u, uo) < 1e-13
    with pytest.raises(ValueError):
        rk.ETD4(lin, nl).evolve(u0, 0.0, 0.01, 0.025)


# ------------------------------------------------------------------------------------
# adaptive, FP64: same accept/reject sequence as the reference
# ------------------------------------------------------------------------------------
def test_adaptive_if34_config1_fp64(golden):
    g = golden("adaptive")
    kx, lin, nl0, u0 = P.ks_config1()
    lin, nl = models.ks_ops(kx)
    s = rk.IF34(lin, nl, config=rk.SolverConfig())
    uf = s.evolve(u0, 0.0, 50.0, store_freq=20)
    st = s.stats
    assert st["attempts"] == len(g["ks1024_IF34_s"])
    np.testing.assert_allclose(s.t, g["ks1024_IF34_t"], rtol=1e-10)
    assert rel(s.u[5], g["ks1024_IF34_u5"]) < 1e-10
    assert rel(uf, g["ks1024_IF34_final"]) < 1e-8


@pytest.mark.parametrize("method", ["ETD35", "ETD34", "IF34", "IF45DP"])
def test_adaptive_ks256_fp64(golden, method):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_rfft(256, 0.0, float(g["ks256_L"]))
    lin, nl = models.ks_ops(kx)
    s = getattr(rk, method)(lin, nl, config=rk.SolverConfig(epsilon=1e-5))
    tf = 0.5 if method == "IF45DP" else 20.0
    uf = s.evolve(g["ks256_u0"], 0.0, tf, store_freq=10)
    assert s.stats["attempts"] == len(g[f"ks256_{method}_s"])
    np.testing.assert_allclose(s.t, g[f"ks256_{method}_t"], rtol=1e-10)
    assert rel(uf, g[f"ks256_{method}_final"]) < 1e-8


def test_adaptive_kdv_if45dp_long_fp64(golden):
    """IF45DP adaptive over a long span (t in [0, 5], 3627 attempts, KdV soliton) with the
    reference's attempt count and snapshot times; the stiff KS case above stops at t = 0.5."""
    g = golden("if45dp")
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, nl = models.kdv_ops(kx)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0))
    s = rk.IF45DP(lin, nl, config=rk.SolverConfig(epsilon=1e-4))
    uf = s.evolve(u0, 0.0, 5.0, h_init=0.025, store_freq=100)
    assert s.stats["attempts"] == len(g["kdv_IF45DP_s"])
    np.testing.assert_allclose(s.t, g["kdv_IF45DP_t"], rtol=1e-10)
    assert rel(uf, g["kdv_IF45DP_final"]) < 1e-9


def test_adaptive_nls_etd35_fp64(golden):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_fft(256, -20.0, 20.0)
    lin, nl = models.nls_ops(kx)
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6))
    uf = s.evolve(g["nls256_u0"], 0.0, 2.0, store_freq=5)
    assert s.stats["attempts"] == len(g["nls256_ETD35_s"])
    np.testing.assert_allclose(s.t, g["nls256_ETD35_t"], rtol=1e-10)
    assert rel(uf, g["nls256_ETD35_final"]) < 1e-10


def test_adaptive_burgers_and_kdv_fp64(golden):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_rfft(512, 0.0, 2 * np.pi)
    lin, nl = models.burgers_ops(kx, 0.02)
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-5))
    uf = s.evolve(g["burg512_u0"], 0.0, 5.0, store_data=False)
    assert s.stats["attempts"] == len(g["burg512_ETD35_s"])
    assert rel(uf, g["burg512_ETD35_final"]) < 1e-10
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, nl = models.kdv_ops(kx)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0))
    for method in ("ETD34", "ETD35", "IF34"):
        s = getattr(rk, method)(lin, nl, config=rk.SolverConfig(epsilon=1e-4))
        uf = s.evolve(u0, 0.0, 5.0, h_init=0.025, store_data=False)
        assert rel(uf, g[f"kdv_{method}_adapt_final"]) < 1e-10, method


def test_adaptive_step_api_fp64(golden):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, nl = models.kdv_ops(kx)
    u = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0))
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-1))
    for _ in range(200):
        u, h, hs = s.step(u, 0.025)
        assert h == 0.025
    assert rel(u, g["kdv_ETD35_step200"]) < 1e-12
    assert s._accept


def test_minimum_step_reached_like_reference(golden):
    g = golden("failure")
    x, kx = rk.grids.construct_x_kx_rfft(512, 0.0, 2 * np.pi)
    lin, nl = models.burgers_ops(kx, float(g["fail_burg_nu"]))
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-5))
    with pytest.raises(rk.BaseSolverAS.MinimumStepReached):
        s.evolve(g["fail_burg_u0"], 0.0, 5.0, store_data=False)


def test_snapshot_buffer_resume_is_transparent():
    x, kx = rk.grids.construct_x_kx_rfft(128, 0.0, 32 * np.pi)
    lin, nl = models.ks_ops(kx)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    a = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-5))
    ua = a.evolve(u0, 0.0, 10.0, store_freq=3)
    b = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-5), device_options=rk.DeviceOptions(snap_cap=2))
    ub = b.evolve(u0, 0.0, 10.0, store_freq=3)
    assert np.array_equal(ua, ub)
    assert a.t == b.t
    assert all(np.array_equal(p, q) for p, q in zip(a.u, b.u))
    o = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-5))
    o.evolve(u0, 0.0, 10.0, store_freq=3)
    np.testing.assert_allclose(a.t, o.t, rtol=1e-10)


def test_negative_span_and_torch_io():
    x, kx = rk.grids.construct_x_kx_rfft(64, 0.0, 22.0)
    lin, nl = models.ks_ops(kx)
    u0 = np.fft.rfft(np.cos(2 * np.pi * x / 22.0))
    s = rk.ETD35(lin, nl)
    np.testing.assert_array_equal(s.evolve(u0, 1.0, 0.0, 0.1, False), u0)
    ut = torch.from_numpy(u0).cuda()
    out = rk.ETD35(lin, nl).evolve(ut, 0.0, 1.0, store_data=False)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    ref = rk.ETD35(lin, nl).evolve(u0, 0.0, 1.0, store_data=False)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


# ------------------------------------------------------------------------------------
# FP32 form: bounded error against the FP64 oracle
# ------------------------------------------------------------------------------------
def test_fp32_one_step_error(golden):
    x, kx = rk.grids.construct_x_kx_rfft(256, 0.0, 50.0)
    lin, nl = models.ks_ops(kx)
    u0 = golden("adaptive")["ks256_u0"]
    o = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-5))
    uo, ho, _ = o.step(u0, 0.05)
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-5), device_options=rk.DeviceOptions(precision="fp32"))
    u, h, _ = s.step(u0, 0.05)
    assert h == ho
    assert rel(u, uo) < 1e-6


@pytest.mark.parametrize("method", ["ETD35", "IF34", "ETD34"])
def test_fp32_short_trajectory(golden, method):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_rfft(256, 0.0, float(g["ks256_L"]))
    lin, nl = models.ks_ops(kx)
    o = O.OracleSolver(method, lin, nl, O.SolverConfig(epsilon=1e-9))
    uo = o.evolve(g["ks256_u0"], 0.0, 2.0, store_data=False)
    s = getattr(rk, method)(lin, nl, config=rk.SolverConfig(epsilon=1e-5),
                            device_options=rk.DeviceOptions(precision="fp32"))
    u = s.evolve(g["ks256_u0"], 0.0, 2.0, store_data=False)
    assert rel(u, uo) < 1e-4


def test_fp32_nls(golden):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_fft(256, -20.0, 20.0)
    lin, nl = models.nls_ops(kx)
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6), device_options=rk.DeviceOptions(precision="fp32"))
    u = s.evolve(g["nls256_u0"], 0.0, 2.0, store_data=False)
    assert rel(u, g["nls256_ETD35_final"]) < 1e-4


# (stage fraction s, a, b, g, D) of each coefficient h (a psi_1 + b psi_2 + g psi_3)(s z) / D
# (etd35.py:157-288, etd34.py:107-149); the exponentials are marked with D = 0
_COMB35 = [(0.25, 0, 0, 0, 0), (0.5, 0, 0, 0, 0), (0.75, 0, 0, 0, 0), (1.0, 0, 0, 0, 0),
           (0.25, 1, 0, 0, 4), (0.25, 2, -1, 0, 8), (0.25, 0, 1, 0, 8), (0.5, 1, -1, 0, 2), (0.5, 0, 1, 0, 2),
           (0.75, 12, -9, 0, 16), (0.75, -3, 0, 0, 8), (0.75, 0, 9, 0, 16), (1.0, -77, 59, 0, 42),
           (1.0, 8, 0, 0, 7), (1.0, 111, -87, 0, 28), (1.0, -47, 143, 0, 84), (1.0, 1799, -3479, 1890, 2700),
           (1.0, 1097, -467, -150, 1350), (1.0, -98, 398, -270, 225), (1.0, -313, 883, -90, 1350),
           (1.0, 509, -2129, 1830, 2700)]
_COMB34 = [(1.0, 0, 0, 0, 0), (0.5, 0, 0, 0, 0), (0.5, 1, 0, 0, 2), (0.5, 1, -1, 0, 2), (0.5, 0, 1, 0, 2),
           (1.0, 1, -1, 0, 1), (1.0, 0, 1, 0, 1), (1.0, 6, -9, 4, 6), (1.0, 0, 3, -2, 3), (1.0, 0, -3, 4, 6)]


def _psi_term_scale(comb, z, h, value):
    """h (|a psi_1| + |b psi_2| + |g psi_3|)(s z) / D in FP64 (the value itself for the
    exponentials): the magnitude the combination is formed from."""
    s, a, b, g, D = comb
    if D == 0:
        return np.abs(value)
    x = s * z
    with np.errstate(all="ignore"):
        em1 = np.expm1(x)
        p1 = em1 / x
        p2 = 2 * (em1 - x) / x**2
        p3 = 6 * (em1 - x - x**2 / 2) / x**3
    return h * (abs(a) * np.abs(p1) + abs(b) * np.abs(p2) + abs(g) * np.abs(p3)) / D


@pytest.mark.parametrize("method", ["ETD35", "ETD5", "ETD34", "ETD4"])
@pytest.mark.parametrize("h", [1e-3, 0.1, 1.7])
def test_fp32_coefficients_round_fp64(method, h):
    """FP32 coefficients of a real operator against the FP64 evaluation rounded to FP32 over
    z = h lambda from -1e9 to +50 (stiff, moderate, near the modecutoff, growing modes).
    Below z = -32 they come from the stiff form in FP32 (expf, whose error of up to 2 ulps
    carries through the exponentials' products: within 6 FP32 ulps, plus 1e-13 |z| relative:
    combinations such as ETD34 a51 = psi1 - 1.5 psi2 + 2/3 psi3 cancel their O(h/z) parts
    down to O(h/z^2) by ~|z|, on coefficients whose contribution is below FP32 resolution).
    From -32 to 80 each combination comes from its own FP32 Taylor series (or the stiff form
    where its scaled argument is >= 9): within 4 ulps of the value or 3 ulps of the
    combination's psi-term scale h (|a psi_1| + |b psi_2| + |g psi_3|)/D, the rounding an FP32
    evaluation of any form leaves near a zero of the combination."""
    lam = np.concatenate([-np.logspace(-6, 9, 300), np.logspace(-6, np.log10(50.0 / h), 60), [0.0]])
    order = ETD35_ORDER if method in ("ETD35", "ETD5") else ETD34_ORDER
    combs = _COMB35 if method in ("ETD35", "ETD5") else _COMB34
    c32 = device_coeffs(method, lam, h, nat.RK_FP32).real
    c64 = device_coeffs(method, lam, h, nat.RK_FP64).real
    r32 = c64.astype(np.float32).astype(np.float64)
    ulp = np.spacing(np.abs(r32).astype(np.float32)).astype(np.float64)
    z = h * lam
    zmag = np.maximum(1.0, np.abs(z))
    # below the modecutoff both precisions use small-mode series (FP32 storage: Taylor;
    # FP64: the reference's contour mean), whose ~1/z cancellation in combinations such as
    # a41 = (psi1 - psi2)/2 leaves them ~1e-16/|z| apart: compared on the array's scale
    direct = np.abs(z) >= 0.01
    for i, name in enumerate(order):
        scale = _psi_term_scale(combs[i], z, h, c64[i])
        ulp_s = np.spacing(np.abs(scale).astype(np.float32)).astype(np.float64)
        tol = np.where(z < -32.0, 6.0 * ulp[i], 4.0 * ulp[i] + 3.0 * ulp_s) + 1e-13 * zmag * np.abs(r32[i]) + 1e-37
        bad = direct & (np.abs(c32[i] - r32[i]) > tol)
        assert not np.any(bad), (method, h, name, lam[bad][:3], c32[i][bad][:3], r32[i][bad][:3])
        small = ~direct
        assert np.max(np.abs(c32[i][small] - c64[i][small])) <= 1e-6 * np.max(np.abs(c64[i])), (method, h, name)
