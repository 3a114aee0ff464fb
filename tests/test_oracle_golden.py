"""Pin the CPU oracle against golden vectors written by the reference itself (CPU only)."""

import math

import numpy as np
import pytest

import problems as P
from oracle import rk_oracle as O

ETD35_NAMES = ("a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54", "a61", "a62", "a63", "a65",
               "a71", "a73", "a74", "a75", "a76")


def _close(a, b, rtol):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = max(np.max(np.abs(b)), 1e-300)
    return np.max(np.abs(a - b)) <= rtol * scale


@pytest.mark.parametrize("tag", ["ks", "nls"])
@pytest.mark.parametrize("h", [0.05, 0.3])
def test_diag_coeffs_match_reference(golden, tag, h):
    g = golden("coeffs")
    lin = g[f"coef_{tag}_lin"]
    ht = f"{tag}_h{h}"
    c = O.diag_coeffs("ETD35", lin, h)
    for name, key in (("E14", "EL14"), ("E12", "EL12"), ("E34", "EL34"), ("E", "EL")):
        assert np.array_equal(c[name], g[f"coef_ETD35_{ht}_{key}"])
    for name in ETD35_NAMES:
        assert _close(c[name], g[f"coef_ETD35_{ht}_{name}"], 1e-15), name
    c = O.diag_coeffs("ETD5", lin, h)
    for name, key in (("a71", "b1"), ("a73", "b3"), ("a74", "b4"), ("a75", "b5"), ("a76", "b6"), ("a61", "a61")):
        assert _close(c[name], g[f"coef_ETD5_{ht}_{key}"], 1e-15), name
    for meth in ("ETD34", "ETD4"):
        c = O.diag_coeffs(meth, lin, h)
        keys = {"a51": "b1", "a52": "b2", "a54": "b4"} if meth == "ETD4" else {}
        assert np.array_equal(c["E"], g[f"coef_{meth}_{ht}_EL"])
        assert np.array_equal(c["E2"], g[f"coef_{meth}_{ht}_EL2"])
        for name in ("a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54"):
            assert _close(c[name], g[f"coef_{meth}_{ht}_{keys.get(name, name)}"], 1e-15), (meth, name)
    c = O.diag_coeffs("IF34", lin, h)
    assert np.array_equal(c["E"], g[f"coef_IF34_{ht}_EL"])
    assert np.array_equal(c["E2"], g[f"coef_IF34_{ht}_EL2"])
    c = O.diag_coeffs("IF45DP", lin, h)
    for name in ("E15", "E310", "E45", "E89", "E"):
        assert np.array_equal(c[name], g[f"coef_IF45DP_{ht}_EL{name[1:]}"])
    for name in ("a21", "a31", "a32", "a41", "a42", "a43", "a51", "a52", "a53", "a54", "a61", "a62", "a63",
                 "a64", "a65", "a71", "a73", "a74", "a75", "r1", "r3", "r4", "r5"):
        assert _close(c[name], g[f"coef_IF45DP_{ht}_{name}"], 1e-15), name
    np.testing.assert_array_equal([c["a76"], c["r6"], c["r7"]], g[f"coef_IF45DP_{ht}_scalars"])


def test_diag_coeffs_nondefault_etdconfig(golden):
    g = golden("coeffs")
    cfg = O.ETDConfig(modecutoff=0.5, contour_points=16, contour_radius=2.0)
    c = O.diag_coeffs("ETD35", g["coef_ks_lin"], 0.1, cfg)
    for name in ("a21", "a54", "a61", "a71", "a75", "a76"):
        assert _close(c[name], g[f"coef_ETD35cfg2_{name}"], 1e-15), name


@pytest.mark.parametrize("method", ["ETD4", "ETD5", "IF4"])
def test_fixed_step_kdv(golden, method):
    g = golden("fixed_step")
    kx, lin, nl, u0 = P.kdv_problem()
    np.testing.assert_array_equal(u0, g["kdv_u0"])
    s = O.OracleSolver(method, lin, nl)
    uf = s.evolve(u0, 0.0, 0.025 * 200, 0.025, store_data=False)
    assert _close(uf, g[f"kdv_{method}_final"], 1e-13)
    s = O.OracleSolver(method, lin, nl)
    s.evolve(u0, 0.0, 0.5, 0.025, store_data=True, store_freq=4)
    np.testing.assert_allclose(s.t, g[f"kdv_{method}_snap_t"], rtol=0, atol=1e-15)
    assert _close(np.array(s.u), g[f"kdv_{method}_snap_u"], 1e-14)


@pytest.mark.parametrize("method", ["ETD4", "IF4", "ETD5"])
def test_fixed_step_ks(golden, method):
    g = golden("fixed_step")
    x, kx, lin, nl = P.ks(128, 32 * np.pi)
    u0 = g["ks128_u0"]
    s = O.OracleSolver(method, lin, nl)
    uf = s.evolve(u0, 0.0, 10.0, 0.02, store_data=False)
    assert _close(uf, g[f"ks128_{method}_final"], 1e-12)


def test_adaptive_ks_config1_if34(golden):
    g = golden("adaptive")
    kx, lin, nl, u0 = P.ks_config1()
    s = O.OracleSolver("IF34", lin, nl, O.SolverConfig())
    uf = s.evolve(u0, 0.0, 50.0, store_freq=20)
    ref_s = g["ks1024_IF34_s"]
    got_s = np.array([r[2] for r in s.log])
    assert got_s.shape == ref_s.shape
    np.testing.assert_allclose(got_s, ref_s, rtol=1e-9)
    np.testing.assert_allclose(s.t, g["ks1024_IF34_t"], rtol=1e-13)
    assert _close(uf, g["ks1024_IF34_final"], 1e-9)
    assert _close(s.u[5], g["ks1024_IF34_u5"], 1e-11)


@pytest.mark.parametrize("method", ["ETD35", "ETD34", "IF34", "IF45DP"])
def test_adaptive_ks256(golden, method):
    g = golden("adaptive")
    kx, lin, nl, u0 = P.ks256_problem(golden)
    s = O.OracleSolver(method, lin, nl, O.SolverConfig(epsilon=1e-5))
    uf = s.evolve(u0, 0.0, 0.5 if method == "IF45DP" else 20.0, store_freq=10)
    got_s = np.array([r[2] for r in s.log])
    np.testing.assert_allclose(got_s, g[f"ks256_{method}_s"], rtol=1e-9)
    np.testing.assert_allclose(s.t, g[f"ks256_{method}_t"], rtol=1e-13)
    assert _close(uf, g[f"ks256_{method}_final"], 1e-9)


def test_adaptive_nls256_etd35(golden):
    g = golden("adaptive")
    kx, lin, nl = P.nls256()
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-6))
    uf = s.evolve(g["nls256_u0"], 0.0, 2.0, store_freq=5)
    np.testing.assert_allclose([r[2] for r in s.log], g["nls256_ETD35_s"], rtol=1e-9)
    np.testing.assert_allclose(s.t, g["nls256_ETD35_t"], rtol=1e-13)
    assert _close(uf, g["nls256_ETD35_final"], 1e-11)


def test_adaptive_burgers_etd35(golden):
    g = golden("adaptive")
    x, kx, lin, nl = P.burgers(512, 0.02)
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-5))
    uf = s.evolve(g["burg512_u0"], 0.0, 5.0, store_data=False)
    np.testing.assert_allclose([r[2] for r in s.log], g["burg512_ETD35_s"], rtol=1e-9)
    assert _close(uf, g["burg512_ETD35_final"], 1e-11)


@pytest.mark.parametrize("method", ["ETD34", "ETD35", "IF34"])
def test_adaptive_kdv(golden, method):
    g = golden("adaptive")
    kx, lin, nl, u0 = P.kdv_problem()
    s = O.OracleSolver(method, lin, nl, O.SolverConfig(epsilon=1e-4))
    uf = s.evolve(u0, 0.0, 5.0, h_init=0.025, store_data=False)
    assert _close(uf, g[f"kdv_{method}_adapt_final"], 1e-11)


def test_step_api_kdv_etd35(golden):
    g = golden("adaptive")
    kx, lin, nl, u0 = P.kdv_problem()
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-1))
    uu = u0.copy()
    for _ in range(200):
        uu, hh, hs = s.step(uu, 0.025)
        assert hh == 0.025
    assert _close(uu, g["kdv_ETD35_step200"], 1e-13)


def test_controller_clamps(golden):
    g = golden("controller")
    cfg = O.SolverConfig()
    for s, rej, acc in zip(g["ctl_s"], g["ctl_reject"], g["ctl_accept"]):
        assert O.reject_step_size(float(s), 0.1, cfg) == rej
        if math.isfinite(s):
            assert O.accept_step_size(float(s), 0.1, cfg) == acc


def test_controller_compute_s(golden):
    g = golden("controller")
    cfg = O.SolverConfig()
    for u, e, s in zip(g["ctl_u"], g["ctl_e"], g["ctl_s_out"]):
        assert O.compute_s(u, e, cfg, 4) == pytest.approx(s, rel=1e-15)


def test_failures(golden):
    g = golden("failure")
    assert int(g["fail_explosive"]) == 2
    s = O.OracleSolver("ETD35", np.array([-1.0]), lambda u: 1e12 * u, O.SolverConfig(epsilon=1e-6))
    with pytest.raises(O.MinimumStepReached):
        s.evolve(np.array([1.0]), 0, 1e-3, h_init=1e-2, store_data=False)
    assert int(g["fail_burg"]) == 2
    x, kx, lin, nl = P.burgers(512, float(g["fail_burg_nu"]))
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-5))
    with pytest.raises(O.MinimumStepReached):
        s.evolve(g["fail_burg_u0"], 0.0, 5.0, store_data=False)


def test_dense_allen_cahn(golden):
    g = golden("dense")
    x, D = P.cheb(20)
    np.testing.assert_allclose(D, g["cheb20_D"], rtol=0, atol=1e-12)
    x, lin, nl = P.allen_cahn(20)
    np.testing.assert_allclose(lin, g["ac20_lin"], rtol=0, atol=1e-12)
    w0 = g["ac20_w0"]
    cfg = O.ETDConfig(contour_points=32, contour_radius=10)
    C = O.dense_coeffs("ETD35", g["ac20_lin"], 0.05, cfg)
    for name in ("a21", "a54", "a65", "a76"):
        assert _close(C[name], g[f"ac20_ETD35_dense_{name}"], 1e-12), name
    assert _close(C["E"], g["ac20_ETD35_dense_EL"], 1e-13)
    s = O.OracleSolver("ETD35", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), cfg)
    assert _close(s.evolve(w0, 0, 60, store_data=False), g["ac20_ETD35_nondiag_final"], 1e-9)
    s = O.OracleSolver("ETD35", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), diagonalize=True)
    assert _close(s.evolve(w0, 0, 60, store_data=False), g["ac20_ETD35_diagz_final"], 1e-9)
    s = O.OracleSolver("ETD34", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), diagonalize=True)
    assert _close(s.evolve(w0, 0, 10, store_data=False), g["ac20_ETD34_diagz_final"], 1e-9)
    # non-diagonal ETD34: the reference's contour-mean matrices exactly; the eigenbasis
    # matrices (the dense GPU paths' form) differ by the contour's truncation error at R = 10
    s = O.OracleSolver("ETD34", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), cfg)
    assert _close(s.evolve(w0, 0, 10, store_data=False), g["ac20_ETD34_nondiag_final"], 1e-12)
    n_ref = s.attempts
    s = O.OracleSolver("ETD34", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), cfg, dense_psi="eig")
    assert _close(s.evolve(w0, 0, 10, store_data=False), g["ac20_ETD34_nondiag_final"], 3e-4)
    assert s.attempts == n_ref
    s = O.OracleSolver("IF34", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4), diagonalize=True)
    assert _close(s.evolve(w0, 0, 10, store_data=False), g["ac20_IF34_diagz_final"], 1e-9)
    s = O.OracleSolver("IF34", g["ac20_lin"], nl, O.SolverConfig(epsilon=1e-4))
    assert _close(s.evolve(w0, 0, 10, store_data=False), g["ac20_IF34_dense_final"], 1e-9)
    s = O.OracleSolver("IF4", g["ac20_lin"], nl)
    assert _close(s.evolve(w0, 0, 2, 0.01, store_data=False), g["ac20_IF4_dense_final"], 1e-12)
    s = O.OracleSolver("ETD4", g["ac20_lin"], nl, etd_config=cfg)
    assert _close(s.evolve(w0, 0, 2, 0.01, store_data=False), g["ac20_ETD4_dense_final"], 1e-12)


def _augmented_phis(Z):
    """phi_1..3(Z) from the exponential of the block matrix [[Z, I, 0, 0], [0, 0, I, 0],
    [0, 0, 0, I], [0, 0, 0, 0]] (its top row holds e^Z, phi_1, phi_2, phi_3)."""
    import scipy.linalg as sl

    n = Z.shape[0]
    A = np.zeros((4 * n, 4 * n))
    A[:n, :n] = Z
    for k in range(3):
        A[k * n:(k + 1) * n, (k + 1) * n:(k + 2) * n] = np.eye(n)
    E = sl.expm(A)
    return E[:n, n:2 * n], E[:n, 2 * n:3 * n], E[:n, 3 * n:]


def test_dense_coeffs_eig_matches_augmented_expm(golden):
    """The eigenbasis psi-matrices the dense tensor-core path uses, against an independent
    FP64 method, for every ETD35 coefficient of the reference's n=20 Allen-Cahn operator."""
    lin = golden("dense")["ac20_lin"]
    for h in (0.05, 0.4):
        C = O.dense_coeffs_eig("ETD35", lin, h)
        ph = {c: _augmented_phis(c * h * lin) for c in (0.25, 0.5, 0.75, 1.0)}
        p = {c: (ph[c][0], 2 * ph[c][1], 6 * ph[c][2]) for c in ph}  # psi_k = k! phi_k
        ref = {
            "a21": h * p[0.25][0] / 4.0, "a32": h * p[0.25][1] / 8.0, "a43": h * p[0.5][1] / 2.0,
            "a54": h * 9 * p[0.75][1] / 16.0, "a62": h * 8 * p[1.0][0] / 7.0,
            "a65": h * (-47 * p[1.0][0] + 143 * p[1.0][1]) / 84.0,
            "a76": h * (509 * p[1.0][0] - 2129 * p[1.0][1] + 1830 * p[1.0][2]) / 2700,
        }
        for k, v in ref.items():
            assert _close(C[k], v, 1e-9), (h, k)
        import scipy.linalg as sl
        assert _close(C["E"], sl.expm(h * lin), 1e-12)


def test_dense_coeffs_eig_vs_reference_contour_arrays(golden):
    """Against the reference's own dense arrays (contour radius 10, 32 points, h=0.05): they
    agree to the contour's truncation error (the trapezoidal rule's aliasing term is of
    order R^32/32! for these entire functions, about 1e-5 at R=10)."""
    g = golden("dense")
    C = O.dense_coeffs_eig("ETD35", g["ac20_lin"], 0.05)
    for name in ("a21", "a54", "a65", "a76"):
        assert _close(C[name], g[f"ac20_ETD35_dense_{name}"], 3e-5), name
    assert _close(C["E"], g["ac20_ETD35_dense_EL"], 1e-13)


def test_failure_nan_state_max_loops(golden):
    """A non-finite state with minh = 1e-300: the reference raises MaxLoopsExceeded after 51
    attempts (more than 50 retries, solveras.py:399-406); the oracle does the same."""
    g = golden("failure")
    assert int(g["fail_nan"]) == 1 and int(g["fail_nan_attempts"]) == 51
    x, kx, lin, nl = P.ks(64, 22.0)
    u0 = np.fft.rfft(np.cos(2 * np.pi * x / 22.0))
    u0[3] = np.nan
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(minh=1e-300))
    with pytest.raises(O.MaxLoopsExceeded):
        s.evolve(u0, 0.0, 1.0, h_init=0.1, store_data=False)
    assert s.attempts == 51


def test_adaptive_nls4096_etd35(golden):
    """The NLS soliton configuration at full size (n = 4096, eps = 1e-6, t in [0, 20])."""
    g = golden("nls4096")
    kx, lin, nl = P.nls4096()
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-6))
    uf = s.evolve(g["nls4096_u0"], 0.0, 20.0, store_freq=50)
    np.testing.assert_allclose([r[2] for r in s.log], g["nls4096_ETD35_s"], rtol=1e-9)
    np.testing.assert_allclose(s.t, g["nls4096_ETD35_t"], rtol=1e-13)
    assert _close(uf, g["nls4096_ETD35_final"], 1e-11)
    o = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-6))
    u1, h1, hs1 = o.step(g["nls4096_u0"], 0.02)
    assert [h1, hs1] == pytest.approx(list(g["nls4096_step_h"]), rel=1e-12)
    assert _close(u1, g["nls4096_step_u"], 1e-13)


def test_grids_and_derivatives(golden):
    """The oracle's grids and spectral derivatives against the reference's own outputs
    (grids bitwise; derivatives to rounding)."""
    from oracle import derivs as OD

    g = golden("derivs")
    specs = {"g1024": (1024, 0.0, 32 * np.pi), "g4096": (4096, -50.0, 50.0), "g256": (256, -30.0, 30.0),
             "g100": (100, 0.0, 2 * np.pi), "g400": (400, -30.0, 30.0), "g8": (8, 0.0, 2 * np.pi)}
    for tag, (n, a, b) in specs.items():
        x, kx = OD.fourier_grid(n, a, b, True)
        assert np.array_equal(x, g[f"rfft_{tag}_x"]) and np.array_equal(kx, g[f"rfft_{tag}_kx"]), tag
        assert np.array_equal(OD.fourier_grid(n, a, b, False)[1], g[f"fft_{tag}_kx"]), tag
    for tag, (n, a, b) in {"c20": (20, -1, 1), "c30": (30, -3, 3), "c128": (128, -1, 1)}.items():
        x, D = OD.cheb_grid(n, a, b)
        assert _close(x, g[f"cheb_{tag}_x"], 1e-15), tag
        if f"cheb_{tag}_D" in g:
            assert _close(D, g[f"cheb_{tag}_D"], 1e-13), tag
    for N, order in ((8, 1), (16, 2)):
        L = 2 * np.pi
        x = np.linspace(0, L, N, endpoint=False)
        kx = np.fft.rfftfreq(N, d=L / N) * 2 * np.pi
        assert _close(OD.dx_rfft(kx, np.sin(x), order), g[f"drfft_{N}_{order}"], 1e-14)
    for N in (1024, 100):
        _, kx = OD.fourier_grid(N, 0.0, 22.0, True)
        for order in (1, 2, 3):
            assert _close(OD.dx_rfft(kx, g[f"drfft_rand{N}_u"], order), g[f"drfft_rand{N}_{order}"], 1e-13)
    x, kx = OD.fourier_grid(128, 0, 2 * np.pi, False)
    assert _close(OD.dx_fft(kx, np.sin(x), 8), g["dfft_order8"], 1e-12)
    x, D = OD.cheb_grid(20, -1, 1)
    U = np.stack([np.sin(x), np.cos(2 * x), x**3], axis=1)
    assert _close(OD.dx_cheb(D, U, 2), g["dcheb_c20_2d_2"], 1e-11)


def test_adaptive_kdv_if45dp_long(golden):
    """IF45DP over t in [0, 5] on the KdV soliton (3627 attempts), against the reference."""
    g = golden("if45dp")
    kx, lin, nl, u0 = P.kdv_problem()
    s = O.OracleSolver("IF45DP", lin, nl, O.SolverConfig(epsilon=1e-4))
    uf = s.evolve(u0, 0.0, 5.0, h_init=0.025, store_freq=100)
    assert s.attempts == len(g["kdv_IF45DP_s"])
    np.testing.assert_allclose([r[2] for r in s.log], g["kdv_IF45DP_s"], rtol=1e-8)
    np.testing.assert_allclose(s.t, g["kdv_IF45DP_t"], rtol=1e-12)
    assert _close(uf, g["kdv_IF45DP_final"], 1e-10)
