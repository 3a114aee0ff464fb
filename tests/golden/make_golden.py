"""Write golden vectors by running the reference rkstiff implementation itself.

Run in a container where the reference source tree is available:

    python tests/golden/make_golden.py <path of the rkstiff source tree> [case ...]

The reference package is copied to a scratch directory (its ``__init__`` imports a
setuptools-scm generated ``__version__`` module, which the copy supplies) and imported
from there.  The outputs are small ``.npz`` files in this directory; tests load them on
any machine without the reference.  Seeds are fixed so the script is reproducible.
"""

from __future__ import annotations

import os
import shutil
import sys
import tempfile
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(ref_root: str):
    tmp = tempfile.mkdtemp(prefix="rkstiff_ref_")
    shutil.copytree(os.path.join(ref_root, "rkstiff"), os.path.join(tmp, "rkstiff"))
    with open(os.path.join(tmp, "rkstiff", "__version__.py"), "w") as f:
        f.write('version = "0.0.0"\n')
    sys.path.insert(0, tmp)
    import rkstiff  # noqa: F401
    return tmp


def ks_problem(n, L):
    from rkstiff import grids
    x, kx = grids.construct_x_kx_rfft(n, 0.0, L)
    lin = kx**2 * (1 - kx**2)

    def nl(u):
        return -np.fft.rfft(np.fft.irfft(u) * np.fft.irfft(1j * kx * u))
    return x, kx, lin, nl


def burgers_problem(n, nu):
    from rkstiff import grids, models
    x, kx = grids.construct_x_kx_rfft(n, 0.0, 2 * np.pi)
    lin, nl = models.burgers_ops(kx, nu)
    return x, kx, lin, nl


def nls_problem(n, a, b):
    from rkstiff import grids
    x, kx = grids.construct_x_kx_fft(n, a, b)
    lin = -0.5j * kx**2

    def nl(u):
        v = np.fft.ifft(u)
        return np.fft.fft(1j * np.abs(v) ** 2 * v)
    return x, kx, lin, nl


class Recorder:
    """Wraps a solver's _compute_s to log (h_attempt, s) pairs."""

    def __init__(self, solver):
        self.s = []
        orig = solver._compute_s

        def wrapped(u, err):
            s = orig(u, err)
            self.s.append(s)
            return s
        solver._compute_s = wrapped


def coeff_cases(out):
    from rkstiff import etd35, etd34, etd4, etd5, if34, if4, if45dp, etd
    _, kx, lin_ks, _ = ks_problem(64, 22.0)
    _, kxn, lin_nls, _ = nls_problem(64, -10.0, 10.0)
    nl = lambda u: u  # noqa: E731
    cfg = etd.ETDConfig()
    for tag, lin in (("ks", lin_ks), ("nls", lin_nls)):
        out[f"coef_{tag}_lin"] = lin
        for h in (0.05, 0.3):
            ht = f"{tag}_h{h}"
            m = etd35._Etd35Diagonal(lin, nl, cfg)
            m.update_coeffs(h)
            for name in ("EL14", "EL12", "EL34", "EL", "a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54",
                         "a61", "a62", "a63", "a65", "a71", "a73", "a74", "a75", "a76"):
                out[f"coef_ETD35_{ht}_{name}"] = getattr(m, "_" + name)
            m = etd34._Etd34Diagonal(lin, nl, cfg)
            m.update_coeffs(h)
            for name in ("EL", "EL2", "a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54"):
                out[f"coef_ETD34_{ht}_{name}"] = getattr(m, "_" + name)
            m = etd4._Etd4Diagonal(lin, nl, cfg)
            m.update_coeffs(h)
            for name in ("EL", "EL2", "a21", "a31", "a32", "a41", "a43", "b1", "b2", "b4"):
                out[f"coef_ETD4_{ht}_{name}"] = getattr(m, "_" + name)
            m = etd5._Etd5Diagonal(lin, nl, cfg)
            m.update_coeffs(h)
            for name in ("EL14", "EL12", "EL34", "EL", "a21", "a31", "a32", "a41", "a43", "a51", "a52", "a54",
                         "a61", "a62", "a63", "a65", "b1", "b3", "b4", "b5", "b6"):
                out[f"coef_ETD5_{ht}_{name}"] = getattr(m, "_" + name)
            m = if34._If34Diagonal(lin, nl)
            m.update_coeffs(h)
            out[f"coef_IF34_{ht}_EL"] = m._EL
            out[f"coef_IF34_{ht}_EL2"] = m._EL2
            s = if45dp.IF45DP(lin, nl)
            s._update_coeffs(h)
            for name in ("EL15", "EL310", "EL45", "EL89", "EL", "a21", "a31", "a32", "a41", "a42", "a43", "a51",
                         "a52", "a53", "a54", "a61", "a62", "a63", "a64", "a65", "a71", "a73", "a74", "a75",
                         "r1", "r3", "r4", "r5"):
                out[f"coef_IF45DP_{ht}_{name}"] = getattr(s, "_" + name)
            out[f"coef_IF45DP_{ht}_scalars"] = np.array([s._a76, s._r6, s._r7])
    # a non-default ETDConfig (fewer contour points, larger cutoff) on the KS operator
    cfg2 = etd.ETDConfig(modecutoff=0.5, contour_points=16, contour_radius=2.0)
    m = etd35._Etd35Diagonal(lin_ks, nl, cfg2)
    m.update_coeffs(0.1)
    for name in ("a21", "a54", "a61", "a71", "a75", "a76"):
        out[f"coef_ETD35cfg2_{name}"] = getattr(m, "_" + name)


def fixed_step_cases(out):
    from rkstiff import etd4, etd5, if4, models, grids
    x, kx = grids.construct_x_kx_rfft(256, -30, 30)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0, t=0))
    lin, nl = models.kdv_ops(kx)
    out["kdv_u0"] = u0
    out["kdv_kx"] = kx
    for name, cls in (("ETD4", etd4.ETD4), ("ETD5", etd5.ETD5), ("IF4", if4.IF4)):
        s = cls(lin, nl)
        out[f"kdv_{name}_final"] = s.evolve(u0, t0=0.0, tf=0.025 * 200, h=0.025, store_data=False)
        s = cls(lin, nl)
        s.evolve(u0, t0=0.0, tf=0.5, h=0.025, store_data=True, store_freq=4)
        out[f"kdv_{name}_snap_t"] = np.array(s.t)
        out[f"kdv_{name}_snap_u"] = np.array(s.u)
    # KS fixed-step, n=128 on [0, 32pi)
    x, kx, lin, nl = ks_problem(128, 32 * np.pi)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    out["ks128_u0"] = u0
    for name, cls in (("ETD4", etd4.ETD4), ("IF4", if4.IF4), ("ETD5", etd5.ETD5)):
        s = cls(lin, nl)
        out[f"ks128_{name}_final"] = s.evolve(u0, t0=0.0, tf=10.0, h=0.02, store_data=False)


def adaptive_cases(out):
    from rkstiff import if34, etd35, etd34, if45dp, models, grids
    from rkstiff.solveras import SolverConfig
    # config-1 shape: KS n=1024 IF34 eps=1e-4, tf=50, store_freq=20
    x, kx, lin, nl = ks_problem(1024, 32 * np.pi)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    s = if34.IF34(lin, nl, config=SolverConfig())
    rec = Recorder(s)
    uf = s.evolve(u0, t0=0.0, tf=50.0, store_freq=20)
    out["ks1024_IF34_final"] = uf
    out["ks1024_IF34_t"] = np.array(s.t)
    out["ks1024_IF34_u5"] = s.u[5]
    out["ks1024_IF34_s"] = np.array(rec.s)

    # KS ETD35 n=256, L=50, eps=1e-5, tf=20
    rng = np.random.default_rng(7)
    L = 50.0
    x, kx, lin, nl = ks_problem(256, L)
    k = np.arange(1, 9)
    a = rng.standard_normal(8) * np.exp(-k / 4)
    ph = rng.uniform(0, 2 * np.pi, 8)
    u0 = np.fft.rfft(np.sum(a[:, None] * np.cos(2 * np.pi * k[:, None] * x[None, :] / L + ph[:, None]), axis=0))
    out["ks256_u0"] = u0
    out["ks256_L"] = np.array(L)
    for name, cls in (("ETD35", etd35.ETD35), ("ETD34", etd34.ETD34), ("IF34", if34.IF34), ("IF45DP", if45dp.IF45DP)):
        s = cls(lin, nl, config=SolverConfig(epsilon=1e-5))
        rec = Recorder(s)
        # IF45DP needs ~6e3 attempts per unit time on this stiff operator: keep its span short
        uf = s.evolve(u0, t0=0.0, tf=(0.5 if name == "IF45DP" else 20.0), store_freq=10)
        out[f"ks256_{name}_final"] = uf
        out[f"ks256_{name}_t"] = np.array(s.t)
        out[f"ks256_{name}_s"] = np.array(rec.s)

    # NLS ETD35 n=256 on [-20, 20), two solitons, eps=1e-6, tf=2
    x, kx, lin, nl = nls_problem(256, -20.0, 20.0)
    u0x = 1.0 / np.cosh(x + 5) * np.exp(0.5j * x) + 1.5 / np.cosh(1.5 * (x - 4)) * np.exp(-0.3j * x)
    u0 = np.fft.fft(u0x)
    out["nls256_u0"] = u0
    s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-6))
    rec = Recorder(s)
    out["nls256_ETD35_final"] = s.evolve(u0, t0=0.0, tf=2.0, store_freq=5)
    out["nls256_ETD35_t"] = np.array(s.t)
    out["nls256_ETD35_s"] = np.array(rec.s)

    # Burgers n=512, nu=0.02, ETD35 eps=1e-5 tf=5 (six sine modes, amplitude N(0, 1/k))
    rng = np.random.default_rng(11)
    x, kx, lin, nl = burgers_problem(512, 0.02)
    kk = np.arange(1, 7)
    amp = rng.standard_normal(6) / kk
    u0 = np.fft.rfft(np.sum(amp[:, None] * np.sin(kk[:, None] * x[None, :]), axis=0))
    out["burg512_u0"] = u0
    s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-5))
    rec = Recorder(s)
    out["burg512_ETD35_final"] = s.evolve(u0, t0=0.0, tf=5.0, store_data=False)
    out["burg512_ETD35_s"] = np.array(rec.s)

    # KdV ETD34 / ETD35 evolve (reference tests test_etd34.py, test_etd35.py)
    x, kx = grids.construct_x_kx_rfft(256, -30, 30)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0, t=0))
    lin, nl = models.kdv_ops(kx)
    for name, cls in (("ETD34", etd34.ETD34), ("ETD35", etd35.ETD35), ("IF34", if34.IF34)):
        s = cls(lin, nl, config=SolverConfig(epsilon=1e-4))
        out[f"kdv_{name}_adapt_final"] = s.evolve(u0, t0=0.0, tf=5.0, h_init=0.025, store_data=False)

    # step() with eps=1e-1: h never changes (test_etd35.py:24-27)
    s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-1))
    uu = u0.copy()
    for _ in range(200):
        uu, hh, hs = s.step(uu, 0.025)
    out["kdv_ETD35_step200"] = uu


def controller_cases(out):
    from rkstiff.solveras import BaseSolverAS, SolverConfig
    from rkstiff.if34 import IF34
    s = IF34(np.array([-1.0, -2.0]), lambda u: u, config=SolverConfig())
    svals = np.array([np.nan, np.inf, -np.inf, 0.0, 0.1, 0.25, 0.3, 0.84, 0.85, 0.9, 0.999, 1.0, 1.2, 1.25, 1.26,
                      2.0, 3.99, 4.0, 10.0])
    rej = np.array([s._reject_step_size(v, 0.1) for v in svals])
    acc = np.array([s._accept_step_size(v, 0.1) if np.isfinite(v) else np.nan for v in svals])
    out["ctl_s"] = svals
    out["ctl_reject"] = rej
    out["ctl_accept"] = acc
    rng = np.random.default_rng(3)
    us, es, ss = [], [], []
    for i in range(16):
        n = 40
        u = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * np.exp(-np.arange(n) / 6.0)
        e = 1e-6 * (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * (1 + i)
        us.append(u)
        es.append(e)
        ss.append(s._compute_s(u, e))
    out["ctl_u"] = np.array(us)
    out["ctl_e"] = np.array(es)
    out["ctl_s_out"] = np.array(ss)


def dense_cases(out):
    from rkstiff import grids, models, etd35, etd34, if34, etd4, if4
    from rkstiff.solveras import SolverConfig
    from rkstiff.etd import ETDConfig
    x, D = grids.construct_x_dx_cheb(20, -1, 1)
    out["cheb20_x"] = x
    out["cheb20_D"] = D
    lin, nl = models.allen_cahn_ops(x, D, 0.01)
    u0 = 0.53 * x + 0.47 * np.sin(-1.5 * np.pi * x)
    w0 = (u0 - x)[1:-1]
    out["ac20_lin"] = lin
    out["ac20_w0"] = w0
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-4), etd_config=ETDConfig(contour_points=32,
                                                                                            contour_radius=10))
        out["ac20_ETD35_nondiag_final"] = s.evolve(w0, t0=0, tf=60, store_data=False)
        s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-4), diagonalize=True)
        out["ac20_ETD35_diagz_final"] = s.evolve(w0, t0=0, tf=60, store_data=False)
        s = etd34.ETD34(lin, nl, config=SolverConfig(epsilon=1e-4), diagonalize=True)
        out["ac20_ETD34_diagz_final"] = s.evolve(w0, t0=0, tf=10, store_data=False)
        s = etd34.ETD34(lin, nl, config=SolverConfig(epsilon=1e-4), etd_config=ETDConfig(contour_points=32,
                                                                                          contour_radius=10))
        out["ac20_ETD34_nondiag_final"] = s.evolve(w0, t0=0, tf=10, store_data=False)
        s = if34.IF34(lin, nl, config=SolverConfig(epsilon=1e-4), diagonalize=True)
        out["ac20_IF34_diagz_final"] = s.evolve(w0, t0=0, tf=10, store_data=False)
        s = if34.IF34(lin, nl, config=SolverConfig(epsilon=1e-4))
        out["ac20_IF34_dense_final"] = s.evolve(w0, t0=0, tf=10, store_data=False)
        s = if4.IF4(lin, nl)
        out["ac20_IF4_dense_final"] = s.evolve(w0, t0=0, tf=2, h=0.01, store_data=False)
        s = etd4.ETD4(lin, nl, etd_config=ETDConfig(contour_points=32, contour_radius=10))
        out["ac20_ETD4_dense_final"] = s.evolve(w0, t0=0, tf=2, h=0.01, store_data=False)
    # ETD35 dense coefficient matrices at one h (contour R=10)
    m = etd35._Etd35NonDiagonal(lin, nl, ETDConfig(contour_points=32, contour_radius=10))
    m.update_coeffs(0.05)
    for name in ("EL", "a21", "a54", "a65", "a76"):
        out[f"ac20_ETD35_dense_{name}"] = getattr(m, "_" + name)


def failure_cases(out):
    from rkstiff import etd35
    from rkstiff.solveras import SolverConfig, BaseSolverAS
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        s = etd35.ETD35(np.array([-1.0]), lambda u: 1e12 * u, config=SolverConfig(epsilon=1e-6))
        try:
            s.evolve(np.array([1.0]), t0=0, tf=1e-3, h_init=1e-2, store_data=False)
            out["fail_explosive"] = np.array(0)
        except BaseSolverAS.MinimumStepReached:
            out["fail_explosive"] = np.array(2)
        except BaseSolverAS.MaxLoopsExceeded:
            out["fail_explosive"] = np.array(1)
        # under-resolved Burgers at n=512: nu log-uniform in [1e-3, 1e-1] drawn with seed 2 (nu ~ 3.3e-3)
        rng = np.random.default_rng(2)
        nu = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1))))
        x, kx, lin, nl = burgers_problem(512, nu)
        kk = np.arange(1, 7)
        amp = rng.standard_normal(6) / kk
        out["fail_burg_nu"] = np.array(nu)
        u0 = np.fft.rfft(np.sum(amp[:, None] * np.sin(kk[:, None] * x[None, :]), axis=0))
        out["fail_burg_u0"] = u0
        s = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-5))
        try:
            s.evolve(u0, t0=0.0, tf=5.0, store_data=False)
            out["fail_burg"] = np.array(0)
        except BaseSolverAS.MinimumStepReached:
            out["fail_burg"] = np.array(2)
        except BaseSolverAS.MaxLoopsExceeded:
            out["fail_burg"] = np.array(1)
        # a non-finite state: every attempt's s is NaN, h shrinks by 0.25 per rejection, and
        # with minh = 1e-300 the retry bound (more than 50 loops) is met first
        x, kx, lin, nl = ks_problem(64, 22.0)
        u0 = np.fft.rfft(np.cos(2 * np.pi * x / 22.0))
        u0[3] = np.nan
        s = etd35.ETD35(lin, nl, config=SolverConfig(minh=1e-300))
        rec = Recorder(s)
        try:
            s.evolve(u0, t0=0.0, tf=1.0, h_init=0.1, store_data=False)
            out["fail_nan"] = np.array(0)
        except BaseSolverAS.MaxLoopsExceeded:
            out["fail_nan"] = np.array(1)
        except BaseSolverAS.MinimumStepReached:
            out["fail_nan"] = np.array(2)
        out["fail_nan_attempts"] = np.array(len(rec.s))


def nls_solitons_u0(n, seed):
    """Three seeded solitons on [-50, 50): A_j sech(A_j (x - x_j)) exp(i v_j x) with
    A_j ~ U[0.5, 2], x_j ~ U[-30, 30], v_j ~ U[-1, 1] (the draw order of
    rkstiff_gb300.workloads.nls_solitons)."""
    rng = np.random.default_rng(seed)
    x = -50.0 + np.arange(n) * (100.0 / n)
    A = rng.uniform(0.5, 2.0, 3)
    x0 = rng.uniform(-30.0, 30.0, 3)
    v = rng.uniform(-1.0, 1.0, 3)
    return np.fft.fft(sum(A[j] / np.cosh(A[j] * (x - x0[j])) * np.exp(1j * v[j] * x) for j in range(3)))


def nls4096_cases(out):
    """The NLS soliton configuration at its full size: n = 4096 on [-50, 50), ETD35,
    epsilon = 1e-6, t in [0, 20], snapshots every 50 accepted steps."""
    from rkstiff import etd35
    from rkstiff.solveras import SolverConfig
    x, kx, lin, nl = nls_problem(4096, -50.0, 50.0)
    u0 = nls_solitons_u0(4096, 0)
    calls = [0]

    def counted(u):
        calls[0] += 1
        return nl(u)
    s = etd35.ETD35(lin, counted, config=SolverConfig(epsilon=1e-6))
    rec = Recorder(s)
    out["nls4096_u0"] = u0
    out["nls4096_ETD35_final"] = s.evolve(u0, t0=0.0, tf=20.0, store_freq=50)
    out["nls4096_ETD35_t"] = np.array(s.t)
    out["nls4096_ETD35_s"] = np.array(rec.s)
    out["nls4096_ETD35_nl_calls"] = np.array(calls[0])
    # one step of the same problem from u0 at h = 0.02 (the one-step gate of FP32 runs)
    s1 = etd35.ETD35(lin, nl, config=SolverConfig(epsilon=1e-6))
    u1, h1, hs1 = s1.step(u0, 0.02)
    out["nls4096_step_u"] = u1
    out["nls4096_step_h"] = np.array([h1, hs1])


def derivs_cases(out):
    """Grids and spectral derivatives of rkstiff/grids.py and rkstiff/derivatives.py on the
    inputs of the reference's own tests plus larger seeded ones."""
    from rkstiff import grids, derivatives
    for tag, (n, a, b) in {"g1024": (1024, 0.0, 32 * np.pi), "g4096": (4096, -50.0, 50.0), "g256": (256, -30.0, 30.0),
                           "g100": (100, 0.0, 2 * np.pi), "g400": (400, -30.0, 30.0), "g8": (8, 0.0, 2 * np.pi)}.items():
        x, kx = grids.construct_x_kx_rfft(n, a, b)
        out[f"rfft_{tag}_x"], out[f"rfft_{tag}_kx"] = x, kx
        out[f"fft_{tag}_kx"] = grids.construct_x_kx_fft(n, a, b)[1]
    for tag, (n, a, b) in {"c20": (20, -1, 1), "c30": (30, -3, 3), "c128": (128, -1, 1)}.items():
        x, D = grids.construct_x_dx_cheb(n, a, b)
        out[f"cheb_{tag}_x"] = x
        if n <= 30:
            out[f"cheb_{tag}_D"] = D
    # dx_rfft: tests/test_derivatives_rfft.py inputs (N = 8, 16) and seeded rows
    for N, order in ((8, 1), (16, 2)):
        L = 2 * np.pi
        x = np.linspace(0, L, N, endpoint=False)
        kx = np.fft.rfftfreq(N, d=L / N) * 2 * np.pi
        out[f"drfft_{N}_{order}"] = derivatives.dx_rfft(kx, np.sin(x), n=order)
    rng = np.random.default_rng(31)
    for N in (1024, 100):
        x, kx = grids.construct_x_kx_rfft(N, 0.0, 22.0)
        u = rng.standard_normal(N) * np.exp(-np.abs(np.fft.fftfreq(N) * N) / 8)
        out[f"drfft_rand{N}_u"] = u
        for order in (1, 2, 3):
            out[f"drfft_rand{N}_{order}"] = derivatives.dx_rfft(kx, u, n=order)
    # dx_fft: tests/test_derivatives_fft.py inputs
    x, kx = grids.construct_x_kx_fft(128, 0, 2 * np.pi)
    v = np.sin(x)
    for _ in range(4):
        v = derivatives.dx_fft(kx, v)
    out["dfft_many4"] = v
    out["dfft_order8"] = derivatives.dx_fft(kx, np.sin(x), 8)
    x, kx = grids.construct_x_kx_fft(100, 0, 2 * np.pi)
    out["dfft_periodic100"] = derivatives.dx_fft(kx, np.sin(x))
    x, kx = grids.construct_x_kx_fft(400, -30.0, 30.0)
    out["dfft_sech400"] = derivatives.dx_fft(kx, 1.0 / np.cosh(x))
    x, kx = grids.construct_x_kx_fft(128, -10, 10)
    out["dfft_gauss128"] = derivatives.dx_fft(kx, np.exp(-(x**2)))
    x, kx = grids.construct_x_kx_fft(4096, -50.0, 50.0)
    uc = (rng.standard_normal(4096) + 1j * rng.standard_normal(4096)) * np.exp(-np.abs(x) / 10)
    out["dfft_rand4096_2"] = derivatives.dx_fft(kx, uc, 2)
    # dx_cheb: tests/test_derivatives_cheb.py inputs, higher orders and a 2-D u
    for tag, (n, a, b) in {"c20": (20, -1, 1), "c30": (30, -3, 3)}.items():
        x, D = grids.construct_x_dx_cheb(n, a, b)
        u = np.exp(x) * np.sin(5 * x)
        for order in (1, 2, 3):
            out[f"dcheb_{tag}_{order}"] = derivatives.dx_cheb(D, u, n=order)
    x, D = grids.construct_x_dx_cheb(20, -1, 1)
    U = np.stack([np.sin(x), np.cos(2 * x), x**3], axis=1)
    out["dcheb_c20_2d_2"] = derivatives.dx_cheb(D, U, n=2)
    arr = np.linspace(-1, 1, 8)
    out["dcheb_swapped"] = derivatives.dx_cheb(arr, np.eye(8))


def if45dp_cases(out):
    """IF45DP adaptive over a longer span than the stiff KS case allows: the KdV soliton
    (n = 256 on [-30, 30)), epsilon = 1e-4, t in [0, 5] (~3600 accepted steps)."""
    from rkstiff import if45dp, models, grids
    from rkstiff.solveras import SolverConfig
    x, kx = grids.construct_x_kx_rfft(256, -30, 30)
    u0 = np.fft.rfft(models.kdv_soliton(x, ampl=1.0, x0=-5.0, t=0))
    lin, nl = models.kdv_ops(kx)
    s = if45dp.IF45DP(lin, nl, config=SolverConfig(epsilon=1e-4))
    rec = Recorder(s)
    out["kdv_IF45DP_final"] = s.evolve(u0, t0=0.0, tf=5.0, h_init=0.025, store_freq=100)
    out["kdv_IF45DP_t"] = np.array(s.t)
    out["kdv_IF45DP_s"] = np.array(rec.s)


def multid_cases(out):
    """The multi-dimensional spectral problems of the reference's NLS demo (demos/nls.ipynb):
    the radial NLS on a Hankel grid, the (r, t) NLS with a Hankel transform in r and an FFT
    in t, and the 2-D NLS with fft2; all ETD35 with a flattened diagonal lin_op.  Smaller
    grids and horizons than the demo, the same operators and initial shapes."""
    from rkstiff.transforms import HankelTransform
    from rkstiff.grids import construct_x_kx_fft, mirror_grid
    from rkstiff.etd35 import ETD35
    from rkstiff.solveras import SolverConfig
    gamma = 2.0
    # the transform itself
    HT = HankelTransform(nr=16, rmax=4.0)
    out["ht16_r"], out["ht16_kr"] = HT.r, HT.kr
    out["ht16_Y"], out["ht16_zeros"] = HT.hankel_matrix(), HT.bessel_zeros()
    f = np.exp(-HT.r**2) * (1 + 0.5j * HT.r)
    out["ht16_f"], out["ht16_ht"] = f, HT.ht(f)
    out["ht16_iht"] = HT.iht(HT.ht(f))
    rm, um = mirror_grid(HT.r, np.abs(f) ** 2)
    out["ht16_mirror_r"], out["ht16_mirror_u"] = rm, um
    # radial NLS (cells 6-12): L = -i kr^2, N = i gamma ht(|f|^2 f), f = iht(g)
    HT = HankelTransform(nr=32, rmax=5.0)
    L = -1j * HT.kr**2

    def nl_r(g):
        fr = HT.iht(g)
        return 1j * gamma * HT.ht((fr.real**2 + fr.imag**2) * fr)
    u0 = HT.ht(2.0 * np.exp(-HT.r**2))
    s = ETD35(lin_op=L, nl_func=nl_r, config=SolverConfig(epsilon=1e-5))
    out["hnls_u0"] = u0
    out["hnls_final"] = s.evolve(u0, t0=0, tf=0.2, store_data=True, store_freq=5)
    out["hnls_t"] = np.array(s.t)
    # (r, t) NLS (cells 14-20): Hankel transform over axis 0, FFT over axis 1
    nr, nt, sigma = 12, 32, 0.5
    HT = HankelTransform(nr=nr, rmax=4.0)
    t, omega = construct_x_kx_fft(nt, -6, 6)
    R, T = np.meshgrid(HT.r, t, indexing="ij")
    KR, OM = np.meshgrid(HT.kr, omega, indexing="ij")
    L = (-1j * KR**2 + 1j * sigma * OM**2).flatten()

    def nl_rt(g):
        F = np.fft.ifft(HT.iht(g.reshape(nr, nt)), axis=1)
        return 1j * gamma * np.fft.fft(HT.ht((F.real**2 + F.imag**2) * F), axis=1).flatten()
    U0 = 4.0 * np.exp(-(R / 1.0) ** 2 - (T / 0.5) ** 2)
    u0 = np.fft.fft(HT.ht(U0), axis=1).flatten()
    s = ETD35(lin_op=L, nl_func=nl_rt, config=SolverConfig(epsilon=1e-5))
    out["rtnls_u0"] = u0
    out["rtnls_final"] = s.evolve(u0, t0=0, tf=0.03, store_data=False)
    out["rtnls_shape"] = np.array([nr, nt])
    # 2-D NLS (cells 27-29): fft2 on a 32 x 32 grid
    nx = ny = 32
    x, kx = construct_x_kx_fft(nx, -6, 6)
    y, ky = construct_x_kx_fft(ny, -6, 6)
    X, Y = np.meshgrid(x, y, indexing="ij")
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    L = (-1j * (KX**2 + KY**2)).flatten()

    def nl_2d(g):
        F = np.fft.ifft2(g.reshape(nx, ny))
        return 1j * gamma * np.fft.fft2((F.real**2 + F.imag**2) * F).flatten()
    u0 = np.fft.fft2(2.0 * np.exp(-X**2 - Y**2)).flatten()
    s = ETD35(lin_op=L, nl_func=nl_2d)
    out["nls2d_u0"] = u0
    out["nls2d_final"] = s.evolve(u0, t0=0, tf=0.2, store_data=True, store_freq=4)
    out["nls2d_t"] = np.array(s.t)


CASES = (("coeffs", coeff_cases), ("fixed_step", fixed_step_cases), ("adaptive", adaptive_cases),
         ("controller", controller_cases), ("dense", dense_cases), ("failure", failure_cases),
         ("multid", multid_cases), ("nls4096", nls4096_cases),
         ("derivs", derivs_cases), ("if45dp", if45dp_cases))


def main():
    """make_golden.py [reference root] [case names...]: every case file by default."""
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the rkstiff source tree> [case ...]")
    ref_root = sys.argv[1]
    only = set(sys.argv[2:])
    tmp = import_reference(ref_root)
    try:
        for fname, fn in CASES:
            if only and fname not in only:
                continue
            out = {}
            fn(out)
            path = os.path.join(HERE, f"{fname}.npz")
            np.savez_compressed(path, **out)
            print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path)} bytes")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
