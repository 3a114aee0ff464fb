"""GPU: device grids and spectral derivatives (rkstiff_gb300.grids with device=,
rkstiff_gb300.derivatives) against the reference's own outputs (tests/golden/derivs.npz)
and the CPU oracle.

Tolerances: Fourier grids bitwise (the kernels round every step as NumPy does);
Chebyshev points 1e-15 and matrices 1e-11 (the device cosine may differ from the host's by
an ulp, and 1/(x_i - x_j) of the clustered end points magnifies that ~1e3-fold);
derivatives relative to the largest entry: 1e-13 for first and second orders of FFT
derivatives of smooth data, 1e-12 beyond, and the Chebyshev products 1e-11 (D^3 of a
128-point matrix amplifies rounding by its norm)."""

import numpy as np
import pytest
import torch

from oracle import derivs as OD
from rkstiff_gb300 import derivatives as dv
from rkstiff_gb300 import grids

pytestmark = pytest.mark.gpu

SPECS = {"g1024": (1024, 0.0, 32 * np.pi), "g4096": (4096, -50.0, 50.0), "g256": (256, -30.0, 30.0),
         "g100": (100, 0.0, 2 * np.pi), "g400": (400, -30.0, 30.0), "g8": (8, 0.0, 2 * np.pi)}


def close(a, b, rtol):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)) <= rtol


def test_fourier_grids_bitwise(golden):
    g = golden("derivs")
    for tag, (n, a, b) in SPECS.items():
        x, kx = grids.construct_x_kx_rfft(n, a, b, device="cuda")
        assert x.is_cuda and kx.shape == (n // 2 + 1,)
        assert np.array_equal(x.cpu().numpy(), g[f"rfft_{tag}_x"]), tag
        assert np.array_equal(kx.cpu().numpy(), g[f"rfft_{tag}_kx"]), tag
        x2, kx2 = grids.construct_x_kx_fft(n, a, b, device="cuda")
        assert np.array_equal(x2.cpu().numpy(), g[f"rfft_{tag}_x"]), tag
        assert np.array_equal(kx2.cpu().numpy(), g[f"fft_{tag}_kx"]), tag


def test_cheb_grids(golden):
    g = golden("derivs")
    for tag, (n, a, b) in {"c20": (20, -1, 1), "c30": (30, -3, 3), "c128": (128, -1, 1)}.items():
        x, D = grids.construct_x_dx_cheb(n, a, b, device="cuda")
        assert close(x, g[f"cheb_{tag}_x"], 1e-15), tag
        assert close(grids.construct_x_cheb(n, a, b, device="cuda"), g[f"cheb_{tag}_x"], 1e-15), tag
        Dref = g[f"cheb_{tag}_D"] if f"cheb_{tag}_D" in g else OD.cheb_grid(n, a, b)[1]
        assert close(D, Dref, 1e-11), tag


def test_dx_rfft_reference_cases(golden):
    g = golden("derivs")
    for N, order in ((8, 1), (16, 2)):
        L = 2 * np.pi
        x = np.linspace(0, L, N, endpoint=False)
        kx = np.fft.rfftfreq(N, d=L / N) * 2 * np.pi
        out = dv.dx_rfft(kx, np.sin(x), n=order)
        assert isinstance(out, np.ndarray) and out.shape == x.shape and not np.iscomplexobj(out)
        assert close(out, g[f"drfft_{N}_{order}"], 1e-13)
        np.testing.assert_allclose(out, np.cos(x) if order == 1 else -np.sin(x), atol=1e-9)
    for N in (1024, 100):
        _, kx = grids.construct_x_kx_rfft(N, 0.0, 22.0, device="cuda")
        u = torch.as_tensor(g[f"drfft_rand{N}_u"], device="cuda")
        for order in (1, 2, 3):
            out = dv.dx_rfft(kx, u, n=order)
            assert out.is_cuda
            assert close(out, g[f"drfft_rand{N}_{order}"], 1e-13 if order < 3 else 1e-12), (N, order)


def test_dx_fft_reference_cases(golden):
    g = golden("derivs")
    x, kx = grids.construct_x_kx_fft(128, 0, 2 * np.pi)
    v = np.sin(x)
    for _ in range(4):
        v = dv.dx_fft(kx, v)
    # four differentiations amplify rounding by up to max|kx|^4 ~ 1.7e7, an eighth-order
    # one by ~3e14: these follow the reference's own tolerances against the exact
    # derivative (tests/test_derivatives_fft.py:9-26), and the reference's output to the
    # same amplified rounding
    assert np.linalg.norm(v - np.sin(x)) / np.linalg.norm(np.sin(x)) < 1e-6
    assert close(v, g["dfft_many4"], 1e-7)
    v8 = dv.dx_fft(kx, np.sin(x), 8)
    assert np.linalg.norm(v8 - np.sin(x)) / np.linalg.norm(np.sin(x)) < 0.1
    x, kx = grids.construct_x_kx_fft(100, 0, 2 * np.pi)
    assert close(dv.dx_fft(kx, np.sin(x)), g["dfft_periodic100"], 1e-13)
    x, kx = grids.construct_x_kx_fft(400, -30.0, 30.0)
    assert close(dv.dx_fft(kx, 1.0 / np.cosh(x)), g["dfft_sech400"], 1e-13)
    x, kx = grids.construct_x_kx_fft(128, -10, 10)
    assert close(dv.dx_fft(kx, np.exp(-(x**2))), g["dfft_gauss128"], 1e-13)
    # the 4096-point seeded case: the same draws as the generator
    rng = np.random.default_rng(31)
    for N in (1024, 100):
        rng.standard_normal(N)
    x, kx = grids.construct_x_kx_fft(4096, -50.0, 50.0, device="cuda")
    xh = x.cpu().numpy()
    uc = (rng.standard_normal(4096) + 1j * rng.standard_normal(4096)) * np.exp(-np.abs(xh) / 10)
    out = dv.dx_fft(kx, torch.as_tensor(uc, device="cuda"), 2)
    assert out.is_cuda and out.dtype == torch.complex128
    assert close(out, g["dfft_rand4096_2"], 1e-12)


def test_dx_cheb_reference_cases(golden):
    g = golden("derivs")
    for tag, (n, a, b) in {"c20": (20, -1, 1), "c30": (30, -3, 3)}.items():
        x, D = grids.construct_x_dx_cheb(n, a, b, device="cuda")
        u = torch.exp(x) * torch.sin(5 * x)
        for order in (1, 2, 3):
            assert close(dv.dx_cheb(D, u, n=order), g[f"dcheb_{tag}_{order}"], 1e-11), (tag, order)
    x, D = grids.construct_x_dx_cheb(20, -1, 1)
    U = np.stack([np.sin(x), np.cos(2 * x), x**3], axis=1)
    out = dv.dx_cheb(D, U, n=2)
    assert isinstance(out, np.ndarray) and out.shape == U.shape
    assert close(out, g["dcheb_c20_2d_2"], 1e-11)
    out = dv.dx_cheb(np.linspace(-1, 1, 8), np.eye(8))
    assert close(out, g["dcheb_swapped"], 1e-15)


def test_batched_rows_match_single_rows():
    """Extension: 2-D u differentiates row by row with one launch."""
    _, kx = grids.construct_x_kx_rfft(256, 0.0, 40.0, device="cuda")
    rng = np.random.default_rng(5)
    U = torch.as_tensor(rng.standard_normal((5, 256)), device="cuda")
    out = dv.dx_rfft(kx, U, 2)
    for r in range(5):
        assert torch.equal(out[r], dv.dx_rfft(kx, U[r].contiguous(), 2))
