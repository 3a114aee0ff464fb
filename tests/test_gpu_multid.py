"""Multi-dimensional NLS problems of the reference's NLS demo on the device (ETD35 with a
flattened diagonal lin_op and a device-side torch nonlinearity: 2-D FFTs, and the Hankel
transform as a GEMM on the device), against the reference's own runs
(tests/golden/multid.npz).

Tolerances: FP64 final states 1e-10 relative L2 and snapshot times rtol 1e-10 (the same
controller decisions; rounding differs between torch/cuFFT and numpy/pocketfft, and the
error estimate cancels, so s and the h it sets differ at ~1e-11); FP32
2-D run 1e-4 (complex64 stages and FFTs against the FP64 reference).
"""

import numpy as np
import pytest
import torch

import rkstiff_gb300 as rk
from rkstiff_gb300 import models
from rkstiff_gb300.device import DeviceOptions
from rkstiff_gb300.grids import construct_x_kx_fft
from rkstiff_gb300.transforms import HankelTransform

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_radial_nls_on_a_hankel_grid(golden):
    g = golden("multid")
    L, nl = models.nls_radial_ops(HankelTransform(nr=32, rmax=5.0), 2.0)
    s = rk.ETD35(L, nl, config=rk.SolverConfig(epsilon=1e-5))
    uf = s.evolve(g["hnls_u0"], t0=0.0, tf=0.2, store_data=True, store_freq=5)
    assert type(s._engine()).__name__ == "CallableBackend"
    np.testing.assert_allclose(s.t, g["hnls_t"], rtol=1e-10)
    assert rel(uf, g["hnls_final"]) < 1e-10


def test_radial_time_nls_hankel_and_fft(golden):
    g = golden("multid")
    nr, nt = (int(v) for v in g["rtnls_shape"])
    _, om = construct_x_kx_fft(nt, -6, 6)
    L, nl = models.nls_radial_time_ops(HankelTransform(nr=nr, rmax=4.0), om, 0.5, 2.0)
    s = rk.ETD35(L, nl, config=rk.SolverConfig(epsilon=1e-5))
    uf = s.evolve(g["rtnls_u0"], t0=0.0, tf=0.03, store_data=False)
    assert rel(uf, g["rtnls_final"]) < 1e-10


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-4)])
def test_nls_2d_fft2(golden, precision, tol):
    g = golden("multid")
    _, kx = construct_x_kx_fft(32, -6, 6)
    _, ky = construct_x_kx_fft(32, -6, 6)
    L, nl = models.nls_2d_ops(kx, ky, 2.0)
    s = rk.ETD35(L, nl, device_options=DeviceOptions(precision=precision))
    uf = s.evolve(g["nls2d_u0"], t0=0.0, tf=0.2, store_data=True, store_freq=4)
    if precision == "fp64":
        np.testing.assert_allclose(s.t, g["nls2d_t"], rtol=1e-10)
    assert rel(uf, g["nls2d_final"]) < tol


def _torch_eval(nl, g):
    F = nl._inv(g.reshape(nl.shape))
    a2 = F.real * F.real + F.imag * F.imag
    return nl._fwd((1j * nl.gamma) * (a2 * F)).reshape(-1)


@pytest.mark.parametrize("dtype,tol", [(torch.complex128, 1e-13), (torch.complex64, 2e-6)])
def test_multid_kernels_match_the_torch_composition(dtype, tol):
    """The library's line-FFT / Hankel kernels against torch's FFTs and matrix product for
    the three demo nonlinearities (random spectra; FP64 to rounding, FP32 to a few ulps of
    the transform sizes)."""
    rng = np.random.default_rng(4)
    _, kx = construct_x_kx_fft(32, -6, 6)
    _, ky = construct_x_kx_fft(64, -8, 8)
    ht = HankelTransform(nr=24, rmax=4.0)
    _, om = construct_x_kx_fft(32, -6, 6)
    for L, nl in (models.nls_2d_ops(kx, ky, 2.0), models.nls_radial_ops(ht, 2.0),
                  models.nls_radial_time_ops(ht, om, 0.5, 2.0)):
        n = int(np.prod(nl.shape))
        g = torch.as_tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n), device="cuda").to(dtype)
        g0 = g.clone()
        dev = nl._device(g)
        assert dev is not None, nl.name
        assert torch.equal(g, g0), nl.name  # the input is left as it was
        ref = _torch_eval(nl, g) if dtype == torch.complex128 else \
            _torch_eval(nl, g.to(torch.complex128)).to(dtype)
        err = float(torch.linalg.norm(dev - ref) / torch.linalg.norm(ref))
        assert err < tol, (nl.name, err)
        assert torch.equal(nl(g), dev)


def test_hankel_kernel_matches_host_product():
    """rk_dht (device) against the NumPy product of the reference's form, S Y f and Y g / S,
    on real and complex, 1-D and 2-D inputs."""
    rng = np.random.default_rng(9)
    ht = HankelTransform(nr=40, rmax=3.0)
    for shape in ((40,), (40, 7)):
        for cplx in (False, True):
            f = rng.standard_normal(shape) + (1j * rng.standard_normal(shape) if cplx else 0.0)
            ft = torch.as_tensor(f, device="cuda")
            for fn in (ht.ht, ht.iht):
                got = fn(ft).cpu().numpy()
                ref = fn(f)
                assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-13
