"""A user-supplied nonlinearity (a torch callable on the device) with every method, against
the reference's own results (tests/golden) and the oracle.

Tolerances (FP64), as for the fused kernels:
  * fixed-step ETD4 / ETD5 / IF4: 1e-12 relative L2 against the reference
  * adaptive ETD35 / ETD34 / IF34 / IF45DP: the reference's number of attempts, snapshot
    times to 1e-10, final state 1e-8 (chaotic KS amplifies 1e-16 differences)
  * FP32 one adaptive step against the FP64 oracle: 1e-5
"""

import numpy as np
import pytest
import torch

import rkstiff_gb300 as rk
from oracle import rk_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def uux_torch(kx, n, c=-1.0):
    """c * rfft(irfft(u) * irfft(i kx u)) written as a plain torch function."""
    cache = {}

    def nl(u):
        key = (u.device, u.dtype)
        if key not in cache:
            cache[key] = torch.as_tensor(kx, device=u.device, dtype=u.real.dtype)
        k = cache[key]
        return c * torch.fft.rfft(torch.fft.irfft(u, n=n) * torch.fft.irfft(1j * k * u, n=n))
    return nl


@pytest.mark.parametrize("method", ["ETD4", "IF4", "ETD5"])
def test_fixed_step_kdv_callable(golden, method):
    g = golden("fixed_step")
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    lin, _ = rk.models.kdv_ops(kx)
    s = getattr(rk, method)(lin, uux_torch(kx, 256, -6.0))
    uf = s.evolve(g["kdv_u0"], 0.0, 0.025 * 200, 0.025, store_data=False)
    assert rel(uf, g[f"kdv_{method}_final"]) < 1e-12
    s = getattr(rk, method)(lin, uux_torch(kx, 256, -6.0))
    s.evolve(g["kdv_u0"], 0.0, 0.5, 0.025, store_data=True, store_freq=4)
    np.testing.assert_allclose(s.t, g[f"kdv_{method}_snap_t"], rtol=0, atol=1e-15)
    for a, b in zip(s.u, g[f"kdv_{method}_snap_u"]):
        assert rel(a, b) < 1e-12


@pytest.mark.parametrize("method", ["ETD35", "ETD34", "IF34", "IF45DP"])
def test_adaptive_ks256_callable(golden, method):
    g = golden("adaptive")
    x, kx = rk.grids.construct_x_kx_rfft(256, 0.0, float(g["ks256_L"]))
    lin, _ = rk.models.ks_ops(kx)
    s = getattr(rk, method)(lin, uux_torch(kx, 256), config=rk.SolverConfig(epsilon=1e-5))
    tf = 0.5 if method == "IF45DP" else 20.0
    uf = s.evolve(g["ks256_u0"], 0.0, tf, store_freq=10)
    assert s.stats["attempts"] == len(g[f"ks256_{method}_s"])
    np.testing.assert_allclose(s.t, g[f"ks256_{method}_t"], rtol=1e-10)
    assert rel(uf, g[f"ks256_{method}_final"]) < 1e-8


def test_nls_callable_with_torch_tensors():
    """A complex grid (NLS), torch tensors in and out, the step API."""
    x, kx = rk.grids.construct_x_kx_fft(256, -20, 20)
    lin, _ = rk.models.nls_ops(kx)

    def nl(u):
        v = torch.fft.ifft(u)
        return torch.fft.fft(1j * (v.abs() ** 2) * v)

    u0 = np.fft.fft(1.0 / np.cosh(x) * np.exp(0.5j * x))
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6))
    ud = torch.as_tensor(u0, device="cuda")
    uf = s.evolve(ud, 0.0, 2.0, store_data=False)
    assert isinstance(uf, torch.Tensor) and uf.is_cuda
    o = O.OracleSolver("ETD35", lin, lambda v: np.fft.fft(1j * np.abs(np.fft.ifft(v)) ** 2 * np.fft.ifft(v)),
                       O.SolverConfig(epsilon=1e-6))
    ref = o.evolve(u0, 0.0, 2.0, store_data=False)
    assert s.stats["attempts"] == o.attempts
    assert rel(uf, ref) < 1e-9
    unew, h_used, h_next = s.step(ud, 0.01)
    assert h_used <= 0.01 and h_next > 0 and unew.shape == ud.shape


def test_fp32_callable_one_step():
    x, kx = rk.grids.construct_x_kx_rfft(512, 0.0, 32 * np.pi)
    lin, _ = rk.models.ks_ops(kx)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    s = rk.ETD35(lin, uux_torch(kx, 512), config=rk.SolverConfig(epsilon=1e-4),
                 device_options=rk.DeviceOptions(precision="fp32"))
    unew, h_used, _ = s.step(u0, 0.1)
    o = O.OracleSolver("ETD35", lin, lambda v: -np.fft.rfft(np.fft.irfft(v) * np.fft.irfft(1j * kx * v)),
                       O.SolverConfig(epsilon=1e-4))
    ref, h_ref, _ = o.step(u0, 0.1)
    assert h_used == h_ref
    assert rel(unew, ref) < 1e-5


def test_callable_must_return_device_tensor():
    x, kx = rk.grids.construct_x_kx_rfft(64, 0.0, 22.0)
    lin, _ = rk.models.ks_ops(kx)
    s = rk.ETD35(lin, lambda u: np.zeros(33, complex))
    with pytest.raises(TypeError):
        s.evolve(np.fft.rfft(np.cos(2 * np.pi * x / 22)), 0.0, 1.0)
