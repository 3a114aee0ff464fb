"""GPU: the NLS soliton configuration at its full size, and the reference's two failure
exceptions, through the solver API (the C ABI underneath).

* NLS, n = 4096 on [-50, 50), three seeded solitons, ETD35, epsilon = 1e-6, t in [0, 20]
  (rkstiff/etd35.py:320-345 with N = fft(i |v|^2 v)):
  - FP64 against the reference's own run: the same 600 attempts and 3598 nonlinear
    evaluations, snapshot times to 1e-10, final state to 1e-10 relative L2;
  - FP32 (complex64 stages and transforms): one step from u0 at h = 0.02 to 1e-6 relative
    L2 of the reference's FP64 step; the whole run to tf = 20 to 1e-4.
* MaxLoopsExceeded (more than 50 retries, solveras.py:399-406): a non-finite state makes
  every attempt's s NaN; with minh = 1e-300 the retry bound is met before the step bound
  (the reference: 51 attempts), on the fused kernels in FP64 and FP32 and on the
  torch-callable path.
* MinimumStepReached for the reference's explosive nonlinearity 1e12 u
  (tests/test_etd35.py:111-121) on the torch-callable path.
"""

import numpy as np
import pytest
import torch

import problems as P
import rkstiff_gb300 as rk
from rkstiff_gb300 import models

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _nls4096():
    x, kx = rk.grids.construct_x_kx_fft(4096, -50.0, 50.0)
    return models.nls_ops(kx)


def test_nls4096_fp64_matches_reference(golden):
    g = golden("nls4096")
    lin, nl = _nls4096()
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6))
    uf = s.evolve(g["nls4096_u0"], 0.0, 20.0, store_freq=50)
    st = s.stats
    assert st["attempts"] == len(g["nls4096_ETD35_s"]) == 600
    assert st["nl_evals"] == int(g["nls4096_ETD35_nl_calls"]) == 3598
    np.testing.assert_allclose(s.t, g["nls4096_ETD35_t"], rtol=1e-10)
    assert rel(uf, g["nls4096_ETD35_final"]) < 1e-10


def test_nls4096_fp32_one_step_and_run(golden):
    g = golden("nls4096")
    lin, nl = _nls4096()
    opts = rk.DeviceOptions(precision="fp32")
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6), device_options=opts)
    u1, h1, hs1 = s.step(g["nls4096_u0"], 0.02)
    assert h1 == 0.02
    e1 = rel(u1, g["nls4096_step_u"])
    assert e1 < 1e-6, e1
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(epsilon=1e-6), device_options=opts)
    uf = s.evolve(g["nls4096_u0"], 0.0, 20.0, store_data=False)
    ef = rel(uf, g["nls4096_ETD35_final"])
    assert ef < 1e-4, ef


def _nan_state():
    x, kx, lin, nl = P.ks(64, 22.0)
    u0 = np.fft.rfft(np.cos(2 * np.pi * x / 22.0))
    u0[3] = np.nan
    return kx, lin, u0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_max_loops_exceeded_fused(golden, precision):
    g = golden("failure")
    kx, lin, u0 = _nan_state()
    _, nl = models.ks_ops(kx)
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(minh=1e-300),
                 device_options=rk.DeviceOptions(precision=precision))
    with pytest.raises(rk.BaseSolverAS.MaxLoopsExceeded):
        s.evolve(u0, 0.0, 1.0, h_init=0.1, store_data=False)
    assert s.stats["attempts"] == int(g["fail_nan_attempts"]) == 51


def test_max_loops_exceeded_callable(golden):
    g = golden("failure")
    kx, lin, u0 = _nan_state()
    kxt = torch.as_tensor(kx, device="cuda")

    def nl(u):
        return -torch.fft.rfft(torch.fft.irfft(u, n=64) * torch.fft.irfft(1j * kxt * u, n=64))
    s = rk.ETD35(lin, nl, config=rk.SolverConfig(minh=1e-300))
    with pytest.raises(rk.BaseSolverAS.MaxLoopsExceeded):
        s.evolve(u0, 0.0, 1.0, h_init=0.1, store_data=False)
    assert int(g["fail_nan"]) == 1


def test_explosive_nl_minimum_step_callable(golden):
    g = golden("failure")
    assert int(g["fail_explosive"]) == 2  # the reference raises MinimumStepReached
    s = rk.ETD35(np.array([-1.0]), lambda u: 1e12 * u, config=rk.SolverConfig(epsilon=1e-6))
    with pytest.raises(rk.BaseSolverAS.MinimumStepReached):
        s.evolve(np.array([1.0]), t0=0, tf=1e-3, h_init=1e-2, store_data=False)
