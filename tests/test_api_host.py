"""Host-side API behaviour that needs no GPU: configs, validation, enums, built-in NLs."""

import logging

import numpy as np
import pytest
import torch

import problems as P
import rkstiff_gb300 as rk
from rkstiff_gb300 import models


def test_solver_config_validation():
    c = rk.SolverConfig()
    assert (c.epsilon, c.incr_f, c.decr_f, c.safety_f, c.adapt_cutoff, c.minh) == (1e-4, 1.25, 0.85, 0.8, 0.01, 1e-16)
    for kw in ({"epsilon": 0}, {"incr_f": 1.0}, {"decr_f": 1.0}, {"safety_f": 1.1}, {"adapt_cutoff": 1.0},
               {"minh": 0.0}):
        with pytest.raises(ValueError):
            rk.SolverConfig(**kw)


def test_etd_config_validation():
    c = rk.ETDConfig()
    assert (c.modecutoff, c.contour_points, c.contour_radius) == (0.01, 32, 1.0)
    with pytest.raises(ValueError):
        rk.ETDConfig(modecutoff=0)
    with pytest.raises(ValueError):
        rk.ETDConfig(modecutoff=1.5)
    with pytest.raises(TypeError):
        rk.ETDConfig(contour_points=3.0)
    with pytest.raises(ValueError):
        rk.ETDConfig(contour_points=1)
    with pytest.raises(ValueError):
        rk.ETDConfig(contour_radius=0)


def test_psi_functions_match_series():
    z = np.array([0.5, -2.0 + 1j, 3.0])
    np.testing.assert_allclose(rk.psi1(z), (np.exp(z) - 1) / z)
    np.testing.assert_allclose(rk.psi2(z), 2 * (np.exp(z) - 1 - z) / z**2)
    np.testing.assert_allclose(rk.psi3(z), 6 * (np.exp(z) - 1 - z - z**2 / 2) / z**3)


def test_operator_shape_validation_and_types():
    nl = lambda u: u  # noqa: E731
    with pytest.raises(ValueError):
        rk.ETD35(np.zeros((2, 3)), nl)
    with pytest.raises(ValueError):
        rk.ETD35(np.zeros((2, 2, 2)), nl)
    with pytest.raises(ValueError):
        rk.IF45DP(np.eye(3), nl)
    s = rk.ETD35(np.array([-1.0, -2.0]), nl)
    assert s.solver_type == rk.SolverType.ADAPTIVE_STEP
    assert rk.SolverType.from_solver(s) == rk.SolverType.ADAPTIVE_STEP
    assert rk.ETD4(np.array([-1.0]), nl).solver_type == rk.SolverType.CONSTANT_STEP
    assert str(rk.SolverType.CONSTANT_STEP) == "Constant Step"
    assert rk.SolverType.CS is rk.SolverType.CONSTANT_STEP
    with pytest.raises(TypeError):
        rk.SolverType.from_solver(object())
    assert s._diag and not rk.ETD35(np.eye(2), nl)._diag


def test_dense_operator_checks_before_any_device_work(caplog):
    """diagonalize=True checks cond(lin_op) when the solver is built, as the reference's
    diagonalized strategies do (ValueError above 1e16, a warning above 1000); a defective
    operator (a Jordan block) cannot be stepped in an eigenbasis and is refused with
    NotImplementedError before anything touches the device."""
    nl = lambda u: u  # noqa: E731
    for cls in (rk.ETD35, rk.ETD34, rk.IF34):
        with pytest.raises(ValueError):
            cls(np.zeros((3, 3)), nl, diagonalize=True)
    with caplog.at_level(logging.WARNING):
        rk.ETD34(np.diag([1.0, 1e-4]), nl, diagonalize=True)
    assert "condition number" in caplog.text
    rk.ETD35(np.zeros(3), nl, diagonalize=True)  # 1-D: the diagonal strategy, no check
    for s in (rk.ETD35(np.array([[-1.0, 1.0], [0.0, -1.0]]), nl), rk.IF4(np.array([[-1.0, 1.0], [0.0, -1.0]]), nl)):
        with pytest.raises(NotImplementedError):
            if s.solver_type == rk.SolverType.ADAPTIVE_STEP:
                s.evolve(np.ones(2), 0.0, 1.0)
            else:
                s.evolve(np.ones(2), 0.0, 1.0, 0.1)


def test_fresh_config_per_solver():
    nl = lambda u: u  # noqa: E731
    a = rk.ETD35(np.array([-1.0]), nl)
    a.config.epsilon = 0.5
    b = rk.ETD35(np.array([-1.0]), nl)
    assert b.config.epsilon == 1e-4


def test_exceptions_and_constants():
    assert issubclass(rk.BaseSolverAS.MaxLoopsExceeded, rk.BaseSolverAS.SolverError)
    assert issubclass(rk.BaseSolverAS.MinimumStepReached, RuntimeError)
    assert (rk.BaseSolverAS.MAX_LOOPS, rk.BaseSolverAS.MAX_S, rk.BaseSolverAS.MIN_S) == (50, 4.0, 0.25)


def test_logger_names_and_levels():
    s = rk.IF34(np.array([-1.0]), lambda u: u, loglevel="DEBUG")
    assert s.logger.name == "rkstiff.IF34"
    assert s.logger.level == logging.DEBUG
    s.set_loglevel("ERROR")
    assert s.logger.level == logging.ERROR
    with pytest.raises(ValueError):
        s.set_loglevel("LOUD")


def test_builtin_nl_matches_numpy_closures():
    x, kx = rk.grids.construct_x_kx_rfft(64, 0.0, 22.0)
    lin, nl = models.ks_ops(kx)
    rng = np.random.default_rng(0)
    u = rng.standard_normal(33) + 1j * rng.standard_normal(33)
    np.testing.assert_allclose(nl(u), P.uux_nl(kx)(u), rtol=1e-12, atol=1e-12)
    lin2, nl2 = models.kdv_ops(kx)
    np.testing.assert_allclose(nl2(u), P.uux_nl(kx, -6.0)(u), rtol=1e-12, atol=1e-11)
    x, kxn = rk.grids.construct_x_kx_fft(64, -10, 10)
    linn, nln = models.nls_ops(kxn)
    v = rng.standard_normal(64) + 1j * rng.standard_normal(64)
    np.testing.assert_allclose(nln(v), P.nls_nl(v), rtol=1e-12, atol=1e-12)
    assert isinstance(nln(torch.from_numpy(v)), torch.Tensor)
    np.testing.assert_allclose(lin, kx**2 * (1 - kx**2))
    np.testing.assert_allclose(models.burgers_ops(kx, 0.1)[0], -0.1 * kx**2)


def test_grids_match_reference_golden(golden):
    x, D = rk.grids.construct_x_dx_cheb(20, -1, 1)
    np.testing.assert_allclose(D, golden("dense")["cheb20_D"], rtol=0, atol=1e-12)
    with pytest.raises(ValueError):
        rk.grids.construct_x_kx_rfft(7)
    x, kx = rk.grids.construct_x_kx_rfft(256, -30, 30)
    np.testing.assert_array_equal(kx, golden("fixed_step")["kdv_kx"])


def test_dense_tensor_core_routing_and_methods():
    """FP32 ETD35 / ETD34 / IF34 with a 2-D lin_op and the built-in Allen-Cahn nonlinearity
    go to the tensor-core batch kernel (the per-instance controller); FP64, other methods
    and other nonlinearities stay on the eigenbasis path.  The lockstep controller runs ETD35
    only; methods outside the kernel are refused before any device work."""
    from rkstiff_gb300 import DeviceOptions
    from rkstiff_gb300._backend import DenseBackend
    from rkstiff_gb300.dense import DenseEnsemble

    x, D = P.cheb(20)
    lin, nl = models.allen_cahn_ops(x, D, 0.01)
    fp32 = DeviceOptions(precision="fp32")
    for cls in (rk.ETD35, rk.ETD34, rk.IF34):
        assert DenseBackend.takes(cls(lin, nl, device_options=fp32))
        assert not DenseBackend.takes(cls(lin, nl))
        assert not DenseBackend.takes(cls(lin, lambda u: u, device_options=fp32))
    assert not DenseBackend.takes(rk.IF4(lin, nl, device_options=fp32))
    for method, controller in (("IF34", "lockstep"), ("ETD34", "lockstep"), ("IF45DP", "instance"),
                               ("ETD4", "instance")):
        with pytest.raises(NotImplementedError):
            DenseEnsemble(lin, nl, 4, method=method, controller=controller)
