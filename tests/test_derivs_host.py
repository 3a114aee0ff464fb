"""Host-side argument checks of the device grid and derivative helpers: the reference's
exceptions (rkstiff/derivatives.py:47-253, rkstiff/grids.py:40-219) are raised before any
device work, so these run without a GPU."""

import numpy as np
import pytest

from rkstiff_gb300 import derivatives as dv
from rkstiff_gb300 import grids


def test_dx_rfft_checks():
    with pytest.raises(TypeError):
        dv.dx_rfft(np.array([0.0, 1.0]), np.array([1.0, 2.0, 3.0]) * (1 + 1j))
    with pytest.raises(TypeError):
        dv.dx_rfft(np.zeros(3), np.ones(4), n=1.5)
    with pytest.raises(ValueError):
        dv.dx_rfft(np.zeros(3), np.ones(4), n=-1)
    with pytest.raises(ValueError):
        dv.dx_rfft(np.array([0.0, 1.0]), np.array([1.0, 2.0, 3.0, 4.0]))
    out = dv.dx_rfft(np.array([]), np.array([]))
    assert isinstance(out, np.ndarray) and out.size == 0
    arr = np.arange(8.0)
    np.testing.assert_array_equal(dv.dx_rfft(np.fft.rfftfreq(8, d=1.0), arr, n=0), arr)


def test_dx_fft_checks():
    kx = np.array([0.0, 1.0, 2.0])
    u = np.array([1.0, 2.0, 3.0])
    np.testing.assert_array_equal(dv.dx_fft(kx, u, n=0), u)
    with pytest.raises(ValueError):
        dv.dx_fft(kx, u, n=-1)
    with pytest.raises(TypeError):
        dv.dx_fft(kx, u, n=1.5)
    with pytest.raises(TypeError):
        dv.dx_fft(kx, u, n="second")
    with pytest.raises(ValueError):
        dv.dx_fft(np.array([0.0, 1.0]), u)


def test_dx_cheb_checks():
    u = np.array([1.0, 2.0, 3.0])
    np.testing.assert_array_equal(dv.dx_cheb(np.eye(3), u, n=0), u)
    with pytest.raises(ValueError):
        dv.dx_cheb(np.eye(3, 4), np.array([1.0, 2.0, 3.0, 4.0]))
    with pytest.raises(ValueError):
        dv.dx_cheb(np.eye(3), np.ones((2, 3, 4)))
    with pytest.raises(ValueError):
        dv.dx_cheb(np.eye(3), np.ones(4))
    with pytest.raises(TypeError):
        dv.dx_cheb(np.eye(3), u, n=2.0)


def test_device_grid_checks():
    with pytest.raises(ValueError):
        grids.construct_x_kx_rfft(7, device="cuda")
    with pytest.raises(TypeError):
        grids.construct_x_kx_fft("10", device="cuda")
    with pytest.raises(ValueError):
        grids.construct_x_dx_cheb(1, device="cuda")
