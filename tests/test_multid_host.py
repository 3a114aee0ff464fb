"""Host side of the multi-dimensional NLS problems (the reference's NLS demo): the Hankel
transform, mirror_grid and the flattened operators / nonlinearities, against the
reference's own values (tests/golden/multid.npz).  Tolerances: 1e-13 relative (FP64, the
same formulas; torch and numpy order the matrix product differently)."""

import numpy as np
import pytest
import torch

import rkstiff_gb300 as rk
from rkstiff_gb300 import models
from rkstiff_gb300.grids import construct_x_kx_fft, mirror_grid
from rkstiff_gb300.transforms import HankelTransform


def rel(a, b):
    a = a.numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_hankel_transform_matches_reference(golden):
    g = golden("multid")
    HT = HankelTransform(nr=16, rmax=4.0)
    for mine, ref in ((HT.r, "ht16_r"), (HT.kr, "ht16_kr"), (HT.hankel_matrix(), "ht16_Y"),
                      (HT.bessel_zeros(), "ht16_zeros")):
        assert rel(mine, g[ref]) < 1e-14, ref
    assert rel(HT.ht(g["ht16_f"]), g["ht16_ht"]) < 1e-14
    assert rel(HT.iht(HT.ht(g["ht16_f"])), g["ht16_iht"]) < 1e-14
    # tensors: the same transform as a GEMM over axis 0, real or complex, 1-D or 2-D
    ft = torch.from_numpy(g["ht16_f"])
    assert rel(HT.ht(ft), g["ht16_ht"]) < 1e-13
    F2 = np.stack([g["ht16_f"], 2j * g["ht16_f"], g["ht16_f"].real], axis=1)
    assert rel(HT.iht(torch.from_numpy(F2)), HT.iht(F2)) < 1e-13
    assert rel(HT.ht(torch.from_numpy(F2[:, 2].real.copy())), HT.ht(F2[:, 2].real)) < 1e-13
    r, u = mirror_grid(HT.r, np.abs(g["ht16_f"]) ** 2)
    np.testing.assert_array_equal(r, g["ht16_mirror_r"])
    np.testing.assert_array_equal(u, g["ht16_mirror_u"])


def test_hankel_setters_validate_and_rebuild():
    HT = HankelTransform(nr=8, rmax=2.0)
    with pytest.raises(ValueError):
        HT.nr = 3
    with pytest.raises(ValueError):
        HT.rmax = 0.0
    with pytest.raises(ValueError):
        rk.grids.construct_r_kr_hankel(3, 1.0)
    HT.nr = 16
    HT.rmax = 4.0
    assert HT.hankel_matrix().shape == (16, 16) and np.isclose(HT.r[-1] / HT.rmax, HT.bessel_zeros()[-1] / HT._jN)
    _ = HT.ht(torch.ones(16, dtype=torch.float64))
    HT.nr = 12  # the cached device matrices follow the new grid
    assert HT.ht(torch.ones(12, dtype=torch.float64)).shape == (12,)


def test_multid_nonlinearities_match_the_demo_closures(golden):
    g = golden("multid")
    gamma = 2.0
    # 2-D
    nx = ny = 32
    x, kx = construct_x_kx_fft(nx, -6, 6)
    _, ky = construct_x_kx_fft(ny, -6, 6)
    L, nl = models.nls_2d_ops(kx, ky, gamma)
    KX, KY = np.meshgrid(kx, ky, indexing="ij")
    np.testing.assert_array_equal(L, (-1j * (KX**2 + KY**2)).flatten())
    u = g["nls2d_final"]
    F = np.fft.ifft2(u.reshape(nx, ny))
    ref = 1j * gamma * np.fft.fft2((F.real**2 + F.imag**2) * F).flatten()
    assert rel(nl(u), ref) < 1e-13
    assert rel(nl(torch.from_numpy(u)), ref) < 1e-13
    # (r, t)
    nr, nt = (int(v) for v in g["rtnls_shape"])
    HT = HankelTransform(nr=nr, rmax=4.0)
    _, om = construct_x_kx_fft(nt, -6, 6)
    L, nl = models.nls_radial_time_ops(HT, om, 0.5, gamma)
    u = g["rtnls_final"]
    F = np.fft.ifft(HT.iht(u.reshape(nr, nt)), axis=1)
    ref = 1j * gamma * np.fft.fft(HT.ht((F.real**2 + F.imag**2) * F), axis=1).flatten()
    assert rel(nl(torch.from_numpy(u)), ref) < 1e-13
    KR, OM = np.meshgrid(HT.kr, om, indexing="ij")
    np.testing.assert_array_equal(L, (-1j * KR**2 + 1j * 0.5 * OM**2).flatten())
    # radial
    HT = HankelTransform(nr=32, rmax=5.0)
    L, nl = models.nls_radial_ops(HT, gamma)
    u = g["hnls_final"]
    f = HT.iht(u)
    assert rel(nl(torch.from_numpy(u)), 1j * gamma * HT.ht((f.real**2 + f.imag**2) * f)) < 1e-13
