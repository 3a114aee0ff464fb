"""Spectral derivatives on the GPU: ``dx_rfft``, ``dx_fft`` and ``dx_cheb`` of
rkstiff/derivatives.py:47-253, with the reference's signatures, argument checks and
exceptions.

The arithmetic runs in FP64 in the library's kernels (``rk_dx_fourier``: one row per block,
shared-memory FFTs for power-of-two sizes and direct transforms over the n roots of unity
otherwise; ``rk_dx_cheb``: D^n by repeated products, then D^n u).  A CUDA tensor in gives a
CUDA tensor out, so that set-up code can stay on the device; NumPy arrays in give NumPy
arrays out, as the reference does.  There is no CPU fallback: without a GPU these functions
raise.  Extension: a 2-D ``u`` of real or complex rows is differentiated row by row
(``kx`` then matches one row).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .engine import _dev, stream_handle, twiddles

MAX_N = 4096


def _check_order(n):
    if not isinstance(n, (int, np.integer)) or isinstance(n, bool):
        raise TypeError(f"derivative order n must be an integer, it is {n}")
    if n < 0:
        raise ValueError(f"derivative order n must be non-negative, it is {n}")


def _to_device(a, dtype, device):
    if isinstance(a, torch.Tensor):
        return a.detach().to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.dtype(str(dtype).split(".")[-1]))).to(
        device)


def _is_complex(u) -> bool:
    return u.is_complex() if isinstance(u, torch.Tensor) else np.iscomplexobj(u)


def _shape(a):
    return tuple(a.shape)


def _device_of(*arrays):
    for a in arrays:
        if isinstance(a, torch.Tensor) and a.is_cuda:
            return a.device
    return None


def _out(t: torch.Tensor, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


def _fourier(kx, u, n, real_grid):
    dev = _dev(_device_of(u, kx))
    npts = int(_shape(u)[-1])
    rows = int(np.prod(_shape(u)[:-1])) if len(_shape(u)) > 1 else 1
    if npts > MAX_N:
        raise ValueError(f"grids of more than {MAX_N} points are not supported on the device")
    dt = torch.float64 if real_grid else torch.complex128
    ud = _to_device(u, dt, dev).reshape(rows, npts)
    kd = _to_device(kx, torch.float64, dev).reshape(-1)
    out = torch.empty_like(ud)
    lib = nat.load()
    tw = twiddles(dev, nat.RK_FP64)
    with torch.cuda.device(dev):
        nat.check(lib.rk_dx_fourier(1 if real_grid else 0, int(n), npts, rows, kd.data_ptr(), ud.data_ptr(),
                                    out.data_ptr(), tw.data_ptr(), stream_handle(dev)), "rk_dx_fourier")
    return _out(out.reshape(_shape(u)), u)


def dx_rfft(kx, u, n: int = 1):
    """n-th derivative of real samples u by the real FFT: irfft((i kx)^n rfft(u))
    (rkstiff/derivatives.py:47-124); kx has len(u)//2 + 1 entries."""
    _check_order(n)
    if _is_complex(u):
        raise TypeError("dx_rfft requires real-valued input. Use dx_fft for complex arrays.")
    if int(np.prod(_shape(u))) == 0:
        return torch.empty(0, dtype=torch.float64, device=u.device) if isinstance(u, torch.Tensor) \
            else np.array([], dtype=float)
    if n == 0:
        return u
    m = _shape(u)[-1] // 2 + 1
    if _shape(kx) != (m,):
        raise ValueError(
            f"kx shape {_shape(kx)} does not match rFFT output shape {(m,)}. "
            "For input size N, kx should have size N//2 + 1.")
    return _fourier(kx, u, n, True)


def dx_fft(kx, u, n: int = 1):
    """n-th derivative of samples u by the complex FFT: ifft((i kx)^n fft(u))
    (rkstiff/derivatives.py:126-180); kx has len(u) entries."""
    _check_order(n)
    if n == 0:
        return u
    if _shape(kx) != (_shape(u)[-1],):
        raise ValueError(f"kx shape {_shape(kx)} must match FFT output {(_shape(u)[-1],)}")
    return _fourier(kx, u, n, False)


def dx_cheb(d_cheb_matrix, u, n: int = 1):
    """n-th derivative D^n u with a Chebyshev differentiation matrix D
    (rkstiff/derivatives.py:182-253); u of shape (N,) or (N, M)."""
    _check_order(n)
    if n == 0:
        return u
    D_shape, u_shape = _shape(d_cheb_matrix), _shape(u)
    if len(D_shape) == 1 and len(u_shape) == 2 and n == 1 and u_shape[0] == u_shape[1] == D_shape[0]:
        # the reference's matmul also takes a vector on the left (d @ u, as its own test
        # tests/test_derivatives_cheb.py:38-43 does): that is u^T d
        return dx_cheb(u.T if isinstance(u, np.ndarray) else u.transpose(0, 1), d_cheb_matrix, 1)
    if len(u_shape) == 1:
        if len(D_shape) != 2 or D_shape[0] != D_shape[1]:
            raise ValueError("d_cheb_matrix must be square.")
        if D_shape[0] != u_shape[0]:
            raise ValueError("Shape mismatch: d_cheb_matrix and u must align in the first dimension.")
    elif len(u_shape) == 2:
        if D_shape[0] != u_shape[0]:
            raise ValueError("Shape mismatch: d_cheb_matrix and u must align in the first dimension.")
        if len(D_shape) != 2 or D_shape[0] != D_shape[1]:
            raise ValueError("d_cheb_matrix must be square.")
    else:
        raise ValueError(f"u must be 1D or 2D, got shape {u_shape}")
    if _is_complex(u) or _is_complex(d_cheb_matrix):
        raise TypeError("dx_cheb on the device takes real (float64) matrices and samples")
    dev = _dev(_device_of(u, d_cheb_matrix))
    N = int(D_shape[0])
    cols = 1 if len(u_shape) == 1 else int(u_shape[1])
    Dd = _to_device(d_cheb_matrix, torch.float64, dev)
    ud = _to_device(u, torch.float64, dev).reshape(N, cols)
    out = torch.empty((N, cols), dtype=torch.float64, device=dev)
    lib = nat.load()
    work = torch.empty(max(1, int(lib.rk_dx_cheb_work_bytes(N))), dtype=torch.uint8, device=dev) if n > 1 else None
    with torch.cuda.device(dev):
        nat.check(lib.rk_dx_cheb(int(n), N, cols, Dd.data_ptr(), ud.data_ptr(), out.data_ptr(),
                                 work.data_ptr() if work is not None else None, stream_handle(dev)), "rk_dx_cheb")
    return _out(out.reshape(u_shape), u)
