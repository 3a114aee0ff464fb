"""Device-side options shared by all solvers (not part of the reference API)."""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Union

import torch


@dataclass
class DeviceOptions:
    """How a solver runs on the GPU.

    precision : 'fp64' (complex128 stages, the reference's arithmetic) or 'fp32'
                (complex64 stages and FFTs; coefficients still built in FP64, error norm
                accumulated in FP64, time kept in FP64)
    device    : CUDA device (default: the current one)
    threads   : threads per instance group (0: the kernel default, 256)
    snap_cap  : snapshots the device buffers hold before the host drains them
    dense_psi : for a 2-D lin_op with diagonalize=False: 'exact' (default) applies the
                psi-functions of the eigenvalues; 'contour' reproduces the reference's own
                psi-matrices, its mean of r psi(r) (rI - cZ)^-1 over a contour centred at 0
                (etd35.py:602-658), whose error grows with |h eig| beyond the radius
    stream_snapshots : stream the snapshots of evolve through a pinned, mapped host ring
                while the launch runs (one launch to tf, no device snapshot buffer)
    snapshot_file : path of an .npz file (arrays t and u) the streamed snapshots are
                written to, including the initial state; solver.u then stays empty
                (solver.t still lists the times).  Implies stream_snapshots.
    """

    precision: str = "fp64"
    device: Optional[Union[str, torch.device]] = None
    threads: int = 0
    snap_cap: int = 256
    dense_psi: str = "exact"
    stream_snapshots: bool = False
    snapshot_file: Optional[str] = None
