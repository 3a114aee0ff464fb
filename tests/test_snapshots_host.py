"""The .npz snapshot writer on the host (no GPU): the archive holds t and u exactly as
appended, and np.load reads it."""

import numpy as np
import pytest

from rkstiff_gb300.snapshots import NpzSnapshotWriter


def test_npz_writer_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    us = [rng.standard_normal(33) + 1j * rng.standard_normal(33) for _ in range(17)]
    ts = np.cumsum(rng.uniform(0.01, 0.1, 17))
    path = tmp_path / "snaps.npz"
    with NpzSnapshotWriter(path) as w:
        for t, u in zip(ts, us):
            w.append(t, u)
    d = np.load(path)
    assert np.array_equal(d["t"], ts)
    assert d["u"].shape == (17, 33) and d["u"].dtype == np.complex128
    assert np.array_equal(d["u"], np.array(us))
    assert not list(tmp_path.glob("rk_snap_*"))  # the temporary state file is gone


def test_npz_writer_rejects_ragged(tmp_path):
    w = NpzSnapshotWriter(tmp_path / "x.npz")
    w.append(0.0, np.zeros(4, np.complex64))
    with pytest.raises(ValueError):
        w.append(1.0, np.zeros(5, np.complex64))
    w.close()
    d = np.load(tmp_path / "x.npz")
    assert d["u"].shape == (1, 4) and d["u"].dtype == np.complex64
