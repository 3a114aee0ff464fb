"""GPU: snapshots streamed through the pinned, mapped host ring while the launch runs
(DeviceOptions(stream_snapshots=True) / snapshot_file=...), against the buffered path and
the reference's own snapshot times (rkstiff/solveras.py:643-646)."""

import ctypes

import numpy as np
import pytest
import torch

import problems as P
import rkstiff_gb300 as rk
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models
from rkstiff_gb300.ensemble import Ensemble
from rkstiff_gb300.snapshots import SnapshotRing, SnapshotStreamOverrun

pytestmark = pytest.mark.gpu


def _config1():
    x, kx = rk.grids.construct_x_kx_rfft(1024, 0.0, 32 * np.pi)
    lin, nl = models.ks_ops(kx)
    u0 = np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16)))
    return lin, nl, u0


def test_config1_every_step_streamed_in_one_launch():
    """Every accepted step's snapshot of config 1 (567 attempts) streamed in one launch:
    the same times and states, bit for bit, as the buffered path run in one launch (a device
    buffer of 1024 snapshots)."""
    lin, nl, u0 = _config1()
    a = rk.IF34(lin, nl, device_options=rk.DeviceOptions(snap_cap=1024))
    ua = a.evolve(u0, 0.0, 50.0, store_freq=1)
    assert a._engine().ens.launches == 1
    b = rk.IF34(lin, nl, device_options=rk.DeviceOptions(stream_snapshots=True))
    ub = b.evolve(u0, 0.0, 50.0, store_freq=1)
    assert b._engine().ens.launches == 1
    assert b.stats["steps"] + 1 == len(b.t)
    assert b.t == a.t  # bit-equal times
    assert len(b.u) == len(a.u) and all(np.array_equal(p, q) for p, q in zip(a.u, b.u))
    assert np.array_equal(ua, ub)


def test_config1_stream_matches_reference_times(golden):
    g = golden("adaptive")
    lin, nl, u0 = _config1()
    s = rk.IF34(lin, nl, device_options=rk.DeviceOptions(stream_snapshots=True))
    s.evolve(u0, 0.0, 50.0, store_freq=20)
    np.testing.assert_allclose(s.t, g["ks1024_IF34_t"], rtol=1e-10)
    assert np.linalg.norm(s.u[5] - g["ks1024_IF34_u5"]) / np.linalg.norm(g["ks1024_IF34_u5"]) < 1e-8


def test_snapshot_file(tmp_path):
    lin, nl, u0 = _config1()
    a = rk.IF34(lin, nl)
    a.evolve(u0, 0.0, 10.0, store_freq=3)
    path = tmp_path / "ks.npz"
    b = rk.IF34(lin, nl, device_options=rk.DeviceOptions(snapshot_file=str(path)))
    b.evolve(u0, 0.0, 10.0, store_freq=3)
    d = np.load(path)
    assert b.u == [] and b.t == a.t
    assert np.array_equal(d["t"], np.array(a.t))
    assert np.array_equal(d["u"], np.array(a.u))


def test_ensemble_stream_per_instance():
    inst = [P.ks(n, L) for n, L in ((256, 30.0), (512, 50.0), (256, 22.0))]
    lins = [p[2] for p in inst]
    nls = [models.ks_ops(p[1])[1] for p in inst]
    u0s = [np.fft.rfft(np.cos(2 * np.pi * p[0] / L)) for p, L in zip(inst, (30.0, 50.0, 22.0))]
    ens = Ensemble("ETD35", lins, nls, config=rk.SolverConfig(epsilon=1e-5))
    eng = ens.engine
    # buffered reference
    got_buf = {i: [] for i in range(3)}

    def on_snaps(st, su, stt):
        from rkstiff_gb300.engine import snapshot_views
        for i in range(3):
            ts, us = snapshot_views(eng, st, su, stt, i)
            got_buf[i] += [(float(t), u.cpu().numpy()) for t, u in zip(ts, us)]

    u = eng.pack_u(u0s)
    eng.evolve(u, 0.0, 5.0, 0.05, store_freq=2, snap_cap=8, on_snapshots=on_snaps)
    ub = u.cpu().numpy()
    got = {i: [] for i in range(3)}
    u = eng.pack_u(u0s)
    eng.evolve_stream(u, 0.0, 5.0, 0.05, 2, lambda i, t, step, uu: got[i].append((t, uu)), slots=4)
    assert np.array_equal(u.cpu().numpy(), ub)
    for i in range(3):
        assert [t for t, _ in got[i]] == [t for t, _ in got_buf[i]]
        assert all(np.array_equal(p, q) for (_, p), (_, q) in zip(got[i], got_buf[i]))


def test_ring_wait_runs_out_and_pauses():
    """A ring of one slot that the host does not drain during the launch: the second
    snapshot's bounded wait runs out (1 ms), the instance pauses with RK_ST_SNAP_FULL, and the
    drain reports the overrun."""
    lin, nl, u0 = _config1()
    ens = Ensemble("IF34", [lin], [nl])
    eng = ens.engine
    ring = SnapshotRing(1, int(eng.ms.max()), eng.prec, timeout_ms=1)
    try:
        u = eng.pack_u([u0])
        eng.put_state(eng.fresh_state(0.0, 50.0, 0.5))
        eng.launch(u, nat.RK_RUN_EVOLVE, store_freq=1, ring=ring)
        torch.cuda.synchronize()
        st = eng.get_state()
        assert int(st["status"][0]) == nat.RK_ST_SNAP_FULL
        assert int(st["steps"][0]) == 2  # the first snapshot went out, the second did not
        assert ring.claimed() == 2
        with pytest.raises(SnapshotStreamOverrun):
            ring.drain(lambda: True, eng.ms, lambda *a: None)
    finally:
        ring.close()
