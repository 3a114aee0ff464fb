"""rk_evolve_noalloc: the entry point for callers that cannot allocate device memory
(code running inside someone else's stream capture, plugins whose host owns every device
allocation, hosts that forbid allocation after start-up).  It must give the same states as
rk_evolve with caller-allocated scratch, call after call, although every call shares the
library's one scratch array and finds there whatever the previous call left.  The
reference here is rk_evolve with one launch over all instances (n_classes = 0), which runs
the same runtime-size kernel, so the two agree bit for bit.  This file is collected last so
that a failure here stops a run only after every other test has run."""

import ctypes

import numpy as np
import pytest
import torch

import bench
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models
from rkstiff_gb300.ensemble import Ensemble
from rkstiff_gb300.solveras import SolverConfig

pytestmark = pytest.mark.gpu

TF = 0.5


def _instances(seed, sizes):
    inst = bench.make_instances(64, seed)
    out = []
    for n, count in sizes:
        out += [i for i in inst if i[0] == n][:count]
    return out


def _ensemble(inst, precision):
    lins, nls, u0s = [], [], []
    for n, L, u0 in inst:
        kx, lin = bench.ks_operator(n, L)
        lins.append(lin)
        nls.append(models.ks_ops(kx)[1])
        u0s.append(u0)
    return Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=1e-5), precision=precision), u0s


def _batch(eng, u_dev, state_dev, with_scratch):
    """The rk_batch of one launch over all instances (no per-size class split); with_scratch
    adds the engine's own slab, slab offsets and queue (what rk_evolve needs)."""
    b = nat.RkBatch()
    b.method = eng.method
    b.precision = eng.prec
    b.coef_complex = eng.coef_complex
    b.nl_kind = eng.nl_kind
    b.nl_coef = eng.nl_coef
    b.n_inst = eng.n_inst
    b.n_max = int(eng.ns.max())
    b.n = eng.n_dev.data_ptr()
    b.mode_off = eng.off_dev.data_ptr()
    b.order = eng.order_dev.data_ptr()
    b.lin_op = eng.lin_dev.data_ptr()
    b.kx = eng.kx_dev.data_ptr()
    b.u = u_dev.data_ptr()
    b.state = state_dev.data_ptr()
    b.twiddle = eng.tw.data_ptr()
    b.max_steps = 200_000
    b.run_mode = nat.RK_RUN_EVOLVE
    b.ctl = eng.ctl
    b.etd = eng.etd
    b.placement = nat.RK_PLACE_AUTO
    b.n_classes = 0
    if with_scratch:
        b.slab = eng.slab.data_ptr()
        b.slab_off = eng.slab_off_dev.data_ptr()
        b.queue = eng.queue.data_ptr()
    return b


def _run(lib, eng, u0, entry):
    """One evolve from u0 over [0, TF] through `entry` ("rk_evolve" or "rk_evolve_noalloc");
    returns (final spectra, state records)."""
    u = u0.clone()
    st = torch.from_numpy(eng.fresh_state(0.0, TF, TF / 100.0).view(np.uint8)).to(eng.device)
    b = _batch(eng, u, st, with_scratch=(entry == "rk_evolve"))
    rc = getattr(lib, entry)(ctypes.byref(b), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.rk_last_error()
    torch.cuda.synchronize()
    return u.cpu().numpy(), st.cpu().numpy().view(nat.STATE_DTYPE).copy()


def _check_same(got, ref):
    (gu, gs), (ru, rs) = got, ref
    assert np.all(gs["status"] == nat.RK_ST_DONE)
    np.testing.assert_array_equal(gs["attempts"], rs["attempts"])
    np.testing.assert_array_equal(gs["steps"], rs["steps"])
    # the same kernel on the same inputs: equal to the last bit, well inside the 1e-12
    # relative tolerance of the FP64 parity tests
    assert np.array_equal(gu, ru)
    assert np.array_equal(gs["t"], rs["t"])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_matches_rk_evolve_twice(precision):
    lib = nat.load()
    # a different batch goes through the shared scratch array first, so the calls below
    # find its slabs and queue counters there
    other, other_u0 = _ensemble(_instances(29, [(512, 5), (256, 2)]), precision)
    _run(lib, other.engine, other.engine.pack_u(other_u0), "rk_evolve_noalloc")
    ens, u0s = _ensemble(_instances(13, [(256, 4), (512, 3)]), precision)
    eng = ens.engine
    u0 = eng.pack_u(u0s)
    ref = _run(lib, eng, u0, "rk_evolve")
    assert np.all(ref[1]["status"] == nat.RK_ST_DONE)
    first = _run(lib, eng, u0, "rk_evolve_noalloc")
    second = _run(lib, eng, u0, "rk_evolve_noalloc")
    _check_same(first, ref)
    _check_same(second, ref)
    # and the per-size class launches of the ordinary path agree to rounding
    cls = torch.cat(ens.evolve(u0s, 0.0, TF)).cpu().numpy()
    tol = 1e-9 if precision == "fp64" else 1e-5
    assert np.linalg.norm(first[0] - cls) / np.linalg.norm(cls) < tol


def test_noalloc_rejects_oversize_batch_before_launch():
    lib = nat.load()
    ens, u0s = _ensemble(_instances(13, [(256, 2)]), "fp64")
    eng = ens.engine
    u = eng.pack_u(u0s)
    # records for every instance the call is told about (only the size check stands between
    # the call and its launches, and it rejects: 13 FP64 ETD35 slabs of n_max 4096 fit)
    st0 = np.concatenate([eng.fresh_state(0.0, TF, TF / 100.0)] * 500)
    st = torch.from_numpy(st0.view(np.uint8).copy()).to(eng.device)
    b = _batch(eng, u, st, with_scratch=False)
    b.n_max = 4096
    b.n_inst = 1_000
    rc = lib.rk_evolve_noalloc(ctypes.byref(b), None)
    assert rc == nat.RK_E_SIZE
    assert b"scratch" in lib.rk_last_error()
    torch.cuda.synchronize()
    # nothing ran: the state records (h_coeff included) are as they were
    assert np.array_equal(st.cpu().numpy(), st0.view(np.uint8))
