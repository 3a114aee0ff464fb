"""rk_evolve_noalloc: the entry point for callers that cannot allocate device memory
(code running inside someone else's stream capture, plugins whose host owns every device
allocation, hosts that forbid allocation after start-up).  It must give the same states as
rk_evolve with caller-allocated scratch, call after call, although every call shares the
library's one scratch array.  This file is collected last so that a failure here stops a
run only after every other test has run."""

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


def _instances():
    inst = bench.make_instances(48, 13)
    out = [i for i in inst if i[0] == 256][:4] + [i for i in inst if i[0] == 512][:3]
    return out


def _ensemble(inst):
    lins, nls, u0s = [], [], []
    for n, L, u0 in inst:
        kx, lin = bench.ks_operator(n, L)
        lins.append(lin)
        nls.append(models.ks_ops(kx)[1])
        u0s.append(u0)
    return Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=1e-5), precision="fp64"), u0s


def _noalloc_batch(eng, u_dev, state_dev):
    """The rk_batch the engine would build, without slab, slab offsets or queue."""
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
    return b


def test_noalloc_matches_rk_evolve_twice():
    lib = nat.load()
    inst = _instances()
    ens, u0s = _ensemble(inst)
    eng = ens.engine
    ref = torch.cat(ens.evolve(u0s, 0.0, 0.5)).cpu().numpy()
    ref_state = ens.state.copy()
    assert np.all(ref_state["status"] == nat.RK_ST_DONE)
    u0 = eng.pack_u(u0s)
    h0 = 0.5 / 100.0
    results = []
    for _ in range(2):
        u = u0.clone()
        st = torch.from_numpy(eng.fresh_state(0.0, 0.5, h0).view(np.uint8)).to(eng.device)
        b = _noalloc_batch(eng, u, st)
        rc = lib.rk_evolve_noalloc(ctypes.byref(b), torch.cuda.current_stream().cuda_stream)
        assert rc == 0, lib.rk_last_error()
        torch.cuda.synchronize()
        got_state = st.cpu().numpy().view(nat.STATE_DTYPE)
        assert np.all(got_state["status"] == nat.RK_ST_DONE)
        np.testing.assert_array_equal(got_state["attempts"], ref_state["attempts"])
        got = u.cpu().numpy()
        # FP64: the two entry points run different FFT kernels (compile-time radix-16 per
        # size class vs one runtime radix-4 launch), so agreement is to rounding only
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9
        results.append(got)
    assert np.array_equal(results[0], results[1])


def test_noalloc_rejects_oversize_batch():
    lib = nat.load()
    b = nat.RkBatch()
    b.method = nat.RK_ETD35
    b.precision = nat.RK_FP64
    b.nl_kind = nat.RK_NL_UUX
    b.n_inst = 100_000
    b.n_max = 2048
    dummy = torch.zeros(1, dtype=torch.uint8, device="cuda")
    b.state = dummy.data_ptr()
    rc = lib.rk_evolve_noalloc(ctypes.byref(b), None)
    assert rc == -4  # RK_E_SIZE
    assert b"scratch" in lib.rk_last_error()
