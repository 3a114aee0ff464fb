"""GPU parity of the batched ensemble path (one launch per grid-size class, compile-time
FFT kernels) against the CPU oracle.

Tolerances (relative L2):
  * FP64 ensembles vs the oracle after a short span: 1e-9 (same accept/reject sequence)
  * FP32 ensembles, one adaptive step from the same state and h: 1e-6
  * FP32 ensembles vs the oracle after a short span (tf = 1): 1e-4
"""

import numpy as np
import pytest
import torch

import bench
from oracle import rk_oracle as O
from rkstiff_gb300 import models
from rkstiff_gb300.ensemble import Ensemble
from rkstiff_gb300.solveras import SolverConfig

pytestmark = pytest.mark.gpu

SIZES = (256, 512, 1024, 2048)


def ks_instances(per_size=3, seed=5):
    inst = bench.make_instances(64, seed)
    out = []
    for n in SIZES:
        out += [i for i in inst if i[0] == n][:per_size]
    return out


def build(inst, precision, eps=1e-5):
    lins, nls, u0s = [], [], []
    for n, L, u0 in inst:
        kx, lin = bench.ks_operator(n, L)
        lins.append(lin)
        nls.append(models.ks_ops(kx)[1])
        u0s.append(u0)
    return Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=eps), precision=precision), u0s


def oracle_run(n, L, u0, tf, eps=1e-5):
    kx, lin = bench.ks_operator(n, L)
    nl = models.ks_ops(kx)[1]
    s = O.OracleSolver("ETD35", lin, lambda u: nl(u), O.SolverConfig(epsilon=eps))
    u = s.evolve(u0, 0.0, tf, store_data=False)
    return u, s


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_ensemble_fp64_matches_oracle():
    inst = ks_instances()
    ens, u0s = build(inst, "fp64")
    out = ens.evolve(u0s, 0.0, 1.0)
    st = ens.stats()
    assert np.all(st["status"] == 0)
    for k, (n, L, u0) in enumerate(inst):
        ref, s = oracle_run(n, L, u0, 1.0)
        assert st["attempts"][k] == s.attempts, (n, L)
        assert rel(out[k].cpu().numpy(), ref) < 1e-9, (n, L)


def test_ensemble_fp32_one_step_and_short_span():
    inst = ks_instances()
    ens, u0s = build(inst, "fp32")
    # one adaptive step from the initial state (tf = h_init so the step is exactly h)
    out = ens.evolve(u0s, 0.0, 0.01, h_init=0.01)
    for k, (n, L, u0) in enumerate(inst):
        kx, lin = bench.ks_operator(n, L)
        nl = models.ks_ops(kx)[1]
        o = O.OracleSolver("ETD35", lin, lambda u: nl(u), O.SolverConfig(epsilon=1e-5))
        ref, h, _ = o.step(u0, 0.01)
        assert h == 0.01
        assert rel(out[k].cpu().numpy(), ref) < 1e-6, (n, L)
    out = ens.evolve(u0s, 0.0, 1.0)
    assert np.all(ens.stats()["status"] == 0)
    for k, (n, L, u0) in enumerate(inst):
        ref, _ = oracle_run(n, L, u0, 1.0)
        assert rel(out[k].cpu().numpy(), ref) < 1e-4, (n, L)


def test_ensemble_placements_agree():
    """Placement choices of a class agree: bit-exactly between the shared-memory variants
    of the same kernel and thread count, to FP32 rounding across thread counts and the
    global-scratch kernel (the controller's reductions then sum in another order)."""
    from rkstiff_gb300 import _native as nat

    inst = ks_instances(per_size=2)
    ens, u0s = build(inst, "fp32")
    eng = ens.engine
    ncls = len(eng.class_n)

    def run(thr, place):
        eng.class_threads = np.full(ncls, thr, dtype=np.int32)
        eng.class_place = np.full(ncls, place, dtype=np.int32)
        return torch.cat(ens.evolve(u0s, 0.0, 0.5)).cpu().numpy()

    a = run(128, nat.RK_PLACE_SMEM_STATE)
    b = run(128, nat.RK_PLACE_SMEM_ALL)
    assert np.array_equal(a, b)
    for thr, place in ((64, nat.RK_PLACE_SMEM_STATE), (256, nat.RK_PLACE_SMEM_STATE), (128, nat.RK_PLACE_GLOBAL),
                       (128, nat.RK_PLACE_SMEM_U), (64, nat.RK_PLACE_SMEM_U)):
        assert rel(run(thr, place), a) < 1e-5, (thr, place)
    eng.class_threads = None
    eng.class_place = None
    eng.class_groups = None


def test_graph_replay_matches_launch():
    """evolve_graph (captured CUDA graph) gives bit-identical states and counters to the
    ordinary launch, also on a replay after the input changed."""
    inst = ks_instances(per_size=3, seed=9)
    ens, u0s = build(inst, "fp32")
    u0 = ens.pack(u0s)
    u = torch.empty_like(u0)
    u.copy_(u0)
    st_ref = ens.evolve_packed(u, 0.0, 5.0)
    ref = u.clone()
    u2 = torch.empty_like(u0)
    for _ in range(2):
        st = ens.evolve_graph(u2, u0, 0.0, 5.0)
        assert torch.equal(u2, ref)
        for k in ("steps", "attempts", "rejects", "nl_evals", "status"):
            np.testing.assert_array_equal(st[k], st_ref[k])
    u0.mul_(0.5)  # new input, same buffers: the replay reads it
    u.copy_(u0)
    ens.evolve_packed(u, 0.0, 5.0)
    ens.evolve_graph(u2, u0, 0.0, 5.0)
    assert torch.equal(u2, u)


def test_longest_first_schedule_keeps_results():
    """The 'history' schedule queues each grid-size class longest-first by the previous
    evolve's attempts; the states and counters are bit-identical to index order."""
    inst = ks_instances(per_size=6, seed=21)
    ens, u0s = build(inst, "fp32")
    eng = ens.engine
    u0 = ens.pack(u0s)
    eng.schedule = "size"
    u_ref = u0.clone()
    st_ref = ens.evolve_packed(u_ref, 0.0, 3.0)
    assert np.array_equal(eng.order_dev.cpu().numpy(), eng._size_order)
    eng.schedule = "history"
    u1 = u0.clone()
    ens.evolve_packed(u1, 0.0, 3.0)  # index order; sets the longest-first order after it
    order = eng.order_dev.cpu().numpy()
    assert not np.array_equal(order, eng._size_order)
    for c in range(len(eng.class_n)):
        idx = order[eng.class_start[c]:eng.class_start[c + 1]]
        assert np.all(eng.ns[idx] == eng.class_n[c])
        assert np.all(np.diff(st_ref["attempts"][idx]) <= 0)
    u2 = u0.clone()
    st2 = ens.evolve_packed(u2, 0.0, 3.0)
    assert torch.equal(u2, u_ref)
    for k in ("steps", "attempts", "rejects", "nl_evals", "status", "t"):
        np.testing.assert_array_equal(st2[k], st_ref[k])
