"""Learned step-size controller on the GPU: the CUDA training kernels against the NumPy
FP64 oracle, the BF16 inference fused into the evolve kernel replayed from its attempt
log, a short training run, and the gain of the shipped controller over the plain one.

Tolerances:
  * forward / gradient of the FP32 CUDA kernels vs the FP64 oracle: 2e-5 relative
  * one Adam update: 1e-6 of the magnitude of each moment update's terms; the parameter
    step to 1e-4 of itself (FP32 bias correction)
  * the in-kernel step factor vs the oracle forward with the same BF16-rounded weights:
    |log h_{k+1}/h_k - expected| <= 2e-3 (FP32 features and activation differences)
"""

import math

import numpy as np
import pytest
import torch

from oracle import mlp as MO
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import workloads
from rkstiff_gb300.controller import LearnedController, accepted_features, collect_logs
from rkstiff_gb300.ensemble import Ensemble
from rkstiff_gb300.solveras import SolverConfig

pytestmark = pytest.mark.gpu


def _bf16(a):
    return torch.as_tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float32).numpy().astype(np.float64)


@pytest.fixture(scope="module")
def ctl():
    c = LearnedController(seed=11)
    rng = np.random.default_rng(2)
    c.params = torch.as_tensor((c.params.cpu().numpy() + 0.05 * rng.standard_normal(nat.RK_MLP_NPARAM)).astype(np.float32),
                               device=c.device)
    return c


@pytest.mark.parametrize("batch", [1, 63, 300, 4096])
def test_forward_and_gradient_match_oracle(ctl, batch):
    rng = np.random.default_rng(batch)
    X = rng.standard_normal((batch, nat.RK_MLP_IN)).astype(np.float32)
    T = (0.1 * rng.standard_normal(batch)).astype(np.float32)
    Xd = torch.as_tensor(X, device=ctl.device)
    Y = torch.empty(batch, dtype=torch.float32, device=ctl.device)
    nat.check(ctl.lib.rk_mlp_forward(ctl.params.data_ptr(), Xd.data_ptr(), batch, Y.data_ptr(), ctl._stream()), "fwd")
    p64 = ctl.params.cpu().numpy().astype(np.float64)
    y_ref, _ = MO.forward(p64, X.astype(np.float64))
    np.testing.assert_allclose(Y.cpu().numpy(), y_ref, rtol=2e-5, atol=2e-5)
    g, loss = ctl.grad(Xd, torch.as_tensor(T, device=ctl.device), float(batch))
    lo, go = MO.loss_and_grad(p64, X.astype(np.float64), T.astype(np.float64), float(batch))
    assert abs(loss - lo) <= 2e-5 * abs(lo) + 1e-9
    assert np.linalg.norm(g.cpu().numpy() - go) <= 2e-5 * np.linalg.norm(go)


def test_adam_update_matches_numpy(ctl):
    rng = np.random.default_rng(4)
    p = ctl.params.clone()
    g = torch.as_tensor(rng.standard_normal(nat.RK_MLP_NPARAM).astype(np.float32), device=ctl.device)
    m = torch.as_tensor(0.01 * rng.standard_normal(nat.RK_MLP_NPARAM).astype(np.float32), device=ctl.device)
    v = torch.as_tensor(np.abs(0.01 * rng.standard_normal(nat.RK_MLP_NPARAM)).astype(np.float32), device=ctl.device)
    p0, m0, v0, g0 = (t.cpu().numpy().astype(np.float64) for t in (p, m, v, g))
    step, lr, b1, b2, eps = 7, 1e-3, 0.9, 0.999, 1e-8
    nat.check(ctl.lib.rk_mlp_adam(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), step, lr, b1, b2, eps,
                                  ctl._stream()), "adam")
    # the kernel receives the hyper-parameters as FP32
    b1, b2, lr, eps = (float(np.float32(x)) for x in (b1, b2, lr, eps))
    m1 = b1 * m0 + (1 - b1) * g0
    v1 = b2 * v0 + (1 - b2) * g0 * g0
    upd = lr * (m1 / (1 - b1**step)) / (np.sqrt(v1 / (1 - b2**step)) + eps)
    p1 = p0 - upd
    # FP32 rounding of each update, measured against the size of its terms; the bias
    # correction 1 - b2^t cancels in FP32 at small t (about 1e-5 relative at t = 7)
    np.testing.assert_array_less(np.abs(m.cpu().numpy() - m1), 1e-6 * (np.abs(b1 * m0) + np.abs((1 - b1) * g0)) + 1e-12)
    np.testing.assert_array_less(np.abs(v.cpu().numpy() - v1), 1e-6 * (b2 * v0 + (1 - b2) * g0 * g0) + 1e-15)
    np.testing.assert_array_less(np.abs(p.cpu().numpy() - p1), 1e-4 * np.abs(upd) + 1e-6 * np.abs(p0) + 1e-12)


def _burgers_ensemble(count, seed, precision="fp32", eps=1e-5):
    inst = workloads.burgers_ensemble(count, seed)
    e = Ensemble("ETD35", [a[0] for a in inst], [a[1] for a in inst], config=SolverConfig(epsilon=eps),
                 precision=precision)
    return e, [a[2] for a in inst]


def test_fused_inference_replays_from_attempt_log():
    """Every step size the kernel chose after an accept equals h * clamp(exp(log s +
    clamp(y, -1, 1)) / target, 0.5, 4) with y the oracle forward of the logged features."""
    c = LearnedController.pretrained()
    e, u0s = _burgers_ensemble(24, 31)
    tf = 1.0
    log, counts = collect_logs(e, u0s, 0.0, tf, cap=4096, controller=c)
    # weights rounded to BF16 as the packed buffer holds them; biases stay FP32
    _, b1, _, b2, _, b3 = MO.split(c.params.cpu().numpy())
    W1, _, W2, _, w3, _ = MO.split(_bf16(c.params.cpu().numpy()))
    p_mixed = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])
    mu = c.mu.cpu().numpy().astype(np.float64)
    isd = (1.0 / c.sd.cpu().numpy()).astype(np.float32).astype(np.float64)
    checked = 0
    worst = 0.0
    for i in range(log.shape[0]):
        K = int(min(counts[i], log.shape[1]))
        r = log[i, :K].astype(np.float64)
        for k, f in accepted_features(r):
            if k + 1 >= K:
                continue
            t_next, h, h_next = r[k + 1, 0], r[k, 1], r[k + 1, 1]
            if t_next + h_next >= tf * (1 - 1e-6):
                continue  # the step was cut to end at tf
            x = (np.asarray(f, dtype=np.float32).astype(np.float64) - mu) * isd
            y, _ = MO.forward(p_mixed, x[None, :])
            d = min(max(float(y[0]), -1.0), 1.0)
            fac = min(max(math.exp(f[0] + d) / c.target, 0.5), 4.0)
            err = abs(math.log(h_next / h) - math.log(fac))
            worst = max(worst, err)
            checked += 1
    assert checked > 500
    assert worst <= 2e-3, worst


def test_training_run_reduces_loss():
    c = LearnedController(seed=5)
    e, u0s = _burgers_ensemble(48, 77)
    rep = c.train([(e, u0s, 0.0, 2.0)], rounds=2, steps=300)
    r0, r1 = rep["rounds"]
    assert r1["samples"] > r0["samples"] > 1000
    # the fit explains part of the target's variance: at least 20% on the plain controller's
    # logs, at least 10% on the first on-policy round (its logs come from the network itself)
    assert r0["loss"] < 0.8 * r0["var"] and r1["loss"] < 0.9 * r1["var"]
    assert np.all(np.isfinite(c.params.cpu().numpy()))


def test_learned_controller_gain_over_plain():
    """Shipped controller vs the plain rule on 512 Burgers instances the training never saw
    (same epsilon, FP32 stages): fewer NL evaluations and rejected steps on the instances
    both finish, at comparable accuracy against an FP64 run at epsilon = 1e-10."""
    c = LearnedController.pretrained()
    inst = workloads.burgers_ensemble(512, 7)
    res = {}
    for name in ("plain", "learned"):
        e = Ensemble("ETD35", [a[0] for a in inst], [a[1] for a in inst], config=SolverConfig(epsilon=1e-5),
                     precision="fp32")
        if name == "learned":
            c.install(e)
        out = e.evolve([a[2] for a in inst], 0.0, 5.0, max_steps=20000, max_launches=3)
        res[name] = (e.stats(), [o.cpu().numpy() for o in out])
    both = (res["plain"][0]["status"] == 0) & (res["learned"][0]["status"] == 0)
    assert both.sum() > 300
    nl_p = res["plain"][0]["nl_evals"][both].sum()
    nl_l = res["learned"][0]["nl_evals"][both].sum()
    rj_p = res["plain"][0]["rejects"][both].sum()
    rj_l = res["learned"][0]["rejects"][both].sum()
    assert nl_l <= 0.97 * nl_p, (nl_l, nl_p)
    assert rj_l <= rj_p, (rj_l, rj_p)
    idx = np.where(both)[0][::8]
    ref_e = Ensemble("ETD35", [inst[i][0] for i in idx], [inst[i][1] for i in idx],
                     config=SolverConfig(epsilon=1e-10), precision="fp64")
    ref = [o.cpu().numpy() for o in ref_e.evolve([inst[i][2] for i in idx], 0.0, 5.0, max_steps=50000, max_launches=2)]
    med = {}
    for name in res:
        out = res[name][1]
        med[name] = np.median([np.linalg.norm(out[i] - r) / np.linalg.norm(r) for i, r in zip(idx, ref)])
    assert med["learned"] <= 2.0 * med["plain"] + 1e-7, med
    assert med["learned"] <= 2e-6, med


def test_coefficient_block_cache_is_transparent():
    """Four coefficient blocks keyed by h (rk_batch.coef_blocks) under the plain controller:
    the same coefficients are served from the cache instead of rebuilt, so every state and
    counter but the rebuild count is bitwise that of the reference's single-entry cache."""
    inst = workloads.burgers_ensemble(96, 21)
    out, st = {}, {}
    for blocks in (1, 4):
        e = Ensemble("ETD35", [a[0] for a in inst], [a[1] for a in inst], config=SolverConfig(epsilon=1e-5),
                     precision="fp32")
        e.engine.set_coef_cache(blocks)
        out[blocks] = torch.cat(e.evolve([a[2] for a in inst], 0.0, 2.0, max_steps=20000, max_launches=3)).cpu()
        st[blocks] = e.stats()
    assert torch.equal(out[1], out[4])
    for k in ("attempts", "steps", "nl_evals", "status"):
        assert np.array_equal(st[1][k], st[4][k]), k
    assert st[4]["coeff_updates"].sum() <= st[1]["coeff_updates"].sum()


def test_learned_ladder_cuts_coefficient_rebuilds():
    """The learned controller with its steps on the 2^(1/16) ladder and four cached blocks
    per instance rebuilds the coefficients on fewer of its attempts (without the ladder on
    almost every one; measured on this set: 58% of attempts), at nearly the same number of
    NL evaluations."""
    c = LearnedController.pretrained()
    inst = workloads.burgers_ensemble(256, 7)
    st = {}
    for ladder in (False, True):
        e = Ensemble("ETD35", [a[0] for a in inst], [a[1] for a in inst], config=SolverConfig(epsilon=1e-5),
                     precision="fp32")
        c.install(e, ladder=ladder)
        e.evolve([a[2] for a in inst], 0.0, 5.0, max_steps=20000, max_launches=3)
        st[ladder] = e.stats()
    both = (st[False]["status"] == 0) & (st[True]["status"] == 0)
    assert both.sum() > 150
    rebuild = {k: st[k]["coeff_updates"][both].sum() / st[k]["attempts"][both].sum() for k in st}
    assert rebuild[False] > 0.5, rebuild
    assert rebuild[True] < 0.75 * rebuild[False], rebuild
    nl = {k: st[k]["nl_evals"][both].sum() for k in st}
    assert nl[True] <= 1.03 * nl[False], nl
