"""Dense ETD35 with a per-instance controller (rk_dense_eig_evolve): every instance under the
reference's accept/reject rule with its own h, stages in the eigenbasis, basis changes as
3xTF32 tensor-core GEMMs.

Tolerances (the same FP32-stage bounds as the lockstep path):
  * one attempt against the oracle's FP64 step (non-diagonal ETD35 with eigenbasis
    psi-matrices, or its diagonalized form for the eigenbasis error vector): 5e-6 relative
    L2; s and the next h within 2e-3 relative (the error combination cancels to ~1e-5 of the
    stage values, so FP32 stages move s by ~1e-3)
  * instances are independent: a 130-instance batch (three tiles, the last padded) gives
    every instance bitwise the state and counters of that instance run alone
  * Allen-Cahn n=20 to t=10 per instance against the oracle: 5e-4, attempts within 2
  * the Allen-Cahn config (128 interior points) on 512 ICs to tf=70 against per-IC FP64 runs
    at eps=1e-8: 2e-3 (the run's own tolerance is eps=1e-4)
"""

import numpy as np
import pytest

from oracle import rk_oracle as O
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models
from rkstiff_gb300.dense import DenseEnsemble
from rkstiff_gb300.solveras import SolverConfig
import problems as P

pytestmark = pytest.mark.gpu


def ac_ops(n):
    x, D = P.cheb(n)
    return x, models.allen_cahn_ops(x, D, 0.01)


def ics(count, seed, xi, amp=0.1):
    rng = np.random.default_rng(seed)
    base = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi)
    noise = amp * rng.standard_normal((count, xi.size))
    k = np.ones(5) / 5.0
    sm = np.stack([np.convolve(r, k, mode="same") for r in noise])
    return base[None, :] + sm - xi[None, :]


@pytest.mark.parametrize("err_basis", ["physical", "eigen"])
def test_one_attempt_matches_oracle(err_basis):
    x, (lin, nl) = ac_ops(129)
    xi = x[1:-1]
    w0 = ics(1, 3, xi, 0.05)[0]
    h = 0.05
    ens = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-3), controller="instance", err_basis=err_basis)
    u = ens.pack_u(w0[None, :])
    ens.put_state(ens.fresh_state(0.0, 10.0, h))
    st = ens.run(u, 1)
    assert int(st["attempts"][0]) == 1 and int(st["steps"][0]) == 1
    s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-3), dense_psi="eig",
                       diagonalize=err_basis == "eigen")
    s.reset()
    unew, h_used, h_next = s.step(w0.astype(np.complex128), h)
    got = u.cpu().numpy()[0].astype(np.float64)
    err = np.linalg.norm(got - unew.real) / np.linalg.norm(unew.real)
    print(f"instance controller, one attempt ({err_basis} error) vs FP64 oracle: rel L2 {err:.3e}, "
          f"s {float(st['s_last'][0]):.6f} vs {s.log[0][2]:.6f}")
    assert err <= 5e-6
    assert abs(float(st["s_last"][0]) - s.log[0][2]) <= 2e-3 * s.log[0][2]
    assert abs(float(st["h"][0]) - h_next) <= 2e-3 * h_next


def test_instances_are_independent():
    x, (lin, nl) = ac_ops(64)
    xi = x[1:-1]
    w0 = ics(130, 11, xi)
    many = DenseEnsemble(lin, nl, 130, config=SolverConfig(epsilon=1e-4), controller="instance")
    um = many.evolve(w0, 0.0, 5.0).cpu().numpy()
    sm = many.stats()
    assert np.all(sm["status"] == nat.RK_ST_DONE)
    assert len(set(sm["attempts"].tolist())) > 1  # the instances do take different paths
    for i in (0, 63, 64, 129):
        one = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-4), controller="instance")
        u1 = one.evolve(w0[i][None, :], 0.0, 5.0).cpu().numpy()
        s1 = one.stats()
        np.testing.assert_array_equal(um[i], u1[0])
        for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates"):
            assert sm[k][i] == s1[k][0], (i, k)


def test_allen_cahn_n20_per_instance_against_oracle(golden):
    g = golden("dense")
    x, (lin, nl) = ac_ops(20)
    w0 = g["ac20_w0"]
    batch = np.stack([w0, w0 * 0.9, w0 * 1.1])
    ens = DenseEnsemble(lin, nl, 3, config=SolverConfig(epsilon=1e-4), controller="instance")
    out = ens.evolve(batch, 0.0, 10.0).cpu().numpy().astype(np.float64)
    st = ens.stats()
    for i in range(3):
        s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-4), dense_psi="eig")
        ref = s.evolve(batch[i].astype(np.complex128), 0.0, 10.0, store_data=False).real
        err = np.linalg.norm(out[i] - ref) / np.linalg.norm(ref)
        print(f"instance {i}: rel L2 {err:.3e}, attempts {st['attempts'][i]} vs {s.attempts}")
        assert abs(int(st["attempts"][i]) - s.attempts) <= 2
        assert err <= 5e-4
        assert st["status"][i] == nat.RK_ST_DONE and abs(st["t"][i] - 10.0) < 1e-12


def test_config5_sample_against_tight_fp64():
    x, (lin, nl) = ac_ops(129)
    xi = x[1:-1]
    w0 = ics(512, 5, xi)
    ens = DenseEnsemble(lin, nl, 512, config=SolverConfig(epsilon=1e-4), controller="instance")
    out = ens.evolve(w0, 0.0, 70.0).cpu().numpy().astype(np.float64)
    st = ens.stats()
    assert np.all(st["status"] == nat.RK_ST_DONE)
    for i in (0, 1, 255, 511):
        s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-8), diagonalize=True)
        ref = s.evolve(w0[i].astype(np.complex128), 0.0, 70.0, store_data=False).real
        err = np.linalg.norm(out[i] - ref) / np.linalg.norm(ref)
        print(f"config-5 instance {i}: rel L2 vs FP64 eps=1e-8 {err:.3e} (attempts {st['attempts'][i]})")
        assert err <= 2e-3, (i, err)


def test_calls_continue_bitwise():
    """A run split into calls of a few attempts each (the state and N1 carried in the work
    buffer between calls) gives bitwise the run of one call."""
    x, (lin, nl) = ac_ops(64)
    xi = x[1:-1]
    w0 = ics(70, 2, xi)
    one = DenseEnsemble(lin, nl, 70, config=SolverConfig(epsilon=1e-4), controller="instance")
    u1 = one.evolve(w0, 0.0, 3.0).cpu().numpy()
    s1 = one.stats()
    split = DenseEnsemble(lin, nl, 70, config=SolverConfig(epsilon=1e-4), controller="instance")
    u = split.pack_u(w0)
    split.put_state(split.fresh_state(0.0, 3.0, 0.03))
    calls = 0
    while True:
        st = split.run(u, 7)
        calls += 1
        if not np.any(st["status"] == nat.RK_ST_RUNNING):
            break
        assert calls < 1000
    assert calls > 3
    np.testing.assert_array_equal(u.cpu().numpy(), u1)
    for k in ("steps", "attempts", "rejects", "nl_evals", "coeff_updates"):
        np.testing.assert_array_equal(st[k], s1[k])
