"""Dense (non-diagonal) ETD35 on the tensor cores against the reference and the oracle.

Tolerances:
  * 3xTF32 product vs FP64: |D - D64| <= 1e-5 * (|B| |A|^T) elementwise (three TF32
    products with FP32 accumulation over K <= 768; one TF32 product would be ~5e-4)
  * one ETD35 attempt from the same state and h vs the FP64 oracle (the non-diagonal form,
    rkstiff/etd35.py:498-720, with psi-matrices from the eigenbasis, oracle dense_psi="eig"):
    5e-6 relative L2 (measured 2.0e-6: six chained stages of
    3xTF32 products, FP32 accumulation and FP32 stage vectors)
  * Allen-Cahn n=20 (19 interior points), eps=1e-4, vs the same oracle: 5e-4 relative L2 at
    t=10 (FP32 per-step error amplified by the flow), attempts within 2
  * 8192 Allen-Cahn ICs (128 interior points) to tf=70 vs per-IC FP64 oracle runs at
    eps=1e-8 on a sample: 2e-3 relative L2 (the adaptive error at eps=1e-4)
"""

import numpy as np
import pytest
import torch

from oracle import rk_oracle as O
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models
from rkstiff_gb300.dense import DenseEnsemble
from rkstiff_gb300.device import DeviceOptions
from rkstiff_gb300.solveras import SolverConfig
import problems as P

pytestmark = pytest.mark.gpu


def gemm(A, B):
    lib = nat.load()
    K, N = A.shape[1], B.shape[0]
    dev = torch.device("cuda")
    At = torch.as_tensor(A, dtype=torch.float32, device=dev).contiguous()
    Bt = torch.as_tensor(B, dtype=torch.float32, device=dev).contiguous()
    D = torch.empty((N, 128), dtype=torch.float32, device=dev)
    work = torch.empty(int(lib.rk_tf32x3_work_bytes(K, N)), dtype=torch.uint8, device=dev)
    nat.check(lib.rk_tf32x3_gemm(At.data_ptr(), Bt.data_ptr(), D.data_ptr(), K, N, work.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream), "rk_tf32x3_gemm")
    return D.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("K,N", [(32, 64), (128, 64), (384, 256), (768, 128)])
def test_tf32x3_product_matches_fp64(K, N):
    rng = np.random.default_rng(K + N)
    A = rng.standard_normal((128, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    D = gemm(A, B)
    ref = B.astype(np.float64) @ A.astype(np.float64).T
    bound = np.abs(B.astype(np.float64)) @ np.abs(A.astype(np.float64)).T
    assert np.all(np.abs(D - ref) <= 1e-5 * bound), np.max(np.abs(D - ref) / bound)


def test_tf32x3_product_structure():
    # with integer entries (exact in TF32) an identity A returns B exactly and a permutation
    # permutes it
    K, N = 128, 64
    rng = np.random.default_rng(1)
    B = rng.integers(-1000, 1000, size=(N, K)).astype(np.float32)
    np.testing.assert_array_equal(gemm(np.eye(128, K, dtype=np.float32), B), B.astype(np.float64))
    perm = rng.permutation(128)
    np.testing.assert_array_equal(gemm(np.eye(128, dtype=np.float32)[perm], B), B[:, perm].astype(np.float64))


def ac_ops(n):
    x, D = P.cheb(n)
    return x, models.allen_cahn_ops(x, D, 0.01)


def test_one_attempt_matches_oracle():
    x, (lin, nl) = ac_ops(129)
    xi = x[1:-1]
    rng = np.random.default_rng(3)
    w0 = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi) - xi + 0.05 * rng.standard_normal(xi.size)
    h = 0.05
    ens = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-3), controller="lockstep")
    u = ens.pack_u(w0[None, :])
    ens.put_state(ens.fresh_state(0.0, 10.0, h))
    st = ens.run(u, 1)
    assert int(st["attempts"][0]) == 1 and int(st["steps"][0]) == 1  # accepted
    s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-3), dense_psi="eig")
    s.reset()
    unew, h_used, h_next = s.step(w0.astype(np.complex128), h)
    ref = unew.real
    got = u.cpu().numpy()[0].astype(np.float64)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    print(f"dense one-attempt rel L2 vs FP64 oracle: {err:.3e}")
    assert err <= 5e-6
    assert abs(float(st["h"][0]) - h_next) <= 1e-6 * h_next
    assert abs(float(st["s_last"][0]) - s.log[0][2]) <= 1e-5 * s.log[0][2]


def test_allen_cahn_n20_matches_pinned_oracle(golden):
    """The reference's n=20 case (19 interior points, eps=1e-4) against the oracle's
    non-diagonal ETD35 with eigenbasis psi-matrices (pinned in tests/test_oracle_golden.py to
    an augmented-matrix expm and to the reference's own dense arrays).  This flow
    amplifies perturbations (in FP64, a 1e-7 change of w0 grows 3.5x by t=10, 43x by t=30
    and to a different end state by t=60, where a front collapses), so the ~2e-6 per-step
    error of FP32 stages is compared at t=10 (bound 5e-4) and only reported at t=30."""
    g = golden("dense")
    x, (lin, nl) = ac_ops(20)
    np.testing.assert_allclose(lin, g["ac20_lin"], rtol=0, atol=1e-12)
    w0 = g["ac20_w0"]
    errs = {}
    for tf in (10.0, 30.0):
        ens = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-4), controller="lockstep")
        out = ens.evolve(w0[None, :], 0.0, tf).cpu().numpy()[0].astype(np.float64)
        st = ens.stats()
        s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-4), dense_psi="eig")
        ref = s.evolve(w0.astype(np.complex128), 0.0, tf, store_data=False).real
        errs[tf] = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        print(f"dense Allen-Cahn n=20 to t={tf:g} vs oracle: rel L2 {errs[tf]:.3e}, "
              f"attempts {st['attempts']} vs {s.attempts}")
        assert abs(st["attempts"] - s.attempts) <= 2, (st, s.attempts)
        assert st["status"] == nat.RK_ST_DONE and abs(st["t"] - tf) < 1e-12
    assert errs[10.0] <= 5e-4, errs


def test_lockstep_batch_equals_single_instance():
    x, (lin, nl) = ac_ops(64)
    xi = x[1:-1]
    w0 = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi) - xi
    one = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-4), controller="lockstep")
    u1 = one.evolve(w0[None, :], 0.0, 5.0).cpu().numpy()
    many = DenseEnsemble(lin, nl, 130, config=SolverConfig(epsilon=1e-4), controller="lockstep")  # three tiles, the last padded
    u2 = many.evolve(np.repeat(w0[None, :], 130, axis=0), 0.0, 5.0).cpu().numpy()
    np.testing.assert_array_equal(u2, np.repeat(u1, 130, axis=0))
    assert one.stats()["attempts"] == many.stats()["attempts"]


def config5_ics(count, seed, xi):
    """u0 = 0.53 x + 0.47 sin(-1.5 pi x) + 0.1 N(0,1) smoothed by a 5-point moving average on
    the interior; returned as w0 = u0 - x (interior points)."""
    rng = np.random.default_rng(seed)
    base = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi)
    noise = 0.1 * rng.standard_normal((count, xi.size))
    k = np.ones(5) / 5.0
    sm = np.stack([np.convolve(r, k, mode="same") for r in noise])
    return base[None, :] + sm - xi[None, :]


def test_config5_batch_against_tight_fp64():
    x, (lin, nl) = ac_ops(129)
    xi = x[1:-1]
    w0 = config5_ics(8192, 11, xi)
    ens = DenseEnsemble(lin, nl, 8192, config=SolverConfig(epsilon=1e-4), controller="lockstep")
    out = ens.evolve(w0, 0.0, 70.0).cpu().numpy().astype(np.float64)
    st = ens.stats()
    assert st["status"] == nat.RK_ST_DONE and np.all(np.isfinite(out))
    for i in (0, 1, 4095, 8191):
        s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-8), diagonalize=True)
        ref = s.evolve(w0[i].astype(np.complex128), 0.0, 70.0, store_data=False).real
        err = np.linalg.norm(out[i] - ref) / np.linalg.norm(ref)
        print(f"config-5 instance {i}: rel L2 vs FP64 eps=1e-8 {err:.3e} (batch attempts {st['attempts']})")
        assert err <= 2e-3, (i, err)


def test_solver_api_with_a_dense_operator():
    """ETD35(lin_op_2d, Allen-Cahn, precision fp32) runs the tensor-core path with the
    reference's snapshot semantics (solveras.py:622-646): t0, then a snapshot after every
    store_freq-th accepted step.  The step sequence itself is not compared with the FP64
    oracle: where the embedded error is near FP32 resolution (the first attempt here: s =
    3.91 in FP64, err ~2e-7 |u|) FP32 stages move s by a few percent, so h and the snapshot
    times drift from the FP64 ones (by up to ~10% here) while the states stay on the same
    solution: each snapshot matches an FP64 oracle run to the snapshot's own time to 1e-3,
    the final state at tf to 1e-4."""
    from rkstiff_gb300 import ETD35

    x, (lin, nl) = ac_ops(20)
    xi = x[1:-1]
    w0 = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi) - xi
    solver = ETD35(lin_op=lin, nl_func=nl, config=SolverConfig(epsilon=1e-4), device_options=DeviceOptions(precision="fp32"))
    uf = solver.evolve(w0, t0=0.0, tf=5.0, store_freq=3)
    assert type(solver._engine()).__name__ == "DenseBackend"
    steps = solver.stats["steps"]
    assert len(solver.t) == 1 + steps // 3 and solver.t[0] == 0.0
    assert np.all(np.diff(solver.t) > 0) and solver.t[-1] <= 5.0
    for ti, ui in zip(solver.t[1:], solver.u[1:]):
        ref = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-8), dense_psi="eig")
        r = ref.evolve(w0.astype(np.complex128), 0.0, float(ti), store_data=False).real
        assert np.linalg.norm(np.asarray(ui).real - r) <= 2e-5 * np.linalg.norm(r), ti
    ref = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-8), dense_psi="eig")
    rf = ref.evolve(w0.astype(np.complex128), 0.0, 5.0, store_data=False)
    assert np.linalg.norm(np.asarray(uf).real - rf.real) <= 2e-5 * np.linalg.norm(rf.real)
    unew, h_used, h_next = solver.step(w0, 0.01)
    assert h_used == 0.01 and h_next > 0


def test_diagonalized_error_semantics():
    """diagonalize=True forms the error vector in the eigenbasis with the mask of the
    physical state (etd35.py:495): the first attempt's s and the accept/reject sequence to
    t=10 match the oracle's diagonalized ETD35, the reference's result for that form."""
    from rkstiff_gb300 import ETD35

    x, (lin, nl) = ac_ops(20)
    xi = x[1:-1]
    w0 = 0.53 * xi + 0.47 * np.sin(-1.5 * np.pi * xi) - xi
    ens = DenseEnsemble(lin, nl, 1, config=SolverConfig(epsilon=1e-4), err_basis="eigen", controller="lockstep")
    u = ens.pack_u(w0[None, :])
    ens.put_state(ens.fresh_state(0.0, 10.0, 0.05))
    st = ens.run(u, 1)
    o = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-4), diagonalize=True)
    o.reset()
    o.step(w0.astype(np.complex128), 0.05)
    # FP32 stages leave the cancelling error combination ~1e-3 relative, s ~4e-4
    assert abs(float(st["s_last"][0]) - o.log[0][2]) <= 2e-3 * o.log[0][2], (st["s_last"], o.log[0])
    solver = ETD35(lin_op=lin, nl_func=nl, config=SolverConfig(epsilon=1e-4), diagonalize=True,
                   device_options=DeviceOptions(precision="fp32"))
    uf = solver.evolve(w0, t0=0.0, tf=10.0, store_data=False)
    ref = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=1e-4), diagonalize=True)
    rf = ref.evolve(w0.astype(np.complex128), 0.0, 10.0, store_data=False).real
    assert abs(solver.stats["attempts"] - ref.attempts) <= 1, (solver.stats, ref.attempts)
    assert np.linalg.norm(np.asarray(uf).real - rf) <= 5e-4 * np.linalg.norm(rf)
