"""Train the learned ETD35 step-size controller shipped in rkstiff_gb300/data.

    python -m rkstiff_gb300.train_controller [--out PATH] [--rounds 4] [--steps 2000]

Training problems (all FP32 stages, seeded; the Burgers evaluation set of the tests and
benchmarks uses other seeds):
  * 32 three-soliton NLS instances, n = 4096 on [-50, 50), epsilon = 1e-6, t in [0, 20];
  * 256 viscous Burgers instances, n = 512, nu log-uniform in [1e-3, 1e-1], epsilon = 1e-5,
    t in [0, 5];
  * 64 Kuramoto-Sivashinsky instances, n in {256, 512}, L ~ U[22, 120], epsilon = 1e-5,
    t in [0, 20].
The NLS logs alone do not carry over to Burgers (their history features barely vary: the
one-step correction has a spread of about 0.007 there against 0.085 on Burgers), so the
training set mixes the three problems.  Training is on-policy
(LearnedController.train): the plain controller's logs first, then three rounds of logs
written while the network chooses the steps.
"""

from __future__ import annotations

import argparse
import time

import torch

from . import workloads
from .controller import PRETRAINED, LearnedController
from .ensemble import Ensemble
from .solveras import SolverConfig

TRAIN_SEEDS = {"nls": 100, "burgers": 12345, "ks": 777}


def training_problems(nls_count: int = 32, burgers_count: int = 256, ks_count: int = 64, device=None):
    """(ensemble, u0s, t0, tf) for LearnedController.train."""
    sets = [
        (workloads.nls_solitons(nls_count, TRAIN_SEEDS["nls"]), 1e-6, 20.0),
        (workloads.burgers_ensemble(burgers_count, TRAIN_SEEDS["burgers"]), 1e-5, 5.0),
        (workloads.ks_ensemble(ks_count, TRAIN_SEEDS["ks"], n_choices=(256, 512)), 1e-5, 20.0),
    ]
    out = []
    for insts, eps, tf in sets:
        ens = Ensemble("ETD35", [a[0] for a in insts], [a[1] for a in insts], config=SolverConfig(epsilon=eps),
                       precision="fp32", device=device)
        out.append((ens, [a[2] for a in insts], 0.0, tf))
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", default=PRETRAINED)
    ap.add_argument("--rounds", type=int, default=4)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--target", type=float, default=1.05)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    t0 = time.time()
    ctl = LearnedController(target=args.target, seed=args.seed)
    rep = ctl.train(training_problems(device=ctl.device), rounds=args.rounds, steps=args.steps, verbose=True)
    torch.cuda.synchronize()
    ctl.save(args.out)
    print({"out": args.out, "seconds": round(time.time() - t0, 1), "rounds": rep["rounds"]})


if __name__ == "__main__":
    main()
