"""Learned step-size controller for the adaptive methods.

A small MLP (8 inputs, two tanh layers of 64 units, one output) estimates, after an
accepted attempt with controller factor s (safety * (eps |u| / |err|)^(1/q) of
rkstiff/solveras.py:451-455), a bounded correction y: log s of the next attempt, rescaled
to the current step size, is taken as log s + clamp(y, -1, 1), and the next step is
h exp(log s + clamp(y, -1, 1)) / target.  Keeping log s outside the network keeps the
error feedback explicit for inputs unlike the training data.  The embedded error test
still judges every attempt; a rejected attempt takes the reference's reduction rule.

Training data are the per-attempt logs the plain controller writes on the device
(``collect_logs``); ``features_targets`` turns them into samples with exactly the features
the kernel computes; ``fit`` trains with the library's CUDA forward/backward/Adam kernels;
``packed`` gives the bf16 inference buffer the evolve kernel reads.
"""

from __future__ import annotations

import os
from typing import Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native as nat
from .engine import EvolveBoundError


PRETRAINED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "controller_etd35.npz")


def _f_s(s: np.ndarray) -> np.ndarray:
    """clamp(log s, -8, 8) with the log records' encodings (1e30: inf, -1: NaN)."""
    s = np.asarray(s, dtype=np.float64)
    out = np.where(s > 0, np.log(np.where(s > 0, s, 1.0)), -690.0)
    return np.clip(out, -8.0, 8.0)


def accepted_features(rec: np.ndarray):
    """Walk one instance's attempt records [K, RK_LOG_FIELDS] (t, h, s, accepted, tail,
    retries, n, method) and yield (k, features) for every accepted attempt k, with the
    features the evolve kernel forms at that accept: log s, the two previous log s, log of
    the last step ratio, whether the previous attempt was accepted, retries before this
    accept, log10 of the tail-energy fraction and its change since the previous attempt."""
    r = np.asarray(rec, dtype=np.float64)
    s_prev = s_prev2 = 0.0
    acc_prev, tail_prev, h_prev = 1.0, -1.0, 0.0
    for k in range(r.shape[0]):
        h, s, ok, tail, nloop = r[k, 1], r[k, 2], r[k, 3] > 0.5, r[k, 4], r[k, 5]
        fs = float(_f_s(s))
        if ok:
            lt = np.log10(tail + 1e-30)
            yield k, [fs, s_prev, s_prev2,
                      float(np.clip(np.log(h / h_prev), -3, 3)) if h_prev > 0 else 0.0,
                      acc_prev, min(nloop, 5.0), float(np.clip(lt, -30, 0)),
                      float(np.clip(lt - np.log10(tail_prev + 1e-30), -10, 10)) if tail_prev >= 0 else 0.0]
        h_prev, s_prev2, s_prev = h, s_prev, fs
        acc_prev, tail_prev = (1.0 if ok else 0.0), tail


def features_targets(log: np.ndarray, counts: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Samples from attempt logs [n_inst, cap, RK_LOG_FIELDS] (counts[i] records valid).

    One sample per accepted attempt k followed by attempt k+1 with a finite s: the
    features of ``accepted_features`` and the target
    clip(log s_{k+1} + log(h_{k+1}/h_k) - log s_k, -1, 1)."""
    X, T = [], []
    for i in range(log.shape[0]):
        K = int(min(counts[i], log.shape[1]))
        r = log[i, :K].astype(np.float64)
        for k, f in accepted_features(r):
            if k + 1 >= K:
                continue
            h, s_next, h_next = r[k, 1], r[k + 1, 2], r[k + 1, 1]
            if 0.0 < s_next < 1e30 and h > 0:
                X.append(f)
                T.append(float(np.clip(np.log(np.clip(s_next, 1e-8, 1e8)) + np.log(h_next / h) - f[0], -1, 1)))
    return np.asarray(X, dtype=np.float32).reshape(-1, nat.RK_MLP_IN), np.asarray(T, dtype=np.float32)


def collect_logs(ensemble, u0s, t0: float, tf: float, cap: int = 4096, h_init: Optional[float] = None,
                 max_steps: int = 20_000, max_launches: int = 4, controller: Optional["LearnedController"] = None):
    """Run ``ensemble`` with the attempt log on; returns (log, counts).  The plain controller
    chooses the steps unless ``controller`` is given (on-policy logs).  The run is bounded
    by ``max_launches`` launches of ``max_steps`` accepted steps."""
    eng = ensemble.engine
    eng.attempt_log = torch.zeros((eng.n_inst, cap, nat.RK_LOG_FIELDS), dtype=torch.float32, device=eng.device)
    eng.log_cap = cap
    mlp, target, cache = eng.mlp, eng.mlp_target, (eng.coef_blocks, eng.ladder)
    if controller is None:
        eng.mlp = None
    else:
        controller.install(ensemble, ladder=False)  # the logs the shipped network was trained on
    try:
        try:
            ensemble.evolve(u0s, t0, tf, h_init, max_steps=max_steps, max_launches=max_launches)
        except EvolveBoundError:
            pass  # the bound was hit: the logs written so far are still samples
        log = eng.attempt_log.cpu().numpy()
    finally:
        eng.attempt_log = None
        eng.log_cap = 0
        eng.mlp, eng.mlp_target = mlp, target
        eng.set_coef_cache(cache[0], ladder=bool(cache[1]))
    return log, ensemble.stats()["attempts"]


class LearnedController:
    """The MLP, its training state and its packed inference buffer on one device."""

    def __init__(self, device=None, target: float = 1.25, seed: int = 0):
        self.lib = nat.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.target = float(target)
        rng = np.random.default_rng(seed)
        IN, H = nat.RK_MLP_IN, nat.RK_MLP_H
        p = np.concatenate([rng.standard_normal(H * IN) / np.sqrt(IN), np.zeros(H),
                            rng.standard_normal(H * H) / np.sqrt(H), np.zeros(H),
                            rng.standard_normal(H) / np.sqrt(H), np.zeros(1)]).astype(np.float32)
        assert p.size == nat.RK_MLP_NPARAM
        self.params = torch.from_numpy(p).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.mu = torch.zeros(IN, dtype=torch.float32, device=self.device)
        self.sd = torch.ones(IN, dtype=torch.float32, device=self.device)
        self._packed = None

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def set_normalisation(self, X: np.ndarray) -> None:
        mu = X.mean(axis=0)
        sd = X.std(axis=0)
        sd = np.where(sd > 1e-6, sd, 1.0)
        self.mu = torch.from_numpy(mu.astype(np.float32)).to(self.device)
        self.sd = torch.from_numpy(sd.astype(np.float32)).to(self.device)

    def normalise(self, X) -> torch.Tensor:
        Xt = torch.as_tensor(X, dtype=torch.float32, device=self.device)
        return ((Xt - self.mu) / self.sd).contiguous()

    def predict(self, X) -> np.ndarray:
        Xn = self.normalise(X)
        Y = torch.empty(Xn.shape[0], dtype=torch.float32, device=self.device)
        nat.check(self.lib.rk_mlp_forward(self.params.data_ptr(), Xn.data_ptr(), Xn.shape[0], Y.data_ptr(),
                                          self._stream()), "rk_mlp_forward")
        return Y.cpu().numpy()

    def grad(self, Xn: torch.Tensor, T: torch.Tensor, norm: float) -> Tuple[torch.Tensor, float]:
        """Gradient and loss of sum (y - t)^2 / norm on normalised inputs (device tensors)."""
        g = torch.zeros_like(self.params)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        nat.check(self.lib.rk_mlp_grad(self.params.data_ptr(), Xn.data_ptr(), T.data_ptr(), Xn.shape[0], norm,
                                       g.data_ptr(), loss.data_ptr(), self._stream()), "rk_mlp_grad")
        return g, float(loss.item())

    def fit(self, X: np.ndarray, T: np.ndarray, steps: int = 2000, batch: int = 2048, lr: float = 1e-3,
            seed: int = 0) -> list:
        """Adam on mini-batches with the CUDA kernels; returns the loss history."""
        self.set_normalisation(X)
        Xn = self.normalise(X)
        Tt = torch.as_tensor(T, dtype=torch.float32, device=self.device)
        n = Xn.shape[0]
        gen = torch.Generator(device=self.device).manual_seed(seed)
        g = torch.zeros_like(self.params)
        loss_d = torch.zeros(1, dtype=torch.float32, device=self.device)
        hist = []
        for it in range(steps):
            idx = torch.randint(0, n, (min(batch, n),), device=self.device, generator=gen)
            xb = Xn[idx].contiguous()
            tb = Tt[idx].contiguous()
            g.zero_()
            loss_d.zero_()
            nat.check(self.lib.rk_mlp_grad(self.params.data_ptr(), xb.data_ptr(), tb.data_ptr(), xb.shape[0],
                                           float(xb.shape[0]), g.data_ptr(), loss_d.data_ptr(), self._stream()),
                      "rk_mlp_grad")
            self.step += 1
            nat.check(self.lib.rk_mlp_adam(self.params.data_ptr(), g.data_ptr(), self.m.data_ptr(),
                                           self.v.data_ptr(), self.step, lr, 0.9, 0.999, 1e-8, self._stream()),
                      "rk_mlp_adam")
            if it % 100 == 0 or it == steps - 1:
                hist.append(float(loss_d.item()))
        self._packed = None
        return hist

    def train(self, problems: Sequence[Tuple], rounds: int = 3, steps: int = 2000, cap: int = 4096,
              lr: float = 1e-3, max_steps: int = 20_000, max_launches: int = 4, verbose: bool = False) -> dict:
        """On-policy training over ``problems``, a list of (ensemble, u0s, t0, tf).

        Round 0 fits the plain controller's logs; every later round runs this controller on
        the same problems, adds those logs to the samples and refits.  A network fitted to
        the plain controller's logs alone sees, once it chooses the steps itself, history
        features outside that data (more attempts after a rejection, other step ratios);
        the added rounds cover them.  Returns per-round sample counts and losses."""
        Xs, Ts, report = [], [], []
        for r in range(rounds):
            for ens, u0s, t0, tf in problems:
                log, counts = collect_logs(ens, u0s, t0, tf, cap=cap, max_steps=max_steps, max_launches=max_launches,
                                           controller=self if r > 0 else None)
                X, T = features_targets(log, counts)
                Xs.append(X)
                Ts.append(T)
            X, T = np.concatenate(Xs), np.concatenate(Ts)
            hist = self.fit(X, T, steps=steps, lr=lr, seed=r)
            report.append({"round": r, "samples": int(X.shape[0]), "loss": hist[-1], "var": float(np.var(T))})
            if verbose:
                print(report[-1], flush=True)
        return {"rounds": report}

    def packed(self) -> torch.Tensor:
        """bf16 inference buffer for the evolve kernel."""
        if self._packed is None:
            out = torch.empty(nat.RK_MLP_PACK_BYTES, dtype=torch.uint8, device=self.device)
            nat.check(self.lib.rk_mlp_pack(self.params.data_ptr(), self.mu.data_ptr(), self.sd.data_ptr(),
                                           out.data_ptr(), self._stream()), "rk_mlp_pack")
            self._packed = out
        return self._packed

    def install(self, ensemble, ladder: bool = False) -> None:
        """Make ``ensemble`` use this controller on accepted attempts.  With ``ladder`` its
        step sizes are put on the geometric ladder h0 2^(k/16) (the rung nearest the
        proposal; after a rejection the rung below) and each instance keeps four
        coefficient blocks keyed by h, so a return to a recent rung rebuilds nothing (the
        network changes h on most accepted steps, where the reference's single-entry cache
        rebuilds the coefficients every attempt)."""
        ensemble.engine.mlp = self.packed()
        ensemble.engine.mlp_target = self.target
        ensemble.engine.set_coef_cache(4 if ladder else 1, ladder=ladder)

    def save(self, path: str) -> None:
        """Parameters, input normalisation and target as a .npz file."""
        d = self.state_dict()
        np.savez(path, params=d["params"], mu=d["mu"], sd=d["sd"], target=np.float64(d["target"]))

    @classmethod
    def from_file(cls, path: str, device=None) -> "LearnedController":
        c = cls(device=device)
        with np.load(path) as z:
            c.load_state_dict({"params": z["params"], "mu": z["mu"], "sd": z["sd"], "target": float(z["target"])})
        return c

    @classmethod
    def pretrained(cls, device=None) -> "LearnedController":
        """The controller shipped with the package (ETD35; rkstiff_gb300/train_controller.py)."""
        return cls.from_file(PRETRAINED, device=device)

    def state_dict(self) -> dict:
        return {"params": self.params.cpu().numpy(), "mu": self.mu.cpu().numpy(), "sd": self.sd.cpu().numpy(),
                "target": self.target}

    def load_state_dict(self, d: dict) -> None:
        self.params = torch.as_tensor(d["params"], dtype=torch.float32, device=self.device).contiguous()
        self.mu = torch.as_tensor(d["mu"], dtype=torch.float32, device=self.device).contiguous()
        self.sd = torch.as_tensor(d["sd"], dtype=torch.float32, device=self.device).contiguous()
        self.target = float(d["target"])
        self._packed = None
