#!/usr/bin/env python
"""Throughput of the batched uneven Kuramoto-Sivashinsky ensemble (the headline workload).

Workload: 4096 independent KS instances, grid n uniform over {256, 512, 1024, 2048},
domain length L ~ U[22, 120], u0 = sum_{k=1..8} a_k cos(2 pi k x/L + phi_k) with
a_k ~ N(0,1) exp(-k/4), phi_k ~ U[0, 2 pi); ETD35 adaptive (epsilon = 1e-5) with every
instance stepping its own dt to tf = 100, FP32 stages (FP64 coefficients, error norm and
time).  One bench step = the whole ensemble evolved from t = 0 to tf in one persistent
launch.  Metric: mode-steps/s = sum_i m_i * accepted_steps_i / seconds (m_i = n_i/2 + 1).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's NumPy algorithm on this
machine's host cores (a bounded sample of the same workload per step).
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# launch shapes the autotuner chose for the headline workload on a GB300 (its cache format)
SHAPES_FILE = os.path.join(ROOT, "rkstiff_gb300", "data", "ks_ensemble_shapes_gb300.json")

WORKLOAD = {
    "workload": "ks_uneven_ensemble_etd35",
    "instances": 4096,
    "n_choices": [256, 512, 1024, 2048],
    "L_range": [22.0, 120.0],
    "ic_modes": 8,
    "epsilon": 1e-5,
    "tf": 100.0,
    "method": "ETD35",
    "seed": 20261203,
}
METRIC = "mode-steps/s (KS uneven ensemble, ETD35 eps=1e-5, tf=100)"
UNIT = "mode-steps/s"


def make_instances(count: int, seed: int, n_choices=None):
    """(n, L, u0_hat) per instance, seeded."""
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.array(n_choices or WORKLOAD["n_choices"]), size=count)
    Ls = rng.uniform(*WORKLOAD["L_range"], size=count)
    k = np.arange(1, WORKLOAD["ic_modes"] + 1)
    amps = rng.standard_normal((count, k.size)) * np.exp(-k / 4.0)
    phis = rng.uniform(0.0, 2 * np.pi, size=(count, k.size))
    out = []
    for i in range(count):
        n, L = int(ns[i]), float(Ls[i])
        x = np.arange(n) * (L / n)
        u0 = np.sum(amps[i][:, None] * np.cos(2 * np.pi * k[:, None] * x[None, :] / L + phis[i][:, None]), axis=0)
        out.append((n, L, np.fft.rfft(u0)))
    return out


def ks_operator(n: int, L: float):
    kx = 2 * np.pi * np.fft.rfftfreq(n, d=L / n)
    return kx, kx**2 * (1 - kx**2)


# ------------------------------------------------------------------------------------
# CPU baseline: the oracle (NumPy restatement of the reference algorithm), one instance
# per worker process, all host cores
# ------------------------------------------------------------------------------------
def _cpu_instance(args):
    n, L, u0 = args
    from oracle import rk_oracle as O

    kx, lin = ks_operator(n, L)

    def nl(u):
        return -np.fft.rfft(np.fft.irfft(u) * np.fft.irfft(1j * kx * u))

    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=WORKLOAD["epsilon"]))
    status = 0
    uf = None
    try:
        uf = s.evolve(u0, 0.0, WORKLOAD["tf"], store_data=False)
    except (O.MinimumStepReached, O.MaxLoopsExceeded):
        status = 1
    steps = sum(1 for r in s.log if r[3])
    return n // 2 + 1, steps, s.attempts, status, uf


def _cpu_dense_instance(args):
    """One Allen-Cahn IC of the dense config by the oracle's diagonalized ETD35 (the
    reference's eig-based form; its contour form costs tens of seconds per IC)."""
    lin, shift, w0, eps, tf = args
    from oracle import rk_oracle as O

    def nl(v):
        return shift - (v + shift) ** 3

    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=eps), diagonalize=True)
    s.evolve(w0.astype(np.complex128), 0.0, tf, store_data=False)
    return sum(1 for r in s.log if r[3])


def cpu_pool(cores: int):
    for var in ("OMP_NUM_THREADS", "MKL_NUM_THREADS", "OPENBLAS_NUM_THREADS"):
        os.environ[var] = "1"
    return mp.get_context("spawn").Pool(cores)


def cpu_measure(pool, sample):
    t0 = time.perf_counter()
    res = pool.map(_cpu_instance, sample, chunksize=1)
    wall = time.perf_counter() - t0
    mode_steps = sum(r[0] * r[1] for r in res)
    return mode_steps / wall, wall, res


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# ------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ------------------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [p.strip() for p in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------
TRAFFIC_SUMMARY = os.path.join(ROOT, "profiles", "ks_ensemble_etd35_fp32_traffic.md")


PLACE_NAMES = {0: "global", 1: "smem-state", 2: "smem-all", 3: "smem-u"}


def shape_tag(n, threads, groups, place) -> str:
    return "n=%d %dx%d/%s" % (n, threads, groups, PLACE_NAMES[place])


def profiled_traffic(tuned):
    """DRAM bytes (read + write) of one headline launch: the sum over its grid-size class
    kernels of the per-class figures in the committed summary of ncu captures of that launch
    (lines 'traffic n=<n> <threads>x<groups>/<placement>: <bytes>').  A class kernel's traffic
    depends on its launch shape (global scratch writes its stage vectors back), so each class
    is looked up under the shape this run used; returns (bytes or None, [missing shapes])."""
    table = {}
    try:
        with open(TRAFFIC_SUMMARY) as f:
            for line in f:
                m = re.match(r"\s*traffic (n=\d+ \d+x\d+/[a-z-]+):\s*(\d+)", line)
                if m:
                    table[m.group(1)] = float(m.group(2))
    except OSError:
        pass
    total, missing = 0.0, []
    for n, v in tuned.items():
        tag = shape_tag(int(n), v["threads"], v["groups"], v["place"])
        if tag in table:
            total += table[tag]
        else:
            missing.append(tag)
    return (None if missing else total), missing


def pin_shapes(ens, spec: str):
    """Install launch shapes given as 'n:TxG:placement,...' (e.g. '2048:128x1:global') for
    every grid-size class, in place of the tuner's choice."""
    from rkstiff_gb300 import autotune as _at
    by_n = {}
    for item in spec.split(","):
        n, tg, place = item.split(":")
        t, g = tg.split("x")
        by_n[int(n)] = (int(t), int(g), {v: k for k, v in PLACE_NAMES.items()}[place])
    eng = ens.engine
    missing = [int(n) for n in eng.class_n if int(n) not in by_n]
    if missing:
        raise SystemExit(f"--shapes gives no shape for grid size(s) {missing}")
    _at._CACHE[_at._key(eng)] = tuple(by_n[int(n)] for n in eng.class_n)


def flops_of(ens_engine, st) -> float:
    """Algorithmic FP32 FLOPs of one launch from its counters: per nonlinear evaluation
    7.5 n log2 n + n + 2m (one complex inverse FFT of n, one forward of n/2, the product
    and the packing), 215 m per attempt (stage combinations and the error norm)."""
    n = ens_engine.ns.astype(np.float64)
    m = ens_engine.ms.astype(np.float64)
    per_nl = 7.5 * n * np.log2(n) + n + 2 * m
    return float(np.sum(st["nl_evals"] * per_nl + st["attempts"] * 215.0 * m))


def measure_fp32_peak(device) -> float:
    import torch

    from rkstiff_gb300 import _native as nat

    lib = nat.load()
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    blocks, threads, iters = nsm * 8, 256, 1 << 15
    out = torch.empty(blocks * threads, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)
    for _ in range(2):
        nat.check(lib.rk_probe_fp32(out.data_ptr(), blocks, threads, iters, stream.cuda_stream), "probe")
    best = 0.0
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nat.check(lib.rk_probe_fp32(out.data_ptr(), blocks, threads, iters, stream.cuda_stream), "probe")
        e1.record(stream)
        e1.synchronize()
        best = max(best, 16.0 * blocks * threads * iters / (e0.elapsed_time(e1) * 1e-3))
    return best / 1e12


FORMS = {"workload": "burgers_ensemble_etd35", "instances": 2048, "n": 512, "nu_range": [1e-3, 1e-1],
         "epsilon": 1e-5, "tf": 5.0, "seed": 7, "reference_epsilon": 1e-10, "reference_sample": 256,
         "precision_check_h": 0.005}

# accuracy of the headline (FP32) against the FP64 oracle on a sample: one adaptive step from
# u0 (the <= 1e-6 gate), and trajectories to a short horizon; chaotic KS at tf = 100 is
# reported, not gated (the reference's own eps = 1e-5 run differs from a tight one by 1e-4..4e-3)
ACCURACY = {"per_size": 4, "h_step": 0.01, "t_short": 10.0, "gate_one_step": 1e-6}


def _rel(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _stats(v) -> dict:
    v = np.asarray(v, dtype=np.float64)
    if v.size == 0:
        return {"count": 0}
    return {"count": int(v.size), "median": float(np.median(v)), "p90": float(np.quantile(v, 0.9)),
            "max": float(np.max(v))}


def headline_accuracy(dev, inst, gpu_finals=None, oracle_finals=None) -> dict:
    """rel L2 of the FP32 ensemble against the FP64 oracle (the reference's algorithm):
    ACCURACY['per_size'] instances of each grid size, one adaptive step from u0 at
    h = ACCURACY['h_step'] and the trajectory to t = ACCURACY['t_short'] (same epsilon); and,
    when given, the tf = 100 states of the CPU-baseline sample (reported, not gated)."""
    from oracle import rk_oracle as O
    from rkstiff_gb300 import _native as nat
    from rkstiff_gb300 import models
    from rkstiff_gb300.ensemble import Ensemble
    from rkstiff_gb300.solveras import SolverConfig

    idx = []
    for n in WORKLOAD["n_choices"]:
        idx += [i for i, r in enumerate(inst) if r[0] == n][:ACCURACY["per_size"]]
    eps, h, T = WORKLOAD["epsilon"], ACCURACY["h_step"], ACCURACY["t_short"]
    lins, nls, u0s = [], [], []
    for i in idx:
        n, L, u0 = inst[i]
        kx, lin = ks_operator(n, L)
        lins.append(lin)
        nls.append(models.ks_ops(kx)[1])
        u0s.append(u0)
    ens = Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=eps), precision="fp32", device=dev)
    eng = ens.engine
    u = eng.pack_u(u0s)
    eng.put_state(eng.fresh_state(0.0, np.inf, h))
    eng.launch(u, nat.RK_RUN_STEP)
    st = eng.get_state()
    one = [x.cpu().numpy() for x in eng.unpack_u(u)]
    fin = [x.cpu().numpy() for x in ens.evolve(u0s, 0.0, T)]
    one_err, same_h, short_err = [], 0, []
    for k in range(len(idx)):
        o = O.OracleSolver("ETD35", lins[k], nls[k], O.SolverConfig(epsilon=eps))
        un, hu, _ = o.step(u0s[k].astype(np.complex128), h)
        if hu == float(st["h_used"][k]):
            same_h += 1
            one_err.append(_rel(one[k], un))
        o = O.OracleSolver("ETD35", lins[k], nls[k], O.SolverConfig(epsilon=eps))
        short_err.append(_rel(fin[k], o.evolve(u0s[k].astype(np.complex128), 0.0, T, store_data=False)))
    out = {"reference": "FP64 NumPy oracle of the reference's ETD35 (same epsilon)",
           "sample": f"{ACCURACY['per_size']} instances per grid size {WORKLOAD['n_choices']} of the workload",
           "one_step": {**_stats(one_err), "h": h, "same_step_size": same_h,
                        "gate": ACCURACY["gate_one_step"],
                        "pass": bool(one_err) and max(one_err) <= ACCURACY["gate_one_step"]},
           f"t{int(T)}": _stats(short_err)}
    if gpu_finals is not None and oracle_finals:
        errs = [_rel(gpu_finals[i], oracle_finals[i]) for i in sorted(oracle_finals) if i < len(gpu_finals)]
        out["tf100_reported_not_gated"] = {**_stats(errs), "sample": "the CPU baseline's instances (oracle to tf=100)"}
    return out


def single_instance_lines(dev, cpu_single) -> dict:
    """Configs 1 and 2 through the solver API (one instance each): KS n=1024 IF34 FP64 eps=1e-4
    to t=50 storing every 20 steps; NLS n=4096 ETD35 eps=1e-6 to t=20 in FP64 and FP32.  Each:
    mode-steps/s (wall clock of the evolve call, best of 3 after a warm-up), attempts, rel L2
    against the FP64 oracle's final state, and the oracle on one host process beside it."""
    import torch

    import rkstiff_gb300 as rk

    ks, nls = single_instance_problems()
    out = {}
    cases = (("config1_ks1024_if34_fp64", "IF34", ks, "fp64", 1e-4, 50.0, 20, "ks1024_if34"),
             ("config2_nls4096_etd35_fp64", "ETD35", nls, "fp64", 1e-6, 20.0, 0, "nls4096_etd35"),
             ("config2_nls4096_etd35_fp32", "ETD35", nls, "fp32", 1e-6, 20.0, 0, "nls4096_etd35"))
    for name, method, (lin, nl, u0), prec, eps, tf, freq, ref_key in cases:
        best = None
        for rep in range(4):
            s = getattr(rk, method)(lin, nl, config=rk.SolverConfig(epsilon=eps),
                                    device_options=rk.DeviceOptions(precision=prec, device=dev))
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            uf = s.evolve(u0, 0.0, tf, store_data=freq > 0, store_freq=max(freq, 1))
            dt = time.perf_counter() - t0
            if rep > 0:
                best = dt if best is None else min(best, dt)
        m = int(np.asarray(u0).shape[0])
        st = s.stats
        line = {"metric": "mode-steps/s", "value": m * st["steps"] / best, "seconds": best, "modes": m,
                "steps": int(st["steps"]), "attempts": int(st["attempts"]), "nl_evals": int(st["nl_evals"]),
                "precision": prec, "path": "solver API (host arrays in and out, one persistent launch)"}
        ref = (cpu_single or {}).get(ref_key)
        if ref is not None:
            line["attempts_oracle"] = int(ref["attempts"])
            line["rel_l2_vs_fp64_oracle"] = _rel(uf, ref["final"])
            line["cpu_reference"] = {"value": m * ref["steps"] / ref["seconds"], "unit": "mode-steps/s",
                                     "seconds": ref["seconds"], "cores": 1, "kind": "port",
                                     "sample": "the whole run by the NumPy FP64 oracle in one host process"}
        out[name] = line
    return out


def forms_comparison(dev, oracle_refs=None) -> dict:
    """Plain FP64, plain FP32 and FP32 + learned controller on the viscous Burgers ensemble
    (2048 instances the controller was not trained on): mode-steps/s, NL evaluations per
    unit simulated time, rejected steps, and rel L2 error against an FP64 run at
    epsilon = 1e-10 on a sample of the instances every form finishes."""
    import torch

    from rkstiff_gb300 import workloads
    from rkstiff_gb300.controller import LearnedController
    from rkstiff_gb300.ensemble import Ensemble
    from rkstiff_gb300.solveras import SolverConfig

    inst = workloads.burgers_ensemble(FORMS["instances"], FORMS["seed"], n=FORMS["n"], nu_range=FORMS["nu_range"])
    lins, nls, u0s = [a[0] for a in inst], [a[1] for a in inst], [a[2] for a in inst]
    ctl = LearnedController.pretrained(device=dev)
    stream = torch.cuda.current_stream(dev)
    runs = {}
    for name, prec, learned in (("plain_fp64", "fp64", False), ("plain_fp32", "fp32", False),
                                ("learned_fp32", "fp32", True), ("learned_fp32_ladder", "fp32", "ladder")):
        ens = Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=FORMS["epsilon"]), precision=prec, device=dev)
        if learned:
            ctl.install(ens, ladder=learned == "ladder")
        u0 = ens.pack(u0s)
        u = torch.empty_like(u0)
        best = None
        for rep in range(3):  # one warm-up, best of two
            u.copy_(u0)
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = ens.evolve_packed(u, 0.0, FORMS["tf"], max_steps=20000, max_launches=3)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if rep > 0:
                dt = e0.elapsed_time(e1) * 1e-3
                best = dt if best is None else min(best, dt)
        runs[name] = (st, best, [o.cpu().numpy() for o in ens.engine.unpack_u(u)], ens.engine.ms.copy())
    ok = np.ones(len(inst), bool)
    for st, _, _, _ in runs.values():
        ok &= st["status"] == 0
    if oracle_refs:
        # the FP64 NumPy oracle (the reference's algorithm) at the tight epsilon
        idx = np.array([i for i in sorted(oracle_refs) if ok[i]], dtype=np.int64)
        ref = [oracle_refs[int(i)] for i in idx]
        ref_kind = f"FP64 NumPy oracle at epsilon {FORMS['reference_epsilon']:g} on {len(idx)} resolved instances"
    else:
        idx = np.where(ok)[0][:: max(1, int(ok.sum()) // FORMS["reference_sample"])][: FORMS["reference_sample"]]
        ref_ens = Ensemble("ETD35", [lins[i] for i in idx], [nls[i] for i in idx],
                           config=SolverConfig(epsilon=FORMS["reference_epsilon"]), precision="fp64", device=dev)
        ref = [o.cpu().numpy() for o in ref_ens.evolve([u0s[i] for i in idx], 0.0, FORMS["tf"], max_steps=50000,
                                                        max_launches=2)]
        ref_kind = f"GPU FP64 run at epsilon {FORMS['reference_epsilon']:g} on {len(idx)} instances"
    out = {"config": FORMS, "instances_finished_by_all": int(ok.sum()), "error_reference": ref_kind}
    for name, (st, dt, finals, ms) in runs.items():
        errs = np.array([np.linalg.norm(finals[i] - r) / np.linalg.norm(r) for i, r in zip(idx, ref)])
        done = st["status"] == 0
        out[name] = {
            "mode_steps_per_s": float(np.sum(ms * st["steps"])) / dt,
            "mode_time_units_per_s": float(np.sum(ms[done]) * FORMS["tf"]) / dt,
            "seconds": dt,
            "finished": int(np.sum(st["status"] == 0)),
            "nl_evals_per_unit_time": float(np.sum(st["nl_evals"][ok])) / (FORMS["tf"] * ok.sum()),
            "rejects": int(np.sum(st["rejects"][ok])),
            "accepted_steps": int(np.sum(st["steps"][ok])),
            "rel_l2_median": float(np.median(errs)),
            "rel_l2_p90": float(np.quantile(errs, 0.9)),
            "coefficient_rebuilds_per_attempt": float(np.sum(st["coeff_updates"][ok]) / max(np.sum(st["attempts"][ok]), 1)),
        }
    p64, p32, l32 = out["plain_fp64"], out["plain_fp32"], out["learned_fp32"]
    out["learned_fp32_over_plain_fp64"] = {
        "mode_steps_per_s": l32["mode_steps_per_s"] / p64["mode_steps_per_s"],
        "nl_evals_per_unit_time": l32["nl_evals_per_unit_time"] / p64["nl_evals_per_unit_time"],
    }
    # the controller comparison on time to solution (a controller that takes fewer, larger
    # steps lowers mode-steps/s while finishing sooner)
    out["learned_fp32_over_plain_fp32"] = {
        "mode_time_units_per_s": l32["mode_time_units_per_s"] / p32["mode_time_units_per_s"],
        "nl_evals_per_unit_time": l32["nl_evals_per_unit_time"] / p32["nl_evals_per_unit_time"],
        "rejects": l32["rejects"] / max(p32["rejects"], 1),
    }
    lad = out["learned_fp32_ladder"]
    out["learned_fp32_ladder_over_plain_fp32"] = {
        "mode_time_units_per_s": lad["mode_time_units_per_s"] / p32["mode_time_units_per_s"],
        "nl_evals_per_unit_time": lad["nl_evals_per_unit_time"] / p32["nl_evals_per_unit_time"],
        "rejects": lad["rejects"] / max(p32["rejects"], 1),
    }
    # FP32 rounding alone: the same fixed-step trajectory (ETD5, the ETD35 stages without the
    # controller) in FP32 and in FP64 on the error sample, so no step-size decision differs
    hfix = FORMS["precision_check_h"]
    fin = {}
    for prec in ("fp32", "fp64"):
        e5 = Ensemble("ETD5", [lins[i] for i in idx], [nls[i] for i in idx], precision=prec, device=dev)
        fin[prec] = [o.cpu().numpy().astype(np.complex128) for o in
                     e5.evolve([u0s[i] for i in idx], 0.0, FORMS["tf"], h_init=hfix, max_steps=50000)]
    rel_fixed = [_rel(a, b) for a, b in zip(fin["fp32"], fin["fp64"])]
    out["fp32_rounding_fixed_step"] = {**_stats([r for r in rel_fixed if np.isfinite(r)]),
                                       "nonfinite": int(sum(1 for r in rel_fixed if not np.isfinite(r))),
                                       "method": "ETD5", "h": hfix,
                                       "what": "rel L2 of FP32 against FP64 on the same fixed-step trajectory"}
    return out


DENSE = {"workload": "allen_cahn_chebyshev_etd35_dense", "instances": 8192, "interior_points": 128,
         "epsilon_ac": 0.01, "solver_epsilon": 1e-4, "tf": 70.0, "seed": 5, "reference_epsilon": 1e-8,
         "reference_sample": [0, 2731, 5462, 8191]}
# 3xTF32 tensor FLOPs of one basis change (a 128 x 128 matrix times one instance's vector,
# three TF32 products) and the basis changes of one attempt of the per-instance path
DENSE_GEMM_FLOPS = 3 * 2 * 128 * 128  # one 3xTF32 basis change of one instance vector
DENSE_EIG_GEMMS_PER_ATTEMPT = 13


def dense_measurement(dev) -> dict:
    """Config of the dense path: 8192 Allen-Cahn ICs on 128 interior Chebyshev points, ETD35 to
    tf = 70, every IC under the reference's controller (per-instance h; stages in the
    eigenbasis, basis changes as 3xTF32 tcgen05 GEMMs).  Reports mode-steps/s (128 x the
    accepted steps of all ICs / s), ICs per second, the tensor-pipe rate against the TF32 peak,
    rel L2 error against per-IC FP64 oracle runs at epsilon = 1e-8, and the lockstep batch
    path (one h for all ICs, psi-matrices) timed on the same ICs for comparison."""
    import torch

    from oracle import rk_oracle as O
    from rkstiff_gb300 import workloads
    from rkstiff_gb300.dense import DenseEnsemble
    from rkstiff_gb300.solveras import SolverConfig

    lin, nl, w0 = workloads.allen_cahn_batch(DENSE["instances"], DENSE["seed"], epsilon=DENSE["epsilon_ac"])
    stream = torch.cuda.current_stream(dev)

    def timed(ens):
        best = out = None
        for rep in range(3):  # one warm-up, best of two
            torch.cuda.synchronize(dev)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = ens.evolve(w0, 0.0, DENSE["tf"])
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if rep > 0:
                dt = e0.elapsed_time(e1) * 1e-3
                best = dt if best is None else min(best, dt)
        return best, out

    cfg = SolverConfig(epsilon=DENSE["solver_epsilon"])
    ens = DenseEnsemble(lin, nl, DENSE["instances"], config=cfg, device=dev)
    best, out = timed(ens)
    st = ens.stats()
    lock = DenseEnsemble(lin, nl, DENSE["instances"], config=cfg, device=dev, controller="lockstep")
    lbest, _ = timed(lock)
    lst = lock.stats()
    # the same kernel for the first-same-as-last methods (ETD34, IF34) on the same ICs, each
    # checked on one IC against an FP64 oracle run at epsilon = 1e-8
    methods = {}
    for m in ("ETD34", "IF34"):
        me = DenseEnsemble(lin, nl, DENSE["instances"], config=cfg, device=dev, method=m)
        mbest, mout = timed(me)
        mst = me.stats()
        i0 = DENSE["reference_sample"][0]
        o = O.OracleSolver(m, lin, lambda v: nl(v), O.SolverConfig(epsilon=DENSE["reference_epsilon"]),
                           diagonalize=True)
        ref = o.evolve(w0[i0].astype(np.complex128), 0.0, DENSE["tf"], store_data=False).real
        mo = mout[i0].cpu().numpy().astype(np.float64)
        methods[m] = {"seconds": mbest, "instances_per_s": DENSE["instances"] / mbest,
                      "mode_steps_per_s": 128.0 * mst["steps_total"] / mbest,
                      "attempts_total": mst["attempts_total"], "rejects_total": mst["rejects_total"],
                      "all_done": bool(np.all(mst["status"] == 0)),
                      f"rel_l2_vs_fp64_eps1e-8_ic{i0}": float(np.linalg.norm(mo - ref) / np.linalg.norm(ref))}
    out = out.cpu().numpy().astype(np.float64)
    errs = []
    for i in DENSE["reference_sample"]:
        s = O.OracleSolver("ETD35", lin, lambda v: nl(v), O.SolverConfig(epsilon=DENSE["reference_epsilon"]),
                           diagonalize=True)
        ref = s.evolve(w0[i].astype(np.complex128), 0.0, DENSE["tf"], store_data=False).real
        errs.append(float(np.linalg.norm(out[i] - ref) / np.linalg.norm(ref)))
    # 13 basis changes per attempt (S k and S^-1 N for five stages, S err, S unew, S^-1 N(unew))
    # plus the two of the first call (S^-1 u, S^-1 N(u)), three TF32 products each
    flops = (st["attempts_total"] * DENSE_EIG_GEMMS_PER_ATTEMPT + 2 * DENSE["instances"]) * DENSE_GEMM_FLOPS
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    bf16 = peaks.get("bf16_tflops", 1900.0)
    tf32_peak = bf16 / 2.0
    achieved = flops / best / 1e12
    return {
        "config": DENSE,
        "metric": "mode-steps/s",
        "value": 128.0 * st["steps_total"] / best,
        "seconds": best,
        "instances_per_s": DENSE["instances"] / best,
        "controller": "per instance (the reference's rule for every IC)",
        "accepted_steps_total": st["steps_total"], "attempts_total": st["attempts_total"],
        "rejects_total": st["rejects_total"], "coefficient_updates_total": st["coeff_updates_total"],
        "attempts_per_ic": {"mean": float(np.mean(st["attempts"])), "max": int(np.max(st["attempts"]))},
        "rel_l2_vs_fp64_eps1e-8": errs,
        "tensor": {"achieved": achieved, "peak": tf32_peak, "unit": "TFLOP/s", "frac": achieved / tf32_peak,
                   "flops": flops,
                   "peak_source": "TF32 dense = half of the measured bf16 burst in MEASURED_PEAKS.json"
                                  if "bf16_tflops" in peaks else "TF32 dense = half of the 1.9 PFLOP/s bf16 fallback",
                   "counted": "3 TF32 products x 13 basis changes (128 x 128 by the CTA's 64 instance vectors) "
                              "per instance-attempt; the stage combinations are elementwise, off the tensor pipe"},
        "methods": methods,
        "lockstep": {"seconds": lbest, "instances_per_s": DENSE["instances"] / lbest,
                     "mode_steps_per_s": 128.0 * DENSE["instances"] * lst["steps"] / lbest,
                     "batch_attempts": lst["attempts"], "batch_steps": lst["steps"]},
    }


def gpu_arm(args, rank, world, cpu_line, dense_cpu=None, extra=None):
    import torch

    from rkstiff_gb300 import models, sharding
    from rkstiff_gb300.ensemble import Ensemble
    from rkstiff_gb300.solveras import SolverConfig

    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    seed = WORKLOAD["seed"] if world == 1 else sharding.weak_seed(WORKLOAD["seed"], rank)
    inst = make_instances(WORKLOAD["instances"], seed)
    lins, nls, u0s = [], [], []
    for n, L, u0 in inst:
        kx, lin = ks_operator(n, L)
        lins.append(lin)
        nls.append(models.ks_ops(kx)[1])
        u0s.append(u0)
    ens = Ensemble("ETD35", lins, nls, config=SolverConfig(epsilon=WORKLOAD["epsilon"]), precision="fp32",
                   device=dev)
    eng = ens.engine
    from rkstiff_gb300 import autotune as _at
    if args.shapes:
        pin_shapes(ens, args.shapes)
        tuned = ens.autotune(u0s, span=10.0)  # served from the pinned shapes
        shapes_source = "pinned on the command line"
    elif args.tune_cache and _at.load(args.tune_cache):
        tuned = ens.autotune(u0s, span=10.0)  # served from the loaded cache
        shapes_source = f"tuner cache {args.tune_cache}"
    else:
        # the shapes rkstiff_gb300.autotune chose for this workload on a GB300 (its cache file,
        # committed), so that every run launches the shapes whose DRAM traffic is captured in
        # profiles/; --retune (or another device or workload) tunes in the run instead
        cached = (not args.retune) and _at.load(SHAPES_FILE) and _at._key(eng) in _at._CACHE
        tuned = ens.autotune(u0s, span=10.0)
        shapes_source = (f"autotuner result for this workload on a GB300, {os.path.relpath(SHAPES_FILE, ROOT)}"
                         if cached else "tuned in this run by rkstiff_gb300.autotune")
        if args.tune_cache:
            _at.save(args.tune_cache)
    u0_dev = ens.pack(u0s)
    u = torch.empty_like(u0_dev)
    tf = WORKLOAD["tf"]

    def one_step():
        # one replay of the captured CUDA graph: initial state copy, state reset, every
        # class kernel of the persistent evolve launch
        return ens.evolve_graph(u, u0_dev, 0.0, tf)

    l2_flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        st = one_step()
    torch.cuda.synchronize()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    eng.events = []
    eng.record_events = True
    launches0 = eng.launches
    kernels0 = eng.kernel_launches
    mode_steps = 0
    flops = 0.0
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    pairs = []
    for i in range(args.steps):
        # L2 flush between timed steps: a write larger than the 129 MB L2, outside the
        # step's own event pair
        l2_flush.fill_(i & 0xFF)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        st = one_step()
        b.record(stream)
        pairs.append((a, b))
        mode_steps += int(np.sum(eng.ms * st["steps"]))
        flops += flops_of(eng, st)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    eng.record_events = False
    elapsed = sum(a.elapsed_time(b) for a, b in pairs) * 1e-3
    kernel_s = sum(a.elapsed_time(b) for a, b in eng.events) * 1e-3
    n_launch = eng.launches - launches0
    n_kernels = eng.kernel_launches - kernels0
    status = st["status"]
    max_elapsed = sharding.max_over_ranks(elapsed, dev)
    total_mode_steps = sharding.sum_over_ranks(mode_steps, dev)
    value = total_mode_steps / max_elapsed

    # end to end through the public API with host buffers: pinned host ICs in, finals out
    host_in = torch.empty(u0_dev.shape, dtype=u0_dev.dtype, pin_memory=True)
    host_in.copy_(u0_dev.cpu())
    host_out = torch.empty_like(host_in, pin_memory=True)
    e2e_mode_steps = 0
    e2e_s = 0.0
    for i in range(args.steps):
        l2_flush.fill_(i & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u0_dev.copy_(host_in, non_blocking=True)
        st2 = ens.evolve_graph(u, u0_dev, 0.0, tf)
        host_out.copy_(u, non_blocking=True)
        torch.cuda.synchronize()
        e2e_s += time.perf_counter() - t0
        e2e_mode_steps += int(np.sum(eng.ms * st2["steps"]))
    e2e_elapsed = sharding.max_over_ranks(e2e_s, dev)
    e2e_value = sharding.sum_over_ranks(e2e_mode_steps, dev) / e2e_elapsed
    state_bytes = eng.state_dev.numel()
    vec_bytes = u.numel() * u.element_size()

    if rank != 0:
        return
    extra = extra or {}
    gpu_finals = [x.cpu().numpy().astype(np.complex128) for x in eng.unpack_u(u)]
    accuracy = headline_accuracy(dev, inst, gpu_finals, extra.get("tf_finals")) if world == 1 else None
    single = single_instance_lines(dev, extra.get("single")) if (world == 1 and not args.no_single) else None
    peak = measure_fp32_peak(dev)
    forms = forms_comparison(dev, extra.get("forms_ref")) if (world == 1 and not args.no_forms) else None
    dense = dense_measurement(dev) if (world == 1 and not args.no_dense) else None
    if dense is not None:
        dense["cpu_baseline"] = dense_cpu
    achieved = flops / kernel_s / 1e12
    traffic, traffic_missing = profiled_traffic(tuned)
    counts = {name: int(np.sum(status == code)) for name, code in (("done", 0), ("max_loops", 1), ("min_step", 2))}
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_elapsed / args.steps * 1e3,
        "step_ms": [round(a.elapsed_time(b), 3) for a, b in pairs],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 (complex64 stages and FFTs; coefficients formed from the FP64 operator to FP32 accuracy, error sums in double-float FP32 pairs, time and step size in FP64)",
        "data": "synthetic (seeded KS ensemble)",
        "config": {
            **{k: WORKLOAD[k] for k in ("workload", "instances", "n_choices", "L_range", "epsilon", "tf", "method")},
            "precision": "fp32",
            "launch": "one persistent launch per step, replayed from a captured CUDA graph",
            "schedule": "per grid-size class, longest first by the previous launch's attempt counts "
                        "(set after the first warm-up step; the order does not change any instance's result)",
            "parallelism": f"instances per GPU, {world} GPU(s)",
            "l2_flush": "256 MB written between timed steps, outside each step's event pair",
            "instance_status": counts,
            "launch_shapes": {str(n): "%d groups x %d threads per block, %s scratch" % (
                v["groups"], v["threads"], PLACE_NAMES[v["place"]]) for n, v in tuned.items()},
            "launch_shapes_source": shapes_source,
        },
        "roofline": {
            "bound": "fp32",
            "achieved": achieved,
            "peak": peak,
            "unit": "TFLOP/s",
            "frac": achieved / peak,
            "traffic": traffic,
            "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per class kernel of one headline "
                              "launch at this run's launch shapes, summed over the classes; ncu captures "
                              "summarised in profiles/ks_ensemble_etd35_fp32_traffic.md"
                              + ("" if traffic is not None else
                                 "; no capture for " + ", ".join(traffic_missing)),
            "algorithmic_bytes": 2 * vec_bytes + state_bytes,
            "peak_source": "measured in this run by rk_probe_fp32 (FP32 FMA throughput; "
                           "MEASURED_PEAKS.json carries no FP32 CUDA-core figure)",
            "flops_per_launch": flops / max(n_launch, 1),
            "kernel_ms_per_launch": kernel_s / max(n_launch, 1) * 1e3,
            "launch": "one rk_evolve call = %d concurrent grid-size-class kernels, timed together" % (
                n_kernels // max(n_launch, 1)),
        },
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": vec_bytes,
                "d2h_bytes_per_step": vec_bytes + state_bytes,
                "path": "pinned host spectra -> device, graph replay, final spectra and state records -> host"},
        "gpu_launches": n_kernels,
        "cpu_baseline": cpu_line,
    }
    if accuracy is not None:
        line["accuracy"] = accuracy
    if single is not None:
        line["single_instance"] = single
    if forms is not None:
        line["forms"] = forms
    if dense is not None:
        line["dense"] = dense
    print(json.dumps(line), flush=True)


def reference_arm(args, rank, world):
    if rank != 0:
        return
    cores = host_cores()
    per_step = max(cores, 2 * cores)
    inst = make_instances(WORKLOAD["instances"], WORKLOAD["seed"])
    pool = cpu_pool(cores)
    try:
        step = 0
        for _ in range(args.warmup):
            sample = inst[(step * per_step) % len(inst):][:per_step]
            cpu_measure(pool, sample)
            step += 1
        total_ms, total_wall = 0, 0.0
        for _ in range(args.steps):
            sample = inst[(step * per_step) % len(inst):][:per_step]
            _, wall, res = cpu_measure(pool, sample)
            total_ms += sum(r[0] * r[1] for r in res)
            total_wall += wall
            step += 1
    finally:
        pool.close()
        pool.join()
    value = total_ms / total_wall
    sample_desc = (f"{per_step} instances per step (of the {WORKLOAD['instances']}), each run to tf=100 by the "
                   f"NumPy FP64 oracle, one instance per worker, {cores} workers ({cpu_model()})")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_wall / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp64",
        "data": "synthetic (seeded KS ensemble)",
        "config": {k: WORKLOAD[k] for k in ("workload", "instances", "n_choices", "L_range", "epsilon", "tf", "method")},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample_desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _cpu_single(args):
    """One process, one solver: the single-instance configurations timed by the oracle
    (the reference's algorithm), wall time inside the worker."""
    name = args[0]
    from oracle import rk_oracle as O
    if name == "ks1024_if34":
        lin, nl, u0 = args[1:]
        s = O.OracleSolver("IF34", lin, nl, O.SolverConfig())
        t0 = time.perf_counter()
        uf = s.evolve(u0, 0.0, 50.0, store_freq=20)
    else:
        lin, nl, u0 = args[1:]
        s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=1e-6))
        t0 = time.perf_counter()
        uf = s.evolve(u0, 0.0, 20.0, store_data=False)
    wall = time.perf_counter() - t0
    return name, wall, sum(1 for r in s.log if r[3]), s.attempts, s.nl_evals, uf


def _cpu_forms_reference(args):
    """A Burgers instance of the controller comparison to tf by the oracle at a tight
    epsilon (the accuracy reference of every form)."""
    idx, lin, nl, u0, eps, tf = args
    from oracle import rk_oracle as O
    s = O.OracleSolver("ETD35", lin, nl, O.SolverConfig(epsilon=eps))
    return idx, s.evolve(u0, 0.0, tf, store_data=False)


def single_instance_problems():
    """Configs 1 and 2 as (lin, nl, u0): KS n=1024 on [0, 32 pi) with u0 = cos(x/16)(1 +
    sin(x/16)), and the three-soliton NLS n=4096 on [-50, 50) (seed 0)."""
    from rkstiff_gb300 import grids, models, workloads

    x, kx = grids.construct_x_kx_rfft(1024, 0.0, 32 * np.pi)
    lin, nl = models.ks_ops(kx)
    ks = (lin, nl, np.fft.rfft(np.cos(x / 16) * (1 + np.sin(x / 16))))
    nls = workloads.nls_solitons(1, 0)[0]
    return ks, nls


def forms_reference_sample():
    """Indices of the Burgers set whose viscosity resolves the n=512 grid (nu > 5e-3; every
    form and the reference finish them), the first FORMS['reference_sample'] // 4 of them."""
    from rkstiff_gb300 import workloads

    inst = workloads.burgers_ensemble(FORMS["instances"], FORMS["seed"], n=FORMS["n"], nu_range=FORMS["nu_range"])
    nus = np.array([-float(np.real(lin[1])) for lin, _, _ in inst])
    idx = [int(i) for i in np.where(nus > 5e-3)[0][: FORMS["reference_sample"] // 4]]
    return inst, idx


def cpu_baseline_line(cores: int, dense: bool = False, extras: bool = False):
    """The KS ensemble's CPU baseline line and, with ``dense``, the dense config's (or None);
    with ``extras`` also the single-instance configs' one-process timings, the oracle's
    tf = 100 states of the sampled instances and the forms' tight-epsilon references."""
    inst = make_instances(WORKLOAD["instances"], WORKLOAD["seed"])
    sample = inst[: 4 * cores]
    pool = cpu_pool(cores)
    dense_line = None
    extra = {}
    try:
        if extras:
            ks, nls = single_instance_problems()
            singles = pool.map(_cpu_single, [("ks1024_if34",) + ks, ("nls4096_etd35",) + nls], chunksize=1)
            extra["single"] = {r[0]: {"seconds": r[1], "steps": r[2], "attempts": r[3], "nl_evals": r[4],
                                      "final": r[5]} for r in singles}
            finst, fidx = forms_reference_sample()
            refs = pool.map(_cpu_forms_reference, [(i, finst[i][0], finst[i][1], finst[i][2],
                                                    FORMS["reference_epsilon"], FORMS["tf"]) for i in fidx],
                            chunksize=1)
            extra["forms_ref"] = dict(refs)
        value, wall, res = cpu_measure(pool, sample)
        extra["tf_finals"] = {i: r[4] for i, r in enumerate(res) if r[3] == 0}
        if dense:
            from rkstiff_gb300 import workloads

            lin, nl, w0 = workloads.allen_cahn_batch(4 * cores, DENSE["seed"], epsilon=DENSE["epsilon_ac"])
            shift = np.asarray(nl.shift, dtype=np.float64)
            t0 = time.perf_counter()
            steps = pool.map(_cpu_dense_instance, [(lin, shift, w, DENSE["solver_epsilon"], DENSE["tf"]) for w in w0],
                             chunksize=1)
            dwall = time.perf_counter() - t0
            dense_line = {"value": 128.0 * sum(steps) / dwall, "unit": "mode-steps/s", "cores": cores,
                          "kind": "port", "instances_per_s": len(w0) / dwall,
                          "sample": f"first {len(w0)} ICs of the dense config to tf={DENSE['tf']} by the NumPy FP64 "
                                    f"oracle (diagonalized ETD35, per-IC controller), {cores} worker processes, "
                                    f"{dwall:.1f} s wall"}
    finally:
        pool.close()
        pool.join()
    return ({"value": value, "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"first {len(sample)} instances of the workload to tf=100 by the NumPy FP64 oracle, "
                       f"{cores} worker processes ({cpu_model()}), {wall:.1f} s wall"}, dense_line, extra)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the plain/learned Burgers comparison")
    ap.add_argument("--no-dense", action="store_true", help="skip the dense Allen-Cahn measurement")
    ap.add_argument("--no-single", action="store_true", help="skip the single-instance configs (KS n=1024, NLS n=4096)")
    ap.add_argument("--tune-cache", default="", help="JSON file of tuned launch shapes to load, or to write")
    ap.add_argument("--retune", action="store_true",
                    help="tune the launch shapes in the run instead of loading the committed GB300 tuning")
    ap.add_argument("--shapes", default="",
                    help="pin the launch shape of every grid-size class, e.g. "
                         "'2048:128x1:global,1024:128x1:global,512:128x1:smem-all,256:64x2:smem-all'")
    ap.add_argument("--instances", type=int, default=WORKLOAD["instances"], help="smaller cases for profiling")
    ap.add_argument("--sizes", default="", help="comma-separated subset of the grid sizes (profiling)")
    ap.add_argument("--tf", type=float, default=WORKLOAD["tf"], help="final time (profiling)")
    args = ap.parse_args()
    WORKLOAD["instances"] = args.instances
    WORKLOAD["tf"] = args.tf
    if args.sizes:
        WORKLOAD["n_choices"] = [int(v) for v in args.sizes.split(",")]
    world = int(os.environ.get("WORLD_SIZE", 1))
    rank = int(os.environ.get("RANK", 0))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    # the CPU baseline pool is spawned before any CUDA call
    cpu_line = dense_cpu = None
    extra = {}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_line, dense_cpu, extra = cpu_baseline_line(host_cores(), dense=not args.no_dense, extras=True)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        dist.init_process_group("nccl")
    gpu_arm(args, rank, world, cpu_line, dense_cpu, extra)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
