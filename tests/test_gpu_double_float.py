"""The FP32 double-float state on a linear problem: the KS operator L = k^2 (1 - k^2) with the
u u_x nonlinearity switched off by its constant (c = 0, so N = 0 exactly), whose solution is
u(t) = e^{L t} u0.  The FP32 stepping kernels' only error is then rounding: the state is
carried as FP32 pairs, e^(z/2), e^(3z/4) and e^z are formed from the stored e^(z/4) by FP32
products, and the low word of e^z (stored with the coefficients) is taken against that
product, so 1000 steps end within the FP32 rounding of the returned state itself.

Tolerance (relative L2 against the FP64 exact solution): 2e-7.  The result is returned in
FP32 (about 4e-8 from its rounding alone); 1000 steps with an FP32 state, or with a low word
of e^z that does not belong to the e^z the stage code uses, leave 1e-6 .. 1e-4.
"""

import numpy as np
import pytest

import bench
from rkstiff_gb300 import _native as nat
from rkstiff_gb300 import models
from rkstiff_gb300.ensemble import Ensemble
from rkstiff_gb300.solveras import SolverConfig

pytestmark = pytest.mark.gpu

SIZES = (256, 512, 1024, 2048)
H, TF = 0.01, 10.0


def linear_instances(per_size=2, seed=11):
    inst = bench.make_instances(64, seed)
    out = []
    for n in SIZES:
        for n_, L, u0 in [i for i in inst if i[0] == n][:per_size]:
            kx, lin = bench.ks_operator(n_, L)
            out.append((lin, models.BuiltinNL(nat.RK_NL_UUX, 0.0, n_, kx, "ks_linear"), u0))
    return out


def exact(lin, u0, t):
    return np.exp(lin * t) * u0


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("method", ["ETD35", "ETD5"])
def test_fp32_double_float_state_on_linear_problem(method):
    inst = linear_instances()
    lins, nls, u0s = [i[0] for i in inst], [i[1] for i in inst], [i[2] for i in inst]
    # ETD35 (the compile-time class kernels): the zero error estimate gives s = 4, which an
    # increase factor of 10 never acts on, so h stays 0.01; ETD5 (the runtime-size kernel)
    # steps at h by definition
    cfg = SolverConfig(epsilon=1e-5, incr_f=10.0)
    ens = Ensemble(method, lins, nls, config=cfg, precision="fp32")
    out = ens.evolve(u0s, 0.0, TF, h_init=H)
    st = ens.stats()
    assert np.all(st["status"] == 0)
    # 1000 steps of 0.01, and one more: the sum of the steps falls short of tf by its rounding,
    # which ETD35 closes with a clamped last step and the constant-step ETD5 with a whole step
    # (the reference's loops do the same), so each result is compared at the time it reached
    assert np.all(np.abs(st["steps"] - round(TF / H)) <= 1), st["steps"]
    for k, (lin, _, u0) in enumerate(inst):
        ref = exact(lin, u0, float(st["t"][k]))
        assert rel(out[k].cpu().numpy(), ref) < 2e-7, (method, len(lin), rel(out[k].cpu().numpy(), ref))
