"""CPU oracle for the rkstiff stepping path (test infrastructure, not product code).

This package restates, in NumPy FP64, the algorithm that whalenpt/rkstiff runs on its
time-stepping hot path: the psi-coefficient setup, the stage programs of the seven
solvers, the embedded error norm, the accept/reject step-size controller and the
evolve loops.  It is pinned against golden vectors that were produced by running the
reference itself (``tests/golden/make_golden.py``).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline``
leg and ``--impl reference`` arm) may import this package, and only as the checker /
CPU baseline.  The product package ``rkstiff_gb300`` never imports it.
"""

from .rk_oracle import (  # noqa: F401
    SolverConfig,
    ETDConfig,
    MaxLoopsExceeded,
    MinimumStepReached,
    psi1,
    psi2,
    psi3,
    diag_coeffs,
    OracleSolver,
    METHODS,
    ADAPTIVE_METHODS,
    CONSTANT_METHODS,
)
