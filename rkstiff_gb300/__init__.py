"""rkstiff_gb300: the time-stepping hot path of rkstiff (ETD/IF Runge-Kutta solvers for
stiff PDEs u_t = L u + N(u)) as GB300 (sm_103a) CUDA kernels behind rkstiff's solver API.

    from rkstiff_gb300 import grids, models, ETD35, SolverConfig
    x, kx = grids.construct_x_kx_rfft(1024, 0.0, 32 * np.pi)
    lin_op, nl_func = models.ks_ops(kx)
    solver = ETD35(lin_op, nl_func, config=SolverConfig(epsilon=1e-4))
    u_final = solver.evolve(u0_fft, t0=0.0, tf=50.0, store_freq=20)

The native library is built in-tree on first use (``rkstiff_gb300._build.build()``).
"""

from . import derivatives, grids, models, transforms  # noqa: F401
from .device import DeviceOptions  # noqa: F401
from .etd import ETDAS, ETDCS, ETDConfig, psi1, psi2, psi3  # noqa: F401
from .etd34 import ETD34  # noqa: F401
from .etd35 import ETD35  # noqa: F401
from .etd4 import ETD4  # noqa: F401
from .etd5 import ETD5  # noqa: F401
from .if34 import IF34  # noqa: F401
from .if4 import IF4  # noqa: F401
from .if45dp import IF45DP  # noqa: F401
from .solveras import BaseSolverAS, SolverConfig  # noqa: F401
from .solvercs import BaseSolverCS  # noqa: F401
from .util.solver_type import SolverType  # noqa: F401

__version__ = "0.1.0"
