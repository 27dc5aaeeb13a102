"""exwave_gb300: GB300-native (sm_103a) explicit DG operator hot path of
ExWave -- the upwind DG operator for the first-order acoustic system, the
low-storage RK stage update and the ADER Cauchy-Kovalevskaya sweep -- as
CUDA kernels behind a C ABI (include/exwave_gb300.h)."""
from .mesh import Mesh, hypercube, layered_materials, time_step_size  # noqa: F401
from .operator import WaveEquationOperation, reference_mode  # noqa: F401
from .time_integrators import (SSPRK, AderAdconFull, ArbitraryHighOrderDG, ClassRK4,  # noqa: F401
                               ExplicitEuler, LowStorageRK33Reg2, LowStorageRK45Reg2,
                               LowStorageRK45Reg3, LowStorageRK59Reg2)
from .utilities import TimeControl  # noqa: F401
from . import basis, vtu  # noqa: F401
