"""GB300-native velocity solve for UFEMISM 2.0 (SSA/DIVA Picard loop, mesh CSR operators,
CSR matrix-equation solve) and its column temperature solve, behind the C ABI of
include/ufe_gpu.h.

The directory name is not a Python identifier; load it with ``__graft_entry__.load_package()``,
which registers it as ``ufemism_gb300``.
"""
from . import abi, mesh, geometry  # noqa: F401
from .build import build  # noqa: F401
from .solver import CSR, UfeError, VelocitySolver, ensemble_solve, new_diva_state, new_ssa_state  # noqa: F401
from .thermo import ColumnSolver, zeta_operators  # noqa: F401
from . import thermo  # noqa: F401
from . import learned  # noqa: F401
from . import ensemble  # noqa: F401
from .learned import LearnedStart  # noqa: F401
