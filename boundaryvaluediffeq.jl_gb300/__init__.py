"""GB300-native batched MIRK boundary-value solver (host side).

The compute path is libbvpgpu.so (include/bvpgpu.h): JIT-compiled sm_103a kernels for the
MIRK collocation residual, the forward-mode Jacobian blocks, the structured block
factorisation and the defect estimate, driven per instance by a persistent kernel.
"""
from . import problems  # noqa: F401
from ._lib import build_library, load_library, LIB_PATH, EXPORTS  # noqa: F401
from .solver import BatchSolver, BatchResult, BVPError, RET_SUCCESS, RET_FAILURE, RET_MAXITERS  # noqa: F401
from .surrogate import MLP, Surrogate, resample_host  # noqa: F401
from . import sciml  # noqa: F401
from .sciml import solve, EnsembleProblem, MIRK2, MIRK3, MIRK4, MIRK5, MIRK6, MIRK6I  # noqa: F401
from .sciml import (DefectControl, GlobalErrorControl, SequentialErrorControl, HybridErrorControl,  # noqa: F401
                    HOErrorControl, REErrorControl)
from .sciml import (FIRK, RadauIIa1, RadauIIa2, RadauIIa3, RadauIIa5, RadauIIa7, LobattoIIIa2,  # noqa: F401
                    LobattoIIIa3, LobattoIIIa4, LobattoIIIa5, LobattoIIIb2, LobattoIIIb3, LobattoIIIb4, LobattoIIIb5,
                    LobattoIIIc2, LobattoIIIc3, LobattoIIIc4, LobattoIIIc5)
