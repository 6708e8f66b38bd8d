"""HyperFlow-GB300: the reference solver's explicit finite-volume Euler time step
(Godunov / MUSCL-Hancock + HLLC, forward Euler) as hand-written CUDA for sm_103a
behind a C ABI (include/hyperflow_gb300.h)."""
from ._lib import HyperFlowError, lib  # noqa: F401
from .solver import CartSolver  # noqa: F401
from .uns import UnsSolver  # noqa: F401
from .batch import BatchSolver  # noqa: F401
from . import cases  # noqa: F401
