"""GB300-native nodal linear-elastic operator and multigrid solve (libaefast.so).

The compute path is the CUDA library built from csrc/ for sm_103a; this package holds
its ctypes binding (_lib), the stiffness-model constructors (models), the seeded
microstructure generators (microstructure) and a mirror of the reference's
Operator/BC/Solver interface (elastic)."""
from . import _lib, models  # noqa: F401
from ._lib import AeError  # noqa: F401

__all__ = ["AeError", "models", "elastic"]
