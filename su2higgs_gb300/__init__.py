"""su2higgs_gb300: GB300 (sm_103a) implementation of su2higgs's checkerboard
lattice update sweep behind a C ABI (include/su2gpu.h)."""
from . import abi  # noqa: F401
