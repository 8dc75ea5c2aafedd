"""rheotool_gb300: GB300-native rheoFoam time-step hot path (sm_103a CUDA behind a C ABI)."""
from . import abi, mesh, case  # noqa: F401
