"""GB300-native particle-mesh gravity step (drop-in for the step of
tugrul512bit/CosmosSimulationWithCuda's Universe class).

The product is the CUDA library libcosmos_pm.so with the C ABI in
include/cosmos_pm.h and the C++ Universe shim in include/CosmosGB300.cuh; this
package holds its sources (csrc/), its build (build.py), a ctypes binding
(_lib.py) and seeded initial conditions (ics.py).
"""
from . import ics  # noqa: F401


def build(force: bool = False) -> str:
    from ._build import build as _build
    return _build(force=force)


def load():
    from . import _lib
    return _lib.load()
