"""GB300-native (sm_103a) exact-diagonalisation Metropolis path for the
Falicov-Kimball Monte Carlo of aeantipov/fk_mc.

The compute runs in libfkg.so (hand-written CUDA, C ABI in include/fkg.h);
this package holds the Python handle on it (`Solver`), the lattice builders
and the build recipe. There is no CPU fallback.
"""
from .lattice import hopping_csr, dense  # noqa: F401


def build(force=False):
    from . import buildlib
    return buildlib.build(force=force)


def Solver(*a, **k):  # noqa: N802 - factory keeps import of the CUDA library lazy
    from .solver import Solver as _S
    return _S(*a, **k)
