"""carpio_gb300: the projection hot path of hyperpower/carpios, GB300-native.

The product is libcarpio_gpu.so (C ABI in include/carpio_gpu.h; CUDA kernels
for sm_103a in csrc/). This package is the Python host mirror of the
reference's interfaces over that ABI:

  carpio_gb300.algebra    carpio::CG / Jacobi / Dia_BiCGSTAB / BiCGSTAB on CSR
  carpio_gb300.structure  Grid_, BoundaryCondition, Poisson_, NS_explicit_

Importing the package does not need a GPU; calls do, and they fail loudly
when the library or the device is missing.
"""
from . import _lib  # noqa: F401

__all__ = ["algebra", "structure", "build"]


def build(verbose=False, force=False):
    """Compiles libcarpio_gpu.so in place (carpio_gb300/compile.py)."""
    from . import compile as _c
    return _c.build(verbose=verbose, force=force)
