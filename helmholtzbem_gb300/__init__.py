"""GB300-native HelmholtzBEM assembly-and-resonance path.

CUDA kernels for sm_103a behind the C ABI in include/hbem.h (libhbem.so), with
a Python mirror of the reference's GalerkinBuilder / SolutionsOperator /
direct::sv / find_roots interface in ``helmholtzbem_gb300.api``.
"""
from . import geometry  # noqa: F401
from ._capi import LAYER_ALL, LAYER_DOUBLE, LAYER_HYPERSINGULAR, LAYER_SINGLE  # noqa: F401

__all__ = ["geometry", "api", "build"]


def build(**kw):
    from .build import build as _b
    return _b(**kw)
