"""GB300-native HelmholtzBEM assembly-and-resonance path.

CUDA kernels for sm_103a behind the C ABI in include/hbem.h (libhbem.so), with
a Python mirror of the reference's GalerkinBuilder / SolutionsOperator /
direct::sv / find_roots interface in ``helmholtzbem_gb300.api``.
"""
import os

# Up to 24 streams run at once in the plain search; with CUDA's default of 8 hardware
# work queues, launches of one stream wait behind unrelated launches of another that
# shares its queue.  The setting only takes effect if no CUDA context exists yet
# (import this package before anything initialises CUDA); a value already set wins.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import geometry  # noqa: E402,F401
from ._capi import LAYER_ALL, LAYER_DOUBLE, LAYER_HYPERSINGULAR, LAYER_SINGLE  # noqa: E402,F401

__all__ = ["geometry", "api", "build"]


def build(**kw):
    from .build import build as _b
    return _b(**kw)
