"""GB300 (sm_103a) implementation of FRICO's Method-of-Moments hot path.

The compute lives in libfrico_gpu.so (include/frico_gpu.h); this package is the
host-side mirror of FRICO's solver interface plus the synthetic workloads.
"""
from . import meshes  # noqa: F401
from ._abi import FricoError  # noqa: F401

__all__ = ["meshes", "FricoError", "build", "solver"]


def _build(verbose: bool = False, force: bool = False):
    from .build import build as _b
    # importing the submodule frico_gb300.build rebinds the package attribute
    # `build` to that module; put the function back so the call can be repeated
    globals()["build"] = _build
    return _b(verbose=verbose, force=force)


build = _build
