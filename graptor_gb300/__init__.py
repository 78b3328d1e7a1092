"""GB300-native primal-dual TGV/TV tomographic reconstruction.

Drop-in for the device side of Graptor's solver: ``Reconstructionapproach2d`` /
``Reconstructionapproach3d`` (radon_tgv_primal_dual_{2d,3d}.py:69) run here on
hand-written sm_103a CUDA kernels behind a C ABI (include/graptor_gb300.h).
"""
from ._lib import GraptorError, GraptorMemoryError, GraptorTimeoutError  # noqa: F401

__all__ = ["GraptorError", "GraptorMemoryError", "GraptorTimeoutError"]
