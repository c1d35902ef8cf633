"""GB300-native semi-discrete optimal transport (the MongeAmpere++ hot path).

Laguerre cells of weighted sites intersected with a triangulated piecewise-linear
density, computed by hand-written sm_103a CUDA kernels behind the C ABI of
``include/ma.h``: Kantorovich value, cell masses, sparse Hessian, the damped Newton
OT solve, moments and Lloyd.  The CUDA library is loaded on first use; there is no
CPU fallback.
"""
from .mesh import GridMesh, TriMesh, unit_grid  # noqa: F401

__all__ = ["GridMesh", "TriMesh", "unit_grid", "Context", "kantorovich", "ot_solve", "lloyd", "first_moment",
           "second_moment", "solve_laplacian_matrix", "Statistics"]


def __getattr__(name):
    if name in ("Context", "DeviceMesh", "kantorovich", "ot_solve", "lloyd", "first_moment", "second_moment",
                "solve_laplacian_matrix", "Statistics", "Hessian", "default_context"):
        from . import api
        return getattr(api, name)
    raise AttributeError(name)
