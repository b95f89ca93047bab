"""goosefem_gb300 — GooseFEM's element hot path on GB300 (sm_103a).

The Python mirror of the GooseFEM interface for the hot path (Mesh Regular meshes, Vector,
Element Quad4/Hex8 quadrature (+ Quad4 planar), MatrixDiagonal(Partitioned), assembled
Matrix(Partitioned) with an iterative partitioned solver, the explicit velocity-Verlet step). All computation runs in hand-written CUDA kernels of libgfgpu.so behind the C ABI of
include/gfgpu.h; importing this package fails if that library has not been built.
"""

from . import _lib

_lib.lib()  # fail loudly if libgfgpu.so is missing

from . import mesh as Mesh  # noqa: E402
from . import element as Element  # noqa: E402
from .vector import Vector, VectorPartitioned  # noqa: E402
from .matrix import MatrixDiagonal, MatrixDiagonalPartitioned  # noqa: E402
from .matrix import Matrix, MatrixPartitioned, MatrixPartitionedSolver, MatrixSolver  # noqa: E402
from . import tyings as Tyings  # noqa: E402
from .tyings import VectorPartitionedTyings, MatrixPartitionedTyings  # noqa: E402
from .tyings import MatrixPartitionedTyingsSolver  # noqa: E402
from .dynamics import VelocityVerlet, elastic_stress, critical_dt  # noqa: E402
from . import statics  # noqa: E402
from .statics import ElasticStatic  # noqa: E402
from ._lib import set_strict, GFGPUError  # noqa: E402

__all__ = ["Mesh", "Element", "Vector", "VectorPartitioned", "MatrixDiagonal",
           "MatrixDiagonalPartitioned", "Matrix", "MatrixPartitioned", "MatrixPartitionedSolver", "MatrixSolver",
           "Tyings", "VectorPartitionedTyings", "MatrixPartitionedTyings",
           "MatrixPartitionedTyingsSolver", "VelocityVerlet", "elastic_stress", "critical_dt",
           "set_strict", "GFGPUError"]
