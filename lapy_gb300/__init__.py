"""lapy_gb300: the linear-FEM Laplace-Beltrami path of LaPy on GB300 (sm_103a).

Drop-in replacements for ``lapy.Solver`` (assembly, ``eigs``, ``poisson``),
``lapy.heat.diffusion``, the heat-method geodesics of ``lapy.diffgeo`` and
``lapy.shapedna.compute_shapedna``, computed by hand-written CUDA kernels
behind the C ABI of ``include/lapy_gb300.h``.
"""

from .solver import Solver
from .tet_mesh import TetMesh
from .tria_mesh import TriaMesh

__all__ = ["Solver", "TetMesh", "TriaMesh"]
__version__ = "0.1.0"
