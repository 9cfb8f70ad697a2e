"""Tetrahedral mesh container with the members the FEM path reads.

Mirrors lapy/tet_mesh.py:14-60 (TetMesh): vertices ``v`` (n x 3), tetrahedra
``t`` (m x 4) and its index check; ``avg_edge_length`` runs on the GPU.
"""

from __future__ import annotations

import numpy as np


class TetMesh:
    """Tetrahedral mesh (v: n x 3 float, t: m x 4 int)."""

    def __init__(self, v, t):
        self.v = np.array(v)
        self.t = np.array(t)
        vnum = self.v.shape[0]
        if np.max(self.t) >= vnum:
            raise ValueError("Max index exceeds number of vertices")

    def avg_edge_length(self) -> float:
        """Mean edge length (lapy/tet_mesh.py:182-195), computed on the GPU."""
        from ._geometry import avg_edge_length

        return avg_edge_length(self)
