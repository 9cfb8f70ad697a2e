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

    @classmethod
    def read_gmsh(cls, filename: str) -> "TetMesh":
        """ASCII gmsh 2.x file of tetrahedra (lapy/_tet_io.py:17-128); the
        element node ids are taken as stored."""
        from ._meshio import read_gmsh_tet

        v, t = read_gmsh_tet(filename)
        return cls(v, t)

    @classmethod
    def read_vtk(cls, filename: str) -> "TetMesh":
        """Legacy ASCII VTK with POLYGONS / CELLS of tetrahedra
        (lapy/_tet_io.py:131-224)."""
        from ._meshio import read_vtk

        v, t = read_vtk(filename, 4)
        return cls(v, t)

    def write_vtk(self, filename: str) -> None:
        """Legacy ASCII VTK, in the reference's exact text
        (lapy/_tet_io.py:227-259)."""
        from ._meshio import write_vtk

        write_vtk(self.v, self.t, filename)

    def avg_edge_length(self) -> float:
        """Mean edge length (lapy/tet_mesh.py:182-195), computed on the GPU."""
        from ._geometry import avg_edge_length

        return avg_edge_length(self)

    def boundary_volume(self) -> float:
        """Volume enclosed by the boundary surface: the faces that belong to a
        single tetrahedron, each oriented away from its tetrahedron, summed as
        signed volumes with the origin.  This is the measure ShapeDNA
        normalises by (lapy/shapedna.py:50-70: the boundary mesh, oriented,
        then its volume); host, O(m)."""
        t = np.asarray(self.t)
        p = [self.v[t[:, i], :] for i in range(4)]
        flip = np.sum(np.cross(p[1] - p[0], p[2] - p[0]) * (p[3] - p[0]), axis=1) < 0
        # faces opposite vertex 0, 1, 2, 3, outward for a positive tetrahedron
        faces = np.vstack([t[:, [3, 1, 2]], t[:, [2, 0, 3]], t[:, [1, 3, 0]], t[:, [0, 2, 1]]])
        fl = np.tile(flip, 4)
        faces[fl] = faces[fl][:, [0, 2, 1]]
        _, inv, cnt = np.unique(np.sort(faces, axis=1), axis=0, return_inverse=True, return_counts=True)
        bnd = faces[cnt[inv.ravel()] == 1]
        q0, q1, q2 = (self.v[bnd[:, i], :] for i in range(3))
        return np.sum(np.sum(q0 * np.cross(q1 - q0, q2 - q0), axis=1)) / 6.0
