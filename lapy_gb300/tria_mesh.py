"""Triangle mesh container with the members the FEM path reads.

Mirrors the constructor contract of lapy/tria_mesh.py:182-280 (TriaMesh):
vertices ``v`` (n x 3, or n x 2 padded with z = 0), triangles ``t`` (m x 3),
the same validation errors.  Geometry work that lies on the FEM path
(``avg_edge_length`` and the curvature frame of the anisotropic Laplacian,
``curvature`` / ``curvature_tria``) runs on the GPU; ``refine_`` (host-side
mesh construction), the measures used by spectra normalisation and the text
file formats live in NumPy.
"""

from __future__ import annotations

import numpy as np
from scipy import sparse


class TriaMesh:
    """Triangle mesh (v: n x 3 float, t: m x 3 int)."""

    def __init__(self, v, t, fsinfo=None):
        self.v = np.array(v)
        self.t = np.array(t)
        if self.v.ndim == 2 and self.v.shape[0] < self.v.shape[1]:
            self.v = self.v.T
        if self.t.ndim == 2 and self.t.shape[1] != 3 and self.t.shape[0] == 3:
            self.t = self.t.T
        if self.t.size == 0:
            raise ValueError("Mesh has no triangles (empty mesh)")
        if self.v.size == 0:
            raise ValueError("Mesh has no vertices (empty mesh)")
        vnum = np.max(self.v.shape)
        if np.max(self.t) >= vnum:
            raise ValueError("Max index exceeds number of vertices")
        if self.t.shape[1] != 3:
            raise ValueError("Triangles should have 3 vertices")
        if self.v.shape[1] == 2:
            self.v = np.column_stack([self.v, np.zeros(self.v.shape[0], dtype=self.v.dtype)])
            self._is_2d = True
        elif self.v.shape[1] == 3:
            self._is_2d = False
        else:
            raise ValueError("Vertices should have 2 or 3 coordinates")
        self.fsinfo = fsinfo

    def is_2d(self) -> bool:
        return self._is_2d

    # -- text file formats (lapy/_tria_io.py; host) -------------------------
    @classmethod
    def read_off(cls, filename: str) -> "TriaMesh":
        """OFF file: optional ``#`` comment lines, ``OFF``, the counts, the
        vertices (read as float32, as the reference does) and ``3 i j k``
        faces (lapy/_tria_io.py:50-110)."""
        from ._meshio import read_off

        v, t = read_off(filename)
        return cls(v, t)

    @classmethod
    def read_vtk(cls, filename: str) -> "TriaMesh":
        """Legacy ASCII VTK with POLYGONS / CELLS of triangles or
        TRIANGLE_STRIPS (lapy/_tria_io.py:113-227)."""
        from ._meshio import read_vtk

        v, t = read_vtk(filename, 3)
        return cls(v, t)

    def write_vtk(self, filename: str) -> None:
        """Legacy ASCII VTK POLYDATA, in the reference's exact text
        (lapy/_tria_io.py:638-674)."""
        from ._meshio import write_vtk

        write_vtk(self.v, self.t, filename)

    @classmethod
    def read_fssurf(cls, filename: str) -> "TriaMesh":
        """FreeSurfer surface geometry with its volume-info footer in
        ``fsinfo`` (lapy/_tria_io.py:16-47, lapy/_read_geometry.py:112-197)."""
        from ._meshio import read_fssurf

        v, t, info = read_fssurf(filename)
        return cls(v, t, fsinfo=info)

    def write_fssurf(self, filename: str, image=None, coords_are_voxels=None) -> None:
        """FreeSurfer surface geometry, with ``fsinfo`` as the volume-info
        footer (lapy/_tria_io.py:677-760).  Converting voxel coordinates with
        an image header needs nibabel, as in the reference."""
        from ._meshio import write_fssurf

        if coords_are_voxels is None:
            coords_are_voxels = image is not None
        if coords_are_voxels and image is None:
            raise ValueError(
                "coords_are_voxels=True requires an image to be provided for voxel-to-surface-RAS "
                "coordinate conversion. Either provide an image or set coords_are_voxels=False.")
        if image is not None:
            import nibabel  # noqa: F401  (image headers are nibabel objects)

            raise NotImplementedError("image headers are not supported; pass coordinates in surface RAS")
        write_fssurf(self.v, self.t, filename, volume_info=self.fsinfo)

    # -- host-side adjacency (mesh construction only) ---------------------
    def _adj_sym(self) -> sparse.csc_matrix:
        t0, t1, t2 = self.t[:, 0], self.t[:, 1], self.t[:, 2]
        i = np.column_stack((t0, t1, t1, t2, t2, t0)).reshape(-1)
        j = np.column_stack((t1, t0, t2, t1, t0, t2)).reshape(-1)
        n = self.v.shape[0]
        return sparse.csc_matrix((np.ones(i.shape), (i, j)), shape=(n, n))

    def avg_edge_length(self) -> float:
        """Mean edge length (lapy/tria_mesh.py:735-748), computed on the GPU."""
        from ._geometry import avg_edge_length

        return avg_edge_length(self)

    # -- measures used to normalise spectra (host, O(m)) -------------------
    def _edge_counts(self, directed: bool) -> np.ndarray:
        e = np.concatenate([self.t[:, [0, 1]], self.t[:, [1, 2]], self.t[:, [2, 0]]])
        if not directed:
            e = np.sort(e, axis=1)
        return np.unique(e, axis=0, return_counts=True)[1]

    def is_closed(self) -> bool:
        """No boundary edge: every edge lies in two or more triangles
        (lapy/tria_mesh.py:562-572)."""
        return not np.any(self._edge_counts(directed=False) == 1)

    def is_oriented(self) -> bool:
        """Consistent orientation: no directed edge is used twice
        (lapy/tria_mesh.py:604-616)."""
        return int(self._edge_counts(directed=True).max()) == 1

    def tria_areas(self) -> np.ndarray:
        """Triangle areas by Heron's formula from the three edge lengths
        (lapy/tria_mesh.py:636-658)."""
        p0, p1, p2 = (self.v[self.t[:, i], :] for i in range(3))
        a = np.sqrt(np.sum((p1 - p0) ** 2, axis=1))
        b = np.sqrt(np.sum((p2 - p1) ** 2, axis=1))
        c = np.sqrt(np.sum((p0 - p2) ** 2, axis=1))
        s = 0.5 * (a + b + c)
        return np.sqrt(s * (s - a) * (s - b) * (s - c))

    def area(self) -> float:
        """Total surface area (lapy/tria_mesh.py:660-669)."""
        return np.sum(self.tria_areas())

    # -- curvature frame of the anisotropic Laplacian (host pre-step) -------
    def tria_normals(self) -> np.ndarray:
        """Unit triangle normals (lapy/tria_mesh.py:750-773)."""
        from . import _curvature

        return _curvature.tria_normals(self.v, self.t)

    def vertex_normals(self) -> np.ndarray:
        """Area-weighted vertex normals of an oriented mesh
        (lapy/tria_mesh.py:775-817)."""
        from . import _curvature

        if not self.is_oriented():
            raise ValueError("Error: Vertex normals are meaningless for un-oriented triangle meshes!")
        return _curvature.vertex_normals(self.v, self.t)

    def vertex_areas(self) -> np.ndarray:
        """One third of the incident triangle areas (lapy/tria_mesh.py:715-733)."""
        from . import _curvature

        return _curvature.vertex_areas(self.v, self.t)

    def smooth_laplace(self, vfunc=None, n: int = 1, lambda_: float = 0.5, mat=None) -> np.ndarray:
        """Laplace smoothing of a vertex function (default: the vertices)
        with the 1-ring averaging matrix (lapy/tria_mesh.py:1747-1792)."""
        from . import _curvature

        return _curvature.smooth_laplace(self.v, self.t, self.v if vfunc is None else vfunc, n, lambda_, mat)

    def map_vfunc_to_tfunc(self, vfunc) -> np.ndarray:
        """Triangle means of a vertex function (lapy/tria_mesh.py:1668-1694)."""
        from . import _curvature

        if self.v.shape[0] != np.asarray(vfunc).shape[0]:
            raise ValueError("Error: length of vfunc needs to match number of vertices")
        return _curvature.map_vfunc_to_tfunc(self.t, vfunc)

    def curvature(self, smoothit: int = 3):
        """Principal directions and curvatures at the vertices
        (lapy/tria_mesh.py:1078-1219), computed on the GPU: u_min, u_max,
        c_min, c_max, c_mean, c_gauss, normals."""
        from ._device import pattern_of, tria_curvature

        md, pat = pattern_of(self)
        vtx, _ = tria_curvature(md, pat, smoothit, vertex=True, triangle=False)
        b = vtx.cpu().numpy()
        n = md.n
        return (b[:3 * n].reshape(n, 3), b[3 * n:6 * n].reshape(n, 3), b[6 * n:7 * n], b[7 * n:8 * n],
                b[8 * n:9 * n], b[9 * n:10 * n], b[10 * n:].reshape(n, 3))

    def curvature_tria(self, smoothit: int = 3):
        """Principal directions and curvatures on the triangles, the frame of
        the anisotropic Laplace-Beltrami assembly (lapy/tria_mesh.py:1221-1279),
        computed on the GPU: u_min, u_max, c_min, c_max."""
        from ._device import pattern_of, tria_curvature

        md, pat = pattern_of(self)
        _, tri = tria_curvature(md, pat, smoothit, vertex=False, triangle=True)
        b = tri.cpu().numpy()
        m = md.m
        return b[:3 * m].reshape(m, 3), b[3 * m:6 * m].reshape(m, 3), b[6 * m:7 * m], b[7 * m:]

    def centroid(self) -> tuple[np.ndarray, float]:
        """Area-weighted mean of the triangle centres, and the total area
        (lapy/tria_mesh.py:990-1015)."""
        p0, p1, p2 = (self.v[self.t[:, i], :] for i in range(3))
        cr = np.cross(p2 - p1, p0 - p2)
        areas = 0.5 * np.sqrt(np.sum(cr * cr, axis=1))
        total = areas.sum()
        w = areas / total
        return np.sum(((p0 + p1 + p2) / 3.0) * w[:, np.newaxis], axis=0), total

    def normalize_(self) -> None:
        """Centroid to the origin, then scale to unit surface area
        (lapy/tria_mesh.py:1390-1405)."""
        c, area = self.centroid()
        if area <= 0:
            raise ValueError("Mesh surface area must be positive to normalize.")
        self.v = (1.0 / np.sqrt(area)) * (self.v - c)

    def volume(self) -> float:
        """Volume enclosed by a closed, oriented mesh: the signed volumes of
        the tetrahedra the triangles span with the origin
        (lapy/tria_mesh.py:671-703)."""
        if not self.is_closed():
            raise ValueError("Mesh must be closed to compute volume.")
        if not self.is_oriented():
            raise ValueError("Mesh must be oriented to compute volume.")
        p0, p1, p2 = (self.v[self.t[:, i], :] for i in range(3))
        return np.sum(np.sum(p0 * np.cross(p1 - p0, p2 - p0), axis=1)) / 6.0

    def refine_(self, it: int = 1) -> None:
        """1-to-4 midpoint subdivision (lapy/tria_mesh.py:1452-1487).

        New vertices are numbered after the old ones in row-major order of the
        upper-triangular edge list; each parent triangle (a, b, c) with edge
        midpoints ab, bc, ca becomes (a, ab, ca), (b, bc, ab), (c, ca, bc),
        (ab, bc, ca), in that order.
        """
        for _ in range(it):
            adj = sparse.triu(self._adj_sym(), 0, format="csr")
            vno = self.v.shape[0]
            rows, cols = adj.nonzero()
            eid = sparse.csr_matrix((np.arange(vno, vno + rows.size), (rows, cols)), shape=adj.shape)
            eid = (eid + eid.T).tocsr()
            vnew = np.append(self.v, 0.5 * (self.v[rows, :] + self.v[cols, :]), axis=0)
            t = self.t
            e1 = np.asarray(eid[t[:, 0], t[:, 1]]).ravel()
            e2 = np.asarray(eid[t[:, 1], t[:, 2]]).ravel()
            e3 = np.asarray(eid[t[:, 2], t[:, 0]]).ravel()
            tnew = np.column_stack((t[:, 0], e1, e3, t[:, 1], e2, e1, t[:, 2], e3, e2, e1, e2, e3)).reshape(-1, 3)
            self.__init__(vnew, tnew, self.fsinfo)
