"""GPU drop-in for ``lapy.shapedna.compute_shapedna`` (lapy/shapedna.py:96-166),
plus a batched form that computes the spectra of many meshes in one
block-diagonal assembly and one batched eigensolve."""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._device import DeviceCSR, MeshDevice, assemble, build_pattern, dptr, require_cuda, stream
from .solver import DEFAULT_BLOCK, Solver, eigs_batched


def _ev_dict(geom, k, evals, evecs) -> dict:
    d = {"Refine": 0, "Degree": 1}
    if type(geom).__name__ == "TriaMesh":
        d["Dimension"] = 2
    elif type(geom).__name__ == "TetMesh":
        d["Dimension"] = 3
    d["Elements"] = len(geom.t)
    d["DoF"] = len(geom.v)
    d["NumEW"] = k
    d["Eigenvalues"] = evals
    d["Eigenvectors"] = evecs
    return d


def compute_shapedna(geom, k: int = 50, lump: bool = False, aniso=None, aniso_smooth: int = 10,
                     use_cholmod: bool = False) -> dict:
    """ShapeDNA descriptor (eigenvalues and eigenvectors) of one mesh."""
    fem = Solver(geom, lump=lump, aniso=aniso, aniso_smooth=aniso_smooth, use_cholmod=use_cholmod)
    evals, evecs = fem.eigs(k=k)
    return _ev_dict(geom, k, evals, evecs)


def _positive_measure(value: float, name: str) -> float:
    if value <= 0:
        raise ValueError(f"{name} must be positive for normalization")
    return value


def normalize_ev(geom, evals: np.ndarray, method: str = "geometry") -> np.ndarray:
    """Eigenvalues scaled to unit surface area ('surface'), unit volume
    ('volume': the enclosed volume of a closed triangle mesh, or of a
    tetrahedral mesh's boundary, to the power 2/3) or by the mesh type
    ('geometry': surface for triangles, volume for tetrahedra), as
    lapy/shapedna.py:169-227.  Host arithmetic on the k eigenvalues; the
    measures are O(m) host sums."""
    geom_type = type(geom).__name__
    if method == "surface":
        return evals * _positive_measure(geom.area(), "area")
    if method == "volume":
        if geom_type == "TriaMesh":
            return evals * _positive_measure(geom.volume(), "volume") ** (2.0 / 3.0)
        if geom_type == "TetMesh":
            return evals * _positive_measure(geom.boundary_volume(), "boundary volume") ** (2.0 / 3.0)
        raise ValueError("Unsupported geometry type for volume normalization")
    if method == "geometry":
        if geom_type == "TriaMesh":
            return evals * _positive_measure(geom.area(), "area")
        if geom_type == "TetMesh":
            return evals * _positive_measure(geom.boundary_volume(), "boundary volume") ** (2.0 / 3.0)
        raise ValueError("Unsupported geometry type for geometry normalization")
    raise ValueError(f"Unknown normalization method: {method}")


def reweight_ev(evals: np.ndarray) -> np.ndarray:
    """Eigenvalue i (0-based) divided by i + 1 (lapy/shapedna.py:230-255)."""
    return evals / np.arange(1, len(evals) + 1)


def compute_distance(ev1: np.ndarray, ev2: np.ndarray, dist: str = "euc") -> float:
    """Euclidean distance of two spectra; other measures raise ValueError as
    in lapy/shapedna.py:258-295."""
    if dist != "euc":
        raise ValueError(f"Distance metric {dist} is not implemented.")
    from scipy.spatial import distance

    return distance.euclidean(ev1, ev2)


class BatchInput:
    """Meshes of one element type concatenated on the device.

    Vertex arrays are stacked and element indices offset, so the batch is one
    mesh whose connected pieces are the input meshes; its matrices are block
    diagonal, one block (segment) per mesh."""

    def __init__(self, meshes):
        require_cuda()
        if not meshes:
            raise ValueError("empty batch")
        L = _lib.lib()
        npe = np.asarray(meshes[0].t).shape[1]
        f32 = all(np.asarray(m.v).dtype == np.float32 for m in meshes)
        vdt = np.float32 if f32 else np.float64
        vs, ts, seg, segel = [], [], [0], [0]
        for m in meshes:
            t = np.asarray(m.t)
            if t.ndim != 2 or t.shape[1] != npe:
                raise ValueError("a batch holds meshes of one element type")
            v = np.ascontiguousarray(m.v, dtype=vdt)
            vs.append(v)
            ts.append(t)
            seg.append(seg[-1] + len(v))
            segel.append(segel[-1] + len(t))
        if seg[-1] >= 2**31 or segel[-1] * npe >= 2**31:
            raise ValueError("batch exceeds the int32 index range")
        idx64 = not all(t.dtype == np.int32 for t in ts)
        ts = [np.ascontiguousarray(t, dtype=np.int64 if idx64 else np.int32) for t in ts]
        n, m_tot, nseg = seg[-1], segel[-1], len(meshes)
        s = stream()
        # the meshes' arrays are gathered into one pinned host buffer (by the
        # library, on a few host threads) and sent with one copy per array
        # kind: many small copies from pageable memory were several times
        # slower, and their cost varied from call to call
        vbytes = sum(a.nbytes for a in vs)
        tbytes = sum(a.nbytes for a in ts)
        pinned = torch.empty(vbytes + tbytes, dtype=torch.uint8, pin_memory=True)

        def upload(arrays, out, off, nbytes):
            ptrs = (C.c_void_p * len(arrays))(*[a.ctypes.data for a in arrays])
            sizes = (C.c_size_t * len(arrays))(*[a.nbytes for a in arrays])
            _lib.check(L.lapy_h2d_concat(len(arrays), ptrs, sizes, dptr(out), pinned.data_ptr() + off, nbytes, s),
                       "h2d_concat")

        # every mesh's arrays into the device buffers; the element indices are
        # offset (and checked) on the device
        v = torch.empty((n, 3), dtype=torch.float32 if f32 else torch.float64, device="cuda")
        upload(vs, v, 0, vbytes)
        traw = torch.empty((m_tot, npe), dtype=torch.int64 if idx64 else torch.int32, device="cuda")
        upload(ts, traw, vbytes, tbytes)
        self.seg_row = np.array(seg, dtype=np.int32)
        self.seg_elem = np.array(segel, dtype=np.int32)
        self.seg_row_dev = torch.from_numpy(self.seg_row).to("cuda")
        self.seg_elem_dev = torch.from_numpy(self.seg_elem).to("cuda")
        t = torch.empty((m_tot, npe), dtype=torch.int32, device="cuda")
        segmax = torch.empty(nseg + 1, dtype=torch.int32, device="cuda")
        _lib.check(L.lapy_seg_offset_elements(m_tot, npe, nseg, dptr(self.seg_elem_dev), dptr(self.seg_row_dev),
                                              dptr(traw), int(idx64), dptr(t), dptr(segmax), s), "seg_offset_elements")
        sm = segmax.cpu().numpy()  # also the end of the copies out of `pinned`
        del pinned
        if sm[nseg] != 0:
            raise ValueError("element indices outside their mesh's vertices")
        if np.any(sm[:nseg] + 1 != np.diff(self.seg_row)):
            raise ValueError("batched meshes must reference every vertex")
        self.mesh = MeshDevice(v, t, n, n, m_tot, npe)


class BatchedFEM:
    """Block-diagonal stiffness and mass of a batch, assembled on the device.

    Each mesh's degenerate elements are clamped with that mesh's own mean
    element measure, as a separate ``Solver`` per mesh would
    (lapy/solver.py:158-159)."""

    def __init__(self, meshes=None, lump: bool = False, _input: BatchInput | None = None):
        inp = _input if _input is not None else BatchInput(meshes)
        pat = build_pattern(inp.mesh)
        a, m = assemble(inp.mesh, pat, lump, seg_elem=inp.seg_elem_dev)
        self.input = inp
        self.pattern = pat
        self.seg_row = inp.seg_row
        self.indptr, self.indices = pat.indptr, pat.indices
        self.a_vals, self.m_vals = a, m
        self.m_is_diag = bool(lump)
        self.n = pat.n
        self.nnz = pat.nnz

    @classmethod
    def from_input(cls, inp: BatchInput, lump: bool = False) -> "BatchedFEM":
        return cls(lump=lump, _input=inp)

    def eigs(self, k: int = 50, sigma: float = -0.01, block: int = DEFAULT_BLOCK, **kw):
        return eigs_batched(self.indptr, self.indices, self.a_vals, self.m_vals, self.m_is_diag, self.seg_row, k,
                            sigma, block, **kw)


def compute_shapedna_batch(meshes, k: int = 50, lump: bool = False, block: int = 2,
                           return_vectors: bool = True, tuning: dict | str | None = None, **kw) -> list[dict]:
    """ShapeDNA of many meshes in one batched shift-invert Lanczos solve.

    ``tuning``: solver knobs (see ``lapy_gb300.autotune``), or ``"auto"`` for
    the choice cached for this batch's shape class on this device (the
    defaults when none was calibrated; the block width then comes from the
    choice too)."""
    if tuning == "auto":
        from . import autotune

        choice = autotune.choice_for(meshes, k)
        block = int(choice["block"])
        tuning = autotune.solver_tuning(choice)
    batch = BatchedFEM(meshes, lump=lump)
    evals, evecs, info = batch.eigs(k=k, block=block, tuning=tuning, **kw)
    bad = [int(s) for s in info["status"] if s != 0]
    if bad:
        _lib.check(bad[0], "compute_shapedna_batch")
    ev = evals.cpu().numpy()
    vec = evecs.cpu().numpy() if return_vectors else None
    out = []
    for i, geom in enumerate(meshes):
        r0, r1 = batch.seg_row[i], batch.seg_row[i + 1]
        out.append(_ev_dict(geom, k, ev[i], vec[r0:r1] if vec is not None else None))
    return out


__all__ = ["compute_shapedna", "compute_shapedna_batch", "BatchedFEM", "BatchInput", "DeviceCSR"]
