"""Device-side building blocks shared by the LaPy-compatible façade.

PyTorch is used only for device memory and the current CUDA stream; every
computation is a call into the CUDA library through ``lapy_gb300._lib``.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch
from scipy import sparse

from . import _lib

__all__ = [
    "DeviceCSR", "FemPattern", "MeshDevice", "mesh_device", "build_pattern", "assemble",
    "require_cuda", "stream", "dptr", "workspace",
]


def require_cuda() -> torch.device:
    """Return the CUDA device; raise when no GPU is usable (no CPU fallback)."""
    if not torch.cuda.is_available():
        raise RuntimeError("lapy_gb300 needs a CUDA GPU (sm_103a); no CPU fallback exists")
    _lib.lib()
    return torch.device("cuda", torch.cuda.current_device())


def stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def dptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous()
    return t.data_ptr()


def workspace(nbytes: int) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device="cuda")


@dataclass
class MeshDevice:
    """Vertex and element arrays of a mesh on the device."""

    v: torch.Tensor          # n x 3, float32 or float64 (the mesh's own dtype)
    t: torch.Tensor          # m x npe, int32
    n: int                   # matrix dimension (max index + 1, as SciPy infers it)
    nv: int                  # number of vertices
    m: int
    npe: int

    @property
    def coords_f32(self) -> int:
        return 1 if self.v.dtype == torch.float32 else 0


def mesh_device(mesh) -> MeshDevice:
    """Upload (and cache on the mesh object) the vertex/element arrays."""
    v = np.asarray(mesh.v)
    t = np.asarray(mesh.t)
    key = (v.__array_interface__["data"][0], v.shape, v.dtype.str, t.__array_interface__["data"][0], t.shape)
    cache = getattr(mesh, "_gb300_dev", None)
    if cache is not None and cache[0] == key:
        return cache[1]
    require_cuda()
    if v.dtype != np.float32:
        v = v.astype(np.float64, copy=False)
    if t.size and (t.min() < 0 or t.max() >= 2**31 - 1):
        raise ValueError("element indices out of the int32 range")
    vd = torch.from_numpy(np.ascontiguousarray(v)).to("cuda")
    td = torch.from_numpy(np.ascontiguousarray(t, dtype=np.int32)).to("cuda")
    n = int(t.max()) + 1 if t.size else 0
    md = MeshDevice(vd, td, n, v.shape[0], t.shape[0], t.shape[1])
    try:
        mesh._gb300_dev = (key, md)
    except AttributeError:
        pass
    return md


@dataclass
class FemPattern:
    """CSR pattern of the assembled matrices plus the assembly map."""

    n: int
    nnz: int
    npe: int
    indptr: torch.Tensor     # n+1 int32
    indices: torch.Tensor    # nnz int32
    seg_ptr: torch.Tensor    # nnz+1 int32
    seg_src: torch.Tensor    # m*L int32
    diag_pos: torch.Tensor   # n int32


def build_pattern(md: MeshDevice) -> FemPattern:
    L = _lib.lib()
    s = stream()
    ws_bytes = L.lapy_csr_symbolic_workspace_bytes(md.n, md.m, md.npe)
    ws = workspace(ws_bytes)
    indptr = torch.empty(md.n + 1, dtype=torch.int32, device="cuda")
    nnz = C.c_int64(0)
    _lib.check(L.lapy_csr_symbolic_count(dptr(md.t), md.m, md.npe, md.n, dptr(indptr), C.byref(nnz),
                                         dptr(ws), ws.numel(), s), "csr_symbolic_count")
    nnz = int(nnz.value)
    indices = torch.empty(nnz, dtype=torch.int32, device="cuda")
    seg_ptr = torch.empty(nnz + 1, dtype=torch.int32, device="cuda")
    seg_src = torch.empty(md.m * md.npe * md.npe, dtype=torch.int32, device="cuda")
    _lib.check(L.lapy_csr_symbolic_fill(dptr(md.t), md.m, md.npe, md.n, dptr(indptr), nnz, dptr(indices),
                                        dptr(seg_ptr), dptr(seg_src), dptr(ws), ws.numel(), s),
               "csr_symbolic_fill")
    diag = torch.empty(md.n, dtype=torch.int32, device="cuda")
    _lib.check(L.lapy_csr_diag_index(md.n, dptr(indptr), dptr(indices), dptr(diag), s), "csr_diag_index")
    return FemPattern(md.n, nnz, md.npe, indptr, indices, seg_ptr, seg_src, diag)


def pattern_of(mesh) -> tuple[MeshDevice, FemPattern]:
    """Device arrays and (cached) CSR pattern of a mesh."""
    md = mesh_device(mesh)
    pat = getattr(md, "_pattern", None)
    if pat is None:
        pat = build_pattern(md)
        md._pattern = pat
    return md, pat


def assemble(md: MeshDevice, pat: FemPattern, lump: bool, out_dtype=torch.float64, aniso=None,
             seg_elem: torch.Tensor | None = None):
    """Numeric assembly: returns (A values on the pattern, M values or M diagonal).

    ``seg_elem`` (device int32, nseg+1 element offsets) marks a batch of
    concatenated meshes: each mesh's degenerate elements are then clamped with
    its own mean element measure (lapy/solver.py:158-159)."""
    L = _lib.lib()
    s = stream()
    out_f32 = 1 if out_dtype == torch.float32 else 0
    a = torch.empty(pat.nnz, dtype=out_dtype, device="cuda")
    mvals = torch.empty(pat.n if lump else pat.nnz, dtype=out_dtype, device="cuda")
    if seg_elem is not None:
        if aniso is not None:
            raise ValueError("batched assembly has no anisotropic form")
        nseg = seg_elem.numel() - 1
        ws = workspace(L.lapy_fem_batch_numeric_workspace_bytes(md.m, md.npe, nseg))
        _lib.check(L.lapy_fem_batch_numeric(md.npe, dptr(md.v), md.coords_f32, dptr(md.t), md.m, nseg,
                                            dptr(seg_elem), md.n, dptr(pat.indptr), dptr(pat.indices),
                                            dptr(pat.seg_ptr), dptr(pat.seg_src), pat.nnz, int(bool(lump)),
                                            out_f32, dptr(a), dptr(mvals), dptr(ws), ws.numel(), s),
                   "fem_batch_numeric")
        return a, mvals
    ws = workspace(L.lapy_fem_numeric_workspace_bytes(md.m, md.npe))
    common = (md.n, dptr(pat.indptr), dptr(pat.indices), dptr(pat.seg_ptr), dptr(pat.seg_src), pat.nnz,
              int(bool(lump)), out_f32, dptr(a), dptr(mvals), dptr(ws), ws.numel(), s)
    if md.npe == 4:
        st = L.lapy_fem_tet_numeric(dptr(md.v), md.coords_f32, dptr(md.t), md.m, *common)
        where = "fem_tet_numeric"
    elif aniso is None:
        st = L.lapy_fem_tria_numeric(dptr(md.v), md.coords_f32, dptr(md.t), md.m, *common)
        where = "fem_tria_numeric"
    else:
        u1, u2, am = (x.contiguous() if isinstance(x, torch.Tensor)
                      else torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to("cuda") for x in aniso)
        st = L.lapy_fem_tria_aniso_numeric(dptr(md.v), md.coords_f32, dptr(md.t), md.m, dptr(u1), dptr(u2),
                                           dptr(am), *common)
        where = "fem_tria_aniso_numeric"
    _lib.check(st, where)
    return a, mvals


class DeviceCSR:
    """A symmetric n x n matrix on the device: CSR arrays, or a diagonal."""

    def __init__(self, n, indptr=None, indices=None, data=None, diag=None):
        self.n = int(n)
        self.indptr = indptr
        self.indices = indices
        self.data = data
        self.diag = diag

    @property
    def is_diag(self) -> bool:
        return self.diag is not None

    @property
    def dtype(self):
        return (self.diag if self.is_diag else self.data).dtype

    def to_scipy(self) -> sparse.csc_matrix:
        """Host SciPy CSC copy (A is symmetric, so its CSR arrays are its CSC arrays)."""
        if self.is_diag:
            d = self.diag.cpu().numpy()
            idx = np.arange(self.n, dtype=np.int32)
            return sparse.csc_matrix((d, idx, np.arange(self.n + 1, dtype=np.int32)), shape=(self.n, self.n))
        return sparse.csc_matrix((self.data.cpu().numpy(), self.indices.cpu().numpy(),
                                  self.indptr.cpu().numpy()), shape=(self.n, self.n))

    @classmethod
    def from_scipy(cls, mat) -> "DeviceCSR":
        require_cuda()
        mat = sparse.csr_matrix(mat)
        mat.sum_duplicates()
        mat.sort_indices()
        n = mat.shape[0]
        if mat.shape[0] != mat.shape[1]:
            raise ValueError("matrix must be square")
        if mat.nnz == n and np.array_equal(mat.indices, np.arange(n)) and np.array_equal(mat.indptr, np.arange(n + 1)):
            return cls(n, diag=torch.from_numpy(mat.data.astype(np.float64)).to("cuda"))
        return cls(n, torch.from_numpy(mat.indptr.astype(np.int32)).to("cuda"),
                   torch.from_numpy(mat.indices.astype(np.int32)).to("cuda"),
                   torch.from_numpy(mat.data.astype(np.float64)).to("cuda"))

    def as_f64(self) -> "DeviceCSR":
        if self.dtype == torch.float64:
            return self
        if self.is_diag:
            return DeviceCSR(self.n, diag=self.diag.double())
        return DeviceCSR(self.n, self.indptr, self.indices, self.data.double())

    def on_pattern(self, pat_indptr, pat_indices, pat_nnz) -> torch.Tensor:
        """Values of this matrix scattered onto another (containing) pattern."""
        L = _lib.lib()
        out = torch.zeros(pat_nnz, dtype=torch.float64, device="cuda")
        if self.is_diag:
            diag_pos = torch.empty(self.n, dtype=torch.int32, device="cuda")
            _lib.check(L.lapy_csr_diag_index(self.n, dptr(pat_indptr), dptr(pat_indices), dptr(diag_pos), stream()),
                       "csr_diag_index")
            if bool((diag_pos < 0).any()):
                raise _lib.LapyGpuError(_lib.ERR_PATTERN, "on_pattern", "diagonal entry missing from the pattern")
            _lib.check(L.lapy_csr_add_diag(self.n, dptr(diag_pos), 1.0, dptr(self.diag.double().contiguous()),
                                           dptr(out), stream()), "csr_add_diag")
            return out
        pos = torch.empty(self.data.numel(), dtype=torch.int32, device="cuda")
        w = workspace(256)
        _lib.check(L.lapy_csr_pattern_map(self.n, dptr(pat_indptr), dptr(pat_indices), dptr(self.indptr),
                                          dptr(self.indices), self.data.numel(), dptr(pos), dptr(w), stream()),
                   "csr_pattern_map")
        out.index_put_((pos.long(),), self.data.double(), accumulate=False)
        return out

    def matmul(self, x: torch.Tensor, alpha: float = 1.0) -> torch.Tensor:
        """Y = alpha * self @ X for X (n x F) float64 on the device."""
        L = _lib.lib()
        x = x.contiguous()
        ncol = 1 if x.dim() == 1 else x.shape[1]
        y = torch.empty_like(x)
        if self.is_diag:
            _lib.check(L.lapy_diag_mm_f64(self.n, dptr(self.diag.double().contiguous()), ncol, dptr(x), dptr(y),
                                          alpha, 0.0, stream()), "diag_mm_f64")
        else:
            _lib.check(L.lapy_csr_spmm_f64(self.n, dptr(self.indptr), dptr(self.indices),
                                           dptr(self.data.double().contiguous()), ncol, dptr(x), dptr(y), alpha,
                                           0.0, 0, stream()), "csr_spmm_f64")
        return y


def axpby(a: float, x: torch.Tensor, b: float, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    """out = a x + b y element-wise on the device (float64; out may alias y)."""
    out = torch.empty_like(y) if out is None else out
    _lib.check(_lib.lib().lapy_vec_axpby(y.numel(), float(a), dptr(x), float(b), dptr(y), dptr(out), stream()),
               "vec_axpby")
    return out


def pcg_solve(indptr, indices, k_vals, n, nnz, b: torch.Tensor, rtol: float, maxiter: int = 20000,
              mixed: bool = True, inner_rtol: float = 1e-4, seg_row=None):
    """Solve K X = B on the device (B: n or n x F float64); returns (X, relres, iters)."""
    L = _lib.lib()
    squeeze = b.dim() == 1
    B = b.reshape(n, -1).contiguous()
    ncol = B.shape[1]
    if seg_row is None:
        seg_row = np.array([0, n], dtype=np.int32)
    seg_row = np.ascontiguousarray(seg_row, dtype=np.int32)
    nseg = len(seg_row) - 1
    X = torch.empty_like(B)
    ws = workspace(L.lapy_pcg_solve_workspace_bytes(n, nnz, nseg, seg_row.ctypes.data, ncol, int(mixed)))
    status = np.zeros(nseg * ncol, dtype=np.int32)
    relres = np.zeros(nseg * ncol, dtype=np.float64)
    iters = C.c_int64(0)
    _lib.check(L.lapy_pcg_solve(n, dptr(indptr), dptr(indices), dptr(k_vals), nnz, nseg, seg_row.ctypes.data, ncol,
                                dptr(B), dptr(X), rtol, maxiter, int(mixed), inner_rtol, status.ctypes.data,
                                relres.ctypes.data, C.byref(iters), dptr(ws), ws.numel(), stream()), "pcg_solve")
    bad = status[status != 0]
    if bad.size:
        _lib.check(int(bad[0]), "pcg_solve")
    return (X[:, 0] if squeeze else X), relres, int(iters.value)


class SellF32:
    """FP32 SELL copy of a CSR matrix (float64 values cast) for the standalone
    pipelined product ``Y = Mat X`` (X, Y: n x ncol float32, ncol in 1, 2, 4, 8)."""

    def __init__(self, indptr, indices, vals, n: int, nnz: int, seg_row=None):
        L = _lib.lib()
        seg = np.ascontiguousarray(seg_row if seg_row is not None else [0, n], dtype=np.int32)
        self.n = n
        self.nnz = nnz
        self.ws = workspace(L.lapy_sell_f32_workspace_bytes(n, nnz, len(seg) - 1, seg.ctypes.data))
        self.handle = _lib.SellF32()
        _lib.check(L.lapy_sell_f32_build(n, dptr(indptr), dptr(indices), dptr(vals), nnz, len(seg) - 1,
                                         seg.ctypes.data, C.byref(self.handle), dptr(self.ws), self.ws.numel(),
                                         stream()), "sell_f32_build")

    def spmm(self, x: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
        ncol = 1 if x.dim() == 1 else x.shape[1]
        if x.dtype != torch.float32 or y.dtype != torch.float32 or not x.is_contiguous() or not y.is_contiguous():
            raise ValueError("SellF32.spmm wants contiguous float32 x and y")
        _lib.check(_lib.lib().lapy_sell_f32_spmm(C.byref(self.handle), ncol, dptr(x), dptr(y), stream()),
                   "sell_f32_spmm")
        return y


def ic0_pcg_solve(indptr, indices, k_vals, n, nnz, b: torch.Tensor, rtol: float, maxiter: int = 20000,
                  inner_rtol: float = 1e-4, seg_row=None):
    """Solve K X = B with IC(0)-preconditioned PCG (FP32 iterations inside FP64
    refinement); returns (X, relres, iters, replaced pivots)."""
    L = _lib.lib()
    squeeze = b.dim() == 1
    B = b.reshape(n, -1).contiguous()
    ncol = B.shape[1]
    if seg_row is None:
        seg_row = np.array([0, n], dtype=np.int32)
    seg_row = np.ascontiguousarray(seg_row, dtype=np.int32)
    nseg = len(seg_row) - 1
    X = torch.empty_like(B)
    ws = workspace(L.lapy_ic0_pcg_workspace_bytes(n, nnz, nseg, seg_row.ctypes.data, ncol))
    status = np.zeros(nseg * ncol, dtype=np.int32)
    relres = np.zeros(nseg * ncol, dtype=np.float64)
    iters = C.c_int64(0)
    fixed = C.c_int32(0)
    _lib.check(L.lapy_ic0_pcg_solve(n, dptr(indptr), dptr(indices), dptr(k_vals), nnz, nseg, seg_row.ctypes.data,
                                    ncol, dptr(B), dptr(X), rtol, maxiter, inner_rtol, status.ctypes.data,
                                    relres.ctypes.data, C.byref(iters), C.byref(fixed), dptr(ws), ws.numel(),
                                    stream()), "ic0_pcg_solve")
    bad = status[status != 0]
    if bad.size:
        _lib.check(int(bad[0]), "ic0_pcg_solve")
    return (X[:, 0] if squeeze else X), relres, int(iters.value), int(fixed.value)


def ic0_factor(indptr, indices, k_vals, n, nnz):
    """IC(0) factor of K on its own pattern (lower part L, upper part mirrored),
    with the workspace that holds its level plan; returns (l_vals, work,
    replaced pivots, (forward levels, backward levels))."""
    L = _lib.lib()
    lv = torch.empty(nnz, dtype=torch.float64, device="cuda")
    ws = workspace(L.lapy_ic0_workspace_bytes(n, nnz, 16))
    fixed = C.c_int32(0)
    levels = (C.c_int32 * 2)()
    _lib.check(L.lapy_ic0_factor(n, dptr(indptr), dptr(indices), dptr(k_vals.contiguous()), nnz, dptr(lv),
                                 C.byref(fixed), levels, dptr(ws), ws.numel(), stream()), "ic0_factor")
    return lv, ws, int(fixed.value), (int(levels[0]), int(levels[1]))


def ic0_apply(indptr, indices, l_vals, n, nnz, r: torch.Tensor, work: torch.Tensor) -> torch.Tensor:
    """z = (L L')^-1 r with a factor from ic0_factor (r: n or n x ncol, ncol <= 16)."""
    L = _lib.lib()
    R = r.reshape(n, -1).contiguous()
    Z = torch.empty_like(R)
    _lib.check(L.lapy_ic0_apply(n, dptr(indptr), dptr(indices), dptr(l_vals), nnz, R.shape[1], dptr(R), dptr(Z),
                                dptr(work), work.numel(), stream()), "ic0_apply")
    return Z[:, 0] if r.dim() == 1 else Z


def tria_curvature(md: MeshDevice, pat: FemPattern, smoothit: int, vertex: bool = True, triangle: bool = True):
    """Curvature frame of a triangle mesh on the device (lapy/tria_mesh.py:
    1078-1279): (vertex block 13 n or None, triangle block 8 m or None),
    planar f64 blocks as include/lapy_gb300.h describes."""
    L = _lib.lib()
    v = md.v if md.v.dtype == torch.float64 else md.v.double()
    vtx = torch.empty(13 * md.n, dtype=torch.float64, device="cuda") if vertex else None
    tri = torch.empty(8 * md.m, dtype=torch.float64, device="cuda") if triangle else None
    ws = workspace(L.lapy_tria_curvature_workspace_bytes(md.n, md.m, pat.nnz))
    st = L.lapy_tria_curvature(dptr(v.contiguous()), md.n, dptr(md.t), md.m, dptr(pat.indptr), dptr(pat.indices),
                               pat.nnz, int(smoothit), dptr(vtx), dptr(tri), dptr(ws), ws.numel(), stream())
    if st == _lib.ERR_INVALID and "oriented" in L.lapy_last_error().decode(errors="replace"):
        raise ValueError("Error: Can only compute edge information for oriented meshes!")
    _lib.check(st, "tria_curvature")
    return vtx, tri
