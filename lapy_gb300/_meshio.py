"""Mesh files as lapy's _tria_io.py / _tet_io.py / _read_geometry.py read and
write them: OFF and legacy ASCII VTK (same accepted layouts, same float32
vertex parsing, same error types and the same written text), ASCII gmsh
tetrahedra, and FreeSurfer surface geometry (big-endian binary).  Host code:
files are parsed with NumPy's readers in whole blocks, not line by line."""

from __future__ import annotations

import os
from collections import OrderedDict

import numpy as np


def _skip_comments(fh) -> str:
    line = fh.readline()
    while line.startswith("#"):
        line = fh.readline()
    return line


def read_off(filename: str) -> tuple[np.ndarray, np.ndarray]:
    """(v, t) of an OFF triangle file (lapy/_tria_io.py:50-110)."""
    with open(filename) as fh:
        if not _skip_comments(fh).startswith("OFF"):
            raise OSError("[OFF keyword not found] --> FAILED\n")
        counts = fh.readline().split()
        nv, nf = int(counts[0]), int(counts[1])
        v = np.fromfile(fh, "float32", 3 * nv, " ").reshape(nv, 3)
        faces = np.fromfile(fh, "int", 4 * nf, " ").reshape(nf, 4)
    if faces.size == 0 or np.amax(faces[:, 0]) != 3:
        raise OSError("[no triangle data] --> FAILED\n")
    return v, faces[:, 1:]


def _strip_triangles(fh, nstrips: int, err) -> np.ndarray:
    """Triangles of TRIANGLE_STRIPS records ``n i0 i1 ... i_{n-1}``: every
    window of three, odd windows with their first two corners swapped so the
    strip keeps one orientation."""
    tris = []
    for _ in range(nstrips):
        rec = fh.readline().split()
        if not rec:
            raise err("[error reading triangle strip (i)] --> FAILED\n")
        n = int(rec[0])
        if len(rec) != n + 1:
            raise err("[error reading triangle strip (ii)] --> FAILED\n")
        ids = rec[1:]
        for k in range(n - 2):
            a, b, c = ids[k], ids[k + 1], ids[k + 2]
            tris.append([a, b, c] if k % 2 == 0 else [b, a, c])
    return np.array(tris, dtype=int)


def read_vtk(filename: str, npe: int) -> tuple[np.ndarray, np.ndarray]:
    """(v, t) of a legacy ASCII VTK file with cells of ``npe`` corners
    (lapy/_tria_io.py:113-227 for triangles, which raise OSError;
    lapy/_tet_io.py:131-224 for tetrahedra, which raise ValueError)."""
    err = OSError if npe == 3 else ValueError
    what = "tria" if npe == 3 else "tetra"
    with open(filename) as fh:
        line = _skip_comments(fh)
        for _ in range(5):
            if line.startswith("ASCII"):
                break
            line = fh.readline()
        if not line.startswith("ASCII"):
            raise err("[ASCII keyword not found] --> FAILED\n")
        line = fh.readline()
        if not (line.startswith("DATASET POLYDATA") or line.startswith("DATASET UNSTRUCTURED_GRID")):
            raise err(f"[read: {line} expected DATASET POLYDATA or DATASET UNSTRUCTURED_GRID] --> FAILED\n")
        line = fh.readline()
        rec = line.split()
        if rec[0] != "POINTS" or rec[2] not in ("float", "double"):
            raise err(f"[read: {line} expected POINTS # float or POINTS # double ] --> FAILED\n")
        nv = int(rec[1])
        v = np.fromfile(fh, "float32", 3 * nv, " ").reshape(nv, 3)
        line = fh.readline()
        rec = line.split()
        if rec[0] in ("POLYGONS", "CELLS"):
            nc, ntot = int(rec[1]), int(rec[2])
            per = float(ntot) / nc
            if per != npe + 1.0:
                raise err(f"[having: {per} data per {what}, expected {'trias 3' if npe == 3 else '4'}+1] --> FAILED\n")
            cells = np.fromfile(fh, "int", ntot, " ").reshape(nc, npe + 1)
            if cells[nc - 1][0] != npe:
                raise err(f"[can only read {'triangles' if npe == 3 else 'tetras'}] --> FAILED\n")
            t = cells[:, 1:]
        elif rec[0] == "TRIANGLE_STRIPS" and npe == 3:
            t = _strip_triangles(fh, int(rec[1]), err)
        else:
            expected = "POLYGONS or TRIANGLE_STRIPS" if npe == 3 else "POLYGONS or CELLS"
            raise err(f"[read: {line} expected {expected}] --> FAILED\n")
    return v, t


def write_vtk(v: np.ndarray, t: np.ndarray, filename: str) -> None:
    """Legacy ASCII VTK POLYDATA with the reference's header and number
    formatting (``str`` of each element): lapy/_tria_io.py:638-674,
    lapy/_tet_io.py:227-259."""
    v = np.asarray(v)
    t = np.asarray(t)
    npe = t.shape[1]
    lines = ["# vtk DataFile Version 1.0", "vtk output", "ASCII", "DATASET POLYDATA", f"POINTS {v.shape[0]} float"]
    lines += [" ".join(map(str, row)) for row in v]
    lines.append(f"POLYGONS {t.shape[0]} {(npe + 1) * t.shape[0]}")
    lines += [" ".join(map(str, np.append(npe, row))) for row in t]
    with open(filename, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_gmsh_tet(filename: str) -> tuple[np.ndarray, np.ndarray]:
    """(v, t) of an ASCII gmsh 2.x file of tetrahedra (lapy/_tet_io.py:17-128):
    node coordinates read as float32 without their id column, and the last
    four columns of every element row (the node ids as stored)."""
    if os.path.splitext(filename)[1] != ".msh":
        raise ValueError("[no .msh file] --> FAILED\n")
    with open(filename) as fh:
        if not fh.readline().startswith("$MeshFormat"):
            raise ValueError("[$MeshFormat keyword not found] --> FAILED\n")
        fmt = fh.readline().split()
        if int(fmt[1]) != 0:
            raise ValueError("[binary format not implemented] --> FAILED\n")
        for key in ("$EndMeshFormat", "$Nodes"):
            if not fh.readline().startswith(key):
                raise ValueError(f"[{key} keyword not found] --> FAILED\n")
        nv = int(fh.readline())
        v = np.fromfile(fh, "float32", 4 * nv, " ").reshape(nv, 4)[:, 1:]
        for key in ("$EndNodes", "$Elements"):
            if not fh.readline().startswith(key):
                raise ValueError(f"[{key} keyword not found] --> FAILED\n")
        ne = int(fh.readline())
        pos = fh.tell()
        first = fh.readline().split()
        fh.seek(pos)
        if int(first[1]) != 4:
            raise ValueError("[can only read tetras] --> FAILED\n")
        ncol = len(first)
        t = np.fromfile(fh, "int", ne * ncol, " ").reshape(ne, ncol)[:, ncol - 4:]
        if not fh.readline().startswith("$EndElements"):
            raise ValueError("[$EndElements keyword not found] --> FAILED\n")
    return v, t


# FreeSurfer surface geometry: 3-byte magic 0xFFFFFE, a creation line, an
# optional empty line, vertex and face counts (big-endian int32), float32
# coordinates, int32 faces, then an optional volume-info footer
# (lapy/_read_geometry.py:42-197).
_FS_MAGIC = b"\xff\xff\xfe"
_FS_KEYS = ("valid", "filename", "volume", "voxelsize", "xras", "yras", "zras", "cras")


def _read_fs_volume_info(fh) -> OrderedDict:
    info = OrderedDict()
    head = np.fromfile(fh, ">i4", 1)
    if not np.array_equal(head, [20]):
        head = np.concatenate([head, np.fromfile(fh, ">i4", 2)])
        if not (np.array_equal(head, [2, 0, 20]) or np.array_equal(head, [2, 1, 20])):
            return info  # unknown extension: no volume info
        head = [2, 0, 20]
    info["head"] = head
    for key in _FS_KEYS:
        pair = fh.readline().decode("utf-8").split("=")
        if pair[0].strip() != key or len(pair) != 2:
            raise OSError("Error parsing volume info.")
        if key in ("valid", "filename"):
            info[key] = pair[1].strip()
        elif key == "volume":
            info[key] = np.array(pair[1].split()).astype(int)
        else:
            info[key] = np.array(pair[1].split()).astype(float)
    # the footer may hold more (e.g. a command history): not used here
    return info


def read_fssurf(filename: str):
    """(v float64, t int32, volume info) of a FreeSurfer surface file."""
    with open(filename, "rb") as fh:
        if fh.read(3) != _FS_MAGIC:
            raise ValueError("File does not appear to be a Freesurfer surface (triangle file)")
        fh.readline()  # creation stamp
        if fh.peek(1)[:1] == b"\n":
            fh.readline()
        nv = int(np.fromfile(fh, ">i4", 1)[0])
        nf = int(np.fromfile(fh, ">i4", 1)[0])
        v = np.fromfile(fh, ">f4", nv * 3).reshape(nv, 3)
        t = np.fromfile(fh, ">i4", nf * 3).reshape(nf, 3)
        info = _read_fs_volume_info(fh)
    return v.astype(float), t, info


def write_fssurf(v, t, filename: str, volume_info=None, stamp: str = "created by lapy_gb300") -> None:
    """FreeSurfer surface file in the layout read_fssurf reads (the format
    FreeSurfer and nibabel write), with the volume-info footer when given."""
    v = np.asarray(v, dtype=">f4")
    t = np.asarray(t, dtype=">i4")
    with open(filename, "wb") as fh:
        fh.write(_FS_MAGIC)
        fh.write((stamp + "\n\n").encode("utf-8"))
        np.array([v.shape[0], t.shape[0]], dtype=">i4").tofile(fh)
        v.tofile(fh)
        t.tofile(fh)
        if volume_info:
            np.array(volume_info.get("head", [2, 0, 20]), dtype=">i4").tofile(fh)
            for key in _FS_KEYS:
                val = volume_info[key]
                if key in ("valid", "filename"):
                    text = str(val)
                elif key == "volume":
                    text = " ".join(str(int(x)) for x in val)
                else:
                    text = " ".join(repr(float(x)) for x in val)
                fh.write(f"{key} = {text}\n".encode("utf-8"))
