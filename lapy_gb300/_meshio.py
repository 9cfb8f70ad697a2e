"""OFF and legacy ASCII VTK mesh files, read and written as lapy's
_tria_io.py / _tet_io.py do (same accepted layouts, same float32 vertex
parsing, same error types and the same written text).  Host code: files are
parsed with NumPy's text reader in whole blocks, not line by line."""

from __future__ import annotations

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
