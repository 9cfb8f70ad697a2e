"""Mesh files against the reference's own readers and writers
(tests/golden/ref_meshio.npz, made by make_golden_meshio.py): OFF, legacy
ASCII VTK, ASCII gmsh tetrahedra and FreeSurfer surface geometry.  Host code
only."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLD / "ref_meshio.npz")


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(str(text))
    return str(p)


def test_read_off_and_cells(ref, tmp_path):
    from lapy_gb300 import TriaMesh

    m = TriaMesh.read_off(_write(tmp_path, "a.off", ref["off_text"]))
    np.testing.assert_array_equal(m.v, ref["off_v"])
    assert m.v.dtype == ref["off_v"].dtype
    np.testing.assert_array_equal(m.t, ref["off_t"])
    m = TriaMesh.read_vtk(_write(tmp_path, "c.vtk", ref["vtk_cells_text"]))
    np.testing.assert_array_equal(m.v, ref["cells_v"])
    np.testing.assert_array_equal(m.t, ref["cells_t"])


def test_triangle_strips(ref, tmp_path):
    """A strip 0 1 2 3 4 is the triangles (0 1 2), (2 1 3), (2 3 4).  The
    reference's reader keeps the indices as text and fails on them
    (recorded in the fixture); this one returns the integer triangles."""
    from lapy_gb300 import TriaMesh

    assert "strips_error" in ref.files
    m = TriaMesh.read_vtk(_write(tmp_path, "s.vtk", ref["vtk_strips_text"]))
    np.testing.assert_array_equal(m.t, [[0, 1, 2], [2, 1, 3], [2, 3, 4]])
    assert m.v.shape == (5, 3)


@pytest.mark.parametrize("name", ["ico3", "deformed3"])
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_tria_write_read_matches_reference(ref, tmp_path, name, dt):
    from lapy_gb300 import TriaMesh

    f = np.load(GOLD / f"ref_{name}.npz")
    p = str(tmp_path / "w.vtk")
    TriaMesh(f["v"].astype(dt), f["t"]).write_vtk(p)
    assert Path(p).read_text() == str(ref[f"write_{name}_{dt}"])
    back = TriaMesh.read_vtk(p)
    np.testing.assert_array_equal(back.v, ref[f"read_{name}_{dt}_v"])
    np.testing.assert_array_equal(back.t, ref[f"read_{name}_{dt}_t"])


def test_tet_write_read_matches_reference(ref, tmp_path):
    from lapy_gb300 import TetMesh

    f = np.load(GOLD / "ref_kuhn5.npz")
    p = str(tmp_path / "k.vtk")
    TetMesh(f["v"], f["t"]).write_vtk(p)
    assert Path(p).read_text() == str(ref["write_kuhn5"])
    back = TetMesh.read_vtk(p)
    np.testing.assert_array_equal(back.v, ref["read_kuhn5_v"])
    np.testing.assert_array_equal(back.t, ref["read_kuhn5_t"])


def test_reader_errors(ref, tmp_path):
    from lapy_gb300 import TetMesh, TriaMesh

    with pytest.raises(OSError, match="OFF keyword"):
        TriaMesh.read_off(_write(tmp_path, "b.off", "NOFF\n1 0 0\n"))
    with pytest.raises(OSError, match="no triangle data"):
        TriaMesh.read_off(_write(tmp_path, "q.off", "OFF\n4 1 0\n0 0 0\n1 0 0\n0 1 0\n1 1 0\n4 0 1 3 2\n"))
    with pytest.raises(OSError):
        TriaMesh.read_off(str(tmp_path / "missing.off"))
    with pytest.raises(OSError, match="ASCII"):
        TriaMesh.read_vtk(_write(tmp_path, "b1.vtk", "# vtk\nx\nBINARY\nDATASET POLYDATA\n"))
    with pytest.raises(OSError, match="DATASET"):
        TriaMesh.read_vtk(_write(tmp_path, "b2.vtk", "# vtk\nx\nASCII\nDATASET STRUCTURED_POINTS\n"))
    with pytest.raises(OSError, match="POINTS"):
        TriaMesh.read_vtk(_write(tmp_path, "b3.vtk", "# vtk\nx\nASCII\nDATASET POLYDATA\nPOINTS 3 int\n"))
    tet_text = str(ref["write_kuhn5"])
    with pytest.raises(OSError, match="data per tria"):  # a tetrahedral file read as triangles
        TriaMesh.read_vtk(_write(tmp_path, "t.vtk", tet_text))
    tria_text = str(ref["write_ico3_float64"])
    with pytest.raises(ValueError, match="data per tetra"):  # and the other way round (ValueError, as the reference)
        TetMesh.read_vtk(_write(tmp_path, "r.vtk", tria_text))


def test_gmsh_tetrahedra(ref, tmp_path):
    from lapy_gb300 import TetMesh

    m = TetMesh.read_gmsh(_write(tmp_path, "k.msh", ref["gmsh_text"]))
    np.testing.assert_array_equal(m.v, ref["gmsh_v"])
    assert m.v.dtype == ref["gmsh_v"].dtype
    np.testing.assert_array_equal(m.t, ref["gmsh_t"])
    with pytest.raises(ValueError, match="no .msh file"):
        TetMesh.read_gmsh(_write(tmp_path, "k.txt", ref["gmsh_text"]))
    with pytest.raises(ValueError, match="binary format"):
        TetMesh.read_gmsh(_write(tmp_path, "b.msh", str(ref["gmsh_text"]).replace("2.2 0 8", "2.2 1 8")))
    with pytest.raises(ValueError, match="can only read tetras"):
        TetMesh.read_gmsh(_write(tmp_path, "c.msh", str(ref["gmsh_text"]).replace("1 4 2 0 1", "1 2 2 0 1")))


@pytest.mark.parametrize("tag", ["plain", "volinfo"])
def test_freesurfer_surface(ref, tmp_path, tag):
    """Files written here are read by the reference's FreeSurfer reader (the
    fixture holds what it returned) and by this reader alike."""
    from lapy_gb300 import TriaMesh

    f = np.load(GOLD / "ref_deformed3.npz")
    info = None
    if tag == "volinfo":
        info = {k: ref[f"fs_volinfo_info_{k}"] for k in ("head", "valid", "filename", "volume", "voxelsize",
                                                          "xras", "yras", "zras", "cras")}
        info = {k: (str(v) if v.dtype.kind == "U" else v) for k, v in info.items()}
    p = str(tmp_path / "s.surf")
    TriaMesh(f["v"], f["t"], fsinfo=info).write_fssurf(p)
    assert np.array_equal(np.frombuffer(Path(p).read_bytes(), dtype=np.uint8), ref[f"fs_{tag}_bytes"])
    m = TriaMesh.read_fssurf(p)
    np.testing.assert_array_equal(m.v, ref[f"fs_{tag}_v"])
    np.testing.assert_array_equal(m.t, ref[f"fs_{tag}_t"])
    if tag == "volinfo":
        for key, val in m.fsinfo.items():
            np.testing.assert_array_equal(np.asarray(val), ref[f"fs_volinfo_info_{key}"])
    else:
        assert len(m.fsinfo) == 0
    bad = tmp_path / "bad.surf"
    bad.write_bytes(b"\x00\x01\x02rest")
    with pytest.raises(ValueError, match="Freesurfer"):
        TriaMesh.read_fssurf(str(bad))
