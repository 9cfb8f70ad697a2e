"""Generate tests/golden/ref_meshio.npz from the reference itself: the text
its mesh writers produce (TriaMesh.write_vtk, TetMesh.write_vtk) and what its
readers return (read_off, read_vtk with POLYGONS, CELLS and TRIANGLE_STRIPS,
TetMesh.read_vtk) for small meshes.

Runs only where the reference is available:

    python tests/golden/make_golden_meshio.py [--ref /root/reference]
"""

from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import import_reference  # noqa: E402

OFF_TEXT = "# a comment\nOFF\n4 2 0\n0 0 0\n1 0 0\n0 1 0\n1 1 0.5\n3 0 1 2\n3 1 3 2\n"
VTK_CELLS = ("# vtk DataFile Version 2.0\nmesh\nASCII\nDATASET UNSTRUCTURED_GRID\nPOINTS 4 double\n"
             "0 0 0 1 0 0\n0 1 0 1 1 0.25\nCELLS 2 8\n3 0 1 2\n3 1 3 2\n")
GMSH_TEXT = ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n5\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n"
             "5 1 1 1\n$EndNodes\n$Elements\n2\n1 4 2 0 1 0 1 2 3\n2 4 2 0 1 1 2 3 4\n$EndElements\n")
VTK_STRIPS = ("# vtk DataFile Version 1.0\nstrip\nASCII\nDATASET POLYDATA\nPOINTS 5 float\n"
              "0 0 0\n1 0 0\n0 1 0\n1 1 0\n0 2 0\nTRIANGLE_STRIPS 1 6\n5 0 1 2 3 4\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    RTria, RTet, _, _, _ = import_reference(Path(args.ref))
    out = {"off_text": np.array(OFF_TEXT), "vtk_cells_text": np.array(VTK_CELLS),
           "vtk_strips_text": np.array(VTK_STRIPS)}
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        (tmp / "a.off").write_text(OFF_TEXT)
        m = RTria.read_off(str(tmp / "a.off"))
        out["off_v"], out["off_t"] = m.v, m.t
        (tmp / "c.vtk").write_text(VTK_CELLS)
        m = RTria.read_vtk(str(tmp / "c.vtk"))
        out["cells_v"], out["cells_t"] = m.v, m.t
        (tmp / "s.vtk").write_text(VTK_STRIPS)
        try:
            m = RTria.read_vtk(str(tmp / "s.vtk"))
            out["strips_v"], out["strips_t"] = m.v, np.asarray(m.t).astype(int)
        except Exception as exc:  # recorded: the reference's strip reader
            out["strips_error"] = np.array(f"{type(exc).__name__}: {exc}")
        for name in ("ico3", "deformed3"):
            f = np.load(HERE / f"ref_{name}.npz")
            for dt in ("float32", "float64"):
                RTria(f["v"].astype(dt), f["t"]).write_vtk(str(tmp / "w.vtk"))
                out[f"write_{name}_{dt}"] = np.array((tmp / "w.vtk").read_text())
                back = RTria.read_vtk(str(tmp / "w.vtk"))
                out[f"read_{name}_{dt}_v"], out[f"read_{name}_{dt}_t"] = back.v, back.t
        f = np.load(HERE / "ref_kuhn5.npz")
        RTet(f["v"], f["t"]).write_vtk(str(tmp / "k.vtk"))
        out["write_kuhn5"] = np.array((tmp / "k.vtk").read_text())
        back = RTet.read_vtk(str(tmp / "k.vtk"))
        out["read_kuhn5_v"], out["read_kuhn5_t"] = back.v, back.t
        # gmsh tetrahedra (ASCII 2.2; element rows: id, type 4, 2 tags, 4 node ids)
        (tmp / "k.msh").write_text(GMSH_TEXT)
        m = RTet.read_gmsh(str(tmp / "k.msh"))
        out["gmsh_text"], out["gmsh_v"], out["gmsh_t"] = np.array(GMSH_TEXT), m.v, m.t
        # FreeSurfer surfaces written by lapy_gb300's writer, read by the reference
        sys.path.insert(0, str(HERE.parent.parent))
        from lapy_gb300._meshio import write_fssurf

        f = np.load(HERE / "ref_deformed3.npz")
        info = {"head": [2, 0, 20], "valid": "1  # volume info valid", "filename": "vol.mgz",
                "volume": np.array([256, 256, 256]), "voxelsize": np.array([1.0, 1.0, 1.0]),
                "xras": np.array([-1.0, 0.0, 0.0]), "yras": np.array([0.0, 0.0, -1.0]),
                "zras": np.array([0.0, 1.0, 0.0]), "cras": np.array([0.5, -12.25, 3.0])}
        for tag, vi in (("plain", None), ("volinfo", info)):
            write_fssurf(f["v"], f["t"], str(tmp / "s.surf"), volume_info=vi)
            out[f"fs_{tag}_bytes"] = np.frombuffer((tmp / "s.surf").read_bytes(), dtype=np.uint8)
            m = RTria.read_fssurf(str(tmp / "s.surf"))
            out[f"fs_{tag}_v"], out[f"fs_{tag}_t"] = m.v, m.t
            if vi is not None:
                for key, val in m.fsinfo.items():
                    out[f"fs_{tag}_info_{key}"] = np.asarray(val)
    np.savez_compressed(HERE / "ref_meshio.npz", **out)
    print("wrote", HERE / "ref_meshio.npz", sorted(out))


if __name__ == "__main__":
    main()
