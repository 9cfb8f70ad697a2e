"""Generate tests/golden/ref_aniso.npz from the reference itself: the
curvature frame (TriaMesh.curvature, TriaMesh.curvature_tria) and the
anisotropic Laplace-Beltrami matrices (Solver(mesh, aniso=...)) of deformed
icospheres.

Runs only where the reference is available:

    python tests/golden/make_golden_aniso.py [--ref /root/reference]
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

from make_golden import csr_arrays, import_reference  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    RTria, _, RSolver, _, _ = import_reference(Path(args.ref))
    from lapy_gb300 import meshes

    out = {}
    cases = {"d3": np.load(HERE / "ref_deformed3.npz"),
             "d4": meshes.sh_deform(meshes.icosphere(4), seed=21)}
    for name, m in cases.items():
        v, t = (m["v"], m["t"]) if isinstance(m, np.lib.npyio.NpzFile) else (m.v, m.t)
        tria = RTria(v, t)
        out[f"{name}_v"], out[f"{name}_t"] = np.asarray(v), np.asarray(t, dtype=np.int32)
        if name == "d3":  # vertex-level frame of the small mesh only (fixture size)
            for key, val in zip(("umin", "umax", "cmin", "cmax", "cmean", "cgauss", "normals"), tria.curvature(3)):
                out[f"{name}_vtx_{key}"] = val
        for key, val in zip(("umin", "umax", "cmin", "cmax"), tria.curvature_tria(3)):
            out[f"{name}_tri_{key}"] = val
        for tag, aniso in ((("a12", (1.0, 2.0)), ("a05", 0.5)) if name == "d3" else (("a12", (1.0, 2.0)),)):
            for lump in (False, True):
                fem = RSolver(tria, lump=lump, aniso=aniso, aniso_smooth=3)
                out.update(csr_arrays(f"{name}_{tag}_lump{int(lump)}_A", fem.stiffness))
                out.update(csr_arrays(f"{name}_{tag}_lump{int(lump)}_M", fem.mass))
    np.savez_compressed(HERE / "ref_aniso.npz", **out)
    print("wrote", HERE / "ref_aniso.npz", len(out), "entries")


if __name__ == "__main__":
    main()
