"""Generate the golden fixtures of tests/golden from the reference itself.

Runs only where the reference (Deep-MI/LaPy, pure Python) is available:

    python tests/golden/make_golden.py [--ref /root/reference]

The reference package is copied to a temporary directory (it must be
importable without being installed; ``lapy._version`` reads package metadata,
so a stub module stands in for it), its Solver / heat / diffgeo functions are
run on a set of small meshes, and their outputs are stored as .npz files next
to this script.  Inputs are stored too, so the tests never read the
reference.  The oracle (``oracle/``) is checked against the same outputs in
``tests/test_oracle.py``.
"""

from __future__ import annotations

import argparse
import shutil
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def import_reference(ref: Path):
    tmp = Path(tempfile.mkdtemp(prefix="lapy_ref_"))
    shutil.copytree(ref / "lapy", tmp / "lapy")
    stub = types.ModuleType("lapy._version")
    stub.__version__ = "reference"
    sys.modules["lapy._version"] = stub
    sys.path.insert(0, str(tmp))
    import lapy  # noqa: F401
    from lapy import TetMesh, TriaMesh, Solver, heat, diffgeo
    return TriaMesh, TetMesh, Solver, heat, diffgeo


def csr_arrays(prefix, mat):
    m = mat.tocsc()
    m.sort_indices()
    return {f"{prefix}_indptr": m.indptr.astype(np.int64), f"{prefix}_indices": m.indices.astype(np.int64),
            f"{prefix}_data": m.data}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    ref = Path(args.ref)
    RTria, RTet, RSolver, rheat, rdiffgeo = import_reference(ref)
    from lapy_gb300 import meshes

    out = {}
    # --- reference fixture meshes (float32 coordinates, as the readers produce)
    sq = RTria.read_off(str(ref / "data" / "square-mesh.off"))
    cube = RTria.read_vtk(str(ref / "data" / "cubeTria.vtk"))
    ctet = RTet.read_vtk(str(ref / "data" / "cubeTetra.vtk"))
    ico3 = meshes.icosphere(3)
    defo = meshes.sh_deform(meshes.icosphere(3), seed=11)
    kuhn = meshes.kuhn_cube(5, jitter=0.2, seed=3)

    cases = {
        "square": (sq.v, sq.t),
        "cubetria": (cube.v, cube.t),
        "ico3": (ico3.v, ico3.t),
        "deformed3": (defo.v, defo.t),
        "kuhn5": (kuhn.v, kuhn.t),
    }
    for name, (v, t) in cases.items():
        d = {"v": np.asarray(v), "t": np.asarray(t, dtype=np.int32)}
        geo = RTria(v, t) if t.shape[1] == 3 else RTet(v, t)
        for lump in (False, True):
            fem = RSolver(geo, lump=lump)
            d.update(csr_arrays(f"A_lump{int(lump)}", fem.stiffness))
            d.update(csr_arrays(f"M_lump{int(lump)}", fem.mass))
        k = 10
        fem = RSolver(geo, lump=False)
        ev, evec = fem.eigs(k=k)
        d["eigs_k"] = np.array(k)
        d["evals"] = ev
        d["evecs"] = evec
        fem_l = RSolver(geo, lump=True)
        evl, evecl = fem_l.eigs(k=k)
        d["evals_lump"] = evl
        d["evecs_lump"] = evecl
        d["avg_edge"] = np.array(geo.avg_edge_length())
        u = rheat.diffusion(geo, 0, m=1.0)
        d["heat0"] = u
        seeds = [np.array([0]), np.array([1, 2])]
        d["heat_multi"] = rheat.diffusion(geo, seeds, m=1.0)
        # Poisson with Dirichlet data on the first vertices, h = second eigenvector
        dtup = (np.array([0, 1]), np.array([0.0, 0.5]))
        d["poisson_dir"] = fem_l.poisson(evecl[:, 1], dtup=dtup)
        d["poisson_dir_2d"] = fem_l.poisson(evecl[:, 1:4], dtup=dtup)
        grad = rdiffgeo.compute_gradient(geo, u)
        d["grad_heat0"] = grad
        d["div_grad_heat0"] = rdiffgeo.compute_divergence(geo, grad)
        d["geodesic0"] = rdiffgeo.compute_geodesic_f(geo, u)
        out[name] = d
        np.savez_compressed(HERE / f"ref_{name}.npz", **d)
        print(f"{name}: n={len(v)} m={len(t)} evals[:3]={ev[:3]}")

    # cubeTetra: eigenvalues only (the mesh is stored, its matrices are not)
    ev, _ = RSolver(ctet, lump=False).eigs(k=3)
    np.savez_compressed(HERE / "ref_cubetetra.npz", v=np.asarray(ctet.v), t=np.asarray(ctet.t, dtype=np.int32),
                        evals=ev)
    print("cubetetra", ev)


if __name__ == "__main__":
    main()
