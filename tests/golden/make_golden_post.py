"""Generate tests/golden/ref_post.npz from the reference itself: ShapeDNA
post-processing (normalize_ev, reweight_ev, compute_distance), the .ev /
PSOL text formats (write_ev, write_vfunc, read_ev, read_vfunc) and the heat
kernel values of lapy.heat (diagonal, kernel).

Runs only where the reference is available:

    python tests/golden/make_golden_post.py [--ref /root/reference]

Inputs are the meshes and eigenvalues already stored in the ref_*.npz
fixtures; outputs (numbers, and the files' text) are stored next to this
script so the tests never read the reference.
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

# text files the reader must accept, in the layouts the reference documents
VFUNC_TEXTS = {
    "comma": "Solution:\n(1.5,2.25,-3.0,4e-05)",
    "semicolon_braces": "Solution:\n{1.5;2.25;-3.0;4e-05}\n",
    "one_per_line": "Solution:\n1.5\n2.25\n-3.0\n\n4e-05\n",
}
EV_TEXT_MULTILINE = (" Creator: 7\n Refine: 0\n Degree: 1\n Dimension: 2\n Elements: 12\n DoF: 8\n NumEW: 3\n\n"
                     " Area: 2.5\n Volume: 0.75\n BLength: 1.25\n EulerChar: 2\n\n Time(pre): 3\n Time(calcAB): 4\n"
                     " Time(calcEW): 5\n\nEigenvalues:\n{ 0.0 ;\n 1.5 ;\n 2.75 }\n\nEigenvectors:\nsizes: 2 3\n\n"
                     "{ (1.0,2.0) ;\n(3.0,4.0) ;\n(5.0,6.0) }\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    RTria, RTet, _, _, _ = import_reference(Path(args.ref))
    import lapy.io as rio
    import lapy.shapedna as rsd

    out = {}
    meshes = {}
    for name in ("ico3", "deformed3", "cubetria", "kuhn5"):
        f = np.load(HERE / f"ref_{name}.npz")
        geo = RTria(f["v"], f["t"]) if f["t"].shape[1] == 3 else RTet(f["v"], f["t"])
        meshes[name] = (geo, f["evals"])
        methods = ("surface", "volume", "geometry") if f["t"].shape[1] == 3 else ("volume", "geometry")
        for m in methods:
            out[f"{name}_norm_{m}"] = rsd.normalize_ev(geo, f["evals"], method=m)
        out[f"{name}_reweight"] = rsd.reweight_ev(f["evals"])
    out["dist_ico3_deformed3"] = np.array(rsd.compute_distance(
        rsd.reweight_ev(rsd.normalize_ev(meshes["ico3"][0], meshes["ico3"][1])),
        rsd.reweight_ev(rsd.normalize_ev(meshes["deformed3"][0], meshes["deformed3"][1]))))

    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        # writer: a descriptor with every header field, eigenvalues and eigenvectors
        f = np.load(HERE / "ref_kuhn5.npz")
        d = {"Creator": "1", "File": "2", "User": "3", "Refine": 0, "Degree": 1, "Dimension": 3,
             "Elements": int(len(f["t"])), "DoF": int(len(f["v"])), "NumEW": 4, "Area": 6.0, "Volume": 1.0,
             "BLength": 0.0, "EulerChar": 2, "TimePre": 0.5, "TimeCalcAB": 1.25, "TimeCalcEW": 2.0,
             "Eigenvalues": f["evals"][:4], "Eigenvectors": f["evecs"][:, :4]}
        rio.write_ev(str(tmp / "a.ev"), d)
        out["ev_written"] = np.array((tmp / "a.ev").read_text())
        back = rio.read_ev(str(tmp / "a.ev"))
        out["ev_read_keys"] = np.array(sorted(back.keys()))
        out["ev_read_evals"] = back["Eigenvalues"]
        out["ev_read_evecs"] = back["Eigenvectors"]
        out["ev_input_evals"] = d["Eigenvalues"]
        out["ev_input_evecs"] = d["Eigenvectors"]
        (tmp / "b.ev").write_text(EV_TEXT_MULTILINE)
        back = rio.read_ev(str(tmp / "b.ev"))
        out["ev_multi_text"] = np.array(EV_TEXT_MULTILINE)
        out["ev_multi_keys"] = np.array(sorted(back.keys()))
        for key in ("Creator", "Refine", "Degree", "Dimension", "Elements", "DoF", "NumEW", "Area", "Volume",
                    "BLength", "EulerChar", "TimePre", "TimeCalcAB", "TimeCalcEW"):
            out[f"ev_multi_{key}"] = np.array(back[key])
        out["ev_multi_evals"] = back["Eigenvalues"]
        out["ev_multi_evecs"] = back["Eigenvectors"]
        out["ev_multi_sizes"] = back["EigenvectorsSize"]
        vf = np.array([0.5, -1.25, 3.0e-7, 12.0])
        rio.write_vfunc(str(tmp / "a.psol"), vf)
        out["vfunc_input"] = vf
        out["vfunc_written"] = np.array((tmp / "a.psol").read_text())
        for key, text in VFUNC_TEXTS.items():
            (tmp / f"{key}.psol").write_text(text)
            out[f"vfunc_text_{key}"] = np.array(text)
            out[f"vfunc_read_{key}"] = np.array(rio.read_vfunc(str(tmp / f"{key}.psol")))
    # heat kernel values from eigenpairs (evals as a column, times as a row)
    import lapy.heat as rheat

    f = np.load(HERE / "ref_deformed3.npz")
    ev, evec = f["evals"], f["evecs"]
    out["hk_evals"], out["hk_evecs"] = ev, evec
    out["hk_t3"] = np.array([[0.1, 1.0, 5.0]])
    out["hk_x"] = np.arange(0, len(evec), 7)
    out["hk_diag_rows"] = rheat.diagonal(out["hk_t3"], out["hk_x"], evec, ev[:, None], 8)
    out["hk_diag_one"] = rheat.diagonal(out["hk_t3"], 5, evec, ev[:, None], 8)
    out["hk_kernel_n3"] = rheat.kernel(np.array([[0.2, 0.7, 3.0]]), 3, evec, ev[:, None], 3)
    out["hk_kernel_t1"] = rheat.kernel(np.array([[0.5]]), 11, evec, ev[:, None], 6)
    np.savez_compressed(HERE / "ref_post.npz", **out)
    print("wrote", HERE / "ref_post.npz", len(out), "entries")


if __name__ == "__main__":
    main()
