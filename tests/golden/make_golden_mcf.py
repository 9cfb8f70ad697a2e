"""Generate tests/golden/ref_mcf.npz from the reference itself: the
mean-curvature flow of lapy.diffgeo (tria_mean_curvature_flow) on a deformed
icosphere (level 3), for 5 steps and with the default stopping rule.

Runs only where the reference is available:

    python tests/golden/make_golden_mcf.py [--ref /root/reference]
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

from make_golden import import_reference  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    RTria, _, _, _, rdiffgeo = import_reference(Path(args.ref))
    f = np.load(HERE / "ref_deformed3.npz")
    tria = RTria(f["v"], f["t"])
    out = {"v": f["v"], "t": f["t"]}
    out["mcf5_v"] = rdiffgeo.tria_mean_curvature_flow(tria, max_iter=5).v
    out["mcf5_step05_v"] = rdiffgeo.tria_mean_curvature_flow(tria, max_iter=5, step=0.5).v
    res = rdiffgeo.tria_mean_curvature_flow(tria)
    out["mcf_default_v"] = res.v
    np.savez_compressed(HERE / "ref_mcf.npz", **out)
    print("wrote", HERE / "ref_mcf.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
