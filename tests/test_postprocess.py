"""ShapeDNA post-processing, the .ev / PSOL text formats and the heat kernel
values against the reference's own outputs (tests/golden/ref_post.npz, made
by tests/golden/make_golden_post.py): normalize_ev, reweight_ev,
compute_distance, write_ev / read_ev, write_vfunc / read_vfunc (host code),
heat.diagonal / heat.kernel (GPU product; argument checks on the host)."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def post():
    return np.load(GOLD / "ref_post.npz")


def _mesh(name):
    from lapy_gb300 import TetMesh, TriaMesh

    f = np.load(GOLD / f"ref_{name}.npz")
    geo = TriaMesh(f["v"], f["t"]) if f["t"].shape[1] == 3 else TetMesh(f["v"], f["t"])
    return geo, f["evals"]


@pytest.mark.parametrize("name", ["ico3", "deformed3", "cubetria", "kuhn5"])
def test_normalize_and_reweight(post, name):
    from lapy_gb300 import shapedna

    geo, evals = _mesh(name)
    methods = ("surface", "volume", "geometry") if name != "kuhn5" else ("volume", "geometry")
    for m in methods:
        np.testing.assert_allclose(shapedna.normalize_ev(geo, evals, method=m), post[f"{name}_norm_{m}"],
                                   rtol=1e-12, atol=0)
    np.testing.assert_array_equal(shapedna.reweight_ev(evals), post[f"{name}_reweight"])
    with pytest.raises(ValueError, match="Unknown normalization method"):
        shapedna.normalize_ev(geo, evals, method="length")


def test_normalize_errors_and_distance(post):
    from lapy_gb300 import TriaMesh, shapedna

    tet, ev = _mesh("kuhn5")
    with pytest.raises(AttributeError):  # a tetrahedral mesh has no surface area (as in the reference)
        shapedna.normalize_ev(tet, ev, method="surface")
    # an open surface has no volume
    open_mesh = TriaMesh(np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]]), np.array([[0, 1, 2], [1, 3, 2]]))
    with pytest.raises(ValueError, match="closed"):
        shapedna.normalize_ev(open_mesh, np.ones(3), method="volume")
    a, ea = _mesh("ico3")
    b, eb = _mesh("deformed3")
    d = shapedna.compute_distance(shapedna.reweight_ev(shapedna.normalize_ev(a, ea)),
                                  shapedna.reweight_ev(shapedna.normalize_ev(b, eb)))
    np.testing.assert_allclose(d, post["dist_ico3_deformed3"], rtol=1e-12)
    with pytest.raises(ValueError, match="not implemented"):
        shapedna.compute_distance(ea, eb, dist="cos")


def test_mesh_measures():
    from lapy_gb300 import TriaMesh

    geo, _ = _mesh("ico3")
    assert geo.is_closed() and geo.is_oriented()
    flipped = TriaMesh(geo.v, geo.t[:, [0, 2, 1]])
    assert flipped.is_oriented()
    np.testing.assert_allclose(flipped.volume(), -geo.volume(), rtol=1e-14)
    mixed = geo.t.copy()
    mixed[0] = mixed[0, [0, 2, 1]]
    assert not TriaMesh(geo.v, mixed).is_oriented()
    with pytest.raises(ValueError, match="oriented"):
        TriaMesh(geo.v, mixed).volume()
    tet, _ = _mesh("kuhn5")
    # the boundary encloses the whole (jittered) cube: the sum of |tet volumes|
    p = [tet.v[tet.t[:, i]] for i in range(4)]
    vols = np.abs(np.sum(np.cross(p[1] - p[0], p[2] - p[0]) * (p[3] - p[0]), axis=1)) / 6
    np.testing.assert_allclose(tet.boundary_volume(), vols.sum(), rtol=1e-12)


def test_write_ev_matches_reference_text(post, tmp_path):
    from lapy_gb300 import io

    f = np.load(GOLD / "ref_kuhn5.npz")
    d = {"Creator": "1", "File": "2", "User": "3", "Refine": 0, "Degree": 1, "Dimension": 3,
         "Elements": int(len(f["t"])), "DoF": int(len(f["v"])), "NumEW": 4, "Area": 6.0, "Volume": 1.0,
         "BLength": 0.0, "EulerChar": 2, "TimePre": 0.5, "TimeCalcAB": 1.25, "TimeCalcEW": 2.0,
         "Eigenvalues": post["ev_input_evals"], "Eigenvectors": post["ev_input_evecs"]}
    io.write_ev(str(tmp_path / "a.ev"), d)
    assert (tmp_path / "a.ev").read_text() == str(post["ev_written"])
    back = io.read_ev(str(tmp_path / "a.ev"))
    assert sorted(back.keys()) == list(post["ev_read_keys"])
    np.testing.assert_array_equal(back["Eigenvalues"], post["ev_read_evals"])
    np.testing.assert_array_equal(back["Eigenvectors"], post["ev_read_evecs"])
    with pytest.raises(ValueError, match="no Eigenvalues"):
        io.write_ev(str(tmp_path / "b.ev"), {"NumEW": 3})


def test_read_ev_multiline_and_errors(post, tmp_path):
    from lapy_gb300 import io

    p = tmp_path / "m.ev"
    p.write_text(str(post["ev_multi_text"]))
    back = io.read_ev(str(p))
    assert sorted(back.keys()) == list(post["ev_multi_keys"])
    for key in ("Creator", "Refine", "Degree", "Dimension", "Elements", "DoF", "NumEW", "Area", "Volume",
                "BLength", "EulerChar", "TimePre", "TimeCalcAB", "TimeCalcEW"):
        assert back[key] == post[f"ev_multi_{key}"].item(), key
        assert type(back[key]) is type(post[f"ev_multi_{key}"].item()), key
    np.testing.assert_array_equal(back["Eigenvalues"], post["ev_multi_evals"])
    np.testing.assert_array_equal(back["Eigenvectors"], post["ev_multi_evecs"])
    np.testing.assert_array_equal(back["EigenvectorsSize"], post["ev_multi_sizes"])
    # header fields are read as numbers, as the reference does
    p.write_text(" Creator: lapy\n\nEigenvalues:\n{ 1.0 ; 2.0 }\n")
    with pytest.raises(ValueError):
        io.read_ev(str(p))
    with pytest.raises(OSError):
        io.read_ev(str(tmp_path / "missing.ev"))


def test_vfunc_roundtrip(post, tmp_path):
    from lapy_gb300 import io

    io.write_vfunc(str(tmp_path / "a.psol"), post["vfunc_input"])
    assert (tmp_path / "a.psol").read_text() == str(post["vfunc_written"])
    for key in ("comma", "semicolon_braces", "one_per_line"):
        p = tmp_path / f"{key}.psol"
        p.write_text(str(post[f"vfunc_text_{key}"]))
        assert io.read_vfunc(str(p)) == list(post[f"vfunc_read_{key}"])
    p = tmp_path / "bad.psol"
    p.write_text("1.0,2.0\n")
    with pytest.raises(ValueError, match="Solution"):
        io.read_vfunc(str(p))
    p.write_text("Solution:\n\n")
    with pytest.raises(ValueError, match="No vertex function"):
        io.read_vfunc(str(p))


def test_heat_kernel_argument_errors(post):
    """Checks that run before any device work (no GPU needed)."""
    from lapy_gb300 import heat

    ev, evec = post["hk_evals"], post["hk_evecs"]
    with pytest.raises(ValueError, match="exceeds"):
        heat.diagonal(post["hk_t3"], post["hk_x"], evec, ev[:, None], evec.shape[1] + 1)
    with pytest.raises(ValueError, match="exceeds"):
        heat.kernel(post["hk_t3"], 0, evec, ev[:, None], evec.shape[1] + 1)
    # a scalar time with 1-D eigenvalues: np.matmul rejects it, as in the reference
    with pytest.raises(ValueError):
        heat.diagonal(0.5, post["hk_x"], evec, ev, 4)
    # times as a row that does not broadcast against the n eigenvector entries
    with pytest.raises(ValueError):
        heat.kernel(np.array([[0.1, 0.2]]), 0, evec, ev[:, None], 3)


@pytest.mark.gpu
def test_heat_kernel_gpu_matches_reference(cuda_ok, post):
    from lapy_gb300 import heat

    ev, evec = post["hk_evals"], post["hk_evecs"]
    cases = [
        (heat.diagonal(post["hk_t3"], post["hk_x"], evec, ev[:, None], 8), post["hk_diag_rows"]),
        (heat.diagonal(post["hk_t3"], 5, evec, ev[:, None], 8), post["hk_diag_one"]),
        (heat.kernel(np.array([[0.2, 0.7, 3.0]]), 3, evec, ev[:, None], 3), post["hk_kernel_n3"]),
        (heat.kernel(np.array([[0.5]]), 11, evec, ev[:, None], 6), post["hk_kernel_t1"]),
    ]
    for got, want in cases:
        assert got.shape == want.shape
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14 * np.abs(want).max())
