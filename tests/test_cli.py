"""The command-line driver (rti_gb300/rtg, the counterpart of rti's dev.cpp).

CPU tests cover argument handling up to the first GPU call; the GPU test runs
a trace from a VTP file and checks the output file against the same trace
through the Python binding (bit-identical hit counts)."""
import os
import subprocess
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from rti_gb300 import scenes, vtk

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "rti_gb300", "rtg")


@pytest.fixture(scope="module")
def cli(rtg_lib):
    if not os.path.exists(CLI):
        from rti_gb300 import build
        build.build_cli()
    return CLI


def test_usage_and_vtk_extension(cli, tmp_path):
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode != 0 and "usage" in r.stdout
    r = subprocess.run([cli, "-i", str(tmp_path / "a.vtk"), "-s", "7"], capture_output=True, text=True)
    assert r.returncode != 0
    assert "reset to sane value" in r.stdout and "sticking coefficient == 1" in r.stdout
    assert "convert the input file to vtp" in r.stdout
    r = subprocess.run([cli, "-i", str(tmp_path / "missing.vtp")], capture_output=True, text=True)
    assert r.returncode != 0 and "cannot read" in r.stderr


def _cells(path):
    piece = ET.parse(path).getroot().find("PolyData/Piece")
    return {da.get("Name"): np.array(da.text.split(), dtype=np.float64) for da in piece.find("CellData")}


@pytest.mark.gpu
def test_cli_trace_matches_binding(cli, tmp_path):
    from rti_gb300 import Engine
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    inp = tmp_path / "trench.vtp"
    vtk.write_vtp_discs(str(inp), t.points, t.normals, t.radii)
    out = tmp_path / "res"
    r = subprocess.run([cli, "-i", str(inp), "-o", str(out), "-r", "200000", "-s", "0.1", "--seed", "3",
                        "--ray-log", "20"], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert os.path.exists(str(out) + ".vtp") and os.path.exists(str(out) + ".bounding-box.vtp")
    cells = _cells(str(out) + ".vtp")
    lo = t.points.min(axis=0)
    hi = t.points.max(axis=0)
    hi[2] = np.float32(hi[2] + t.radii.max())
    with Engine(0) as e:
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(lo, hi), x_bound=1, y_bound=1, sticking=0.1, reflection=0, source_exponent=1.0,
                    reset=True)
        e.trace(200000, seed=3)
        np.testing.assert_array_equal(cells["hitcnt"], e.hit_counts().astype(np.float64))
        np.testing.assert_allclose(cells["value"], e.values(), rtol=1e-15)
        np.testing.assert_allclose(cells["exposed-area"], e.exposed_areas(), rtol=1e-7)
        np.testing.assert_allclose(cells["relative-error"], e.relative_error(), rtol=1e-12, atol=1e-300)
        # the ray log of the first 20 rays (rti's raylog.vtp) equals the binding's segment log
        e.set_segment_log(0, 20, 1 << 20)
        e.trace(200000, seed=3)
        log, _ = e.segment_log()
    assert cells["hitcnt"].sum() > 0
    piece = ET.parse(tmp_path / "raylog.vtp").getroot().find("PolyData/Piece")
    assert int(piece.get("NumberOfLines")) == len(log) > 20
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(pts[0::2], log["org"])
    v, tri = vtk.read_triangles(str(out) + ".bounding-box.vtp")
    assert v.shape == (8, 3) and tri.shape == (8, 3)


@pytest.mark.gpu
def test_write_vtp_mixed_context(rtg_lib, tmp_path):
    from rti_gb300 import Engine
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    h = scenes.hole_triangles(n_theta=32, n_wall=8, n_top=4, n_bottom=3, depth=1.0, cell=1.2)
    with Engine(0) as e:
        e.upload_mixed(t.points, t.normals, t.radii, h.vertices + np.float32([0.6, 0.6, -2.0]), h.indices)
        e.configure(box=((0.0, 0.0, -3.5), (1.2, 1.2, 0.1)), x_bound=1, y_bound=1, sticking=0.2, reset=True)
        e.trace(100000, seed=1)
        f = tmp_path / "mixed.vtp"
        vtk.write_vtp(e, str(f), {"geo-name": "mixed"})
        piece = ET.parse(f).getroot().find("PolyData/Piece")
        assert int(piece.get("NumberOfVerts")) == t.n and int(piece.get("NumberOfPolys")) == h.n
        cells = _cells(f)
        np.testing.assert_array_equal(cells["hitcnt"], e.hit_counts().astype(np.float64))
        np.testing.assert_allclose(cells["value"], e.values(), rtol=1e-15)
        nrm = cells["Normals"].reshape(-1, 3)
        np.testing.assert_allclose(nrm[:t.n], t.normals, atol=1e-7)
        np.testing.assert_allclose(np.linalg.norm(nrm[t.n:], axis=1), 1.0, atol=1e-6)
