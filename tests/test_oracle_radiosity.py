"""The oracle itself against the reference's analytical radiosity curves (CPU).

Same check as tests/test_gpu_radiosity.py with fewer rays: the oracle traces
a triangle-mesh cylinder of radius 0.5 and depth 45 and its max-normalised
wall flux per depth bin must match verification/radiosity/analytical_solution/
sp.{1,0.1}.data to 3 % relative L2 error.
"""
import os

import numpy as np
import pytest

from rti_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def cyl_scene(oracle_lib):
    c = scenes.cylinder_triangles(radius=0.5, depth=45.0, cell=1.5, n_theta=64, n_wall=300, n_top=4, n_bottom=4)
    return c, oracle_lib.Scene(tri_vertices=c.vertices, tri_indices=c.indices)


@pytest.mark.parametrize("sp,n_rays", [("1", 1_500_000), ("0.1", 800_000)])
def test_oracle_ar45_wall_flux(oracle_lib, cyl_scene, sp, n_rays):
    cyl, scene = cyl_scene
    s = float(sp)
    cfg = oracle_lib.make_config(cyl.box_lo, cyl.box_hi, sticking=s, seed=77)
    r = scene.trace(cfg, 0, n_rays)
    area = scene.areas((cyl.box_lo[0], cyl.box_lo[1], cyl.box_hi[0], cyl.box_hi[1]))
    V = cyl.vertices.astype(np.float64)
    c = V[cyl.indices].mean(axis=1)
    wall = (c[:, 2] < -1e-6) & (c[:, 2] > -45.0 + 1e-6)
    bins = np.minimum((-c[wall, 2] / 0.15).astype(int), 299)
    flux = np.bincount(bins, weights=r.s1[wall] / s, minlength=300)
    a = np.bincount(bins, weights=area[wall].astype(np.float64), minlength=300)
    gamma = flux / a
    ref = np.loadtxt(os.path.join(GOLDEN, f"radiosity_ar45_sp{sp}.txt"))
    err = np.linalg.norm(gamma / gamma.max() - ref[:, 1]) / np.linalg.norm(ref[:, 1])
    assert err < 0.03, err


# ---- the deterministic radiosity solvers (oracle/radiosity.py) -------------

@pytest.mark.parametrize("sp,tol", [("1", 1e-9), ("0.1", 0.005), ("0.01", 0.005)])
def test_radiosity_solver_reproduces_rti_ar45(sp, tol):
    """The cylinder solver against rti's analytical curves: at sticking 1 the
    curve is the direct view factor to the opening, reproduced to rounding;
    with re-emission the 900-band discretisation agrees to 0.5 %."""
    from oracle import radiosity as RD
    h = RD.hole(0.5, 45.0, float(sp), n_wall=900, n_bottom=20)
    assert np.allclose(h["row_sums"], 1.0, atol=1e-9)
    g = h["wall"].reshape(300, 3).mean(1)
    ref = np.loadtxt(os.path.join(GOLDEN, f"radiosity_ar45_sp{sp}.txt"))
    err = np.linalg.norm(g / g.max() - ref[:, 1]) / np.linalg.norm(ref[:, 1])
    assert err < tol, err
    if sp == "1":
        assert abs(g[0] - 0.4306) < 1e-3  # absolute top-bin flux, units of the flat-surface flux


def test_trench_solver_is_an_enclosure():
    from oracle import radiosity as RD
    t = RD.trench(1.0, 5.0, 0.2, n_wall=100, n_bottom=40)
    assert np.allclose(t["row_sums"], 1.0, atol=1e-9)
    assert np.allclose(t["wall"], t["right_wall"], rtol=1e-12)
    # sticking 1: the flux is the direct view factor to the opening; from the
    # middle of the bottom the opening spans +-atan(0.5 / 5), F = sin of that
    t1 = RD.trench(1.0, 5.0, 1.0, n_wall=100, n_bottom=40)
    mid = 0.5 * (t1["bottom"][19] + t1["bottom"][20])
    assert abs(mid - 0.5 / np.hypot(0.5, 5.0)) < 1e-4, mid
    assert np.all(np.diff(t1["wall"]) < 0)  # the direct flux falls with depth


def _band_flux(values, area, key, edges):
    """Area-weighted mean of values over primitives grouped by key into bins."""
    b = np.digitize(key, edges) - 1
    ok = (b >= 0) & (b < len(edges) - 1)
    num = np.bincount(b[ok], weights=values[ok], minlength=len(edges) - 1)
    den = np.bincount(b[ok], weights=area[ok], minlength=len(edges) - 1)
    return num / den


def test_oracle_trench_matches_radiosity(oracle_lib):
    """The oracle's Monte Carlo flux in a triangle-mesh trench (width 1, depth 5,
    diffuse, sticking 0.3) against the crossed-string radiosity solution."""
    from oracle import radiosity as RD
    t = scenes.trench_triangles(width=1.0, depth=5.0, cell=3.0, n_wall=10, n_bottom=5, n_top=2, n_y=2)
    scene = oracle_lib.Scene(tri_vertices=t.vertices, tri_indices=t.indices)
    s, n = 0.3, 600_000
    r = scene.trace(oracle_lib.make_config(t.box_lo, t.box_hi, sticking=s, seed=5), 0, n)
    V = t.vertices.astype(np.float64)
    area = 0.5 * np.linalg.norm(np.cross(V[t.indices[:, 1]] - V[t.indices[:, 0]],
                                         V[t.indices[:, 2]] - V[t.indices[:, 0]]), axis=1)
    c = V[t.indices].mean(axis=1)
    g = r.s1 / s / (n / 9.0)                      # incoming flux per primitive, units of E0 x area
    wall = (np.abs(c[:, 0] - 1.0) < 1e-6) | (np.abs(c[:, 0] - 2.0) < 1e-6)
    sim = _band_flux(g[wall], area[wall], -c[wall, 2], np.linspace(0, 5, 11))
    ref = RD.trench(1.0, 5.0, s, n_wall=100, n_bottom=50)["wall"].reshape(10, 10).mean(1)
    err = np.linalg.norm(sim - ref) / np.linalg.norm(ref)
    assert err < 0.04, (err, sim, ref)


def test_radiosity_derivatives_match_differences():
    """dG/ds of both solvers and the per-strip field gradient of the trench
    against central differences of the solutions themselves."""
    from oracle import radiosity as RD
    h = 1e-6
    for solve in (lambda s: RD.trench(1.0, 5.0, s, 60, 20), lambda s: RD.hole(0.5, 10.0, s, 200, 20)):
        a, p, m = solve(0.1), solve(0.1 + h), solve(0.1 - h)
        fd = (p["wall"] - m["wall"]) / (2 * h)
        assert np.max(np.abs(fd - a["d_wall"])) < 1e-7 * np.max(np.abs(a["d_wall"])) + 1e-9
    r = RD.trench_field_gradient(1.0, 5.0, 0.1, 20, 10, length=3.0)
    sig = np.full(50, 0.1)
    for j in (0, 7, 19, 20, 24, 29, 30, 49):
        sp, sm = sig.copy(), sig.copy()
        sp[j] += h
        sm[j] -= h
        fd = (RD.trench_field_gradient(1.0, 5.0, sp, 20, 10, 3.0)["L"] -
              RD.trench_field_gradient(1.0, 5.0, sm, 20, 10, 3.0)["L"]) / (2 * h)
        assert abs(fd - r["grad"][j]) < 1e-7 * np.max(np.abs(r["grad"])), (j, fd, r["grad"][j])
