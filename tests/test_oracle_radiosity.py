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
