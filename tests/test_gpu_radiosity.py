"""End-to-end flux against the reference's radiosity verification data.

verification/radiosity/analytical_solution/sp.{1,0.1,0.01}.data (copied to
tests/golden/) is the analytical wall flux of a cylinder of radius 0.5 and
length 45 under a cosine source, with diffuse re-emission at sticking
1 / 0.1 / 0.01, as max-normalised flux against normalised depth in 300 bins.
The GPU traces a triangle-mesh hole of the same shape (128 facets around,
600 rings, so two rings per analytical bin) and the wall flux per bin, divided
by the flux density on the flat top, must match the curve to a relative L2
error of 2 % (max-normalised, as the reference's own plots compare them).
"""
import os

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
L2_TOL = 0.02


@pytest.fixture(scope="module")
def cyl():
    return scenes.cylinder_triangles(radius=0.5, depth=45.0, cell=1.5, n_theta=128, n_wall=600, n_top=8,
                                     n_bottom=8)


@pytest.mark.parametrize("sp,n_rays", [("1", 20_000_000), ("0.1", 20_000_000), ("0.01", 20_000_000)])
def test_ar45_wall_flux_matches_radiosity(rtg_lib, cyl, sp, n_rays):
    from rti_gb300 import Engine
    s = float(sp)
    with Engine(0) as e:
        e.upload_triangles(cyl.vertices, cyl.indices)
        e.configure(box=(cyl.box_lo, cyl.box_hi), sticking=s, x_bound=1, y_bound=1, reflection=0)
        e.trace(n_rays, seed=123)
        s1 = e.values()
        area = e.exposed_areas()
        tal = e.tally()
    assert tal.errors == 0 and tal.truncated == 0
    V, T = cyl.vertices.astype(np.float64), cyl.indices
    c = V[T].mean(axis=1)
    wall = (c[:, 2] < -1e-6) & (c[:, 2] > -45.0 + 1e-6)
    depth = -c[wall, 2]
    bins = np.minimum((depth / 0.15).astype(int), 299)
    flux = np.bincount(bins, weights=s1[wall] / s, minlength=300)
    a = np.bincount(bins, weights=area[wall].astype(np.float64), minlength=300)
    cell_area = (cyl.box_hi[0] - cyl.box_lo[0]) * (cyl.box_hi[1] - cyl.box_lo[1])
    gamma = flux / a / (n_rays / cell_area)          # wall flux / flat-surface flux density
    ref = np.loadtxt(os.path.join(GOLDEN, f"radiosity_ar45_sp{sp}.txt"))
    sim = gamma / gamma.max()
    err = np.linalg.norm(sim - ref[:, 1]) / np.linalg.norm(ref[:, 1])
    print(f"sp={sp}: L2 relative error {err:.4f}, top-bin flux {gamma[0]:.4f}, hits/ray {tal.hitc / n_rays:.2f}")
    assert err < L2_TOL
