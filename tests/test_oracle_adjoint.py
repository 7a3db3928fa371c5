"""The oracle's field adjoint (held estimator) against central differences of
its own traces with common random numbers (CPU only).

The held estimator is the derivative that CRN differences measure: a step of
1e-3 s_j moves the weights of the paths through element j but flips a
roulette decision only rarely.  Two sticking levels exercise both ways the
deferred terms -T/(1 - s_j) are added: from the per-stretch list (short
stretches, s = 0.3) and by tracing a long stretch again (s = 0.02, more than
32 deposits between roulette resets)."""
import numpy as np
import pytest

from rti_gb300 import scenes

RAYS = 20000


@pytest.mark.parametrize("level", [0.3, 0.02])
def test_field_gradient_vs_crn_differences(oracle_lib, level):
    O = oracle_lib
    t = scenes.trench_discs(domain=0.6, width=0.2, depth=0.4)
    s = O.Scene(t.xyzr, t.normals)
    s.neighbors()
    rng = np.random.default_rng(4)
    field = (level * rng.uniform(0.8, 1.2, t.n)).astype(np.float32)
    g = (t.points[:, 2] < -0.2).astype(np.float64)
    cfg = O.make_config(t.box_lo, t.box_hi, seed=3)
    _, _, fg, _ = O.adjoint(s, cfg, g, 0, RAYS, nthreads=2, sticking_field=field, unbiased=False)

    def L(f):
        c = O.make_config(t.box_lo, t.box_hi, seed=3)
        return float(g @ s.trace(c, 0, RAYS, nthreads=2, sticking_field=f).s1)

    hit = np.nonzero(s.trace(cfg, 0, RAYS, nthreads=2, sticking_field=field).counts > 20)[0]
    bad = 0
    for j in rng.choice(hit, 6, replace=False):
        h = np.float32(1e-3) * field[j]
        fp, fm = field.copy(), field.copy()
        fp[j] += h
        fm[j] -= h
        fd = (L(fp) - L(fm)) / (float(fp[j]) - float(fm[j]))
        if not abs(fg[j] - fd) <= 1e-3 * max(abs(fd), 1e-6 * np.abs(fg).max()):
            bad += 1
    assert bad <= 1


def test_oracle_fixed_point_flux_is_order_independent(oracle_lib):
    """accum_fixed: S1 summed as integer multiples of 2^-32 does not depend on
    how the rays are split over threads, and stays within 1e-6 of FP64 sums."""
    from rti_gb300 import scenes
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    s = oracle_lib.Scene(t.xyzr, t.normals)
    s.neighbors()
    cfg = lambda fixed: oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.1, seed=3, accum_fixed=fixed)
    a = s.trace(cfg(1), 0, 40000, nthreads=1)
    b = s.trace(cfg(1), 0, 40000, nthreads=4)
    c = s.trace(cfg(0), 0, 40000, nthreads=4)
    assert np.array_equal(a.s1, b.s1) and np.array_equal(a.counts, c.counts)
    np.testing.assert_allclose(a.s1, c.s1, rtol=1e-6, atol=1e-9)
