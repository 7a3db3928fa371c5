"""GPU against the oracle on the workloads the metric is quoted on, at full size.

* Trench of oriented discs: width 1, depth 5, 3.0 x 3.0 x/y-periodic cell,
  0.02 grid (98,301 discs), source plane 0.1 above the top, cosine source,
  sticking 0.1, diffuse, 1e6 rays from Philox seed 0.
* Cylindrical hole: radius 0.5, depth 10, 2 x 2 periodic cell, 200,192 jittered
  triangles, sticking 0.01, 10 % specular / 90 % diffuse, 2e6 rays.
* The batch's extremes: aspect-ratio-20 trench and hole of about 5e5 discs
  each, sticking 0.01 with a cos^50 source (and the trench with a cosine
  source), 2e6 rays per job, traced through one CUDA-graph batch launch.

Bars (as in test_gpu_parity.py): hit counts and every tally bit for bit,
S1..S4 to 1e-9 relative (FP64 summation order), and, with fixed-point S1
accumulation, S1 bit for bit.  With independent random streams the flux per
depth band agrees within 4 sigma.
"""
import math

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
S1_RTOL = 1e-9


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def trench():
    t = scenes.trench_discs()  # width 1, depth 5, 3 x 3 cell, 0.02 grid, source 0.1 above the top
    assert t.n == 98301 and t.box_hi[2] == np.float32(0.1)
    return t


@pytest.fixture(scope="module")
def trench_oracle(trench, oracle_lib):
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    return s


@pytest.fixture(scope="module")
def hole():
    h = scenes.hole_triangles()
    assert h.n == 200192
    return h


def _compare(eng, c):
    t = eng.tally()
    assert np.array_equal(eng.hit_counts(), c.counts), "hit counts differ"
    assert (t.hitc, t.nonhitc, t.total, t.segments, t.truncated, t.nb_deposits) == \
        (c.hitc, c.nonhitc, c.total, c.segments, c.truncated, c.nb_deposits)
    assert t.errors == 0
    for a, b in zip(eng.accumulators(), (c.s1, c.s2, c.s3, c.s4)):
        np.testing.assert_allclose(a, b, rtol=S1_RTOL, atol=0)


def test_trench_discs_full_size(eng, trench, trench_oracle, oracle_lib):
    from rti_gb300 import _lib as L
    n = 1_000_000
    eng.upload_discs(trench.points, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), sticking=0.1, reflection=0, x_bound=1, y_bound=1,
                  source_exponent=1.0, reset=True)
    eng.trace(n, seed=0)
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, x_bound=1, y_bound=1, seed=0)
    c = trench_oracle.trace(cfg, 0, n)
    assert c.hitc > 3 * n and c.nb_deposits > n
    _compare(eng, c)
    eng.set_accumulation(L.RTG_ACCUM_FIXED)
    try:
        eng.trace(n, seed=0)
        cf = trench_oracle.trace(oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, seed=0,
                                                        accum_fixed=1), 0, n)
        assert np.array_equal(eng.values(), cf.s1)  # bit for bit
        assert np.array_equal(eng.hit_counts(), cf.counts)
    finally:
        eng.set_accumulation(L.RTG_ACCUM_FP64)


def test_trench_discs_full_size_independent_streams_4_sigma(eng, trench, trench_oracle, oracle_lib):
    """GPU (seed 100) and oracle (seed 200), 1e6 rays each: the flux summed over
    25 depth bands agrees within 4 sigma (sigma from the S2 sums, x4 for the
    correlated neighbour deposits of one path)."""
    n = 1_000_000
    eng.upload_discs(trench.points, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    eng.trace(n, seed=100)
    s1g, s2g, _, _ = eng.accumulators()
    c = trench_oracle.trace(oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, seed=200), 0, n)
    z = trench.points[:, 2]
    edges = np.quantile(z, np.linspace(0, 1, 26))
    band = np.clip(np.searchsorted(edges, z, side="right") - 1, 0, 24)
    xg = np.bincount(band, weights=s1g, minlength=25)
    xc = np.bincount(band, weights=c.s1, minlength=25)
    var = 4 * (np.bincount(band, weights=s2g, minlength=25) + np.bincount(band, weights=c.s2, minlength=25))
    ok = xg + xc > 0
    assert ok.sum() >= 20
    assert np.all(np.abs(xg - xc)[ok] <= 4 * np.sqrt(var[ok]))
    assert not np.array_equal(eng.hit_counts(), c.counts)


def test_hole_triangles_full_size(eng, hole, oracle_lib):
    from rti_gb300 import _lib as L
    n = 2_000_000
    eng.upload_triangles(hole.vertices, hole.indices)
    eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1,
                  x_bound=1, y_bound=1, source_exponent=1.0, reset=True)
    eng.trace(n, seed=0)
    s = oracle_lib.Scene(tri_vertices=hole.vertices, tri_indices=hole.indices)
    cfg = oracle_lib.make_config(hole.box_lo, hole.box_hi, sticking=0.01, reflection=2, specular_fraction=0.1,
                                 seed=0)
    c = s.trace(cfg, 0, n)
    assert c.segments > 8 * n
    _compare(eng, c)
    eng.set_accumulation(L.RTG_ACCUM_FIXED)
    try:
        eng.trace(n, seed=0)
        cf = s.trace(oracle_lib.make_config(hole.box_lo, hole.box_hi, sticking=0.01, reflection=2,
                                            specular_fraction=0.1, seed=0, accum_fixed=1), 0, n)
        assert np.array_equal(eng.values(), cf.s1)
        assert np.array_equal(eng.hit_counts(), cf.counts)
    finally:
        eng.set_accumulation(L.RTG_ACCUM_FP64)


def _extreme_instances():
    """The batch generator's rules at its largest aspect ratio (20) and disc
    count (5e5): a trench in a 3 x 3 cell and a hole of diameter 1 in a 2 x 2 cell."""
    ar, target = 20.0, 500_000
    s = 3.0 / round(3.0 / math.sqrt(3.0 * (3.0 + 2.0 * ar) / target))
    trench = scenes.trench_discs(width=1.0, depth=ar, domain=3.0, spacing=s)
    s = 2.0 / round(2.0 / math.sqrt((4.0 + math.pi * ar) / target))
    hole = scenes.hole_discs(radius=0.5, depth=ar, cell=2.0, spacing=s)
    return trench, hole


def test_batch_extreme_jobs_match_oracle(rtg_lib, oracle_lib):
    from rti_gb300 import Engine
    from rti_gb300.batch import Batch
    rays = 2_000_000
    inst = _extreme_instances()
    assert all(abs(s.n - 500_000) < 10_000 for s in inst)
    species = [(0, 0.01, 50.0), (1, 0.01, 50.0), (0, 0.01, 1.0)]  # (instance, sticking, exponent)
    engines = []
    with Batch(0) as b:
        for s in inst:
            e = Engine(0)
            e.upload_discs(s.points, s.normals, s.radii)
            e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, reset=True)
            engines.append(e)
        jobs = []
        for i, stick, expo in species:
            c = engines[i].config()
            c.sticking, c.source_exponent = stick, expo
            jobs.append((b.add(engines[i], rays, seed=11, config=c), i, stick, expo))
        b.run(use_graph=True)
        b.synchronize()
        t = b.tally()
        assert t.errors == 0 and t.num_rays == rays * len(jobs)
        results = {j: b.results(j) for j, *_ in jobs}
        segs = 0
        for i, s in enumerate(inst):
            sc = oracle_lib.Scene(s.xyzr, s.normals)
            sc.neighbors()
            for j, ii, stick, expo in jobs:
                if ii != i:
                    continue
                cfg = oracle_lib.make_config(s.box_lo, s.box_hi, sticking=stick, source_exponent=expo, seed=11,
                                             job=j)
                c = sc.trace(cfg, 0, rays)
                s1, cnt, _ = results[j]
                assert np.array_equal(cnt, c.counts), f"job {j}"
                np.testing.assert_allclose(s1, c.s1, rtol=S1_RTOL, atol=0)
                segs += c.segments
        assert segs == t.segments
    for e in engines:
        e.close()
