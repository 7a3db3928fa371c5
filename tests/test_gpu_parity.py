"""GPU path (librtg through its C ABI) against the CPU oracle on the same inputs.

Integer results (hit primitive ids, hit counts, tallies, neighbour lists) must
match bit for bit; hit distances too.  FP64 accumulators differ only by the
order of the additions: |S1_gpu - S1_cpu| <= 1e-9 * S1 (atomics on the GPU,
per-thread sums on the CPU).  Areas use CUDA's acos/sin: rtol 2e-5.
"""
import json
import os

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
S1_RTOL = 1e-9


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def trench():
    return scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)


@pytest.fixture(scope="module")
def hole():
    return scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)


def _random_rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def _upload_discs(eng, t, **cfg):
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), reset=True, **cfg)


def _compare_trace(g, c, np_):
    cnt = g["counts"]
    assert np.array_equal(cnt, c.counts), "hit counts differ"
    assert g["tally"].hitc == c.hitc
    assert g["tally"].nonhitc == c.nonhitc
    assert g["tally"].total == c.total
    assert g["tally"].segments == c.segments
    assert g["tally"].truncated == c.truncated
    assert g["tally"].nb_deposits == c.nb_deposits
    assert g["tally"].errors == 0
    for a, b in zip(g["s"], (c.s1, c.s2, c.s3, c.s4)):
        np.testing.assert_allclose(a, b, rtol=S1_RTOL, atol=0)


def _gpu_trace(eng, n, seed):
    eng.trace(n, seed)
    return {"counts": eng.hit_counts(), "s": eng.accumulators(), "tally": eng.tally()}


def test_closest_hit_discs_bit_exact(eng, trench, oracle_lib):
    _upload_discs(eng, trench)
    lo = np.array(trench.box_lo, np.float32)
    hi = np.array(trench.box_hi, np.float32)
    rays = _random_rays(50000, lo, hi, 0)
    pg, tg = eng.trace_rays(rays)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    pc, tc = s.closest_hit(rays)
    assert (pg >= 0).mean() > 0.3
    assert np.array_equal(pg, pc)
    assert np.array_equal(tg.view(np.uint32), tc.view(np.uint32))


def test_closest_hit_triangles_bit_exact(eng, hole, oracle_lib):
    eng.upload_triangles(hole.vertices, hole.indices)
    rays = _random_rays(50000, np.array(hole.box_lo, np.float32), np.array(hole.box_hi, np.float32), 1)
    pg, tg = eng.trace_rays(rays)
    s = oracle_lib.Scene(tri_vertices=hole.vertices, tri_indices=hole.indices)
    pc, tc = s.closest_hit(rays)
    assert (pg >= 0).mean() > 0.3
    assert np.array_equal(pg, pc)
    assert np.array_equal(tg.view(np.uint32), tc.view(np.uint32))


def test_compare_with_embree_two_discs(eng, oracle_lib):
    """test/rti/trace/local_intersector.cpp:131-268 restated at this boundary:
    two tilted discs, rays from z=10 to z=-1; whenever the closest hit is disc 1,
    local_intersector must report a hit on disc 1 and none on disc 0."""
    discs = np.array([[-2, -2, 0, 3], [3, 5, 0, 2.76]], np.float32)
    nrm = np.array([[0.5, 0.2, 1], [0.1, -0.155, 1]], np.float64)
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    eng.upload_discs(discs[:, :3], nrm, discs[:, 3])
    rng = np.random.default_rng(5)
    n = 1 << 20
    p1 = np.stack([rng.random(n) * 600 - 10, rng.random(n) * 20 - 10, np.full(n, 10.0)], 1)
    p2 = np.stack([rng.random(n) * 20 - 10, rng.random(n) * 20 - 10, np.full(n, -1.0)], 1)
    d = p2 - p1
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([p1, d], 1).astype(np.float32)
    prim, _ = eng.trace_rays(rays, tnear=0.0)
    idx = np.nonzero(prim == 1)[0]
    assert len(idx) > 1000
    for i in idx[:3000]:
        o, dd = rays[i, :3], rays[i, 3:]
        assert oracle_lib.local_intersect(o, dd, discs[1], nrm[1])
        assert not oracle_lib.local_intersect(o, dd, discs[0], nrm[0])


def test_neighbors_match_oracle(eng, trench, oracle_lib):
    _upload_discs(eng, trench)
    rg, cg = eng.neighbors()
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    rc, cc = s.neighbors()
    assert np.array_equal(rg, rc) and np.array_equal(cg, cc)


def test_neighbors_random_cloud(eng, oracle_lib):
    rng = np.random.default_rng(7)
    n = 20000
    p = (rng.random((n, 3)) * [2.0, 2.0, 0.5]).astype(np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm = (nrm / np.linalg.norm(nrm, axis=1, keepdims=True)).astype(np.float32)
    r = (0.005 + 0.02 * rng.random(n)).astype(np.float32)
    eng.upload_discs(p, nrm, r)
    rg, cg = eng.neighbors()
    s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
    rc, cc = s.neighbors()
    assert np.array_equal(rg, rc) and np.array_equal(cg, cc)


@pytest.mark.parametrize("builder", ["karras", "ploc"])
def test_large_surface_matches_oracle(eng, oracle_lib, builder):
    """70 000 discs on a bumpy plane: the build's scans (disc ranks, neighbour
    counts, PLOC compaction) run as multi-block passes; neighbour lists and
    the traced hits equal the oracle's under either tree."""
    from rti_gb300 import _lib as L
    rng = np.random.default_rng(8)
    side = 265
    g1 = (np.arange(side) + 0.5) * (2.0 / side)
    X, Y = np.meshgrid(g1, g1, indexing="ij")
    Z = 0.05 * np.sin(7 * X) * np.cos(5 * Y) + 0.01 * rng.standard_normal(X.shape)
    p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float32)
    nrm = np.tile(np.float32([0, 0, 1]), (len(p), 1))
    r = np.full(len(p), np.float32(1.1 * 2.0 / side), np.float32)
    assert len(p) > 4 * 16384
    eng.set_tree_builder(L.RTG_TREE_PLOC if builder == "ploc" else L.RTG_TREE_KARRAS)
    try:
        eng.upload_discs(p, nrm, r)
        lo, hi = np.float32([0, 0, -0.2]), np.float32([2, 2, 0.2])
        eng.configure(box=((0, 0, -0.2), (2, 2, 0.2)), sticking=0.3, x_bound=1, y_bound=1, reset=True)
        g = _gpu_trace(eng, 30000, seed=5)
        rg, cg = eng.neighbors()
        s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
        rc, cc = s.neighbors()
        assert np.array_equal(rg, rc) and np.array_equal(cg, cc)
        c = s.trace(oracle_lib.make_config(lo, hi, sticking=0.3, x_bound=1, y_bound=1, seed=5), 0, 30000)
        _compare_trace(g, c, len(p))
    finally:
        eng.set_tree_builder(L.RTG_TREE_KARRAS)


@pytest.mark.parametrize("bound", [1, 0], ids=["periodic", "reflective"])
def test_trace_trench_matches_oracle(eng, trench, oracle_lib, bound):
    _upload_discs(eng, trench, sticking=0.1, x_bound=bound, y_bound=bound)
    n = 200000
    g = _gpu_trace(eng, n, seed=11)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, x_bound=bound, y_bound=bound, seed=11)
    c = s.trace(cfg, 0, n)
    assert c.hitc > n
    _compare_trace(g, c, trench.n)


def test_trace_hole_mixed_reflection_matches_oracle(eng, hole, oracle_lib):
    eng.upload_triangles(hole.vertices, hole.indices)
    eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1,
                  x_bound=1, y_bound=1, reset=True)
    n = 100000
    g = _gpu_trace(eng, n, seed=3)
    s = oracle_lib.Scene(tri_vertices=hole.vertices, tri_indices=hole.indices)
    cfg = oracle_lib.make_config(hole.box_lo, hole.box_hi, sticking=0.01, reflection=2, specular_fraction=0.1,
                                 seed=3)
    c = s.trace(cfg, 0, n)
    assert c.hitc > 2 * n
    _compare_trace(g, c, hole.n)


def test_trace_power_cosine_and_sticking_field(eng, trench, oracle_lib):
    rng = np.random.default_rng(9)
    field = rng.uniform(0.05, 0.9, trench.n).astype(np.float32)
    _upload_discs(eng, trench, source_exponent=5.0, reflection=1, x_bound=1, y_bound=1)
    eng.set_sticking_field(field)
    n = 100000
    g = _gpu_trace(eng, n, seed=5)
    eng.set_sticking_field(None)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, source_exponent=5.0, reflection=1, seed=5)
    c = s.trace(cfg, 0, n, sticking_field=field)
    _compare_trace(g, c, trench.n)


def test_truncation_matches_oracle(eng, trench, oracle_lib):
    _upload_discs(eng, trench, sticking=0.02, max_segments=3, x_bound=1, y_bound=1)
    n = 50000
    g = _gpu_trace(eng, n, seed=2)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.02, max_segments=3, seed=2)
    c = s.trace(cfg, 0, n)
    assert c.truncated > 0
    _compare_trace(g, c, trench.n)
    eng.configure(max_segments=1 << 16)


def test_areas_estimates_and_stats(eng, trench, oracle_lib):
    _upload_discs(eng, trench, sticking=0.1, x_bound=1, y_bound=1)
    eng.trace(100000, 1)
    ag = eng.exposed_areas()
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    rp, cols = s.neighbors()
    ac = s.areas((trench.box_lo[0], trench.box_lo[1], trench.box_hi[0], trench.box_hi[1]))
    np.testing.assert_allclose(ag, ac, rtol=2e-5, atol=1e-12)
    s1, s2, s3, s4 = eng.accumulators()
    cnt = eng.hit_counts()
    tot = eng.tally().total
    est = eng.mc_estimates()
    ref = oracle_lib.normalize(s1, ag, rp, cols)
    np.testing.assert_allclose(est, ref, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(eng.relative_error(), oracle_lib.relative_error(s1, s2, tot), rtol=1e-12)
    np.testing.assert_allclose(eng.vov(), oracle_lib.vov(s1, s2, s3, s4, cnt, tot), rtol=1e-9)


def test_area_known_answers_on_gpu(eng):
    """The 37 exposed-area known answers, evaluated by the GPU area kernel."""
    cases = json.load(open(os.path.join(GOLDEN, "area_inside_cases.json")))
    by_box = {}
    for c in cases:
        by_box.setdefault(tuple(c["box"]), []).append(c)
    for box, cs in by_box.items():
        d = np.array([c["disc"] for c in cs], np.float32)
        n = np.array([c["normal"] for c in cs], np.float64)
        n = (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(np.float32)
        eng.upload_discs(d[:, :3], n, d[:, 3])
        eng.configure(box=((box[0], box[1], -100.0), (box[2], box[3], 100.0)), reset=True)
        a = eng.exposed_areas()
        for c, v in zip(cs, a):
            tol = max(c["tol"], 2e-6 * abs(c["expected"]))
            assert abs(float(v) - c["expected"]) <= tol, (c["name"], float(v), c["expected"])


def test_refit_after_move_equals_fresh_upload(eng, trench, oracle_lib):
    _upload_discs(eng, trench, sticking=0.1, x_bound=1, y_bound=1)
    moved = trench.points.copy()
    moved[:, 2] += (0.003 * np.sin(moved[:, 0] * 7)).astype(np.float32)
    eng.update_discs(moved, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    a = _gpu_trace(eng, 50000, seed=4)
    eng.upload_discs(moved, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    b = _gpu_trace(eng, 50000, seed=4)
    assert np.array_equal(a["counts"], b["counts"])
    assert a["tally"].segments == b["tally"].segments


def test_vertex_update_equals_fresh_upload(eng, hole):
    """Moved triangle vertices (rtg_update_vertices: refit, same topology) trace
    like a fresh upload of the moved mesh, and a refused update is reported."""
    from rti_gb300 import RtgError
    eng.upload_triangles(hole.vertices, hole.indices)
    moved = hole.vertices.copy()
    moved[:, 2] += (0.002 * np.cos(moved[:, 1] * 5)).astype(np.float32)
    eng.update_vertices(moved)
    eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, x_bound=1, y_bound=1, reset=True)
    a = _gpu_trace(eng, 50000, seed=6)
    with pytest.raises(RtgError):
        eng.update_vertices(moved[:-1])
    eng.upload_triangles(moved, hole.indices)
    eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, x_bound=1, y_bound=1, reset=True)
    b = _gpu_trace(eng, 50000, seed=6)
    assert np.array_equal(a["counts"], b["counts"])
    assert a["tally"].segments == b["tally"].segments


def test_abort_returns_status(eng, trench):
    from rti_gb300 import RtgError
    _upload_discs(eng, trench, sticking=0.001, x_bound=1, y_bound=1)
    eng.trace(50_000_000, 0)
    eng.request_abort()
    with pytest.raises(RtgError) as ei:
        eng.hit_counts()
    assert ei.value.code == 6
    eng.configure(sticking=0.1)


def test_visit_limit_returns_budget_error(eng, trench):
    """A closest-hit query that reaches the node-visit limit ends and is
    counted; the getters of that trace return RTG_ERR_BUDGET (5) in every
    schedule, as do explicit rays, the adjoint and a batch; the context stays
    usable, and with the limit lifted it traces exactly as before."""
    from rti_gb300 import RtgError
    from rti_gb300 import _lib as L
    from rti_gb300.batch import Batch
    _upload_discs(eng, trench, sticking=0.1, x_bound=1, y_bound=1)
    n = 20000
    ref = _gpu_trace(eng, n, seed=4)
    rays = _random_rays(2000, np.array(trench.box_lo, np.float32), np.array(trench.box_hi, np.float32), 1)
    prim_ref, t_ref = eng.trace_rays(rays)
    eng.set_visit_limit(1 << 40)  # capped at the automatic limit: no change
    assert np.array_equal(_gpu_trace(eng, n, seed=4)["counts"], ref["counts"])
    eng.set_visit_limit(3)
    assert eng.visit_limit == 3
    for sched in (L.RTG_SCHED_MEGAKERNEL, L.RTG_SCHED_WAVEFRONT, L.RTG_SCHED_PLAIN):
        eng.set_launch_config(scheduling=sched)
        eng.trace(n, 4)
        with pytest.raises(RtgError) as ei:
            eng.hit_counts()
        assert ei.value.code == L.RTG_ERR_BUDGET
        t = eng.tally()
        assert 0 < t.errors <= t.segments
    eng.set_launch_config()
    with pytest.raises(RtgError) as ei:
        eng.trace_rays(rays)
    assert ei.value.code == L.RTG_ERR_BUDGET
    with pytest.raises(RtgError) as ei:
        eng.adjoint(np.ones(trench.n), n, seed=4)
    assert ei.value.code == L.RTG_ERR_BUDGET
    with Batch(0) as b:
        b.add(eng, n, seed=4)
        b.run(use_graph=False)
        with pytest.raises(RtgError) as ei:
            b.synchronize()
        assert ei.value.code == L.RTG_ERR_BUDGET
    eng.set_visit_limit(0)
    again = _gpu_trace(eng, n, seed=4)
    assert np.array_equal(again["counts"], ref["counts"])
    assert again["tally"].errors == 0 and again["tally"].segments == ref["tally"].segments
    prim, t = eng.trace_rays(rays)
    assert np.array_equal(prim, prim_ref) and np.array_equal(t, t_ref)


def test_independent_streams_agree_within_4_sigma(eng, trench, oracle_lib):
    """GPU (seed 100) and oracle (seed 200) are independent Monte Carlo runs:
    the flux summed over 25 depth bands must agree within 4 sigma, sigma from
    the S2 sums (x4 for the correlated neighbour deposits of one path)."""
    _upload_discs(eng, trench, sticking=0.1, x_bound=1, y_bound=1)
    n = 400000
    g = _gpu_trace(eng, n, seed=100)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    c = s.trace(oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, seed=200), 0, n)
    z = trench.points[:, 2]
    edges = np.quantile(z, np.linspace(0, 1, 26))
    band = np.clip(np.searchsorted(edges, z, side="right") - 1, 0, 24)
    xg = np.bincount(band, weights=g["s"][0], minlength=25)
    xc = np.bincount(band, weights=c.s1, minlength=25)
    var = 4 * (np.bincount(band, weights=g["s"][1], minlength=25) + np.bincount(band, weights=c.s2, minlength=25))
    ok = xg + xc > 0
    assert np.all(np.abs(xg - xc)[ok] <= 4 * np.sqrt(var[ok]))
    assert not np.array_equal(g["counts"], c.counts)  # the streams really are independent


def test_fixed_point_flux_is_bit_exact(eng, trench, hole, oracle_lib):
    """RTG_ACCUM_FIXED: the GPU's S1 equals the oracle's bit for bit (order-
    independent integer sums), repeated traces give identical S1, and a trace
    split into two accumulated ray ranges equals the whole trace."""
    from rti_gb300 import RtgError, _lib as L
    from rti_gb300.batch import Batch
    eng.set_accumulation(L.RTG_ACCUM_FIXED)
    assert eng.accumulation == L.RTG_ACCUM_FIXED
    try:
        _upload_discs(eng, trench, sticking=0.1, x_bound=1, y_bound=1)
        n = 200000
        g1 = _gpu_trace(eng, n, seed=11)
        g2 = _gpu_trace(eng, n, seed=11)
        s = oracle_lib.Scene(trench.xyzr, trench.normals)
        s.neighbors()
        c = s.trace(oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, seed=11, accum_fixed=1), 0, n)
        assert np.array_equal(g1["s"][0], c.s1) and np.array_equal(g1["s"][0], g2["s"][0])
        eng.trace(n // 2, 11)
        eng.trace(n - n // 2, 11, ray_begin=n // 2, accumulate=True)
        assert np.array_equal(eng.accumulators()[0], g1["s"][0])
        eng.upload_triangles(hole.vertices, hole.indices)
        eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1,
                      x_bound=1, y_bound=1, reset=True)
        g = _gpu_trace(eng, 100000, seed=3)
        ch = oracle_lib.Scene(tri_vertices=hole.vertices, tri_indices=hole.indices).trace(
            oracle_lib.make_config(hole.box_lo, hole.box_hi, sticking=0.01, reflection=2, specular_fraction=0.1,
                                   seed=3, accum_fixed=1), 0, 100000)
        assert np.array_equal(g["s"][0], ch.s1)
        with Batch(0) as b:
            with pytest.raises(RtgError, match="FP64"):
                b.add(eng, 1000)
    finally:
        eng.set_accumulation(L.RTG_ACCUM_FP64)
