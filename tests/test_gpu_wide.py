"""The compressed 8-wide tree of the closest-hit query (rtg_set_node_width).

Its child boxes are byte-quantised on a per-node grid that contains the binary
tree's float boxes, and its slab test is widened by a bound on every rounding,
so it enters every box the binary traversal would need and the closest hit
(ties to the lower id) cannot change: every result below is compared with the
binary tree bit for bit -- explicit rays (primitive ids and distances), full
traces (hit counts, tallies, S1..S4 to the FP64 summation order), the window
deposit, the adjoint replays, the plain and wavefront schedules, batches,
refits -- and with the oracle.
"""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
BINARY, WIDE = 2, 8


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


def _rays(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    o = np.asarray(lo, np.float64) + (np.asarray(hi, np.float64) - np.asarray(lo, np.float64)) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # a few exactly axis-parallel directions (1/d clamped) as well
    d[: n // 50] = np.eye(3)[rng.integers(0, 3, n // 50)] * rng.choice([-1.0, 1.0], (n // 50, 1))
    return np.concatenate([o, d], 1).astype(np.float32)


def _both(eng, fn):
    out = []
    for w in (BINARY, WIDE):
        eng.set_node_width(w)
        out.append(fn())
    eng.set_node_width(0)
    return out


def _trace(eng, n, seed):
    eng.trace(n, seed)
    t = eng.tally()
    return eng.hit_counts(), eng.accumulators(), (t.hitc, t.nonhitc, t.total, t.segments, t.nb_deposits, t.errors)


def _same_trace(a, b):
    assert np.array_equal(a[0], b[0]), "hit counts differ"
    assert a[2] == b[2] and a[2][-1] == 0
    for x, y in zip(a[1], b[1]):
        np.testing.assert_allclose(x, y, rtol=1e-9, atol=0)


def _scenes():
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    h = scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    r = scenes.rough_discs(n=128, spacing=0.01, rms=0.05, corr=0.2, seed=3)
    quad = np.float32([[-0.6, -0.6, -0.55], [0.6, -0.6, -0.55], [0.6, 0.6, -0.55], [-0.6, 0.6, -0.55]])
    return {
        "trench": (lambda e: e.upload_discs(t.points, t.normals, t.radii), (t.box_lo, t.box_hi), 0.1),
        "hole": (lambda e: e.upload_triangles(h.vertices, h.indices), (h.box_lo, h.box_hi), 0.01),
        "rough": (lambda e: e.upload_discs(r.points, r.normals, r.radii), (r.box_lo, r.box_hi), 0.2),
        "mixed": (lambda e: e.upload_mixed(t.points, t.normals, t.radii, quad, np.uint32([[0, 1, 2], [0, 2, 3]])),
                  (t.box_lo, t.box_hi), 0.2),
    }


@pytest.mark.parametrize("kind", ["trench", "hole", "rough", "mixed"])
@pytest.mark.parametrize("builder", [0, 1], ids=["karras", "ploc"])
def test_wide_equals_binary(eng, kind, builder):
    upload, box, sticking = _scenes()[kind]
    eng.set_tree_builder(builder)
    try:
        upload(eng)
        eng.configure(box=box, sticking=sticking, reflection=2, specular_fraction=0.1, x_bound=1, y_bound=1,
                      reset=True)
        rays = _rays(200000, box[0], box[1], 11)
        (pb, tb), (pw, tw) = _both(eng, lambda: eng.trace_rays(rays))
        assert (pb >= 0).mean() > 0.2
        assert np.array_equal(pb, pw) and np.array_equal(tb.view(np.uint32), tw.view(np.uint32))
        a, b = _both(eng, lambda: _trace(eng, 100000, 5))
        _same_trace(a, b)
    finally:
        eng.set_tree_builder(0)


def test_wide_matches_oracle_on_the_trench(eng, oracle_lib):
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    eng.set_node_width(WIDE)
    try:
        g = _trace(eng, 200000, 11)
    finally:
        eng.set_node_width(0)
    s = oracle_lib.Scene(t.xyzr, t.normals)
    s.neighbors()
    c = s.trace(oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.1, seed=11), 0, 200000)
    assert np.array_equal(g[0], c.counts)
    assert g[2][:5] == (c.hitc, c.nonhitc, c.total, c.segments, c.nb_deposits)
    np.testing.assert_allclose(g[1][0], c.s1, rtol=1e-9, atol=0)


def test_wide_in_every_schedule_window_and_adjoint(eng):
    from rti_gb300 import _lib as L
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    for kw in ({"scheduling": L.RTG_SCHED_PLAIN}, {"scheduling": L.RTG_SCHED_WAVEFRONT},
               {"threads_per_block": 256, "packet": 8, "stack_memory": L.RTG_STACK_SHARED}):
        eng.set_launch_config(**kw)
        a, b = _both(eng, lambda: _trace(eng, 60000, 3))
        _same_trace(a, b)
    eng.set_launch_config()
    eng.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
    a, b = _both(eng, lambda: _trace(eng, 60000, 4))
    _same_trace(a, b)
    eng.set_deposit_mode(L.RTG_DEPOSIT_NEIGHBORS, 5.0)
    g = np.random.default_rng(2).random(t.n)
    for unbiased in (False, True):
        a, b = _both(eng, lambda: eng.adjoint(g, 60000, seed=6, unbiased=unbiased))
        np.testing.assert_allclose(a[:2], b[:2], rtol=1e-9)
    field = np.random.default_rng(3).uniform(0.05, 0.5, t.n).astype(np.float32)
    eng.set_sticking_field(field)
    a, b = _both(eng, lambda: eng.adjoint(g, 60000, seed=6, unbiased=False))
    np.testing.assert_allclose(a[2], b[2], rtol=1e-9, atol=1e-12 * np.abs(a[2]).max())
    eng.set_sticking_field(None)


def test_wide_batch_and_refit(eng, rtg_lib):
    from rti_gb300 import Engine
    from rti_gb300.batch import Batch
    inst = scenes.batch_instances(n=3, seed=4, min_discs=3000, max_discs=9000, aspect=(2.0, 6.0))
    engines, res = [], {}
    for s in inst:
        e = Engine(0)
        e.upload_discs(s.points, s.normals, s.radii)
        e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, sticking=0.05, reset=True)
        engines.append(e)
    with Batch(0) as b:
        for e in engines:
            b.add(e, 30000, seed=2)
        for w in (BINARY, WIDE):
            for e in engines:
                e.set_node_width(w)  # the batch prepares the changed contexts again
            b.run(use_graph=True)
            b.synchronize()
            res[w] = [b.results(j)[1] for j in range(len(b))]
    for x, y in zip(res[BINARY], res[WIDE]):
        assert np.array_equal(x, y)
    for e in engines:
        e.close()
    # the wide tree follows a refit (moved discs, same topology) like the binary one
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    moved = t.points.copy()
    moved[:, 2] += (0.003 * np.sin(moved[:, 0] * 7)).astype(np.float32)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.update_discs(moved, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    a, b = _both(eng, lambda: _trace(eng, 50000, 4))
    _same_trace(a, b)


def test_single_primitive_and_far_coordinates(eng):
    """One disc (its leaf twice in the binary root), and a trench far from the
    origin and 6000 units wide (wider than the byte grid allows: the wide tree
    is left out and the binary one serves; results unchanged)."""
    eng.upload_discs(np.float32([[0.5, 0.5, 0.0]]), np.float32([[0, 0, 1]]), np.float32([0.3]))
    eng.configure(box=((0, 0, -1), (1, 1, 0.1)), sticking=0.5, x_bound=1, y_bound=1, reset=True)
    a, b = _both(eng, lambda: _trace(eng, 20000, 1))
    _same_trace(a, b)
    assert a[0][0] > 0
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    for scale, shift in ((1.0, 3.0e3), (5000.0, 0.0)):
        p = (t.points.astype(np.float64) * scale + shift).astype(np.float32)
        eng.upload_discs(p, t.normals, (t.radii.astype(np.float64) * scale).astype(np.float32))
        lo = tuple(float(np.float32(x * scale + shift)) for x in t.box_lo)
        hi = tuple(float(np.float32(x * scale + shift)) for x in t.box_hi)
        eng.configure(box=(lo, hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
        a, b = _both(eng, lambda: _trace(eng, 50000, 2))
        _same_trace(a, b)


def test_node_width_setting_and_autotune(eng):
    from rti_gb300 import RtgError
    from rti_gb300 import _lib as L
    assert eng.node_width == L.RTG_NODES_AUTO
    with pytest.raises(RtgError, match="node width"):
        eng.set_node_width(4)
    # automatic: a surface whose tree stays in L2 is traced over the binary tree
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    assert not eng.uses_wide_tree
    eng.set_node_width(L.RTG_NODES_WIDE)
    assert eng.uses_wide_tree
    eng.set_node_width(L.RTG_NODES_AUTO)
    h = scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    eng.upload_triangles(h.vertices, h.indices)
    eng.configure(box=(h.box_lo, h.box_hi), sticking=0.01, x_bound=1, y_bound=1, reset=True)
    ref = _trace(eng, 60000, 1)
    cfg, rate = eng.autotune(60000, seed=1)
    assert rate > 0 and eng.node_width in (L.RTG_NODES_BINARY, L.RTG_NODES_WIDE)
    _same_trace(ref, _trace(eng, 60000, 1))
    eng.set_node_width(0)
    eng.set_launch_config()
    eng.set_tree_builder(0)
