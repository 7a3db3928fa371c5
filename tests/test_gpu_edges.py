"""Edge cases of the GPU path against the oracle, and input validation.

Tiny and degenerate surfaces (one disc, one triangle, a flat plane, duplicate
discs sharing a centre, a zero-area triangle), an empty trace, and the inputs
the C ABI must refuse (non-finite values, non-unit normals, out-of-range
indices, a sticking field of the wrong length, an invalid configuration)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


def _box(lo, hi):
    return (tuple(float(x) for x in lo), tuple(float(x) for x in hi))


def _compare(eng, oracle_lib, scene, cfg_kw, n=20000, seed=1, **ekw):
    eng.configure(reset=True, **ekw)
    eng.trace(n, seed)
    cnt, s1, t = eng.hit_counts(), eng.values(), eng.tally()
    c = scene.trace(oracle_lib.make_config(seed=seed, **cfg_kw), 0, n)
    assert np.array_equal(cnt, c.counts)
    np.testing.assert_allclose(s1, c.s1, rtol=1e-9, atol=0)
    assert (t.hitc, t.nonhitc, t.segments, t.errors) == (c.hitc, c.nonhitc, c.segments, 0)
    return cnt


def test_single_disc_and_duplicates(eng, oracle_lib):
    lo, hi = np.array([-1, -1, -0.5], np.float32), np.array([1, 1, 0.5], np.float32)
    for pts in ([[0, 0, 0]], [[0, 0, 0], [0, 0, 0]], [[0, 0, 0], [0.1, 0, 0]]):
        p = np.array(pts, np.float32)
        nrm = np.tile(np.float32([0, 0, 1]), (len(p), 1))
        r = np.full(len(p), 0.5, np.float32)
        eng.upload_discs(p, nrm, r)
        s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
        s.neighbors()
        cnt = _compare(eng, oracle_lib, s, dict(box_lo=lo, box_hi=hi, sticking=0.5),
                       box=_box(lo, hi), x_bound=1, y_bound=1, sticking=0.5)
        assert cnt.sum() > 0
        if len(p) == 2 and p[1, 0] == 0:
            assert cnt[1] == 0 or cnt[0] > 0  # ties go to the lower id


def test_single_triangle_and_degenerate_triangle(eng, oracle_lib):
    lo, hi = np.array([-1, -1, -0.5], np.float32), np.array([1, 1, 0.5], np.float32)
    v = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0, 0, -0.2], [0, 0, -0.2], [0.5, 0.5, -0.2]], np.float32)
    for idx in ([[0, 1, 2]], [[0, 1, 2], [3, 4, 5]]):
        i = np.array(idx, np.uint32)
        eng.upload_triangles(v, i)
        s = oracle_lib.Scene(tri_vertices=v, tri_indices=i)
        cnt = _compare(eng, oracle_lib, s, dict(box_lo=lo, box_hi=hi, sticking=0.3),
                       box=_box(lo, hi), x_bound=1, y_bound=1, sticking=0.3)
        assert cnt[0] > 0
        if len(i) == 2:
            assert cnt[1] == 0  # zero area: never hit


def test_flat_plane_of_discs(eng, oracle_lib):
    g = np.arange(40) * 0.05
    X, Y = np.meshgrid(g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1).astype(np.float32)
    nrm = np.tile(np.float32([0, 0, 1]), (len(p), 1))
    r = np.full(len(p), np.float32(0.05 * np.sqrt(2) / 2), np.float32)
    eng.upload_discs(p, nrm, r)
    assert eng.tree_depth >= 1
    s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
    s.neighbors()
    lo, hi = np.array([0, 0, -0.1], np.float32), np.array([1.95, 1.95, 0.1], np.float32)
    _compare(eng, oracle_lib, s, dict(box_lo=lo, box_hi=hi, sticking=0.2), box=_box(lo, hi), x_bound=1, y_bound=1,
             sticking=0.2)


def test_empty_trace(eng):
    p = np.zeros((1, 3), np.float32)
    eng.upload_discs(p, np.float32([[0, 0, 1]]), np.float32([0.5]))
    eng.configure(box=((-1, -1, -1), (1, 1, 1)), reset=True)
    eng.trace(0, 0)
    assert eng.hit_counts().sum() == 0 and eng.tally().segments == 0


def test_invalid_inputs_are_refused(eng):
    from rti_gb300 import RtgError
    p = np.zeros((2, 3), np.float32)
    n = np.tile(np.float32([0, 0, 1]), (2, 1))
    r = np.full(2, 0.1, np.float32)
    with pytest.raises(RtgError, match="non-finite"):
        eng.upload_discs(np.float32([[0, 0, np.nan], [1, 0, 0]]), n, r)
    with pytest.raises(RtgError, match="unit length"):
        eng.upload_discs(p, np.float32([[0, 0, 2], [0, 0, 1]]), r)
    with pytest.raises(RtgError, match="radius"):
        eng.upload_discs(p, n, np.float32([0.1, -1]))
    with pytest.raises(RtgError, match="out of range"):
        eng.upload_triangles(np.zeros((3, 3), np.float32), np.uint32([[0, 1, 3]]))
    eng.upload_discs(p + np.float32([[0, 0, 0], [1, 0, 0]]), n, r)
    with pytest.raises(RtgError, match="length"):
        eng.set_sticking_field(np.full(3, 0.5, np.float32))
    with pytest.raises(RtgError, match="sticking"):
        eng.configure(sticking=2.0)
    with pytest.raises(RtgError, match="roulette"):
        eng.configure(roulette_threshold=0.5, roulette_weight=0.3)


def test_refused_upload_keeps_the_surface(eng):
    """A refused upload (of either half of a mixed surface) leaves the previous
    surface as it was: the same trace gives the same hits afterwards."""
    from rti_gb300 import RtgError
    from rti_gb300 import scenes
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), x_bound=1, y_bound=1, sticking=0.1, reset=True)
    eng.trace(50000, 3)
    before = eng.hit_counts()
    v = np.zeros((3, 3), np.float32)
    with pytest.raises(RtgError, match="out of range"):
        eng.upload_triangles(v, np.uint32([[0, 1, 3]]))
    with pytest.raises(RtgError, match="out of range"):
        eng.upload_mixed(t.points, t.normals, t.radii, v, np.uint32([[0, 1, 7]]))
    bad = t.points.copy()
    bad[5, 2] = np.nan
    with pytest.raises(RtgError, match="non-finite"):
        eng.upload_discs(bad, t.normals, t.radii)
    assert eng.num_primitives == t.n
    eng.trace(50000, 3)
    assert np.array_equal(eng.hit_counts(), before)


@pytest.mark.parametrize("n", [1, 2, 3, 8192, 8193, 20000])
def test_ploc_sizes_around_the_single_block_tail(eng, oracle_lib, n):
    """PLOC builds whose last rounds run in one block (at most 8 Ki clusters)
    and builds that reach it after round-by-round launches: each builds
    without error and traces as the oracle does."""
    from rti_gb300 import _lib as L
    rng = np.random.default_rng(n)
    c = np.stack([rng.uniform(0, 1, n), rng.uniform(0, 1, n), rng.uniform(-0.5, 0, n)], 1).astype(np.float32)
    nrm = rng.normal(size=(n, 3)) + [0, 0, 1.5]
    nrm = (nrm / np.linalg.norm(nrm, axis=1)[:, None]).astype(np.float32)
    r = rng.uniform(0.003, 0.02, n).astype(np.float32)
    eng.set_tree_builder(L.RTG_TREE_PLOC)
    try:
        eng.upload_discs(c, nrm, r)
        assert 1 <= eng.tree_depth <= 256 or n == 1
        s = oracle_lib.Scene(np.concatenate([c, r[:, None]], 1), nrm)
        s.neighbors(bruteforce=True)
        lo, hi = np.array([0, 0, -0.6], np.float32), np.array([1, 1, 0.1], np.float32)
        _compare(eng, oracle_lib, s, dict(box_lo=lo, box_hi=hi, sticking=0.3), n=5000, box=_box(lo, hi),
                 x_bound=1, y_bound=1, sticking=0.3)
    finally:
        eng.set_tree_builder(L.RTG_TREE_KARRAS)
