"""The oracle's multi-hit window deposit (rti trace/point_cloud_context.hpp:
132-173,265-286) on scenes whose outcome is known in closed form.

Two large parallel discs, 0.1 apart, under a periodic 1 x 1 cell, sticking 1:
every source ray hits the upper disc first from the front, which opens the
window; the lower disc is collected when its hit lies within window_factor
radii of the first hit and before the ray leaves the cell sideways.  A
back-facing disc between the two closes the window.  With window_factor 0 the
window holds only the first hit, so the trace equals the plain trace without
neighbour deposits."""
import numpy as np
import pytest

N = 20000
LO, HI = np.float32([-0.5, -0.5, -1.0]), np.float32([0.5, 0.5, 0.5])


def _stack(oracle_lib, middle=False):
    xyzr = [[0, 0, 0, 10], [0, 0, -0.1, 10]]
    nrm = [[0, 0, 1], [0, 0, 1]]
    if middle:
        xyzr.append([0, 0, -0.05, 10])
        nrm.append([0, 0, -1])
    return oracle_lib.Scene(np.float32(xyzr), np.float32(nrm))


def _expected_lower(oracle_lib, cfg, factor):
    """Source rays whose lower-disc hit lies in the window of their upper-disc hit."""
    n = 0
    for i in range(N):
        o, d = (v.astype(np.float64) for v in oracle_lib.source_ray(cfg, i))
        if d[2] == 0.0:  # a horizontal source ray (u = 0) wraps until it is cut
            continue
        t0, t1 = (0.0 - o[2]) / d[2], (-0.1 - o[2]) / d[2]
        p0, p1 = o + d * t0, o + d * t1
        same_cell = all(np.floor(p0[a] + 0.5) == np.floor(p1[a] + 0.5) for a in (0, 1))
        n += bool(same_cell and t1 - t0 <= factor * 10.0)
    return n


@pytest.mark.parametrize("factor", [5.0, 0.02])
def test_window_collects_the_lower_disc(oracle_lib, factor):
    s = _stack(oracle_lib)
    cfg = oracle_lib.make_config(LO, HI, sticking=1.0, window=1, window_factor=factor)
    c = s.trace(cfg, 0, N)
    want = _expected_lower(oracle_lib, cfg, factor)
    # a ray wrapped within tnear of the upper disc meets the lower one first (rare)
    assert c.hitc == N - c.truncated and c.counts[0] >= c.hitc - 2 and c.truncated <= 2
    assert abs(int(c.counts[1]) - want) <= 3 and 0 < want < N
    assert c.total == c.counts.sum() and c.nb_deposits == c.total - c.hitc
    np.testing.assert_allclose(c.s1, c.counts.astype(np.float64))  # each deposit is w s = 1
    plain = s.trace(oracle_lib.make_config(LO, HI, sticking=1.0), 0, N)
    assert plain.counts[1] <= 2 and plain.hitc == N - plain.truncated


def test_back_face_closes_the_window(oracle_lib):
    s = _stack(oracle_lib, middle=True)
    c = s.trace(oracle_lib.make_config(LO, HI, sticking=1.0, window=1, window_factor=5.0), 0, N)
    assert c.counts[0] >= N - c.truncated - 2 and c.counts[1] <= 2 and c.counts[2] == 0


def test_weight_drops_by_the_mean_deposit(oracle_lib):
    """Sticking 0.5 on both discs: two deposits of 0.5, w drops to 0.5; the
    diffuse re-emission from the upper disc leaves through the source plane."""
    s = _stack(oracle_lib)
    cfg = oracle_lib.make_config(LO, HI, sticking=0.5, window=1, window_factor=5.0)
    c = s.trace(cfg, 0, 4000)
    assert c.counts[0] >= 4000 - c.truncated - 2 and c.counts[1] > 0
    np.testing.assert_allclose(c.s1, 0.5 * c.counts.astype(np.float64))
    assert c.nonhitc == 4000 - c.truncated


def test_factor_zero_equals_the_plain_trace(oracle_lib):
    rng = np.random.default_rng(3)
    g = np.arange(10) * 0.1 - 0.45
    X, Y = np.meshgrid(g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), -0.3 * rng.random(X.size)], 1)
    nrm = np.concatenate([rng.normal(size=(X.size, 2)) * 0.4, np.ones((X.size, 1))], 1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    xyzr = np.concatenate([p, np.full((X.size, 1), 0.03)], 1)
    xyzr = np.vstack([xyzr, [[0, 0, -0.5, 10]]]).astype(np.float32)
    nrm = np.vstack([nrm, [[0, 0, 1]]]).astype(np.float32)
    s = oracle_lib.Scene(xyzr, nrm)
    kw = dict(sticking=0.3, reflection=2, specular_fraction=0.2, seed=4)
    a = s.trace(oracle_lib.make_config(LO, HI, **kw), 0, 5000)
    b = s.trace(oracle_lib.make_config(LO, HI, window=1, window_factor=0.0, **kw), 0, 5000)
    assert a.hitc > 5000 and a.counts[:-1].sum() > 0
    assert np.array_equal(a.counts, b.counts)
    np.testing.assert_array_equal(a.s1, b.s1)
    assert (a.hitc, a.nonhitc, a.total, a.segments) == (b.hitc, b.nonhitc, b.total, b.segments)
