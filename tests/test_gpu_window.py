"""The multi-hit window deposit (RTG_DEPOSIT_WINDOW; rti trace/
point_cloud_context.hpp:132-173,265-286) on the GPU against the oracle.

Same bar as the neighbour deposit: hit counts and tallies bit for bit, FP64
accumulators within 1e-9 relative (atomic addition order).  Scenes: the trench
(coplanar overlapping discs, periodic and reflective), a rough surface with a
sticking field, two stacked discs with a back-facing one between them, a
surface of discs and triangles, and the plain schedule; the adjoint and the
batch refuse a context in this mode."""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
S1_RTOL = 1e-9


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine, _lib as L
    e = Engine(0)
    e.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
    yield e
    e.close()


def _compare(eng, c):
    t = eng.tally()
    assert np.array_equal(eng.hit_counts(), c.counts), "hit counts differ"
    assert (t.hitc, t.nonhitc, t.total, t.segments, t.truncated, t.nb_deposits, t.errors) == \
        (c.hitc, c.nonhitc, c.total, c.segments, c.truncated, c.nb_deposits, 0)
    for a, b in zip(eng.accumulators(), (c.s1, c.s2, c.s3, c.s4)):
        np.testing.assert_allclose(a, b, rtol=S1_RTOL, atol=0)


@pytest.mark.parametrize("bound", [1, 0], ids=["periodic", "reflective"])
def test_window_trench_matches_oracle(eng, oracle_lib, bound):
    from rti_gb300 import _lib as L
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=bound, y_bound=bound, reset=True)
    assert eng.deposit_mode == (L.RTG_DEPOSIT_WINDOW, 5.0)
    n = 100000
    eng.trace(n, 7)
    s = oracle_lib.Scene(t.xyzr, t.normals)
    c = s.trace(oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.1, x_bound=bound, y_bound=bound, seed=7,
                                       window=1, window_factor=5.0), 0, n)
    assert c.nb_deposits > c.hitc // 4  # overlapping coplanar discs: several per window
    _compare(eng, c)


def test_window_rough_sticking_field_matches_oracle(eng, oracle_lib):
    r = scenes.rough_discs(n=96, spacing=0.01, rms=0.02, corr=0.1, seed=3)
    field = np.random.default_rng(1).uniform(0.05, 0.6, r.n).astype(np.float32)
    eng.upload_discs(r.points, r.normals, r.radii)
    eng.configure(box=(r.box_lo, r.box_hi), reflection=2, specular_fraction=0.3, x_bound=1, y_bound=1, reset=True)
    eng.set_sticking_field(field)
    eng.set_deposit_mode(1, 2.5)
    n = 100000
    eng.trace(n, 2)
    eng.set_sticking_field(None)
    s = oracle_lib.Scene(r.xyzr, r.normals)
    c = s.trace(oracle_lib.make_config(r.box_lo, r.box_hi, reflection=2, specular_fraction=0.3, seed=2, window=1,
                                       window_factor=2.5), 0, n, sticking_field=field)
    assert c.hitc > n
    _compare(eng, c)
    eng.set_deposit_mode(1, 5.0)


def test_window_stacked_discs_and_back_face(eng, oracle_lib):
    lo, hi = np.float32([-0.5, -0.5, -1.0]), np.float32([0.5, 0.5, 0.5])
    for middle in (False, True):
        xyzr = [[0, 0, 0, 10], [0, 0, -0.1, 10]] + ([[0, 0, -0.05, 10]] if middle else [])
        nrm = [[0, 0, 1], [0, 0, 1]] + ([[0, 0, -1]] if middle else [])
        xyzr, nrm = np.float32(xyzr), np.float32(nrm)
        eng.upload_discs(xyzr[:, :3], nrm, xyzr[:, 3])
        eng.configure(box=(lo, hi), sticking=1.0, x_bound=1, y_bound=1, reset=True)
        eng.trace(50000, 0)
        c = oracle_lib.Scene(xyzr, nrm).trace(oracle_lib.make_config(lo, hi, sticking=1.0, window=1,
                                                                     window_factor=5.0), 0, 50000)
        assert (c.counts[1] <= 2) if middle else (c.counts[1] > 10000)
        _compare(eng, c)


def test_window_discs_and_triangles(eng, oracle_lib):
    """Triangles deposit alone and close a window they cut."""
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    v = np.float32([[-0.6, -0.6, -0.55], [0.6, -0.6, -0.55], [0.6, 0.6, -0.55], [-0.6, 0.6, -0.55]])
    idx = np.uint32([[0, 1, 2], [0, 2, 3]])
    eng.upload_mixed(t.points, t.normals, t.radii, v, idx)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.2, x_bound=1, y_bound=1, reset=True)
    n = 50000
    eng.trace(n, 5)
    s = oracle_lib.Scene(t.xyzr, t.normals, tri_vertices=v, tri_indices=idx)
    c = s.trace(oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.2, seed=5, window=1, window_factor=5.0), 0, n)
    _compare(eng, c)


def test_window_plain_schedule_and_refusals(eng, oracle_lib):
    from rti_gb300 import RtgError
    from rti_gb300.batch import Batch
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    for sched in (2, 1):  # plain; a wavefront request runs the window megakernel
        eng.set_launch_config(scheduling=sched)
        eng.trace(40000, 9)
        s = oracle_lib.Scene(t.xyzr, t.normals)
        _compare(eng, s.trace(oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.1, seed=9, window=1,
                                                     window_factor=5.0), 0, 40000))
    eng.set_launch_config()
    with pytest.raises(RtgError, match="neighbour deposit"):
        eng.adjoint(np.ones(t.n), 1000, 0)
    b = Batch(0)
    with pytest.raises(RtgError, match="neighbour deposit"):
        b.add(eng, 1000)
    b.close()
    with pytest.raises(RtgError, match="window_factor"):
        eng.set_deposit_mode(1, -1.0)
    with pytest.raises(RtgError, match="mode must be"):
        eng.set_deposit_mode(7, 5.0)
