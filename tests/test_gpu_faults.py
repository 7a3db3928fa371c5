"""Failure paths of the C ABI, made on the host (no GPU fault is involved).

* Allocation failures: the context's device allocator is told to fail at its
  k-th allocation (rtg_inject_alloc_failure), for every k that a sequence of
  calls reaches: upload, tree rebuild, sticking field, traces in the
  megakernel and wavefront schedules, estimates, explicit rays, the adjoint
  and a refit.  The call that meets the failure returns RTG_ERR_OUT_OF_MEMORY;
  right after it a trace either works or reports RTG_ERR_NO_GEOMETRY (a
  failed upload or rebuild drops the surface); and the same context then runs
  the whole sequence exactly as a context that never failed.
* Batches follow their contexts: a refit whose neighbour lists grow, a new
  tree, a sticking field and a new upload of as many discs are seen by the
  next run (the same results as a new batch); an upload of another size makes
  the run fail instead of tracing stale buffers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 20000


@pytest.fixture(scope="module")
def surf():
    from rti_gb300 import scenes
    return scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)


def _sequence(e, t):
    """The calls under test; returns what each step produced."""
    from rti_gb300 import _lib as L
    out = {}
    e.set_launch_config()
    e.set_tree_builder(L.RTG_TREE_KARRAS)
    e.upload_discs(t.points, t.normals, t.radii)
    e.configure(box=(t.box_lo, t.box_hi), x_bound=1, y_bound=1, sticking=0.1, reset=True)
    e.set_tree_builder(L.RTG_TREE_PLOC)
    field = np.full(t.n, 0.1, np.float32)
    field[::7] = 0.4
    e.set_sticking_field(field)
    e.trace(N, 4)
    out["counts"], out["s1"], out["est"] = e.hit_counts(), e.values(), e.mc_estimates()
    e.set_launch_config(scheduling=L.RTG_SCHED_WAVEFRONT)
    e.trace(N, 5)
    out["wf_counts"] = e.hit_counts()
    e.set_launch_config()
    rng = np.random.default_rng(2)
    rays = np.concatenate([rng.uniform(0, 1.2, (500, 3)), np.tile([0, 0, -1.0], (500, 1))], 1).astype(np.float32)
    rays[:, 2] = 0.5
    out["rays"] = e.trace_rays(rays)
    out["adjoint"] = e.adjoint(np.ones(t.n), N, seed=4)
    moved = t.points.copy()
    moved[:, 2] += (0.01 * np.sin(moved[:, 0] * 9)).astype(np.float32)
    e.update_discs(moved, t.normals, t.radii)
    e.trace(N, 6)
    out["moved_counts"] = e.hit_counts()
    return out


def _same(a, b):
    for k in ("counts", "wf_counts", "moved_counts"):
        assert np.array_equal(a[k], b[k]), k
    np.testing.assert_allclose(a["s1"], b["s1"], rtol=1e-9, atol=0)
    np.testing.assert_allclose(a["est"], b["est"], rtol=1e-5, atol=0)
    assert np.array_equal(a["rays"][0], b["rays"][0]) and np.array_equal(a["rays"][1], b["rays"][1])
    np.testing.assert_allclose(a["adjoint"][0], b["adjoint"][0], rtol=1e-9)
    np.testing.assert_allclose(a["adjoint"][2], b["adjoint"][2], rtol=1e-9, atol=1e-12)


def test_injected_allocation_failures(rtg_lib, surf):
    from rti_gb300 import Engine, RtgError
    from rti_gb300 import _lib as L
    with Engine(0) as e:
        ref = _sequence(e, surf)
    failures = 0
    for k in range(400):
        with Engine(0) as e:
            e.inject_alloc_failure(k)
            try:
                out = _sequence(e, surf)
            except RtgError as err:
                assert err.code == L.RTG_ERR_OUT_OF_MEMORY, str(err)
                assert "injected" in str(err)
            else:
                _same(out, ref)
                break  # k is past the sequence's last allocation
            failures += 1
            e.inject_alloc_failure(-1)
            try:
                e.trace(1000, 1)
                e.hit_counts()
            except RtgError as err:
                assert err.code == L.RTG_ERR_NO_GEOMETRY, str(err)
            _same(_sequence(e, surf), ref)
    assert 40 < failures < 400


def test_batch_follows_its_surfaces(rtg_lib, surf):
    from rti_gb300 import Engine, RtgError
    from rti_gb300 import _lib as L
    from rti_gb300.batch import Batch

    def fresh(e):
        with Batch(0) as b2:
            j2 = b2.add(e, N, seed=5)
            b2.run(use_graph=False)
            b2.synchronize()
            return b2.results(j2)

    t = surf
    with Engine(0) as e, Batch(0) as b:
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(t.box_lo, t.box_hi), x_bound=1, y_bound=1, sticking=0.1, reset=True)
        j = b.add(e, N, seed=5)
        b.run()
        b.synchronize()
        assert np.array_equal(b.results(j)[1], fresh(e)[1])
        nnz0 = len(e.neighbors()[1])
        # refit with larger discs: the neighbour lists grow (new device buffers)
        e.update_discs(t.points, t.normals, t.radii * np.float32(1.6))
        assert len(e.neighbors()[1]) > nnz0
        for use_graph in (True, False):
            b.run(use_graph=use_graph)
            b.synchronize()
            got = b.results(j)
            want = fresh(e)
            assert np.array_equal(got[1], want[1])
            np.testing.assert_allclose(got[2], want[2], rtol=1e-6)
        e.set_tree_builder(L.RTG_TREE_PLOC)
        field = np.full(t.n, 0.05, np.float32)
        e.set_sticking_field(field)
        b.run()
        b.synchronize()
        assert np.array_equal(b.results(j)[1], fresh(e)[1])
        # a new upload of as many discs (shifted surface)
        shifted = t.points + np.float32([0, 0, 0.01])
        e.upload_discs(shifted, t.normals, t.radii)
        b.run()
        b.synchronize()
        assert np.array_equal(b.results(j)[1], fresh(e)[1])
        # another size: the run is refused, the results stay readable
        e.upload_discs(t.points[:-10], t.normals[:-10], t.radii[:-10])
        with pytest.raises(RtgError) as ei:
            b.run()
        assert ei.value.code == L.RTG_ERR_INVALID_ARGUMENT
        with pytest.raises(RtgError):
            b.run_sequential()
        assert len(b.results(j)[1]) == t.n
