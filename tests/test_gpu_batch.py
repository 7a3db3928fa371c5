"""Batched tracing (rtg_batch_*): many surfaces x species in one launch.

Every job's paths come from its own Philox stream (seed, job index), so the
batched launch, its CUDA-graph replay, one plain launch per job, a single
rtg_trace with the same job tag and the oracle all give the same hit counts
bit for bit; FP64 sums may differ only in the order of additions.
"""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
S1_RTOL = 1e-9
RAYS = 30000


@pytest.fixture(scope="module")
def setup(rtg_lib):
    from rti_gb300 import Engine, _lib as L
    from rti_gb300.batch import Batch
    inst = scenes.batch_instances(n=5, seed=3, min_discs=3000, max_discs=12000, aspect=(2.0, 6.0))
    engines = []
    for s in inst:
        e = Engine(0)
        e.upload_discs(s.points, s.normals, s.radii)
        e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, reset=True)
        engines.append(e)
    b = Batch(0)
    jobs = []
    for i, e in enumerate(engines):
        for sp, (stick, expo) in enumerate(scenes.BATCH_SPECIES):
            c = e.config()
            c.sticking, c.source_exponent = stick, expo
            j = b.add(e, RAYS + 1000 * i, seed=7, config=c)
            jobs.append((j, i, stick, expo))
    yield inst, engines, b, jobs
    b.close()
    for e in engines:
        e.close()


def _all(b, jobs):
    return [b.results(j) for j, *_ in jobs]


def _same(ra, rb):
    for (s1a, ca, aa), (s1b, cb, ab) in zip(ra, rb):
        assert np.array_equal(ca, cb)
        np.testing.assert_allclose(s1a, s1b, rtol=S1_RTOL, atol=0)
        assert np.array_equal(aa, ab)


def test_batched_equals_sequential_and_graph(setup):
    inst, engines, b, jobs = setup
    assert len(b) == len(jobs) == 15
    b.run(use_graph=False)
    b.synchronize()
    r_batched = _all(b, jobs)
    t_b = b.tally()
    assert t_b.errors == 0 and t_b.num_rays == sum(RAYS + 1000 * i for _, i, _, _ in jobs)
    b.run_sequential()
    b.synchronize()
    r_seq = _all(b, jobs)
    t_s = b.tally()
    _same(r_batched, r_seq)
    for k in ("hitc", "nonhitc", "total", "segments", "nb_deposits", "truncated"):
        assert getattr(t_b, k) == getattr(t_s, k), k
    for _ in range(2):  # first call captures the graph, the second replays it
        b.run(use_graph=True)
        b.synchronize()
        _same(r_batched, _all(b, jobs))
    # every job has hits, and the species differ
    for s1, cnt, areas in r_batched:
        assert cnt.sum() > 0 and areas.min() >= 0.0


def test_batched_equals_single_trace(setup):
    inst, engines, b, jobs = setup
    b.run(use_graph=True)
    b.synchronize()
    for j, i, stick, expo in jobs:
        e = engines[i]
        e.configure(sticking=stick, source_exponent=expo, job=j)
        e.trace(RAYS + 1000 * i, seed=7)
        s1, cnt, areas = b.results(j)
        assert np.array_equal(cnt, e.hit_counts())
        np.testing.assert_allclose(s1, e.values(), rtol=S1_RTOL, atol=0)
        assert np.array_equal(areas, e.exposed_areas())
        e.configure(job=0)


def test_batched_job_matches_oracle(setup, oracle_lib):
    inst, engines, b, jobs = setup
    b.run(use_graph=True)
    b.synchronize()
    for j, i, stick, expo in (jobs[1], jobs[-1]):
        s = inst[i]
        sc = oracle_lib.Scene(s.xyzr, s.normals)
        sc.neighbors()
        cfg = oracle_lib.make_config(s.box_lo, s.box_hi, sticking=stick, source_exponent=expo, seed=7, job=j)
        c = sc.trace(cfg, 0, RAYS + 1000 * i)
        s1, cnt, _ = b.results(j)
        assert np.array_equal(cnt, c.counts)
        np.testing.assert_allclose(s1, c.s1, rtol=S1_RTOL, atol=0)


def test_batch_rejects_bad_jobs(setup, rtg_lib):
    from rti_gb300 import Engine, RtgError
    from rti_gb300.batch import Batch
    with Batch(0) as b, Engine(0) as empty:
        with pytest.raises(RtgError):
            b.add(empty, 100)  # no geometry
        _, engines, _, _ = setup
        c = engines[0].config()
        c.sticking = 2.0
        with pytest.raises(RtgError):
            b.add(engines[0], 100, config=c)
        assert len(b) == 0
        b.run(use_graph=True)  # an empty batch is a no-op
        b.synchronize()
