"""Launch configurations and the autotuner change the speed, never a result.

Every path is computed from its Philox counters whichever lane, block size,
refill packet, stack variant or scheduling (megakernel or wavefront) runs it,
so hit counts and tallies are identical bit for bit; FP64 sums differ only in
the order of the atomics (1e-9 relative).
"""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
S1_RTOL = 1e-9
MK, WF, PL = 0, 1, 2
LOCAL, SHARED = 1, 2  # stack memory
CONFIGS = [(64, 1, 0, MK), (256, 8, 0, MK), (128, 32, 256, MK), (128, 1, 32, MK), (128, 1, 0, WF),
           (256, 1, 256, WF), (64, 1, 64, WF), (128, 1, 0, PL), (256, 1, 64, PL),
           (128, 1, 0, MK, 1), (256, 8, 256, MK, 1), (128, 1, 0, PL, 1),
           (128, 1, 0, MK, 0, SHARED), (64, 8, 64, MK, 1, SHARED), (256, 1, 0, PL, 0, SHARED),
           (128, 1, 64, MK, 0, SHARED), (128, 1, 0, MK, 0, LOCAL), (256, 1, 256, MK, 0, SHARED), (64, 1, 64, MK, 0, SHARED)]


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


def _run(eng, n, seed):
    eng.trace(n, seed)
    return eng.hit_counts(), eng.values(), eng.tally()


def _same(a, b):
    assert np.array_equal(a[0], b[0])
    np.testing.assert_allclose(a[1], b[1], rtol=S1_RTOL, atol=0)
    for k in ("hitc", "nonhitc", "total", "segments", "truncated", "nb_deposits"):
        assert getattr(a[2], k) == getattr(b[2], k), k
    assert a[2].errors == 0 and b[2].errors == 0


def _trench(eng):
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), x_bound=1, y_bound=1, sticking=0.1, reset=True)


def _hole(eng):
    h = scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    eng.upload_triangles(h.vertices, h.indices)
    eng.configure(box=(h.box_lo, h.box_hi), x_bound=1, y_bound=1, sticking=0.01, reflection=2,
                  specular_fraction=0.1, reset=True)


@pytest.mark.parametrize("scene", ["trench", "hole"])
def test_every_launch_config_gives_the_same_trace(eng, scene):
    (_trench if scene == "trench" else _hole)(eng)
    assert 1 <= eng.tree_depth <= 256
    eng.set_launch_config()
    ref = _run(eng, 60000, 4)
    for cfg in CONFIGS:
        eng.set_launch_config(*cfg)
        _same(ref, _run(eng, 60000, 4))
    eng.set_launch_config()
    # the clustered tree (PLOC) instead of the radix tree: same hits
    eng.set_tree_builder(1)
    assert eng.tree_builder == 1 and 1 <= eng.tree_depth <= 256
    _same(ref, _run(eng, 60000, 4))
    eng.set_launch_config(256, 8, 0, MK)
    _same(ref, _run(eng, 60000, 4))
    eng.set_tree_builder(0)
    eng.set_launch_config()


def test_wavefront_truncation_field_and_reflective_box(eng):
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.upload_discs(t.points, t.normals, t.radii)
    rng = np.random.default_rng(2)
    eng.configure(box=(t.box_lo, t.box_hi), x_bound=0, y_bound=0, max_segments=3, source_exponent=5.0,
                  reflection=1, reset=True)
    eng.set_sticking_field(rng.uniform(0.05, 0.9, t.n).astype(np.float32))
    eng.set_launch_config()
    ref = _run(eng, 40000, 8)
    assert ref[2].truncated > 0
    for cfg in ((128, 1, 0, WF), (128, 1, 0, PL), (128, 1, 0, MK, 1)):
        eng.set_launch_config(*cfg)
        _same(ref, _run(eng, 40000, 8))
    # a sample larger than the queue capacity is generated over several waves
    eng.set_sticking_field(None)
    eng.configure(max_segments=1 << 16, reflection=0, source_exponent=1.0)
    eng.set_launch_config()
    ref = _run(eng, 1_500_000, 9)
    eng.set_launch_config(256, 1, 0, WF)
    _same(ref, _run(eng, 1_500_000, 9))
    eng.set_launch_config()


def test_invalid_launch_configs_are_refused(eng):
    from rti_gb300 import RtgError
    _trench(eng)
    for kw, msg in ((dict(threads_per_block=96), "threads_per_block"), (dict(packet=0), "packet"),
                    (dict(stack_depth=48), "stack_depth"), (dict(scheduling=7), "scheduling"),
                    (dict(leaf_tests=3), "leaf_tests"), (dict(stack_memory=5), "stack_memory")):
        with pytest.raises(RtgError, match=msg):
            eng.set_launch_config(**kw)
    eng.set_launch_config()


def test_autotune_picks_a_valid_config_and_results_stay(eng):
    _hole(eng)
    eng.set_launch_config()
    ref = _run(eng, 80000, 1)
    cfg, rate = eng.autotune(80000, seed=1)
    assert rate > 0
    assert cfg["threads_per_block"] in (64, 128, 256) and 1 <= cfg["packet"] <= 32
    assert cfg["scheduling"] != WF  # the wavefront is no autotune candidate
    assert eng.launch_config().as_dict() == cfg and eng.tree_builder in (0, 1)
    _same(ref, _run(eng, 80000, 1))
    eng.set_launch_config()
    eng.set_tree_builder(0)


def test_batch_wavefront_and_autotune(rtg_lib):
    from rti_gb300 import Engine
    from rti_gb300.batch import Batch
    inst = scenes.batch_instances(n=3, seed=5, min_discs=3000, max_discs=9000, aspect=(2.0, 5.0))
    engines = []
    with Batch(0) as b:
        for s in inst:
            e = Engine(0)
            e.upload_discs(s.points, s.normals, s.radii)
            e.configure(box=(s.box_lo, s.box_hi), x_bound=1, y_bound=1, reset=True)
            engines.append(e)
            for stick, expo in scenes.BATCH_SPECIES:
                c = e.config()
                c.sticking, c.source_exponent = stick, expo
                b.add(e, 20000, seed=3, config=c)
        b.run(use_graph=True)
        b.synchronize()
        ref = [b.results(j) for j in range(len(b))]
        t_ref = b.tally()
        for cfg in [(128, 1, 0, WF), (64, 8, 256, MK), (256, 32, 0, MK), (128, 1, 0, PL), (128, 8, 0, MK, 1),
                    (128, 1, 0, MK, 0, SHARED), (64, 8, 64, PL, 1, SHARED)]:
            b.set_launch_config(*cfg)
            b.run(use_graph=True)
            b.synchronize()
            t = b.tally()
            assert t.segments == t_ref.segments and t.errors == 0
            for j in range(len(b)):
                r = b.results(j)
                assert np.array_equal(r[1], ref[j][1])
                np.testing.assert_allclose(r[0], ref[j][0], rtol=S1_RTOL, atol=0)
        cfg, rate = b.autotune(0.25)
        assert rate > 0 and b.launch_config() == cfg and cfg["scheduling"] != WF
        b.run(use_graph=True)
        b.synchronize()
        for j in range(len(b)):
            assert np.array_equal(b.results(j)[1], ref[j][1])
    for e in engines:
        e.close()


def test_adjoint_with_the_stack_in_shared_memory(eng):
    """Asking for shared-memory stacks leaves the adjoint replays' gradients as
    they were (their 64-entry stacks exceed the 16 KB per block that a shared
    stack may take, so they stay in local memory)."""
    rng = np.random.default_rng(4)
    _trench(eng)
    g = rng.random(eng.num_primitives)
    field_in = rng.uniform(0.05, 0.5, eng.num_primitives).astype(np.float32)
    out = []
    for mem in (LOCAL, SHARED):
        eng.set_launch_config(stack_memory=mem)
        ds, dn, _ = eng.adjoint(g, 50000, seed=2)
        eng.set_sticking_field(field_in)
        _, dn2, field = eng.adjoint(g, 50000, seed=2)
        eng.set_sticking_field(None)
        out.append((ds, dn, dn2, field))
    eng.set_launch_config()
    for a, b in zip(out[0], out[1]):
        np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12)
