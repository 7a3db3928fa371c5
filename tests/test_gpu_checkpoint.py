"""Checkpoint and resume (rtg_set_accumulators): a trace stopped after ray k,
saved, and continued over [k, n) in a new context equals the trace of [0, n)
in one go.  Paths depend only on (seed, ray id) (Philox counters), so the hit
counts and tallies are equal, S1 bit for bit under RTG_ACCUM_FIXED, and the
other sums up to the order of their FP64 additions."""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu

N, K, SEED = 400_000, 123_457, 5


def _scene(kind):
    if kind == "hole":
        return scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    return scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)


def _engine(kind, s, fixed):
    from rti_gb300 import Engine
    from rti_gb300 import _lib as L
    e = Engine(0)
    if kind == "hole":
        e.upload_triangles(s.vertices, s.indices)
        e.configure(box=(s.box_lo, s.box_hi), sticking=0.05, reflection=2, specular_fraction=0.1,
                    x_bound=1, y_bound=1, reset=True)
    else:
        e.upload_discs(s.points, s.normals, s.radii)
        e.configure(box=(s.box_lo, s.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    if fixed:
        e.set_accumulation(L.RTG_ACCUM_FIXED)
    return e


@pytest.mark.parametrize("fixed", [True, False], ids=["fixed_s1", "fp64_s1"])
@pytest.mark.parametrize("kind", ["hole", "trench"])
def test_resume_equals_one_trace(rtg_lib, kind, fixed):
    surface = _scene(kind)
    with _engine(kind, surface, fixed) as a:
        a.trace(N, seed=SEED)
        ref = a.checkpoint()
        est_ref = a.mc_estimates()
    with _engine(kind, surface, fixed) as b:
        b.trace(K, seed=SEED)
        state = b.checkpoint()
    assert state["tally"]["num_rays"] == K
    with _engine(kind, surface, fixed) as c:
        c.resume(state)
        c.trace(N - K, seed=SEED, ray_begin=K, accumulate=True)
        got = c.checkpoint()
        est = c.mc_estimates()
    assert got["tally"] == ref["tally"] and got["tally"]["num_rays"] == N
    assert np.array_equal(got["counts"], ref["counts"])
    if fixed:
        assert np.array_equal(got["s1"].view(np.uint64), ref["s1"].view(np.uint64))
        np.testing.assert_array_equal(est, est_ref)
    else:
        np.testing.assert_allclose(got["s1"], ref["s1"], rtol=1e-12, atol=0)
        np.testing.assert_allclose(est, est_ref, rtol=1e-6, atol=0)
    for k in ("s2", "s3", "s4"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-10, atol=0)


def test_resume_checks_its_input(rtg_lib):
    from rti_gb300 import Engine, RtgError
    from rti_gb300 import _lib as L
    with _engine("trench", _scene("trench"), False) as e:
        e.trace(1000, seed=1)
        state = e.checkpoint()
        with pytest.raises(ValueError):
            e.resume(dict(state, s2=state["s2"][:-1]))
        with pytest.raises(RtgError, match="all needed"):
            e._check(e._L.rtg_set_accumulators(e._h, None, None, None, None, None, None))
    one = np.zeros(1)
    cnt = np.zeros(1, np.uint64)
    t = L.RtgTally()
    with Engine(0) as empty:  # no surface: nothing to resume into
        with pytest.raises(RtgError, match="no geometry"):
            empty._check(empty._L.rtg_set_accumulators(empty._h, *[one.ctypes.data_as(L._f64p)] * 4,
                                                       cnt.ctypes.data_as(L._u64p), t))
