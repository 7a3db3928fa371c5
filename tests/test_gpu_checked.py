"""The checked build (-DRTG_CHECKED: every node, slot, primitive and
neighbour index read from device data is verified before use and a bad one is
counted in tally.errors) traces the parity scenes without a single violation
and with the same hit counts as the production library.  compute-sanitizer is
not available to these tests; this is the bounds check that stands in for it."""
import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu


def _run_all(L, width=2):
    """Traces through the loaded library: discs with neighbours (megakernel,
    wavefront, window deposit), triangles, an adjoint, a batch; closest hits
    over the binary (width 2) or the compressed 8-wide tree (width 8)."""
    from rti_gb300 import Engine
    from rti_gb300.batch import Batch
    out = {}
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    h = scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    with Engine(0) as e:
        e.set_node_width(width)
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
        for name, kw in (("mk", {}), ("wf", {"scheduling": L.RTG_SCHED_WAVEFRONT}),
                         ("pp", {"leaf_tests": L.RTG_LEAF_POSTPONED})):
            e.set_launch_config(**kw)
            e.trace(100000, 5)
            out[name] = (e.hit_counts(), e.tally().errors)
        e.set_launch_config()
        e.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
        e.trace(50000, 6)
        out["window"] = (e.hit_counts(), e.tally().errors)
        e.set_deposit_mode(L.RTG_DEPOSIT_NEIGHBORS, 5.0)
        ds, dn, _ = e.adjoint(np.ones(t.n), 20000, seed=2)
        out["adjoint"] = (np.array([ds, dn]), 0)
    with Engine(0) as e:
        e.set_node_width(width)
        e.upload_triangles(h.vertices, h.indices)
        e.configure(box=(h.box_lo, h.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1, x_bound=1,
                    y_bound=1, reset=True)
        e.trace(100000, 7)
        out["tri"] = (e.hit_counts(), e.tally().errors)
        with Batch(0) as b:
            b.add(e, 20000, seed=1)
            b.run(use_graph=False)
            b.synchronize()
            out["batch"] = (b.results(0)[1], b.tally().errors)
    return out


@pytest.mark.parametrize("width", [2, 8], ids=["binary", "wide"])
def test_checked_build_has_no_violations_and_the_same_hits(rtg_lib, width):
    from rti_gb300 import build, _lib
    ref = _run_all(_lib)
    path = build.build(checked=True)
    keep = _lib._lib
    _lib._lib = None
    try:
        _lib.load(path)
        got = _run_all(_lib, width)
    finally:
        _lib._lib = keep
    for k, (v, err) in got.items():
        assert err == 0, k
        if k == "adjoint":
            np.testing.assert_allclose(v, ref[k][0], rtol=1e-9)
        else:
            assert np.array_equal(v, ref[k][0]), k
