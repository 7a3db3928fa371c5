"""The segment log (rtg_set_segment_log): rti's RAYLOG / RAYSRCLOG
(util/ray_logger.hpp:23-71, trace/tracer.hpp:166,183) on the GPU.

Every closest-hit query of a logged source ray is one record; the oracle
restates the same path with the same arithmetic, so the records -- origin,
end point, kind, primitive, weight -- must equal its per-path log bit for bit,
over the binary and the wide tree, for discs with neighbours and for
triangles.  Logging changes no result; records beyond the capacity are counted.
"""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
FIELDS = ("ray", "segment", "kind", "primitive")


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.set_segment_log(0, 0, 0)
    e.close()


def _same(gpu, ref):
    assert len(gpu) == len(ref)
    for f in FIELDS:
        assert np.array_equal(gpu[f], ref[f]), f
    for f in ("org", "end", "weight"):
        assert np.array_equal(gpu[f].view(np.uint32), ref[f].view(np.uint32)), f


def _oracle_logs(oracle_lib, scene, cfg, ids):
    return np.concatenate([oracle_lib.trace_log(scene, cfg, int(i)) for i in ids])


@pytest.mark.parametrize("width", [2, 8], ids=["binary", "wide"])
def test_log_equals_oracle_discs(eng, oracle_lib, width):
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    eng.set_node_width(width)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    eng.set_segment_log(0, 300, 100000)
    try:
        eng.trace(300, seed=3)
        log, dropped = eng.segment_log()
        tal = eng.tally()
    finally:
        eng.set_node_width(0)
    s = oracle_lib.Scene(t.xyzr, t.normals)
    s.neighbors()
    ref = _oracle_logs(oracle_lib, s, oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.1, seed=3), range(300))
    assert dropped == 0 and len(log) == tal.segments
    assert (log["kind"] == 0).sum() == tal.hitc and (log["kind"] == 3).sum() == tal.nonhitc
    _same(log, ref)
    # the source points are the segment-0 origins, on the source plane
    src = log[log["segment"] == 0]
    assert len(src) == 300 and np.all(src["org"][:, 2] == np.float32(t.box_hi[2]))


def test_log_range_capacity_and_no_effect_on_results(eng, oracle_lib):
    from rti_gb300 import RtgError
    from rti_gb300 import _lib as L
    h = scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)
    eng.upload_triangles(h.vertices, h.indices)
    eng.configure(box=(h.box_lo, h.box_hi), sticking=0.05, reflection=2, specular_fraction=0.1, x_bound=1,
                  y_bound=1, reset=True)
    eng.set_segment_log(0, 0, 0)
    eng.trace(2000, seed=8)
    counts = eng.hit_counts()
    eng.set_segment_log(100, 160, 1 << 20)
    eng.trace(2000, seed=8)
    assert np.array_equal(eng.hit_counts(), counts)  # logging changes no result
    log, dropped = eng.segment_log()
    assert dropped == 0 and set(np.unique(log["ray"])) == set(range(100, 160))
    s = oracle_lib.Scene(tri_vertices=h.vertices, tri_indices=h.indices)
    cfg = oracle_lib.make_config(h.box_lo, h.box_hi, sticking=0.05, reflection=2, specular_fraction=0.1, seed=8)
    _same(log, _oracle_logs(oracle_lib, s, cfg, range(100, 160)))
    # a triangle's hits in the log are its hit count over the logged rays
    hits = log[log["kind"] == L.RTG_SEG_HIT]["primitive"]
    eng.set_segment_log(0, 0, 0)
    eng.trace(60, seed=8, ray_begin=100)
    assert np.array_equal(np.bincount(hits, minlength=h.n), eng.hit_counts())
    # capacity: kept up to it, the rest counted
    eng.set_segment_log(0, 2000, 50)
    eng.trace(2000, seed=8)
    kept, dropped = eng.segment_log()
    assert len(kept) == 50 and dropped == eng.tally().segments - 50
    # accumulated traces extend the log
    eng.set_segment_log(0, 2000, 1 << 20)
    eng.trace(1000, seed=8)
    eng.trace(1000, seed=8, ray_begin=1000, accumulate=True)
    log2, _ = eng.segment_log()
    assert set(np.unique(log2["ray"])) == set(range(2000))
    # not with the multi-hit window deposit
    eng.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
    with pytest.raises(RtgError, match="segment log"):
        eng.trace(10, seed=1)
    eng.set_deposit_mode(L.RTG_DEPOSIT_NEIGHBORS, 5.0)
    eng.set_segment_log(0, 0, 0)


def test_log_as_vtp(eng, tmp_path):
    t = scenes.trench_discs(domain=0.8, width=0.3, depth=0.8)
    eng.upload_discs(t.points, t.normals, t.radii)
    eng.configure(box=(t.box_lo, t.box_hi), sticking=0.2, x_bound=1, y_bound=1, reset=True)
    eng.set_segment_log(0, 50, 10000)
    eng.trace(50, seed=2)
    log, _ = eng.segment_log()
    f = tmp_path / "raylog.vtp"
    eng.write_segment_log(str(f))
    piece = ET.parse(f).getroot().find("PolyData/Piece")
    assert int(piece.get("NumberOfLines")) == len(log) > 50
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(pts[0::2], log["org"])
    np.testing.assert_array_equal(pts[1::2], log["end"])
    eng.set_segment_log(0, 0, 0)
