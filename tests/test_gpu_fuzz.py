"""Randomised parity: seeded random surfaces and configurations, GPU against
the oracle on the same inputs.

Each case draws a surface of discs, triangles or both (random positions,
orientations and sizes; overlapping discs with rti's neighbour deposit), a
random configuration (periodic or reflective x and y, diffuse, specular or
mixed re-emission, sticking, source exponent, sometimes a per-primitive
sticking field, binary or wide tree, FP64 or fixed-point S1, and on disc
surfaces sometimes rti's multi-hit window deposit instead of the neighbour
deposit) and traces it on both sides.  Hit counts and tallies must be equal;
S1 equal bit for bit under fixed-point accumulation, else to the order of the
FP64 additions.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = 60
N_RAYS = 5000


def _unit(v):
    return (v / np.linalg.norm(v, axis=1)[:, None]).astype(np.float32)


def _case(k):
    rng = np.random.default_rng(7000 + k)
    kind = ("discs", "triangles", "mixed")[k % 3]
    depth = float(rng.uniform(0.2, 2.0))
    out = {"kind": kind}
    if kind != "triangles":
        nd = int(rng.integers(1, 3000))
        c = np.stack([rng.uniform(0, 1, nd), rng.uniform(0, 1, nd), rng.uniform(-depth, 0, nd)], 1)
        n = _unit(rng.normal(size=(nd, 3)) + [0, 0, rng.uniform(0, 2)])
        r = rng.uniform(0.005, 0.06, nd)
        out.update(points=c.astype(np.float32), normals=n, radii=r.astype(np.float32))
    if kind != "discs":
        nt = int(rng.integers(1, 2000))
        v0 = np.stack([rng.uniform(0, 1, nt), rng.uniform(0, 1, nt), rng.uniform(-depth, 0, nt)], 1)
        e1 = rng.normal(scale=0.05, size=(nt, 3))
        e2 = rng.normal(scale=0.05, size=(nt, 3))
        e2[rng.random(nt) < 0.02] = 0  # a few degenerate triangles
        V = np.concatenate([v0, v0 + e1, v0 + e2]).astype(np.float32)
        T = np.stack([np.arange(nt), np.arange(nt) + nt, np.arange(nt) + 2 * nt], 1).astype(np.uint32)
        out.update(vertices=V, indices=T)
    npr = (len(out["points"]) if "points" in out else 0) + (len(out["indices"]) if "indices" in out else 0)
    out["cfg"] = dict(x_bound=int(rng.integers(0, 2)), y_bound=int(rng.integers(0, 2)),
                      reflection=int(rng.integers(0, 3)), specular_fraction=float(np.float32(rng.uniform(0, 1))),
                      sticking=float(np.float32(rng.uniform(0.01, 1.0))),
                      source_exponent=float(rng.choice([1.0, 2.5, 10.0])))
    out["field"] = (rng.uniform(0.01, 1.0, npr).astype(np.float32) if rng.random() < 0.3 else None)
    out["width"] = int(rng.choice([2, 8]))
    out["fixed"] = bool(rng.random() < 0.5)
    out["box"] = (np.array([0, 0, -depth - 0.1], np.float32), np.array([1, 1, 0.1], np.float32))
    out["seed"] = int(rng.integers(0, 1 << 30))
    out["window"] = kind == "discs" and rng.random() < 0.3
    return out


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.mark.parametrize("k", range(CASES))
def test_random_surface_and_configuration(eng, oracle_lib, k):
    from rti_gb300 import _lib as L
    c = _case(k)
    lo, hi = c["box"]
    eng.set_node_width(c["width"])
    if c["kind"] == "discs":
        eng.upload_discs(c["points"], c["normals"], c["radii"])
    elif c["kind"] == "triangles":
        eng.upload_triangles(c["vertices"], c["indices"])
    else:
        eng.upload_mixed(c["points"], c["normals"], c["radii"], c["vertices"], c["indices"])
    eng.configure(box=(lo, hi), reset=True, **c["cfg"])
    eng.set_sticking_field(c["field"])
    eng.set_accumulation(L.RTG_ACCUM_FIXED if c["fixed"] else L.RTG_ACCUM_FP64)
    if c["window"]:
        eng.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
    try:
        eng.trace(N_RAYS, seed=c["seed"])
        cnt, s1, t = eng.hit_counts(), eng.values(), eng.tally()
    finally:
        eng.set_node_width(0)
        eng.set_sticking_field(None)
        eng.set_accumulation(L.RTG_ACCUM_FP64)
        eng.set_deposit_mode(L.RTG_DEPOSIT_NEIGHBORS, 5.0)
    xyzr = (np.concatenate([c["points"], c["radii"][:, None]], 1) if "points" in c else None)
    s = oracle_lib.Scene(xyzr, c.get("normals"), c.get("vertices"), c.get("indices"))
    if s.nd:
        s.neighbors(bruteforce=True)  # every pair under rti's distance test, as the GPU grid
    cfg = oracle_lib.make_config(lo, hi, seed=c["seed"], accum_fixed=int(c["fixed"]), window=int(c["window"]),
                                 window_factor=5.0, **c["cfg"])
    ref = s.trace(cfg, 0, N_RAYS, sticking_field=c["field"])
    assert t.errors == 0
    assert np.array_equal(cnt, ref.counts)
    assert (t.hitc, t.nonhitc, t.total, t.segments, t.truncated, t.nb_deposits) == \
        (ref.hitc, ref.nonhitc, ref.total, ref.segments, ref.truncated, ref.nb_deposits)
    if c["fixed"]:
        assert np.array_equal(s1.view(np.uint64), ref.s1.view(np.uint64))
    else:
        np.testing.assert_allclose(s1, ref.s1, rtol=1e-9, atol=0)


ADJ_CASES = 24


@pytest.mark.parametrize("k", range(ADJ_CASES))
def test_random_adjoint(eng, oracle_lib, k):
    """The adjoint replay on the same random surfaces (with the neighbour
    deposit): dL/ds, dL/dn and, with a sticking field, dL/ds_j for random
    weights g, held or unbiased estimator, to the order of the FP64 sums."""
    c = _case(k)
    lo, hi = c["box"]
    rng = np.random.default_rng(9000 + k)
    unbiased = bool(rng.random() < 0.5)
    eng.set_node_width(c["width"])
    if c["kind"] == "discs":
        eng.upload_discs(c["points"], c["normals"], c["radii"])
    elif c["kind"] == "triangles":
        eng.upload_triangles(c["vertices"], c["indices"])
    else:
        eng.upload_mixed(c["points"], c["normals"], c["radii"], c["vertices"], c["indices"])
    eng.configure(box=(lo, hi), reset=True, **c["cfg"])
    eng.set_sticking_field(c["field"])
    g = rng.random(eng.num_primitives)
    try:
        ds, dn, fg = eng.adjoint(g, N_RAYS, seed=c["seed"], unbiased=unbiased)
    finally:
        eng.set_node_width(0)
        eng.set_sticking_field(None)
    xyzr = (np.concatenate([c["points"], c["radii"][:, None]], 1) if "points" in c else None)
    s = oracle_lib.Scene(xyzr, c.get("normals"), c.get("vertices"), c.get("indices"))
    if s.nd:
        s.neighbors(bruteforce=True)
    cfg = oracle_lib.make_config(lo, hi, seed=c["seed"], **c["cfg"])
    ods, odn, ofg, _ = oracle_lib.adjoint(s, cfg, g, 0, N_RAYS, sticking_field=c["field"], unbiased=unbiased)
    assert abs(dn - odn) <= 1e-9 * abs(odn) + 1e-12
    if c["field"] is None:
        assert abs(ds - ods) <= 1e-9 * abs(ods) + 1e-12
    else:
        assert ds == 0.0
        np.testing.assert_allclose(fg, ofg, rtol=1e-9, atol=1e-9 * np.abs(ofg).max())


BATCH_JOBS = 12


def test_random_batch(rtg_lib, oracle_lib):
    """One batched launch (CUDA graph) over 12 of the random surfaces, each
    with its own configuration, sticking field and tree width; lanes of a warp
    carry paths of different jobs.  Every job equals the oracle's trace with
    the job's Philox tag."""
    from rti_gb300 import Engine
    from rti_gb300.batch import Batch
    cases = [_case(k) for k in range(BATCH_JOBS)]
    engines = []
    try:
        for c in cases:
            e = Engine(0)
            engines.append(e)
            e.set_node_width(c["width"])
            if c["kind"] == "discs":
                e.upload_discs(c["points"], c["normals"], c["radii"])
            elif c["kind"] == "triangles":
                e.upload_triangles(c["vertices"], c["indices"])
            else:
                e.upload_mixed(c["points"], c["normals"], c["radii"], c["vertices"], c["indices"])
            e.configure(box=c["box"], reset=True, **c["cfg"])
            e.set_sticking_field(c["field"])
        with Batch(0) as b:
            jobs = [b.add(e, N_RAYS + 100 * i, seed=c["seed"]) for i, (e, c) in enumerate(zip(engines, cases))]
            b.run(use_graph=True)
            b.synchronize()
            assert b.tally().errors == 0
            got = [b.results(j) for j in jobs]
    finally:
        for e in engines:
            e.close()
    for i, (c, j, (s1, cnt, _)) in enumerate(zip(cases, jobs, got)):
        lo, hi = c["box"]
        xyzr = (np.concatenate([c["points"], c["radii"][:, None]], 1) if "points" in c else None)
        s = oracle_lib.Scene(xyzr, c.get("normals"), c.get("vertices"), c.get("indices"))
        if s.nd:
            s.neighbors(bruteforce=True)
        cfg = oracle_lib.make_config(lo, hi, seed=c["seed"], job=j, **c["cfg"])
        ref = s.trace(cfg, 0, N_RAYS + 100 * i, sticking_field=c["field"])
        assert np.array_equal(cnt, ref.counts), i
        np.testing.assert_allclose(s1, ref.s1, rtol=1e-9, atol=0)


@pytest.mark.parametrize("k", range(0, CASES, 2))
def test_random_explicit_rays(eng, oracle_lib, k):
    """rtg_trace_rays on the random surfaces over both trees: 20,000 random
    rays (origins in and around the surface, directions uniform on the sphere,
    some axis-parallel) give the same primitive ids and distances, bit for bit,
    as the oracle's closest hit."""
    c = _case(k)
    lo, hi = c["box"]
    rng = np.random.default_rng(11000 + k)
    n = 20000
    o = rng.uniform(lo - 0.2, hi + 0.2, size=(n, 3))
    d = rng.normal(size=(n, 3))
    ax = rng.random(n) < 0.05  # axis-parallel directions
    d[ax] = np.eye(3)[rng.integers(0, 3, ax.sum())] * rng.choice([-1.0, 1.0], size=(ax.sum(), 1))
    d /= np.linalg.norm(d, axis=1)[:, None]
    rays = np.concatenate([o, d], 1).astype(np.float32)
    if c["kind"] == "discs":
        eng.upload_discs(c["points"], c["normals"], c["radii"])
    elif c["kind"] == "triangles":
        eng.upload_triangles(c["vertices"], c["indices"])
    else:
        eng.upload_mixed(c["points"], c["normals"], c["radii"], c["vertices"], c["indices"])
    xyzr = (np.concatenate([c["points"], c["radii"][:, None]], 1) if "points" in c else None)
    s = oracle_lib.Scene(xyzr, c.get("normals"), c.get("vertices"), c.get("indices"))
    pc, tc = s.closest_hit(rays)
    for width in (2, 8):
        eng.set_node_width(width)
        try:
            pg, tg = eng.trace_rays(rays)
        finally:
            eng.set_node_width(0)
        assert np.array_equal(pg, pc), width
        assert np.array_equal(tg.view(np.uint32), tc.view(np.uint32)), width
    assert (pc >= 0).any()


def _log_cases():
    out = []
    for k in range(CASES):
        c = _case(k)
        if c["field"] is None and not c["window"]:
            out.append(k)
    return out[:10]


@pytest.mark.parametrize("k", _log_cases())
def test_random_segment_logs(eng, oracle_lib, k):
    """Every segment of the first 400 paths on random surfaces (origin, end
    point, kind, primitive, weight), GPU segment log against the oracle's
    per-path log, bit for bit."""
    c = _case(k)
    lo, hi = c["box"]
    n = 400
    eng.set_node_width(c["width"])
    if c["kind"] == "discs":
        eng.upload_discs(c["points"], c["normals"], c["radii"])
    elif c["kind"] == "triangles":
        eng.upload_triangles(c["vertices"], c["indices"])
    else:
        eng.upload_mixed(c["points"], c["normals"], c["radii"], c["vertices"], c["indices"])
    eng.configure(box=(lo, hi), reset=True, **c["cfg"])
    eng.set_segment_log(0, n, 1 << 22)
    try:
        eng.trace(n, seed=c["seed"])
        log, dropped = eng.segment_log()
    finally:
        eng.set_segment_log(0, 0, 0)
        eng.set_node_width(0)
    assert dropped == 0
    xyzr = (np.concatenate([c["points"], c["radii"][:, None]], 1) if "points" in c else None)
    s = oracle_lib.Scene(xyzr, c.get("normals"), c.get("vertices"), c.get("indices"))
    if s.nd:
        s.neighbors(bruteforce=True)
    cfg = oracle_lib.make_config(lo, hi, seed=c["seed"], **c["cfg"])
    ref = np.concatenate([oracle_lib.trace_log(s, cfg, i) for i in range(n)])
    assert len(log) == len(ref)
    for f in ("ray", "segment", "kind", "primitive"):
        assert np.array_equal(log[f], ref[f]), f
    for f in ("org", "end", "weight"):
        assert np.array_equal(log[f].view(np.uint32), ref[f].view(np.uint32)), f
