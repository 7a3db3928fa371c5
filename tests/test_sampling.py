"""The distributions of the path's random draws, as Kolmogorov-Smirnov tests.

rti's own sampler tests only plot histograms (test/rti/ray/rectangle_origin_z.cpp:147-195,
cosine_direction_z.cpp, power_cosine_direction_z.cpp).  Here every closest-hit
query is a segment record (origin, end point, kind).  On a flat plane of discs
(normal +z) under the source plane:
* segment 0 starts on the source rectangle: x, y ~ U(box), z = the source plane
  (rectangle_origin_z.hpp:23-37);
* its direction is the source's: with cos(theta) = -d.z, cos(theta)^(n+1) ~ U[0, 1)
  (cosine_direction_z.hpp:13-27 for n = 1, power_cosine_direction_z.hpp:13-32),
  and the azimuth is uniform;
* the segment after a hit leaves in the diffuse re-emission about the normal +z
  (diffuse.hpp:13-27, cos_hemi.hpp:11-45): d.z^2 ~ U[0, 1), azimuth uniform.
The oracle's per-path log checks the restated samplers on the CPU, the GPU's
segment log the kernel's (the two agree record for record in
test_gpu_segment_log.py).  Fixed seeds: the p-values are deterministic.
"""
import numpy as np
import pytest

stats = pytest.importorskip("scipy.stats")

N_RAYS = 20_000
P_MIN = 1e-3


def _plane():
    g = np.arange(40) * 0.05
    X, Y = np.meshgrid(g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1).astype(np.float32)
    nrm = np.tile(np.float32([0, 0, 1]), (len(p), 1))
    r = np.full(len(p), np.float32(0.05 * np.sqrt(2) / 2), np.float32)
    lo, hi = np.array([0, 0, -0.1], np.float32), np.array([1.95, 1.95, 0.1], np.float32)
    return p, nrm, r, lo, hi


def _uniform_samples(log, lo, hi, n):
    """Each array should be U[0, 1)."""
    d = (log["end"] - log["org"]).astype(np.float64)
    d /= np.linalg.norm(d, axis=1)[:, None]
    out = {}
    s0 = log["segment"] == 0
    org = log["org"][s0].astype(np.float64)
    out["origin x"] = (org[:, 0] - lo[0]) / (hi[0] - lo[0])
    out["origin y"] = (org[:, 1] - lo[1]) / (hi[1] - lo[1])
    assert np.all(org[:, 2] == hi[2])
    out["source cos^(n+1)"] = (-d[s0, 2]) ** (n + 1)
    out["source azimuth"] = (np.arctan2(d[s0, 1], d[s0, 0]) + np.pi) / (2 * np.pi)
    # the record after a hit of the same path is the re-emitted segment
    order = np.lexsort((log["segment"], log["ray"]))
    lg, dd = log[order], d[order]
    after_hit = np.zeros(len(lg), bool)
    after_hit[1:] = ((lg["kind"][:-1] == 0) & (lg["ray"][1:] == lg["ray"][:-1])
                     & (lg["segment"][1:] == lg["segment"][:-1] + 1))
    out["diffuse cos^2"] = dd[after_hit, 2] ** 2
    out["diffuse azimuth"] = (np.arctan2(dd[after_hit, 1], dd[after_hit, 0]) + np.pi) / (2 * np.pi)
    assert np.all(dd[after_hit, 2] > 0)  # into the upper half space of the normal
    return out


def _check(samples):
    assert len(samples["origin x"]) == N_RAYS and len(samples["diffuse cos^2"]) > N_RAYS // 2
    for name, u in samples.items():
        p = stats.kstest(u, "uniform").pvalue
        assert p > P_MIN, (name, p)
    # and a sampler that is off is caught: cos(theta) itself is not uniform
    assert stats.kstest(np.sqrt(samples["diffuse cos^2"]), "uniform").pvalue < 1e-10


@pytest.mark.parametrize("n", [1.0, 5.0])
def test_oracle_samplers(oracle_lib, n):
    p, nrm, r, lo, hi = _plane()
    s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
    s.neighbors()
    cfg = oracle_lib.make_config(lo, hi, sticking=0.2, source_exponent=n, seed=11)
    log = np.concatenate([oracle_lib.trace_log(s, cfg, i) for i in range(N_RAYS)])
    _check(_uniform_samples(log, lo, hi, n))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1.0, 5.0])
def test_gpu_samplers(rtg_lib, n):
    from rti_gb300 import Engine
    p, nrm, r, lo, hi = _plane()
    with Engine(0) as e:
        e.upload_discs(p, nrm, r)
        e.configure(box=(lo, hi), sticking=0.2, source_exponent=n, x_bound=1, y_bound=1, reset=True)
        e.set_segment_log(0, N_RAYS, 8 * N_RAYS)
        e.trace(N_RAYS, seed=11)
        log, dropped = e.segment_log()
        e.set_segment_log(0, 0, 0)
    assert dropped == 0
    _check(_uniform_samples(log, lo, hi, n))


# ---- Russian roulette and the diffuse/specular mixture ----------------------

ROULETTE_RAYS = 30_000
MIX_RAYS = 20_000
SPEC = 0.3


def _roulette(log, s):
    """Roulette events (rejection_control.hpp:28-61): a hit after which the
    weight w' = w - w s falls below 0.1; the path goes on with weight 0.3 with
    probability w' / 0.3, else it ends.  Returns (events, kills, expected kills,
    variance)."""
    order = np.lexsort((log["segment"], log["ray"]))
    lg = log[order]
    w = lg["weight"]
    w_after = w - w * np.float32(s)  # the kernel's float arithmetic
    has_next = np.zeros(len(lg), bool)
    has_next[:-1] = (lg["ray"][1:] == lg["ray"][:-1]) & (lg["segment"][1:] == lg["segment"][:-1] + 1)
    ev = (lg["kind"] == 0) & (w_after.astype(np.float64) < 0.1) & (w_after > 0)
    survived = ev & has_next
    nxt_w = np.zeros(len(lg), np.float32)
    nxt_w[:-1] = w[1:]
    assert np.all(nxt_w[survived] == np.float32(0.3))  # survivors carry the renewal weight
    p_kill = 1.0 - w_after[ev].astype(np.float64) / 0.3
    return int(ev.sum()), int((ev & ~has_next).sum()), float(p_kill.sum()), float((p_kill * (1 - p_kill)).sum())


def _mirror_fraction(log):
    """On a plane with normal +z: the share of re-emissions that leave in the
    mirror direction of the incoming one (specular.hpp:16-40)."""
    d = (log["end"] - log["org"]).astype(np.float64)
    d /= np.linalg.norm(d, axis=1)[:, None]
    order = np.lexsort((log["segment"], log["ray"]))
    lg, dd = log[order], d[order]
    pair = ((lg["kind"][:-1] == 0) & (lg["ray"][1:] == lg["ray"][:-1])
            & (lg["segment"][1:] == lg["segment"][:-1] + 1))
    d_in, d_out = dd[:-1][pair], dd[1:][pair]
    mirror = np.all(np.abs(d_out - d_in * [1, 1, -1]) < 1e-4, axis=1)
    return int(pair.sum()), int(mirror.sum())


def _check_roulette(events, kills, expected, var):
    assert events > 2000
    assert abs(kills - expected) < 4 * np.sqrt(var), (events, kills, expected)


def _check_mixture(n, mirrored):
    assert n > MIX_RAYS // 2
    assert abs(mirrored - SPEC * n) < 4 * np.sqrt(n * SPEC * (1 - SPEC)), (n, mirrored)


def _trench():
    from rti_gb300 import scenes
    return scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)


def test_oracle_roulette_and_mixture(oracle_lib):
    t = _trench()
    s = oracle_lib.Scene(t.xyzr, t.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(t.box_lo, t.box_hi, sticking=0.3, seed=21)
    log = np.concatenate([oracle_lib.trace_log(s, cfg, i) for i in range(ROULETTE_RAYS)])
    _check_roulette(*_roulette(log, 0.3))
    p, nrm, r, lo, hi = _plane()
    s = oracle_lib.Scene(np.concatenate([p, r[:, None]], 1), nrm)
    cfg = oracle_lib.make_config(lo, hi, sticking=0.2, reflection=2, specular_fraction=SPEC, seed=22)
    log = np.concatenate([oracle_lib.trace_log(s, cfg, i) for i in range(MIX_RAYS)])
    _check_mixture(*_mirror_fraction(log))


@pytest.mark.gpu
def test_gpu_roulette_and_mixture(rtg_lib):
    from rti_gb300 import Engine
    t = _trench()
    with Engine(0) as e:
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(t.box_lo, t.box_hi), sticking=0.3, x_bound=1, y_bound=1, reset=True)
        e.set_segment_log(0, ROULETTE_RAYS, 64 * ROULETTE_RAYS)
        e.trace(ROULETTE_RAYS, seed=21)
        log, dropped = e.segment_log()
        assert dropped == 0
        _check_roulette(*_roulette(log, 0.3))
        p, nrm, r, lo, hi = _plane()
        e.upload_discs(p, nrm, r)
        e.configure(box=(lo, hi), sticking=0.2, reflection=2, specular_fraction=SPEC, x_bound=1, y_bound=1,
                    reset=True)
        e.set_segment_log(0, MIX_RAYS, 8 * MIX_RAYS)
        e.trace(MIX_RAYS, seed=22)
        log, dropped = e.segment_log()
        e.set_segment_log(0, 0, 0)
    assert dropped == 0
    _check_mixture(*_mirror_fraction(log))
