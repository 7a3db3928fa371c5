"""The CPU oracle against the reference's own known answers (no GPU).

* 37 exposed-area cases of test/rti/geo/disc_bounding_box_intersector.cpp
* 9 hand-built cases of test/rti/trace/local_intersector.cpp
* Philox4x32-10 known-answer vectors (Random123's published kat_vectors)
* the neighbourhood divide-and-conquer against the brute-force pair test
"""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("case", _load("area_inside_cases.json"), ids=lambda c: c["name"])
def test_area_inside_known_answers(oracle_lib, case):
    a = oracle_lib.area_inside(case["box"], case["disc"], case["normal"])
    if case["tol"] == 0:
        assert a == case["expected"], (a, case)
    else:
        assert abs(a - case["expected"]) < case["tol"], (a, case)


@pytest.mark.parametrize("case", _load("local_intersector_cases.json"), ids=lambda c: c["name"])
def test_local_intersector_known_answers(oracle_lib, case):
    assert oracle_lib.local_intersect(case["org"], case["dir"], case["disc"], case["normal"]) == case["expected"]


def test_philox_known_answers(oracle_lib):
    P = oracle_lib.philox4x32_10
    assert list(P([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(P([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(P([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_sincos2pi_accuracy(oracle_lib):
    rng = np.random.default_rng(1)
    us = np.concatenate([rng.random(20000), [0.0, 0.125, 0.25, 0.375, 0.5, 0.75, 1.0]]).astype(np.float32)
    err = 0.0
    for u in us:
        s, c = oracle_lib.sincos2pi(float(u))
        a = 2 * math.pi * float(u)
        err = max(err, abs(s - math.sin(a)), abs(c - math.cos(a)))
    assert err < 2e-7


def test_powf_accuracy(oracle_lib):
    rng = np.random.default_rng(2)
    for e in (2 / 6, 2 / 51, 2 / 3, 1.5):
        for x in rng.random(2000).astype(np.float32):
            x = max(float(x), 2 ** -24)
            r = oracle_lib.powf(x, e)
            assert abs(r - x ** e) <= 2e-6 * x ** e


def test_diffuse_direction_is_unit_and_in_hemisphere(oracle_lib):
    rng = np.random.default_rng(3)
    for _ in range(500):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        d = oracle_lib.diffuse_dir(n.astype(np.float32), int(rng.integers(0, 2 ** 32)), int(rng.integers(0, 2 ** 32)))
        assert abs(np.linalg.norm(d.astype(np.float64)) - 1) < 1e-5
        assert float(np.dot(d, n)) > 0


def _random_cloud(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.random((n, 3)).astype(np.float32) * np.array([1.0, 1.0, 0.3], np.float32)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    r = (0.02 + 0.03 * rng.random(n)).astype(np.float32)
    return np.concatenate([p, r[:, None]], 1), nrm.astype(np.float32)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_neighborhood_dac_matches_bruteforce(oracle_lib, seed):
    xyzr, nrm = _random_cloud(3000, seed)
    s = oracle_lib.Scene(xyzr, nrm)
    rp1, c1 = s.neighbors()
    rp2, c2 = s.neighbors(bruteforce=True)
    assert np.array_equal(rp1, rp2) and np.array_equal(c1, c2)


def test_neighborhood_trench_grid(oracle_lib):
    from rti_gb300 import scenes
    t = scenes.trench_discs(domain=0.6, width=0.2, depth=0.3)
    s = oracle_lib.Scene(t.xyzr, t.normals)
    rp1, c1 = s.neighbors()
    rp2, c2 = s.neighbors(bruteforce=True)
    assert np.array_equal(rp1, rp2) and np.array_equal(c1, c2)
    deg = np.diff(rp1)
    # a grid of radius spacing*sqrt(2)/2: the 4 axis neighbours in a face, a few more where faces meet
    assert deg.max() <= 12 and np.median(deg) >= 4


def test_normalize_and_stats_match_reference_formulas(oracle_lib):
    rng = np.random.default_rng(4)
    n = 50
    s1 = rng.random(n)
    areas = (0.5 + rng.random(n)).astype(np.float32)
    rp = np.arange(0, 2 * n + 1, 2, dtype=np.int64)
    cols = rng.integers(0, n, 2 * n).astype(np.int32)
    out = oracle_lib.normalize(s1, areas, rp, cols)
    vv = np.array([(s1[i] / areas[i] + s1[cols[2 * i]] / areas[cols[2 * i]] + s1[cols[2 * i + 1]] /
                    areas[cols[2 * i + 1]]) / 3 for i in range(n)])
    ref = (vv.astype(np.float32).astype(np.float64) / vv.max()).astype(np.float32)
    np.testing.assert_allclose(out, ref, rtol=1e-6)
    s2 = s1 ** 2 * (1 + rng.random(n))
    rel = oracle_lib.relative_error(s1, s2, 1000)
    np.testing.assert_allclose(rel, np.sqrt(s2 / s1 ** 2 - 1.0 / 1000), rtol=1e-12)


def test_radiosity_fixture_shape():
    for sp in ("1", "0.1", "0.01"):
        d = np.loadtxt(os.path.join(GOLDEN, f"radiosity_ar45_sp{sp}.txt"))
        assert d.shape == (300, 2)
        assert d[0, 1] == 1.0 and np.all(np.diff(d[:, 0]) > 0)
