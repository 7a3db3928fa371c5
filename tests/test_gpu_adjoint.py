"""Adjoint (differentiation path) on the GPU.

* the replay equals the oracle's restatement on the same inputs: dL/ds, dL/dn
  and dL/ds_j to FP64 summation order (rtol 1e-9), for both estimators;
* central differences with common random numbers of GPU forward traces: the
  unbiased global-sticking gradient within 2 % (Richardson-extrapolated from
  h = 0.1 s, 0.2 s), the exponent gradient within 5 %, per-primitive gradients
  of the held estimator (h = 1e-3 relative) within 1e-3 relative;
* the torch.autograd.Function returns the same numbers as the C ABI.
"""
import math

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng(rtg_lib):
    from rti_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def trench():
    return scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)


@pytest.fixture(scope="module")
def hole():
    return scenes.hole_triangles(n_theta=128, n_wall=40, n_top=8, n_bottom=6, depth=4.0)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("unbiased", [False, True], ids=["held", "unbiased"])
def test_adjoint_global_matches_oracle(eng, trench, oracle_lib, unbiased):
    eng.upload_discs(trench.points, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
    g = np.random.default_rng(1).random(trench.n)
    ds, dn, _ = eng.adjoint(g, 100000, seed=7, unbiased=unbiased)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, sticking=0.1, seed=7)
    ods, odn, _, _ = oracle_lib.adjoint(s, cfg, g, 0, 100000, unbiased=unbiased)
    assert _rel(ds, ods) < 1e-9 and _rel(dn, odn) < 1e-9


@pytest.mark.parametrize("unbiased", [False, True], ids=["held", "unbiased"])
def test_adjoint_field_matches_oracle(eng, trench, oracle_lib, unbiased):
    rng = np.random.default_rng(2)
    field = rng.uniform(0.05, 0.4, trench.n).astype(np.float32)
    eng.upload_discs(trench.points, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), x_bound=1, y_bound=1, reset=True)
    eng.set_sticking_field(field)
    g = rng.random(trench.n)
    ds, dn, fg = eng.adjoint(g, 60000, seed=8, unbiased=unbiased)
    s = oracle_lib.Scene(trench.xyzr, trench.normals)
    s.neighbors()
    cfg = oracle_lib.make_config(trench.box_lo, trench.box_hi, seed=8)
    _, odn, ofg, _ = oracle_lib.adjoint(s, cfg, g, 0, 60000, sticking_field=field, unbiased=unbiased)
    assert ds == 0.0 and _rel(dn, odn) < 1e-9
    np.testing.assert_allclose(fg, ofg, rtol=1e-9, atol=1e-9 * np.abs(ofg).max())


def test_adjoint_hole_mixed_matches_oracle(eng, hole, oracle_lib):
    eng.upload_triangles(hole.vertices, hole.indices)
    eng.configure(box=(hole.box_lo, hole.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1,
                  x_bound=1, y_bound=1, reset=True)
    g = np.random.default_rng(3).random(hole.n)
    ds, dn, _ = eng.adjoint(g, 50000, seed=9)
    s = oracle_lib.Scene(tri_vertices=hole.vertices, tri_indices=hole.indices)
    cfg = oracle_lib.make_config(hole.box_lo, hole.box_hi, sticking=0.01, reflection=2, specular_fraction=0.1,
                                 seed=9)
    ods, odn, _, _ = oracle_lib.adjoint(s, cfg, g, 0, 50000, unbiased=True)
    assert _rel(ds, ods) < 1e-9 and _rel(dn, odn) < 1e-9


def _bottom_quarter_weights(h):
    V = h.vertices.astype(np.float64)
    c = V[h.indices].mean(axis=1)
    depth = h.meta["depth"]
    return (c[:, 2] < -0.75 * depth).astype(np.float64)


def test_global_sticking_gradient_vs_crn_differences(eng):
    """Hole of the bench workload (s = 0.01, 10 % specular), L = bottom-quarter
    flux, 1e7 rays.  With Russian roulette a step of 1e-3 s flips a few roulette
    decisions whose jumps dominate the difference quotient, so the unbiased
    gradient is checked against central differences at h = 0.1 s and 0.2 s,
    Richardson-extrapolated to h -> 0."""
    h = scenes.hole_triangles()
    eng.upload_triangles(h.vertices, h.indices)
    s0, n = 0.01, 10_000_000
    eng.configure(box=(h.box_lo, h.box_hi), sticking=s0, reflection=2, specular_fraction=0.1, x_bound=1, y_bound=1,
                  reset=True)
    g = _bottom_quarter_weights(h)
    ds, _, _ = eng.adjoint(g, n, seed=11, unbiased=True)

    def L(s):
        eng.configure(sticking=s)
        eng.trace(n, 11)
        return float(g @ eng.values())

    d1 = (L(s0 * 1.1) - L(s0 * 0.9)) / (0.2 * s0)
    d2 = (L(s0 * 1.2) - L(s0 * 0.8)) / (0.4 * s0)
    fd = (4 * d1 - d2) / 3
    print(f"dL/ds adjoint {ds:.6g}  central differences {d1:.6g} (0.1 s), {d2:.6g} (0.2 s) -> {fd:.6g}")
    assert _rel(ds, fd) < 0.02


def test_roulette_flips_at_a_relative_step_of_1e3(eng, oracle_lib):
    """Why the sticking gradient is not checked against h = 1e-3 s differences.

    Hole of the bench workload at 1e7 rays, s = 0.01, L = bottom-quarter flux.
    The oracle traces every path once with weights at s - h, s and s + h
    (h = 1e-3 s) on its shared geometry and counts the Russian-roulette
    decisions that differ (rejection_control.hpp:44-57).  Every path starts at
    w = 1 and loses a factor (1 - s) per deposit, so the first roulette comes at
    the same collision on every path, ceil(ln 0.1 / ln(1 - s)): 229 at s + h,
    230 at s - h.  The step therefore moves the roulette of every path that
    reaches it, and the difference quotient over all paths is far from the
    derivative with the decisions held.  Over the paths with no flipped
    decision the quotient equals the held derivative (bar 2 %), and the held
    derivative over all paths equals the GPU's held replay (FP64 order); the
    GPU's own +-h traces give the oracle's quotient."""
    h_ = scenes.hole_triangles()
    eng.upload_triangles(h_.vertices, h_.indices)
    s0, n = 0.01, 10_000_000
    eng.configure(box=(h_.box_lo, h_.box_hi), sticking=s0, reflection=2, specular_fraction=0.1, x_bound=1,
                  y_bound=1, reset=True)
    g = _bottom_quarter_weights(h_)
    held_gpu, _, _ = eng.adjoint(g, n, seed=11, unbiased=False)
    sc = oracle_lib.Scene(tri_vertices=h_.vertices, tri_indices=h_.indices)
    cfg = oracle_lib.make_config(h_.box_lo, h_.box_hi, sticking=s0, reflection=2, specular_fraction=0.1, seed=11)
    hh = float(np.float32(1e-3) * np.float32(s0))
    r = oracle_lib.fd_pair(sc, cfg, g, 0, n, hh)
    print(f"h = 1e-3 s: {r['decisions_flipped']} roulette decisions flipped on {r['paths_flipped']} paths "
          f"({r['paths_with_roulette']} paths meet the roulette, {n} rays); difference quotient "
          f"{r['fd_all']:.6g} over all paths, held derivative {r['held_all']:.6g}; over the unflipped paths "
          f"{r['fd_unflipped']:.6g} vs {r['held_unflipped']:.6g}")
    k_plus = math.ceil(math.log(0.1) / math.log(1.0 - (s0 + hh)))
    k_minus = math.ceil(math.log(0.1) / math.log(1.0 - (s0 - hh)))
    assert k_plus != k_minus and r["paths_flipped"] == r["paths_with_roulette"] > 0
    assert _rel(r["fd_unflipped"], r["held_unflipped"]) < 0.02
    assert _rel(r["held_all"], held_gpu) < 1e-9
    assert _rel(r["fd_all"], r["held_all"]) > 0.2  # the flips dominate the plain quotient

    def L(s):
        eng.configure(sticking=s)
        eng.trace(n, 11)
        return float(g @ eng.values())

    fd_gpu = (L(float(np.float32(s0) + np.float32(hh))) - L(float(np.float32(s0) - np.float32(hh)))) / r["two_h"]
    eng.configure(sticking=s0)
    assert _rel(fd_gpu, r["fd_all"]) < 1e-4


def test_exponent_gradient_vs_crn_differences(eng):
    """Score-function dL/dn at n = 1 against central differences of 4e7-ray
    traces at h = 0.2 (the directions move with n, so the difference quotient
    is noisy at about 2 % here)."""
    h = scenes.hole_triangles()
    eng.upload_triangles(h.vertices, h.indices)
    n = 40_000_000
    eng.configure(box=(h.box_lo, h.box_hi), sticking=0.01, reflection=2, specular_fraction=0.1, x_bound=1,
                  y_bound=1, source_exponent=1.0, reset=True)
    g = _bottom_quarter_weights(h)
    _, dn, _ = eng.adjoint(g, n, seed=21, unbiased=True)

    def L(ex):
        eng.configure(source_exponent=ex)
        eng.trace(n, 21)
        return float(g @ eng.values())

    fd = (L(1.2) - L(0.8)) / 0.4
    print(f"dL/dn score {dn:.6g}  central difference {fd:.6g}")
    assert _rel(dn, fd) < 0.05


def test_field_gradient_spot_checks_vs_crn_differences(eng):
    """Rough surface with a logistic-normal sticking field; held estimator vs
    central differences of single elements (the roulette decisions of a
    1e-3 perturbation almost never flip)."""
    r = scenes.rough_discs(n=96, spacing=0.01, rms=0.05, corr=0.2, seed=4)
    rng = np.random.default_rng(5)
    field = (1.0 / (1.0 + np.exp(-rng.normal(-2.0, 0.5, r.n)))).astype(np.float32)
    eng.upload_discs(r.points, r.normals, r.radii)
    eng.configure(box=(r.box_lo, r.box_hi), x_bound=1, y_bound=1, reset=True)
    eng.set_sticking_field(field)
    z = r.points[:, 2]
    g = (z < np.quantile(z, 0.25)).astype(np.float64)
    n = 400000
    _, _, fg = eng.adjoint(g, n, seed=12, unbiased=False)
    bad = 0
    for j in rng.choice(r.n, 12, replace=False):
        hj = np.float32(1e-3) * field[j]
        fp, fm = field.copy(), field.copy()
        fp[j] += hj
        fm[j] -= hj
        eng.set_sticking_field(fp)
        eng.trace(n, 12)
        lp = float(g @ eng.values())
        eng.set_sticking_field(fm)
        eng.trace(n, 12)
        lm = float(g @ eng.values())
        fd = (lp - lm) / (float(fp[j]) - float(fm[j]))
        if not abs(fg[j] - fd) <= 1e-3 * max(abs(fd), 1e-6 * np.abs(fg).max()):
            bad += 1
    assert bad <= 1  # one roulette flip among 12 checks is tolerated


def test_autograd_function_matches_abi(eng, trench):
    import torch

    from rti_gb300.autograd import flux
    eng.upload_discs(trench.points, trench.normals, trench.radii)
    eng.configure(box=(trench.box_lo, trench.box_hi), x_bound=1, y_bound=1, reset=True)
    g = np.random.default_rng(6).random(trench.n)
    s = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    e = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    s1 = flux(eng, s, e, 50000, seed=13)
    (torch.from_numpy(g).to(s1.device) * s1).sum().backward()
    eng.configure(sticking=0.2, source_exponent=1.0)
    ds, dn, _ = eng.adjoint(g, 50000, seed=13, unbiased=True)
    assert _rel(float(s.grad), ds) < 1e-12 and _rel(float(e.grad), dn) < 1e-12
    # field form
    f = torch.full((trench.n,), 0.2, dtype=torch.float32, requires_grad=True)
    s1f = flux(eng, f, 1.0, 50000, seed=13)
    np.testing.assert_allclose(s1f.detach().cpu().numpy(), s1.detach().cpu().numpy(), rtol=1e-12)
    (torch.from_numpy(g).to(s1f.device) * s1f).sum().backward()
    assert abs(float(f.grad.double().sum()) - ds) <= 1e-6 * abs(ds)
