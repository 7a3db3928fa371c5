"""Calibrating sticking coefficients by gradient, through rti_gb300.autograd.flux.

A process model fits the sticking probability of its particles (what
i_particle::get_sticking_probability returns in the reference,
particle/i_particle.hpp:14) to measured profiles.  Here the "measurement" is a
flux traced with a hidden sticking and an independent random stream; the fit
starts from 0.05 and takes Newton steps whose derivatives come from the adjoint
replay (one replay per backward call), with common random numbers across its
iterations (one seed), so the objective it solves is smooth.

* Hole of 200,192 triangles (radius 0.5, depth 10), one global sticking, hidden
  0.01: the observable is the conformality ratio, flux onto the lowest quarter
  of the hole over flux onto the top surface, which falls monotonically with
  the sticking (the bottom flux alone does not: it is s times the arrivals,
  which rise as s falls, so it peaks near s = 0.02 and has two roots).
* Trench of 98,301 discs (width 1, depth 5), a sticking field of four regions
  (top, upper wall, lower wall, bottom), hidden (0.4, 0.2, 0.1, 0.05): the
  observables are the four regions' fluxes; each Gauss-Newton step takes the
  4 x 4 Jacobian from four backward calls (four adjoint replays).

Bar: every hidden value recovered within 2 % in at most 20 adjoint evaluations.
The remaining error is the Monte Carlo error of target and fit (1e7 rays each).
"""
import math

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
N_RAYS = 10_000_000
TARGET_SEED, FIT_SEED = 1234, 99


def test_calibrate_global_sticking_on_hole(rtg_lib):
    import torch

    from rti_gb300 import Engine
    from rti_gb300.autograd import flux
    h = scenes.hole_triangles()
    dev = torch.device("cuda", 0)
    zc = h.vertices.astype(np.float64)[h.indices].mean(axis=1)[:, 2]
    low = torch.from_numpy(zc < -0.75 * h.meta["depth"]).to(dev)
    top = torch.from_numpy(zc > -1e-3).to(dev)

    def ratio(s1):
        return s1[low].sum() / s1[top].sum()

    with Engine(0) as e:
        e.upload_triangles(h.vertices, h.indices)
        e.configure(box=(h.box_lo, h.box_hi), reflection=2, specular_fraction=0.1, x_bound=1, y_bound=1,
                    reset=True)
        r_target = float(ratio(flux(e, 0.01, 1.0, N_RAYS, TARGET_SEED)))
        s, evals, history = 0.05, 0, []
        for _ in range(10):
            st = torch.tensor(s, dtype=torch.float64, requires_grad=True)
            r = ratio(flux(e, st, 1.0, N_RAYS, FIT_SEED))
            r.backward()  # one adjoint replay
            evals += 1
            rv, dr = r.item(), st.grad.item()
            history.append((s, rv, dr))
            if abs(rv - r_target) <= 1e-4 * r_target:
                break
            # Newton in log s (keeps s positive); at most a factor e^2 per step
            s *= math.exp(max(-2.0, min(2.0, (r_target - rv) / (s * dr))))
        assert evals <= 20, history
        assert abs(s - 0.01) <= 0.02 * 0.01, history


def test_calibrate_region_field_on_trench(rtg_lib):
    import torch

    from rti_gb300 import Engine
    from rti_gb300.autograd import flux
    t = scenes.trench_discs()
    dev = torch.device("cuda", 0)
    z = t.points[:, 2]
    region = np.where(z >= -1e-6, 0, np.where(z > -2.5, 1, np.where(z > -5.0 + 1e-3, 2, 3)))
    assert np.bincount(region).min() > 5000
    reg = torch.from_numpy(region).to(dev)
    hidden = torch.tensor([0.4, 0.2, 0.1, 0.05], dtype=torch.float64, device=dev)

    def region_flux(theta, seed):
        s1 = flux(e, theta[reg], 1.0, N_RAYS, seed)  # a per-disc sticking field from the 4 values
        return torch.zeros(4, dtype=torch.float64, device=dev).index_add(0, reg, s1)

    with Engine(0) as e:
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(t.box_lo, t.box_hi), x_bound=1, y_bound=1, reset=True)
        target = region_flux(hidden, TARGET_SEED).detach()
        theta, evals, history = torch.full((4,), 0.05, dtype=torch.float64, device=dev), 0, []
        for _ in range(5):
            th = theta.clone().requires_grad_(True)
            j = region_flux(th, FIT_SEED)
            resid = (j.detach() - target) / target
            history.append((theta.tolist(), resid.tolist()))
            if float(resid.abs().max()) <= 1e-4:
                break
            jac = torch.stack([torch.autograd.grad(j[k], th, retain_graph=k < 3)[0] for k in range(4)])
            evals += 4  # one adjoint replay per row
            theta = (theta + torch.linalg.solve(jac, target - j.detach())).clamp(1e-3, 0.99)
        assert evals <= 20, history
        rel = ((theta - hidden) / hidden).abs()
        assert float(rel.max()) <= 0.02, (theta.tolist(), history)
