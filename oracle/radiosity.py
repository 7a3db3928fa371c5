"""Deterministic radiosity solutions of the flux problem (test infrastructure).

A physics check of the Monte Carlo flux that does not share any code or
arithmetic with it.  A cosine (Lambertian) source above an opening, diffuse
re-emission of the part that does not stick (sticking s), and a convex cavity
below the opening, so that every pair of cavity patches sees each other.  The
incoming flux density G_i on patch i obeys

    G_i = E0 F_{i,open} + (1 - s) sum_j F_{i,j} G_j,

with F the patch-to-patch view factors; E0 = 1 is the flux density through the
opening plane (the flux density on the flat top surface of the Monte Carlo
scenes).  Both solvers also return dG/ds, the exact derivative of the solution
with respect to a global sticking (what an unbiased adjoint estimates).  rti ships radiosity data only for one cylinder (verification/
radiosity/analytical_solution: radius 0.5, length 45); these solvers give the
same for any cylindrical hole and for an infinite trench, and are checked
against that data first.

* ``hole``: cylindrical hole of radius R and depth H (wall bands and bottom
  annuli).  All view factors are closed forms built from the coaxial-disc view
  factor (Siegel & Howell, "Thermal Radiation Heat Transfer", disc to parallel
  coaxial disc) by view-factor algebra: a wall band of height d2 - d1 at
  distances [d1, d2] from a cross-section sends R (F(d1) - F(d2)) / (2 (d2 -
  d1)) of its radiation through it (F = disc-to-disc factor of two sections,
  reciprocity), and a band sends to a band further down what crosses the
  cross-section at the near edge of that band minus what crosses its far edge;
  annuli of the bottom likewise by differences of discs.
* ``trench``: infinitely long rectangular trench of width W and depth D (wall
  and bottom strips of the cross-section); view factors by Hottel's crossed
  strings, exact for two-dimensional geometry.
"""
from __future__ import annotations

import numpy as np


def _solve(F, f_open, s):
    """G = (I - (1 - s) F)^-1 f_open and its derivative with respect to the
    sticking s, dG/ds = -(I - (1 - s) F)^-1 F G."""
    A = np.eye(len(f_open)) - (1.0 - s) * F
    G = np.linalg.solve(A, f_open)
    return G, np.linalg.solve(A, -(F @ G))


def disc_to_disc(r1, r2, h):
    """View factor from a disc of radius r1 to a parallel coaxial disc of radius
    r2 at distance h (h = 0: min(1, (r2/r1)^2))."""
    r1 = np.asarray(r1, dtype=np.float64)
    h = np.asarray(h, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        R1, R2 = r1 / h, r2 / h
        S = 1.0 + (1.0 + R2 * R2) / (R1 * R1)
        f = 0.5 * (S - np.sqrt(np.maximum(S * S - 4.0 * (r2 / r1) ** 2, 0.0)))
    return np.where(h > 0, f, np.minimum(1.0, (r2 / np.maximum(r1, 1e-300)) ** 2))


def hole(radius: float, depth: float, sticking: float, n_wall: int = 400, n_bottom: int = 40):
    """Radiosity of a cylindrical hole.  Returns a dict with the wall band
    centres (depth below the opening) and their incoming flux density G, the
    bottom annulus centres (radius) and theirs, the direct part alone, and the
    row sums of the view factors including the opening (1 by construction)."""
    R, H, s = float(radius), float(depth), float(sticking)
    zw = np.linspace(0.0, H, n_wall + 1)          # band edges, depth below the opening
    rb = np.linspace(0.0, R, n_bottom + 1)        # annulus edges on the bottom
    nw, nb = n_wall, n_bottom
    n = nw + nb
    area = np.concatenate([2 * np.pi * R * np.diff(zw), np.pi * np.diff(rb ** 2)])

    # S[i, m]: band i to the cross-section at edge depth m (every edge lies
    # outside or on the boundary of band i)
    a, b = zw[:-1, None], zw[1:, None]
    z = zw[None, :]
    d1 = np.where(z >= b, z - b, a - z)
    S = R * (disc_to_disc(R, R, d1) - disc_to_disc(R, R, d1 + (b - a))) / (2.0 * (b - a))
    F = np.zeros((n, n))
    f_open = np.zeros(n)
    D = S[:, :-1] - S[:, 1:]           # what crosses the top edge of band j minus its bottom edge
    i_idx, j_idx = np.indices((nw, nw))
    F[:nw, :nw] = np.where(j_idx > i_idx, D, np.where(j_idx < i_idx, -D, 0.0))
    F[np.arange(nw), np.arange(nw)] = 1.0 - S[np.arange(nw), np.arange(nw)] - S[np.arange(nw), np.arange(nw) + 1]
    f_open[:nw] = S[:, 0]
    # bottom annulus k: sec[k, m] = to the cross-section at edge depth m
    ra, rk = rb[:-1, None], rb[1:, None]
    h = H - zw[None, :]
    a_b, a_a = np.pi * rk * rk, np.pi * ra * ra
    fa = np.where(ra > 0, disc_to_disc(np.maximum(ra, 1e-12), R, h), 0.0)
    sec = (a_b * disc_to_disc(rk, R, h) - a_a * fa) / (a_b - a_a)
    F[nw:, :nw] = sec[:, 1:] - sec[:, :-1]
    F[:nw, nw:] = (F[nw:, :nw] * area[nw:, None] / area[None, :nw]).T
    f_open[nw:] = sec[:, 0]
    G, dG = _solve(F, f_open, s)
    return {"wall_depth": 0.5 * (zw[1:] + zw[:-1]), "wall": G[:nw], "d_wall": dG[:nw],
            "bottom_radius": 0.5 * (rb[1:] + rb[:-1]), "bottom": G[nw:], "d_bottom": dG[nw:],
            "direct_wall": f_open[:nw], "direct_bottom": f_open[nw:], "row_sums": F.sum(1) + f_open}


def _strings(p, q, u, v):
    """Crossed minus uncrossed string lengths between segments pq and uv that
    see each other (the crossed pair is the longer one)."""
    d = lambda x, y: float(np.hypot(x[0] - y[0], x[1] - y[1]))
    return abs((d(p, v) + d(q, u)) - (d(p, u) + d(q, v)))


def _trench_system(W, D, n_wall, n_bottom):
    """Strips of the trench cross-section (left wall top-down, bottom left to
    right, right wall bottom-up), their lengths, view factors and view factors
    to the opening."""
    zw = np.linspace(0.0, D, n_wall + 1)
    xb = np.linspace(0.0, W, n_bottom + 1)
    segs = []  # each strip as its two end points
    for i in range(n_wall):   # left wall, x = 0, going down
        segs.append(((0.0, -zw[i]), (0.0, -zw[i + 1])))
    for i in range(n_bottom):  # bottom, z = -D, going right
        segs.append(((xb[i], -D), (xb[i + 1], -D)))
    for i in range(n_wall):   # right wall, x = W, going up
        segs.append(((W, -zw[n_wall - i]), (W, -zw[n_wall - i - 1])))
    opening = ((W, 0.0), (0.0, 0.0))
    n = len(segs)
    L = np.array([np.hypot(q[0] - p[0], q[1] - p[1]) for p, q in segs])
    F = np.zeros((n, n))
    f_open = np.zeros(n)
    for i, (p, q) in enumerate(segs):
        for j, (u, v) in enumerate(segs):
            if i == j:
                continue
            # strips on one straight side do not see each other
            same_line = (p[0] == q[0] == u[0] == v[0]) or (p[1] == q[1] == u[1] == v[1])
            if not same_line:
                F[i, j] = _strings(p, q, u, v) / (2.0 * L[i])
        f_open[i] = _strings(p, q, opening[0], opening[1]) / (2.0 * L[i])
    return zw, xb, L, F, f_open


def trench(width: float, depth: float, sticking: float, n_wall: int = 200, n_bottom: int = 100):
    """Radiosity of an infinitely long rectangular trench (cross-section in the
    x-z plane, opening at z = 0 between x = 0 and x = width).  Returns the left
    wall strip centres (depth), the bottom strip centres (x) and their incoming
    flux densities G and dG/ds (the right wall mirrors the left)."""
    zw, xb, L, F, f_open = _trench_system(float(width), float(depth), n_wall, n_bottom)
    G, dG = _solve(F, f_open, float(sticking))
    return {"wall_depth": 0.5 * (zw[1:] + zw[:-1]), "wall": G[:n_wall], "d_wall": dG[:n_wall],
            "bottom_x": 0.5 * (xb[1:] + xb[:-1]), "bottom": G[n_wall:n_wall + n_bottom],
            "d_bottom": dG[n_wall:n_wall + n_bottom],
            "right_wall": G[n_wall + n_bottom:][::-1], "row_sums": F.sum(1) + f_open}


def trench_field_gradient(width: float, depth: float, sticking, n_wall: int, n_bottom: int,
                          length: float = 1.0, target: str = "bottom"):
    """Per-strip sticking sigma (a scalar or one value per strip, in the strip
    order of the cross-section: left wall top-down, bottom, right wall
    bottom-up) and L = sum over the target strips of sigma_i G_i A_i (A_i =
    strip length x `length`): returns L and dL/dsigma_j for every strip, from
    G = f + F diag(1 - sigma) G and one adjoint solve,
        dL/dsigma_j = [j in target] A_j G_j - lambda^T F[:, j] G_j,
        lambda = (I - F diag(1 - sigma))^-T (sigma A [target])."""
    zw, xb, Ls, F, f_open = _trench_system(float(width), float(depth), n_wall, n_bottom)
    n = len(f_open)
    sigma = np.broadcast_to(np.asarray(sticking, dtype=np.float64), (n,)).copy()
    area = Ls * float(length)
    q = np.zeros(n)
    if target == "bottom":
        q[n_wall:n_wall + n_bottom] = 1.0
    else:
        raise ValueError("target must be 'bottom'")
    M = np.eye(n) - F * (1.0 - sigma)[None, :]
    G = np.linalg.solve(M, f_open)
    w = sigma * area * q
    lam = np.linalg.solve(M.T, w)
    grad = q * area * G - (lam @ F) * G
    return {"L": float(w @ G), "grad": grad, "n_wall": n_wall, "n_bottom": n_bottom}
