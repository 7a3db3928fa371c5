"""Seeded synthetic surfaces for the benchmark and test workloads.

* ``trench_discs``  -- 2-D-extruded trench sampled with oriented discs on a
  regular grid (top, walls, bottom), x/y periodic cell.
* ``hole_triangles`` -- cylindrical hole in a square periodic cell as a
  structured triangle mesh (top annulus-to-square rings, wall, bottom disc)
  with seeded vertex jitter.
* ``hole_discs`` -- the same hole sampled with discs (one disc per wall facet).
* ``rough_discs`` -- discs on a Gaussian random height field.
All coordinates are built in float64 and rounded once to float32.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class DiscSurface:
    points: np.ndarray
    normals: np.ndarray
    radii: np.ndarray
    box_lo: tuple
    box_hi: tuple
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.points)

    @property
    def xyzr(self) -> np.ndarray:
        return np.concatenate([self.points, self.radii[:, None]], axis=1).astype(np.float32)


@dataclass
class TriangleSurface:
    vertices: np.ndarray
    indices: np.ndarray
    box_lo: tuple
    box_hi: tuple
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.indices)


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))


def trench_discs(width: float = 1.0, depth: float = 5.0, domain: float = 3.0, spacing: float = 0.02,
                 source_gap: float = 0.1) -> DiscSurface:
    """Trench extruded along y, centred in a domain x domain cell; disc centres
    on a `spacing` grid whose extreme columns sit on x = 0 and x = domain, so
    that the centre extents (rti's box rule) span exactly the periodic length."""
    nx = int(round(domain / spacing))
    ny = nx
    x0 = (domain - width) / 2.0
    x1 = x0 + width
    i0 = int(round(x0 / spacing))
    i1 = int(round(x1 / spacing))
    nz = int(round(depth / spacing))
    ys = np.arange(ny + 1) * spacing
    pts, nrm = [], []
    top_x = [i * spacing for i in range(nx + 1) if i <= i0 or i >= i1]
    X, Y = np.meshgrid(top_x, ys, indexing="ij")
    pts.append(np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1))
    nrm.append(np.tile([0.0, 0.0, 1.0], (X.size, 1)))
    zw = -np.arange(1, nz) * spacing
    for xw, nx_ in ((i0 * spacing, 1.0), (i1 * spacing, -1.0)):
        Z, Y = np.meshgrid(zw, ys, indexing="ij")
        pts.append(np.stack([np.full(Z.size, xw), Y.ravel(), Z.ravel()], 1))
        nrm.append(np.tile([nx_, 0.0, 0.0], (Z.size, 1)))
    bx = np.arange(i0, i1 + 1) * spacing
    X, Y = np.meshgrid(bx, ys, indexing="ij")
    pts.append(np.stack([X.ravel(), Y.ravel(), np.full(X.size, -nz * spacing)], 1))
    nrm.append(np.tile([0.0, 0.0, 1.0], (X.size, 1)))
    P = _f32(np.concatenate(pts))
    N = _f32(np.concatenate(nrm))
    r = np.float32(spacing * math.sqrt(2.0) / 2.0)
    R = np.full(len(P), r, dtype=np.float32)
    lo = (0.0, 0.0, float(np.float32(-nz * spacing)))
    hi = (float(np.float32(domain)), float(np.float32(domain)), float(np.float32(source_gap)))
    return DiscSurface(P, N, R, lo, hi, {"kind": "trench", "width": width, "depth": depth, "domain": domain,
                                          "spacing": spacing})


def _square_point(theta: float, half: float):
    c, s = math.cos(theta), math.sin(theta)
    m = max(abs(c), abs(s))
    return half * c / m, half * s / m


def hole_triangles(radius: float = 0.5, depth: float = 10.0, cell: float = 2.0, n_theta: int = 512,
                   n_wall: int = 160, n_top: int = 24, n_bottom: int = 12, jitter: float = 0.01, seed: int = 0,
                   source_gap: float = 0.1) -> TriangleSurface:
    """Cylindrical hole of `radius` and `depth` centred in a `cell` x `cell`
    periodic square.  Normals (right-handed winding) point up on the top and
    bottom and towards the axis on the wall.  Interior vertices are jittered by
    up to `jitter` of the local grid step, seeded; the square border, the rim
    and the bottom edge are shared by neighbouring patches and stay watertight."""
    assert n_theta % 8 == 0, "n_theta must include the square's corner directions"
    rng = np.random.default_rng(seed)
    half = cell / 2.0
    dth = 2.0 * math.pi / n_theta
    th = np.arange(n_theta) * dth
    verts = []

    def add(v):
        verts.append(v)
        return len(verts) - 1

    # rings of the top surface: k = 0 is the rim (shared with the wall), k = n_top the square border
    top = np.zeros((n_top + 1, n_theta), dtype=np.int64)
    for k in range(n_top + 1):
        for j in range(n_theta):
            a = th[j]
            if 0 < k < n_top:
                a = a + jitter * dth * rng.uniform(-1, 1)
            f = k / n_top
            if 0 < k < n_top:
                f = f + jitter / n_top * rng.uniform(-1, 1)
            rx, ry = radius * math.cos(a), radius * math.sin(a)
            sx, sy = _square_point(a, half)
            top[k, j] = add((rx + f * (sx - rx), ry + f * (sy - ry), 0.0))
    # wall rings: m = 0 is the rim, m = n_wall the bottom edge
    wall = np.zeros((n_wall + 1, n_theta), dtype=np.int64)
    wall[0] = top[0]
    dz = depth / n_wall
    for m in range(1, n_wall + 1):
        for j in range(n_theta):
            a = th[j]
            z = -m * dz
            if m < n_wall:
                a = a + jitter * dth * rng.uniform(-1, 1)
                z = z + jitter * dz * rng.uniform(-1, 1)
            wall[m, j] = add((radius * math.cos(a), radius * math.sin(a), z))
    # bottom rings: b = 0 the bottom edge, b = n_bottom the centre
    bot = np.zeros((n_bottom, n_theta), dtype=np.int64)
    bot[0] = wall[n_wall]
    dr = radius / n_bottom
    for b in range(1, n_bottom):
        for j in range(n_theta):
            a = th[j] + jitter * dth * rng.uniform(-1, 1)
            rr = radius - b * dr + jitter * dr * rng.uniform(-1, 1)
            bot[b, j] = add((rr * math.cos(a), rr * math.sin(a), -depth))
    centre = add((0.0, 0.0, -depth))
    tris = []
    J = np.arange(n_theta)
    J1 = (J + 1) % n_theta
    # top: rings grow outwards with increasing angle -> (inner_j, outer_j, outer_j1) has +z normal
    for k in range(n_top):
        a, b_, c, d = top[k, J], top[k + 1, J], top[k + 1, J1], top[k, J1]
        tris.append(np.stack([a, b_, c], 1))
        tris.append(np.stack([a, c, d], 1))
    # wall: normal towards the axis
    for m in range(n_wall):
        a, b_, c, d = wall[m, J], wall[m, J1], wall[m + 1, J1], wall[m + 1, J]
        tris.append(np.stack([a, b_, c], 1))
        tris.append(np.stack([a, c, d], 1))
    # bottom: rings shrink inwards, +z normal
    for b in range(n_bottom - 1):
        a, b_, c, d = bot[b, J], bot[b, J1], bot[b + 1, J1], bot[b + 1, J]
        tris.append(np.stack([a, b_, c], 1))
        tris.append(np.stack([a, c, d], 1))
    tris.append(np.stack([bot[n_bottom - 1, J], bot[n_bottom - 1, J1], np.full(n_theta, centre)], 1))
    V = _f32(np.array(verts))
    T = np.ascontiguousarray(np.concatenate(tris).astype(np.uint32))
    lo = (float(np.float32(-half)), float(np.float32(-half)), float(np.float32(-depth)))
    hi = (float(np.float32(half)), float(np.float32(half)), float(np.float32(source_gap)))
    return TriangleSurface(V, T, lo, hi, {"kind": "hole", "radius": radius, "depth": depth, "cell": cell,
                                          "n_theta": n_theta, "n_wall": n_wall, "jitter": jitter, "seed": seed})


def trench_triangles(width: float = 1.0, depth: float = 5.0, cell: float = 3.0, n_wall: int = 50,
                     n_bottom: int = 20, n_top: int = 4, n_y: int = 6, source_gap: float = 0.1) -> TriangleSurface:
    """A rectangular trench along y (infinite through the periodic cell) as a
    triangle mesh, every face wound so that its normal points into the open
    space: flat top on both sides (z = 0), walls of n_wall bands in depth,
    bottom of n_bottom strips across.  Primitive order: top, left wall (bands
    from the top down), bottom (strips left to right), right wall (bands from
    the top down), n_y pieces along y in each, two triangles per quad."""
    x0 = (cell - width) / 2.0
    x1 = x0 + width
    ys = np.linspace(0.0, cell, n_y + 1)
    V, T = [], []

    def quad(p00, p10, p11, p01):  # counter-clockwise seen from the side the normal points to
        b = len(V)
        V.extend([p00, p10, p11, p01])
        T.extend([(b, b + 1, b + 2), (b, b + 2, b + 3)])

    for xa, xb in list(zip(np.linspace(0.0, x0, n_top + 1)[:-1], np.linspace(0.0, x0, n_top + 1)[1:])) + \
            list(zip(np.linspace(x1, cell, n_top + 1)[:-1], np.linspace(x1, cell, n_top + 1)[1:])):
        for ya, yb in zip(ys[:-1], ys[1:]):  # top, normal +z
            quad((xa, ya, 0.0), (xb, ya, 0.0), (xb, yb, 0.0), (xa, yb, 0.0))
    zs = np.linspace(0.0, -depth, n_wall + 1)
    for za, zb in zip(zs[:-1], zs[1:]):
        for ya, yb in zip(ys[:-1], ys[1:]):  # left wall at x0, normal +x
            quad((x0, ya, zb), (x0, yb, zb), (x0, yb, za), (x0, ya, za))
    xs = np.linspace(x0, x1, n_bottom + 1)
    for xa, xb in zip(xs[:-1], xs[1:]):
        for ya, yb in zip(ys[:-1], ys[1:]):  # bottom, normal +z
            quad((xa, ya, -depth), (xb, ya, -depth), (xb, yb, -depth), (xa, yb, -depth))
    for za, zb in zip(zs[:-1], zs[1:]):
        for ya, yb in zip(ys[:-1], ys[1:]):  # right wall at x1, normal -x
            quad((x1, ya, zb), (x1, ya, za), (x1, yb, za), (x1, yb, zb))
    V = _f32(np.array(V))
    T = np.array(T, dtype=np.uint32)
    lo = (0.0, 0.0, float(-depth))
    hi = (float(np.float32(cell)), float(np.float32(cell)), float(np.float32(source_gap)))
    return TriangleSurface(V, T, lo, hi, {"kind": "trench", "width": width, "depth": depth, "cell": cell,
                                          "n_wall": n_wall, "n_bottom": n_bottom, "n_top": n_top, "n_y": n_y})


def triangle_normals(V: np.ndarray, T: np.ndarray) -> np.ndarray:
    e1 = V[T[:, 1]].astype(np.float64) - V[T[:, 0]]
    e2 = V[T[:, 2]].astype(np.float64) - V[T[:, 0]]
    n = np.cross(e1, e2)
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def hole_discs(radius: float = 0.5, depth: float = 10.0, cell: float = 2.0, spacing: float = 0.02,
               source_gap: float = 0.1) -> DiscSurface:
    """The hole sampled with discs: a square grid on the top outside the hole,
    rings on the wall and a grid on the bottom disc; radius spacing*sqrt(2)/2."""
    half = cell / 2.0
    n = int(round(cell / spacing))
    g = -half + np.arange(n + 1) * spacing
    X, Y = np.meshgrid(g, g, indexing="ij")
    keep = np.hypot(X, Y) >= radius
    pts = [np.stack([X[keep], Y[keep], np.zeros(keep.sum())], 1)]
    nrm = [np.tile([0.0, 0.0, 1.0], (keep.sum(), 1))]
    n_th = int(round(2 * math.pi * radius / spacing))
    th = np.arange(n_th) * 2 * math.pi / n_th
    nz = int(round(depth / spacing))
    for m in range(1, nz):
        z = -m * spacing
        pts.append(np.stack([radius * np.cos(th), radius * np.sin(th), np.full(n_th, z)], 1))
        nrm.append(np.stack([-np.cos(th), -np.sin(th), np.zeros(n_th)], 1))
    inside = np.hypot(X, Y) < radius
    pts.append(np.stack([X[inside], Y[inside], np.full(inside.sum(), -nz * spacing)], 1))
    nrm.append(np.tile([0.0, 0.0, 1.0], (inside.sum(), 1)))
    P, N = _f32(np.concatenate(pts)), _f32(np.concatenate(nrm))
    R = np.full(len(P), np.float32(spacing * math.sqrt(2.0) / 2.0), dtype=np.float32)
    lo = (float(np.float32(-half)), float(np.float32(-half)), float(np.float32(-nz * spacing)))
    hi = (float(np.float32(half)), float(np.float32(half)), float(np.float32(source_gap)))
    return DiscSurface(P, N, R, lo, hi, {"kind": "hole_discs", "radius": radius, "depth": depth})


def rough_discs(n: int = 2048, spacing: float = 0.01, rms: float = 0.05, corr: float = 0.2, seed: int = 0,
                source_gap: float = 0.1) -> DiscSurface:
    """n x n discs on a periodic Gaussian random height field (Gaussian
    correlation of length `corr`, standard deviation `rms`), normals from the
    central-difference gradient, radius spacing*sqrt(2)/2."""
    rng = np.random.default_rng(seed)
    L = n * spacing
    k = np.fft.fftfreq(n, d=spacing) * 2 * math.pi
    KX, KY = np.meshgrid(k, k, indexing="ij")
    spec = np.exp(-(KX ** 2 + KY ** 2) * corr ** 2 / 8.0)
    noise = rng.standard_normal((n, n))
    h = np.real(np.fft.ifft2(np.fft.fft2(noise) * np.sqrt(spec)))
    h *= rms / h.std()
    gx = (np.roll(h, -1, 0) - np.roll(h, 1, 0)) / (2 * spacing)
    gy = (np.roll(h, -1, 1) - np.roll(h, 1, 1)) / (2 * spacing)
    nrm = np.stack([-gx, -gy, np.ones_like(h)], -1)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    g = np.arange(n) * spacing
    X, Y = np.meshgrid(g, g, indexing="ij")
    P = _f32(np.stack([X.ravel(), Y.ravel(), h.ravel()], 1))
    N = _f32(nrm.reshape(-1, 3))
    R = np.full(len(P), np.float32(spacing * math.sqrt(2.0) / 2.0), dtype=np.float32)
    lo = (float(np.float32(-spacing / 2)), float(np.float32(-spacing / 2)), float(P[:, 2].min()))
    hi = (float(np.float32(L - spacing / 2)), float(np.float32(L - spacing / 2)), float(P[:, 2].max() + source_gap))
    return DiscSurface(P, N, R, lo, hi, {"kind": "rough", "n": n, "spacing": spacing, "rms": rms, "corr": corr,
                                          "seed": seed})


def cylinder_triangles(radius: float = 0.5, depth: float = 45.0, cell: float = 1.5, n_theta: int = 128,
                       n_wall: int = 600, n_top: int = 8, n_bottom: int = 8, source_gap: float = 0.1):
    """Deep cylinder for the radiosity check (the reference's verification
    cylinder has radius 0.5 and length 45): the hole mesh without jitter."""
    return hole_triangles(radius=radius, depth=depth, cell=cell, n_theta=n_theta, n_wall=n_wall, n_top=n_top,
                          n_bottom=n_bottom, jitter=0.0, seed=0, source_gap=source_gap)


# (sticking, cosine exponent) of the three species of the batched workload
BATCH_SPECIES = ((0.01, 1.0), (0.1, 5.0), (1.0, 50.0))


def batch_instances(n: int = 64, seed: int = 0, min_discs: int = 10_000, max_discs: int = 500_000,
                    aspect: tuple = (2.0, 20.0)) -> list:
    """Ragged set of `n` disc surfaces for the batched workload: trenches and
    holes alternating, aspect ratio (depth / opening) uniform in `aspect` and a
    target disc count uniform in [min_discs, max_discs]; the grid spacing is
    chosen so that the sampled surface has about that many discs
    (trench in a 3x3 cell: N ~ 3 (3 + 2 AR) / s^2; hole of diameter 1 in a 2x2
    cell: N ~ (4 + pi AR) / s^2)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ar = float(rng.uniform(*aspect))
        target = float(rng.uniform(min_discs, max_discs))
        if i % 2 == 0:
            s = math.sqrt(3.0 * (3.0 + 2.0 * ar) / target)
            nx = max(4, int(round(3.0 / s)))
            s = 3.0 / nx
            surf = trench_discs(width=1.0, depth=ar, domain=3.0, spacing=s)
        else:
            s = math.sqrt((4.0 + math.pi * ar) / target)
            nx = max(4, int(round(2.0 / s)))
            s = 2.0 / nx
            surf = hole_discs(radius=0.5, depth=ar, cell=2.0, spacing=s)
        surf.meta.update({"aspect": ar, "target": int(target), "index": i})
        out.append(surf)
    return out
