"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle restates the reference's flux-tracing algorithm in plain C
(``rtg_oracle.c``).  Only the tests, the smoke check and the CPU-baseline leg
of ``bench.py`` use this module; the product library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_u64p = C.POINTER(C.c_uint64)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)


class OrcConfig(C.Structure):
    _fields_ = [
        ("x_bound", C.c_int32),
        ("y_bound", C.c_int32),
        ("reflection", C.c_int32),
        ("specular_fraction", C.c_float),
        ("sticking", C.c_float),
        ("source_exponent", C.c_float),
        ("box_lo", C.c_float * 3),
        ("box_hi", C.c_float * 3),
        ("src_lo", C.c_float * 2),
        ("src_hi", C.c_float * 2),
        ("tnear", C.c_float),
        ("roulette_threshold", C.c_double),
        ("roulette_weight", C.c_double),
        ("max_segments", C.c_uint32),
        ("job", C.c_uint32),
        ("seed", C.c_uint64),
        ("sticking_field", _f32p),
        ("window", C.c_int32),
        ("window_factor", C.c_float),
        ("accum_fixed", C.c_int32),
    ]


class OrcTally(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in
                ("hitc", "nonhitc", "total", "segments", "truncated", "nb_deposits")]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(HERE, "rtg_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_scene_create.restype = C.c_void_p
        L.orc_scene_create.argtypes = [_f32p, _f32p, C.c_int64, _f32p, _u32p, C.c_int64, C.c_int64]
        L.orc_scene_destroy.argtypes = [C.c_void_p]
        L.orc_num_primitives.restype = C.c_int64
        L.orc_num_primitives.argtypes = [C.c_void_p]
        for name in ("orc_neighbors", "orc_neighbors_bruteforce"):
            f = getattr(L, name)
            f.restype = C.c_int64
            f.argtypes = [C.c_void_p, _i64p, _i32p, C.c_int64]
        L.orc_area_inside.restype = C.c_float
        L.orc_area_inside.argtypes = [C.c_float] * 4 + [_f32p, _f32p]
        L.orc_areas.argtypes = [C.c_void_p] + [C.c_float] * 4 + [_f32p]
        L.orc_local_intersect.restype = C.c_int
        L.orc_local_intersect.argtypes = [_f32p, _f32p, _f32p, _f32p]
        L.orc_closest_hit.argtypes = [C.c_void_p, _f32p, C.c_int64, C.c_float, _i32p, _f32p]
        L.orc_trace.restype = C.c_int
        L.orc_trace.argtypes = [C.c_void_p, C.POINTER(OrcConfig), C.c_uint64, C.c_uint64, C.c_int,
                                _f64p, _f64p, _f64p, _f64p, _u64p, C.POINTER(OrcTally)]
        L.orc_adjoint.restype = C.c_int
        L.orc_adjoint.argtypes = [C.c_void_p, C.POINTER(OrcConfig), C.c_uint64, C.c_uint64, C.c_int, _f64p, C.c_int,
                                  _f64p, _f64p, _u64p]
        L.orc_trace_log.restype = C.c_int64
        L.orc_trace_log.argtypes = [C.c_void_p, C.POINTER(OrcConfig), C.c_uint64, C.c_void_p, C.c_int64]
        L.orc_fd_pair.restype = C.c_int
        L.orc_fd_pair.argtypes = [C.c_void_p, C.POINTER(OrcConfig), C.c_uint64, C.c_uint64, C.c_int, _f64p,
                                  C.c_float, _f64p]
        L.orc_source_ray.argtypes = [C.POINTER(OrcConfig), C.c_uint64, _f32p, _f32p]
        L.orc_diffuse_dir.argtypes = [_f32p, C.c_uint32, C.c_uint32, _f32p]
        L.orc_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
        L.orc_sincos2pi.argtypes = [C.c_float, _f32p, _f32p]
        L.orc_powf.restype = C.c_float
        L.orc_powf.argtypes = [C.c_float, C.c_float]
        L.orc_normalize.argtypes = [C.c_int64, _f64p, _f32p, _i64p, _i32p, _f32p]
        L.orc_relative_error.argtypes = [C.c_int64, _f64p, _f64p, C.c_uint64, _f64p]
        L.orc_vov.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, _u64p, C.c_uint64, _f64p]
        _lib = L
    return _lib


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def philox4x32_10(ctr, key):
    L = lib()
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    L.orc_philox4x32_10(_p(c, _u32p), _p(k, _u32p), _p(o, _u32p))
    return o


def sincos2pi(u: float):
    s, c = C.c_float(), C.c_float()
    lib().orc_sincos2pi(C.c_float(u), C.byref(s), C.byref(c))
    return s.value, c.value


def powf(x: float, e: float) -> float:
    return lib().orc_powf(C.c_float(x), C.c_float(e))


def area_inside(box, disc, normal) -> float:
    d = np.ascontiguousarray(disc, dtype=np.float32)
    n = np.ascontiguousarray(normal, dtype=np.float32)
    return float(lib().orc_area_inside(*[C.c_float(v) for v in box], _p(d, _f32p), _p(n, _f32p)))


def local_intersect(org, dir_, disc, normal) -> bool:
    o = np.ascontiguousarray(org, dtype=np.float32)
    d = np.ascontiguousarray(dir_, dtype=np.float32)
    c = np.ascontiguousarray(disc, dtype=np.float32)
    n = np.ascontiguousarray(normal, dtype=np.float32)
    return bool(lib().orc_local_intersect(_p(o, _f32p), _p(d, _f32p), _p(c, _f32p), _p(n, _f32p)))


def source_ray(cfg: OrcConfig, ray_id: int):
    """(origin, direction) of source ray `ray_id` under cfg."""
    o = np.zeros(3, dtype=np.float32)
    d = np.zeros(3, dtype=np.float32)
    lib().orc_source_ray(C.byref(cfg), C.c_uint64(ray_id), _p(o, _f32p), _p(d, _f32p))
    return o, d


def diffuse_dir(normal, u_phi: int, u_t: int):
    n = np.ascontiguousarray(normal, dtype=np.float32)
    o = np.zeros(3, dtype=np.float32)
    lib().orc_diffuse_dir(_p(n, _f32p), C.c_uint32(u_phi), C.c_uint32(u_t), _p(o, _f32p))
    return o


@dataclass
class TraceResult:
    s1: np.ndarray
    s2: np.ndarray
    s3: np.ndarray
    s4: np.ndarray
    counts: np.ndarray
    hitc: int
    nonhitc: int
    total: int
    segments: int
    truncated: int
    nb_deposits: int


class Scene:
    """Oracle scene: discs (x, y, z, r + normal) and/or triangles."""

    def __init__(self, disc_xyzr=None, disc_normals=None, tri_vertices=None, tri_indices=None):
        L = lib()
        self.disc_xyzr = np.ascontiguousarray(
            disc_xyzr if disc_xyzr is not None else np.zeros((0, 4)), dtype=np.float32).reshape(-1, 4)
        self.disc_normals = np.ascontiguousarray(
            disc_normals if disc_normals is not None else np.zeros((0, 3)), dtype=np.float32).reshape(-1, 3)
        self.tri_vertices = np.ascontiguousarray(
            tri_vertices if tri_vertices is not None else np.zeros((0, 3)), dtype=np.float32).reshape(-1, 3)
        self.tri_indices = np.ascontiguousarray(
            tri_indices if tri_indices is not None else np.zeros((0, 3)), dtype=np.uint32).reshape(-1, 3)
        self.nd = len(self.disc_xyzr)
        self.nt = len(self.tri_indices)
        self.np = self.nd + self.nt
        self._h = L.orc_scene_create(_p(self.disc_xyzr, _f32p), _p(self.disc_normals, _f32p), self.nd,
                                     _p(self.tri_vertices, _f32p), _p(self.tri_indices, _u32p),
                                     len(self.tri_vertices), self.nt)
        self.row_ptr = None
        self.cols = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.orc_scene_destroy(self._h)
            self._h = None

    def neighbors(self, bruteforce: bool = False):
        L = lib()
        f = L.orc_neighbors_bruteforce if bruteforce else L.orc_neighbors
        rp = np.zeros(self.nd + 1, dtype=np.int64)
        nnz = f(self._h, _p(rp, _i64p), None, 0)
        cols = np.zeros(max(int(nnz), 1), dtype=np.int32)
        nnz = f(self._h, _p(rp, _i64p), _p(cols, _i32p), len(cols))
        self.row_ptr, self.cols = rp, cols[:nnz]
        return self.row_ptr, self.cols

    def areas(self, box):
        out = np.zeros(self.np, dtype=np.float32)
        lib().orc_areas(self._h, *[C.c_float(v) for v in box], _p(out, _f32p))
        return out

    def closest_hit(self, rays: np.ndarray, tnear: float = 1e-4):
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        prim = np.zeros(len(r), dtype=np.int32)
        t = np.zeros(len(r), dtype=np.float32)
        lib().orc_closest_hit(self._h, _p(r, _f32p), len(r), C.c_float(tnear), _p(prim, _i32p), _p(t, _f32p))
        return prim, t

    def trace(self, cfg: OrcConfig, ray_begin: int, ray_end: int, nthreads: int = 0,
              sticking_field: np.ndarray | None = None) -> TraceResult:
        n = self.np
        s1, s2, s3, s4 = (np.zeros(max(n, 1)) for _ in range(4))
        cnt = np.zeros(max(n, 1), dtype=np.uint64)
        tally = OrcTally()
        keep = None
        if sticking_field is not None:
            keep = np.ascontiguousarray(sticking_field, dtype=np.float32)
            cfg.sticking_field = _p(keep, _f32p)
        else:
            cfg.sticking_field = None
        lib().orc_trace(self._h, C.byref(cfg), ray_begin, ray_end, nthreads, _p(s1, _f64p), _p(s2, _f64p),
                        _p(s3, _f64p), _p(s4, _f64p), _p(cnt, _u64p), C.byref(tally))
        del keep
        return TraceResult(s1[:n], s2[:n], s3[:n], s4[:n], cnt[:n], tally.hitc, tally.nonhitc, tally.total,
                           tally.segments, tally.truncated, tally.nb_deposits)


def adjoint(scene: "Scene", cfg: OrcConfig, g, ray_begin: int, ray_end: int, nthreads: int = 0,
            sticking_field=None, unbiased: bool = False):
    """Oracle adjoint replay: returns (dL/ds, dL/dn, dL/ds_j or None, segments)."""
    gg = np.ascontiguousarray(g, dtype=np.float64)
    keep = None
    fg = None
    if sticking_field is not None:
        keep = np.ascontiguousarray(sticking_field, dtype=np.float32)
        cfg.sticking_field = _p(keep, _f32p)
        fg = np.zeros(scene.np)
    else:
        cfg.sticking_field = None
    sc = np.zeros(2)
    segs = C.c_uint64()
    rc = lib().orc_adjoint(scene._h, C.byref(cfg), ray_begin, ray_end, nthreads, _p(gg, _f64p), int(unbiased),
                           None if fg is None else _p(fg, _f64p), _p(sc, _f64p), C.byref(segs))
    cfg.sticking_field = None
    del keep
    if rc != 0:
        raise RuntimeError("orc_adjoint failed")
    return sc[0], sc[1], fg, segs.value


SEGMENT_DTYPE = [("ray", "<u8"), ("segment", "<u4"), ("kind", "<i4"), ("org", "<f4", (3,)), ("end", "<f4", (3,)),
                 ("primitive", "<i4"), ("weight", "<f4")]


def trace_log(scene: "Scene", cfg: OrcConfig, ray_id: int) -> np.ndarray:
    """Every closest-hit query of one path (orc_trace_log), in order."""
    L = lib()
    cfg.sticking_field = None
    n = L.orc_trace_log(scene._h, C.byref(cfg), ray_id, None, 0)
    out = np.zeros(n, dtype=SEGMENT_DTYPE)
    L.orc_trace_log(scene._h, C.byref(cfg), ray_id, C.c_void_p(out.ctypes.data), n)
    return out


def fd_pair(scene: "Scene", cfg: OrcConfig, g, ray_begin: int, ray_end: int, h: float, nthreads: int = 0) -> dict:
    """Central differences with common random numbers at sticking s +- h,
    decomposed by roulette decisions (orc_fd_pair): every path traced once with
    weights at s - h, s and s + h on its shared geometry."""
    gg = np.ascontiguousarray(g, dtype=np.float64)
    out = np.zeros(8)
    L = lib()
    cfg.sticking_field = None
    if L.orc_fd_pair(scene._h, C.byref(cfg), ray_begin, ray_end, nthreads, _p(gg, _f64p), h, _p(out, _f64p)) != 0:
        raise RuntimeError("orc_fd_pair failed")
    two_h = float(np.float32(cfg.sticking + np.float32(h))) - float(np.float32(cfg.sticking - np.float32(h)))
    return {"fd_all": out[0] / two_h, "fd_unflipped": out[1] / two_h, "held_all": out[2],
            "held_unflipped": out[3], "paths_flipped": int(out[4]), "decisions_flipped": int(out[5]),
            "paths_with_roulette": int(out[6]), "L": out[7], "two_h": two_h}


def make_config(box_lo, box_hi, *, x_bound=1, y_bound=1, reflection=0, specular_fraction=0.0,
                sticking=0.1, source_exponent=1.0, tnear=1e-4, max_segments=1 << 16, job=0, seed=0,
                src_lo=None, src_hi=None, window=0, window_factor=5.0, accum_fixed=0) -> OrcConfig:
    c = OrcConfig()
    c.x_bound, c.y_bound, c.reflection = x_bound, y_bound, reflection
    c.specular_fraction, c.sticking, c.source_exponent = specular_fraction, sticking, source_exponent
    for i in range(3):
        c.box_lo[i] = box_lo[i]
        c.box_hi[i] = box_hi[i]
    sl = src_lo if src_lo is not None else box_lo[:2]
    sh = src_hi if src_hi is not None else box_hi[:2]
    for i in range(2):
        c.src_lo[i] = sl[i]
        c.src_hi[i] = sh[i]
    c.tnear = tnear
    c.roulette_threshold, c.roulette_weight = 0.1, 0.3
    c.max_segments, c.job, c.seed = max_segments, job, seed
    c.sticking_field = None
    c.window, c.window_factor = window, window_factor
    c.accum_fixed = accum_fixed
    return c


def normalize(s1, areas, row_ptr, cols):
    n = len(s1)
    out = np.zeros(n, dtype=np.float32)
    s1 = np.ascontiguousarray(s1, dtype=np.float64)
    a = np.ascontiguousarray(areas, dtype=np.float32)
    rp = None if row_ptr is None else np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = None if cols is None else np.ascontiguousarray(cols, dtype=np.int32)
    lib().orc_normalize(n, _p(s1, _f64p), _p(a, _f32p), None if rp is None else _p(rp, _i64p),
                        None if cl is None else _p(cl, _i32p), _p(out, _f32p))
    return out


def relative_error(s1, s2, total):
    out = np.zeros(len(s1))
    lib().orc_relative_error(len(s1), _p(np.ascontiguousarray(s1), _f64p), _p(np.ascontiguousarray(s2), _f64p),
                             total, _p(out, _f64p))
    return out


def vov(s1, s2, s3, s4, cnt, total):
    out = np.zeros(len(s1))
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (s1, s2, s3, s4)]
    c = np.ascontiguousarray(cnt, dtype=np.uint64)
    lib().orc_vov(len(s1), *[_p(x, _f64p) for x in a], _p(c, _u64p), total, _p(out, _f64p))
    return out
