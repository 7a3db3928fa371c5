"""VTK XML files through librtg (rti's io layer without VTK).

write_vtp(engine, path, metadata)           -- rti io/vtp_writer.hpp: results of a trace
write_vtp_discs / write_vtp_triangles(...)  -- the same from host arrays
read_point_cloud(path) -> (points, normals, radii)   -- io/vtp_point_cloud_reader.hpp
read_triangles(path) -> (vertices, indices)           -- io/vtp_triangle_reader.hpp
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L


def _meta(metadata):
    items = list((metadata or {}).items())
    keys = (C.c_char_p * max(len(items), 1))(*[str(k).encode() for k, _ in items])
    vals = (C.c_char_p * max(len(items), 1))(*[str(v).encode() for _, v in items])
    return keys, vals, len(items)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def _arr(a, dtype, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=dtype)
    return a.reshape(shape) if shape is not None else a


def _check(rc: int, what: str):
    if rc != L.RTG_OK:
        raise L.RtgError(rc, what)


def write_vtp(engine, path: str, metadata: dict | None = None):
    keys, vals, n = _meta(metadata)
    rc = engine._L.rtg_write_vtp(engine._h, os.fsencode(path), keys, vals, n)
    if rc != L.RTG_OK:
        msg = engine._L.rtg_last_error(engine._h)
        raise L.RtgError(rc, msg.decode() if msg else "write_vtp failed")


def _results(value, hitcnt, area, relerr, vov):
    return (_arr(value, np.float64), _arr(hitcnt, np.uint64), _arr(area, np.float32), _arr(relerr, np.float64),
            _arr(vov, np.float64))


def write_vtp_discs(path: str, points, normals, radii, *, value=None, hitcnt=None, exposed_area=None,
                    relative_error=None, vov=None, metadata: dict | None = None):
    lib = L.load()
    p, n, r = _arr(points, np.float32, (-1, 3)), _arr(normals, np.float32, (-1, 3)), _arr(radii, np.float32)
    v, c, a, e, w = _results(value, hitcnt, exposed_area, relative_error, vov)
    keys, vals, m = _meta(metadata)
    _check(lib.rtg_write_vtp_discs(os.fsencode(path), len(p), _p(p, L._f32p), _p(n, L._f32p), _p(r, L._f32p),
                                   _p(v, L._f64p), _p(c, L._u64p), _p(a, L._f32p), _p(e, L._f64p), _p(w, L._f64p),
                                   keys, vals, m), f"cannot write {path}")


def write_vtp_triangles(path: str, vertices, indices, *, value=None, hitcnt=None, exposed_area=None,
                        relative_error=None, vov=None, metadata: dict | None = None):
    lib = L.load()
    vx, ix = _arr(vertices, np.float32, (-1, 3)), _arr(indices, np.uint32, (-1, 3))
    v, c, a, e, w = _results(value, hitcnt, exposed_area, relative_error, vov)
    keys, vals, m = _meta(metadata)
    _check(lib.rtg_write_vtp_triangles(os.fsencode(path), len(vx), _p(vx, L._f32p), len(ix), _p(ix, L._u32p),
                                       _p(v, L._f64p), _p(c, L._u64p), _p(a, L._f32p), _p(e, L._f64p),
                                       _p(w, L._f64p), keys, vals, m), f"cannot write {path}")


def read_point_cloud(path: str):
    """(points (n,3), unit normals (n,3), radii (n,)) as float32."""
    lib = L.load()
    err = C.create_string_buffer(512)
    n = C.c_int64(0)
    _check_read(lib.rtg_read_point_cloud(os.fsencode(path), C.byref(n), None, None, None, err, 512), err)
    pts = np.zeros((n.value, 3), np.float32)
    nrm = np.zeros((n.value, 3), np.float32)
    rad = np.zeros(n.value, np.float32)
    _check_read(lib.rtg_read_point_cloud(os.fsencode(path), C.byref(n), _p(pts, L._f32p), _p(nrm, L._f32p),
                                         _p(rad, L._f32p), err, 512), err)
    return pts, nrm, rad


def read_triangles(path: str):
    """(vertices (nv,3) float32, indices (nt,3) uint32)."""
    lib = L.load()
    err = C.create_string_buffer(512)
    nv, nt = C.c_int64(0), C.c_int64(0)
    _check_read(lib.rtg_read_triangles(os.fsencode(path), C.byref(nv), None, C.byref(nt), None, err, 512), err)
    vx = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros((nt.value, 3), np.uint32)
    _check_read(lib.rtg_read_triangles(os.fsencode(path), C.byref(nv), _p(vx, L._f32p), C.byref(nt),
                                       _p(ix, L._u32p), err, 512), err)
    return vx, ix


def read_point_cloud_vtu(path: str, flavor: int = L.RTG_VTU_AREA):
    """rti's special-purpose VTU point readers: L.RTG_VTU_AREA
    (io/christoph: radius from area_around_vertex, z inverted) or
    L.RTG_VTU_SPACING (io/xaver: radius from gridSpacing).  Returns the kept
    (points, unit normals, radii) as float32."""
    lib = L.load()
    err = C.create_string_buffer(512)
    n = C.c_int64(0)
    _check_read(lib.rtg_read_point_cloud_vtu(os.fsencode(path), int(flavor), C.byref(n), None, None, None, err, 512),
                err)
    pts = np.zeros((n.value, 3), np.float32)
    nrm = np.zeros((n.value, 3), np.float32)
    rad = np.zeros(n.value, np.float32)
    _check_read(lib.rtg_read_point_cloud_vtu(os.fsencode(path), int(flavor), C.byref(n), _p(pts, L._f32p),
                                             _p(nrm, L._f32p), _p(rad, L._f32p), err, 512), err)
    return pts, nrm, rad


def read_triangles_vtu(path: str):
    """rti's io/christoph VTU mesh reader: (vertices (nv,3), indices (nt,3) with
    each cell's second and third vertex swapped, per-triangle mean vertex
    normals (nt,3))."""
    lib = L.load()
    err = C.create_string_buffer(512)
    nv, nt = C.c_int64(0), C.c_int64(0)
    _check_read(lib.rtg_read_triangles_vtu(os.fsencode(path), C.byref(nv), None, C.byref(nt), None, None, err, 512),
                err)
    vx = np.zeros((nv.value, 3), np.float32)
    ix = np.zeros((nt.value, 3), np.uint32)
    nx = np.zeros((nt.value, 3), np.float32)
    _check_read(lib.rtg_read_triangles_vtu(os.fsencode(path), C.byref(nv), _p(vx, L._f32p), C.byref(nt),
                                           _p(ix, L._u32p), _p(nx, L._f32p), err, 512), err)
    return vx, ix, nx


def _check_read(rc: int, err):
    if rc != L.RTG_OK:
        raise L.RtgError(rc, err.value.decode(errors="replace"))
