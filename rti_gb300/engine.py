"""Engine: one GPU's flux-tracing context (a thin owner of an ``rtg_context``).

Every method calls the C ABI of librtg.so; nothing here computes flux on the
host.  Arrays are numpy (host) arrays; ``device_view()`` exposes the
device-resident accumulators for zero-copy use (e.g. torch.distributed).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(shape) if shape is not None else a


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


@dataclass
class Tally:
    num_rays: int
    hitc: int
    nonhitc: int
    total: int
    segments: int
    truncated: int
    nb_deposits: int
    errors: int
    trace_ms: float
    kernel_ms: float


class Engine:
    """Flux engine on one CUDA device (rti::device + tracer on a GB300)."""

    def __init__(self, device: int = 0):
        self._L = L.load()
        self._h = C.c_void_p()
        rc = self._L.rtg_create(C.byref(self._h), int(device))
        if rc != L.RTG_OK:
            raise L.RtgError(rc, "rtg_create failed (no usable CUDA device?)")
        self.device = device
        self.n_discs = 0
        self.n_triangles = 0

    # -- lifetime -------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.rtg_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != L.RTG_OK:
            msg = self._L.rtg_last_error(self._h)
            raise L.RtgError(rc, msg.decode() if msg else "")

    # -- geometry -------------------------------------------------------------
    def upload_discs(self, points, normals, radii):
        p = _f32(points, (-1, 3))
        n = _f32(normals, (-1, 3))
        r = _f32(radii, (-1,))
        if not (len(p) == len(n) == len(r)):
            raise ValueError("points, normals and radii must have the same length")
        self._check(self._L.rtg_upload_discs(self._h, _ptr(p, L._f32p), _ptr(n, L._f32p), _ptr(r, L._f32p), len(p)))
        self.n_discs, self.n_triangles = len(p), 0

    def upload_triangles(self, vertices, indices):
        v = _f32(vertices, (-1, 3))
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        self._check(self._L.rtg_upload_triangles(self._h, _ptr(v, L._f32p), _ptr(i, L._u32p), len(v), len(i)))
        self.n_discs, self.n_triangles = 0, len(i)

    def upload_mixed(self, points, normals, radii, vertices, indices):
        """Discs (ids 0..nd-1) and triangles (ids nd..nd+nt-1) in one surface."""
        p, n, r = _f32(points, (-1, 3)), _f32(normals, (-1, 3)), _f32(radii, (-1,))
        v = _f32(vertices, (-1, 3))
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        self._check(self._L.rtg_upload_mixed(self._h, _ptr(p, L._f32p), _ptr(n, L._f32p), _ptr(r, L._f32p), len(p),
                                             _ptr(v, L._f32p), _ptr(i, L._u32p), len(v), len(i)))
        self.n_discs, self.n_triangles = len(p), len(i)

    def update_discs(self, points, normals, radii):
        p, n, r = _f32(points, (-1, 3)), _f32(normals, (-1, 3)), _f32(radii, (-1,))
        self._check(self._L.rtg_update_discs(self._h, _ptr(p, L._f32p), _ptr(n, L._f32p), _ptr(r, L._f32p), len(p)))

    def update_vertices(self, vertices):
        v = _f32(vertices, (-1, 3))
        self._check(self._L.rtg_update_vertices(self._h, _ptr(v, L._f32p), len(v)))

    @property
    def num_primitives(self) -> int:
        n = C.c_int64()
        self._check(self._L.rtg_num_primitives(self._h, C.byref(n)))
        return n.value

    # -- configuration --------------------------------------------------------
    def configure(self, *, x_bound=None, y_bound=None, reflection=None, specular_fraction=None, sticking=None,
                  source_exponent=None, box=None, tnear=None, roulette_threshold=None, roulette_weight=None,
                  max_segments=None, job=None, reset=False):
        """Updates the trace configuration (starting from rti's defaults when
        ``reset``); ``box`` = ((xlo, ylo, zlo), (xhi, yhi, zhi)), else the box
        stays as configured (rti's rule by default)."""
        c = L.RtgConfig()
        if reset:
            self._L.rtg_config_default(C.byref(c))
        else:
            self._check(self._L.rtg_get_config(self._h, C.byref(c)))
        for name, val in (("x_bound", x_bound), ("y_bound", y_bound), ("reflection", reflection),
                          ("specular_fraction", specular_fraction), ("sticking", sticking),
                          ("source_exponent", source_exponent), ("tnear", tnear),
                          ("roulette_threshold", roulette_threshold), ("roulette_weight", roulette_weight),
                          ("max_segments", max_segments), ("job", job)):
            if val is not None:
                setattr(c, name, val)
        if box is not None:
            c.box_mode = L.RTG_BOX_EXPLICIT
            for a in range(3):
                c.box_lo[a] = box[0][a]
                c.box_hi[a] = box[1][a]
        self._check(self._L.rtg_set_config(self._h, C.byref(c)))
        return self

    def config(self) -> L.RtgConfig:
        c = L.RtgConfig()
        self._check(self._L.rtg_get_config(self._h, C.byref(c)))
        return c

    def box(self):
        lo = np.zeros(3, dtype=np.float32)
        hi = np.zeros(3, dtype=np.float32)
        self._check(self._L.rtg_get_box(self._h, _ptr(lo, L._f32p), _ptr(hi, L._f32p)))
        return lo, hi

    def set_sticking_field(self, field):
        if field is None:
            self._check(self._L.rtg_set_sticking_field(self._h, None, 0))
            return
        f = _f32(field, (-1,))
        self._check(self._L.rtg_set_sticking_field(self._h, _ptr(f, L._f32p), len(f)))

    # -- scheduling -----------------------------------------------------------
    def launch_config(self) -> L.RtgLaunchConfig:
        lc = L.RtgLaunchConfig()
        self._check(self._L.rtg_get_launch_config(self._h, C.byref(lc)))
        return lc

    def set_launch_config(self, threads_per_block: int = 128, packet: int = 1, stack_depth: int = 0,
                          scheduling: int = L.RTG_SCHED_MEGAKERNEL, leaf_tests: int = L.RTG_LEAF_IMMEDIATE,
                          stack_memory: int = L.RTG_STACK_AUTO):
        lc = L.RtgLaunchConfig(threads_per_block, packet, stack_depth, scheduling, leaf_tests, stack_memory)
        self._check(self._L.rtg_set_launch_config(self._h, C.byref(lc)))

    @property
    def tree_depth(self) -> int:
        d = C.c_int32()
        self._check(self._L.rtg_get_tree_depth(self._h, C.byref(d)))
        return d.value

    @property
    def tree_builder(self) -> int:
        b = C.c_int32()
        self._check(self._L.rtg_get_tree_builder(self._h, C.byref(b)))
        return b.value

    def set_tree_builder(self, builder: int):
        """L.RTG_TREE_KARRAS (fast build) or L.RTG_TREE_PLOC (clustering); rebuilds the current tree."""
        self._check(self._L.rtg_set_tree_builder(self._h, int(builder)))

    @property
    def node_width(self) -> int:
        w = C.c_int32()
        self._check(self._L.rtg_get_node_width(self._h, C.byref(w)))
        return w.value

    # -- segment log (rti's RAYLOG / RAYSRCLOG) -------------------------------
    def set_segment_log(self, ray_begin: int, ray_end: int, capacity: int):
        """Record every closest-hit query of the source rays [ray_begin, ray_end)
        of later traces, up to `capacity` records; capacity 0 stops logging."""
        self._check(self._L.rtg_set_segment_log(self._h, int(ray_begin), int(ray_end), int(capacity)))

    def segment_log(self):
        """(records, dropped): a numpy structured array (L.SEGMENT_DTYPE) sorted by
        (ray, segment), and the number of records that did not fit."""
        kept, dropped = C.c_uint64(), C.c_uint64()
        self._check(self._L.rtg_get_segment_log(self._h, None, 0, C.byref(kept), C.byref(dropped)))
        out = np.zeros(kept.value, dtype=L.SEGMENT_DTYPE)
        assert out.dtype.itemsize == C.sizeof(L.RtgSegment)
        self._check(self._L.rtg_get_segment_log(self._h, C.c_void_p(out.ctypes.data), kept.value, C.byref(kept),
                                                C.byref(dropped)))
        return out[:kept.value], dropped.value

    def write_segment_log(self, path: str):
        """The segment log as VTK XML PolyData (one line cell per segment)."""
        self._check(self._L.rtg_write_segment_log_vtp(self._h, str(path).encode()))

    @property
    def uses_wide_tree(self) -> bool:
        """Whether the closest-hit queries of the next trace traverse the 8-wide tree."""
        w = C.c_int32()
        self._check(self._L.rtg_get_traversal_width(self._h, C.byref(w)))
        return w.value == L.RTG_NODES_WIDE

    def set_node_width(self, width: int):
        """L.RTG_NODES_AUTO (default: wide when the tree outgrows L2), L.RTG_NODES_BINARY
        or L.RTG_NODES_WIDE (the compressed 8-wide tree); results do not depend on it."""
        self._check(self._L.rtg_set_node_width(self._h, int(width)))

    @property
    def deposit_mode(self):
        """(mode, window_factor): L.RTG_DEPOSIT_NEIGHBORS (rti's tracer) or
        L.RTG_DEPOSIT_WINDOW (rti's multi-hit window of window_factor radii)."""
        m, f = C.c_int32(), C.c_float()
        self._check(self._L.rtg_get_deposit_mode(self._h, C.byref(m), C.byref(f)))
        return m.value, f.value

    @property
    def accumulation(self) -> int:
        """L.RTG_ACCUM_FP64 or L.RTG_ACCUM_FIXED (order-independent, bit-reproducible S1)."""
        m = C.c_int32()
        self._check(self._L.rtg_get_accumulation(self._h, C.byref(m)))
        return m.value

    def set_accumulation(self, mode: int):
        self._check(self._L.rtg_set_accumulation(self._h, int(mode)))

    @property
    def visit_limit(self) -> int:
        """Node visits per closest-hit query before it ends as an error (0: automatic)."""
        v = C.c_uint64()
        self._check(self._L.rtg_get_visit_limit(self._h, C.byref(v)))
        return v.value

    def set_visit_limit(self, visits: int):
        self._check(self._L.rtg_set_visit_limit(self._h, int(visits)))

    def inject_alloc_failure(self, after: int):
        """Test hook: the device allocation after ``after`` more successful ones
        fails as if the device were out of memory (once); negative cancels."""
        self._check(self._L.rtg_inject_alloc_failure(self._h, int(after)))

    def set_deposit_mode(self, mode: int, window_factor: float = 5.0):
        """Selects the deposit of a front-face disc hit for later traces."""
        self._check(self._L.rtg_set_deposit_mode(self._h, int(mode), float(window_factor)))

    def autotune(self, sample_rays: int, seed: int = 0):
        """Times the candidate launch configurations on a sample trace and keeps
        the fastest; returns (config dict, rays/s of the sample)."""
        lc = L.RtgLaunchConfig()
        r = C.c_double()
        self._check(self._L.rtg_autotune(self._h, int(sample_rays), int(seed), C.byref(lc), C.byref(r)))
        return lc.as_dict(), r.value

    # -- tracing --------------------------------------------------------------
    def trace(self, n_rays: int, seed: int = 0, stream=None, *, ray_begin: int = 0, accumulate: bool = False):
        """Enqueues source rays [ray_begin, ray_begin + n_rays); returns immediately.

        stream: a cudaStream_t handle as an int (e.g. torch.cuda.Stream().cuda_stream);
        0 is the legacy default stream (torch's default), None the context's own stream."""
        if stream is None:
            s = None
        else:
            s = C.c_void_p(int(stream) if int(stream) != 0 else 1)  # 1 == cudaStreamLegacy
        self._check(self._L.rtg_trace_range(self._h, int(ray_begin), int(ray_begin + n_rays), int(seed),
                                            1 if accumulate else 0, s))

    def synchronize(self):
        self._check(self._L.rtg_synchronize(self._h))

    def request_abort(self):
        self._check(self._L.rtg_request_abort(self._h))

    def trace_rays(self, rays, tnear: float = 1e-4):
        r = _f32(rays, (-1, 6))
        prim = np.zeros(len(r), dtype=np.int32)
        t = np.zeros(len(r), dtype=np.float32)
        self._check(self._L.rtg_trace_rays(self._h, _ptr(r, L._f32p), len(r), float(tnear), _ptr(prim, L._i32p),
                                           _ptr(t, L._f32p)))
        return prim, t

    def set_sticking_field_device(self, d_field: int, n: int, stream=None):
        """Sticking field from a float32 device array at address d_field (None/0 clears)."""
        s = None if stream is None else C.c_void_p(int(stream) if int(stream) != 0 else 1)
        self._check(self._L.rtg_set_sticking_field_device(self._h, C.c_void_p(int(d_field or 0)) if d_field else None,
                                                          int(n), s))

    # -- adjoint ----------------------------------------------------------------
    def adjoint(self, g, n_rays: int, seed: int = 0, unbiased: bool = True):
        """dL/ds, dL/dn and (with a sticking field) dL/ds_j for L = sum_i g_i S1_i,
        by replaying rays [0, n_rays) of the trace with `seed` (host arrays)."""
        gg = np.ascontiguousarray(g, dtype=np.float64)
        if len(gg) != self.num_primitives:
            raise ValueError("g must have one entry per primitive")
        field = np.zeros(len(gg))
        ds, dn = C.c_double(), C.c_double()
        est = L.RTG_ADJ_UNBIASED if unbiased else L.RTG_ADJ_HELD
        self._check(self._L.rtg_adjoint_host(self._h, _ptr(gg, L._f64p), int(n_rays), int(seed), est,
                                             _ptr(field, L._f64p), C.byref(ds), C.byref(dn)))
        return ds.value, dn.value, field

    def adjoint_device(self, d_g: int, ray_begin: int, ray_end: int, seed: int, d_field_grad: int, d_scalars: int,
                       unbiased: bool = True, stream=None):
        """rtg_adjoint on device arrays (addresses); adds into d_field_grad / d_scalars."""
        s = None if stream is None else C.c_void_p(int(stream) if int(stream) != 0 else 1)
        est = L.RTG_ADJ_UNBIASED if unbiased else L.RTG_ADJ_HELD
        self._check(self._L.rtg_adjoint(self._h, C.c_void_p(int(d_g)), int(ray_begin), int(ray_end), int(seed), est,
                                        C.c_void_p(int(d_field_grad)) if d_field_grad else None,
                                        C.c_void_p(int(d_scalars)), s))

    # -- results --------------------------------------------------------------
    def mc_estimates(self) -> np.ndarray:
        out = np.zeros(self.num_primitives, dtype=np.float32)
        self._check(self._L.rtg_get_mc_estimates(self._h, _ptr(out, L._f32p)))
        return out

    def mc_estimates_noalloc(self, d_out: int, stream=None):
        """Writes the normalised estimates into the caller's device buffer at
        address d_out (float32 per primitive) without allocating device memory;
        enqueued on `stream` (int handle) or the context's stream."""
        s = None if stream is None else C.c_void_p(int(stream) if int(stream) != 0 else 1)
        self._check(self._L.rtg_get_mc_estimates_noalloc(self._h, C.c_void_p(int(d_out)), s))

    def _out(self, out, dtype):
        """A result array: the caller's (e.g. pinned host memory) after a shape/type check, or a new one."""
        n = self.num_primitives
        if out is None:
            return np.zeros(n, dtype=dtype)
        if out.dtype != dtype or out.shape != (n,) or not out.flags.c_contiguous:
            raise ValueError(f"out must be a contiguous {np.dtype(dtype).name} array of {n} elements")
        return out

    def hit_counts(self, out: np.ndarray | None = None) -> np.ndarray:
        out = self._out(out, np.uint64)
        self._check(self._L.rtg_get_hit_counts(self._h, _ptr(out, L._u64p)))
        return out

    def accumulators(self):
        n = self.num_primitives
        s = [np.zeros(n) for _ in range(4)]
        self._check(self._L.rtg_get_accumulators(self._h, *[_ptr(x, L._f64p) for x in s]))
        return s

    def values(self, out: np.ndarray | None = None) -> np.ndarray:
        """S1 (the flux per primitive, hit_accumulator::get_values) alone."""
        out = self._out(out, np.float64)
        self._check(self._L.rtg_get_accumulators(self._h, _ptr(out, L._f64p), None, None, None))
        return out

    def exposed_areas(self) -> np.ndarray:
        out = np.zeros(self.num_primitives, dtype=np.float32)
        self._check(self._L.rtg_get_exposed_areas(self._h, _ptr(out, L._f32p)))
        return out

    def relative_error(self) -> np.ndarray:
        out = np.zeros(self.num_primitives)
        self._check(self._L.rtg_get_relative_error(self._h, _ptr(out, L._f64p)))
        return out

    def vov(self) -> np.ndarray:
        out = np.zeros(self.num_primitives)
        self._check(self._L.rtg_get_vov(self._h, _ptr(out, L._f64p)))
        return out

    def checkpoint(self) -> dict:
        """The state of the trace so far (S1..S4, hit counts, tally): with
        resume() on a context holding the same surface and configuration, a
        trace of the remaining rays (trace(..., ray_begin=k, accumulate=True))
        continues it as if it had not stopped."""
        s1, s2, s3, s4 = self.accumulators()
        t = self.tally()
        return {"s1": s1, "s2": s2, "s3": s3, "s4": s4, "counts": self.hit_counts().copy(),
                "tally": {f: getattr(t, f) for f in ("num_rays", "hitc", "nonhitc", "total", "segments",
                                                     "truncated", "nb_deposits", "errors")}}

    def resume(self, state: dict):
        """Puts a checkpoint() back (rtg_set_accumulators)."""
        n = self.num_primitives
        arrs = [np.ascontiguousarray(state[k], dtype=np.float64) for k in ("s1", "s2", "s3", "s4")]
        cnt = np.ascontiguousarray(state["counts"], dtype=np.uint64)
        if any(a.shape != (n,) for a in arrs) or cnt.shape != (n,):
            raise ValueError(f"checkpoint arrays must hold {n} values")
        t = L.RtgTally()
        for f, v in state["tally"].items():
            setattr(t, f, int(v))
        self._check(self._L.rtg_set_accumulators(self._h, *[_ptr(a, L._f64p) for a in arrs], _ptr(cnt, L._u64p),
                                                 C.byref(t)))

    def tally(self) -> Tally:
        t = L.RtgTally()
        self._check(self._L.rtg_get_tally(self._h, C.byref(t)))
        return Tally(t.num_rays, t.hitc, t.nonhitc, t.total, t.segments, t.truncated, t.nb_deposits, t.errors,
                     t.trace_ms, t.kernel_ms)

    def neighbors(self):
        nnz = C.c_int64()
        self._check(self._L.rtg_get_neighbors(self._h, None, None, 0, C.byref(nnz)))
        rp = np.zeros(self.n_discs + 1, dtype=np.int64)
        cols = np.zeros(max(nnz.value, 1), dtype=np.int32)
        self._check(self._L.rtg_get_neighbors(self._h, _ptr(rp, L._i64p), _ptr(cols, L._i32p), len(cols),
                                              C.byref(nnz)))
        return rp, cols[:nnz.value]

    def device_view(self) -> L.RtgDeviceView:
        v = L.RtgDeviceView()
        self._check(self._L.rtg_get_device_view(self._h, C.byref(v)))
        return v


def device_run(points, normals, radii, *, n_rays: int, seed: int = 0, config: L.RtgConfig | None = None,
               sticking_field=None, device: int = 0):
    """rti::device::run in one C call: host arrays in, (estimates, hit counts) out."""
    lib = L.load()
    p, n, r = _f32(points, (-1, 3)), _f32(normals, (-1, 3)), _f32(radii, (-1,))
    est = np.zeros(len(p), dtype=np.float32)
    cnt = np.zeros(len(p), dtype=np.uint64)
    sf = None if sticking_field is None else _f32(sticking_field, (-1,))
    rc = lib.rtg_device_run(_ptr(p, L._f32p), _ptr(n, L._f32p), _ptr(r, L._f32p), len(p),
                            None if config is None else C.byref(config),
                            None if sf is None else _ptr(sf, L._f32p), int(n_rays), int(seed),
                            _ptr(est, L._f32p), _ptr(cnt, L._u64p), int(device))
    if rc != L.RTG_OK:
        raise L.RtgError(rc, "rtg_device_run failed")
    return est, cnt
