"""Batch: many (surface, species) traces in one persistent launch.

rti traces one geometry per ``tracer::run`` (rti/trace/tracer.hpp:66-330); a
process-simulation step that needs the flux on many features for several
species calls it back to back.  ``Batch`` holds such a list of jobs and runs
them through the C ABI (``rtg_batch_*`` in include/rtg.h): one launch of the
batched path kernel over the concatenated ray ranges, optionally replayed from
a CUDA graph, or one plain launch per job (``run_sequential``) for comparison.
Job j draws its paths from the Philox stream (seed, j), so every mode gives
the same per-job results as an ``Engine.trace`` with ``job=j``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .engine import Engine, Tally, _ptr


class Batch:
    def __init__(self, device: int = 0):
        self._L = L.load()
        self._h = C.c_void_p()
        rc = self._L.rtg_batch_create(C.byref(self._h), int(device))
        if rc != L.RTG_OK:
            raise L.RtgError(rc, "rtg_batch_create failed (no usable CUDA device?)")
        self._scenes: list[Engine] = []  # keeps the contexts alive as long as the batch
        self._sizes: list[int] = []

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.rtg_batch_destroy(self._h)
            self._h = C.c_void_p()
        self._scenes = []
        self._sizes = []

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
            msg = self._L.rtg_batch_last_error(self._h)
            raise L.RtgError(rc, msg.decode() if msg else "")

    def add(self, scene: Engine, n_rays: int, seed: int = 0, config: L.RtgConfig | None = None) -> int:
        """Adds a job (the scene's current configuration unless ``config``); returns its index."""
        j = C.c_int32()
        self._check(self._L.rtg_batch_add(self._h, scene._h, None if config is None else C.byref(config),
                                          int(n_rays), int(seed), C.byref(j)))
        self._scenes.append(scene)
        self._sizes.append(scene.num_primitives)  # the job's accumulators have this size
        return j.value

    def __len__(self) -> int:
        n = C.c_int32()
        self._check(self._L.rtg_batch_num_jobs(self._h, C.byref(n)))
        return n.value

    @staticmethod
    def _stream(stream):
        if stream is None:
            return None
        return C.c_void_p(int(stream) if int(stream) != 0 else 1)  # 1 == cudaStreamLegacy

    def run(self, use_graph: bool = True, stream=None):
        """Enqueues one batched launch (from a CUDA graph when ``use_graph``)."""
        self._check(self._L.rtg_batch_run(self._h, 1 if use_graph else 0, self._stream(stream)))

    def run_sequential(self, stream=None):
        """Enqueues one plain launch per job."""
        self._check(self._L.rtg_batch_run_sequential(self._h, self._stream(stream)))

    def synchronize(self) -> float:
        """Waits for the last run and returns its device time in ms."""
        ms = C.c_double()
        self._check(self._L.rtg_batch_synchronize(self._h, C.byref(ms)))
        return ms.value

    def results(self, job: int):
        """(S1, hit counts, exposed areas) of one job."""
        n = self._sizes[job]
        s1 = np.zeros(n)
        cnt = np.zeros(n, dtype=np.uint64)
        areas = np.zeros(n, dtype=np.float32)
        self._check(self._L.rtg_batch_get_results(self._h, int(job), _ptr(s1, L._f64p), _ptr(cnt, L._u64p),
                                                  _ptr(areas, L._f32p)))
        return s1, cnt, areas

    def set_launch_config(self, threads_per_block: int = 128, packet: int = 1, stack_depth: int = 0,
                          scheduling: int = L.RTG_SCHED_MEGAKERNEL, leaf_tests: int = L.RTG_LEAF_IMMEDIATE,
                          stack_memory: int = L.RTG_STACK_AUTO):
        lc = L.RtgLaunchConfig(threads_per_block, packet, stack_depth, scheduling, leaf_tests, stack_memory)
        self._check(self._L.rtg_batch_set_launch_config(self._h, C.byref(lc)))

    def launch_config(self) -> dict:
        lc = L.RtgLaunchConfig()
        self._check(self._L.rtg_batch_get_launch_config(self._h, C.byref(lc)))
        return lc.as_dict()

    def autotune(self, sample_fraction: float = 0.05):
        """Times the candidate launch configurations of the batched launch on
        the first ``sample_fraction`` of every job's rays and keeps the fastest;
        returns (config dict, rays/s of the sample).  Run again afterwards."""
        lc = L.RtgLaunchConfig()
        r = C.c_double()
        self._check(self._L.rtg_batch_autotune(self._h, float(sample_fraction), C.byref(lc), C.byref(r)))
        return lc.as_dict(), r.value

    def tally(self) -> Tally:
        t = L.RtgTally()
        self._check(self._L.rtg_batch_get_tally(self._h, C.byref(t)))
        return Tally(t.num_rays, t.hitc, t.nonhitc, t.total, t.segments, t.truncated, t.nb_deposits, t.errors,
                     t.trace_ms, t.kernel_ms)
