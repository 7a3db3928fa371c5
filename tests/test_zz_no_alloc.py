"""rtg_get_mc_estimates_noalloc: the estimates for callers that cannot allocate.

A process simulator that owns all GPU memory through its own pool, or that
cannot take the device-wide synchronisation of cudaFree between a trace and
the next surface update, gets the normalised estimates written into a device
buffer it already owns; the library keeps its scratch in a fixed array.  These
tests call it through the C ABI and check, on two calls in a row (after two
different traces), that it returns what rtg_get_mc_estimates returns: on a disc
surface, a triangle surface and a mixed one, each time enqueued on a stream
other than the trace's straight after the trace (no host synchronisation in
between: the entry point must order itself after the trace); and that a
surface above its fixed limit is refused.  The file sorts last so a run that
stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
RTOL = 1e-6  # the tolerance of the estimates check in test_gpu_parity.py
MAX_PRIMITIVES = 8_388_352  # the entry point's documented limit


def _surfaces():
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    h = scenes.hole_triangles(n_theta=64, n_wall=24, n_top=6, n_bottom=4, depth=2.0, cell=1.2)
    quad = np.float32([[-0.6, -0.6, -0.55], [0.6, -0.6, -0.55], [0.6, 0.6, -0.55], [-0.6, 0.6, -0.55]])
    return {
        "discs": (lambda e: e.upload_discs(t.points, t.normals, t.radii), (t.box_lo, t.box_hi), 0.1),
        "triangles": (lambda e: e.upload_triangles(h.vertices, h.indices), (h.box_lo, h.box_hi), 0.05),
        # two triangles across the trench at half depth take flux beside the discs
        "mixed": (lambda e: e.upload_mixed(t.points, t.normals, t.radii, quad, np.uint32([[0, 1, 2], [0, 2, 3]])),
                  (t.box_lo, t.box_hi), 0.2),
    }


@pytest.mark.parametrize("kind", ["discs", "triangles", "mixed"])
def test_noalloc_estimates_match_existing_entry_point(rtg_lib, kind):
    import torch

    from rti_gb300 import Engine
    upload, box, sticking = _surfaces()[kind]
    dev = torch.device("cuda", 0)
    trace_stream = torch.cuda.Stream(dev)
    est_stream = torch.cuda.Stream(dev)
    with Engine(0) as e:
        upload(e)
        e.configure(box=box, sticking=sticking, x_bound=1, y_bound=1, reset=True)
        out = torch.full((e.num_primitives,), -1.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        for seed in (21, 22):
            e.trace(300000, seed, stream=trace_stream.cuda_stream)
            # no synchronisation: the entry point orders itself after the trace
            rc = rtg_lib.rtg_get_mc_estimates_noalloc(e._h, C.c_void_p(out.data_ptr()),
                                                     C.c_void_p(est_stream.cuda_stream))
            assert rc == 0, rtg_lib.rtg_last_error(e._h)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            ref = e.mc_estimates()  # the existing entry point
            assert np.isfinite(got).all() and got.max() == 1.0
            np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)


def test_noalloc_refuses_surfaces_above_its_limit(rtg_lib):
    """One primitive more than the fixed scratch covers: a clear error, and the
    existing entry point still serves the same context."""
    from rti_gb300 import Engine, RtgError
    from rti_gb300 import _lib as L
    side = 2897  # 2897^2 = 8,392,609 discs
    assert side * side > MAX_PRIMITIVES
    g = (np.arange(side, dtype=np.float64) + 0.5) / side
    X, Y = np.meshgrid(g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], 1).astype(np.float32)
    nrm = np.tile(np.float32([0, 0, 1]), (len(p), 1))
    r = np.full(len(p), np.float32(0.3 / side), np.float32)  # no two discs overlap
    with Engine(0) as e:
        e.upload_discs(p, nrm, r)
        e.configure(box=((0, 0, -0.1), (1, 1, 0.1)), sticking=1.0, x_bound=1, y_bound=1, reset=True)
        e.trace(10000, 1)
        import torch
        out = torch.empty(len(p), dtype=torch.float32, device="cuda:0")
        with pytest.raises(RtgError) as ei:
            e.mc_estimates_noalloc(out.data_ptr())
        assert ei.value.code == L.RTG_ERR_INVALID_ARGUMENT
        assert "8388352" in str(ei.value)
        assert e.mc_estimates().shape == (len(p),)
