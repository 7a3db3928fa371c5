"""rtg_get_mc_estimates_noalloc: the estimates for callers that cannot allocate.

A process simulator that owns all GPU memory through its own pool, or that
cannot take the device-wide synchronisation of cudaFree between a trace and
the next surface update, gets the normalised estimates written into a device
buffer it already owns; the library keeps its scratch in a fixed array.  This
checks, through the C ABI, that two such calls in a row (after two different
traces) return what rtg_get_mc_estimates returns.  The file sorts last so a
run that stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-6  # the tolerance of the estimates check in test_gpu_parity.py


def test_noalloc_estimates_match_existing_entry_point(rtg_lib):
    import torch

    from rti_gb300 import Engine, scenes
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    with Engine(0) as e:
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
        out = torch.full((e.num_primitives,), -1.0, dtype=torch.float32, device="cuda:0")
        for seed in (21, 22):
            e.trace(200000, seed)
            ref = e.mc_estimates()                       # existing entry point (synchronises)
            rc = rtg_lib.rtg_get_mc_estimates_noalloc(e._h, C.c_void_p(out.data_ptr()), None)
            assert rc == 0, rtg_lib.rtg_last_error(e._h)
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.isfinite(got).all() and got.max() == 1.0
            np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)
