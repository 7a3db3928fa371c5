"""The multi-GPU exchange of rti_gb300.sharding on the device.

Ranks trace disjoint ray ranges and sum their accumulators in place over
torch.distributed.  Here, on one GPU: a one-rank NCCL group runs
allreduce_results on the zero-copy views of device_accumulators (the code the
bench's N > 1 step runs), and the fixed-point S1 of two ray ranges traced by
separate contexts, summed as integers the way allreduce_results(fixed_s1=True)
sums ranks, equals one context tracing every ray bit for bit.  (Ranks whose
kernels wait on one another are not run on one GPU; the 2- and 3-rank sums are
the gloo tests of test_sharding_cpu.py.)
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _worker(rank, port):
    import torch
    import torch.distributed as dist

    from rti_gb300 import Engine, scenes
    from rti_gb300 import _lib as L
    from rti_gb300.sharding import allreduce_results, device_accumulators, s1_from_fixed, s1_to_fixed
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
        n, cut = 200_000, 73_001
        engines = []
        for begin, end in ((0, cut), (cut, n), (0, n)):
            e = Engine(0)
            e.set_accumulation(L.RTG_ACCUM_FIXED)
            e.upload_discs(t.points, t.normals, t.radii)
            e.configure(box=(t.box_lo, t.box_hi), sticking=0.1, x_bound=1, y_bound=1, reset=True)
            e.trace(end - begin, seed=5, ray_begin=begin)
            engines.append(e)
        torch.cuda.synchronize()
        views = [device_accumulators(e) for e in engines]
        np_ = t.n
        for e, (acc, cnt) in zip(engines, views):  # zero-copy views = the host getters
            s = e.accumulators()
            assert np.array_equal(acc.cpu().numpy(), np.concatenate(s))
            assert np.array_equal(cnt.cpu().numpy().view(np.uint64), e.hit_counts())
        (a0, c0), (a1, c1), (aw, cw) = views
        before = a0.clone(), c0.clone()
        allreduce_results(a0, c0, {"hitc": engines[0].tally().hitc}, fixed_s1=True)  # NCCL, one rank
        torch.cuda.synchronize()
        assert torch.equal(a0, before[0]) and torch.equal(c0, before[1])
        s1 = s1_from_fixed(s1_to_fixed(a0[:np_]) + s1_to_fixed(a1[:np_]))
        assert torch.equal(s1, aw[:np_]), "integer sum of the ranges differs from the whole trace"
        assert torch.equal(c0 + c1, cw)
        for e in engines:
            e.close()
    finally:
        dist.destroy_process_group()


def test_device_views_and_nccl_exchange(rtg_lib):
    import torch.multiprocessing as mp
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp.start_processes(_worker, args=(port,), nprocs=1, join=True, start_method="spawn")
