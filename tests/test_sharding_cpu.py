"""Multi-rank path on CPU: gloo ranks trace disjoint ray ranges with the
oracle and sum their accumulators with rti_gb300.sharding; the result equals
one rank tracing every ray (counts and tallies bit for bit, S1..S4 to the FP64
summation order; with fixed-point S1 accumulation, S1 bit for bit too, for 2
and 3 ranks with uneven splits)."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from rti_gb300.sharding import allreduce_gradients, allreduce_results, ray_range, stack_accumulators

N_TOTAL = 6000


def _scene():
    from oracle import oracle as O
    from rti_gb300 import scenes
    t = scenes.trench_discs(domain=0.6, width=0.2, depth=0.4)
    s = O.Scene(t.xyzr, t.normals)
    s.neighbors()
    cfg = O.make_config(t.box_lo, t.box_hi, sticking=0.2, seed=9)
    return s, cfg


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, cfg = _scene()
    b, e = ray_range(rank, world, N_TOTAL, scaling="strong")
    r = s.trace(cfg, b, e, nthreads=1)
    acc = torch.from_numpy(stack_accumulators(r.s1, r.s2, r.s3, r.s4))
    cnt = torch.from_numpy(r.counts.astype(np.int64))
    tally = {"hitc": r.hitc, "nonhitc": r.nonhitc, "total": r.total, "segments": r.segments}
    allreduce_results(acc, cnt, tally)
    if rank == 0:
        np.save(os.path.join(out_dir, "acc.npy"), acc.numpy())
        np.save(os.path.join(out_dir, "cnt.npy"), cnt.numpy())
        np.save(os.path.join(out_dir, "tally.npy"), np.array([tally[k] for k in sorted(tally)]))
    dist.destroy_process_group()


def test_ray_range_partitions():
    assert [ray_range(r, 3, 10, "strong") for r in range(3)] == [(0, 4), (4, 7), (7, 10)]
    assert [ray_range(r, 2, 5, "weak") for r in range(2)] == [(0, 5), (5, 10)]
    with pytest.raises(ValueError):
        ray_range(2, 2, 5)


def test_two_gloo_ranks_equal_one_rank(tmp_path, oracle_lib):
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    s, cfg = _scene()
    ref = s.trace(cfg, 0, N_TOTAL, nthreads=1)
    acc = np.load(tmp_path / "acc.npy")
    cnt = np.load(tmp_path / "cnt.npy")
    tally = np.load(tmp_path / "tally.npy")
    assert np.array_equal(cnt, ref.counts.astype(np.int64))
    np.testing.assert_allclose(acc, stack_accumulators(ref.s1, ref.s2, ref.s3, ref.s4), rtol=1e-12)
    assert list(tally) == [ref.hitc, ref.nonhitc, ref.segments, ref.total]


def _adjoint_worker(rank, world, port, out_dir):
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, cfg = _scene()
    n = len(s.neighbors()[0]) - 1
    g = np.linspace(0.0, 1.0, n)
    field = np.linspace(0.05, 0.5, n).astype(np.float32)
    b, e = ray_range(rank, world, N_TOTAL, scaling="strong")
    ds, dn, fg, _ = O.adjoint(s, cfg, g, b, e, nthreads=1, sticking_field=field, unbiased=True)
    sc = torch.tensor([ds, dn], dtype=torch.float64)
    fgt = torch.from_numpy(np.asarray(fg, dtype=np.float64))
    allreduce_gradients(sc, fgt)
    if rank == 0:
        np.save(os.path.join(out_dir, "sc.npy"), sc.numpy())
        np.save(os.path.join(out_dir, "fg.npy"), fgt.numpy())
    dist.destroy_process_group()


def test_two_gloo_ranks_adjoint_equals_one_rank(tmp_path, oracle_lib):
    """The adjoint of the sharded trace: per-rank replays of disjoint ray ranges
    summed over two gloo ranks equal one replay of every ray."""
    import socket
    from oracle import oracle as O
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp.start_processes(_adjoint_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    s, cfg = _scene()
    n = len(s.neighbors()[0]) - 1
    g = np.linspace(0.0, 1.0, n)
    field = np.linspace(0.05, 0.5, n).astype(np.float32)
    ds, dn, fg, _ = O.adjoint(s, cfg, g, 0, N_TOTAL, nthreads=1, sticking_field=field, unbiased=True)
    sc = np.load(tmp_path / "sc.npy")
    np.testing.assert_allclose(sc, [ds, dn], rtol=1e-10)
    np.testing.assert_allclose(np.load(tmp_path / "fg.npy"), fg, rtol=1e-10, atol=1e-12 * np.abs(fg).max())


# uneven ray ranges: (world, boundaries)
FIXED_SPLITS = {2: [0, 1234, 7001], 3: [0, 100, 5000, 7001]}


def _fixed_worker(rank, world, port, out_dir):
    from oracle import oracle as O
    from rti_gb300 import scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = scenes.trench_discs(domain=0.6, width=0.2, depth=0.4)
    s = O.Scene(t.xyzr, t.normals)
    s.neighbors()
    cfg = O.make_config(t.box_lo, t.box_hi, sticking=0.2, seed=9, accum_fixed=1)
    cuts = FIXED_SPLITS[world]
    r = s.trace(cfg, cuts[rank], cuts[rank + 1], nthreads=1)
    acc = torch.from_numpy(stack_accumulators(r.s1, r.s2, r.s3, r.s4))
    cnt = torch.from_numpy(r.counts.astype(np.int64))
    allreduce_results(acc, cnt, fixed_s1=True)
    if rank == 0:
        np.save(os.path.join(out_dir, f"acc{world}.npy"), acc.numpy())
        np.save(os.path.join(out_dir, f"cnt{world}.npy"), cnt.numpy())
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_fixed_point_sharded_sum_is_bit_identical(tmp_path, oracle_lib, world):
    """RTG_ACCUM_FIXED: S1 of every rank is an integer multiple of 2^-32 and
    allreduce_results(fixed_s1=True) sums the integers, so the sharded S1 equals
    one rank's S1 bit for bit whatever the split."""
    import socket
    from oracle import oracle as O
    from rti_gb300 import scenes
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp.start_processes(_fixed_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    t = scenes.trench_discs(domain=0.6, width=0.2, depth=0.4)
    s = O.Scene(t.xyzr, t.normals)
    s.neighbors()
    ref = s.trace(O.make_config(t.box_lo, t.box_hi, sticking=0.2, seed=9, accum_fixed=1), 0, 7001, nthreads=1)
    acc = np.load(tmp_path / f"acc{world}.npy")
    n = len(ref.s1)
    assert np.array_equal(acc[:n], ref.s1)  # bit for bit
    assert np.array_equal(np.load(tmp_path / f"cnt{world}.npy"), ref.counts.astype(np.int64))
    np.testing.assert_allclose(acc[n:], np.concatenate([ref.s2, ref.s3, ref.s4]), rtol=1e-12)
    # the plain FP64 sum of the same per-rank S1 is not guaranteed to be exact;
    # the integer sum is, by construction
    from rti_gb300.sharding import s1_from_fixed, s1_to_fixed
    q = s1_to_fixed(torch.from_numpy(ref.s1))
    assert torch.equal(s1_from_fixed(q), torch.from_numpy(ref.s1))
