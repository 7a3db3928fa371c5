"""Ray-range sharding across ranks and the one exchange step of the path.

Source rays are independent (Philox counters are indexed by the global ray
id), so ranks trace disjoint ranges of ray ids against full replicas of the
surface; the only exchange is the sum of the per-primitive accumulators
(S1..S4, counts) and of the tallies, which reproduces tracer.hpp's OpenMP
reduction of per-thread hit_accumulators (hit_accumulator.hpp:47-80) across
processes -- and, for the adjoint, the sum of the gradients.  On GPUs the accumulators are viewed in place (no copy) and summed
with NCCL; the same functions run on CPU tensors with gloo.
"""
from __future__ import annotations

import numpy as np


def ray_range(rank: int, world: int, n_rays: int, scaling: str = "weak") -> tuple[int, int]:
    """Global ray ids [begin, end) of `rank`.  weak: every rank traces n_rays;
    strong: n_rays are split as evenly as possible."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    if scaling == "weak":
        return rank * n_rays, (rank + 1) * n_rays
    if scaling == "strong":
        base, rem = divmod(n_rays, world)
        b = rank * base + min(rank, rem)
        return b, b + base + (1 if rank < rem else 0)
    raise ValueError("scaling must be 'weak' or 'strong'")


class _CudaArray:
    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False), "version": 3}


def device_accumulators(engine):
    """torch views of an Engine's device accumulators: (S1..S4 as one float64
    tensor of 4n, counts as int64 of n).  Valid until the geometry changes."""
    import torch
    v = engine.device_view()
    dev = torch.device("cuda", engine.device)
    acc = torch.as_tensor(_CudaArray(v.s1, 4 * v.n, "<f8"), device=dev)
    cnt = torch.as_tensor(_CudaArray(v.counts, v.n, "<i8"), device=dev)
    return acc, cnt


FIXED_SCALE = 4294967296.0  # RTG_ACCUM_FIXED: S1 holds integer multiples of 2^-32


def s1_to_fixed(s1):
    """The int64 multiples of 2^-32 behind an RTG_ACCUM_FIXED S1 (a float64
    tensor).  Exact while |S1| < 2^21 on every primitive (the integer fits the
    53-bit mantissa of the double that carries it)."""
    import torch
    return torch.round(s1 * FIXED_SCALE).to(torch.int64)


def s1_from_fixed(q):
    """float64 S1 from int64 multiples of 2^-32, rounded as the library
    rounds them at the end of a trace: (double)q * 2^-32."""
    import torch
    return q.to(torch.float64) * (1.0 / FIXED_SCALE)


def allreduce_results(acc, cnt, tally: dict | None = None, group=None, fixed_s1: bool = False):
    """Sums accumulators, counts and integer tallies over all ranks in place.

    fixed_s1: the ranks traced with RTG_ACCUM_FIXED; S1 (the first n entries
    of acc) is then summed as int64 multiples of 2^-32, so the sum does not
    depend on the order of the ranks and equals, bit for bit, one rank that
    traced every ray (while every rank's |S1| < 2^21 per primitive).  S2..S4
    are FP64 sums either way."""
    import torch
    import torch.distributed as dist
    if fixed_s1:
        n = cnt.numel()
        q = s1_to_fixed(acc[:n])
        dist.all_reduce(q, group=group)
        dist.all_reduce(acc[n:], group=group)
        acc[:n] = s1_from_fixed(q)
    else:
        dist.all_reduce(acc, group=group)
    dist.all_reduce(cnt, group=group)
    if tally is not None:
        keys = sorted(tally)
        t = torch.tensor([int(tally[k]) for k in keys], dtype=torch.int64, device=acc.device)
        dist.all_reduce(t, group=group)
        for k, v in zip(keys, t.tolist()):
            tally[k] = v
    return acc, cnt, tally


def allreduce_gradients(scalars, field_grad=None, group=None):
    """Sums the adjoint's outputs over ranks in place: scalars = [dL/ds, dL/dn]
    and, with a sticking field, dL/ds_j.  The replay of each rank's ray range
    adds to its own buffers (rtg_adjoint accumulates), so the sum over ranks is
    the gradient of the whole trace."""
    import torch.distributed as dist
    dist.all_reduce(scalars, group=group)
    if field_grad is not None:
        dist.all_reduce(field_grad, group=group)
    return scalars, field_grad


def stack_accumulators(s1, s2, s3, s4) -> np.ndarray:
    return np.concatenate([np.asarray(s1), np.asarray(s2), np.asarray(s3), np.asarray(s4)])
