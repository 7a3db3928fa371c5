"""Differentiable flux: a torch.autograd.Function over librtg's trace and adjoint.

    s1 = flux(engine, sticking, exponent, n_rays, seed)        # float64 (N,), on the GPU
    loss = (weights * s1).sum(); loss.backward()               # d/d sticking, d/d exponent

`sticking` is a 0-d tensor (one global sticking) or an (N,) tensor (one value
per primitive); `exponent` is the cosine exponent of the source.  The forward
pass is rtg_trace; the backward pass is rtg_adjoint, which replays the same
Philox paths with grad_output as the weights g of L = sum_i g_i S1_i.  No
per-path memory is kept between the passes.  estimator="unbiased" adds the
likelihood ratio of the Russian-roulette survivals (an unbiased gradient of the
expected flux); estimator="held" holds those decisions as drawn (what central
differences with common random numbers measure).
"""
from __future__ import annotations

import torch

from . import _lib as L
from .engine import Engine


def _apply(engine: Engine, sticking: torch.Tensor, exponent: float, stream: int):
    if sticking.dim() == 0:
        engine.configure(sticking=float(sticking), source_exponent=float(exponent))
        engine.set_sticking_field(None)
        return None
    field = sticking.detach().to(device=torch.device("cuda", engine.device), dtype=torch.float32).contiguous()
    if field.numel() != engine.num_primitives:
        raise ValueError("a sticking field needs one value per primitive")
    if bool(((field < 0) | (field > 1)).any()):
        raise ValueError("sticking values must lie in [0, 1]")
    engine.configure(source_exponent=float(exponent))
    engine.set_sticking_field_device(field.data_ptr(), field.numel(), stream)
    return field


class _Flux(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sticking, exponent, engine, n_rays, seed, unbiased):
        dev = torch.device("cuda", engine.device)
        stream = torch.cuda.current_stream(dev).cuda_stream
        field = _apply(engine, sticking, float(exponent), stream)
        engine.trace(n_rays, seed, stream=stream)
        v = engine.device_view()
        n = v.n
        from .sharding import _CudaArray
        s1 = torch.as_tensor(_CudaArray(v.s1, n, "<f8"), device=dev).clone()
        ctx.engine, ctx.n_rays, ctx.seed, ctx.unbiased = engine, n_rays, seed, unbiased
        ctx.exponent = float(exponent)
        ctx.field_mode = field is not None
        ctx.exp_meta = (exponent.dtype, exponent.device)
        ctx.save_for_backward(sticking)
        return s1

    @staticmethod
    def backward(ctx, grad_s1):
        (sticking,) = ctx.saved_tensors
        engine = ctx.engine
        dev = torch.device("cuda", engine.device)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _apply(engine, sticking, ctx.exponent, stream)   # the replay needs the forward's configuration
        g = grad_s1.detach().to(device=dev, dtype=torch.float64).contiguous()
        scalars = torch.zeros(2, dtype=torch.float64, device=dev)
        fgrad = torch.zeros(engine.num_primitives, dtype=torch.float64, device=dev) if ctx.field_mode else None
        engine.adjoint_device(g.data_ptr(), 0, ctx.n_rays, ctx.seed, fgrad.data_ptr() if fgrad is not None else 0,
                              scalars.data_ptr(), unbiased=ctx.unbiased, stream=stream)
        if ctx.field_mode:
            gs = fgrad.to(dtype=sticking.dtype, device=sticking.device)
        else:
            gs = scalars[0].to(dtype=sticking.dtype, device=sticking.device).reshape(sticking.shape)
        ge = scalars[1].to(dtype=ctx.exp_meta[0], device=ctx.exp_meta[1])
        return gs, ge, None, None, None, None


def flux(engine: Engine, sticking, exponent, n_rays: int, seed: int = 0, estimator: str = "unbiased"):
    """Per-primitive deposited flux S1 (float64, on the engine's GPU), differentiable
    with respect to `sticking` (0-d or per-primitive) and `exponent`."""
    if estimator not in ("unbiased", "held"):
        raise ValueError("estimator must be 'unbiased' or 'held'")
    dev = torch.device("cuda", engine.device)
    s = sticking if isinstance(sticking, torch.Tensor) else torch.tensor(float(sticking), dtype=torch.float64)
    e = exponent if isinstance(exponent, torch.Tensor) else torch.tensor(float(exponent), dtype=torch.float64)
    return _Flux.apply(s, e, engine, int(n_rays), int(seed), estimator == "unbiased")


__all__ = ["flux", "L"]
