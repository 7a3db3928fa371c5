"""rti_gb300 -- GB300-native Monte Carlo flux engine behind rti's device API.

librtg.so (hand-written sm_103a CUDA, C ABI in include/rtg.h) does all the
tracing; this package holds the host-side mirror of the reference interface
(`Device`, after rti::device), a context wrapper (`Engine`), the batched and
adjoint front ends, and seeded synthetic surfaces (`scenes`).
"""
from ._lib import RtgError, load  # noqa: F401
from .device import (BoundCondition, ConstantSticking, CosineDirectionZ, Device, Diffuse, Mixed,  # noqa: F401
                     Particle, PowerCosineDirectionZ, Specular)
from .engine import Engine, device_run  # noqa: F401

__all__ = ["Engine", "Device", "BoundCondition", "ConstantSticking", "Particle", "Diffuse", "Specular", "Mixed",
           "CosineDirectionZ", "PowerCosineDirectionZ", "device_run", "RtgError", "load"]
