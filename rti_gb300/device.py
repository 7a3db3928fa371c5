"""Python mirror of rti::device<T, particle_type, reflection_type> (src/rti/device.hpp:34-297).

Same setters, same argument meaning (the grid spacing of each point is the
disc radius, device.hpp:213-216), same defaults (1024 rays, reflective x/y
boundaries, cosine source), same outputs: ``get_mc_estimates()`` returns the
normalised, neighbourhood-smoothed flux (device.hpp:154-187) and
``get_hit_cnts()`` the per-disc hit counts.  ``run()`` traces on the GPU through
librtg; mismatched input sizes raise ValueError where the reference asserts.

Plug-ins map as follows:
* particle: ``get_sticking_probability(prim_id)`` is evaluated once per disc on
  the host and uploaded as a sticking field (a sticking that depends on the
  incoming ray or on random state cannot be expressed; the reference's own
  examples use a constant, main/dev.cpp:214-228);
* reflection: ``Diffuse()`` (reflection/diffuse.hpp), ``Specular()``
  (reflection/specular.hpp) or ``Mixed(p)``;
* direction: ``set(direction)`` changes nothing, as in the reference, where
  ``device::set`` assigns through a reference member bound to the cosine source
  and copies only the empty ``i_direction`` base (device.hpp:77-80, 295-296);
  ``set_source_exponent(n)`` (no counterpart there) selects a cos^n source.
"""
from __future__ import annotations

from enum import IntEnum

import numpy as np

from . import _lib as L
from .engine import Engine


class BoundCondition(IntEnum):
    """rti::geo::bound_condition (geo/bound_condition.hpp:4-6)."""
    REFLECTIVE = L.RTG_BOUND_REFLECTIVE
    PERIODIC = L.RTG_BOUND_PERIODIC


class Particle:
    """rti::particle::i_particle: sticking probability per hit primitive."""

    def get_sticking_probability(self, prim_id: int) -> float:  # pragma: no cover - interface
        raise NotImplementedError

    def init_new(self) -> None:
        pass


class ConstantSticking(Particle):
    def __init__(self, sticking: float):
        self.sticking = float(sticking)

    def get_sticking_probability(self, prim_id: int) -> float:
        return self.sticking


class Diffuse:
    mode = L.RTG_REFLECT_DIFFUSE
    specular_fraction = 0.0


class Specular:
    mode = L.RTG_REFLECT_SPECULAR
    specular_fraction = 1.0


class Mixed:
    mode = L.RTG_REFLECT_MIXED

    def __init__(self, specular_fraction: float):
        self.specular_fraction = float(specular_fraction)


class CosineDirectionZ:
    """ray::cosine_direction_z (ray/cosine_direction_z.hpp)."""
    exponent = 1.0


class PowerCosineDirectionZ:
    """ray::power_cosine_direction_z (ray/power_cosine_direction_z.hpp)."""

    def __init__(self, exponent: float):
        self.exponent = float(exponent)


class Device:
    def __init__(self, particle: Particle | None = None, reflection=None, device: int = 0):
        self.particle = particle if particle is not None else ConstantSticking(1.0)
        self.reflection = reflection if reflection is not None else Diffuse()
        self.cuda_device = device
        self.points = np.zeros((0, 3), dtype=np.float32)
        self.normals = np.zeros((0, 3), dtype=np.float32)
        self.spacing = np.zeros(0, dtype=np.float32)
        self.numofrays = 1024                      # device.hpp:289
        self.x_cond = BoundCondition.REFLECTIVE    # device.hpp:292
        self.y_cond = BoundCondition.REFLECTIVE    # device.hpp:293
        self.source_exponent = 1.0               # cosine_direction_z, device.hpp:295
        self.seed = 0
        self.mcestimates = np.zeros(0, dtype=np.float32)
        self.hitcnts = np.zeros(0, dtype=np.uint64)
        self.engine: Engine | None = None

    def set_points(self, points):
        self.points = np.array(points, dtype=np.float32).reshape(-1, 3)

    def set_normals(self, normals):
        self.normals = np.array(normals, dtype=np.float32).reshape(-1, 3)

    def set_grid_spacing(self, spacing):
        self.spacing = np.array(spacing, dtype=np.float32).reshape(-1)

    def set_number_of_rays(self, n: int):
        self.numofrays = int(n)

    def set_x(self, cond: BoundCondition):
        self.x_cond = BoundCondition(cond)

    def set_y(self, cond: BoundCondition):
        self.y_cond = BoundCondition(cond)

    def set(self, direction):
        """rti's ``device::set``: the source stays cosine (device.hpp:77-80)."""
        del direction

    def set_source_exponent(self, n: float):
        """Extension: a cos^n source (power_cosine_direction_z), n >= 0."""
        self.source_exponent = float(n)

    def set_seed(self, seed: int):
        self.seed = int(seed)

    def _sticking(self):
        if isinstance(self.particle, ConstantSticking):
            return self.particle.sticking, None
        field = np.array([self.particle.get_sticking_probability(i) for i in range(len(self.points))],
                         dtype=np.float32)
        if len(field) and np.all(field == field[0]):
            return float(field[0]), None
        return 1.0, field

    def run(self):
        if not (len(self.points) == len(self.normals) == len(self.spacing)):
            raise ValueError("points, normals and grid spacing must have the same length (device.hpp:210)")
        if self.engine is None:
            self.engine = Engine(self.cuda_device)
        e = self.engine
        e.upload_discs(self.points, self.normals, self.spacing)
        s, field = self._sticking()
        cfg = L.default_config()
        cfg.x_bound = int(self.x_cond)
        cfg.y_bound = int(self.y_cond)
        cfg.reflection = self.reflection.mode
        cfg.specular_fraction = getattr(self.reflection, "specular_fraction", 0.0)
        cfg.sticking = s
        cfg.source_exponent = self.source_exponent
        e.configure(**{k: getattr(cfg, k) for k in ("x_bound", "y_bound", "reflection", "specular_fraction",
                                                    "sticking", "source_exponent")})
        e.set_sticking_field(field)
        e.trace(self.numofrays, self.seed)
        self.mcestimates = e.mc_estimates()
        self.hitcnts = e.hit_counts()

    def get_mc_estimates(self) -> np.ndarray:
        return self.mcestimates.copy()

    def get_hit_cnts(self) -> np.ndarray:
        return self.hitcnts.copy()
