"""Particle emitter for MPM entities (genesis/engine/entities/emitter.py).

`Scene.add_emitter(material, max_particles)` adds an MPM entity of `max_particles` inactive
particles (a Nowhere morph); `Emitter.emit` samples a droplet (circle / sphere / square /
rectangle nozzle shapes), places it at the nozzle, and activates the next particles of the pool
with the droplet's positions and the emission velocity, recycling the pool when it runs out
(emitter.py:56-194); `emit_omni` emits a spherical shell radially (emitter.py:196-242).  The
per-particle writes go through the entity setters, i.e. libgbmpm's particle-field kernels.
"""

from __future__ import annotations

import numpy as np
import torch

from . import morphs as _m
from .exceptions import GenesisException


def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / max(np.linalg.norm(v), 1e-12)


def z_up_frame(z, eps):
    """Rotation whose third column is the unit vector z; the first column is horizontal
    ((z_y, -z_x, 0), or (z_z, 0, -z_x) when z is vertical), as utils/geom.py:1565-1611."""
    z = np.asarray(z, dtype=np.float64)
    n = np.linalg.norm(z)
    z = z / n if n > eps else np.array([0.0, 1.0, 0.0])
    x = np.array([z[1], -z[0], 0.0]) if abs(z[2]) < 1.0 - eps else np.array([z[2], 0.0, -z[0]])
    xn = np.linalg.norm(x)
    if xn <= eps:
        return np.eye(3)
    x = x / xn
    return np.stack([x, np.cross(z, x), z], axis=1)


def axis_angle_R(axis, theta):
    """Rotation about `axis` built from cos(theta) with sin = sqrt(1 - cos^2), as
    utils/geom.py:1802-1839 does (so theta and -theta give the same matrix)."""
    a = _normalize(axis)
    c = float(np.cos(theta))
    s = float(np.sqrt(max(0.0, 1.0 - c * c)))
    K = np.array([[0.0, -a[2], a[1]], [a[2], 0.0, -a[0]], [-a[1], a[0], 0.0]])
    return c * np.eye(3) + s * K + (1.0 - c) * np.outer(a, a)


def shell_to_particles(p_size=0.01, pos=(0, 0, 0), inner_radius=0.5, outer_radius=0.7, sampler="random"):
    """utils/particle.py:279-304: box lattice / random samples kept with inner <= r <= outer."""
    p = _m.box_to_particles(p_size, pos, (2 * outer_radius,) * 3, sampler)
    r = np.linalg.norm(p - np.asarray(pos), axis=1)
    return p[(r <= outer_radius) & (r >= inner_radius)]


class Emitter:
    def __init__(self, max_particles: int):
        self._max_particles = int(max_particles)
        self._entity = None
        self._acc_droplet_len = 0.0
        self._next_particle = 0

    def set_entity(self, entity):
        self._entity = entity
        self._solver = entity._solver
        self._next_particle = 0

    def reset(self):
        self._next_particle = 0

    @property
    def entity(self):
        return self._entity

    @property
    def max_particles(self):
        return self._max_particles

    def _activate(self, positions, vels):
        n = len(positions)
        if n > self._entity.n_particles:
            raise GenesisException(
                f"Number of particles to emit ({n}) at the current step is larger than the maximum number of "
                f"particles ({self._entity.n_particles})."
            )
        idx = torch.arange(self._next_particle, self._next_particle + n, device="cuda")
        self._entity.set_particles_pos(torch.as_tensor(positions, dtype=torch.float32), idx)
        self._entity.set_particles_vel(torch.as_tensor(vels, dtype=torch.float32), idx)
        self._entity.set_particles_active(True, idx)
        self._next_particle += n
        if self._next_particle + n > self._entity.n_particles:  # recycle particles
            self._next_particle = 0

    def emit(self, droplet_shape, droplet_size, droplet_length=None, pos=(0.5, 0.5, 1.0), direction=(0, 0, -1),
             theta=0.0, speed=1.0, p_size=None):
        if self._entity is None:
            raise GenesisException("Emitter has no entity.")
        if droplet_shape in ("circle", "sphere", "square"):
            if not isinstance(droplet_size, (int, float)):
                raise GenesisException("droplet_size must be a number for this shape.")
        elif droplet_shape == "rectangle":
            if not (isinstance(droplet_size, (tuple, list)) and len(droplet_size) == 2):
                raise GenesisException("droplet_size must be (width, height) for a rectangle.")
        else:
            raise GenesisException(f"Unsupported nozzle shape: {droplet_shape}.")
        import genesis_gb300 as gs

        direction = np.asarray(direction, dtype=np.float64)
        if np.linalg.norm(direction) < gs.EPS:
            raise GenesisException("Zero-length direction.")
        direction = _normalize(direction)
        p_size = self._entity.particle_size if p_size is None else p_size
        if droplet_length is None:
            droplet_length = speed * self._solver.substep_dt * self._solver._sim.substeps + self._acc_droplet_len
            if droplet_length < p_size:  # too short: accumulate and emit later
                self._acc_droplet_len = droplet_length
                droplet_length = 0.0
            else:
                self._acc_droplet_len = 0.0
        if droplet_length <= 0.0:
            return
        sampler = self._entity.sampler
        if droplet_shape == "circle":
            positions = _m.cylinder_to_particles(p_size, (0, 0, 0), droplet_size / 2, droplet_length, sampler)
        elif droplet_shape == "sphere":
            positions = _m.sphere_to_particles(p_size, (0, 0, 0), droplet_size / 2, sampler)
        elif droplet_shape == "square":
            positions = _m.box_to_particles(p_size, (0, 0, 0), (droplet_size, droplet_size, droplet_length), sampler)
        else:
            positions = _m.box_to_particles(p_size, (0, 0, 0), (droplet_size[0], droplet_size[1], droplet_length),
                                            sampler)
        R = z_up_frame(direction, gs.EPS) @ axis_angle_R(np.array([0.0, 0.0, 1.0]), theta)
        positions = positions @ R.T + np.asarray(pos, dtype=np.float64)
        if not self._solver.boundary.is_inside(positions):
            raise GenesisException("Emitted particles are outside the boundary.")
        self._activate(positions, np.tile(speed * direction, (len(positions), 1)))

    def emit_omni(self, source_radius=0.1, pos=(0.5, 0.5, 1.0), speed=1.0, particle_size=None):
        import genesis_gb300 as gs

        if self._entity is None:
            raise GenesisException("Emitter has no entity.")
        pos = np.asarray(pos, dtype=np.float64)
        particle_size = self._entity.particle_size if particle_size is None else particle_size
        rel = shell_to_particles(particle_size, (0, 0, 0), source_radius * 0.4, source_radius, self._entity.sampler)
        positions = pos + rel
        if not self._solver.boundary.is_inside(positions):
            raise GenesisException("Emitted particles are outside the boundary.")
        dists = np.linalg.norm(rel, axis=1)
        positions[dists < gs.EPS] = gs.EPS
        vels = (speed / (dists[:, None] + gs.EPS)) * rel
        self._activate(positions, vels)
