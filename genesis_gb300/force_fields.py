"""External acceleration fields (genesis/engine/force_fields.py) applied in the MPM grid op.

`scene.add_force_field(ff)` registers a field; it acts on grid velocities as
v += acc(x, v) * dt after gravity (legacy_coupler.py:381-383), on the device.  Fields start
inactive, as in the reference; `activate()` / `deactivate()` take effect at the next substep.
`Custom(func)` takes a batched torch function in place of the reference's Quadrants function; it
runs between stages of the grid op (mpm_substep_grid_stage), at its place in the field order.
"""

from __future__ import annotations

import numpy as np

from . import _lib


class ForceField:
    _type = -1

    def __init__(self):
        self._active = False
        self._solver = None

    def activate(self):
        self._active = True
        self._sync()

    def deactivate(self):
        self._active = False
        self._sync()

    @property
    def active(self):
        return self._active

    def _sync(self):
        if self._solver is not None:
            self._solver._upload_force_fields()

    def to_c(self) -> "_lib.MpmForceField":
        f = _lib.MpmForceField()
        f.type = self._type
        f.active = int(self._active)
        f.falloff_max = float("inf")
        self._fill(f)
        return f

    def _fill(self, f):
        raise NotImplementedError


def _dir(direction):
    d = np.array(direction, dtype=np.float64)
    if d.shape != (3,):
        raise ValueError("direction must have shape (3,)")
    return d / np.linalg.norm(d)


def _vec3(v, name):
    a = np.array(v, dtype=np.float64)
    if a.shape != (3,):
        raise ValueError(f"{name} must have shape (3,)")
    return a


class Constant(ForceField):
    """force_fields.py:49-82: acc = direction * strength everywhere."""

    _type = _lib.FF_CONSTANT

    def __init__(self, direction=(1, 0, 0), strength=1.0):
        super().__init__()
        self._direction = _dir(direction)
        self._strength = strength

    def _fill(self, f):
        f.direction[:] = tuple(self._direction)
        f.strength = float(self._strength)

    @property
    def direction(self):
        return self._direction

    @property
    def strength(self):
        return self._strength


class Wind(ForceField):
    """force_fields.py:85-144: constant acceleration inside a cylinder about `center` along
    `direction`."""

    _type = _lib.FF_WIND

    def __init__(self, direction=(1, 0, 0), strength=1.0, radius=1, center=(0, 0, 0)):
        super().__init__()
        self._direction = _dir(direction)
        self._center = _vec3(center, "center")
        self._strength = strength
        self._radius = radius

    def _fill(self, f):
        f.direction[:] = tuple(self._direction)
        f.center[:] = tuple(self._center)
        f.strength = float(self._strength)
        f.radius = float(self._radius)

    @property
    def radius(self):
        return self._radius

    @property
    def center(self):
        return self._center


class Point(ForceField):
    """force_fields.py:147-198: towards (strength > 0) or away from a point, with flow and falloff."""

    _type = _lib.FF_POINT

    def __init__(self, strength=1.0, position=(0, 0, 0), falloff_pow=0.0, flow=1.0):
        super().__init__()
        self._strength = strength
        self._position = _vec3(position, "position")
        self._falloff_pow = falloff_pow
        self._flow = flow

    def _fill(self, f):
        f.center[:] = tuple(self._position)
        f.strength = float(self._strength)
        f.falloff_pow = float(self._falloff_pow)
        f.flow = float(self._flow)

    @property
    def position(self):
        return self._position


class Drag(ForceField):
    """force_fields.py:201-229: -linear v - quadratic |v| v."""

    _type = _lib.FF_DRAG

    def __init__(self, linear=0.0, quadratic=0.0):
        super().__init__()
        self._linear = linear
        self._quadratic = quadratic

    def _fill(self, f):
        f.linear = float(self._linear)
        f.quadratic = float(self._quadratic)


class Vortex(ForceField):
    """force_fields.py:263-369: swirl about the z axis through `center` with radial pull, falloff
    and damping."""

    _type = _lib.FF_VORTEX

    def __init__(self, direction=(0.0, 0.0, 1.0), center=(0.0, 0.0, 0.0), strength_perpendicular=20.0,
                 strength_radial=0.0, falloff_pow=2.0, falloff_min=0.01, falloff_max=np.inf, damping=0.0):
        super().__init__()
        self._direction = _dir(direction)
        self._center = _vec3(center, "center")
        self._strength_perpendicular = strength_perpendicular
        self._strength_radial = strength_radial
        self._falloff_pow = falloff_pow
        self._falloff_min = falloff_min
        self._falloff_max = falloff_max
        self._damping = damping

    def _fill(self, f):
        f.direction[:] = tuple(self._direction)
        f.center[:] = tuple(self._center)
        f.strength_perpendicular = float(self._strength_perpendicular)
        f.strength_radial = float(self._strength_radial)
        f.falloff_pow = float(self._falloff_pow)
        f.falloff_min = float(self._falloff_min)
        f.falloff_max = float(self._falloff_max)
        f.damping = float(self._damping)

    @property
    def center(self):
        return self._center


class Noise(ForceField):
    """force_fields.py:232-259: acc = strength * (2u - 1) per node, component and substep, u uniform
    in [0, 1).  The draws come from a counter-based hash (splitmix64 over seed, substep, scene, node
    and component) instead of the reference's generator state: the same distribution, repeatable
    for a given seed, not the reference's numbers."""

    _type = _lib.FF_NOISE

    def __init__(self, strength=1.0, seed=0):
        super().__init__()
        self._strength = strength
        self._seed = int(seed) & 0xFFFFFFFFFFFFFFFF

    def _fill(self, f):
        f.strength = float(self._strength)
        f.seed = self._seed

    @property
    def strength(self):
        return self._strength


def perlin_permutation(seed, seed_offset, wrap_size=256):
    """PerlinNoiseField's table (force_fields.py:448-460): the identity, shuffled by numpy's global
    generator seeded with seed + seed_offset when a seed is given (the global state is restored)."""
    perm = np.arange(wrap_size, dtype=np.int32)
    if seed is not None:
        state = np.random.get_state()
        np.random.seed(seed + seed_offset)
        np.random.shuffle(perm)
        np.random.set_state(state)
    return perm


class Turbulence(ForceField):
    """force_fields.py:372-421: acc_k = strength * perlin_k(frequency * x) for three Perlin noise
    fields (seed offsets 0, 1, 2), then acc += (acc - v) * flow."""

    _type = _lib.FF_TURBULENCE

    def __init__(self, strength=1.0, frequency=3, flow=0.0, seed=None):
        super().__init__()
        self._strength = strength
        self._frequency = frequency
        self._flow = flow
        self._perms = [perlin_permutation(seed, k) for k in range(3)]

    def _fill(self, f):
        f.strength = float(self._strength)
        f.frequency = float(self._frequency)
        f.flow = float(self._flow)
        for k in range(3):
            f.perm[k][:] = [int(v) for v in self._perms[k]]

    @property
    def strength(self):
        return self._strength

    @property
    def frequency(self):
        return self._frequency


class Custom(ForceField):
    """force_fields.py:424-437: a user-defined acceleration acc = func(pos, vel, t, i).

    The reference compiles `func` (a Quadrants function of one node's position and velocity) into
    its grid op, where i = -1 and t is the simulation time of the substep.  Here `func` is a batched
    torch function: pos and vel are float32 CUDA tensors [M, 3] of the M grid nodes that hold mass
    (velocity after gravity and the fields listed before this one), t a float, i = -1; it returns
    the accelerations [M, 3].  As in the reference, `get_acc` is replaced by `func`, so the field
    acts whether or not it was activated.  A scene with a Custom field runs its substeps through the
    staged grid op (one library call per stage and a torch call per Custom field per substep)
    instead of the captured graph.  In differentiable mode `func` is differentiated by torch
    autograd (its parameters that require grad receive gradients too)."""

    _type = -2

    def __init__(self, func):
        super().__init__()
        if not callable(func):
            raise TypeError("Custom force field needs a callable func(pos, vel, t, i) -> acc.")
        self.get_acc = func

    def to_c(self):
        raise TypeError("a Custom force field has no device record")
