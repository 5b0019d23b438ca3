"""Option classes of the MPM path, with the reference's fields, defaults and validation.

Mirrors genesis/options/solvers.py (SimOptions :17-69, MPMOptions :548-604) and
genesis/options/options.py (model_copy_from :100-107) without pydantic, which the GPU
hosts do not ship.  Unknown keyword arguments raise, like the reference's extra="forbid".
"""

from __future__ import annotations

import copy
import math

import numpy as np

from .exceptions import GenesisException


class Options:
    """Keyword-only option container: class attributes are the defaults."""

    _fields: tuple[str, ...] = ()

    def __init__(self, **data):
        unknown = set(data) - set(self._fields)
        if unknown:
            raise GenesisException(f"Unrecognized option(s) for {type(self).__name__}: {sorted(unknown)}")
        for f in self._fields:
            object.__setattr__(self, f, copy.deepcopy(data.get(f, getattr(type(self), f))))
        self._post_init()

    def _post_init(self) -> None:
        pass

    def copy_attributes_from(self, other: "Options", override: bool = False) -> None:
        for f in self._fields:
            if hasattr(other, f) and (override or getattr(self, f) is None):
                object.__setattr__(self, f, copy.deepcopy(getattr(other, f)))

    def model_copy_from(self, other: "Options") -> "Options":
        """Fill fields that are None from `other` (options.py:100-107)."""
        out = copy.deepcopy(self)
        out.copy_attributes_from(other)
        return out

    def __eq__(self, other) -> bool:
        return type(self) is type(other) and all(getattr(self, f) == getattr(other, f) for f in self._fields)

    def __hash__(self) -> int:
        return id(self)

    def __repr__(self) -> str:
        args = ", ".join(f"{f}={getattr(self, f)!r}" for f in self._fields)
        return f"{type(self).__name__}({args})"


def _vec3(v, name):
    a = tuple(float(x) for x in v)
    if len(a) != 3 or not all(math.isfinite(x) for x in a):
        raise GenesisException(f"'{name}' must be a finite 3-vector")
    return a


class SimOptions(Options):
    """genesis/options/solvers.py:17-69."""

    _fields = ("dt", "substeps", "substeps_local", "gravity", "floor_height", "requires_grad")
    dt = 1e-2
    substeps = 1
    substeps_local = None
    gravity = (0.0, 0.0, -9.81)
    floor_height = 0.0
    requires_grad = False

    def _post_init(self) -> None:
        if not (self.dt > 0):
            raise GenesisException("'dt' must be positive")
        if int(self.substeps) != self.substeps or self.substeps < 1:
            raise GenesisException("'substeps' must be a positive integer")
        self.gravity = _vec3(self.gravity, "gravity")
        if self.substeps_local is None:
            self.substeps_local = self.substeps if self.requires_grad else 1
        self._steps_local = None
        if self.requires_grad:
            if self.substeps_local % self.substeps != 0:
                raise GenesisException("`substeps_local` must be divisible by `substeps` when `requires_grad` is True.")
            self._steps_local = self.substeps_local // self.substeps


class MPMOptions(Options):
    """genesis/options/solvers.py:548-604."""

    _fields = ("dt", "gravity", "particle_size", "grid_density", "enable_CPIC", "lower_bound", "upper_bound")
    dt = None
    gravity = None
    particle_size = None
    grid_density = 64
    enable_CPIC = False
    lower_bound = (-1.0, -1.0, 0.0)
    upper_bound = (1.0, 1.0, 1.0)

    def __init__(self, *, use_sparse_grid: bool = False, leaf_block_size: int = 8, **data):
        super().__init__(**data)

    def _post_init(self) -> None:
        if not (self.grid_density > 0):
            raise GenesisException("'grid_density' must be positive")
        if self.particle_size is None:
            self.particle_size = 0.01 * 64.0 / self.grid_density
        self.lower_bound = _vec3(self.lower_bound, "lower_bound")
        self.upper_bound = _vec3(self.upper_bound, "upper_bound")
        if not np.all(np.array(self.upper_bound) > np.array(self.lower_bound)):
            raise GenesisException("Invalid pair of upper_bound and lower_bound.")


class ToolOptions(Options):
    """genesis/options/solvers.py:376-393: the tool solver's dt and floor height (None: inherited
    from SimOptions); a tool's position never goes below the floor (FloorBoundary.impose_pos)."""

    _fields = ("dt", "floor_height")
    dt = None
    floor_height = None


class LegacyCouplerOptions(Options):
    """Accepted for API compatibility; no coupling partner exists in this path."""

    _fields = ("rigid_mpm", "rigid_sph", "rigid_pbd", "rigid_fem", "mpm_sph", "mpm_pbd", "fem_mpm", "fem_sph")
    rigid_mpm = rigid_sph = rigid_pbd = rigid_fem = mpm_sph = mpm_pbd = fem_mpm = fem_sph = True


class ViewerOptions(Options):
    """Accepted and ignored (no viewer in this path)."""

    _fields = ("camera_pos", "camera_lookat", "camera_fov", "res", "max_FPS")
    camera_pos = (3.5, 0.5, 2.5)
    camera_lookat = (0.0, 0.0, 0.5)
    camera_fov = 40
    res = None
    max_FPS = 60


class VisOptions(Options):
    """Accepted and ignored except `n_support_neighbors`."""

    _fields = ("visualize_mpm_boundary", "rendered_envs_idx", "n_support_neighbors", "show_world_frame")
    visualize_mpm_boundary = False
    rendered_envs_idx = None
    n_support_neighbors = 12
    show_world_frame = True


class ProfilingOptions(Options):
    _fields = ("show_FPS", "FPS_tracker_alpha")
    show_FPS = False
    FPS_tracker_alpha = 0.95
