"""Batched form: many independent MPM scenes of uneven particle counts in one context.

All scenes share the particle pool, the grid-block key space and every launch: one P2G,
one grid-op and one G2P launch per substep cover all scenes through the scene tables
(per-scene dx, dt, gravity, boundary, grid offset and block range), and the substep loop
runs as a replayed CUDA graph.  The P2G launch shape comes from the autotuner.

The reference's `n_envs` batching replicates one particle set (mpm_solver.py:121-136);
scenes of different sizes and materials, as here, have no reference counterpart: each
scene's result is checked against the same scene run alone.
"""

from __future__ import annotations

import ctypes
import dataclasses
import math

import numpy as np
import torch

from . import _lib
from .materials import Elastic, Liquid, Sand, Snow, _MPMBase
from .morphs import box_to_particles


@dataclasses.dataclass
class SceneSpec:
    """One scene: a box of particles of one material dropped in a unit-cube domain."""

    material: _MPMBase
    n_particles: int
    extent: float
    center: tuple = (0.5, 0.5, 0.5)
    grid_density: float = 64.0
    lower_bound: tuple = (0.0, 0.0, 0.0)
    upper_bound: tuple = (1.0, 1.0, 1.0)
    substep_dt: float = 2e-4
    gravity: tuple = (0.0, 0.0, -9.81)
    seed: int = 0
    substeps: int = -1  # serving: substeps to run before the scene freezes (-1: unlimited)

    @property
    def particle_size(self) -> float:
        return self.extent / self.n_particles ** (1.0 / 3.0)

    def positions(self) -> np.ndarray:
        """n_particles uniform samples in the box (seeded), as the 'random' sampler does."""
        rng = np.random.default_rng(self.seed)
        c = np.asarray(self.center, dtype=np.float64)
        return rng.uniform(c - self.extent / 2, c + self.extent / 2, size=(self.n_particles, 3))


def batched_workload(n_scenes=256, seed=1234, n_range=(2000, 64000), extent_range=(0.1, 0.3), substep_dt=2e-4,
                     grid_density=64.0):
    """Config 3: N ~ logUniform[2k, 64k], material uniform over {Elastic, Liquid, Sand, Snow},
    box extent ~ U[0.1, 0.3], each scene its own 65^3-node grid over the unit cube."""
    rng = np.random.default_rng(seed)
    mats = (lambda: Elastic(), lambda: Liquid(), lambda: Sand(), lambda: Snow())
    specs = []
    for i in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        ext = float(rng.uniform(*extent_range))
        m = mats[int(rng.integers(0, 4))]()
        center = (0.5, 0.5, 0.06 + ext / 2 + 0.02)
        specs.append(SceneSpec(m, n, ext, center, grid_density=grid_density, substep_dt=substep_dt,
                               seed=int(rng.integers(0, 2**31))))
    return specs


def scene_config(spec: SceneSpec, eps: float) -> _lib.MpmSceneConfig:
    c = _lib.MpmSceneConfig()
    c.substep_dt = spec.substep_dt
    for d in range(3):
        c.gravity[d] = spec.gravity[d]
        c.lower_bound[d] = spec.lower_bound[d]
        c.upper_bound[d] = spec.upper_bound[d]
    c.grid_density = spec.grid_density
    c.particle_size = spec.particle_size
    c.mass_eps = eps
    c.restitution = 0.0
    c.n_particles = spec.n_particles
    return c


class BatchedMPM:
    """One libgbmpm context holding every scene of `specs`."""

    def __init__(self, specs, tune: bool = True, device=None, positions=None):
        self.specs = list(specs)
        self.lib = _lib.load()
        eps = float(np.finfo(np.float32).eps)
        S = (_lib.MpmSceneConfig * len(specs))(*[scene_config(s, eps) for s in specs])
        M = (_lib.MpmMaterial * len(specs))(*[s.material.to_c(i) for i, s in enumerate(specs)])
        self.ctx = ctypes.c_void_p()
        dev = torch.cuda.current_device() if device is None else device
        _lib.check(self.lib.mpm_ctx_create(S, len(specs), M, len(specs), dev, ctypes.byref(self.ctx)), None,
                   "mpm_ctx_create")
        self.offsets = np.concatenate([[0], np.cumsum([s.n_particles for s in specs])]).astype(np.int64)
        h = self._stream()
        for i, s in enumerate(specs):
            host = s.positions() if positions is None or positions[i] is None else positions[i]
            p = torch.as_tensor(host, dtype=torch.float32, device="cuda")
            _lib.check(self.lib.mpm_add_particles(self.ctx, i, i + 1, 0, s.n_particles, 0, 1, p.data_ptr(), h),
                       self.ctx, "mpm_add_particles")
        torch.cuda.current_stream().synchronize()
        self.tuning = None
        if tune:
            self.tune()

    @staticmethod
    def _stream():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    @property
    def n_particles(self) -> int:
        return int(self.offsets[-1])

    def tune(self):
        from .autotune import autotune

        state = self.get_state_all()
        self.tuning = autotune(self.ctx)
        self.set_state_all(state)
        return self.tuning

    def step(self, n_substeps: int) -> None:
        _lib.check(self.lib.mpm_substeps(self.ctx, int(n_substeps), self._stream()), self.ctx, "mpm_substeps")

    def check(self) -> int:
        st = ctypes.c_uint32()
        _lib.check(self.lib.mpm_status_word(self.ctx, ctypes.byref(st), None, 1, self._stream()), self.ctx, "status")
        return st.value

    def get_state_all(self) -> dict:
        n = self.n_particles
        out = dict(pos=torch.empty(n, 3), vel=torch.empty(n, 3), C=torch.empty(n, 3, 3), F=torch.empty(n, 3, 3),
                   Jp=torch.empty(n), active=torch.empty(n, dtype=torch.uint8))
        out = {k: v.cuda() for k, v in out.items()}
        _lib.check(self.lib.mpm_get_state(self.ctx, 0, len(self.specs),
                                          *[out[k].data_ptr() for k in ("pos", "vel", "C", "F", "Jp", "active")],
                                          self._stream()), self.ctx, "mpm_get_state")
        return out

    def set_state_all(self, st: dict) -> None:
        _lib.check(self.lib.mpm_set_state(self.ctx, 0, len(self.specs),
                                          *[st[k].contiguous().data_ptr() for k in ("pos", "vel", "C", "F", "Jp", "active")],
                                          self._stream()), self.ctx, "mpm_set_state")
        torch.cuda.current_stream().synchronize()

    def scene_state(self, i: int, st: dict | None = None) -> dict:
        st = st or self.get_state_all()
        a, b = int(self.offsets[i]), int(self.offsets[i + 1])
        return {k: v[a:b] for k, v in st.items()}

    def close(self) -> None:
        if self.ctx:
            self.lib.mpm_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
