"""Scene and Simulator: the user API around the MPM path.

Mirrors genesis/engine/scene.py (add_entity :348, build :841-905, step :1017-1034,
get_state :1005-1015, reset :958-996) and genesis/engine/simulator.py (step :272-296,
substep :320-324) for scenes whose only solver is MPM.  A Genesis `scene.step()` runs
`substeps` substeps; here they are enqueued as one fused call to libgbmpm.so and the
NaN check of every substep (mpm_solver.py:542-546) is read once per step.
"""

from __future__ import annotations

import numpy as np
import torch

from . import morphs as _morphs
from .exceptions import GenesisException
from .options import (LegacyCouplerOptions, MPMOptions, ProfilingOptions, SimOptions, ToolOptions, ViewerOptions,
                      VisOptions)
from .solver import MPMSolver
from .states import SimState


class Simulator:
    def __init__(self, scene, options: SimOptions, mpm_options: MPMOptions):
        self.scene = scene
        self._options = options
        self._substeps = int(options.substeps)
        self._substeps_local = int(options.substeps_local)
        self._requires_grad = bool(options.requires_grad)
        self._dt = float(options.dt)
        self._substep_dt = self._dt / self._substeps
        self._B = 1
        self._cur_substep_global = 0
        self.mpm_solver = MPMSolver(scene, self, mpm_options)
        self._queried_states = []

    def build(self, B: int):
        self._B = B
        self.mpm_solver.build(B)

    def step(self, check_state: bool = True):
        """simulator.py:272-296 for the MPM solver alone."""
        self.mpm_solver.process_input()
        self.mpm_solver.substeps(self._substeps)
        self._cur_substep_global += self._substeps
        if check_state:
            self.mpm_solver.check_state()

    def substep(self, f=0):
        """simulator.py:320-324: pre-coupling, coupling (grid op), post-coupling."""
        self.mpm_solver.substep_pre_coupling(f)
        self.mpm_solver.couple(f)
        self.mpm_solver.substep_post_coupling(f)
        self._cur_substep_global += 1

    @property
    def substeps(self):
        return self._substeps

    @property
    def substeps_local(self):
        return self._substeps_local

    @property
    def cur_substep_global(self):
        return self._cur_substep_global

    @property
    def cur_step_global(self):
        return self._cur_substep_global // self._substeps

    @property
    def cur_substep_local(self):
        return self._cur_substep_global % self._substeps_local

    @property
    def cur_t(self):
        return self._cur_substep_global * self._substep_dt

    @property
    def dt(self):
        return self._dt

    @property
    def substep_dt(self):
        return self._substep_dt

    @property
    def requires_grad(self):
        return self._requires_grad

    @property
    def solvers(self):
        return [self.mpm_solver]

    @property
    def active_solvers(self):
        return [self.mpm_solver] if self.mpm_solver.is_active else []


class Scene:
    def __init__(
        self,
        sim_options: SimOptions | None = None,
        coupler_options: LegacyCouplerOptions | None = None,
        mpm_options: MPMOptions | None = None,
        viewer_options: ViewerOptions | None = None,
        vis_options: VisOptions | None = None,
        profiling_options: ProfilingOptions | None = None,
        show_viewer: bool = False,
        show_FPS: bool | None = None,
        **other_solver_options,
    ):
        import genesis_gb300 as gs

        if not gs._initialized:
            raise GenesisException("Genesis hasn't been initialized. Did you call `gs.init()`?")
        for k in other_solver_options:
            if not k.endswith("_options"):
                raise GenesisException(f"Unrecognized Scene argument: {k}")
        self.sim_options = sim_options or SimOptions()
        mpm_options = mpm_options or MPMOptions()
        if self.sim_options.requires_grad and mpm_options.enable_CPIC:
            raise GenesisException(  # mpm_solver.py:213-216
                "CPIC is not supported in differentiable mode yet. Submit a feature request if you need it.")
        # MPMOptions inherits dt and gravity from SimOptions (scene.py:157)
        self.mpm_options = mpm_options.model_copy_from(self.sim_options)
        self.vis_options = vis_options or VisOptions()
        self.show_viewer = False
        self._sim = Simulator(self, self.sim_options, self.mpm_options)
        # ToolOptions.floor_height inherits SimOptions.floor_height (options/solvers.py:376-393)
        self.tool_options = other_solver_options.get("tool_options") or ToolOptions()
        floor = self.tool_options.floor_height
        self._sim.mpm_solver._tool_floor = float(self.sim_options.floor_height if floor is None else floor)
        self._entities = []
        self._emitters = []
        self._is_built = False
        self._n_envs = 0
        self._envs_idx = None
        self._init_state = None

    # ------------------------------------------------------------------ construction
    def add_entity(self, morph, material=None, surface=None, visualize_contact=False, vis_mode=None, name=None):
        from .materials import Tool, _MPMBase

        if self._is_built:
            raise GenesisException("Scene is already built.")
        if isinstance(material, Tool):  # ToolSolver.add_entity: a kinematic mesh coupled to MPM
            entity = self._sim.mpm_solver.add_tool(len(self._entities), material, morph, surface, name=name)
            self._entities.append(entity)
            return entity
        if material is None or not isinstance(material, _MPMBase):
            raise GenesisException("Only MPM materials (gs.materials.MPM.*) are supported by this MPM path.")
        if not isinstance(morph, _morphs.Morph):
            raise GenesisException(f"Unsupported morph: {morph}.")
        entity = self._sim.mpm_solver.add_entity(len(self._entities), material, morph, surface, name=name)
        self._entities.append(entity)
        return entity

    def add_force_field(self, force_field):
        """scene.py:820-836: an external acceleration field acting on the MPM grid."""
        if self._is_built:
            raise GenesisException("Scene is already built.")
        force_field.scene = self
        self._sim.mpm_solver._add_force_field(force_field)
        return force_field

    def add_emitter(self, material, max_particles=20000, surface=None):
        """scene.py:765-818: an MPM entity of `max_particles` inactive particles driven by an Emitter."""
        from .emitter import Emitter
        from .materials import _MPMBase

        if self.requires_grad:
            raise GenesisException("Emitter is not supported in differentiable mode.")
        if not isinstance(material, _MPMBase):
            raise GenesisException("Non-supported material for emitter. Supported materials are: `gs.materials.MPM.Base`.")
        emitter = Emitter(max_particles)
        entity = self.add_entity(morph=_morphs.Nowhere(n_particles=max_particles), material=material, surface=surface)
        emitter.set_entity(entity)
        self._emitters.append(emitter)
        return emitter

    @property
    def emitters(self):
        return self._emitters

    def build(self, n_envs: int = 0, env_spacing=(0.0, 0.0), n_envs_per_row=None, center_envs_at_origin=True,
              compile_kernels=None):
        if self._is_built:
            raise GenesisException("Scene is already built.")
        self._n_envs = int(n_envs)
        B = max(self._n_envs, 1)
        self._envs_idx = torch.arange(B, dtype=torch.int32, device="cuda")
        self._sim.build(B)
        self._is_built = True
        self._init_state = self._sim.mpm_solver.get_state()

    # ------------------------------------------------------------------ stepping
    def step(self, update_visualizer=True, refresh_visualizer=True):
        if not self._is_built:
            raise GenesisException("Scene is not built yet.")
        self._sim.step()

    def reset(self, state=None, envs_idx=None):
        """scene.py:958-996: restore the initial (or given) state."""
        if not self._is_built:
            raise GenesisException("Scene is not built yet.")
        if state is None:
            state = self._init_state
        elif isinstance(state, SimState):
            state = state.solvers_state[0]
        if state is not None:
            self._sim.mpm_solver.set_state(0, state, envs_idx)
        solver = self._sim.mpm_solver
        if solver._tools:
            for t in solver._tools:
                t.reset()
            solver._upload_colliders()
        if solver._diff is not None:
            solver._diff.reset(list(range(solver._B)) if envs_idx is None else [int(e) for e in np.atleast_1d(envs_idx)])
        self._sim._cur_substep_global = 0

    def get_state(self) -> SimState:
        st = SimState(self._sim.cur_step_global, self._sim.cur_substep_local, self._sim.mpm_solver.get_state())
        return st

    # ------------------------------------------------------------------ checkpoints (scene.py:1381-1446)
    def dump_ckpt_to_numpy(self) -> dict:
        """Flat {"Class.attr[.member]": ndarray} of the physics state: the MPM solver's particle state
        and gravity, and the simulator's substep counter."""
        arrays = {"Simulator._cur_substep_global": np.asarray(self._sim._cur_substep_global, dtype=np.int64)}
        if self._is_built:
            arrays.update(self._sim.mpm_solver.dump_ckpt_to_numpy())
        return arrays

    def save_checkpoint(self, path) -> None:
        """Pickle the full physics state to one file (scene.py:1402-1417)."""
        import pickle
        import time

        state = {"timestamp": time.time(), "step_index": self.t, "arrays": self.dump_ckpt_to_numpy()}
        with open(path, "wb") as f:
            pickle.dump(state, f)

    def load_checkpoint(self, path) -> None:
        """Restore a file written by save_checkpoint (scene.py:1419-1446)."""
        import pickle

        with open(path, "rb") as f:
            state = pickle.load(f)
        arrays = state["arrays"]
        self._sim.mpm_solver.load_ckpt_from_numpy(arrays)
        if "Simulator._cur_substep_global" in arrays:
            self._sim._cur_substep_global = int(arrays["Simulator._cur_substep_global"])

    # ------------------------------------------------------------------ lookup
    @property
    def entity_names(self) -> tuple:
        return tuple(e.name for e in self._entities)

    def get_entity(self, name=None, *, uid=None):
        """By exact name or by uid (scene.py:1556-1592); raises when not found."""
        if (name is None) == (uid is None):
            raise GenesisException("Pass exactly one of `name` or `uid`.")
        for e in self._entities:
            if (name is not None and e.name == name) or (uid is not None and str(e.uid).startswith(str(uid))):
                return e
        raise GenesisException(f"Entity not found: {name if name is not None else uid}.")

    @property
    def gravity(self):
        return self._sim.mpm_solver.gravity

    def destroy(self) -> None:
        """Release the device state (scene.py:304-318)."""
        if self._sim is not None and self._is_built:
            self._sim.mpm_solver.destroy()
        self._is_built = False

    # ------------------------------------------------------------------ properties
    @property
    def sim(self):
        return self._sim

    @property
    def entities(self):
        return self._entities

    @property
    def is_built(self):
        return self._is_built

    @property
    def n_envs(self):
        return self._n_envs

    @property
    def dt(self):
        return self._sim.dt

    @property
    def substeps(self):
        return self._sim.substeps

    @property
    def requires_grad(self):
        return self._sim.requires_grad

    @property
    def t(self):
        return self._sim.cur_step_global

    @property
    def mpm_solver(self):
        return self._sim.mpm_solver
