"""MPMSolver: the drop-in for genesis/engine/solvers/mpm_solver.py::MPMSolver.

Keeps the reference solver's construction, properties and Solver-protocol methods
(build, add_entity, add_material, substep_pre_coupling/substep_post_coupling, get_state,
set_state, set_gravity, ...) and runs every substep through libgbmpm.so.  Each reference
env is one scene of the library context.
"""

from __future__ import annotations

import ctypes
import warnings

import numpy as np
import torch

from . import _lib
from .exceptions import GenesisException
from .states import MPMSolverState


class CubeBoundary:
    """genesis/engine/boundaries/boundaries.py:10-32 (host-side description)."""

    def __init__(self, lower, upper, restitution=0.0):
        self.restitution = restitution
        self.upper = np.array(upper, dtype=np.float32)
        self.lower = np.array(lower, dtype=np.float32)
        assert (self.upper >= self.lower).all()

    def is_inside(self, pos) -> bool:
        return bool(np.all(pos < self.upper) and np.all(pos > self.lower))

    def __repr__(self):
        return f"CubeBoundary(lower={self.lower.tolist()}, upper={self.upper.tolist()})"


def gs_exc(msg: str):
    raise GenesisException(msg)


def _stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _DeviceArray:
    """A device buffer of the library seen by torch without a copy (CUDA array interface)."""

    def __init__(self, ptr: int, shape, typestr: str = "<f4"):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2}


class MPMSolver:
    def __init__(self, scene, sim, options):
        import genesis_gb300 as gs

        self._scene = scene
        self._sim = sim
        self._options = options
        self._dt = options.dt
        self._substep_dt = options.dt / sim.substeps
        self._init_gravity = options.gravity
        self._entities = []
        self._tools = []  # genesis_gb300.tool.ToolEntity (colliders of shape "tool", after the user's)
        self._user_colliders = []
        self._tool_floor = 0.0
        self._materials = []
        self._materials_idx = []
        self._ctx = None
        self._diff = None  # differentiable mode (requires_grad): genesis_gb300.grad.SceneDiffEngine
        self._B = 1
        self._eps = gs.EPS
        # mpm_solver.py:36-80
        self._grid_density = options.grid_density
        self._particle_size = options.particle_size
        self._upper_bound = np.array(options.upper_bound)
        self._lower_bound = np.array(options.lower_bound)
        self._enable_CPIC = options.enable_CPIC
        self._particle_volume_real = float(self._particle_size**3)
        self._particle_volume_scale = 1e3
        self._particle_volume = self._particle_volume_real * self._particle_volume_scale
        self._dx = float(1.0 / self._grid_density)
        self._inv_dx = float(self._grid_density)
        self._lower_bound_cell = np.round(self._grid_density * self._lower_bound).astype(np.int32)
        self._upper_bound_cell = np.round(self._grid_density * self._upper_bound).astype(np.int32)
        self._grid_res = self._upper_bound_cell - self._lower_bound_cell + 1
        self._grid_offset = self._lower_bound_cell.copy()
        if np.prod(self._grid_res.astype(np.float64)) > 1e9:
            raise GenesisException(
                "Grid size larger than 1e9 not supported by MPM solver. Please reduce 'grid_density', or set tighter "
                "boundaries via 'lower_bound' / 'upper_bound'."
            )
        self.boundary_padding = 3 * self._dx
        self.boundary = CubeBoundary(
            lower=self._lower_bound + self.boundary_padding, upper=self._upper_bound - self.boundary_padding
        )
        self._gravity = None

    # ------------------------------------------------------------------ entities / materials
    @property
    def is_active(self) -> bool:
        return self.n_particles > 0

    def add_material(self, material):
        """mpm_solver.py:272-283: dedupe equal materials, assign material.idx."""
        for m in self._materials:
            if material == m:
                material.idx = m.idx
                break
        else:
            material.idx = len(self._materials_idx)
            self._materials_idx.append(material.idx)
        self._materials.append(material)

    def add_entity(self, idx, material, morph, surface, name=None):
        from .entity import MPMEntity

        self.add_material(material)
        entity = MPMEntity(
            scene=self._scene,
            solver=self,
            material=material,
            morph=morph,
            surface=surface,
            particle_size=self._particle_size,
            idx=idx,
            particle_start=self.n_particles,
            name=name,
        )
        self._entities.append(entity)
        return entity

    def add_tool(self, idx, material, morph, surface=None, name=None):
        """A tool entity (ToolSolver.add_entity) coupled to the MPM particles in the grid op."""
        from .tool import ToolEntity

        tool = ToolEntity(self._scene, idx, self, material, morph, surface, name=name)
        self._tools.append(tool)
        return tool

    def _unique_materials(self):
        seen = {}
        for m in self._materials:
            seen.setdefault(m.idx, m)
        return [seen[i] for i in sorted(seen)]

    # ------------------------------------------------------------------ build
    def build(self, B: int) -> None:
        self._B = B
        if not self.is_active:
            return
        lib = _lib.load()
        n = self.n_particles
        if n * B * 3 > np.iinfo(np.int32).max:
            raise GenesisException("Particle count too large for int32 indexing.")
        g = np.asarray(self._init_gravity if self._init_gravity is not None else (0.0, 0.0, 0.0), dtype=np.float64)
        self._gravity = np.tile(g, (B, 1))
        cfgs = (_lib.MpmSceneConfig * B)()
        for b in range(B):
            c = cfgs[b]
            c.substep_dt = self._substep_dt
            for d in range(3):
                c.gravity[d] = float(g[d])
                c.lower_bound[d] = float(self._lower_bound[d])
                c.upper_bound[d] = float(self._upper_bound[d])
            c.grid_density = float(self._grid_density)
            c.particle_size = float(self._particle_size)
            c.mass_eps = float(self._eps)
            c.restitution = 0.0
            c.n_particles = n
        mats = self._unique_materials()
        mat_arr = (_lib.MpmMaterial * (len(mats) * B))()
        for b in range(B):
            for j, m in enumerate(mats):
                mat_arr[b * len(mats) + j] = m.to_c(b)
        ctx = ctypes.c_void_p()
        dev = torch.cuda.current_device()
        ret = lib.mpm_ctx_create(cfgs, B, mat_arr, len(mats) * B, dev, ctypes.byref(ctx))
        _lib.check(ret, None, "mpm_ctx_create")
        self._ctx = ctx
        self._lib = lib
        # dt stability warning (mpm_solver.py:230-235)
        suggested_dt = 2e-2 * self._dx
        if self._substep_dt > suggested_dt:
            warnings.warn(
                f"Current `substep_dt` ({self._substep_dt:.6g}) is greater than suggested_dt ({suggested_dt:.6g}, "
                "calculated based on `grid_density`). Simulation might be unstable."
            )
        for entity in self._entities:
            entity._add_to_solver()
        if getattr(self, "_ffs", None):
            self._upload_force_fields()
        for t in self._tools:
            t._build(B, self._tool_floor)
        if self._tools:
            self._upload_colliders()
        if self._sim.requires_grad:  # the state lives in torch tensors advanced by the adjoint kernels
            from .grad import SceneDiffEngine

            self._diff = SceneDiffEngine(self, B)

    def _add_particles(self, particle_start, n, material_idx, active, pos_np):
        pos = torch.as_tensor(np.ascontiguousarray(pos_np, dtype=np.float32), device="cuda")
        ret = self._lib.mpm_add_particles(
            self._ctx, 0, self._B, particle_start, n, material_idx, int(active), _lib.ptr(pos), _stream_handle()
        )
        _lib.check(ret, self._ctx, "mpm_add_particles")
        torch.cuda.current_stream().synchronize()

    def destroy(self) -> None:
        if self._ctx is not None:
            self._lib.mpm_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # ------------------------------------------------------------------ stepping
    def process_input(self, in_backward=False):
        for e in self._entities:
            e.process_input(in_backward=in_backward)
        if any(t._pending() for t in self._tools):
            if self._diff is not None:  # the tools' state lives in the differentiable engine
                for t in self._tools:
                    t.process_input(in_backward=in_backward)
                return
            self._sync_tool_poses(user_too=True)
            for t in self._tools:
                t.process_input(in_backward=in_backward)
            self._upload_colliders()

    def substeps(self, n: int) -> None:
        """Run n fused substeps (no host sync).  In differentiable mode the n substeps are one autograd
        node per env (one scene.step())."""
        if self._diff is not None:
            self._diff.step(n)
            return
        if self._ctx is None:
            return
        if getattr(self, "_ff_plan", None):  # Custom force fields: the grid op in stages, per substep
            t0 = self._sim.cur_t
            for k in range(int(n)):
                self.substep_pre_coupling()
                self._staged_grid_op(t0 + k * self._substep_dt)
                self.substep_post_coupling()
            return
        _lib.check(self._lib.mpm_substeps(self._ctx, int(n), _stream_handle()), self._ctx, "mpm_substeps")

    def substep_pre_coupling(self, f=0):
        _lib.check(self._lib.mpm_substep_pre(self._ctx, _stream_handle()), self._ctx, "mpm_substep_pre")

    def couple(self, f=0):
        """LegacyCoupler.mpm_grid_op for MPM alone (legacy_coupler.py:356-501)."""
        if getattr(self, "_ff_plan", None):
            self._staged_grid_op(self._sim.cur_t)
            return
        _lib.check(self._lib.mpm_substep_grid_op(self._ctx, _stream_handle()), self._ctx, "mpm_substep_grid_op")

    def _staged_grid_op(self, t: float) -> None:
        """The grid op with Custom force fields (legacy_coupler.py:372-378 with the fields in list
        order): stage 1 applies gravity and the built-in fields before the first Custom one, each
        Custom field then acts on the node velocities in torch, stage 2 applies the built-in fields
        up to the next Custom one, stage 3 the colliders, coupling and boundary."""
        h = _stream_handle()
        first = True
        for step in self._ff_plan:
            if step[0] == "custom":
                self._apply_custom_field(step[1], t)
            elif first or step[2] > step[1]:
                _lib.check(self._lib.mpm_substep_grid_stage(self._ctx, 1 if first else 2, step[1], step[2], h),
                           self._ctx, "mpm_substep_grid_stage")
                first = False
        _lib.check(self._lib.mpm_substep_grid_stage(self._ctx, 3, 0, 0, h), self._ctx, "mpm_substep_grid_stage")

    def _grid_view(self):
        """(nodes [n, 4] float32 view of the current grid buffer, node positions [n, 3], node scene [n])."""
        ptr, count = ctypes.c_void_p(), ctypes.c_int64()
        _lib.check(self._lib.mpm_grid_nodes(self._ctx, ctypes.byref(ptr), ctypes.byref(count)), self._ctx,
                   "mpm_grid_nodes")
        n = int(count.value)
        if getattr(self, "_node_pos", None) is None or self._node_pos.shape[0] != n:
            self._node_pos = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            self._node_scene = torch.empty((n,), dtype=torch.int32, device="cuda")
            _lib.check(self._lib.mpm_grid_node_positions(self._ctx, _lib.ptr(self._node_pos), _lib.ptr(self._node_scene),
                                                         _stream_handle()), self._ctx, "mpm_grid_node_positions")
        nodes = torch.as_tensor(_DeviceArray(ptr.value, (n, 4)), device="cuda")
        return nodes, self._node_pos, self._node_scene

    def _apply_custom_field(self, ff, t: float) -> None:
        nodes, pos, scene = self._grid_view()
        sel = torch.nonzero((scene >= 0) & (nodes[:, 3] > self._eps)).squeeze(1)
        if sel.numel() == 0:
            return
        v = nodes.index_select(0, sel)[:, :3]
        acc = ff.get_acc(pos.index_select(0, sel), v.clone(), float(t), -1)
        acc = torch.as_tensor(acc, dtype=torch.float32, device=nodes.device).reshape(-1, 3)
        nodes[sel, :3] = v + acc * self._substep_dt

    def substep_post_coupling(self, f=0):
        _lib.check(self._lib.mpm_substep_post(self._ctx, _stream_handle()), self._ctx, "mpm_substep_post")

    def check_state(self) -> None:
        """Raise like mpm_solver.py:542-546 if any substep produced NaN (one host sync)."""
        if self._diff is not None:
            self._diff.check()
            return
        if self._ctx is None:
            return
        st = ctypes.c_uint32()
        ret = self._lib.mpm_status_word(self._ctx, ctypes.byref(st), None, 1, _stream_handle())
        _lib.check(ret, self._ctx, "mpm_status_word")
        if st.value & _lib.STATUS_NAN:
            raise GenesisException(
                "NaN detected in MPM states. Try reducing the time step size or adjusting simulation parameters."
            )
        if st.value & _lib.STATUS_OOB:
            raise GenesisException("MPM particles left the simulation grid (stencil out of bounds).")
        if st.value & _lib.STATUS_WAIT:
            raise GenesisException("MPM internal error: a bounded device-side wait ran out; the state is invalid.")

    def fp64_svd_count(self, reset: bool = False) -> int:
        st = ctypes.c_uint32()
        n = ctypes.c_int64()
        _lib.check(self._lib.mpm_status_word(self._ctx, ctypes.byref(st), ctypes.byref(n), int(reset), _stream_handle()))
        return n.value

    # ------------------------------------------------------------------ state io
    def get_state(self, f=None) -> MPMSolverState | None:
        if not self.is_active:
            return None
        s = MPMSolverState(self._B, self.n_particles, "cuda")
        if self._diff is not None:  # autograd-connected tensors (a loss on them back-propagates)
            s.pos, s.vel, s.C, s.F, s.Jp = self._diff.stacked()
            s.active = torch.ones((self._B, self.n_particles), dtype=torch.bool, device="cuda")
            self._diff.queried.append((self._diff.substeps_taken, s, 0))
            return s
        ret = self._lib.mpm_get_state(
            self._ctx, 0, self._B, _lib.ptr(s.pos), _lib.ptr(s.vel), _lib.ptr(s.C), _lib.ptr(s.F), _lib.ptr(s.Jp),
            _lib.ptr(s.active), _stream_handle()
        )
        _lib.check(ret, self._ctx, "mpm_get_state")
        return s

    def set_state(self, f, state, envs_idx=None) -> None:
        if not self.is_active:
            return
        if self._diff is not None:
            envs = list(range(self._B)) if envs_idx is None else [int(e) for e in np.atleast_1d(envs_idx)]
            self._diff.set_from_state(state, envs)
            return

        def dev(t, dtype=torch.float32):
            return None if t is None else t.detach().to(device="cuda", dtype=dtype).contiguous()

        pos, vel, C, F, Jp = (dev(getattr(state, k)) for k in ("pos", "vel", "C", "F", "Jp"))
        act = dev(state.active, torch.uint8)
        ret = self._lib.mpm_set_state(
            self._ctx, 0, self._B, _lib.ptr(pos), _lib.ptr(vel), _lib.ptr(C), _lib.ptr(F), _lib.ptr(Jp), _lib.ptr(act),
            _stream_handle()
        )
        _lib.check(ret, self._ctx, "mpm_set_state")
        torch.cuda.current_stream().synchronize()

    def get_grid(self, scene: int = 0) -> torch.Tensor:
        """Dense [gx, gy, gz, 4] grid of one env (momentum+mass after P2G, velocity+mass after the grid op)."""
        res = (ctypes.c_int32 * 3)()
        _lib.check(self._lib.mpm_scene_grid_res(self._ctx, scene, res), self._ctx, "mpm_scene_grid_res")
        out = torch.empty((res[0], res[1], res[2], 4), dtype=torch.float32, device="cuda")
        _lib.check(self._lib.mpm_get_grid(self._ctx, scene, _lib.ptr(out), _stream_handle()), self._ctx, "mpm_get_grid")
        return out

    # ------------------------------------------------------------------ Solver protocol members
    def init_ckpt(self):
        """mpm_solver.py:165-166."""
        self._ckpt = dict()

    def save_ckpt(self, ckpt_name):
        """mpm_solver.py:676-701: keep a copy of the current state under `ckpt_name`.  The
        reference keeps it only in differentiable mode (its frames hold the state otherwise);
        here it is always kept, so load_ckpt restores it."""
        if not hasattr(self, "_ckpt"):
            self.init_ckpt()
        st = self.get_state()
        if st is not None:
            self._ckpt[ckpt_name] = st

    def load_ckpt(self, ckpt_name):
        """mpm_solver.py:703-721."""
        ck = getattr(self, "_ckpt", {}).get(ckpt_name)
        if ck is not None:
            self.set_state(0, ck)

    def _is_state_valid(self, f=0) -> bool:
        """mpm_solver.py:484-489 (one host sync on the device status word)."""
        st = ctypes.c_uint32()
        _lib.check(self._lib.mpm_status_word(self._ctx, ctypes.byref(st), None, 0, _stream_handle()), self._ctx,
                   "mpm_status_word")
        return not (st.value & _lib.STATUS_NAN)

    # The reference's per-kernel launch methods map onto the fused split phases: p2g runs
    # compute_F_tmp + svd + material update + scatter in one kernel, g2p the gather and re-sort.
    def p2g(self, f=0):
        self.substep_pre_coupling(f)

    def g2p(self, f=0):
        self.substep_post_coupling(f)

    def setup_boundary(self):
        pad = 3 * self._dx
        self.boundary_padding = pad
        self.boundary = CubeBoundary(np.asarray(self._lower_bound) + pad, np.asarray(self._upper_bound) - pad)

    @property
    def stencil_range(self):
        return [(i, j, k) for i in range(3) for j in range(3) for k in range(3)]

    @property
    def is_built(self):
        return self._ctx is not None

    @property
    def n_vverts(self):
        return sum(e.n_vverts for e in self._entities)

    @property
    def n_vfaces(self):
        return 0  # visual faces come from meshes, which this path does not load

    @property
    def enable_particle_constraints(self):
        return getattr(self, "_constraints_used", False)

    # Differentiable mode: gradients come from genesis_gb300.diff.DifferentiableMPM (hand-written
    # adjoint kernels); the autodiff entry points of the reference are not available here.
    def _no_grad(self, *args, **kwargs):
        raise GenesisException(
            "Differentiable mode runs through genesis_gb300.diff.DifferentiableMPM (hand-written adjoints)."
        )

    substep_pre_coupling_grad = substep_post_coupling_grad = process_input_grad = _no_grad
    add_grad_from_state = collect_output_grads = reset_grad = reset_grad_till_frame = _no_grad

    # ------------------------------------------------------------------ force fields
    def _add_force_field(self, ff) -> None:
        if not hasattr(self, "_ffs"):
            self._ffs = []
        self._ffs.append(ff)
        ff._solver = self
        if self._ctx is not None:
            self._upload_force_fields()

    def _upload_force_fields(self) -> None:
        """Built-in fields go to the device in list order; Custom ones split that list into the
        stages of the grid op (the plan _staged_grid_op follows)."""
        from .force_fields import Custom

        ffs = getattr(self, "_ffs", [])
        if self._ctx is None:
            return
        recs, plan, begin = [], [], 0
        for f in ffs:
            if isinstance(f, Custom):
                plan += [("fields", begin, len(recs)), ("custom", f)]
                begin = len(recs)
            else:
                recs.append(f.to_c())
        plan.append(("fields", begin, len(recs)))
        self._ff_plan = plan if len(plan) > 1 else None
        if getattr(self, "_diff", None) is not None:  # the differentiable steps take the fields from here on
            self._diff.set_force_fields(ffs)
        arr = (_lib.MpmForceField * max(1, len(recs)))(*recs)
        _lib.check(self._lib.mpm_set_force_fields(self._ctx, len(recs), arr), self._ctx, "mpm_set_force_fields")

    # ------------------------------------------------------------------ rigid coupling
    def set_colliders(self, colliders) -> None:
        """Kinematic rigid colliders coupled in the grid op (genesis_gb300.coupling.Collider list;
        call again whenever they move).  Shapes "sdf" and "tool" carry an SDFGrid, uploaded to the
        device once per grid object; tools then move by themselves every substep (see
        get_collider_poses).  The scene's tool entities follow these colliders in the library's
        list and keep their current poses."""
        if self._diff is not None and any(c.shape == "tool" for c in colliders):
            raise GenesisException("Collider shape 'tool' is not supported in differentiable mode; add a tool entity.")
        self._sync_tool_poses()
        self._user_colliders = list(colliders)
        self._upload_colliders()

    def _sync_tool_poses(self, user_too: bool = False) -> None:
        """Read back the poses the library advanced: every tool entity's, and with user_too the
        user colliders of shape "tool" (before their list is uploaded again unchanged)."""
        if self._ctx is None or not getattr(self, "_n_colliders", 0):
            return
        poses = self.get_collider_poses()
        for t in self._tools:
            t._sync_pose(poses)
        if user_too:
            from .tool import replace_pose

            self._user_colliders = [replace_pose(c, poses[i]) if c.shape == "tool" else c
                                    for i, c in enumerate(self._user_colliders)]

    def _upload_colliders(self, sync: bool = False) -> None:
        if sync:
            self._sync_tool_poses(user_too=True)
        colliders = list(self._user_colliders)
        for t in self._tools:
            t._col0 = len(colliders)
            colliders += t._colliders()
        if not hasattr(self, "_sdf_ids"):
            self._sdf_ids = {}  # id(SDFGrid) -> (grid, library grid id)
        ids = []
        for c in colliders:
            if c.sdf is None:
                ids.append(-1)
                continue
            hit = self._sdf_ids.get(id(c.sdf))
            if hit is None or hit[0] is not c.sdf:
                g = c.sdf
                vals = np.ascontiguousarray(g.values, np.float32)
                grads = None if g.grads is None else np.ascontiguousarray(g.grads, np.float32)
                res = np.asarray(vals.shape, np.int32)
                T = np.ascontiguousarray(g.T_mesh_to_sdf, np.float64)
                out = ctypes.c_int32()
                _lib.check(self._lib.mpm_add_sdf_grid(self._ctx, res.ctypes.data, vals.ctypes.data,
                                                      None if grads is None else grads.ctypes.data, T.ctypes.data,
                                                      float(g.cell_size), float(g.sdf_max), ctypes.byref(out)),
                           self._ctx, "mpm_add_sdf_grid")
                hit = (g, out.value)
                self._sdf_ids[id(g)] = hit
            ids.append(hit[1])
        recs = [c.to_c(i) for c, i in zip(colliders, ids)]
        arr = (_lib.MpmCollider * max(1, len(recs)))(*recs)
        if self._enable_CPIC and len(recs) > getattr(self, "_cpic_slots", 0):
            # CPIC (mpm_solver.py:389-411, 445-459): one slot of particle-side normals per collider;
            # growing the slots starts every particle's normals afresh, as the coupler's build does
            _lib.check(self._lib.mpm_enable_cpic(self._ctx, len(recs), _stream_handle()), self._ctx,
                       "mpm_enable_cpic")
            self._cpic_slots = len(recs)
        _lib.check(self._lib.mpm_set_colliders(self._ctx, len(recs), arr), self._ctx, "mpm_set_colliders")
        self._n_colliders = len(recs)
        if getattr(self, "_diff", None) is not None:  # the differentiable steps take the user colliders
            self._diff.set_colliders(recs[:len(self._user_colliders)])

    # ------------------------------------------------------------------ numpy checkpoints (base_solver.py:63-126)
    def dump_ckpt_to_numpy(self) -> dict:
        """{"MPMSolver.particles.<field>": [B, N, ...], "MPMSolver._gravity": [B, 3]} of the current state
        (the particle state the reference's fields hold at the current frame; muscle actuation and
        directions too when a Muscle material is present)."""
        out = {}
        if not self.is_active:
            return out
        st = self.get_state()
        for k in ("pos", "vel", "C", "F", "Jp", "active"):
            out[f"MPMSolver.particles.{k}"] = getattr(st, k).detach().cpu().numpy()
        out["MPMSolver._gravity"] = np.asarray(self.gravity, dtype=np.float64)
        from .materials import Muscle

        if any(isinstance(e.material, Muscle) for e in self._entities):
            for e in self._entities:
                out[f"MPMSolver.entity{e.idx}.actu"] = e._get_field(_lib.FIELD_ACTU, 1, None).cpu().numpy()
                out[f"MPMSolver.entity{e.idx}.muscle_direction"] = e._get_field(_lib.FIELD_MUSCLE_DIR, 3, None).cpu().numpy()
        return out

    def load_ckpt_from_numpy(self, arr_dict: dict) -> None:
        if not self.is_active:
            return
        keys = ("pos", "vel", "C", "F", "Jp", "active")
        if all(f"MPMSolver.particles.{k}" in arr_dict for k in keys):
            st = MPMSolverState(self._B, self.n_particles, "cuda")
            for k in keys:
                v = torch.as_tensor(arr_dict[f"MPMSolver.particles.{k}"], device="cuda")
                setattr(st, k, v.to(getattr(st, k).dtype).reshape(getattr(st, k).shape))
            self.set_state(0, st)
        if "MPMSolver._gravity" in arr_dict:
            self.set_gravity(arr_dict["MPMSolver._gravity"])
        for e in self._entities:
            a = arr_dict.get(f"MPMSolver.entity{e.idx}.actu")
            if a is not None:
                e._write(_lib.FIELD_ACTU, e._envs(None), torch.as_tensor(a, device="cuda").contiguous())
            d = arr_dict.get(f"MPMSolver.entity{e.idx}.muscle_direction")
            if d is not None:
                e._write(_lib.FIELD_MUSCLE_DIR, e._envs(None), torch.as_tensor(d, device="cuda").contiguous())

    # ------------------------------------------------------------------ differentiable-mode protocol members
    # loss.backward() on states from get_state() needs none of these: every scene.step() is a torch
    # autograd node (genesis_gb300.grad).  They replay the reference's imperative walk
    # (Scene._backward -> Simulator._step_grad, simulator.py:298-370) for callers that drive it.
    def _engine(self):
        if self._diff is None:
            raise GenesisException("Gradient members need SimOptions(requires_grad=True).")
        return self._diff

    def reset_grad(self):
        """mpm_solver.py:194-199: zero the solver's adjoint; the walk starts at the current substep."""
        self._engine().reset_grad()

    def reset_grad_till_frame(self, f=None):
        """mpm_solver.py:589-601."""
        self._engine().reset_grad()

    def add_grad_from_state(self, state):
        """mpm_solver.py:614-670: add state.pos/vel/C/F .grad into the adjoint of the current substep."""
        self._engine().add_grad({k: (getattr(getattr(state, k), "grad", None), 0) for k in ("pos", "vel", "C", "F", "Jp")})

    def collect_output_grads(self):
        """mpm_solver.py:607-612: the gradients of states queried (get_state) at the current substep."""
        eng = self._engine()
        for f_q, st, start in eng.queried:
            if f_q == eng.cursor:
                eng.add_grad({k: (getattr(getattr(st, k), "grad", None), start)
                              for k in ("pos", "vel", "C", "F", "Jp")})
        for f_q, st, t in eng.queried_tools:  # ToolEntity.collect_output_grads
            if f_q == eng.cursor:
                eng.add_tool_grad(t, getattr(st.pos, "grad", None), getattr(st.vel, "grad", None))

    def substep_post_coupling_grad(self, f=0):
        """g2p.grad (mpm_solver.py:548-554); the grid-op and P2G adjoints of the same substep run in the
        same library call (mpm_diff_backward_seq_pp), so substep_pre_coupling_grad has nothing left."""
        self._engine().substep_grad()

    def substep_pre_coupling_grad(self, f=0):
        """p2g.grad / svd_grad / compute_F_tmp.grad (mpm_solver.py:517-528): done by the preceding
        substep_post_coupling_grad call."""
        self._engine()

    def process_input_grad(self):
        """mpm_solver.py:499-501: the adjoint at the step start goes back to the entity inputs."""
        self._engine().input_grad()

    @property
    def scene(self):
        return self._scene

    @property
    def sim(self):
        return self._sim

    @property
    def uid(self):
        return id(self)

    @property
    def leaf_block_size(self):
        """Removed in the reference (mpm_solver.py:1172-1174), which raises."""
        from .exceptions import DeprecationError

        raise DeprecationError("This property has been removed.")

    @property
    def use_sparse_grid(self):
        """Removed in the reference (mpm_solver.py:1176-1178), which returns the error object."""
        from .exceptions import DeprecationError

        return DeprecationError("This property has been removed.")

    def get_collider_poses(self) -> np.ndarray:
        """[n_colliders, 7]: current position and quaternion (w, x, y, z) of each collider; tools
        have advanced one substep per substep since set_colliders."""
        n = getattr(self, "_n_colliders", 0)
        out = np.zeros((max(1, n), 7), dtype=np.float64)
        _lib.check(self._lib.mpm_get_collider_poses(self._ctx, out.ctypes.data, _stream_handle()), self._ctx,
                   "mpm_get_collider_poses")
        return out[:n]

    def get_collider_forces(self, reset: bool = True) -> np.ndarray:
        """[n_colliders, 6]: force (xyz) and torque about each collider's com exerted by the
        particles, summed over the substeps since the last reset."""
        if self._diff is not None:
            raise GenesisException("Collider reaction forces are not accumulated in differentiable mode.")
        n = getattr(self, "_n_colliders", 0)
        out = np.zeros((max(1, n), 6), dtype=np.float64)
        _lib.check(self._lib.mpm_get_collider_forces(self._ctx, out.ctypes.data, int(reset), _stream_handle()),
                   self._ctx, "mpm_get_collider_forces")
        return out[:n]

    # ------------------------------------------------------------------ SPH / PBD coupling
    def set_coupled_particles(self, kind: str, pos=None, vel=None, mass=None, free=None) -> None:
        """Couple another solver's particles through the grid op (legacy_coupler.py:404-498).

        kind 'sph' or 'pbd'; pos and vel float32 CUDA tensors [B, n, 3] ([n, 3] with one env),
        mass float32 [B, n] ([n]), free uint8 [B, n] ([n]; PBD only, None: all free).  A node with
        MPM mass takes the mean velocity of the set's particles in its cell and gives each of them
        back the momentum change; vel is updated in place by every grid op.  The tensors stay
        referenced here (and must not be reallocated) until the set is replaced or removed with
        pos=None."""
        k = {"sph": 0, "pbd": 1}.get(kind)
        if k is None:
            gs_exc(f"Unsupported coupled particle kind: {kind!r} (expected 'sph' or 'pbd').")
        if self._diff is not None and pos is not None:
            gs_exc("MPM <-> SPH / PBD coupling is not supported in differentiable mode.")
        if not hasattr(self, "_coupled"):
            self._coupled = [None, None]
        if pos is None:
            _lib.check(self._lib.mpm_set_coupled_particles(self._ctx, k, 0, None, None, None, None, _stream_handle()),
                       self._ctx, "mpm_set_coupled_particles")
            self._coupled[k] = None
            return
        B = self._B

        def arr(t, name, width, dtype):
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == dtype and t.is_contiguous()):
                gs_exc(f"{name} must be a contiguous {dtype} CUDA tensor")
            shape = tuple(t.shape)
            tail = (width,) if width else ()
            if len(shape) == 1 + len(tail) and B == 1:
                shape = (1,) + shape
            if len(shape) != 2 + len(tail) or shape[0] != B or shape[2:] != tail:
                gs_exc(f"{name} must be [B, n{', %d' % width if width else ''}] with B = {B}")
            return shape[1]

        n = arr(pos, "pos", 3, torch.float32)
        if arr(vel, "vel", 3, torch.float32) != n or arr(mass, "mass", 0, torch.float32) != n:
            gs_exc("pos, vel and mass must hold the same particles")
        if free is not None and arr(free, "free", 0, torch.uint8) != n:
            gs_exc("free must hold the same particles as pos")
        _lib.check(self._lib.mpm_set_coupled_particles(
            self._ctx, k, n, pos.data_ptr(), vel.data_ptr(), mass.data_ptr(),
            None if free is None or k == 0 else free.data_ptr(), _stream_handle()), self._ctx,
            "mpm_set_coupled_particles")
        self._coupled[k] = (pos, vel, mass, free)

    # ------------------------------------------------------------------ kinematic links
    def set_link_poses(self, pos, quat) -> None:
        """Poses of the links that particle constraints follow (the reference reads them from the
        rigid solver's links_state): pos [B, L, 3] or [L, 3], quat (w, x, y, z) [B, L, 4] or [L, 4]."""
        p = np.asarray(pos, dtype=np.float32)
        q = np.asarray(quat, dtype=np.float32)
        if p.ndim == 2:
            p = np.broadcast_to(p, (self._B,) + p.shape)
            q = np.broadcast_to(q, (self._B,) + q.shape)
        if p.shape[0] != self._B or q.shape[:2] != p.shape[:2] or p.shape[2] != 3 or q.shape[2] != 4:
            gs_exc("link poses must be [B, L, 3] and [B, L, 4]")
        self._link_pos, self._link_quat = np.ascontiguousarray(p), np.ascontiguousarray(q)
        table = np.ascontiguousarray(np.concatenate([p, q], axis=2), dtype=np.float32)
        _lib.check(self._lib.mpm_set_link_poses(self._ctx, p.shape[1], table.ctypes.data), self._ctx,
                   "mpm_set_link_poses")

    def get_link_pose(self, link_idx: int):
        lp = getattr(self, "_link_pos", None)
        if lp is None or not 0 <= link_idx < lp.shape[1]:
            gs_exc(f"link {link_idx} has no pose; call set_link_poses first")
        return self._link_pos[:, link_idx], self._link_quat[:, link_idx]

    # ------------------------------------------------------------------ render fields
    @property
    def n_vvert_supports(self) -> int:
        vis = getattr(self._scene, "vis_options", None)
        return int(vis.n_support_neighbors) if vis is not None else 12  # VisOptions default (options/vis.py:157)

    def _vverts_changed(self) -> None:
        self._vvert_dev = None

    def update_render_fields(self) -> None:
        """mpm_solver.py:780-803: fills `particles_render` ({pos, vel, active}, [B, N, ...]; inactive
        particles at the reference's nowhere point) and `vverts_render` ({pos, active}, [B, V, ...])
        from the current state, on the device."""
        B, N = self._B, self.n_particles
        if getattr(self, "_render", None) is None or self._render["pos"].shape[:2] != (B, N):
            self._render = {"pos": torch.empty((B, N, 3), device="cuda"), "vel": torch.empty((B, N, 3), device="cuda"),
                            "active": torch.empty((B, N), dtype=torch.bool, device="cuda")}
        ents = [e for e in self._entities if e.n_vverts > 0]
        if getattr(self, "_vvert_dev", None) is None:
            if ents:
                k = max(e._vvert_support_idx.shape[1] for e in ents)
                idx = np.concatenate([np.pad(e._vvert_support_idx, ((0, 0), (0, k - e._vvert_support_idx.shape[1])),
                                             mode="edge") for e in ents])
                w = np.concatenate([np.pad(e._vvert_support_w, ((0, 0), (0, k - e._vvert_support_w.shape[1])))
                                    for e in ents])
                self._vvert_dev = (torch.as_tensor(idx, device="cuda").contiguous(),
                                   torch.as_tensor(w, device="cuda").contiguous())
            else:
                self._vvert_dev = (None, None)
        sidx, sw = self._vvert_dev
        V = 0 if sidx is None else sidx.shape[0]
        vpos = torch.empty((B, V, 3), device="cuda")
        vact = torch.empty((B, V), dtype=torch.bool, device="cuda")
        _lib.check(self._lib.mpm_render_fields(
            self._ctx, 0, B, _lib.ptr(self._render["pos"]), _lib.ptr(self._render["vel"]), _lib.ptr(self._render["active"]),
            V, 0 if sidx is None else sidx.shape[1], None if sidx is None else _lib.ptr(sidx),
            None if sw is None else _lib.ptr(sw), _lib.ptr(vpos) if V else None, _lib.ptr(vact) if V else None,
            _stream_handle()), self._ctx, "mpm_render_fields")
        self._vverts_render = {"pos": vpos, "active": vact}

    @property
    def particles_render(self):
        return self._render

    @property
    def vverts_render(self):
        return self._vverts_render

    def set_gravity(self, gravity, envs_idx=None) -> None:
        g = np.asarray(gravity, dtype=np.float64).reshape(-1, 3)
        envs = list(range(self._B)) if envs_idx is None else [int(e) for e in np.atleast_1d(envs_idx)]
        if g.shape[0] == 1:
            g = np.tile(g, (len(envs), 1))
        for i, e in enumerate(envs):
            self._gravity[e] = g[i]
            arr = (ctypes.c_double * 3)(*g[i])
            _lib.check(self._lib.mpm_set_gravity(self._ctx, e, e + 1, arr), self._ctx, "mpm_set_gravity")

    def get_gravity(self, envs_idx=None):
        return None if self._gravity is None else self._gravity.copy()

    # field helpers used by entities
    def _field(self, field, write, s0, s1, start, n, data):
        fn = self._lib.mpm_set_particles if write else self._lib.mpm_get_particles
        _lib.check(fn(self._ctx, field, s0, s1, start, n, _lib.ptr(data), _stream_handle()), self._ctx, "particles")

    # ------------------------------------------------------------------ properties
    @property
    def n_particles(self) -> int:
        return sum(e.n_particles for e in self._entities)

    @property
    def entities(self):
        return self._entities

    @property
    def n_entities(self):
        return len(self._entities)

    @property
    def dt(self):
        return self._dt

    @property
    def substep_dt(self):
        return self._substep_dt

    @property
    def grid_density(self):
        return self._grid_density

    @property
    def particle_size(self):
        return self._particle_size

    @property
    def particle_radius(self):
        return self._particle_size / 2.0

    @property
    def upper_bound(self):
        return self._upper_bound

    @property
    def lower_bound(self):
        return self._lower_bound

    @property
    def dx(self):
        return self._dx

    @property
    def inv_dx(self):
        return self._inv_dx

    @property
    def particle_volume_real(self):
        return self._particle_volume_real

    @property
    def particle_volume(self):
        return self._particle_volume

    @property
    def particle_volume_scale(self):
        return self._particle_volume_scale

    @property
    def lower_bound_cell(self):
        return self._lower_bound_cell

    @property
    def upper_bound_cell(self):
        return self._upper_bound_cell

    @property
    def grid_res(self):
        return self._grid_res

    @property
    def grid_offset(self):
        return self._grid_offset

    @property
    def enable_CPIC(self):
        return self._enable_CPIC

    @property
    def gravity(self):
        return self._gravity

    @property
    def ctx(self):
        return self._ctx
