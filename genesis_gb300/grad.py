"""Differentiable mode of the scene API (`SimOptions(requires_grad=True)`).

The reference differentiates `scene.step()` with Quadrants autodiff: states queried with
`get_state()` are `gs.Tensor`s whose backward hook runs `Scene._backward`, which walks the
steps in reverse (Simulator._step_grad: load_ckpt, re-simulate the step, then
substep_post_coupling_grad / couple_grad / substep_pre_coupling_grad per substep,
process_input_grad), scene.py:1365-1379, simulator.py:298-404, mpm_solver.py:517-670.

Here the same user-facing flow (entity.set_position / set_velocity / set_actuation and
tool.set_position / set_velocity with tensors that require grad, scene.step(), get_state(),
loss.backward()) runs on torch autograd.  The state of every env is a set of torch tensors:
particles (x, v, C, F, Jp), the tools' position and velocity ([n_tools, 6]) and the Muscle
actuation ([N], constant over a step).  Every scene.step() is one autograd node per env whose
forward runs the step's substeps with the libgbmpm differentiable kernels
(mpm_diff_forward_seq_ex) and whose backward re-simulates the step from its input state (the
checkpoint, as the reference's save_ckpt / load_ckpt keep one per step) and runs the hand-written
adjoint substeps in reverse (mpm_diff_backward_seq_ex).  Entity inputs set between steps enter the
state through differentiable torch ops, so their gradients arrive where the reference's
process_input_grad puts them; the Solver protocol's *_grad members walk the same adjoint
imperatively.

What a step differentiates: every MPM material (Elastic corotated or neo-Hookean, Liquid, Sand,
Snow, ElastoPlastic clamped or von Mises, Muscle; any mix, per-particle constants); tool entities
(Mesh.collide in the grid op and ToolEntity.advect; orientation and angular velocity are carried
as plain tensors); built-in force fields; kinematic rigid colliders (solver.set_colliders, poses
fixed within a step, no reaction forces in this mode); particle constraints (springs towards the
links' poses of solver.set_link_poses); and Custom force fields (a torch function, run between
grid stages of the substep with mpm_diff_substep_stage, its Jacobian taken by torch autograd in
the adjoint).  Each step keeps the fields, colliders, constraint targets and particle activity it
ran with.  As in the reference, CPIC and emitters are rejected in this mode.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .exceptions import GenesisException

KIND_COROTATED, KIND_NEOHOOKEAN, KIND_LIQUID, KIND_SAND, KIND_SNOW = 0, 1, 2, 3, 4
KIND_MUSCLE_COROTATED, KIND_MUSCLE_NEOHOOKEAN, KIND_EP_CLAMP, KIND_EP_VON_MISES = 5, 6, 7, 8
FIELDS = ("pos", "vel", "C", "F", "Jp")
_WIDTH = (3, 3, 9, 9, 1)       # floats per particle of each state field
_OFFSET = (0, 3, 6, 15, 24)    # offsets (in units of n) in the packed gradient buffer of 25 n floats


def material_kind(material) -> tuple[int, float, float]:
    """(kind, aux0, aux1) of a material in differentiable mode."""
    from .materials import Elastic, ElastoPlastic, Liquid, Muscle, Sand, Snow

    if type(material) is Elastic:
        return (KIND_NEOHOOKEAN if material.model == "neohooken" else KIND_COROTATED), 0.0, 0.0
    if type(material) is Muscle:  # aux: the actuation stiffness (muscle.py: stiffness = E)
        kind = KIND_MUSCLE_NEOHOOKEAN if material.model == "neohooken" else KIND_MUSCLE_COROTATED
        return kind, float(material.stiffness), 0.0
    if type(material) is ElastoPlastic:  # the product path's material record (clamp bounds | yield ratio)
        if material.use_von_mises:
            return KIND_EP_VON_MISES, float(material.von_mises_yield_stress) / (2.0 * float(material.mu)), 0.0
        return KIND_EP_CLAMP, 1.0 - float(material.yield_lower), 1.0 + float(material.yield_higher)
    if type(material) is Liquid:
        return KIND_LIQUID, 0.0, 0.0
    if type(material) is Sand:
        return KIND_SAND, float(material.alpha), 0.0
    if type(material) is Snow:
        return KIND_SNOW, 1.0 - float(material.yield_lower), 1.0 + float(material.yield_higher)
    raise GenesisException(
        f"{type(material).__name__} is not differentiable here: requires_grad=True supports the MPM materials "
        "Elastic, Liquid, Sand, Snow, ElastoPlastic and Muscle."
    )


class _StepNode(torch.autograd.Function):
    """One scene.step() of one env: (x, v, C, F, Jp, tool pos/vel, actuation) -> the state after n_sub
    substeps, plus the tools' orientation and angular velocity (not differentiated)."""

    @staticmethod
    def forward(ctx, engine, n_sub, fields, qa, x, v, C, F, Jp, T, A):
        st = tuple(t.detach().float().contiguous() for t in (x, v, C, F, Jp, T, A))
        qa = qa.detach().float().contiguous()
        out, qa_end = engine.run_forward(st, n_sub, qa, fields)
        ctx.engine, ctx.n_sub, ctx.fields = engine, n_sub, fields
        ctx.save_for_backward(*st, qa)  # the step's checkpoint
        ctx.mark_non_differentiable(qa_end)
        return (*out, qa_end)

    @staticmethod
    def backward(ctx, gx, gv, gC, gF, gJp, gT, gA, _gqa):
        saved = ctx.saved_tensors
        grads = ctx.engine.run_backward(saved[:7], ctx.n_sub, (gx, gv, gC, gF, gJp, gT, gA), saved[7], ctx.fields)
        return (None, None, None, None, *grads)


class SceneDiffEngine:
    """The differentiable MPM state of a built scene: per env (x [N,3], v [N,3], C [N,3,3], F [N,3,3],
    Jp [N]) torch tensors; every particle active."""

    def __init__(self, solver, B: int):
        self.solver = solver
        self.lib = _lib.load()
        self.B = B
        ents = solver.entities
        n = solver.n_particles
        self.n = n
        kinds, mass, mu, lam, aux = [], [], [], [], []
        p_vol = solver.particle_volume
        for e in ents:
            m = e.material
            k, a0, a1 = material_kind(m)
            kinds.append(np.full(e.n_particles, k, np.int32))
            aux.append(np.tile(np.array([a0, a1], np.float32), (e.n_particles, 1)))
            mass.append(np.full(e.n_particles, p_vol * m.rho, np.float32))
            mu.append(np.full(e.n_particles, m.mu, np.float32))  # Liquid: 0 unless viscous (liquid.py:27-31)
            lam.append(np.full(e.n_particles, m.lam, np.float32))
        cat = lambda xs, dt: torch.as_tensor(np.concatenate(xs) if xs else np.zeros(0, dt), device="cuda")  # noqa: E731
        self.kind = cat(kinds, np.int32).contiguous()
        self.mass = cat(mass, np.float32).contiguous()
        self.mu = cat(mu, np.float32).contiguous()
        self.lam = cat(lam, np.float32).contiguous()
        self.aux = torch.as_tensor(np.concatenate(aux) if aux else np.zeros((0, 2), np.float32),
                                   device="cuda").contiguous()
        # Muscle particles: fibre direction (set_muscle; default +z as mpm_solver.py:825) and actuation
        self.has_muscle = bool(((self.kind == KIND_MUSCLE_COROTATED) | (self.kind == KIND_MUSCLE_NEOHOOKEAN)).any())
        self.mdir = torch.tensor([0.0, 0.0, 1.0], device="cuda").repeat(n, 1).contiguous()
        self.cfg = _lib.MpmSceneConfig()
        c = self.cfg
        c.substep_dt = solver.substep_dt
        g = solver.gravity[0]
        for d in range(3):
            c.gravity[d] = float(g[d])
            c.lower_bound[d] = float(solver.lower_bound[d])
            c.upper_bound[d] = float(solver.upper_bound[d])
        c.grid_density = float(solver.grid_density)
        c.particle_size = float(solver.particle_size)
        c.mass_eps = float(solver._eps)
        c.restitution = 0.0
        c.n_particles = n
        res = solver.grid_res
        self.nodes = int(res[0]) * int(res[1]) * int(res[2])
        dev = "cuda"
        self.g_grid_v = torch.zeros((self.nodes, 4), device=dev)
        self.g_grid_pm = torch.zeros((self.nodes, 4), device=dev)
        self.scratch = (torch.zeros((self.nodes, 4), device=dev), torch.zeros((self.nodes, 4), device=dev))
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        x0 = torch.as_tensor(np.concatenate([e.init_particles for e in ents]) if ents else np.zeros((0, 3)),
                             dtype=torch.float32, device=dev)
        eye = torch.eye(3, device=dev)
        self.Jp0 = torch.cat([torch.full((e.n_particles,), float(e.material._default_Jp), device=dev) for e in ents]) \
            if ents else torch.zeros(0, device=dev)
        self._init_tools(solver)
        self.set_force_fields(getattr(solver, "_ffs", []))
        self.set_colliders([])
        self.con_k = [torch.zeros(n, device="cuda") for _ in range(B)]   # constraint stiffness (0: none)
        self.con_link = [torch.full((n,), -1, dtype=torch.long, device="cuda") for _ in range(B)]
        self.con_local = [torch.zeros((n, 3), device="cuda") for _ in range(B)]
        self.has_con = False
        # particle activity (entity.set_active): a constant of each step, not differentiated
        self.active = [torch.ones(n, dtype=torch.uint8, device="cuda") for _ in range(B)]
        self.has_inactive = False
        self.states = [(x0.clone(), torch.zeros((n, 3), device=dev), torch.zeros((n, 3, 3), device=dev),
                        eye.repeat(n, 1, 1), self.Jp0.clone(), self.T0.clone(), torch.zeros(n, device=dev))
                       for _ in range(B)]
        self.tool_qa = [self.qa0.clone() for _ in range(B)]
        self.steps_taken = 0
        self.substeps_taken = 0
        self.step_inputs = []  # per step: (per-env state at the step start, substeps)
        self.adj = None        # imperative adjoint walk (Solver protocol members)
        self.cursor = 0
        self._seg = None
        self.queried = []      # (global substep, state, first row) returned by get_state, for collect_output_grads
        self.queried_tools = []  # (global substep, tool state, tool index) returned by ToolEntity.get_state
        self.pending = []      # entity inputs written since the last step: (field, start, count, values, envs)

    def _init_tools(self, solver) -> None:
        """The tools of the scene as the library's differentiable form takes them."""
        tools = list(getattr(solver, "_tools", []))
        if len(tools) > _lib.DIFF_MAX_TOOLS:
            raise GenesisException(f"At most {_lib.DIFF_MAX_TOOLS} tool entities in differentiable mode.")
        if any(t.sdf is None for t in tools):
            raise GenesisException("Tool entities without collision are not supported in differentiable mode.")
        self.tools = tools
        self.tool_sdf = [torch.as_tensor(t.sdf.values, dtype=torch.float32, device="cuda").contiguous() for t in tools]
        self.tool_recs = (_lib.MpmDiffTool * max(1, len(tools)))()
        for rec, t, sdf in zip(self.tool_recs, tools, self.tool_sdf):
            rec.sdf = sdf.data_ptr()
            rec.res[:] = tuple(int(r) for r in sdf.shape)
            rec.T_mesh_to_sdf[:] = tuple(float(v) for v in np.asarray(t.sdf.T_mesh_to_sdf, np.float64).reshape(-1))
            rec.friction = float(t.material.friction)
            rec.softness = float(t.material.coup_softness)
            rec.floor_height = float(solver._tool_floor)
        nt = len(tools)
        self.T0 = torch.zeros((nt, 6), device="cuda")
        self.qa0 = torch.zeros((nt, 7), device="cuda")
        for i, t in enumerate(tools):
            self.T0[i, :3] = torch.as_tensor(t.init_pos, dtype=torch.float32)
            self.qa0[i, :4] = torch.as_tensor(t.init_quat, dtype=torch.float32)

    def set_force_fields(self, ffs) -> None:
        """The scene's force fields for the following steps (their substep counter restarts, as the
        library's does when mpm_set_force_fields replaces them)."""
        from .force_fields import Custom

        recs, plan, begin = [], [], 0
        for f in ffs:  # Custom fields split the built-in ones into grid stages, as in the product path
            if isinstance(f, Custom):
                plan += [("fields", begin, len(recs)), ("custom", f)]
                begin = len(recs)
            else:
                recs.append(f.to_c())
        plan.append(("fields", begin, len(recs)))
        if len(recs) > _lib.DIFF_MAX_FORCE_FIELDS:
            raise GenesisException(f"At most {_lib.DIFF_MAX_FORCE_FIELDS} force fields in differentiable mode.")
        self.ff_recs = (_lib.MpmForceField * max(1, len(recs)))(*recs)
        self.n_ffs = len(recs)
        self.ff_plan = plan if len(plan) > 1 else None
        self.ff_base = getattr(self, "substeps_taken", 0)

    def set_colliders(self, recs) -> None:
        """The user colliders (MpmCollider records) for the following steps."""
        if len(recs) > _lib.DIFF_MAX_COLLIDERS:
            raise GenesisException(f"At most {_lib.DIFF_MAX_COLLIDERS} rigid colliders in differentiable mode.")
        self.col_recs = (_lib.MpmCollider * max(1, len(recs)))(*recs)
        self.n_col = len(recs)

    # ---------------------------------------------------------------- particle constraints
    @staticmethod
    def _rotate(q, v):
        """Rotate v [n, 3] by unit quaternions q [n, 4] (w, x, y, z)."""
        w, u = q[:, :1], q[:, 1:]
        t = 2.0 * torch.cross(u, v, dim=1)
        return v + w * t + torch.cross(u, t, dim=1)

    def set_constraints(self, start: int, mask, link: int, stiffness: float) -> None:
        """Attach the masked particles ([B, count] over rows [start, start+count)) to link `link` at
        their current positions (_kernel_set_particle_constraints: the link-frame offset from the
        link's pose now)."""
        lp, lq = self.solver.get_link_pose(link)
        for b in range(self.B):
            rows = torch.nonzero(mask[b].to(torch.bool)).reshape(-1) + start
            if rows.numel() == 0:
                continue
            x = self.states[b][0].detach()[rows]
            p = torch.as_tensor(np.asarray(lp[b], np.float32), device="cuda")
            q = torch.as_tensor(np.asarray(lq[b], np.float32), device="cuda")
            qi = torch.cat([q[:1], -q[1:]]).expand(len(rows), 4)
            self.con_local[b][rows] = self._rotate(qi, x - p)
            self.con_link[b][rows] = link
            self.con_k[b][rows] = float(stiffness)
        self.has_con = any(bool((k > 0).any()) for k in self.con_k)

    def remove_constraints(self, start: int, mask) -> None:
        for b in range(self.B):
            rows = torch.nonzero(mask[b].to(torch.bool)).reshape(-1) + start
            self.con_k[b][rows] = 0.0
            self.con_link[b][rows] = -1
        self.has_con = any(bool((k > 0).any()) for k in self.con_k)

    def _constraint_targets(self, b: int):
        """(stiffness, targets) of env b for a step starting now (the links' current poses), or None."""
        if not self.has_con:
            return None
        link = self.con_link[b]
        t = torch.zeros((self.n, 3), device="cuda")
        on = link >= 0
        if bool(on.any()):
            lp = torch.as_tensor(np.asarray(self.solver._link_pos[b], np.float32), device="cuda")
            lq = torch.as_tensor(np.asarray(self.solver._link_quat[b], np.float32), device="cuda")
            li = link[on]
            t[on] = self._rotate(lq[li], self.con_local[b][on]) + lp[li]
        return self.con_k[b].clone(), t.contiguous()

    def _fields(self, b: int):
        """The grid op's and the particles' inputs for a step of env b starting now."""
        return {"ff": self.ff_recs, "n_ff": self.n_ffs, "env": b, "ff_step": self.substeps_taken - self.ff_base,
                "col": self.col_recs, "n_col": self.n_col, "con": self._constraint_targets(b), "plan": self.ff_plan,
                "active": self.active[b].clone() if self.has_inactive else None,
                "t0": self.substeps_taken * self.solver.substep_dt}

    def _tool_seq(self, n_sub, T, qa):
        """[(n_sub + 1), n_tools, 13] tool states, entry 0 from (pos, vel) T and (quat, ang) qa."""
        nt = len(self.tools)
        seq = torch.zeros((n_sub + 1, max(1, nt), 13), device="cuda")
        if nt:
            seq[0, :nt, 0:3] = T[:, 0:3].detach()
            seq[0, :nt, 3:7] = qa[:, 0:4]
            seq[0, :nt, 7:10] = T[:, 3:6].detach()
            seq[0, :nt, 10:13] = qa[:, 4:7]
        return seq

    # ---------------------------------------------------------------- kernels
    @staticmethod
    def _s():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def _seq(self, ring, first=None):
        n = self.n
        seq = [torch.empty((ring, n, 3), device="cuda"), torch.empty((ring, n, 3), device="cuda"),
               torch.empty((ring, n, 3, 3), device="cuda"), torch.empty((ring, n, 3, 3), device="cuda"),
               torch.empty((ring, n), device="cuda")]
        if first is not None:
            for t, f in zip(seq, first):
                t[0] = f.detach()
        return seq

    def _extras(self, tool_seq, fields, actu, g_tool=None, g_actu=None):
        """The mpm_diff_extras record of one call (the arrays stay referenced by the caller)."""
        nt = len(self.tools)
        ex = _lib.MpmDiffExtras()
        ex.tools = ctypes.addressof(self.tool_recs)
        ex.n_tools = nt
        ex.tool_seq = tool_seq.data_ptr() if nt else None
        ex.g_tool = g_tool.data_ptr() if (nt and g_tool is not None) else None
        ex.force_fields = ctypes.addressof(fields["ff"])
        ex.n_force_fields = fields["n_ff"]
        ex.scene_index = fields["env"]
        ex.ff_step = fields["ff_step"]
        ex.colliders = ctypes.addressof(fields["col"])
        ex.n_colliders = fields["n_col"]
        ex.sdf_ctx = self.solver._ctx
        if fields["con"] is not None:
            ex.constraint_stiffness = fields["con"][0].data_ptr()
            ex.constraint_target = fields["con"][1].data_ptr()
        if fields.get("active") is not None:
            ex.active = fields["active"].data_ptr()
        if self.has_muscle:
            ex.actu = actu.data_ptr()
            ex.muscle_dir = self.mdir.data_ptr()
            ex.g_actu = g_actu.data_ptr() if g_actu is not None else None
        return ex

    def _forward_seq(self, seq, n_sub, ring, gpm, gv, keep_grids, tool_seq, fields, actu):
        """The step's substeps; with Custom force fields, staged (returns each substep's stage inputs
        when keep_grids, for the backward)."""
        if fields["plan"] is not None:
            return self._staged_forward(seq, n_sub, ring, gpm, gv, keep_grids, tool_seq, fields, actu)
        ex = self._extras(tool_seq, fields, actu)
        r = self.lib.mpm_diff_forward_seq_ex(ctypes.byref(self.cfg), self.mass.data_ptr(), self.kind.data_ptr(),
                                             self.aux.data_ptr(), self.n, int(n_sub), *[t.data_ptr() for t in seq],
                                             ring, self.mu.data_ptr(), self.lam.data_ptr(), ctypes.byref(ex),
                                             gpm.data_ptr(), gv.data_ptr(), int(keep_grids), self.status.data_ptr(),
                                             self._s())
        _lib.check(r, None, "mpm_diff_forward_seq_ex")

    def _backward_seq(self, seq, n_sub, gp, gpm, gv, tool_seq, g_tool, fields, actu, g_actu, stage_inputs=None):
        if fields["plan"] is not None:
            return self._staged_backward(seq, n_sub, gp, gpm, gv, tool_seq, g_tool, fields, actu, g_actu,
                                         stage_inputs)
        n = self.n
        gmu = torch.zeros(n, device="cuda")
        glam = torch.zeros(n, device="cuda")
        ex = self._extras(tool_seq, fields, actu, g_tool, g_actu)
        r = self.lib.mpm_diff_backward_seq_ex(ctypes.byref(self.cfg), self.mass.data_ptr(), self.kind.data_ptr(),
                                              self.aux.data_ptr(), n, int(n_sub), *[t.data_ptr() for t in seq],
                                              self.mu.data_ptr(), self.lam.data_ptr(), ctypes.byref(ex),
                                              gp.data_ptr(), gmu.data_ptr(), glam.data_ptr(), gpm.data_ptr(),
                                              gv.data_ptr(), self.g_grid_v.data_ptr(), self.g_grid_pm.data_ptr(),
                                              self.status.data_ptr(), self._s())
        _lib.check(r, None, "mpm_diff_backward_seq_ex")

    # ---------------------------------------------------------------- Custom force fields (staged)
    # A Custom field is a torch function of the node velocities: the substep runs in parts
    # (mpm_diff_substep_stage: P2G, grid stages, G2P) with the function applied between grid stages,
    # and its transposed Jacobian applied in the adjoint by torch autograd between the stages'
    # adjoints (mpm_diff_substep_stage_adj).  The velocity each stage and each Custom field began
    # from is kept for the backward.
    def _node_pos(self):
        """[nodes, 3] positions of the dense differentiable grid's nodes ((g + offset) dx in float)."""
        if getattr(self, "_npos", None) is None:
            res = [int(r) for r in self.solver.grid_res]
            g = torch.stack(torch.meshgrid(*[torch.arange(r, device="cuda") for r in res], indexing="ij"), -1)
            off = torch.as_tensor(np.asarray(self.solver.grid_offset), device="cuda")
            dx = torch.tensor(self.solver.dx, dtype=torch.float32, device="cuda")
            self._npos = ((g.reshape(-1, 3) + off).to(torch.float32) * dx).contiguous()
        return self._npos

    def _custom_apply(self, f, grid_v, t):
        sel = torch.nonzero(grid_v[:, 3] > self.solver._eps).squeeze(1)
        if sel.numel() == 0:
            return
        v = grid_v.index_select(0, sel)[:, :3]
        with torch.no_grad():
            acc = f.get_acc(self._node_pos().index_select(0, sel), v.clone(), float(t), -1)
        acc = torch.as_tensor(acc, dtype=torch.float32, device="cuda").reshape(-1, 3)
        grid_v[sel, :3] = v + acc * self.solver.substep_dt

    def _custom_vjp(self, f, v_in, g, t):
        """g (dL/d(node velocity after the field), [nodes, 4]) <- dL/d(before): g + dt J^T g on the
        nodes with mass; the function's own parameters collect their gradients on the way."""
        sel = torch.nonzero(v_in[:, 3] > self.solver._eps).squeeze(1)
        if sel.numel() == 0:
            return
        with torch.enable_grad():
            vin = v_in.index_select(0, sel)[:, :3].clone().requires_grad_(True)
            acc = f.get_acc(self._node_pos().index_select(0, sel), vin, float(t), -1)
            acc = torch.as_tensor(acc, dtype=torch.float32, device="cuda").reshape(-1, 3)
            if acc.requires_grad:
                torch.autograd.backward([acc], [g.index_select(0, sel)[:, :3] * self.solver.substep_dt])
        if vin.grad is not None:
            g[sel, :3] += vin.grad

    def _stage_call(self, adj, ex, k_state, args):
        """One mpm_diff_substep_stage(_adj) call on state k_state (x, v, C, F, Jp tensors)."""
        x, v, C, F, Jp = k_state
        fn = self.lib.mpm_diff_substep_stage_adj if adj else self.lib.mpm_diff_substep_stage
        r = fn(ctypes.byref(self.cfg), self.mass.data_ptr(), self.kind.data_ptr(), self.aux.data_ptr(), self.n,
               x.data_ptr(), v.data_ptr(), C.data_ptr(), F.data_ptr(), Jp.data_ptr(), self.mu.data_ptr(),
               self.lam.data_ptr(), ctypes.byref(ex), *args, self.status.data_ptr(), self._s())
        _lib.check(r, None, "mpm_diff_substep_stage_adj" if adj else "mpm_diff_substep_stage")

    def _tool_ptr(self, tool_seq, k):
        nt = len(self.tools)
        return tool_seq[k].data_ptr() if nt else None

    def _staged_forward(self, seq, n_sub, ring, gpm, gv, keep, tool_seq, fields, actu):
        plan = fields["plan"]
        dt = self.solver.substep_dt
        kept = []
        for k in range(n_sub):
            a, b = k % ring, (k + 1) % ring
            cur = [t[a] for t in seq]
            nxt = [t[b] for t in seq]
            pm, vel = (gpm[k], gv[k]) if keep else (gpm, gv)
            ex = self._extras(tool_seq, dict(fields, ff_step=fields["ff_step"] + k), actu)
            ex.tool_seq = self._tool_ptr(tool_seq, k)
            t_k = fields["t0"] + k * dt
            grids = (pm.data_ptr(), vel.data_ptr())
            self._stage_call(False, ex, cur, (0, 0, 0, 0, *[u.data_ptr() for u in nxt], *grids))
            inputs = [None]
            for idx, item in enumerate(plan):
                if idx > 0:
                    inputs.append(vel.clone() if keep else None)
                if item[0] == "fields":
                    self._stage_call(False, ex, cur, (1, 1 if idx == 0 else 2, item[1], item[2],
                                                      *[u.data_ptr() for u in nxt], *grids))
                else:
                    self._custom_apply(item[1], vel, t_k)
            inputs.append(vel.clone() if keep else None)  # the tail's input
            self._stage_call(False, ex, cur, (1, 3, 0, 0, *[u.data_ptr() for u in nxt], *grids))
            self._stage_call(False, ex, cur, (2, 0, 0, 0, *[u.data_ptr() for u in nxt], *grids))
            kept.append(inputs)
        return kept if keep else None

    def _staged_backward(self, seq, n_sub, gp, gpm, gv, tool_seq, g_tool, fields, actu, g_actu, stage_inputs):
        plan = fields["plan"]
        dt = self.solver.substep_dt
        n = self.n
        gmu = torch.zeros(n, device="cuda")
        glam = torch.zeros(n, device="cuda")
        gpm = gpm.reshape(-1, self.nodes, 4)
        gv = gv.reshape(-1, self.nodes, 4)
        cur = 0
        for k in range(n_sub - 1, -1, -1):
            g_in, g_out = gp[cur], gp[1 - cur]
            gi = [g_in[o * n: (o + w) * n] for o, w in zip(_OFFSET, _WIDTH)]
            go = [g_out[o * n: (o + w) * n] for o, w in zip(_OFFSET, _WIDTH)]
            state = [t[k] for t in seq]
            ex = self._extras(tool_seq, dict(fields, ff_step=fields["ff_step"] + k), actu, g_tool, g_actu)
            ex.tool_seq = self._tool_ptr(tool_seq, k)
            t_k = fields["t0"] + k * dt
            inputs = stage_inputs[k]
            ptrs = (*[u.data_ptr() for u in gi], *[u.data_ptr() for u in go], gmu.data_ptr(), glam.data_ptr(),
                    gpm[k].data_ptr(), gv[k].data_ptr(), self.g_grid_v.data_ptr(), self.g_grid_pm.data_ptr())
            self._stage_call(True, ex, state, (2, 0, 0, 0, None, *ptrs))
            self._stage_call(True, ex, state, (1, 3, 0, 0, inputs[len(plan)].data_ptr(), *ptrs))
            for idx in range(len(plan) - 1, -1, -1):
                item = plan[idx]
                if item[0] == "custom":
                    self._custom_vjp(item[1], inputs[idx], self.g_grid_v, t_k)
                elif idx == 0:
                    self._stage_call(True, ex, state, (1, 1, item[1], item[2], None, *ptrs))
                else:
                    self._stage_call(True, ex, state, (1, 2, item[1], item[2], inputs[idx].data_ptr(), *ptrs))
            self._stage_call(True, ex, state, (0, 0, 0, 0, None, *ptrs))
            cur = 1 - cur
        if cur == 1:
            gp[0].copy_(gp[1])

    def _g_tool(self, gT):
        g = torch.zeros((max(1, len(self.tools)), 12), device="cuda")
        if gT is not None and len(self.tools):
            g[:len(self.tools), :6] = gT.float()
        return g

    def _pack(self, grads):
        n = self.n
        gp = torch.zeros((2, 25 * n), device="cuda")
        for k, g in enumerate(grads):
            if g is not None:
                gp[0, _OFFSET[k] * n: (_OFFSET[k] + _WIDTH[k]) * n] = g.reshape(-1).float()
        return gp

    def _unpack(self, gp):
        n = self.n
        shapes = ((n, 3), (n, 3), (n, 3, 3), (n, 3, 3), (n,))
        return [gp[0, _OFFSET[k] * n: (_OFFSET[k] + _WIDTH[k]) * n].view(shapes[k]).clone() for k in range(5)]

    def run_forward(self, st, n_sub, qa, fields):
        """The state after n_sub substeps from st (new tensors), and the tools' (quat, ang) then."""
        seq = self._seq(2, st[:5])
        tseq = self._tool_seq(n_sub, st[5], qa)
        self._forward_seq(seq, n_sub, 2, self.scratch[0], self.scratch[1], False, tseq, fields, st[6])
        k = n_sub % 2
        nt = len(self.tools)
        end = tseq[n_sub, :nt]
        T_end = torch.cat([end[:, 0:3], end[:, 7:10]], 1).clone()
        qa_end = torch.cat([end[:, 3:7], end[:, 10:13]], 1).clone()
        return (*(t[k].clone() for t in seq), T_end, st[6].clone()), qa_end

    def run_backward(self, st, n_sub, grads, qa, fields):
        """dL/d(step input) from dL/d(step output): re-simulates the step keeping every substep's state
        and grid, then runs the adjoint substeps in reverse."""
        seq = self._seq(n_sub + 1, st[:5])
        tseq = self._tool_seq(n_sub, st[5], qa)
        gpm = torch.empty((max(1, n_sub), self.nodes, 4), device="cuda")
        gv = torch.empty((max(1, n_sub), self.nodes, 4), device="cuda")
        kept = self._forward_seq(seq, n_sub, n_sub + 1, gpm, gv, True, tseq, fields, st[6])
        gp = self._pack(grads[:5])
        g_tool = self._g_tool(grads[5])
        g_actu = grads[6].float().clone() if grads[6] is not None else torch.zeros(self.n, device="cuda")
        self._backward_seq(seq, n_sub, gp, gpm, gv, tseq, g_tool, fields, st[6], g_actu, kept)
        self.check()
        return (*self._unpack(gp), g_tool[:len(self.tools), :6].clone(), g_actu)

    def check(self):
        st = int(self.status.item())
        if st & _lib.STATUS_NAN:
            raise GenesisException(
                "NaN detected in MPM states. Try reducing the time step size or adjusting simulation parameters.")
        if st & _lib.STATUS_OOB:
            raise GenesisException("MPM particles left the simulation grid (stencil out of bounds).")

    # ---------------------------------------------------------------- scene-level operations
    def step(self, n_sub: int) -> None:
        # checkpoint of the step (after its inputs) and the inputs written before it
        fields = [self._fields(b) for b in range(self.B)]
        self.step_inputs.append((list(self.states), int(n_sub), self.pending, list(self.tool_qa), fields))
        self.pending = []
        for b, st in enumerate(self.states):
            out = _StepNode.apply(self, int(n_sub), fields[b], self.tool_qa[b], *st)
            self.states[b], self.tool_qa[b] = tuple(out[:7]), out[7]
        self.steps_taken += 1
        self.substeps_taken += int(n_sub)

    # ---------------------------------------------------------------- imperative adjoint (Solver protocol)
    # The reference's Scene._backward drives a solver through add_grad_from_state /
    # collect_output_grads, then per substep substep_post_coupling_grad, the coupler's couple_grad
    # and substep_pre_coupling_grad, then process_input_grad (simulator.py:298-370).  These do the
    # same on the adjoint held here: `adj[b]` is dL/d(state of env b at substep `cursor`).
    def reset_grad(self) -> None:
        dev = "cuda"
        n = self.n
        self.adj = [[torch.zeros((n, 3), device=dev), torch.zeros((n, 3), device=dev),
                     torch.zeros((n, 3, 3), device=dev), torch.zeros((n, 3, 3), device=dev),
                     torch.zeros(n, device=dev), torch.zeros((len(self.tools), 6), device=dev),
                     torch.zeros(n, device=dev)]
                    for _ in range(self.B)]
        self.cursor = self.substeps_taken
        self._seg = None
        self.queried.clear()
        self.queried_tools.clear()

    def add_grad(self, grads_by_field, envs=None) -> None:
        """Add dL/d(pos, vel, C, F, Jp) ([B', N', ...] with N' = count particles from `start`) to the adjoint."""
        if self.adj is None:
            self.reset_grad()
        for field, (g, start) in grads_by_field.items():
            if g is None:
                continue
            k = FIELDS.index(field)
            for i, b in enumerate(range(self.B) if envs is None else envs):
                self.adj[b][k][start: start + g.shape[1]] += g[i].to(torch.float32)

    def add_tool_grad(self, tool: int, gpos, gvel, envs=None) -> None:
        """Add dL/d(pos, vel) ([B', 3] each, or None) of a tool to the adjoint."""
        if self.adj is None:
            self.reset_grad()
        for i, b in enumerate(range(self.B) if envs is None else envs):
            if gpos is not None:
                self.adj[b][5][tool, 0:3] += gpos[i].to(torch.float32)
            if gvel is not None:
                self.adj[b][5][tool, 3:6] += gvel[i].to(torch.float32)

    def _locate(self, f_global):
        """(step index, substep within the step) of the substep that ends at global substep f_global."""
        acc = 0
        for s_i, (_, n_sub, _, _, _) in enumerate(self.step_inputs):
            if f_global <= acc + n_sub:
                return s_i, f_global - acc - 1
            acc += n_sub
        raise GenesisException("No forward substep recorded for this gradient step.")

    def substep_grad(self) -> None:
        """Adjoint of the substep that ends at `cursor` (G2P, grid op and P2G adjoints in one library call);
        the cursor moves one substep back."""
        if self.adj is None:
            self.reset_grad()
        if self.cursor <= 0:
            raise GenesisException("The gradient walk is already at the first substep.")
        s_i, k = self._locate(self.cursor)
        n = self.n
        if self._seg is None or self._seg[0] != s_i:  # re-simulate the step from its checkpoint (load_ckpt)
            inputs, n_sub, _, qas, fields = self.step_inputs[s_i]
            keep = []
            for b in range(self.B):
                seq = self._seq(n_sub + 1, inputs[b][:5])
                tseq = self._tool_seq(n_sub, inputs[b][5], qas[b])
                gpm = torch.empty((n_sub, self.nodes, 4), device="cuda")
                gv = torch.empty((n_sub, self.nodes, 4), device="cuda")
                kept = self._forward_seq(seq, n_sub, n_sub + 1, gpm, gv, True, tseq, fields[b], inputs[b][6])
                keep.append((seq, gpm, gv, tseq, fields[b], inputs[b][6], kept))
            self._seg = (s_i, keep)
        for b in range(self.B):
            seq, gpm, gv, tseq, fields, actu, kept = self._seg[1][b]
            gp = self._pack(self.adj[b][:5])
            g_tool = self._g_tool(self.adj[b][5])
            g_actu = self.adj[b][6]  # the step's actuation adjoint gathers every substep's share
            self._backward_seq([t[k: k + 1].contiguous() for t in seq], 1, gp, gpm[k], gv[k],
                               tseq[k: k + 2].contiguous(), g_tool,
                               dict(fields, ff_step=fields["ff_step"] + k, t0=fields["t0"] + k * self.solver.substep_dt),
                               actu, g_actu, None if kept is None else kept[k: k + 1])
            self.adj[b] = [*self._unpack(gp), g_tool[:len(self.tools), :6].clone(), g_actu]
        self.cursor -= 1

    def input_grad(self) -> None:
        """At a step boundary (process_input_grad): the adjoint of the rows that the step's entity inputs
        wrote goes to those inputs (through torch autograd, into the tensors the caller passed), and
        stops there: a written row does not depend on the state before the write."""
        if self.adj is None:
            return
        s_i, k = self._locate(self.cursor + 1)
        if k != 0:
            raise GenesisException("process_input_grad must follow the first substep of a step.")
        for field, start, count, values, envs in reversed(self.step_inputs[s_i][2]):
            if field.startswith("tool_"):  # a tool's position / velocity input (ToolEntity.process_input_grad)
                cols = slice(0, 3) if field == "tool_pos" else slice(3, 6)
                if values.requires_grad:
                    vb = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), 3))
                    torch.autograd.backward([vb], [torch.stack([self.adj[b][5][start, cols] for b in envs])])
                for b in envs:
                    self.adj[b][5][start, cols] = 0.0
                continue
            rows = slice(start, start + count)
            if field == "actu":  # a Muscle entity's actuation (MPMEntity.process_input_grad)
                if values.requires_grad:
                    vb = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), count))
                    torch.autograd.backward([vb], [torch.stack([self.adj[b][6][rows] for b in envs])])
                for b in envs:
                    self.adj[b][6][rows] = 0.0
                continue
            j = 0 if field == "pos" else 1
            if values.requires_grad:
                vb = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), count, 3))
                torch.autograd.backward([vb], [torch.stack([self.adj[b][j][rows] for b in envs])])
            for b in envs:  # set_position also reset v, C, F, Jp of those rows
                for jj in ((0, 1, 2, 3, 4) if field == "pos" else (1,)):
                    self.adj[b][jj][rows] = 0.0

    def write(self, field: str, start: int, count: int, values: torch.Tensor, envs) -> None:
        """Set one entity's particles [start, start+count) of `field` (pos / vel: values broadcast to
        [len(envs), count, 3]; actu: to [len(envs), count]) in envs, through differentiable torch ops."""
        if field == "actu":
            self.pending.append((field, start, count, values, list(envs)))
            vals = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), count))
            for i, b in enumerate(envs):
                st = list(self.states[b])
                st[6] = torch.cat([st[6][:start], vals[i], st[6][start + count:]], 0)
                self.states[b] = tuple(st)
            return
        k = {"pos": 0, "vel": 1}[field]
        self.pending.append((field, start, count, values, list(envs)))
        vals = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), count, 3))
        for i, b in enumerate(envs):
            st = list(self.states[b])
            t = st[k]
            st[k] = torch.cat([t[:start], vals[i], t[start + count:]], 0)
            if k == 0:  # set_position resets the deformation state like _kernel_set_particles_pos
                st[1] = torch.cat([st[1][:start], torch.zeros((count, 3), device="cuda"), st[1][start + count:]], 0)
                C0 = torch.zeros((count, 3, 3), device="cuda")
                F0 = torch.eye(3, device="cuda").repeat(count, 1, 1)
                st[2] = torch.cat([st[2][:start], C0, st[2][start + count:]], 0)
                st[3] = torch.cat([st[3][:start], F0, st[3][start + count:]], 0)
                st[4] = torch.cat([st[4][:start], self.Jp0[start: start + count], st[4][start + count:]], 0)
            self.states[b] = tuple(st)

    def write_tool(self, field: str, tool: int, values: torch.Tensor, envs) -> None:
        """Set tool `tool`'s position ("tool_pos") or velocity ("tool_vel") in envs through
        differentiable torch ops (values broadcast to [len(envs), 3])."""
        self.pending.append((field, tool, 1, values, list(envs)))
        vals = torch.broadcast_to(values.to(device="cuda", dtype=torch.float32), (len(envs), 3))
        c0 = 0 if field == "tool_pos" else 3
        for i, b in enumerate(envs):
            st = list(self.states[b])
            T = st[5]
            row = torch.cat([T[tool, :c0], vals[i], T[tool, c0 + 3:]], 0)
            st[5] = torch.cat([T[:tool], row[None], T[tool + 1:]], 0)
            self.states[b] = tuple(st)

    def set_tool_orientation(self, tool: int, quat=None, ang=None, envs=None) -> None:
        """Set a tool's orientation or angular velocity (not differentiated)."""
        for i, b in enumerate(range(self.B) if envs is None else envs):
            qa = self.tool_qa[b].clone()
            if quat is not None:
                qa[tool, :4] = torch.broadcast_to(torch.as_tensor(quat, dtype=torch.float32, device="cuda"),
                                                  (len(envs) if envs is not None else self.B, 4))[i]
            if ang is not None:
                qa[tool, 4:] = torch.broadcast_to(torch.as_tensor(ang, dtype=torch.float32, device="cuda"),
                                                  (len(envs) if envs is not None else self.B, 3))[i]
            self.tool_qa[b] = qa

    def tool_state(self, tool: int):
        """(pos [B, 3], quat [B, 4], vel [B, 3], ang [B, 3]) of a tool; pos and vel autograd-connected."""
        T = torch.stack([s[5][tool] for s in self.states])
        qa = torch.stack([q[tool] for q in self.tool_qa])
        return T[:, :3], qa[:, :4], T[:, 3:], qa[:, 4:]

    def stacked(self):
        """[B, N, ...] tensors of the current state (pos, vel, C, F, Jp; autograd-connected)."""
        return tuple(torch.stack([s[k] for s in self.states]) for k in range(5))

    def set_from_state(self, state, envs) -> None:
        for b in envs:
            self.states[b] = (*(getattr(state, k)[b].to(device="cuda", dtype=torch.float32) for k in FIELDS),
                              self.states[b][5], self.states[b][6])

    def reset(self, envs) -> None:
        """Scene.reset (simulator.py:223-232): the tools of envs back to their initial pose, at rest;
        with every env reset the substep count restarts and the recorded steps are dropped (the
        adjoint walk cannot pass a reset), as the reference's reset zeroes _cur_substep_global."""
        for b in envs:
            st = list(self.states[b])
            st[5] = self.T0.clone()
            st[6] = st[6].detach().clone()  # the actuation stays set, off the graph of the steps before
            self.states[b] = tuple(st)
            self.tool_qa[b] = self.qa0.clone()
        if len(list(envs)) == self.B:
            self.step_inputs = []
            self.pending = []
            self.steps_taken = self.substeps_taken = 0
            self.ff_base = 0
            self.queried.clear()
            self.queried_tools.clear()
            self.adj = None
            self._seg = None

    def set_active(self, start: int, count: int, values, envs) -> None:
        """Activity of particles [start, start+count) in envs (values broadcast to [len(envs), count]);
        from the next step on, inactive particles keep their state."""
        vals = torch.broadcast_to(torch.as_tensor(values, device="cuda").to(torch.uint8), (len(envs), count))
        for i, b in enumerate(envs):
            self.active[b][start: start + count] = vals[i]
        self.has_inactive = any(bool((a == 0).any()) for a in self.active)

    def set_muscle_direction(self, start: int, count: int, dirs: torch.Tensor) -> None:
        """Fibre directions [count, 3] of particles [start, start+count) (constants of the steps to come)."""
        self.mdir[start: start + count] = dirs.to(device="cuda", dtype=torch.float32)
