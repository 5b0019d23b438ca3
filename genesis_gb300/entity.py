"""MPMEntity: the drop-in for genesis/engine/entities/mpm_entity.py (+ particle_entity.py).

Sampling happens at construction (particle_entity.py:234-356); state accessors return
torch tensors on the CUDA device in the reference's [B, n, ...] layout.  Target setters
(set_position / set_velocity / set_active) are buffered and applied at the start of the
next step, like ParticleEntity.process_input (particle_entity.py:424-464).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .exceptions import GenesisException
from .states import MPMEntityState


def _stream_ptr():
    return torch.cuda.current_stream().cuda_stream

ACTIVE = 1
INACTIVE = 0


class MPMEntity:
    def __init__(self, scene, solver, material, morph, surface, particle_size, idx, particle_start, name=None):
        from .morphs import Nowhere

        self._scene = scene
        self._solver = solver
        self._material = material
        self._morph = morph
        self._surface = surface
        self._particle_size = particle_size
        self._idx = idx
        self._particle_start = particle_start
        self._uid = id(self)
        if name is None:  # base_entity.py:40-45: morph identifier + short uid
            kind = type(morph).__name__.lower()
            name = f"{kind}_{format(self._uid & 0xFFFFFFF, '07x')}"
        self._name = name
        self.sampler = material.sampler
        particles = morph.sample(particle_size, self.sampler)
        if particles.size == 0:
            raise GenesisException("Entity has zero particles.")
        if not isinstance(morph, Nowhere):
            if not solver.boundary.is_inside(particles):
                raise GenesisException(
                    "Entity has particles outside solver boundary. Note that for MPMSolver, boundary is slightly "
                    "tighter than the specified domain due to safety padding.\n\n"
                    f"Current boundary:\n{solver.boundary}\n\nEntity to be added:\nmin: {particles.min(0)}\n"
                    f"max: {particles.max(0)}\n"
                )
            origin = np.asarray(morph.pos, dtype=np.float64)
        else:
            origin = np.zeros(3)
        self._particles = np.ascontiguousarray(particles, dtype=np.float64)
        self._init_particles_offset = self._particles - origin
        self._n_particles = len(self._particles)
        self.active = not isinstance(morph, Nowhere)
        self._tgt = {"pos": None, "vel": None, "act": None}
        self._vverts = np.zeros((0, 3), dtype=np.float64)
        self._vvert_support_idx = np.zeros((0, 0), dtype=np.int32)
        self._vvert_support_w = np.zeros((0, 0), dtype=np.float32)

    # ------------------------------------------------------------------ particle constraints
    def _mask(self, particles_mask):
        B = self._solver._B
        if particles_mask is None:
            m = torch.ones((B, self._n_particles), dtype=torch.uint8, device="cuda")
        else:
            m = torch.as_tensor(particles_mask, device="cuda").to(torch.uint8)
            if m.ndim == 1:
                m = m.unsqueeze(0).expand(B, -1)
            if tuple(m.shape) != (B, self._n_particles):
                raise GenesisException(f"particles_mask must have shape ({B}, {self._n_particles}).")
        return m.contiguous()

    def set_particle_constraints(self, particles_mask, link_idx, stiffness):
        """mpm_entity.py:631-671: attach the masked particles to kinematic link `link_idx` (its
        pose from MPMSolver.set_link_poses) with a critically damped spring of `stiffness`."""
        if not isinstance(link_idx, int):
            raise GenesisException("link_idx must be an integer.")
        lp, lq = self._solver.get_link_pose(link_idx)
        m = self._mask(particles_mask)
        if self._solver._diff is not None:  # differentiable mode: the springs act in the torch state
            self._solver._diff.set_constraints(self._particle_start, m, link_idx, float(stiffness))
        pos = torch.as_tensor(np.array(lp, dtype=np.float32), device="cuda")
        quat = torch.as_tensor(np.array(lq, dtype=np.float32), device="cuda")
        lib = self._solver._lib
        _lib.check(lib.mpm_set_particle_constraints(self._solver._ctx, 0, self._solver._B, self._particle_start,
                                                    self._n_particles, m.data_ptr(), float(stiffness), link_idx,
                                                    pos.data_ptr(), quat.data_ptr(), _stream_ptr()),
                   self._solver._ctx, "mpm_set_particle_constraints")
        torch.cuda.current_stream().synchronize()

    def remove_particle_constraints(self, particles_mask=None):
        """mpm_entity.py:674-690: remove the constraints of the masked particles (all if None)."""
        m = self._mask(particles_mask)
        if self._solver._diff is not None:
            self._solver._diff.remove_constraints(self._particle_start, m)
        lib = self._solver._lib
        _lib.check(lib.mpm_remove_particle_constraints(self._solver._ctx, 0, self._solver._B, self._particle_start,
                                                       self._n_particles, m.data_ptr(), _stream_ptr()),
                   self._solver._ctx, "mpm_remove_particle_constraints")
        torch.cuda.current_stream().synchronize()

    # ------------------------------------------------------------------ visual vertices
    def set_vverts(self, verts) -> None:
        """Attach visual-mesh vertices [V, 3] (the reference takes them from the entity's visual
        mesh) and compute each vertex's support particles and weights from the sampled particles as
        particle_entity.py:193-232 does: the n_support_neighbors nearest particles ordered by
        (distance, index); with P the supports' positions relative to the last one, b = pinv(P) (v -
        p_last), weights (b, 1 - sum b).  Indices are solver-level (entity particle start + local)."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 3))
        k = min(self._solver.n_vvert_supports, self._n_particles)
        dist2 = np.sum(np.square(v[:, None, :] - self._particles[None, :, :]), axis=2)
        idx = np.argpartition(dist2, k - 1, axis=1)[:, :k]
        rows = np.arange(len(v))[:, None]
        order = np.lexsort((idx, dist2[rows, idx]))
        idx = np.clip(idx[rows, order], 0, self._n_particles - 1)
        ps = self._particles[idx]
        Ps = ps[:, :-1].swapaxes(-2, -1) - np.expand_dims(ps[:, -1], axis=-1)
        b = np.einsum("vij,vj->vi", np.linalg.pinv(Ps), v - ps[:, -1])
        w = np.concatenate([b, 1.0 - b.sum(axis=1, keepdims=True)], axis=1)
        self._vverts = v
        self._vvert_support_idx = (idx + self._particle_start).astype(np.int32)
        self._vvert_support_w = w.astype(np.float32)
        self._solver._vverts_changed()

    @property
    def n_vverts(self) -> int:
        return len(self._vverts)

    @property
    def n_vfaces(self) -> int:
        """Visual faces: none here (vertices come without a mesh, set_vverts)."""
        return 0

    @property
    def vvert_start(self) -> int:
        """First visual vertex of this entity in the solver's vertex buffer (entities in order)."""
        start = 0
        for e in self._solver._entities:
            if e is self:
                return start
            start += e.n_vverts
        return start

    @property
    def vvert_end(self) -> int:
        return self.vvert_start + self.n_vverts

    @property
    def vface_start(self) -> int:
        return 0

    @property
    def vface_end(self) -> int:
        return self.vface_start + self.n_vfaces

    def find_closest_particle(self, pos, envs_idx=None):
        """particle_entity.py:716-743: index of the particle nearest to pos ([3] or [B, 3]) per env."""
        p = torch.as_tensor(pos, dtype=torch.float32, device="cuda")
        B = self._solver._B
        if p.ndim == 1:
            p = p.reshape(1, 3).expand(B, 3)
        if tuple(p.shape) != (B, 3):
            raise GenesisException(f"Invalid tensor shape {tuple(p.shape)} (expected ({B}, 3)).")
        cur = self._get_field(_lib.FIELD_POS, 3, envs_idx)
        if envs_idx is not None:
            p = p[torch.as_tensor(self._envs(envs_idx), device="cuda")]
        idx = torch.argmin(torch.linalg.norm(cur - p[:, None], dim=-1), dim=-1).to(torch.int32)
        return idx[0] if self._scene.n_envs == 0 else idx

    def get_frame(self, f, pos, vel, C, F, Jp, active):
        """mpm_entity.py:305-352: fill the given [B, n, ...] tensors with the particles' state.  Only
        the current frame is kept on the device (no per-substep frame ring), so `f` must name it
        (the solver's current substep-local frame, or None)."""
        cur = getattr(self._scene.sim, "cur_substep_local", None)
        if f is not None and cur is not None and int(f) != int(cur):
            raise GenesisException("Only the current frame is kept on the device.")
        st = self.get_state()
        for dst, src in ((pos, st.pos), (vel, st.vel), (C, st.C), (F, st.F), (Jp, st.Jp), (active, st.active)):
            if dst is not None:
                dst.copy_(src.reshape(dst.shape).to(dst.dtype))

    # ------------------------------------------------------------------ checkpoints (particle_entity.py:371-403)
    def init_ckpt(self):
        self._ckpt = {}

    def save_ckpt(self, ckpt_name):
        """Keep the pending targets (set_position / set_velocity / activation at the next step)."""
        if not hasattr(self, "_ckpt"):
            self._ckpt = {}
        self._ckpt[ckpt_name] = dict(self._tgt)

    def load_ckpt(self, ckpt_name):
        self._tgt = dict(self._ckpt[ckpt_name])

    # ------------------------------------------------------------------ solver plumbing
    def _add_to_solver(self):
        self._solver._add_particles(
            self._particle_start, self._n_particles, self._material.idx, self.active, self._particles
        )

    def _envs(self, envs_idx):
        B = self._solver._B
        if envs_idx is None:
            return list(range(B))
        if self._scene.n_envs == 0:
            raise GenesisException("`envs_idx` is not supported for non-parallelized scene.")
        if isinstance(envs_idx, slice):
            return list(range(B))[envs_idx]
        if isinstance(envs_idx, (int, np.integer)):
            return [int(envs_idx)]
        return [int(e) for e in torch.as_tensor(envs_idx).reshape(-1).tolist()]

    def _get_field(self, field, width, envs_idx):
        envs = self._envs(envs_idx)
        out = torch.empty((len(envs), self._n_particles, width), dtype=torch.float32, device="cuda")
        if envs == list(range(envs[0], envs[0] + len(envs))):
            self._solver._field(field, 0, envs[0], envs[0] + len(envs), self._particle_start, self._n_particles, out)
        else:
            for i, e in enumerate(envs):
                self._solver._field(field, 0, e, e + 1, self._particle_start, self._n_particles, out[i])
        return out

    def _write(self, field, envs, v):
        if envs == list(range(envs[0], envs[0] + len(envs))):
            self._solver._field(field, 1, envs[0], envs[0] + len(envs), self._particle_start, self._n_particles, v)
        else:
            for i, e in enumerate(envs):
                self._solver._field(field, 1, e, e + 1, self._particle_start, self._n_particles, v[i].contiguous())

    def _set_field(self, field, width, values, envs_idx, particles_idx_local=None):
        """values broadcast to [B, n_sel, width]; n_sel = all particles or len(particles_idx_local)."""
        envs = self._envs(envs_idx)
        B = len(envs)
        v = torch.as_tensor(values, dtype=torch.float32, device="cuda")
        if particles_idx_local is None:
            self._write(field, envs, torch.broadcast_to(v, (B, self._n_particles, width)).contiguous())
        else:
            idx = torch.as_tensor(particles_idx_local, device="cuda", dtype=torch.long)
            idx = torch.broadcast_to(idx.reshape(-1) if idx.ndim <= 1 else idx, (B, idx.shape[-1]))
            vv = torch.broadcast_to(v, (B, idx.shape[1], width))
            sel = idx[..., None]
            if field == _lib.FIELD_POS_RESET:  # reset v, C, F, Jp of the selected particles only
                resets = (
                    (_lib.FIELD_POS, 3, vv),
                    (_lib.FIELD_VEL, 3, torch.zeros_like(vv)),
                    (_lib.FIELD_C, 9, torch.zeros((B, idx.shape[1], 9), device="cuda")),
                    (_lib.FIELD_F, 9, torch.eye(3, device="cuda").reshape(1, 1, 9).expand(B, idx.shape[1], 9)),
                    (_lib.FIELD_JP, 1, torch.full((B, idx.shape[1], 1), float(self._material._default_Jp), device="cuda")),
                )
                for f, w, val in resets:
                    full = self._get_field(f, w, envs_idx)
                    full.scatter_(1, sel.expand(-1, -1, w), val)
                    self._write(f, envs, full.contiguous())
            else:
                full = self._get_field(field, width, envs_idx)
                full.scatter_(1, sel.expand(-1, -1, width), vv)
                self._write(field, envs, full.contiguous())
        torch.cuda.current_stream().synchronize()

    def _squeeze(self, t):
        return t[0] if self._scene.n_envs == 0 else t

    # ------------------------------------------------------------------ targets (applied at step start)
    def set_position(self, value, envs_idx=None):
        """Per-particle positions, or the centre of mass relative to the initial shape (particle_entity.py:509-527)."""
        poss = torch.as_tensor(value, dtype=torch.float32, device="cuda")
        if poss.ndim == 1 or (poss.ndim == 2 and poss.shape[0] != self._n_particles):
            off = torch.as_tensor(self._init_particles_offset, dtype=torch.float32, device="cuda")
            poss = off + poss[..., None, :]
        self._tgt["pos"] = (poss, envs_idx)

    def set_velocity(self, vels, envs_idx=None):
        self._tgt["vel"] = (torch.as_tensor(vels, dtype=torch.float32, device="cuda"), envs_idx)

    def set_active(self, actives, envs_idx=None):
        a = torch.as_tensor(actives, device="cuda")
        self._tgt["act"] = (a, envs_idx)
        self.active = bool((a == ACTIVE).any())

    def activate(self):
        self.set_active(ACTIVE)

    def deactivate(self):
        self.set_active(INACTIVE)

    def process_input(self, in_backward=False):
        diff = self._solver._diff
        if diff is not None:  # differentiable mode: the targets enter the torch state (their grads flow back)
            if self._tgt["act"] is not None:  # activity: a constant of the steps to come
                a, envs_idx = self._tgt["act"]
                a = torch.as_tensor(a, device="cuda")
                if a.ndim == 0:
                    a = a.reshape(1).expand(self._n_particles)
                diff.set_active(self._particle_start, self._n_particles, a == ACTIVE, self._envs(envs_idx))
            for key in ("pos", "vel", "actu"):  # positions first: setting positions resets velocities
                if self._tgt.get(key) is not None:
                    val, envs_idx = self._tgt[key]
                    diff.write(key, self._particle_start, self._n_particles, val, self._envs(envs_idx))
            self._tgt = {"pos": None, "vel": None, "act": None}
            return
        # positions first: setting positions resets velocities (particle_entity.py:448-451)
        if self._tgt["pos"] is not None:
            self.set_particles_pos(*self._tgt["pos"][:1], envs_idx=self._tgt["pos"][1])
        if self._tgt["vel"] is not None:
            self.set_particles_vel(self._tgt["vel"][0], envs_idx=self._tgt["vel"][1])
        if self._tgt["act"] is not None:
            self.set_particles_active(self._tgt["act"][0], envs_idx=self._tgt["act"][1])
        self._tgt = {"pos": None, "vel": None, "act": None}

    # ------------------------------------------------------------------ immediate setters/getters
    def set_particles_pos(self, poss, particles_idx_local=None, envs_idx=None):
        """mpm_solver.py:840-859: positions set, v/F/C/Jp reset."""
        self._set_field(_lib.FIELD_POS_RESET, 3, poss, envs_idx, particles_idx_local)

    def set_particles_vel(self, vels, particles_idx_local=None, envs_idx=None):
        self._set_field(_lib.FIELD_VEL, 3, vels, envs_idx, particles_idx_local)

    def set_particles_active(self, actives, particles_idx_local=None, envs_idx=None):
        a = torch.as_tensor(actives, device="cuda").to(torch.float32)
        self._set_field(_lib.FIELD_ACTIVE, 1, a[..., None], envs_idx, particles_idx_local)

    def _n_groups(self):
        n = getattr(self._material, "n_groups", None)
        if n is None:
            raise GenesisException("This entity's material is not a muscle.")
        return int(n)

    def _muscle_groups(self):
        g = getattr(self, "_muscle_group", None)
        if g is None:
            g = torch.zeros(self._n_particles, dtype=torch.long, device="cuda")
            self._muscle_group = g
        return g

    def set_particles_actu(self, actus, particles_idx_local=None, envs_idx=None):
        """Per-particle actuation [B, n_sel] ([n_sel] with one env), or [B, n_sel, n_groups] from which
        each particle takes its own group's value (mpm_solver.py:959-972)."""
        a = torch.as_tensor(actus, dtype=torch.float32, device="cuda")
        if a.ndim == 3:
            grp = self._muscle_groups()
            if particles_idx_local is not None:
                grp = grp[torch.as_tensor(particles_idx_local, device="cuda", dtype=torch.long).reshape(-1)]
            a = torch.gather(a, 2, grp.reshape(1, -1, 1).expand(a.shape[0], -1, 1))[..., 0]
        if self._solver._diff is not None:  # differentiable mode: an input of the next step (process_input)
            if particles_idx_local is not None:
                raise GenesisException("In differentiable mode the actuation is set for all of an entity's particles.")
            self._tgt["actu"] = (a, envs_idx)
            return
        self._set_field(_lib.FIELD_ACTU, 1, a[..., None], envs_idx, particles_idx_local)

    def set_actuation(self, actus, envs_idx=None):
        """Actuation of each muscle group (mpm_entity.py:425-440): a scalar, [n_groups], [B, n_groups]
        or [B, n_particles, n_groups]; every particle takes the value of its group."""
        n_groups = self._n_groups()
        a = torch.as_tensor(actus, dtype=torch.float32, device="cuda")
        if a.ndim == 0:
            a = a.reshape(1).expand(n_groups)
        if a.shape[-1] != n_groups:
            raise GenesisException(f"actuation must end in n_groups = {n_groups} values.")
        B = len(self._envs(envs_idx))
        if a.ndim == 1:
            a = a.reshape(1, 1, n_groups)
        elif a.ndim == 2:
            a = a.reshape(a.shape[0], 1, n_groups)
        a = torch.broadcast_to(a, (B, self._n_particles, n_groups))
        grp = self._muscle_groups()
        per = torch.gather(a, 2, grp.reshape(1, -1, 1).expand(B, -1, 1))
        if self._solver._diff is not None:  # differentiable mode: an input of the next step, on the graph of actus
            self._tgt["actu"] = (per[..., 0], envs_idx)
            return
        self._set_field(_lib.FIELD_ACTU, 1, per, envs_idx)

    def set_muscle_group(self, muscle_group):
        """Group index of every particle (mpm_entity.py:489-506); actuation values are per group."""
        self._n_groups()
        g = torch.as_tensor(muscle_group, device="cuda").to(torch.long).reshape(-1)
        if g.numel() != self._n_particles:
            raise GenesisException(f"muscle_group must have {self._n_particles} entries.")
        self._muscle_group = g.clone()

    def get_muscle_group(self):
        return self._muscle_groups().to(torch.int32)

    def set_muscle(self, muscle_group=None, muscle_direction=None):
        """mpm_entity.py:543-559: muscle group indices and/or fiber directions."""
        if muscle_group is not None:
            self.set_muscle_group(muscle_group)
        if muscle_direction is not None:
            self.set_muscle_direction(muscle_direction)

    def set_muscle_direction(self, muscle_direction):
        d = torch.as_tensor(muscle_direction, dtype=torch.float32, device="cuda").reshape(-1, 3)
        d = d.expand(self._n_particles, 3) if d.shape[0] == 1 else d
        self._set_field(_lib.FIELD_MUSCLE_DIR, 3, d, None)
        if self._solver._diff is not None:
            self._solver._diff.set_muscle_direction(self._particle_start, self._n_particles, d)

    def set_free(self, free):
        f = torch.as_tensor(free, device="cuda").to(torch.float32).reshape(-1)
        f = f.expand(self._n_particles) if f.numel() == 1 else f
        self._set_field(_lib.FIELD_FREE, 1, f[:, None], None)

    def get_free(self):
        return self._get_field(_lib.FIELD_FREE, 1, None)[0, :, 0] != 0

    def _diff_slice(self, k, envs_idx):
        x = self._solver._diff.stacked()[k]
        envs = self._envs(envs_idx)
        return self._squeeze(x[envs, self._particle_start: self._particle_start + self._n_particles])

    def get_particles_pos(self, envs_idx=None):
        if self._solver._diff is not None:
            return self._diff_slice(0, envs_idx)
        return self._squeeze(self._get_field(_lib.FIELD_POS, 3, envs_idx))

    def get_particles_vel(self, envs_idx=None):
        if self._solver._diff is not None:
            return self._diff_slice(1, envs_idx)
        return self._squeeze(self._get_field(_lib.FIELD_VEL, 3, envs_idx))

    def get_particles_active(self, envs_idx=None):
        return self._squeeze(self._get_field(_lib.FIELD_ACTIVE, 1, envs_idx)[..., 0] != 0)

    def get_particles_actu(self, envs_idx=None):
        return self._squeeze(self._get_field(_lib.FIELD_ACTU, 1, envs_idx)[..., 0])

    def get_state(self) -> MPMEntityState:
        """mpm_entity.py:278-302 / get_frame :305-352."""
        B = self._solver._B
        st = MPMEntityState(self, self._scene.sim.cur_step_global, B, self._n_particles, "cuda")
        diff = self._solver._diff
        if diff is not None:  # autograd-connected slices of the differentiable state
            a, b = self._particle_start, self._particle_start + self._n_particles
            x, v, C, F, Jp = diff.stacked()
            st.pos, st.vel, st.C, st.F, st.Jp = x[:, a:b], v[:, a:b], C[:, a:b], F[:, a:b], Jp[:, a:b]
            st.active = torch.ones((B, self._n_particles), dtype=torch.int64, device="cuda")
            diff.queried.append((diff.substeps_taken, st, a))
            return st
        st.pos = self._get_field(_lib.FIELD_POS, 3, None)
        st.vel = self._get_field(_lib.FIELD_VEL, 3, None)
        st.C = self._get_field(_lib.FIELD_C, 9, None).reshape(B, -1, 3, 3)
        st.F = self._get_field(_lib.FIELD_F, 9, None).reshape(B, -1, 3, 3)
        st.Jp = self._get_field(_lib.FIELD_JP, 1, None)[..., 0]
        st.active = (self._get_field(_lib.FIELD_ACTIVE, 1, None)[..., 0] != 0).to(torch.int64)
        return st

    def get_mass(self, envs_idx=None):
        """particle_entity.py:692-714: total mass (particle_volume * rho, unscaled), per env."""
        envs = self._envs(envs_idx)
        m = np.float32(np.float32(self._solver.particle_volume) * np.float32(self._material.rho)) * self._n_particles
        m = float(m) / self._solver.particle_volume_scale
        out = torch.full((len(envs),), m, dtype=torch.float32, device="cuda")
        return out[0] if self._scene.n_envs == 0 else out

    def get_particles_in_bbox(self, bbox_min, bbox_max):
        pos = self._get_field(_lib.FIELD_POS, 3, None)
        lo = torch.as_tensor(bbox_min, dtype=torch.float32, device="cuda")
        hi = torch.as_tensor(bbox_max, dtype=torch.float32, device="cuda")
        return ((pos >= lo) & (pos <= hi)).all(-1)

    # ------------------------------------------------------------------ properties
    @property
    def uid(self):
        return self._uid

    @property
    def idx(self):
        return self._idx

    @property
    def name(self):
        return self._name

    @property
    def morph(self):
        return self._morph

    @property
    def material(self):
        return self._material

    @property
    def surface(self):
        return self._surface

    @property
    def solver(self):
        return self._solver

    @property
    def scene(self):
        return self._scene

    @property
    def sim(self):
        return self._scene.sim

    @property
    def n_particles(self):
        return self._n_particles

    @property
    def particle_start(self):
        return self._particle_start

    @property
    def particle_end(self):
        return self._particle_start + self._n_particles

    @property
    def particle_size(self):
        return self._particle_size

    @property
    def init_particles(self):
        return self._particles
