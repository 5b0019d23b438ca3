"""Differentiation form: MPM rollouts with hand-written adjoints behind torch.autograd.

`DifferentiableMPM.rollout(x0, v0, E)` runs `n_substeps` substeps of one Elastic scene with
per-particle Young's modulus E (Lame parameters from E and nu as in base.py:77-83) and returns
the final particle positions; its backward runs the adjoint substeps of libgbmpm
(mpm_diff_backward) in reverse.  Memory follows checkpoint-and-recompute like Genesis's
differentiable mode (simulator.py:372-404): the forward keeps the particle state only every
`ckpt_every` substeps; the backward re-simulates each segment from its checkpoint, keeping
that segment's states, and then walks it backwards.  The last segment's states and grids are kept
by the forward itself when they fit the same memory budget, so its re-simulation is skipped.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .exceptions import GenesisException


def lame(E: torch.Tensor, nu: float):
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


MATERIALS = {"elastic": 0, "neohookean": 1, "liquid": 2}


class DifferentiableMPM:
    def __init__(self, scene_cfg: "_lib.MpmSceneConfig", nu: float = 0.2, rho: float = 1000.0,
                 neohookean: bool = False, ckpt_every: int = 160, material: str | None = None,
                 viscous: bool = False, keep_segments: bool = False):
        """material: "elastic" (corotated; "neohookean" or neohookean=True for the neo-Hookean
        model) or "liquid" (liquid.py: mu = 0 unless viscous, F reset to J^(1/3) I every substep).
        Young's modulus E is per particle; nu and rho are shared.  keep_segments: the forward keeps
        every segment's states and grids while they fit a quarter of the free device memory (the
        backward then re-simulates none of them; memory for time), instead of the last one only."""
        self.lib = _lib.load()
        self.cfg = scene_cfg
        self.nu = float(nu)
        self.rho = float(rho)
        name = material if material is not None else ("neohookean" if neohookean else "elastic")
        if name not in MATERIALS:
            raise GenesisException(f"Unsupported differentiable material: {name}.")
        self.material = name
        self.viscous = bool(viscous)
        self.neo = MATERIALS[name]
        self.ckpt_every = int(ckpt_every)
        self.keep_segments = bool(keep_segments)
        d = scene_cfg.grid_density
        res = [int(round(d * scene_cfg.upper_bound[k]) - round(d * scene_cfg.lower_bound[k]) + 1) for k in range(3)]
        self.nodes = res[0] * res[1] * res[2]
        dev = "cuda"
        self.grid_pm = torch.zeros((self.nodes, 4), device=dev)
        self.grid_v = torch.zeros((self.nodes, 4), device=dev)
        self.g_grid_v = torch.zeros((self.nodes, 4), device=dev)
        self.g_grid_pm = torch.zeros((self.nodes, 4), device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)

    # ---- segment calls: n substeps per library call (no host round trip per substep)
    def forward_segment(self, st, mu, lam, n_sub, keep=False):
        """Run n_sub substeps from state st.  keep=False: returns the final state.  keep=True: returns
        (states [n_sub+1] as (x, v, C, F) stacked tensors, grids (pm, v) [n_sub, nodes, 4])."""
        x, v, C, F = st
        n = x.shape[0]
        ring = n_sub + 1 if keep else 2
        xs = torch.empty((ring, n, 3), device="cuda")
        vs = torch.empty((ring, n, 3), device="cuda")
        Cs = torch.empty((ring, n, 3, 3), device="cuda")
        Fs = torch.empty((ring, n, 3, 3), device="cuda")
        xs[0], vs[0], Cs[0], Fs[0] = x, v, C, F
        if keep:
            gpm = torch.empty((max(1, n_sub), self.nodes, 4), device="cuda")
            gv = torch.empty((max(1, n_sub), self.nodes, 4), device="cuda")
        else:
            gpm, gv = self.grid_pm, self.grid_v
        r = self.lib.mpm_diff_forward_seq(ctypes.byref(self.cfg), self.rho, self.neo, n, int(n_sub), xs.data_ptr(),
                                          vs.data_ptr(), Cs.data_ptr(), Fs.data_ptr(), ring, mu.data_ptr(),
                                          lam.data_ptr(), gpm.data_ptr(), gv.data_ptr(), int(keep),
                                          self.status.data_ptr(), self._s())
        _lib.check(r, None, "mpm_diff_forward_seq")
        if keep:
            return (xs, vs, Cs, Fs), (gpm, gv)
        last = n_sub % 2
        return xs[last].clone(), vs[last].clone(), Cs[last].clone(), Fs[last].clone()

    def backward_segment(self, states, grids, mu, lam, g_packed, gmu, glam, n_sub):
        """Adjoint of a kept segment; g_packed [2, 24 n]: row 0 in = dL/d(last state), out = dL/d(first)."""
        xs, vs, Cs, Fs = states
        n = xs.shape[1]
        r = self.lib.mpm_diff_backward_seq(ctypes.byref(self.cfg), self.rho, self.neo, n, int(n_sub), xs.data_ptr(),
                                           vs.data_ptr(), Cs.data_ptr(), Fs.data_ptr(), mu.data_ptr(), lam.data_ptr(),
                                           g_packed.data_ptr(), gmu.data_ptr(), glam.data_ptr(), grids[0].data_ptr(),
                                           grids[1].data_ptr(), self.g_grid_v.data_ptr(), self.g_grid_pm.data_ptr(),
                                           self.status.data_ptr(), self._s())
        _lib.check(r, None, "mpm_diff_backward_seq")

    def segment_bytes(self, n, n_sub) -> int:
        return (n_sub + 1) * 24 * 4 * n + 2 * n_sub * self.nodes * 16

    def grid_budget_bytes(self) -> int:
        """Device memory the backward may spend on one segment's grids (a quarter of what is free)."""
        free, _ = torch.cuda.mem_get_info()
        return free // 4

    @staticmethod
    def _s():
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def forward_substep(self, st, mu, lam, grids=None):
        """(x, v, C, F) -> next state (new tensors).  `grids` = (grid_pm, grid_v) buffers that keep
        this substep's grid (default: the shared scratch grid)."""
        x, v, C, F = st
        n = x.shape[0]
        gpm, gv = grids if grids is not None else (self.grid_pm, self.grid_v)
        out = (torch.empty_like(x), torch.empty_like(v), torch.empty_like(C), torch.empty_like(F))
        r = self.lib.mpm_diff_forward(ctypes.byref(self.cfg), self.rho, self.neo, n, x.data_ptr(), v.data_ptr(),
                                      C.data_ptr(), F.data_ptr(), mu.data_ptr(), lam.data_ptr(), out[0].data_ptr(),
                                      out[1].data_ptr(), out[2].data_ptr(), out[3].data_ptr(),
                                      gpm.data_ptr(), gv.data_ptr(), self.status.data_ptr(), self._s())
        _lib.check(r, None, "mpm_diff_forward")
        return out

    def new_grids(self):
        return (torch.empty((self.nodes, 4), device="cuda"), torch.empty((self.nodes, 4), device="cuda"))

    def backward_substep(self, st, mu, lam, g_out, gmu, glam, grids=None):
        """Adjoint of forward_substep at state `st` given dL/d(next state); returns dL/d(state).
        `grids` holds this substep's grid from a kept forward; without it the forward is re-run."""
        x, v, C, F = st
        n = x.shape[0]
        if grids is None:
            self.forward_substep(st, mu, lam)  # rebuild this substep's grid
            grids = (self.grid_pm, self.grid_v)
        gx1, gv1, gC1, gF1 = g_out
        gin = (torch.empty_like(x), torch.empty_like(v), torch.empty_like(C), torch.empty_like(F))
        r = self.lib.mpm_diff_backward(ctypes.byref(self.cfg), self.rho, self.neo, n, x.data_ptr(), v.data_ptr(),
                                       C.data_ptr(), F.data_ptr(), mu.data_ptr(), lam.data_ptr(), gx1.data_ptr(),
                                       gv1.data_ptr(), gC1.data_ptr(), gF1.data_ptr(), gin[0].data_ptr(),
                                       gin[1].data_ptr(), gin[2].data_ptr(), gin[3].data_ptr(), gmu.data_ptr(),
                                       glam.data_ptr(), grids[0].data_ptr(), grids[1].data_ptr(),
                                       self.g_grid_v.data_ptr(), self.g_grid_pm.data_ptr(), self.status.data_ptr(),
                                       self._s())
        _lib.check(r, None, "mpm_diff_backward")
        return gin

    def check(self):
        st = int(self.status.item())
        if st & _lib.STATUS_NAN:
            raise GenesisException("NaN detected in MPM states.")
        if st & _lib.STATUS_OOB:
            raise GenesisException("MPM particles left the simulation grid (stencil out of bounds).")

    def rollout(self, x0: torch.Tensor, v0: torch.Tensor, E: torch.Tensor, n_substeps: int) -> torch.Tensor:
        """Final positions after n_substeps from positions x0 [n,3], velocities v0 ([3] or [n,3]) and
        per-particle Young's modulus E [n] (C = 0, F = I at the start); differentiable w.r.t. x0, v0
        and E."""
        n = x0.shape[0]
        v0 = v0.expand(n, 3) if v0.dim() == 1 else v0
        C = torch.zeros((n, 3, 3), device=x0.device)
        F = torch.eye(3, device=x0.device).repeat(n, 1, 1)
        return self.advance((x0, v0, C, F), E, n_substeps)[0]

    def advance(self, state, E: torch.Tensor, n_substeps: int):
        """The state (x [n,3], v [n,3], C [n,3,3], F [n,3,3]) after n_substeps, differentiable w.r.t.
        every part of the state and E.  Calls chain, so a loss may combine intermediate states (the
        reference's differentiable mode takes losses at any frame of an episode)."""
        x, v, C, F = state
        mu, lam = lame(E, self.nu)
        if self.material == "liquid" and not self.viscous:  # liquid.py:27-31
            mu = mu * 0.0
        return _Advance.apply(self, int(n_substeps), x, v, C, F, mu, lam)


class _Advance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sim: DifferentiableMPM, n_substeps, x0, v0, C0, F0, mu, lam):
        f32 = lambda t: t.detach().float().contiguous()  # noqa: E731
        x, v, C, F = f32(x0), f32(v0), f32(C0), f32(F0)
        mu_d, lam_d = mu.detach().float().contiguous(), lam.detach().float().contiguous()
        st = (x, v, C, F)
        ckpts = {}
        kept = {}  # segments whose states and grids this forward keeps (the last one, or all with
        s = 0      # keep_segments), each while it fits the memory budget
        while s < n_substeps:
            seg = min(sim.ckpt_every, n_substeps - s)
            ckpts[s] = tuple(t.clone() for t in st)
            if ((sim.keep_segments or s + seg == n_substeps)
                    and sim.segment_bytes(x.shape[0], seg) <= sim.grid_budget_bytes()):
                kept[s] = sim.forward_segment(st, mu_d, lam_d, seg, keep=True)
                st = tuple(t[seg].clone() for t in kept[s][0])
            else:
                st = sim.forward_segment(st, mu_d, lam_d, seg)
            s += seg
        sim.check()
        sim.last_segments = (len(kept), len(ckpts))  # (kept by the forward, all)
        ctx.sim, ctx.n_substeps, ctx.ckpts, ctx.kept = sim, n_substeps, ckpts, kept
        ctx.save_for_backward(mu_d, lam_d)
        if n_substeps == 0:
            st = tuple(t.clone() for t in st)
        return st

    @staticmethod
    def backward(ctx, g_x, g_v, g_C, g_F):
        sim, n_sub = ctx.sim, ctx.n_substeps
        mu, lam = ctx.saved_tensors
        n = mu.shape[0]
        dev = mu.device
        z = lambda g, shape: (torch.zeros(shape, device=dev) if g is None else g.contiguous().float())  # noqa: E731
        g = (z(g_x, (n, 3)), z(g_v, (n, 3)), z(g_C, (n, 3, 3)), z(g_F, (n, 3, 3)))
        if n_sub == 0:
            return None, None, g[0], g[1], g[2], g[3], torch.zeros_like(mu), torch.zeros_like(lam)
        gmu = torch.zeros_like(mu)
        glam = torch.zeros_like(lam)
        starts = sorted(ctx.ckpts)
        seg_max = max((starts[i + 1] if i + 1 < len(starts) else n_sub) - starts[i] for i in range(len(starts)))
        sim.last_backward = "segments" if sim.segment_bytes(n, seg_max) <= sim.grid_budget_bytes() else "substeps"
        if sim.last_backward == "segments":
            # whole segments per library call: re-simulate keeping states and grids, then walk back
            gp = torch.zeros((2, 24 * n), device=dev)
            gp[0, : 3 * n] = g[0].reshape(-1)
            gp[0, 3 * n: 6 * n] = g[1].reshape(-1)
            gp[0, 6 * n: 15 * n] = g[2].reshape(-1)
            gp[0, 15 * n:] = g[3].reshape(-1)
            for seg_i in range(len(starts) - 1, -1, -1):
                s0 = starts[seg_i]
                s1 = starts[seg_i + 1] if seg_i + 1 < len(starts) else n_sub
                if s0 in ctx.kept:  # kept by the forward
                    states, grids = ctx.kept.pop(s0)
                else:
                    states, grids = sim.forward_segment(ctx.ckpts[s0], mu, lam, s1 - s0, keep=True)
                sim.backward_segment(states, grids, mu, lam, gp, gmu, glam, s1 - s0)
                del states, grids
            sim.check()
            return (None, None, gp[0, : 3 * n].view(n, 3).clone(), gp[0, 3 * n: 6 * n].view(n, 3).clone(),
                    gp[0, 6 * n: 15 * n].view(n, 3, 3).clone(), gp[0, 15 * n:].view(n, 3, 3).clone(), gmu, glam)
        keep = sim.nodes * 32 * seg_max <= sim.grid_budget_bytes()  # keep every substep's grid of a segment
        for seg_i in range(len(starts) - 1, -1, -1):
            s0 = starts[seg_i]
            s1 = starts[seg_i + 1] if seg_i + 1 < len(starts) else n_sub
            states = [ctx.ckpts[s0]]
            grids = []
            for k in range(s0, s1):  # re-simulate the segment (checkpoint-and-recompute)
                if keep:
                    grids.append(sim.new_grids())
                    nxt = sim.forward_substep(states[-1], mu, lam, grids[-1])
                    if k < s1 - 1:
                        states.append(nxt)
                elif k < s1 - 1:
                    states.append(sim.forward_substep(states[-1], mu, lam))
            for i in range(len(states) - 1, -1, -1):
                g = sim.backward_substep(states[i], mu, lam, g, gmu, glam, grids[i] if keep else None)
            del grids
        sim.check()
        return None, None, g[0], g[1], g[2], g[3], gmu, glam
