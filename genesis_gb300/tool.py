"""Tool entities (genesis/engine/entities/tool_entity/tool_entity.py, mesh.py): a kinematic mesh
that pushes MPM particles.

A tool carries the signed-distance grid of its mesh (Mesh.process_mesh: the mesh centred on its
bounds and divided by its largest extent, then scaled by the morph) and a pose (pos, quat) that
advances every substep from its velocity and angular velocity (ToolEntity.advect, never below the
tool solver's floor height).  In the grid op it acts on the node velocities as Mesh.collide does
(legacy_coupler.py:349-354, 386-387).  Here each tool is one library collider of shape "tool" per
environment: the library moves it, and `get_state` reads its pose back.  Inputs set with
`set_position` / `set_quaternion` / `set_velocity` take effect at the start of the next
`scene.step()`, as the reference's `process_input` applies them at the step's first frame.
"""

from __future__ import annotations

import dataclasses
from pathlib import Path

import numpy as np
import torch

from .exceptions import GenesisException
from .states import ToolEntityState


def _rows(value, B: int, width: int, name: str) -> np.ndarray:
    a = value.detach().cpu().numpy() if isinstance(value, torch.Tensor) else np.asarray(value)
    a = np.asarray(a, dtype=np.float64)
    if a.shape == (width,):
        a = np.broadcast_to(a, (B, width))
    if a.shape != (B, width):
        raise GenesisException(f"{name} must have shape ({width},) or ({B}, {width}).")
    return np.array(a)


class ToolEntity:
    def __init__(self, scene, idx: int, solver, material, morph, surface=None, name: str | None = None):
        from .coupling import SDFGrid
        from .morphs import Mesh

        if not isinstance(morph, Mesh):
            raise GenesisException("A tool entity is made from a single mesh (gs.morphs.Mesh).")
        self._scene, self._idx, self._solver = scene, idx, solver
        self._material, self._morph, self._surface = material, morph, surface
        stem = Path(morph.file).stem if getattr(morph, "file", None) else "tool"
        self._name = name if name is not None else f"{stem}_{idx}"
        self._uid = f"tool{idx:04d}"
        self._init_pos = np.asarray(morph.pos, dtype=np.float64)
        self._init_quat = np.asarray(morph.quat, dtype=np.float64)
        scale = np.broadcast_to(np.asarray(morph.scale, dtype=np.float64), (3,))
        self.sdf = (SDFGrid.from_mesh(morph.vertices / scale, morph.faces, res=material.sdf_res, scale=morph.scale)
                    if material.collision else None)
        self._tgt = {"pos": None, "quat": None, "vel": None, "ang": None}
        self._B = 1
        self._floor = 0.0
        self._pos = self._quat = self._vel = self._ang = None
        self._col0 = -1  # index of this tool's first collider in the solver's list

    # ------------------------------------------------------------------ build and colliders
    def _build(self, B: int, floor_height: float) -> None:
        self._B = B
        self._floor = float(floor_height)
        self.reset()

    def reset(self) -> None:
        """The initial state (ToolEntity.set_init_state): morph pose, at rest."""
        B = self._B
        self._pos = np.tile(self._init_pos, (B, 1))
        self._quat = np.tile(self._init_quat, (B, 1))
        self._vel = np.zeros((B, 3))
        self._ang = np.zeros((B, 3))

    def _colliders(self):
        from .coupling import Collider

        if self.sdf is None:
            return []
        m = self._material
        return [Collider("tool", pos=tuple(self._pos[b]), quat=tuple(self._quat[b]), lin_vel=tuple(self._vel[b]),
                         ang_vel=tuple(self._ang[b]), coup_friction=float(m.friction),
                         coup_softness=float(m.coup_softness), env=b if self._B > 1 else -1, sdf=self.sdf,
                         floor_height=self._floor)
                for b in range(self._B)]

    def _sync_pose(self, poses: np.ndarray) -> None:
        """Take the current pose of this tool's colliders ([n_colliders, 7]) from the library."""
        if self.sdf is None or self._col0 < 0:
            return
        p = poses[self._col0:self._col0 + self._B]
        self._pos, self._quat = p[:, :3].copy(), p[:, 3:].copy()

    # ------------------------------------------------------------------ inputs (applied at the next step)
    def set_position(self, pos):
        self._tgt["pos"] = pos

    def set_quaternion(self, quat):
        self._tgt["quat"] = quat

    def set_velocity(self, vel=None, ang=None):
        if vel is not None:
            self._tgt["vel"] = vel
        if ang is not None:
            self._tgt["ang"] = ang

    def _pending(self) -> bool:
        return any(v is not None for v in self._tgt.values())

    def _tool_index(self) -> int:
        return self._solver._tools.index(self)

    def process_input(self, in_backward: bool = False) -> None:
        """Apply the inputs set since the last step to the host copy of the state (the solver then
        uploads the colliders); in differentiable mode position and velocity enter the scene's
        differentiable state through torch ops (their gradients reach the tensors passed in, as
        process_input_grad delivers them in the reference)."""
        B = self._B
        diff = getattr(self._solver, "_diff", None)
        if diff is not None:
            t = self._tool_index()
            envs = list(range(B))
            for field, key in (("tool_pos", "pos"), ("tool_vel", "vel")):
                v = self._tgt[key]
                if v is not None:
                    v = v if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v, np.float64))
                    if tuple(v.shape) not in ((3,), (B, 3)):
                        raise GenesisException(f"{key} must have shape (3,) or ({B}, 3).")
                    diff.write_tool(field, t, v, envs)
            if self._tgt["quat"] is not None or self._tgt["ang"] is not None:
                q = None if self._tgt["quat"] is None else _rows(self._tgt["quat"], B, 4, "quat")
                a = None if self._tgt["ang"] is None else _rows(self._tgt["ang"], B, 3, "ang")
                diff.set_tool_orientation(t, quat=q, ang=a, envs=envs)
            self._tgt = {"pos": None, "quat": None, "vel": None, "ang": None}
            return
        if self._tgt["pos"] is not None:
            self._pos = _rows(self._tgt["pos"], B, 3, "pos")
        if self._tgt["quat"] is not None:
            self._quat = _rows(self._tgt["quat"], B, 4, "quat")
        if self._tgt["vel"] is not None:
            self._vel = _rows(self._tgt["vel"], B, 3, "vel")
        if self._tgt["ang"] is not None:
            self._ang = _rows(self._tgt["ang"], B, 3, "ang")
        self._tgt = {"pos": None, "quat": None, "vel": None, "ang": None}

    # ------------------------------------------------------------------ state
    def get_state(self) -> ToolEntityState:
        """pos, quat, vel, ang at the current frame (ToolEntity.get_state); in differentiable mode
        pos and vel are on the autograd graph of the steps."""
        diff = self._solver._diff
        if diff is not None:
            st = ToolEntityState(self, self._scene.t if hasattr(self._scene, "t") else 0, self._B, "cuda")
            st.pos, st.quat, st.vel, st.ang = diff.tool_state(self._tool_index())
            diff.queried_tools.append((diff.substeps_taken, st, self._tool_index()))
            return st
        self._solver._sync_tool_poses()
        st = ToolEntityState(self, self._scene.t if hasattr(self._scene, "t") else 0, self._B, "cuda")
        st.pos.copy_(torch.as_tensor(self._pos, dtype=torch.float32))
        st.quat.copy_(torch.as_tensor(self._quat, dtype=torch.float32))
        st.vel.copy_(torch.as_tensor(self._vel, dtype=torch.float32))
        st.ang.copy_(torch.as_tensor(self._ang, dtype=torch.float32))
        return st

    def set_state(self, f, state: ToolEntityState) -> None:
        """Set pos, quat, vel, ang at once (ToolEntity.set_state); effective immediately."""
        B = self._B
        self._pos = _rows(state.pos, B, 3, "pos")
        self._quat = _rows(state.quat, B, 4, "quat")
        self._vel = _rows(state.vel, B, 3, "vel")
        self._ang = _rows(state.ang, B, 3, "ang")
        self._solver._upload_colliders(sync=False)

    # ------------------------------------------------------------------ properties
    @property
    def idx(self):
        return self._idx

    @property
    def uid(self):
        return self._uid

    @property
    def name(self):
        return self._name

    @property
    def material(self):
        return self._material

    @property
    def morph(self):
        return self._morph

    @property
    def surface(self):
        return self._surface

    @property
    def init_pos(self):
        return self._init_pos

    @property
    def init_quat(self):
        return self._init_quat

    @property
    def solver(self):
        return self._solver

    @property
    def scene(self):
        return self._scene


def replace_pose(collider, pose):
    """The collider with the pose (pos xyz, quat wxyz) the library holds for it now."""
    return dataclasses.replace(collider, pos=tuple(float(v) for v in pose[:3]),
                               quat=tuple(float(v) for v in pose[3:7]))
