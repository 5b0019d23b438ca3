"""MPM <-> rigid coupling with kinematic colliders.

The reference couples MPM with its rigid solver inside the grid op (legacy_coupler.py:389-403):
every grid node near a rigid geom has its velocity projected against the geom (friction,
restitution, SDF influence) and the momentum change is applied back to the rigid link.  Without a
rigid solver, a `Collider` is the geom: its pose and velocity are given by the caller every step
(a kinematic body, or the rigid solver of the host application), and the reaction force and
torque the particles exert on it are read back with `MPMSolver.get_collider_forces()`.

Coupling parameters default to gs.materials.Rigid's (materials/rigid.py:81-84).

A rigid geom whose SDF the reference samples on a voxel grid (boxes, meshes) is a collider of
shape "sdf" with an `SDFGrid` (values and gradients).  A tool entity (engine/entities/tool_entity:
a kinematic mesh with a voxel SDF, friction and softness, coupled before the rigid geoms) is a
collider of shape "tool" with an `SDFGrid` of values; the library moves it every substep from its
linear and angular velocity, as ToolEntity.advect does.  Grids come from the caller:
`SDFGrid.from_mesh` bakes a tool's grid from its mesh the way the reference does (normalised mesh,
[-0.6, 0.6]^3, signed distance; here triangle distances and winding-number signs in place of
trimesh/igl), `SDFGrid.from_function` samples an analytic distance function.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import _lib
from .exceptions import GenesisException

_TYPES = {"sphere": _lib.COLLIDER_SPHERE, "plane": _lib.COLLIDER_PLANE, "box": _lib.COLLIDER_BOX,
          "sdf": _lib.COLLIDER_SDF, "tool": _lib.COLLIDER_TOOL}


@dataclasses.dataclass(eq=False)
class SDFGrid:
    """Voxel signed-distance grid in the layout of the reference's SDF data (utils/sdf.py,
    tool_entity/mesh.py): values [r0, r1, r2] in mesh-frame distance units, gradients
    [r0, r1, r2, 3] (rigid geoms; None for a tool), T_mesh_to_sdf the 4x4 map from the mesh frame
    to voxel coordinates, cell_size the voxel edge in mesh units, sdf_max the largest value."""

    values: np.ndarray
    T_mesh_to_sdf: np.ndarray
    grads: np.ndarray | None = None
    cell_size: float = 1.0
    sdf_max: float = 0.0

    @classmethod
    def from_function(cls, sdf, lower, upper, res: int, grads: bool = True) -> "SDFGrid":
        """Sample `sdf` (callable on [n, 3] mesh-frame points) on a res^3 lattice spanning the box
        [lower, upper]; gradients by central differences of half a voxel."""
        lower = np.asarray(lower, np.float64)
        upper = np.asarray(upper, np.float64)
        cell = (upper - lower) / (res - 1)
        if not np.allclose(cell, cell[0]):
            raise GenesisException("SDFGrid.from_function needs a cube (equal voxel edges).")
        ax = [lower[d] + cell[d] * np.arange(res) for d in range(3)]
        pts = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3)
        vals = np.asarray(sdf(pts), np.float64).reshape(res, res, res)
        g = None
        if grads:
            h = 0.5 * cell[0]
            g = np.stack([(np.asarray(sdf(pts + h * e)) - np.asarray(sdf(pts - h * e))) / (2 * h)
                          for e in np.eye(3)], -1).reshape(res, res, res, 3)
        T = np.eye(4)
        T[:3, :3] /= cell[0]
        T[:3, 3] = -lower / cell[0]
        return cls(values=vals.astype(np.float32), T_mesh_to_sdf=T,
                   grads=None if g is None else g.astype(np.float32), cell_size=float(cell[0]),
                   sdf_max=float(vals.max()))

    @classmethod
    def from_mesh(cls, vertices, faces, res: int = 128, scale=1.0, grads: bool = False) -> "SDFGrid":
        """A tool entity's SDF from its mesh as the reference builds it (tool_entity/mesh.py:40-58,
        utils/mesh.py:193-215): the mesh is centred on its bounding box and divided by its largest
        extent, its signed distance is sampled on res^3 points spanning [-0.6, 0.6]^3 of that frame
        (distance to the nearest triangle, negative where the generalized winding number exceeds
        0.5, in place of igl's signed distance), and T_mesh_to_sdf maps the scaled mesh frame
        (`scale`, the morph's) to voxel coordinates.  grads=True adds central-difference gradients
        (for an "sdf" rigid collider)."""
        from .morphs import winding_number

        v = np.asarray(vertices, dtype=np.float64).reshape(-1, 3)
        f = np.asarray(faces, dtype=np.int64).reshape(-1, 3)
        lo, hi = v.min(0), v.max(0)
        vn = (v - (lo + hi) / 2) / np.max(hi - lo)
        r = 0.6
        ax = np.linspace(-r, r, res)
        pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
        dist = triangle_distance(pts, vn, f)
        inside = winding_number(pts, vn, f) > 0.5
        vals = np.where(inside, -dist, dist).reshape(res, res, res)
        T = np.eye(4)
        T[:3, :3] *= (res - 1) / (2 * r)
        T[:3, 3] = (res - 1) / 2
        S = np.diag(np.append(np.broadcast_to(np.asarray(scale, dtype=np.float64), (3,)), 1.0))
        T = T @ np.linalg.inv(S)
        g = None
        if grads:
            h = 2 * r / (res - 1)
            g = np.stack(np.gradient(vals, h), -1)
        return cls(values=vals.astype(np.float32), T_mesh_to_sdf=T,
                   grads=None if g is None else g.astype(np.float32), cell_size=2 * r / (res - 1),
                   sdf_max=float(vals.max()))


def triangle_distance(points, verts, faces, chunk=2048):
    """Distance from each point to the nearest triangle of a mesh: the closest point on each triangle
    by its Voronoi regions (Ericson, Real-Time Collision Detection, 5.1.5), minimised over the
    triangles.  Through torch on the GPU when one is present (set-up work)."""
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    tri = torch.as_tensor(verts[faces], dtype=torch.float64, device=dev)
    a, b, c = tri[None, :, 0], tri[None, :, 1], tri[None, :, 2]
    ab, ac = b - a, c - a
    dot = lambda x, y: (x * y).sum(-1, keepdim=True)  # noqa: E731
    out = []
    step = chunk if dev == "cuda" else max(1, chunk // 8)
    for k in range(0, len(points), step):
        p = torch.as_tensor(points[k:k + step], dtype=torch.float64, device=dev)[:, None, :]
        ap, bp, cp = p - a, p - b, p - c
        d1, d2, d3, d4, d5, d6 = dot(ab, ap), dot(ac, ap), dot(ab, bp), dot(ac, bp), dot(ab, cp), dot(ac, cp)
        va, vb, vc = d3 * d6 - d5 * d4, d5 * d2 - d1 * d6, d1 * d4 - d3 * d2
        den = va + vb + vc
        den = torch.where(den == 0, torch.ones_like(den), den)
        q = a + ab * (vb / den) + ac * (vc / den)  # interior
        t_bc = (d4 - d3) / torch.where((d4 - d3) + (d5 - d6) == 0, torch.ones_like(d4), (d4 - d3) + (d5 - d6))
        q = torch.where((va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0), b + (c - b) * t_bc, q)
        t_ac = d2 / torch.where(d2 - d6 == 0, torch.ones_like(d2), d2 - d6)
        q = torch.where((vb <= 0) & (d2 >= 0) & (d6 <= 0), a + ac * t_ac, q)
        q = torch.where((d6 >= 0) & (d5 <= d6), c.expand_as(q), q)
        t_ab = d1 / torch.where(d1 - d3 == 0, torch.ones_like(d1), d1 - d3)
        q = torch.where((vc <= 0) & (d1 >= 0) & (d3 <= 0), a + ab * t_ab, q)
        q = torch.where((d3 >= 0) & (d4 <= d3), b.expand_as(q), q)
        q = torch.where((d1 <= 0) & (d2 <= 0), a.expand_as(q), q)
        out.append((p - q).norm(dim=-1).min(dim=1).values)
    return torch.cat(out).cpu().numpy()


@dataclasses.dataclass
class Collider:
    shape: str  # "sphere" (radius), "plane" (normal, in the collider frame), "box" (half extents)
    pos: tuple = (0.0, 0.0, 0.0)
    quat: tuple = (1.0, 0.0, 0.0, 0.0)  # (w, x, y, z)
    radius: float = 0.0
    normal: tuple = (0.0, 0.0, 1.0)
    half_extents: tuple = (0.0, 0.0, 0.0)
    lin_vel: tuple = (0.0, 0.0, 0.0)
    ang_vel: tuple = (0.0, 0.0, 0.0)
    com: tuple | None = None  # point the angular velocity turns about; defaults to pos
    coup_friction: float = 0.1
    coup_softness: float = 0.002
    coup_restitution: float = 0.0
    env: int = -1  # environment (scene) index, or -1 for every environment
    sdf: SDFGrid | None = None  # shapes "sdf" and "tool"
    floor_height: float = 0.0  # "tool": ToolOptions.floor_height

    def to_c(self, sdf_id: int = -1) -> "_lib.MpmCollider":
        if self.shape not in _TYPES:
            raise GenesisException(f"Unsupported collider shape: {self.shape}.")
        if self.shape in ("sdf", "tool") and (self.sdf is None or sdf_id < 0):
            raise GenesisException(f"A '{self.shape}' collider needs an SDFGrid.")
        if self.shape == "sdf" and self.sdf.grads is None:
            raise GenesisException("An 'sdf' collider needs an SDFGrid with gradients.")
        if not 0.0 <= self.coup_restitution <= 1.0 or self.coup_friction < 0 or self.coup_softness < 0:
            raise GenesisException("coup_friction and coup_softness must be >= 0 and coup_restitution in [0, 1].")
        c = _lib.MpmCollider()
        c.type = _TYPES[self.shape]
        c.scene = int(self.env)
        c.pos[:] = tuple(float(v) for v in self.pos)
        q = np.asarray(self.quat, dtype=np.float64)
        c.quat[:] = tuple(q)
        if self.shape == "sphere":
            c.size[:] = (float(self.radius), 0.0, 0.0)
        elif self.shape == "plane":
            c.size[:] = tuple(float(v) for v in self.normal)
        else:
            c.size[:] = tuple(float(v) for v in self.half_extents)
        c.com[:] = tuple(float(v) for v in (self.pos if self.com is None else self.com))
        c.lin_vel[:] = tuple(float(v) for v in self.lin_vel)
        c.ang_vel[:] = tuple(float(v) for v in self.ang_vel)
        c.friction = float(self.coup_friction)
        c.softness = float(self.coup_softness)
        c.restitution = float(self.coup_restitution)
        c.sdf_grid = int(sdf_id)
        c.floor_height = float(self.floor_height)
        return c


def tool(sdf: SDFGrid, pos=(0.0, 0.0, 0.0), quat=(1.0, 0.0, 0.0, 0.0), vel=(0.0, 0.0, 0.0), ang=(0.0, 0.0, 0.0),
         friction: float = 0.0, coup_softness: float = 0.01, floor_height: float = 0.0, env: int = -1) -> Collider:
    """A tool entity's collider with gs.materials.Tool defaults (materials/tool.py:29-32)."""
    return Collider(shape="tool", sdf=sdf, pos=pos, quat=quat, lin_vel=vel, ang_vel=ang, coup_friction=friction,
                    coup_softness=coup_softness, floor_height=floor_height, env=env)
