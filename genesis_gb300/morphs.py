"""Morphs and particle sampling of the MPM path.

Mirrors the 'regular' and 'random' samplers of genesis/utils/particle.py
(n_particles_3D :36-41, _box_to_particles :180-208, sphere/cylinder rejection :231-278) and
the morph fields of genesis/options/morphs.py (Box :186, Sphere :351, Cylinder, Mesh :630,
Nowhere :128).  Sampling runs on the host with numpy's global RNG (seeded by gs.init(seed=...)),
like the reference; particles are then rotated by the morph's quaternion and translated
to its position (particle_entity.py:318-329).

Difference from the reference: for Sphere/Cylinder the reference rejects lattice points
against a triangulated icosphere/cylinder mesh (trimesh + igl signed distance); here the
rejection is against the exact shape, so counts can differ by the points between the
polyhedron and the true surface.  Box sampling is identical.  The 'pbs' sampler needs the
reference's prebuilt binary and falls back to 'random' (as the reference does on failure).
"""

from __future__ import annotations

import math

import numpy as np

from .exceptions import GenesisException


def n_particles_1D(p_size=0.01, length=1.0):
    return max(1, round(length / p_size))


def n_particles_3D(p_size=0.01, size=(1.0, 1.0, 1.0)):
    return max(1, round(size[0] / p_size)) * max(1, round(size[1] / p_size)) * max(1, round(size[2] / p_size))


def box_to_particles(p_size=0.01, pos=(0, 0, 0), size=(1, 1, 1), sampler="random"):
    """Lattice ('regular') or uniform ('random') samples of an axis-aligned box centred at pos."""
    size = np.asarray(size, dtype=np.float64)
    pos = np.asarray(pos, dtype=np.float64)
    lower = pos - size / 2
    upper = pos + size / 2
    if sampler == "random":
        n = n_particles_3D(p_size, size)
        return np.random.uniform(low=lower, high=upper, size=(n, 3))
    if sampler == "regular":
        n = [n_particles_1D(p_size, size[d]) for d in range(3)]
        p_lower = lower + 0.5 * p_size
        p_upper = upper - 0.5 * p_size
        axes = [np.linspace(p_lower[d], p_upper[d], n[d]) for d in range(3)]
        return np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape((-1, 3))
    raise GenesisException(f"Unsupported sampler method: {sampler}.")


def sphere_to_particles(p_size=0.01, pos=(0, 0, 0), radius=0.5, sampler="random"):
    p = box_to_particles(p_size, pos, (2 * radius,) * 3, sampler)
    return p[np.linalg.norm(p - np.asarray(pos), axis=1) <= radius]


def cylinder_to_particles(p_size=0.01, pos=(0, 0, 0), radius=0.5, height=1.0, sampler="random"):
    p = box_to_particles(p_size, pos, (2 * radius, 2 * radius, height), sampler)
    r = np.linalg.norm(p[:, :2] - np.asarray(pos)[:2], axis=1)
    return p[r <= radius]


def euler_to_quat(euler_deg) -> np.ndarray:
    """Extrinsic x-y-z (roll, pitch, yaw) in degrees to a (w, x, y, z) quaternion."""
    r, p, y = (math.radians(float(a)) for a in euler_deg)
    cr, sr = math.cos(r / 2), math.sin(r / 2)
    cp, sp = math.cos(p / 2), math.sin(p / 2)
    cy, sy = math.cos(y / 2), math.sin(y / 2)
    return np.array(
        [
            cr * cp * cy + sr * sp * sy,
            sr * cp * cy - cr * sp * sy,
            cr * sp * cy + sr * cp * sy,
            cr * cp * sy - sr * sp * cy,
        ]
    )


def quat_to_R(q) -> np.ndarray:
    w, x, y, z = (float(v) for v in q)
    n = math.sqrt(w * w + x * x + y * y + z * z)
    w, x, y, z = w / n, x / n, y / n, z / n
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
    )


class Morph:
    _fields: tuple[str, ...] = ("pos", "euler", "quat", "visualization", "collision")
    pos = (0.0, 0.0, 0.0)
    euler = (0.0, 0.0, 0.0)
    quat = None
    visualization = True
    collision = True

    def __init__(self, **kw):
        fields = set()
        for cls in type(self).__mro__:
            fields |= set(getattr(cls, "_fields", ()))
        unknown = set(kw) - fields
        if unknown:
            raise GenesisException(f"Unrecognized attribute(s) for {type(self).__name__}: {sorted(unknown)}")
        for f in fields:
            setattr(self, f, kw.get(f, getattr(type(self), f)))
        self.pos = tuple(float(v) for v in self.pos)
        if self.quat is None:
            self.quat = tuple(euler_to_quat(self.euler))
        self._post_init()

    def _post_init(self) -> None:
        pass

    def _local_particles(self, p_size: float, sampler: str) -> np.ndarray:
        raise NotImplementedError

    def sample(self, p_size: float, sampler: str) -> np.ndarray:
        if sampler.startswith("pbs"):
            sampler = "random"
        local = self._local_particles(p_size, sampler)
        R = quat_to_R(self.quat)
        return (local @ R.T + np.asarray(self.pos)).astype(np.float64)


class Box(Morph):
    _fields = ("size", "lower", "upper")
    size = None
    lower = None
    upper = None

    def _post_init(self) -> None:
        if self.lower is not None and self.upper is not None:
            lo, up = np.asarray(self.lower, float), np.asarray(self.upper, float)
            if not np.all(up > lo):
                raise GenesisException("Invalid lower and upper corner.")
            self.pos = tuple((lo + up) / 2)
            self.size = tuple(up - lo)
        if self.size is None:
            raise GenesisException("Either `size` or `lower` and `upper` must be specified.")
        self.size = tuple(float(v) for v in self.size)

    def _local_particles(self, p_size, sampler):
        return box_to_particles(p_size, (0, 0, 0), self.size, sampler)


class Sphere(Morph):
    _fields = ("radius",)
    radius = 0.5

    def _local_particles(self, p_size, sampler):
        return sphere_to_particles(p_size, (0, 0, 0), self.radius, sampler)


class Cylinder(Morph):
    _fields = ("radius", "height")
    radius = 0.5
    height = 1.0

    def _local_particles(self, p_size, sampler):
        return cylinder_to_particles(p_size, (0, 0, 0), self.radius, self.height, sampler)


def load_obj(path):
    """Vertices [V, 3] and triangles [F, 3] of a Wavefront OBJ file ('v' and 'f' records; polygons
    are split into fans; 'f' entries may carry /vt/vn indices; negative indices count from the end)."""
    verts, faces = [], []
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if not parts:
                continue
            if parts[0] == "v" and len(parts) >= 4:
                verts.append([float(parts[1]), float(parts[2]), float(parts[3])])
            elif parts[0] == "f" and len(parts) >= 4:
                idx = []
                for tok in parts[1:]:
                    i = int(tok.split("/")[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                faces.extend([idx[0], idx[k], idx[k + 1]] for k in range(1, len(idx) - 1))
    if not verts or not faces:
        raise GenesisException(f"No triangles in mesh file: {path}.")
    return np.asarray(verts, dtype=np.float64), np.asarray(faces, dtype=np.int64)


def winding_number(points, verts, faces, chunk=4096):
    """Generalized winding number of a triangle mesh at each point (Jacobson, Kavan, Sorkine-Hornung
    2013: the sum of the triangles' signed solid angles over 4 pi, each by the formula of van
    Oosterom and Strackee 1983); close to 1 inside a closed, outward-oriented mesh, 0 outside.
    Runs on the GPU through torch when one is present (set-up work, not the substep path)."""
    try:
        import torch

        dev = "cuda" if torch.cuda.is_available() else "cpu"
        tri = torch.as_tensor(verts[faces], dtype=torch.float64, device=dev)  # [F, 3, 3]
        out = []
        for k in range(0, len(points), chunk):
            p = torch.as_tensor(points[k:k + chunk], dtype=torch.float64, device=dev)
            a, b, c = (tri[None, :, i, :] - p[:, None, :] for i in range(3))
            la, lb, lc = a.norm(dim=-1), b.norm(dim=-1), c.norm(dim=-1)
            det = (a * torch.cross(b, c, dim=-1)).sum(-1)
            den = la * lb * lc + (a * b).sum(-1) * lc + (b * c).sum(-1) * la + (c * a).sum(-1) * lb
            out.append((2.0 * torch.atan2(det, den)).sum(-1) / (4.0 * math.pi))
        return torch.cat(out).cpu().numpy()
    except ImportError:
        tri = verts[faces]
        out = []
        for k in range(0, len(points), chunk):
            p = points[k:k + chunk]
            a, b, c = (tri[None, :, i, :] - p[:, None, :] for i in range(3))
            la, lb, lc = (np.linalg.norm(x, axis=-1) for x in (a, b, c))
            det = np.einsum("pfi,pfi->pf", a, np.cross(b, c))
            den = la * lb * lc + np.einsum("pfi,pfi->pf", a, b) * lc + np.einsum("pfi,pfi->pf", b, c) * la + \
                np.einsum("pfi,pfi->pf", c, a) * lb
            out.append((2.0 * np.arctan2(det, den)).sum(-1) / (4.0 * math.pi))
        return np.concatenate(out)


class Mesh(Morph):
    """A mesh from a Wavefront OBJ `file` (or `vertices` [V, 3] and `faces` [F, 3] given directly),
    scaled by `scale` (float or 3-tuple), then placed by pos / euler / quat (options/morphs.py:630-700).
    Particles: the box sampler over the scaled mesh's bounds, keeping the points inside the mesh
    (utils/particle.py:48-82, where igl's signed distance < 0 decides; here a generalized winding
    number > 0.5, the same test for a closed mesh).  The mesh vertices become the entity's visual
    vertices (skinned to the particles)."""

    _fields = ("file", "scale", "vertices", "faces")
    file = None
    scale = 1.0
    vertices = None
    faces = None

    def _post_init(self) -> None:
        if self.vertices is None or self.faces is None:
            if self.file is None:
                raise GenesisException("Mesh needs `file` or `vertices` and `faces`.")
            self.vertices, self.faces = load_obj(self.file)
        v = np.asarray(self.vertices, dtype=np.float64).reshape(-1, 3)
        self.faces = np.asarray(self.faces, dtype=np.int64).reshape(-1, 3)
        self.vertices = v * np.broadcast_to(np.asarray(self.scale, dtype=np.float64), (3,))

    def _local_particles(self, p_size, sampler):
        lo, hi = self.vertices.min(0), self.vertices.max(0)
        p = box_to_particles(p_size, (lo + hi) / 2, hi - lo, sampler)
        return p[winding_number(p, self.vertices, self.faces) > 0.5]

    def visual_vertices(self) -> np.ndarray:
        """The mesh vertices in the world frame (the reference's vmesh after its transform)."""
        return self.vertices @ quat_to_R(self.quat).T + np.asarray(self.pos)


class Nowhere(Morph):
    """Particles parked outside the domain, inactive until set (morphs.py:128)."""

    _fields = ("n_particles",)
    n_particles = 0

    def _post_init(self) -> None:
        if int(self.n_particles) <= 0:
            raise GenesisException("`n_particles` must be positive.")

    def sample(self, p_size, sampler):
        return np.zeros((int(self.n_particles), 3))


def sample_regular_on_device(shape: str, pos, size, p_size, stream=None):
    """The 'regular' samplers above computed on the GPU (libgbmpm mpm_sample_regular): returns a
    float32 CUDA tensor [n, 3] equal to box/sphere/cylinder_to_particles(..., 'regular') rounded to
    float32.  shape: 'box' (size = extents), 'sphere' (size = radius), 'cylinder' (size =
    (radius, height))."""
    import ctypes

    import torch

    from . import _lib

    kinds = {"box": 0, "sphere": 1, "cylinder": 2}
    if shape not in kinds:
        raise GenesisException(f"Unsupported shape: {shape}.")
    sz = np.zeros(3)
    sz[: np.size(size)] = np.atleast_1d(np.asarray(size, dtype=np.float64))
    p = (ctypes.c_double * 3)(*np.asarray(pos, dtype=np.float64))
    s = (ctypes.c_double * 3)(*sz)
    lib = _lib.load()
    h = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream if stream is None else stream)
    n = ctypes.c_int64()
    _lib.check(lib.mpm_sample_regular(kinds[shape], p, s, float(p_size), None, 0, ctypes.byref(n), h), None,
               "mpm_sample_regular")
    out = torch.empty((max(1, n.value), 3), dtype=torch.float32, device="cuda")
    _lib.check(lib.mpm_sample_regular(kinds[shape], p, s, float(p_size), out.data_ptr(), n.value, ctypes.byref(n), h),
               None, "mpm_sample_regular")
    return out[: n.value]
