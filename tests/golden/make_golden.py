"""Generate golden vectors by executing the reference's own MPM code on the host.

The reference's MPM kernels (genesis/engine/solvers/mpm_solver.py: compute_F_tmp, svd, p2g,
g2p; genesis/engine/couplers/legacy_coupler.py: mpm_grid_op; genesis/engine/boundaries/
boundaries.py: CubeBoundary.impose_pos_vel) and material functions
(genesis/engine/materials/MPM/*.py) are Python bodies decorated for the Quadrants JIT, which
is not installed.  This script parses those source files, takes the function bodies as
written (decorators and type annotations removed), and executes them in float64 against a
small numpy stand-in for the Quadrants primitives they call (Matrix/Vector algebra, ndrange,
static, grouped, log/exp/pow/floor, struct fields).  qd.svd is stood in by LAPACK's SVD
brought to the rotation-variant convention (det U = det V = +1, sign in the last singular
value); that part is not the reference's code and only rotation-invariant results are
compared downstream.  gs.EPS is the float32 value (precision "32").

Outputs (committed, small):
  materials.npz     per material variant: F_tmp, Jp, actu, mdir -> F_new, Jp_new, stress
  substep_small.npz a 9-material scene on a 17^3 grid: input state, grid (momentum, mass)
                    after the first P2G, states after 1 and 10 substeps
  force_fields.npz  the same scene with six force fields in the grid op (force_fields.py):
                    states after 1 and 5 substeps
  rigid_coupling.npz the same scene coupled with a sphere, a tilted plane and a voxel-SDF box
                    (legacy_coupler.py rigid collision, utils/sdf.py, utils/geom.py): state after
                    3 substeps, the reaction accumulated on each link
  cpic_coupling.npz rigid_coupling's scene with MPMOptions.enable_CPIC (mpm_solver.py p2g/g2p,
                    legacy_coupler.py mpm_surface_to_particle)
  particle_coupling.npz the same scene coupled with an SPH and a PBD particle set through their
                    spatial hash (legacy_coupler.py, utils/geom.py SpatialHasher): state and
                    the sets' velocities after 4 substeps
  particle_constraints.npz the same scene with particles attached to two moving kinematic links
                    and to their start positions, some released midway (mpm_solver.py
                    particle constraints): state after 5 substeps
  custom_field.npz  the same scene with a Custom force field (a user function) between Drag and
                    Constant: state after 5 substeps
  tool_coupling.npz the same scene with a moving, spinning box tool (tool_entity/mesh.py,
                    tool_entity.py, boundaries.py FloorBoundary): state and tool pose after 4
                    substeps

Run from the repository root with the reference checked out:
    python tests/golden/make_golden.py /path/to/genesis-reference
"""

from __future__ import annotations

import ast
import itertools
import math
import os
import sys
import textwrap
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EPS32 = float(np.finfo(np.float32).eps)


# ----------------------------------------------------------------------------- Quadrants stand-in
class QMat(np.ndarray):
    """numpy array with the Matrix/Vector methods the reference code calls."""

    def __new__(cls, a, dtype=np.float64):
        return np.array(a, dtype=dtype).view(cls)

    def determinant(self):
        return float(np.linalg.det(np.asarray(self, dtype=np.float64)))

    def transpose(self):  # noqa: A003
        return np.asarray(self).T.copy().view(QMat)

    def norm(self, eps=0.0):
        return float(math.sqrt(float(np.sum(np.asarray(self, dtype=np.float64) ** 2)) + eps))

    def norm_sqr(self):
        return float(np.sum(np.asarray(self, dtype=np.float64) ** 2))

    def normalized(self):
        return (np.asarray(self) / self.norm()).view(QMat)

    def inverse(self):
        return np.linalg.inv(np.asarray(self, dtype=np.float64)).view(QMat)

    def outer_product(self, other):
        return np.outer(np.asarray(self), np.asarray(other)).view(QMat)

    def cast(self, dtype):
        return np.asarray(self).astype(dtype).view(QMat)

    def dot(self, other):
        return float(np.dot(np.asarray(self), np.asarray(other)))

    def cross(self, other):
        return np.cross(np.asarray(self), np.asarray(other)).view(QMat)

    def any(self, *a, **k):  # noqa: A003
        return bool(np.asarray(self).any(*a, **k))

    x = property(lambda self: float(self[0]))
    y = property(lambda self: float(self[1]))
    z = property(lambda self: float(self[2]))

    def fill(self, v):
        np.ndarray.fill(self, v)


class _MatrixNS:
    @staticmethod
    def zero(dt, n, m=None):
        return QMat(np.zeros((n, m) if m else (n,)))

    @staticmethod
    def identity(dt, n):
        return QMat(np.eye(n))

    def __call__(self, rows, dt=None):
        return QMat(rows)


class _VectorNS(_MatrixNS):
    @staticmethod
    def zero(dt, n):
        return QMat(np.zeros(n))

    def __call__(self, vals, dt=None):
        return QMat(vals)


def _ndrange(*dims):
    return itertools.product(*[range(d) if isinstance(d, (int, np.integer)) else range(*d) for d in dims])


def _svd(A, dt=None):
    U, s, Vh = np.linalg.svd(np.asarray(A, dtype=np.float64))
    V = Vh.T.copy()
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(V) < 0:
        V[:, 2] *= -1
        s[2] *= -1
    return QMat(U), QMat(np.diag(s)), QMat(V)


def make_qd():
    qd = types.ModuleType("quadrants_standin")
    qd.Matrix = _MatrixNS()
    qd.Vector = _VectorNS()
    qd.static = lambda x, *a: x
    qd.grouped = lambda it: (QMat(np.array(t, dtype=np.int64), dtype=np.int64) for t in it)
    qd.ndrange = _ndrange
    qd.log = lambda x: np.log(x)
    qd.exp = lambda x: np.exp(x)
    qd.pow = lambda x, y: np.power(x, y)
    qd.sqrt = lambda x: np.sqrt(x)
    qd.cos = lambda x: math.cos(x)
    qd.sin = lambda x: math.sin(x)
    qd.cast = lambda x, dt: dt(x)
    qd.floor = lambda x, dt=None: (np.floor(x).astype(np.int64 if dt is not None else np.float64).view(QMat)
                                   if isinstance(x, np.ndarray) else math.floor(x))
    qd.max = lambda a, b: np.maximum(a, b).view(QMat) if isinstance(a, np.ndarray) or isinstance(b, np.ndarray) else max(a, b)
    qd.min = lambda a, b: np.minimum(a, b).view(QMat) if isinstance(a, np.ndarray) or isinstance(b, np.ndarray) else min(a, b)
    qd.abs = abs
    qd.select = lambda c, a, b: a if c else b
    qd.svd = _svd
    qd.math = types.SimpleNamespace(isnan=lambda x: bool(np.isnan(x)), sqrt=lambda x: math.sqrt(x))
    qd.i32, qd.f32 = np.int64, np.float64
    return qd


def make_gs():
    gs = types.ModuleType("genesis_standin")
    gs.qd_float = np.float64
    gs.qd_int = np.int64
    gs.EPS = EPS32

    def _raise(msg, *a, **k):
        raise RuntimeError(msg)

    gs.raise_exception = _raise
    return gs


def _flat_index(idx):
    if not isinstance(idx, tuple):
        idx = (idx,)
    out = []
    for v in idx:
        if isinstance(v, (tuple, list, np.ndarray)):
            out.extend(int(x) for x in np.asarray(v).reshape(-1))
        else:
            out.append(int(v))
    return tuple(out)


class StructField:
    """Struct field with per-member numpy storage; item access returns a write-through record."""

    def __init__(self, shape, members):
        object.__setattr__(self, "_d", {k: np.zeros(tuple(shape) + tuple(e)) for k, e in members.items()})

    def __getitem__(self, idx):
        return _Record(self, _flat_index(idx))


class _Record:
    __slots__ = ("_f", "_i")

    def __init__(self, f, i):
        object.__setattr__(self, "_f", f)
        object.__setattr__(self, "_i", i)

    def __getattr__(self, k):
        v = self._f._d[k][self._i]
        return QMat(v) if np.ndim(v) else v.item()

    def __setattr__(self, k, v):
        self._f._d[k][self._i] = np.asarray(v)


# ----------------------------------------------------------------------------- source extraction
def extract_functions(path, names, ns):
    """Compile module-level functions `names` of `path` (decorators/annotations removed) into ns,
    so that they call each other through ns."""
    ns.setdefault("_qd_copy", _qd_copy)
    tree = ast.parse(open(path).read())
    found = set()
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            node.decorator_list = []
            node.returns = None
            for a in node.args.args + node.args.kwonlyargs:
                a.annotation = None
            node = _ValueAssign().visit(node)
            exec(compile(ast.fix_missing_locations(ast.Module(body=[node], type_ignores=[])), path, "exec"), ns)
            found.add(node.name)
    if set(names) - found:
        raise RuntimeError(f"{path} lacks {set(names) - found}")
    return {k: ns[k] for k in names}


GEOM_TYPE = types.SimpleNamespace(PLANE=0, SPHERE=1, ELLIPSOID=2, CYLINDER=3, CAPSULE=4, BOX=5, MESH=6, TERRAIN=7)


def rigid_namespace(ref, ns):
    """Namespace for the coupler's rigid-collision methods: the reference's SDF functions
    (genesis/utils/sdf.py), geometry helpers (genesis/utils/geom.py) and rigid-link velocity /
    coupling-force functions (rigid/abd/forward_dynamics.py, rigid/abd/misc.py), all executed as written."""
    gns = dict(ns)
    gns["gs"] = types.SimpleNamespace(**vars(ns["gs"]))
    gns["gs"].GEOM_TYPE = GEOM_TYPE
    gns["gs"].qd_vec3 = lambda v: QMat(v)
    gu = types.SimpleNamespace()
    gns["gu"] = gu
    extract_functions(os.path.join(ref, "genesis/utils/geom.py"),
                      ["qd_normalize", "qd_transform_by_quat", "qd_inv_quat", "qd_inv_transform_by_quat",
                       "qd_transform_by_T", "qd_inv_transform_by_trans_quat"], gns)
    for k in ("qd_normalize", "qd_transform_by_quat", "qd_inv_quat", "qd_inv_transform_by_quat", "qd_transform_by_T",
              "qd_inv_transform_by_trans_quat"):
        setattr(gu, k, gns[k])
    sdf_names = ["sdf_func_world", "sdf_func_world_local", "sdf_func_sdf", "sdf_func_is_outside_sdf_grid",
                 "sdf_func_proxy_sdf", "sdf_func_true_sdf", "sdf_func_ravel_cell_idx", "sdf_func_grad",
                 "sdf_func_proxy_grad", "sdf_func_true_grad", "sdf_func_normal_world", "sdf_func_normal_world_local",
                 "sdf_func_grad_world_local"]
    sdf = types.SimpleNamespace(**extract_functions(os.path.join(ref, "genesis/utils/sdf.py"), sdf_names, gns))
    rig = extract_functions(os.path.join(ref, "genesis/engine/solvers/rigid/abd/forward_dynamics.py"),
                            ["func_vel_at_point"], gns)
    rig.update(extract_functions(os.path.join(ref, "genesis/engine/solvers/rigid/abd/misc.py"),
                                 ["func_apply_coupling_force"], gns))
    out = dict(gns)
    out["sdf"] = sdf
    out["rigid_funcs"] = rig
    return out
TOOL_GEOM_FUNCS = ["qd_normalize", "qd_transform_by_quat", "qd_inv_quat", "qd_inv_transform_by_quat", "qd_transform_by_T",
                   "qd_inv_transform_by_trans_quat", "qd_transform_by_trans_quat", "qd_rotvec_to_quat", "qd_quat_mul",
                   "qd_transform_quat_by_quat"]


def tool_namespace(ref, ns):
    """Namespace for the tool entity's methods (tool_entity/mesh.py, tool_entity.py): the
    reference's geometry helpers (genesis/utils/geom.py) as `gu` and by name, executed as written."""
    tns = dict(ns)
    extract_functions(os.path.join(ref, "genesis/utils/geom.py"), TOOL_GEOM_FUNCS, tns)
    tns["gu"] = types.SimpleNamespace(**{k: tns[k] for k in TOOL_GEOM_FUNCS})
    return tns


class _AtomicAdd(ast.NodeTransformer):
    """`qd.atomic_add(a[i], v)` adds v to the field element a[i] and returns its old value; as a
    Python call it would receive a copy of a[i], so it becomes `_qd_atomic_add(a, i, v)`."""

    def visit_Call(self, node):
        self.generic_visit(node)
        f = node.func
        if (isinstance(f, ast.Attribute) and f.attr == "atomic_add" and isinstance(f.value, ast.Name)
                and f.value.id == "qd" and node.args and isinstance(node.args[0], ast.Subscript)):
            tgt = node.args[0]
            node.func = ast.Name(id="_qd_atomic_add", ctx=ast.Load())
            node.args = [tgt.value, tgt.slice] + node.args[1:]
            tgt.value.ctx = ast.Load()
        return node


def _qd_atomic_add(a, idx, v):
    old = a[idx]
    a[idx] = old + v
    return old


class _ValueAssign(ast.NodeTransformer):
    """`a = b` between names copies b, as Quadrants assigns vectors and matrices by value (numpy
    would alias them: `inc = pos; inc[i] += d` must leave pos unchanged)."""

    def visit_Assign(self, node):
        if len(node.targets) == 1 and isinstance(node.targets[0], ast.Name) and isinstance(node.value, ast.Name):
            node.value = ast.Call(func=ast.Name(id="_qd_copy", ctx=ast.Load()), args=[node.value], keywords=[])
        return node


def _qd_copy(v):
    return v.copy() if isinstance(v, np.ndarray) else v


def extract(path, cls, names, ns):
    """Compile methods `names` of class `cls` in `path` (decorators/annotations removed) into ns."""
    ns.setdefault("_qd_copy", _qd_copy)
    ns.setdefault("_qd_atomic_add", _qd_atomic_add)
    src = open(path).read()
    tree = ast.parse(src)
    out = {}
    for node in tree.body:
        if isinstance(node, ast.ClassDef) and node.name == cls:
            for fn in node.body:
                if isinstance(fn, ast.FunctionDef) and fn.name in names:
                    fn.decorator_list = []
                    fn.returns = None
                    for a in fn.args.args + fn.args.kwonlyargs:
                        a.annotation = None
                    fn = _AtomicAdd().visit(_ValueAssign().visit(fn))
                    mod = ast.Module(body=[fn], type_ignores=[])
                    code = compile(ast.fix_missing_locations(mod), path, "exec")
                    loc = {}
                    exec(code, ns, loc)
                    out[fn.name] = loc[fn.name]
    missing = set(names) - set(out)
    if missing:
        raise RuntimeError(f"{path}: {cls} lacks {missing}")
    return out


def _by_value(fn):
    """Quadrants passes matrices to qd.func by value: copy array arguments."""

    def w(*a, **k):
        a = [x.copy() if isinstance(x, np.ndarray) else x for x in a]
        k = {n: (x.copy() if isinstance(x, np.ndarray) else x) for n, x in k.items()}
        return fn(*a, **k)

    return w


def bind(obj, funcs):
    for name, f in funcs.items():
        setattr(obj, name, _by_value(types.MethodType(f, obj)))
    return obj


def load_reference(ref):
    ns = {"qd": make_qd(), "gs": make_gs(), "np": np, "math": math}
    mat_dir = os.path.join(ref, "genesis/engine/materials/MPM")
    F = {}
    F["base"] = extract(os.path.join(mat_dir, "base.py"), "Base", ["_update_stress_default"], ns)
    F["elastic"] = extract(os.path.join(mat_dir, "elastic.py"), "Elastic",
                           ["_update_F_S_Jp_elastic", "_update_stress_corotation", "_update_stress_neohooken"], ns)
    F["liquid"] = extract(os.path.join(mat_dir, "liquid.py"), "Liquid",
                          ["_update_F_S_Jp_liquid", "_update_stress_liquid"], ns)
    F["sand"] = extract(os.path.join(mat_dir, "sand.py"), "Sand",
                        ["_sand_projection", "_update_F_S_Jp_sand", "_update_stress_sand"], ns)
    F["snow"] = extract(os.path.join(mat_dir, "snow.py"), "Snow", ["_update_F_S_Jp_snow", "_update_stress_snow"], ns)
    F["ep"] = extract(os.path.join(mat_dir, "elasto_plastic.py"), "ElastoPlastic", ["_update_F_S_Jp_elasto_plastic"], ns)
    F["muscle"] = extract(os.path.join(mat_dir, "muscle.py"), "Muscle", ["_update_stress_with_actuation"], ns)
    F["solver"] = extract(os.path.join(ref, "genesis/engine/solvers/mpm_solver.py"), "MPMSolver",
                          ["stencil_range", "compute_F_tmp", "svd", "p2g", "g2p"], ns)
    F["coupler"] = extract(os.path.join(ref, "genesis/engine/couplers/legacy_coupler.py"), "LegacyCoupler",
                           ["mpm_grid_op"], ns)
    rns = rigid_namespace(ref, ns)
    F["coupler_rigid"] = extract(os.path.join(ref, "genesis/engine/couplers/legacy_coupler.py"), "LegacyCoupler",
                                 ["_func_collide_with_rigid", "_func_collide_with_rigid_geom",
                                  "_func_collide_in_rigid_geom"], rns)
    F["rigid_funcs"] = rns["rigid_funcs"]
    F["solver_cpic"] = extract(os.path.join(ref, "genesis/engine/solvers/mpm_solver.py"), "MPMSolver", ["p2g", "g2p"],
                               rns)
    F["coupler_cpic"] = extract(os.path.join(ref, "genesis/engine/couplers/legacy_coupler.py"), "LegacyCoupler",
                                ["mpm_surface_to_particle"], rns)
    F["boundary"] = extract(os.path.join(ref, "genesis/engine/boundaries/boundaries.py"), "CubeBoundary",
                            ["impose_pos_vel"], ns)
    tns = tool_namespace(ref, ns)
    tdir = os.path.join(ref, "genesis/engine/entities/tool_entity")
    F["tool_mesh"] = extract(os.path.join(tdir, "mesh.py"), "Mesh",
                             ["sdf", "sdf_", "normal", "normal_", "vel_collider", "collide"], tns)
    F["tool_entity"] = extract(os.path.join(tdir, "tool_entity.py"), "ToolEntity", ["collide", "advect", "copy_frame"],
                               tns)
    F["floor"] = extract(os.path.join(ref, "genesis/engine/boundaries/boundaries.py"), "FloorBoundary", ["impose_pos"],
                         ns)
    F["hasher"] = extract(os.path.join(ref, "genesis/utils/geom.py"), "SpatialHasher",
                          ["compute_reordered_idx", "pos_to_grid", "grid_to_slot", "pos_to_slot"], ns)
    F["constraints"] = extract(os.path.join(ref, "genesis/engine/solvers/mpm_solver.py"), "MPMSolver",
                               ["_kernel_set_particle_constraints", "_kernel_remove_particle_constraints",
                                "apply_particle_constraints"], tns)
    F["coupler_tool"] = extract(os.path.join(ref, "genesis/engine/couplers/legacy_coupler.py"), "LegacyCoupler",
                                ["_func_mpm_tool"], ns)
    return F


# ----------------------------------------------------------------------------- materials
# (name, derived parameters as computed by the reference's model_post_init, selected functions)
def material_variants():
    def lame(E, nu):
        return E / (2.0 * (1.0 + nu)), E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    out = []
    mu, lam = lame(3e5, 0.2)
    out.append(("elastic", dict(type=0, flags=0, mu=mu, lam=lam)))
    out.append(("elastic_neohookean", dict(type=0, flags=1, mu=mu, lam=lam)))
    mu, lam = lame(1e5, 0.3)
    out.append(("liquid", dict(type=1, flags=0, mu=0.0, lam=lam)))
    out.append(("liquid_viscous", dict(type=1, flags=0, mu=mu, lam=lam)))
    mu, lam = lame(1e6, 0.2)
    s = math.sin(math.radians(45.0))
    out.append(("sand", dict(type=2, flags=0, mu=mu, lam=lam, alpha=math.sqrt(2 / 3) * 2 * s / (3 - s))))
    out.append(("snow", dict(type=3, flags=0, mu=mu, lam=lam, yield_lower=2.5e-2, yield_higher=4.5e-3)))
    out.append(("elastoplastic_vm", dict(type=4, flags=2, mu=mu, lam=lam, yield_lower=2.5e-2, yield_higher=4.5e-3,
                                          vm_yield=1e4)))
    out.append(("elastoplastic_clamp", dict(type=4, flags=0, mu=mu, lam=lam, yield_lower=2.5e-2,
                                             yield_higher=4.5e-3, vm_yield=1e4)))
    out.append(("muscle", dict(type=5, flags=1, mu=mu, lam=lam, stiffness=1e6)))
    return out


def material_callables(F, p):
    """(update_F_S_Jp, update_stress) of the reference bound to a parameter object."""
    self = types.SimpleNamespace(mu=p["mu"], lam=p["lam"], alpha=p.get("alpha", 0.0),
                                 yield_lower=p.get("yield_lower", 0.0), yield_higher=p.get("yield_higher", 0.0),
                                 use_von_mises=bool(p["flags"] & 2), von_mises_yield_stress=p.get("vm_yield", 0.0),
                                 stiffness=p.get("stiffness", 0.0))
    t = p["type"]
    bind(self, F["base"])
    if t == 0 or t == 5:
        bind(self, F["elastic"])
        upd = self._update_F_S_Jp_elastic
        stress = self._update_stress_neohooken if p["flags"] & 1 else self._update_stress_corotation
        if t == 5:
            self._update_stress_without_actuation = stress
            bind(self, F["muscle"])
            stress = self._update_stress_with_actuation
        return upd, stress
    if t == 1:
        bind(self, F["liquid"])
        return self._update_F_S_Jp_liquid, self._update_stress_liquid
    if t == 2:
        bind(self, F["sand"])
        return self._update_F_S_Jp_sand, self._update_stress_sand
    if t == 3:
        bind(self, F["snow"])
        return self._update_F_S_Jp_snow, self._update_stress_snow
    bind(self, F["ep"])
    return self._update_F_S_Jp_elasto_plastic, self._update_stress_default


def gen_materials(F, rng):
    rec = {}
    for name, p in material_variants():
        upd, stress = material_callables(F, p)
        n = 60
        Fts, Jps, actus, mdirs, Fns, Jpns, Ps = [], [], [], [], [], [], []
        for i in range(n):
            amp = [1e-3, 3e-2, 0.15][i % 3]
            Ft = np.eye(3) + amp * rng.normal(size=(3, 3))
            Jp = rng.uniform(-0.05, 0.05) if p["type"] == 2 else rng.uniform(0.9, 1.1)
            actu = rng.uniform(0, 1)
            md = rng.normal(size=3)
            md /= np.linalg.norm(md)
            U, S, V = _svd(Ft)
            J = S.determinant()
            Fn, Sn, Jpn = upd(J=J, F_tmp=QMat(Ft), U=U, S=S, V=V, Jp=Jp)
            P = stress(U=U, S=Sn, V=V, F_tmp=QMat(Ft), F_new=Fn, J=J, Jp=Jp, actu=actu, m_dir=QMat(md))
            Fts.append(Ft), Jps.append(Jp), actus.append(actu), mdirs.append(md)
            Fns.append(np.asarray(Fn)), Jpns.append(float(Jpn)), Ps.append(np.asarray(P))
        for k, v in dict(F_tmp=Fts, Jp=Jps, actu=actus, mdir=mdirs, F_new=Fns, Jp_new=Jpns, stress=Ps).items():
            rec[f"{name}/{k}"] = np.asarray(v)
        rec[f"{name}/params"] = np.array([p["type"], p["flags"], p["mu"], p["lam"], p.get("alpha", 0.0),
                                          p.get("yield_lower", 0.0), p.get("yield_higher", 0.0), p.get("vm_yield", 0.0),
                                          p.get("stiffness", 0.0)])
    return rec


# ----------------------------------------------------------------------------- one scene, full substeps
def gen_substeps(F, rng, ffs=(), n_steps=10, rigid=None, tool=None, cpic=False, coupled=None, constraints=None):
    """A 9-material scene on a 17^3 grid advanced by the reference's substep code; `ffs` are
    reference force-field objects applied in its grid op (legacy_coupler.py:376-378); `rigid`
    (make_rigid_standins) couples the grid op with rigid geoms (legacy_coupler.py:389-403); `tool`
    (make_tool_standin) with a tool entity (legacy_coupler.py:385-387), which advects before the
    grid op (ToolSolver.substep_pre_coupling) and copies its frame f+1 to f after the substep;
    `cpic` (with `rigid`) turns on MPMOptions.enable_CPIC: the coupler's preprocess
    (mpm_surface_to_particle) before P2G and the separated-cell branches of p2g and g2p;
    `coupled` (make_coupled_standin, keys "sph" / "pbd") couples the grid op with another solver's
    particles through its spatial hash (legacy_coupler.py:404-498); `constraints`
    (CONSTRAINT_SETS) attaches particles to kinematic links before the first substep
    (_kernel_set_particle_constraints), moves the links before every substep, removes some
    constraints before one of them (_kernel_remove_particle_constraints) and applies the springs
    after every G2P (apply_particle_constraints, mpm_solver.py:538-540)."""
    # domain [0, 0.25]^3 at density 64 -> 17^3 nodes, boundary [3/64, 0.25 - 3/64]
    density, dt = 64.0, 2e-4
    lower, upper = np.zeros(3), np.full(3, 0.25)
    p_size = 1.0 / 128.0
    dx = 1.0 / density
    variants = material_variants()
    centers = [(0.08, 0.08, 0.09), (0.17, 0.08, 0.09), (0.08, 0.17, 0.09), (0.17, 0.17, 0.09),
               (0.08, 0.125, 0.17), (0.17, 0.125, 0.17), (0.125, 0.08, 0.17), (0.125, 0.17, 0.17),
               (0.125, 0.125, 0.12)]
    pos, mat = [], []
    for m, c in enumerate(centers):
        ax = (np.arange(4) - 1.5) * p_size
        lat = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3) + np.asarray(c)
        pos.append(lat + rng.uniform(-0.25 * dx, 0.25 * dx, size=lat.shape))
        mat.append(np.full(len(lat), m))
    pos = np.concatenate(pos)
    mat = np.concatenate(mat).astype(np.int64)
    n = len(pos)
    vel = rng.normal(scale=0.05, size=(n, 3))
    C = rng.normal(scale=0.5, size=(n, 3, 3))
    Fm = np.eye(3) + rng.normal(scale=0.02, size=(n, 3, 3))
    Jp = np.array([rng.uniform(-0.02, 0.01) if variants[m][1]["type"] == 2 else rng.uniform(0.97, 1.03) for m in mat])
    actu = rng.uniform(0, 1, size=n)
    mdir = rng.normal(size=(n, 3))
    mdir /= np.linalg.norm(mdir, axis=1, keepdims=True)
    rho = 1000.0

    p_vol = p_size**3 * 1e3
    grid_res = tuple(int(v) for v in (np.round(density * upper) - np.round(density * lower) + 1))
    solver = types.SimpleNamespace()
    solver._n_particles, solver._B = n, 1
    solver.substep_dt = dt
    solver._particle_volume, solver._particle_volume_scale = p_vol, 1e3
    solver._inv_dx, solver._dx = density, dx
    solver.dx = dx
    solver._grid_offset = QMat(np.round(density * lower).astype(np.int64), dtype=np.int64)
    solver.grid_offset = solver._grid_offset
    solver.grid_res = grid_res
    solver._enable_CPIC = False
    solver.sim = types.SimpleNamespace(rigid_solver=types.SimpleNamespace(is_active=False))
    solver._gravity = QMat(np.array([[0.0, 0.0, -9.81]]))
    solver._ffs = list(ffs)
    bnd = types.SimpleNamespace(upper_qd=QMat(upper - 3 * dx), lower_qd=QMat(lower + 3 * dx), restitution=0.0)
    bind(bnd, F["boundary"])
    solver.boundary = bnd
    solver.particles = StructField((2, n, 1), dict(pos=(3,), vel=(3,), C=(3, 3), F=(3, 3), F_tmp=(3, 3), U=(3, 3),
                                                   V=(3, 3), S=(3, 3), actu=(), Jp=()))
    solver.particles_ng = StructField((2, n, 1), dict(active=()))
    solver.particles_info = StructField((n,), dict(material_idx=(), mass=(), default_Jp=(), free=(),
                                                   muscle_group=(), muscle_direction=(3,)))
    solver.grid = StructField((2,) + grid_res + (1,), dict(mass=(), vel_in=(3,), vel_out=(3,)))
    fns = [material_callables(F, p) for _, p in variants]
    solver._materials_idx = list(range(len(variants)))
    solver._materials_update_F_S_Jp = [f[0] for f in fns]
    solver._materials_update_stress = [f[1] for f in fns]
    bind(solver, F["solver"])
    coupler = types.SimpleNamespace(mpm_solver=solver, tool_solver=types.SimpleNamespace(is_active=False),
                                    _rigid_mpm=False, _mpm_sph=False, _mpm_pbd=False)
    bind(coupler, F["coupler"])
    grid_op_args = (None, None, None, None, None, None)
    if rigid is not None:
        coupler._rigid_mpm = True
        coupler.rigid_solver = rigid["rigid_solver"]
        bind(coupler, F["coupler_rigid"])
        grid_op_args = tuple(rigid[k] for k in ("geoms_state", "geoms_info", "links_state", "rigid_global_info",
                                                "sdf_info", "collider_static_config"))
    for kind, other in (coupled or {}).items():  # stencil sizes as LegacyCoupler.build computes them
        setattr(coupler, f"_mpm_{kind}", True)
        setattr(coupler, f"{kind}_solver", other)
        setattr(coupler, f"mpm_{kind}_stencil_size", int(np.floor(dx / other.sh.cell_size) + 2))
    if constraints is not None:
        solver.particle_constraints = StructField((n, 1), dict(is_constrained=(), target_pos=(3,), stiffness=(),
                                                                link_idx=(), link_local_pos=(3,)))
        solver.particle_constraints._d["is_constrained"] = np.zeros((n, 1), np.int64)
        solver.particle_constraints._d["link_idx"] = np.full((n, 1), -1, np.int64)
        bind(solver, F["constraints"])
        links = types.SimpleNamespace(pos=constraints["link_pos"][0].copy().view(QMat),
                                      quat=constraints["link_quat"][0].copy().view(QMat))
    if cpic:
        G = rigid["rigid_solver"].n_geoms
        solver._enable_CPIC = True
        solver.n_particles = n
        solver.sim = types.SimpleNamespace(rigid_solver=rigid["rigid_solver"], coupler=coupler)
        solver._coupler = coupler
        bind(solver, F["solver_cpic"])
        coupler.cpic_flag = np.zeros((n, 3, 3, 3, 1), np.int64)
        coupler.mpm_rigid_normal = np.zeros((n, G, 1, 3)).view(QMat)
        bind(coupler, F["coupler_cpic"])
    if tool is not None:
        coupler.tool_solver = tool["tool_solver"]
        bind(coupler, F["coupler_tool"])

    P, I, G = solver.particles._d, solver.particles_info._d, solver.grid._d
    P["pos"][0, :, 0], P["vel"][0, :, 0], P["C"][0, :, 0], P["F"][0, :, 0] = pos, vel, C, Fm
    P["Jp"][0, :, 0], P["actu"][0, :, 0] = Jp, actu
    solver.particles_ng._d["active"][0, :, 0] = 1
    I["material_idx"][:], I["mass"][:], I["free"][:], I["muscle_direction"][:] = mat, p_vol * rho, 1, mdir

    def snapshot():
        return {k: P[k][0, :, 0].copy() for k in ("pos", "vel", "C", "F", "Jp")}

    if constraints is not None:  # attached to the initial state
        for start, mask, stiffness, link in constraints["sets"]:
            lk = max(link, 0)
            solver._kernel_set_particle_constraints(0, mask, start, stiffness, link, links.pos[lk], links.quat[lk])

    out = {"in/" + k: v for k, v in snapshot().items()}
    out.update({"in/mat": mat, "in/actu": actu, "in/mdir": mdir})
    for step in range(n_steps):
        for k in G:
            G[k][...] = 0  # reset_grid_and_grad
        if constraints is not None:
            links.pos[...], links.quat[...] = constraints["link_pos"][step + 1], constraints["link_quat"][step + 1]
            if step == constraints["remove_before"]:
                start, mask = constraints["remove"]
                solver._kernel_remove_particle_constraints(mask, start)
        if cpic:  # LegacyCoupler.preprocess
            coupler.mpm_surface_to_particle(0, rigid["geoms_state"], rigid["geoms_info"], rigid["sdf_info"],
                                            rigid["rigid_global_info"], rigid["collider_static_config"])
        solver.compute_F_tmp(0)
        solver.svd(0)
        if cpic:
            solver.p2g(0, rigid["geoms_state"], rigid["geoms_info"], rigid["links_state"], rigid["rigid_global_info"],
                       rigid["sdf_info"], rigid["collider_static_config"])
        else:
            solver.p2g(0, None, None, None, None, None, None)
        if tool is not None:
            tool["entity"].advect(0)
        if step == 0:
            out["grid1"] = np.concatenate([G["vel_in"][0, ..., 0, :], G["mass"][0, ..., 0, None]], -1).copy()
        coupler.mpm_grid_op(0, step * dt, *grid_op_args)  # t = Simulator.cur_t of the substep
        if cpic:
            solver.g2p(0, rigid["geoms_info"], rigid["links_state"], rigid["rigid_global_info"])
        else:
            solver.g2p(0, None, None, None)
        if constraints is not None:
            solver.apply_particle_constraints(0, links)
        for k in ("pos", "vel", "C", "F", "Jp"):  # copy_frame(1 -> 0)
            P[k][0] = P[k][1]
        if tool is not None:
            tool["entity"].copy_frame(1, 0)
        if step == 0:
            out.update({"out1/" + k: v for k, v in snapshot().items()})
    out.update({f"out{n_steps}/" + k: v for k, v in snapshot().items()})
    out["scene"] = np.array([dt, density, p_size, *lower, *upper, EPS32])
    out["material_params"] = np.array([[p["type"], p["flags"], p["mu"], p["lam"], p.get("alpha", 0.0),
                                        p.get("yield_lower", 0.0), p.get("yield_higher", 0.0), p.get("vm_yield", 0.0),
                                        p.get("stiffness", 0.0), rho] for _, p in variants])
    return out


# ----------------------------------------------------------------------------- force fields
class _FieldStandin:
    """qd.field stand-in: scalar (shape ()) or 1-D integer field."""

    def __init__(self, dtype, shape=()):
        self.a = np.zeros(shape if shape != () else (1,), dtype=np.int64 if dtype in (np.int64, bool) else np.float64)

    def __getitem__(self, i):
        return self.a[0 if i is None else int(i)]

    def __setitem__(self, i, v):
        self.a[0 if i is None else int(i)] = v

    def from_numpy(self, arr):
        self.a[:] = arr


def load_force_fields(ref):
    """Execute genesis/engine/force_fields.py as written, against the stand-ins (the Quadrants
    decorators are identities, fields are numpy arrays)."""
    qd = make_qd()
    qd.func = qd.kernel = qd.data_oriented = lambda f: f
    qd.field = lambda dtype, shape=(): _FieldStandin(dtype, shape)
    gs = make_gs()
    gs.qd_bool = bool
    repr_base = types.ModuleType("genesis.repr_base")
    repr_base.RBC = object
    saved = {k: sys.modules.get(k) for k in ("quadrants", "genesis", "genesis.repr_base")}
    sys.modules.update({"quadrants": qd, "genesis": gs, "genesis.repr_base": repr_base})
    try:
        mod = types.ModuleType("reference_force_fields")
        path = os.path.join(ref, "genesis/engine/force_fields.py")
        exec(compile(open(path).read(), path, "exec"), mod.__dict__)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


# (class, keyword arguments) of the deterministic fields pinned here (Noise draws qd.random)
FORCE_FIELDS = [
    ("Constant", dict(direction=(1.0, 0.5, 0.0), strength=2.0)),
    ("Wind", dict(direction=(0.0, 1.0, 0.2), strength=3.0, radius=0.05, center=(0.1, 0.12, 0.1))),
    ("Point", dict(strength=-1.5, position=(0.125, 0.125, 0.2), falloff_pow=1.5, flow=0.3)),
    ("Drag", dict(linear=0.8, quadratic=0.4)),
    ("Vortex", dict(direction=(0.0, 0.0, 1.0), center=(0.12, 0.13, 0.0), strength_perpendicular=4.0,
                    strength_radial=1.0, falloff_pow=2.0, falloff_min=0.02, falloff_max=0.2, damping=0.5)),
    ("Turbulence", dict(strength=2.0, frequency=7, flow=0.2, seed=5)),
]


def gen_force_fields(F, ref, rng):
    FF = load_force_fields(ref)
    fields = []
    for name, kw in FORCE_FIELDS:
        f = getattr(FF, name)(**kw)
        f.activate()
        fields.append(f)
    out = gen_substeps(F, rng, ffs=fields, n_steps=5)
    out["fields"] = np.array([name for name, _ in FORCE_FIELDS])
    for i, (name, kw) in enumerate(FORCE_FIELDS):
        for k, v in kw.items():
            out[f"field{i}/{k}"] = np.asarray(v, dtype=np.float64)
    return out


# ----------------------------------------------------------------------------- rigid coupling
def _quat_about(axis, deg):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    h = math.radians(deg) / 2
    return np.array([math.cos(h), *(math.sin(h) * a)])


def box_sdf(p, half):
    q = np.abs(p) - half
    out = np.linalg.norm(np.maximum(q, 0), axis=-1)
    return out + np.minimum(q.max(-1), 0)


# geoms of the coupled scene: (type, pos, quat, data, link cd_vel, cd_ang, friction, softness, restitution)
RIGID_GEOMS = [
    ("sphere", (0.125, 0.125, 0.05), _quat_about((0, 0, 1), 0.0), (0.03,), (0.1, 0.0, 0.2), (0.0, 0.0, 1.0),
     0.3, 0.002, 0.1),
    ("plane", (0.125, 0.125, 0.07), _quat_about((1, 0, 0), 15.0), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0),
     0.5, 0.004, 0.0),
    ("box", (0.17, 0.1, 0.1), _quat_about((0, 0, 1), 20.0), (0.03, 0.02, 0.025), (0.0, -0.1, 0.0), (0.5, 0.0, 0.0),
     0.2, 0.002, 0.2),
]
# the CPIC scene swaps the box for a thin tilted plate (an ellipsoid SDF, smooth gradients): the
# box's face normals are exactly perpendicular across its edges, so CPIC's side test
# (normal . normal < 0) would compare rounding noise against zero there
CPIC_GEOMS = RIGID_GEOMS[:2] + [
    ("plate", (0.125, 0.125, 0.12), _quat_about((0, 1, 0), 10.0), (0.035, 0.035, 0.005), (0.0, 0.05, -0.1),
     (0.0, 0.0, 0.3), 0.2, 0.002, 0.1),
]
BOX_GRID = dict(res=24, lower=-0.05, upper=0.05)


def plate_sdf(p, half):
    """Scaled ellipsoid distance (|p / half| - 1) * min(half): zero on the ellipsoid, smooth."""
    half = np.asarray(half)
    return (np.linalg.norm(p / half, axis=-1) - 1.0) * half.min()


def box_grid(half, fn=box_sdf):
    """The SDF geom's grid as the rigid solver stores it (values and mesh-frame gradients on a
    res^3 lattice, T_mesh_to_sdf mapping mesh coordinates to voxel indices), in float32."""
    res, lo, hi = BOX_GRID["res"], BOX_GRID["lower"], BOX_GRID["upper"]
    h = (hi - lo) / (res - 1)
    ax = lo + h * np.arange(res)
    pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    val = fn(pts, np.asarray(half))
    eps = 1e-6
    grad = np.stack([(fn(pts + eps * e, half) - fn(pts - eps * e, half)) / (2 * eps) for e in np.eye(3)], -1)
    grad /= np.maximum(np.linalg.norm(grad, axis=-1, keepdims=True), 1e-12)
    T = np.eye(4)
    T[:3, :3] /= h
    T[:3, 3] = -lo / h
    return (val.astype(np.float32).reshape(res, res, res), grad.astype(np.float32).reshape(res, res, res, 3), T, h,
            float(val.astype(np.float32).max()))


def geom_grid(geom):
    """The grid of the SDF geom (a "box" or a "plate") of a geom list."""
    return box_grid(geom[3], box_sdf if geom[0] == "box" else plate_sdf)


def make_rigid_standins(F, dt, geoms=RIGID_GEOMS):
    """The rigid solver's data the coupler reads, for `geoms` (one env, one link per geom; the
    last geom is the one given by an SDF grid)."""
    G = len(geoms)
    types_ = {"sphere": GEOM_TYPE.SPHERE, "plane": GEOM_TYPE.PLANE, "box": GEOM_TYPE.BOX, "plate": GEOM_TYPE.MESH}
    data = np.zeros((G, 7))
    gpos = np.zeros((G, 1, 3)).view(QMat)
    gquat = np.zeros((G, 1, 4)).view(QMat)
    cd_vel = np.zeros((G, 1, 3)).view(QMat)
    cd_ang = np.zeros((G, 1, 3)).view(QMat)
    com = np.zeros((G, 1, 3)).view(QMat)
    for i, (t, pos, quat, d, v, w, *_rest) in enumerate(geoms):
        data[i, : len(d)] = d
        gpos[i, 0], gquat[i, 0], cd_vel[i, 0], cd_ang[i, 0], com[i, 0] = pos, quat, v, w, pos
    geoms_info = types.SimpleNamespace(
        needs_coup=[1] * G, type=[types_[g[0]] for g in geoms], data=[QMat(r) for r in data],
        coup_friction=[g[6] for g in geoms], coup_softness=[g[7] for g in geoms],
        coup_restitution=[g[8] for g in geoms], link_idx=list(range(G)))
    geoms_state = types.SimpleNamespace(pos=gpos, quat=gquat)
    links_state = types.SimpleNamespace(cd_vel=cd_vel, cd_ang=cd_ang, root_COM=com,
                                        cfrc_coupling_vel=np.zeros((G, 1, 3)).view(QMat),
                                        cfrc_coupling_ang=np.zeros((G, 1, 3)).view(QMat))
    rgi = types.SimpleNamespace(substep_dt=_FieldStandin(np.float64), EPS=_FieldStandin(np.float64))
    rgi.substep_dt[None] = dt
    rgi.EPS[None] = EPS32
    val, grad, T, h, smax = geom_grid(geoms[2])
    res = QMat(np.array(val.shape), dtype=np.int64)
    zero_T = np.eye(4)
    sdf_geoms = types.SimpleNamespace(T_mesh_to_sdf=[QMat(zero_T), QMat(zero_T), QMat(T)], sdf_res=[res, res, res],
                                      sdf_cell_size=[h, h, h], sdf_max=[smax] * 3, sdf_cell_start=[0, 0, 0])
    sdf_info = types.SimpleNamespace(geoms_info=sdf_geoms, geoms_sdf_val=val.astype(np.float64).reshape(-1),
                                     geoms_sdf_grad=grad.astype(np.float64).reshape(-1, 3).view(QMat))
    fns = F["rigid_funcs"]
    rigid_solver = types.SimpleNamespace(
        n_geoms=G, is_active=True,
        _func_vel_at_point=lambda pos_world, link_idx, i_b, links_state: fns["func_vel_at_point"](
            pos_world, link_idx, i_b, links_state),
        _func_apply_coupling_force=lambda pos, force, link_idx, env_idx, links_state: fns["func_apply_coupling_force"](
            pos, force, link_idx, env_idx, links_state))
    return dict(geoms_state=geoms_state, geoms_info=geoms_info, links_state=links_state, rigid_global_info=rgi,
                sdf_info=sdf_info, collider_static_config=types.SimpleNamespace(has_terrain=False),
                rigid_solver=rigid_solver)


def gen_rigid(F, rng, cpic=False):
    geoms = CPIC_GEOMS if cpic else RIGID_GEOMS
    rigid = make_rigid_standins(F, 2e-4, geoms)
    out = gen_substeps(F, rng, n_steps=3, rigid=rigid, cpic=cpic)
    ls = rigid["links_state"]
    out["link_force"] = np.asarray(ls.cfrc_coupling_vel)[:, 0].copy()
    out["link_torque"] = np.asarray(ls.cfrc_coupling_ang)[:, 0].copy()
    out["geom_types"] = np.array([g[0] for g in geoms])
    for i, g in enumerate(geoms):
        out[f"geom{i}/pos"], out[f"geom{i}/quat"], out[f"geom{i}/data"] = np.array(g[1]), np.array(g[2]), np.array(g[3])
        out[f"geom{i}/lin_vel"], out[f"geom{i}/ang_vel"] = np.array(g[4]), np.array(g[5])
        out[f"geom{i}/coup"] = np.array(g[6:9])
    val, grad, T, h, smax = geom_grid(geoms[2])
    out["sdf_grid/values"], out["sdf_grid/grads"], out["sdf_grid/T"] = val, grad, T
    out["sdf_grid/cell_size"], out["sdf_grid/sdf_max"] = np.array(h), np.array(smax)
    return out


# ----------------------------------------------------------------------------- tool coupling
# a rotated box tool (values-only SDF grid) translating down onto its floor height and spinning
TOOL = dict(pos=(0.11, 0.12, 0.1203), quat=_quat_about((1, 1, 0), 25.0), vel=(0.2, -0.1, -0.5), ang=(0.0, 1.0, 2.0),
            half=(0.03, 0.02, 0.025), friction=0.3, coup_softness=0.002, floor_height=0.12015)


class _VoxelField:
    """qd.field stand-in indexed by an integer vector (Mesh.sdf_voxels[voxel_pos])."""

    def __init__(self, a):
        self.a = a

    def __getitem__(self, idx):
        return float(self.a[_flat_index(idx)])


class _ScalarMatrixField:
    """0-d qd.Matrix.field stand-in (Mesh.T_mesh_to_sdf[None])."""

    def __init__(self, m):
        self.m = QMat(m)

    def __getitem__(self, idx):
        return self.m.copy().view(QMat)


def make_tool_standin(F, dt):
    """One tool entity (ToolEntity with its Mesh, one env, frames 0 and 1) on the tool solver's
    FloorBoundary, for TOOL."""
    val = box_grid(TOOL["half"])[0]
    T = box_grid(TOOL["half"])[2]
    ent = types.SimpleNamespace()
    for k, v in (("pos", TOOL["pos"]), ("quat", TOOL["quat"]), ("vel", TOOL["vel"]), ("ang", TOOL["ang"])):
        a = np.zeros((2, 1, len(v))).view(QMat)
        a[0, 0] = v
        setattr(ent, k, a)
    floor = types.SimpleNamespace(height=TOOL["floor_height"])
    bind(floor, F["floor"])
    ent._sim = types.SimpleNamespace(_B=1)
    ent._solver = ent.solver = types.SimpleNamespace(boundary=floor, substep_dt=dt)
    ent.material = types.SimpleNamespace(collision=True, coup_softness=TOOL["coup_softness"])
    mesh = types.SimpleNamespace(entity=ent, material=ent.material, collision=True, friction=TOOL["friction"],
                                 sdf_res=val.shape[0], sdf_voxels=_VoxelField(val.astype(np.float64)),
                                 T_mesh_to_sdf=_ScalarMatrixField(T))
    bind(mesh, F["tool_mesh"])
    ent.mesh = mesh
    bind(ent, F["tool_entity"])
    return dict(entity=ent, tool_solver=types.SimpleNamespace(is_active=True, entities=[ent]))


def gen_tool(F, rng, n_steps=4):
    tool = make_tool_standin(F, 2e-4)
    out = gen_substeps(F, rng, n_steps=n_steps, tool=tool)
    ent = tool["entity"]
    out["n_steps"] = np.array(n_steps)
    out["tool/pos_out"], out["tool/quat_out"] = np.asarray(ent.pos[0, 0]).copy(), np.asarray(ent.quat[0, 0]).copy()
    for k in ("pos", "quat", "vel", "ang"):
        out[f"tool/{k}"] = np.asarray(TOOL[k], np.float64)
    for k in ("friction", "coup_softness", "floor_height"):
        out[f"tool/{k}"] = np.array(TOOL[k])
    val, _, T, h, smax = box_grid(TOOL["half"])
    out["tool_sdf/values"], out["tool_sdf/T"] = val, T
    out["tool_sdf/cell_size"], out["tool_sdf/sdf_max"] = np.array(h), np.array(smax)
    return out


# ----------------------------------------------------------------------------- SPH / PBD coupling
class _SoAField(StructField):
    """A struct field read both ways the coupler reads the other solvers' particles:
    `f.pos[i, b]` (member array) and `f[i, b].vel = ...` (write-through record)."""

    def __getattr__(self, k):
        return self._d[k].view(QMat)


# (kind, block centre the set is spread around, hash cell size, hash grid resolution, mass)
COUPLED_SETS = [("sph", (0.08, 0.125, 0.17), 0.01, (26, 26, 26), 4e-3),
                ("pbd", (0.17, 0.125, 0.17), 0.02, (13, 13, 13), 6e-3)]


def make_coupled_standin(F, rng, centre, cell_size, grid_res, mass, n=60):
    """Another solver's particles as the coupler sees them: reordered by the reference's own
    SpatialHasher (genesis/utils/geom.py) into its slots, with the slot tables it builds."""
    pos = np.asarray(centre) + rng.uniform(-0.012, 0.012, size=(n, 3))
    vel = rng.normal(scale=0.1, size=(n, 3))
    m = np.full(n, mass) * rng.uniform(0.8, 1.2, size=n)
    free = (rng.uniform(size=n) < 0.8).astype(np.int64)
    sh = types.SimpleNamespace(cell_size=cell_size, grid_res=grid_res, n_slots=int(np.prod(grid_res)), _B=1)
    sh.slot_size = np.zeros((sh.n_slots, 1), np.int64)
    sh.slot_start = np.zeros((sh.n_slots, 1), np.int64)
    sh.cur_cnt = np.zeros(1, np.int64)
    bind(sh, F["hasher"])
    order = np.zeros((n, 1), np.int64)
    # its arguments are fields (passed by reference), so the method is called unwrapped
    types.MethodType(F["hasher"]["compute_reordered_idx"], sh)(n, pos[:, None].view(QMat), np.ones((n, 1), np.int64),
                                                              order)
    order = order[:, 0]
    P = _SoAField((n, 1), dict(pos=(3,), vel=(3,), free=()))
    I = _SoAField((n, 1), dict(mass=()))
    P._d["pos"][order, 0], P._d["vel"][order, 0], P._d["free"][order, 0], I._d["mass"][order, 0] = pos, vel, free, m
    other = types.SimpleNamespace(sh=sh, particles_reordered=P, particles_info_reordered=I)
    return other, dict(pos=pos, vel=vel, mass=m, free=free, order=order)


def gen_coupled(F, rng, n_steps=4):
    coupled, sets = {}, {}
    for kind, centre, cell, res, mass in COUPLED_SETS:
        coupled[kind], sets[kind] = make_coupled_standin(F, rng, centre, cell, res, mass)
    out = gen_substeps(F, rng, n_steps=n_steps, coupled=coupled)
    out["n_steps"] = np.array(n_steps)
    for kind, st in sets.items():
        for k in ("pos", "vel", "mass", "free"):
            out[f"{kind}/{k}"] = st[k]
        out[f"{kind}/vel_out"] = coupled[kind].particles_reordered._d["vel"][st["order"], 0].copy()
    return out


# ----------------------------------------------------------------------------- particle constraints
# (first particle, particle count) of the two constrained blocks; (stiffness, link) of each set
CONSTRAINT_SETS = [((192, 64), 300.0, 0), ((384, 64), 600.0, 1), ((448, 64), 150.0, -1)]


def gen_constraints(F, rng, n_steps=5):
    """Particles of three blocks attached to two moving links and (link -1) to their own start
    positions, every other particle of each block; half of the first set released before the
    fourth substep."""
    L = 2
    link_pos = np.zeros((n_steps + 1, L, 1, 3))
    link_quat = np.zeros((n_steps + 1, L, 1, 4))
    for k in range(n_steps + 1):
        link_pos[k, 0, 0] = (0.125 + 0.001 * k, 0.1, 0.1 - 0.0005 * k)
        link_pos[k, 1, 0] = (0.1, 0.15, 0.15 + 0.0008 * k)
        link_quat[k, 0, 0] = _quat_about((0, 0, 1), 5.0 + 2.0 * k)
        link_quat[k, 1, 0] = _quat_about((1, 0.5, 0), -3.0 * k)
    sets = []
    for (start, count), stiffness, link in CONSTRAINT_SETS:
        mask = np.zeros((1, count), np.int64)
        mask[0, ::2] = 1
        sets.append((start, mask, stiffness, link))
    rm = np.zeros((1, 64), np.int64)
    rm[0, :32] = 1
    cons = dict(link_pos=link_pos, link_quat=link_quat, sets=sets, remove_before=3, remove=(192, rm))
    out = gen_substeps(F, rng, n_steps=n_steps, constraints=cons)
    out["n_steps"] = np.array(n_steps)
    out["link_pos"], out["link_quat"] = link_pos[:, :, 0], link_quat[:, :, 0]
    for i, (start, mask, stiffness, link) in enumerate(sets):
        out[f"set{i}/start"], out[f"set{i}/mask"] = np.array(start), mask[0]
        out[f"set{i}/stiffness"], out[f"set{i}/link"] = np.array(stiffness), np.array(link)
    out["remove/start"], out["remove/mask"], out["remove/before"] = np.array(192), rm[0], np.array(3)
    return out


# ----------------------------------------------------------------------------- Custom force field
def custom_acc(pos, vel, t, i):
    """The user function of the Custom-field fixture (one node, as the reference calls it): a swirl
    about the vertical axis through (0.125, 0.125), drag on the horizontal velocity, a time ramp and
    a height-dependent lift.  tests/test_gpu_golden.py evaluates the same formula batched in torch."""
    return QMat([-3.0 * (pos[1] - 0.125) - 0.5 * vel[0] + 2.0 * t,
                 3.0 * (pos[0] - 0.125) - 0.5 * vel[1],
                 -1.0 + 0.3 * pos[2] * (1.0 + t)])


def gen_custom_field(F, ref, rng, n_steps=5):
    """A Custom field (force_fields.py:424) between two built-in ones, Drag before it (it sees the
    velocity Drag left) and Constant after it."""
    FF = load_force_fields(ref)
    fields = [FF.Drag(linear=0.8, quadratic=0.4), FF.Custom(custom_acc), FF.Constant(direction=(0.0, 1.0, 0.5),
                                                                                  strength=1.5)]
    for f in (fields[0], fields[2]):
        f.activate()
    out = gen_substeps(F, rng, ffs=fields, n_steps=n_steps)
    out["n_steps"] = np.array(n_steps)
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GENESIS_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <Genesis project root>  (or set GENESIS_REFERENCE)")
    F = load_reference(ref)
    rng = np.random.default_rng(20261204)
    np.savez_compressed(os.path.join(HERE, "materials.npz"), **gen_materials(F, rng))
    np.savez_compressed(os.path.join(HERE, "substep_small.npz"), **gen_substeps(F, rng))
    np.savez_compressed(os.path.join(HERE, "force_fields.npz"),
                        **gen_force_fields(F, ref, np.random.default_rng(20261205)))
    np.savez_compressed(os.path.join(HERE, "rigid_coupling.npz"), **gen_rigid(F, np.random.default_rng(20261206)))
    np.savez_compressed(os.path.join(HERE, "tool_coupling.npz"), **gen_tool(F, np.random.default_rng(20261207)))
    np.savez_compressed(os.path.join(HERE, "cpic_coupling.npz"),
                        **gen_rigid(F, np.random.default_rng(20261208), cpic=True))
    np.savez_compressed(os.path.join(HERE, "particle_coupling.npz"),
                        **gen_coupled(F, np.random.default_rng(20261209)))
    np.savez_compressed(os.path.join(HERE, "particle_constraints.npz"),
                        **gen_constraints(F, np.random.default_rng(20261210)))
    np.savez_compressed(os.path.join(HERE, "custom_field.npz"),
                        **gen_custom_field(F, ref, np.random.default_rng(20261211)))
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
