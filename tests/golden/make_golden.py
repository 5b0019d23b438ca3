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
  substep_small.npz a 6-material scene on a 17^3 grid: input state, grid (momentum, mass)
                    after the first P2G, states after 1 and 10 substeps

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

    def outer_product(self, other):
        return np.outer(np.asarray(self), np.asarray(other)).view(QMat)

    def cast(self, dtype):
        return np.asarray(self).astype(dtype).view(QMat)

    def dot(self, other):
        return float(np.dot(np.asarray(self), np.asarray(other)))

    def cross(self, other):
        return np.cross(np.asarray(self), np.asarray(other)).view(QMat)

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
    qd.floor = lambda x: np.floor(x).view(QMat) if isinstance(x, np.ndarray) else math.floor(x)
    qd.max = lambda a, b: np.maximum(a, b).view(QMat) if isinstance(a, np.ndarray) or isinstance(b, np.ndarray) else max(a, b)
    qd.min = lambda a, b: np.minimum(a, b).view(QMat) if isinstance(a, np.ndarray) or isinstance(b, np.ndarray) else min(a, b)
    qd.abs = abs
    qd.select = lambda c, a, b: a if c else b
    qd.svd = _svd
    qd.math = types.SimpleNamespace(isnan=lambda x: bool(np.isnan(x)))
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
def extract(path, cls, names, ns):
    """Compile methods `names` of class `cls` in `path` (decorators/annotations removed) into ns."""
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
    F["boundary"] = extract(os.path.join(ref, "genesis/engine/boundaries/boundaries.py"), "CubeBoundary",
                            ["impose_pos_vel"], ns)
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
def gen_substeps(F, rng, ffs=(), n_steps=10):
    """A 9-material scene on a 17^3 grid advanced by the reference's substep code; `ffs` are
    reference force-field objects applied in its grid op (legacy_coupler.py:376-378)."""
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

    P, I, G = solver.particles._d, solver.particles_info._d, solver.grid._d
    P["pos"][0, :, 0], P["vel"][0, :, 0], P["C"][0, :, 0], P["F"][0, :, 0] = pos, vel, C, Fm
    P["Jp"][0, :, 0], P["actu"][0, :, 0] = Jp, actu
    solver.particles_ng._d["active"][0, :, 0] = 1
    I["material_idx"][:], I["mass"][:], I["free"][:], I["muscle_direction"][:] = mat, p_vol * rho, 1, mdir

    def snapshot():
        return {k: P[k][0, :, 0].copy() for k in ("pos", "vel", "C", "F", "Jp")}

    out = {"in/" + k: v for k, v in snapshot().items()}
    out.update({"in/mat": mat, "in/actu": actu, "in/mdir": mdir})
    for step in range(n_steps):
        for k in G:
            G[k][...] = 0  # reset_grid_and_grad
        solver.compute_F_tmp(0)
        solver.svd(0)
        solver.p2g(0, None, None, None, None, None, None)
        if step == 0:
            out["grid1"] = np.concatenate([G["vel_in"][0, ..., 0, :], G["mass"][0, ..., 0, None]], -1).copy()
        coupler.mpm_grid_op(0, 0.0, None, None, None, None, None, None)
        solver.g2p(0, None, None, None)
        for k in ("pos", "vel", "C", "F", "Jp"):  # copy_frame(1 -> 0)
            P[k][0] = P[k][1]
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
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
