"""Python binding of the CPU oracle (oracle/mpm_oracle.cpp).  TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker and
as the timed CPU baseline; never by the product path (genesis_gb300 does not import it).

Parity status of the oracle: checked against golden vectors produced by executing the
reference's own MPM kernels and material functions (tests/golden/); see that folder's
generator script.  The 3x3 SVD of the reference (qd.svd, in the absent quadrants package)
is not pinned: only rotation-invariant quantities are compared.
"""

from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
if _HERE not in sys.path:
    sys.path.insert(0, _HERE)

from build_oracle import LIB_PATH, build  # noqa: E402


class OracleScene(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("lower_bound", ctypes.c_double * 3),
        ("upper_bound", ctypes.c_double * 3),
        ("grid_density", ctypes.c_double),
        ("particle_size", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("restitution", ctypes.c_double),
    ]


class OracleMaterial(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("mu", ctypes.c_double),
        ("lam", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("default_Jp", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("yield_lower", ctypes.c_double),
        ("yield_higher", ctypes.c_double),
        ("vm_yield", ctypes.c_double),
        ("stiffness", ctypes.c_double),
    ]


class _Collider(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("scene", ctypes.c_int32),
        ("pos", ctypes.c_double * 3),
        ("quat", ctypes.c_double * 4),
        ("size", ctypes.c_double * 3),
        ("com", ctypes.c_double * 3),
        ("lin_vel", ctypes.c_double * 3),
        ("ang_vel", ctypes.c_double * 3),
        ("friction", ctypes.c_double),
        ("softness", ctypes.c_double),
        ("restitution", ctypes.c_double),
        ("sdf_grid", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("floor_height", ctypes.c_double),
    ]


MAT_TYPES = {"elastic": 0, "liquid": 1, "sand": 2, "snow": 3, "elastoplastic": 4, "muscle": 5}
FP32_EPS = float(np.finfo(np.float32).eps)

_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        for name in ("oracle_substeps_f64", "oracle_substeps_f32"):
            fn = getattr(lib, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(OracleMaterial), ctypes.c_int, ctypes.c_int64,
                           P, P, P, P, P, P, P, P, P, P, ctypes.c_int, P, ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
        lib.oracle_svd_f64.argtypes = [P, P, P, P]
        lib.oracle_svd_f64.restype = None
        lib.oracle_material_f64.argtypes = [ctypes.POINTER(OracleMaterial), P, ctypes.c_double, ctypes.c_double, P,
                                            ctypes.c_double, P, P, P]
        lib.oracle_material_f64.restype = None
        lib.oracle_grid_res.argtypes = [ctypes.POINTER(OracleScene), P]
        lib.oracle_grid_res.restype = ctypes.c_int
        lib.oracle_set_colliders.argtypes = [ctypes.c_int, P]
        lib.oracle_set_colliders.restype = None
        lib.oracle_set_force_fields.argtypes = [ctypes.c_int, P]
        lib.oracle_set_force_fields.restype = None
        lib.oracle_collider_forces.argtypes = [P]
        lib.oracle_collider_forces.restype = None
        lib.oracle_add_sdf_grid.argtypes = [P, P, P, P, ctypes.c_double, ctypes.c_double]
        lib.oracle_add_sdf_grid.restype = ctypes.c_int
        lib.oracle_clear_sdf_grids.argtypes = []
        lib.oracle_clear_sdf_grids.restype = None
        lib.oracle_collider_poses.argtypes = [P]
        lib.oracle_collider_poses.restype = None
        lib.oracle_set_cpic.argtypes = [ctypes.c_int]
        lib.oracle_set_cpic.restype = None
        lib.oracle_set_coupled.argtypes = [ctypes.c_int, ctypes.c_int64, P, P, P, P]
        lib.oracle_set_coupled.restype = None
        lib.oracle_coupled_vel.argtypes = [ctypes.c_int, P]
        lib.oracle_coupled_vel.restype = None
        _lib = lib
    return _lib


def make_scene(dt, gravity=(0.0, 0.0, -9.81), lower_bound=(0.0, 0.0, 0.0), upper_bound=(1.0, 1.0, 1.0),
               grid_density=64.0, particle_size=None, eps=FP32_EPS, restitution=0.0) -> OracleScene:
    s = OracleScene()
    s.dt = dt
    for d in range(3):
        s.gravity[d] = gravity[d]
        s.lower_bound[d] = lower_bound[d]
        s.upper_bound[d] = upper_bound[d]
    s.grid_density = grid_density
    s.particle_size = particle_size if particle_size is not None else 0.01 * 64.0 / grid_density
    s.eps = eps
    s.restitution = restitution
    return s


def make_material(type_id, mu, lam, rho=1000.0, default_Jp=1.0, alpha=0.0, yield_lower=0.0, yield_higher=0.0,
                  vm_yield=0.0, stiffness=0.0, flags=0) -> OracleMaterial:
    m = OracleMaterial()
    m.type, m.flags = int(type_id), int(flags)
    m.mu, m.lam, m.rho, m.default_Jp = mu, lam, rho, default_Jp
    m.alpha, m.yield_lower, m.yield_higher, m.vm_yield, m.stiffness = alpha, yield_lower, yield_higher, vm_yield, stiffness
    return m


def from_c_material(cm) -> OracleMaterial:
    """Convert a libgbmpm mpm_material record (same field meanings) into an oracle material."""
    return make_material(cm.type, cm.mu, cm.lam, cm.rho, cm.default_Jp, cm.friction_alpha, cm.yield_lower,
                         cm.yield_higher, cm.von_mises_yield_stress, cm.stiffness, cm.flags)


def grid_res(scene: OracleScene) -> tuple[int, int, int]:
    r = np.zeros(3, dtype=np.int64)
    load().oracle_grid_res(ctypes.byref(scene), r.ctypes.data)
    return tuple(int(v) for v in r)


def run(scene: OracleScene, materials, state: dict, n_substeps: int, dtype=np.float64, want_grid=False,
        threads=1):
    """Advance `state` (dict of pos [n,3], vel [n,3], C [n,3,3], F [n,3,3], Jp [n], mat [n] int,
    active [n] bool, optional free [n] bool, actu [n], mdir [n,3]) by n_substeps.

    Returns (new_state, grid or None, n_touched); grid is [gx,gy,gz,4] (momentum, mass)
    after the last P2G.  Raises RuntimeError on NaN (4) or a stencil leaving the grid (5)."""
    lib = load()
    fn = lib.oracle_substeps_f64 if dtype == np.float64 else lib.oracle_substeps_f32
    n = len(state["pos"])
    st = {k: np.ascontiguousarray(np.array(state[k], dtype=dtype)) for k in ("pos", "vel", "C", "F", "Jp")}
    mat = np.ascontiguousarray(np.asarray(state["mat"], dtype=np.int32))
    act = np.ascontiguousarray(np.asarray(state["active"], dtype=np.uint8))
    free = state.get("free")
    free = None if free is None else np.ascontiguousarray(np.asarray(free, dtype=np.uint8))
    actu = state.get("actu")
    actu = None if actu is None else np.ascontiguousarray(np.asarray(actu, dtype=dtype))
    mdir = state.get("mdir")
    mdir = None if mdir is None else np.ascontiguousarray(np.asarray(mdir, dtype=dtype))
    mats = (OracleMaterial * max(1, len(materials)))(*materials)
    grid = None
    if want_grid:
        grid = np.zeros(grid_res(scene) + (4,), dtype=dtype)
    touched = ctypes.c_int64(0)

    def p(a):
        return None if a is None else a.ctypes.data

    ret = fn(ctypes.byref(scene), mats, len(materials), n, p(st["pos"]), p(st["vel"]), p(st["C"]), p(st["F"]),
             p(st["Jp"]), p(mat), p(act), p(free), p(actu), p(mdir), int(n_substeps), p(grid), ctypes.byref(touched),
             int(threads))
    if ret == 4:
        raise RuntimeError("oracle: NaN in particle positions")
    if ret == 5:
        raise RuntimeError("oracle: particle stencil left the grid")
    out = dict(state)
    out.update(st)
    return out, grid, touched.value


def set_colliders(colliders) -> None:
    """Kinematic colliders (list of genesis_gb300._lib.MpmCollider, same layout) for the following
    runs; an empty list removes them.  Resets the accumulated reaction forces."""
    lib = load()
    n = len(colliders)
    arr = (_Collider * max(1, n))(*[_Collider.from_buffer_copy(bytes(c)) for c in colliders])
    lib.oracle_set_colliders(n, arr)


def add_sdf_grid(values, grads, T_mesh_to_sdf, cell_size, sdf_max) -> int:
    """Voxel SDF grid for colliders of type 3 (rigid, with gradients) and 4 (tool, grads None);
    returns its id (0, 1, ... in call order, like the library's mpm_add_sdf_grid)."""
    lib = load()
    v = np.ascontiguousarray(values, np.float32)
    g = None if grads is None else np.ascontiguousarray(grads, np.float32)
    res = np.asarray(v.shape, np.int32)
    T = np.ascontiguousarray(T_mesh_to_sdf, np.float64)
    return lib.oracle_add_sdf_grid(res.ctypes.data, v.ctypes.data, None if g is None else g.ctypes.data, T.ctypes.data,
                                   float(cell_size), float(sdf_max))


def clear_sdf_grids() -> None:
    load().oracle_clear_sdf_grids()


def collider_poses(n) -> np.ndarray:
    """[n, 7] current pose (pos, quat wxyz) of each collider; tools advance every substep."""
    out = np.zeros((n, 7))
    load().oracle_collider_poses(out.ctypes.data)
    return out


def set_force_fields(fields) -> None:
    """Force fields (list of genesis_gb300._lib.MpmForceField, same layout) for the following runs."""
    n = len(fields)
    buf = b"".join(bytes(f) for f in fields) or b"\0" * 8
    arr = ctypes.create_string_buffer(buf, len(buf))
    load().oracle_set_force_fields(n, arr)


def set_cpic(enable: bool) -> None:
    """CPIC (MPMOptions.enable_CPIC) for the following runs; clears the particle-side collider
    normals, which otherwise persist from run to run like the particle state."""
    load().oracle_set_cpic(1 if enable else 0)


_coupled_n = [0, 0]


def set_coupled(kind: int, pos=None, vel=None, mass=None, free=None) -> None:
    """Coupled particle set `kind` (0 SPH, 1 PBD) for the following runs: pos, vel [n, 3],
    mass [n], free [n] (PBD; None: all free).  pos=None removes the set.  Their velocities are
    updated in place by every grid op, run after run, until the set is replaced."""
    lib = load()
    if pos is None:
        z = np.zeros(3)
        lib.oracle_set_coupled(kind, 0, z.ctypes.data, z.ctypes.data, z.ctypes.data, None)
        _coupled_n[kind] = 0
        return
    p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    v = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
    m = np.ascontiguousarray(mass, dtype=np.float64).reshape(-1)
    f = None if free is None else np.ascontiguousarray(free, dtype=np.uint8).reshape(-1)
    lib.oracle_set_coupled(kind, len(p), p.ctypes.data, v.ctypes.data, m.ctypes.data,
                           None if f is None else f.ctypes.data)
    _coupled_n[kind] = len(p)


def coupled_velocities(kind: int) -> np.ndarray:
    out = np.zeros((max(1, _coupled_n[kind]), 3))
    load().oracle_coupled_vel(kind, out.ctypes.data)
    return out[:_coupled_n[kind]]


def collider_forces(n: int) -> np.ndarray:
    out = np.zeros((max(1, n), 6))
    load().oracle_collider_forces(out.ctypes.data)
    return out[:n]


def svd(A):
    A = np.ascontiguousarray(np.asarray(A, dtype=np.float64).reshape(3, 3))
    U, s, V = np.zeros((3, 3)), np.zeros(3), np.zeros((3, 3))
    load().oracle_svd_f64(A.ctypes.data, U.ctypes.data, s.ctypes.data, V.ctypes.data)
    return U, s, V


def material_update(m: OracleMaterial, F_tmp, Jp=1.0, actu=0.0, mdir=(0.0, 0.0, 1.0), eps=FP32_EPS):
    """One particle's (F_new, Jp_new, stress) from F_tmp (before the stress scale)."""
    Ft = np.ascontiguousarray(np.asarray(F_tmp, dtype=np.float64).reshape(3, 3))
    md = np.ascontiguousarray(np.asarray(mdir, dtype=np.float64))
    Fn, st = np.zeros((3, 3)), np.zeros((3, 3))
    jn = ctypes.c_double(0.0)
    load().oracle_material_f64(ctypes.byref(m), Ft.ctypes.data, float(Jp), float(actu), md.ctypes.data, float(eps),
                               Fn.ctypes.data, ctypes.addressof(jn), st.ctypes.data)
    return Fn, jn.value, st
