"""ctypes binding of libgbmpm.so (declared in include/gbmpm.h).

There is no fallback: if the library is missing or fails to load, every solver call raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

from .exceptions import GenesisException

c_int32, c_int64, c_double, c_void_p, c_float = (
    ctypes.c_int32,
    ctypes.c_int64,
    ctypes.c_double,
    ctypes.c_void_p,
    ctypes.c_float,
)

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libgbmpm.so")

MPM_OK = 0
STATUS_NAMES = {
    1: "MPM_ERR_BAD_ARG",
    2: "MPM_ERR_CUDA",
    3: "MPM_ERR_OOM",
    4: "MPM_ERR_NAN",
    5: "MPM_ERR_OOB",
    6: "MPM_ERR_TIMEOUT",
    7: "MPM_ERR_STATE",
}
STATUS_NAN = 0x1
STATUS_OOB = 0x2
STATUS_WAIT = 0x4
STATUS_BAD_INDEX = 0x8

# material types / flags (mpm_material_type, MPM_MATF_*)
MAT_ELASTIC, MAT_LIQUID, MAT_SAND, MAT_SNOW, MAT_ELASTOPLASTIC, MAT_MUSCLE = range(6)
MATF_NEOHOOKEAN = 0x1
MATF_VON_MISES = 0x2

# fields of mpm_set_particles / mpm_get_particles
FIELD_POS, FIELD_VEL, FIELD_C, FIELD_F, FIELD_JP, FIELD_ACTIVE, FIELD_ACTU, FIELD_FREE, FIELD_MUSCLE_DIR = range(9)
FIELD_POS_RESET = 9


class MpmMaterial(ctypes.Structure):
    _fields_ = [
        ("type", c_int32),
        ("flags", c_int32),
        ("scene", c_int32),
        ("reserved", c_int32),
        ("mu", c_double),
        ("lam", c_double),
        ("rho", c_double),
        ("default_Jp", c_double),
        ("friction_alpha", c_double),
        ("yield_lower", c_double),
        ("yield_higher", c_double),
        ("von_mises_yield_stress", c_double),
        ("stiffness", c_double),
    ]


class MpmPoolConfig(ctypes.Structure):
    _fields_ = [
        ("max_scenes", c_int64),
        ("particle_capacity", c_int64),
        ("max_grid_res", c_int32),
        ("max_materials_per_scene", c_int32),
        ("with_muscle", c_int32),
        ("reserved", c_int32),
    ]


class MpmCollider(ctypes.Structure):
    """mpm_collider (include/gbmpm.h)."""

    _fields_ = [
        ("type", c_int32),
        ("scene", c_int32),
        ("pos", c_double * 3),
        ("quat", c_double * 4),
        ("size", c_double * 3),
        ("com", c_double * 3),
        ("lin_vel", c_double * 3),
        ("ang_vel", c_double * 3),
        ("friction", c_double),
        ("softness", c_double),
        ("restitution", c_double),
        ("sdf_grid", c_int32),
        ("pad", c_int32),
        ("floor_height", c_double),
    ]


COLLIDER_SPHERE, COLLIDER_PLANE, COLLIDER_BOX, COLLIDER_SDF, COLLIDER_TOOL = 0, 1, 2, 3, 4


class MpmForceField(ctypes.Structure):
    """mpm_force_field (include/gbmpm.h)."""

    _fields_ = [
        ("type", c_int32),
        ("active", c_int32),
        ("direction", c_double * 3),
        ("center", c_double * 3),
        ("strength", c_double),
        ("radius", c_double),
        ("falloff_pow", c_double),
        ("flow", c_double),
        ("linear", c_double),
        ("quadratic", c_double),
        ("strength_perpendicular", c_double),
        ("strength_radial", c_double),
        ("falloff_min", c_double),
        ("falloff_max", c_double),
        ("damping", c_double),
        ("frequency", c_double),
        ("seed", ctypes.c_uint64),
        ("perm", (ctypes.c_uint8 * 256) * 3),
    ]


FF_CONSTANT, FF_WIND, FF_POINT, FF_DRAG, FF_VORTEX, FF_NOISE, FF_TURBULENCE = 0, 1, 2, 3, 4, 5, 6


class MpmDiffTool(ctypes.Structure):
    """mpm_diff_tool (gbmpm.h): a tool of the differentiable form."""

    _fields_ = [
        ("sdf", c_void_p),
        ("res", c_int32 * 3),
        ("pad0", c_int32),
        ("T_mesh_to_sdf", c_double * 16),
        ("friction", c_double),
        ("softness", c_double),
        ("floor_height", c_double),
    ]


class MpmDiffExtras(ctypes.Structure):
    """mpm_diff_extras (gbmpm.h): tools, force fields and Muscle inputs of a differentiable sequence."""

    _fields_ = [
        ("tools", c_void_p),
        ("n_tools", c_int32),
        ("n_force_fields", c_int32),
        ("tool_seq", c_void_p),
        ("g_tool", c_void_p),
        ("force_fields", c_void_p),
        ("scene_index", c_int32),
        ("pad0", c_int32),
        ("ff_step", ctypes.c_uint64),
        ("actu", c_void_p),
        ("muscle_dir", c_void_p),
        ("g_actu", c_void_p),
        ("colliders", c_void_p),
        ("sdf_ctx", c_void_p),
        ("n_colliders", c_int32),
        ("pad1", c_int32),
        ("constraint_stiffness", c_void_p),
        ("constraint_target", c_void_p),
        ("active", c_void_p),
    ]


DIFF_MAX_TOOLS = 4
DIFF_MAX_FORCE_FIELDS = 8
DIFF_MAX_COLLIDERS = 8


class MpmSceneConfig(ctypes.Structure):
    _fields_ = [
        ("substep_dt", c_double),
        ("gravity", c_double * 3),
        ("lower_bound", c_double * 3),
        ("upper_bound", c_double * 3),
        ("grid_density", c_double),
        ("particle_size", c_double),
        ("mass_eps", c_double),
        ("restitution", c_double),
        ("n_particles", c_int64),
    ]


_P = c_void_p
# name -> (restype, argtypes)
_SIGNATURES = {
    "mpm_ctx_create": (c_int32, [ctypes.POINTER(MpmSceneConfig), c_int64, ctypes.POINTER(MpmMaterial), c_int32, c_int32, ctypes.POINTER(c_void_p)]),
    "mpm_ctx_destroy": (c_int32, [_P]),
    "mpm_last_error": (ctypes.c_char_p, [_P]),
    "mpm_add_particles": (c_int32, [_P, c_int64, c_int64, c_int64, c_int64, c_int32, c_int32, _P, _P]),
    "mpm_get_state": (c_int32, [_P, c_int64, c_int64, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_set_state": (c_int32, [_P, c_int64, c_int64, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_set_particles": (c_int32, [_P, c_int32, c_int64, c_int64, c_int64, c_int64, _P, _P]),
    "mpm_get_particles": (c_int32, [_P, c_int32, c_int64, c_int64, c_int64, c_int64, _P, _P]),
    "mpm_set_gravity": (c_int32, [_P, c_int64, c_int64, ctypes.POINTER(c_double)]),
    "mpm_substeps": (c_int32, [_P, c_int32, _P]),
    "mpm_substep_pre": (c_int32, [_P, _P]),
    "mpm_substep_grid_op": (c_int32, [_P, _P]),
    "mpm_substep_grid_stage": (c_int32, [_P, c_int32, c_int32, c_int32, _P]),
    "mpm_grid_nodes": (c_int32, [_P, ctypes.POINTER(_P), ctypes.POINTER(c_int64)]),
    "mpm_grid_node_positions": (c_int32, [_P, _P, _P, _P]),
    "mpm_substep_post": (c_int32, [_P, _P]),
    "mpm_get_grid": (c_int32, [_P, c_int64, _P, _P]),
    "mpm_count_touched_nodes": (c_int32, [_P, ctypes.POINTER(c_int64), _P]),
    "mpm_status_word": (c_int32, [_P, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(c_int64), c_int32, _P]),
    "mpm_set_tuning": (c_int32, [_P, c_int32, c_int32, c_int32, c_int32]),
    "mpm_get_info": (c_int32, [_P, ctypes.POINTER(c_int64), ctypes.POINTER(c_int64), ctypes.POINTER(c_int64)]),
    "mpm_scene_grid_res": (c_int32, [_P, c_int64, ctypes.POINTER(c_int32)]),
    "mpm_set_profiling": (c_int32, [_P, c_int32]),
    "mpm_kernel_times": (c_int32, [_P, ctypes.POINTER(c_double), ctypes.POINTER(c_int64), c_int32]),
    "mpm_render_fields": (c_int32, [_P, c_int64, c_int64, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P]),
    "mpm_set_particle_constraints": (c_int32, [_P, c_int64, c_int64, c_int64, c_int64, _P, c_double, c_int32, _P, _P,
                                               _P]),
    "mpm_remove_particle_constraints": (c_int32, [_P, c_int64, c_int64, c_int64, c_int64, _P, _P]),
    "mpm_set_link_poses": (c_int32, [_P, c_int32, _P]),
    "mpm_set_colliders": (c_int32, [_P, c_int32, _P]),
    "mpm_diff_forward_seq": (c_int32, [_P, c_double, c_int32, c_int64, c_int32, _P, _P, _P, _P, c_int32, _P, _P,
                                       _P, _P, c_int32, _P, _P]),
    "mpm_diff_backward_seq": (c_int32, [_P, c_double, c_int32, c_int64, c_int32, _P, _P, _P, _P, _P, _P, _P,
                                        _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_diff_forward_seq_pp": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, c_int32, _P, _P,
                                          _P, _P, c_int32, _P, _P]),
    "mpm_diff_backward_seq_pp": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, _P, _P, _P,
                                           _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_diff_forward_seq_tools": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, c_int32, _P, _P,
                                             _P, c_int32, _P, _P, _P, c_int32, _P, _P]),
    "mpm_diff_backward_seq_tools": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, _P, _P, _P,
                                              c_int32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_diff_forward_seq_ex": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, c_int32, _P, _P,
                                          _P, _P, _P, c_int32, _P, _P]),
    "mpm_diff_backward_seq_ex": (c_int32, [_P, _P, _P, _P, c_int64, c_int32, _P, _P, _P, _P, _P, _P, _P, _P,
                                           _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_diff_substep_stage": (c_int32, [_P, _P, _P, _P, c_int64, _P, _P, _P, _P, _P, _P, _P, _P, c_int32, c_int32,
                                         c_int32, c_int32, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_diff_substep_stage_adj": (c_int32, [_P, _P, _P, _P, c_int64, _P, _P, _P, _P, _P, _P, _P, _P, c_int32,
                                             c_int32, c_int32, c_int32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                             _P, _P, _P, _P, _P, _P, _P, _P]),
    "mpm_set_force_fields": (c_int32, [_P, c_int32, _P]),
    "mpm_sample_regular": (c_int32, [c_int32, _P, _P, c_double, _P, c_int64, _P, _P]),
    "mpm_test_wait_timeout": (c_int32, [_P, _P]),
    "mpm_get_collider_forces": (c_int32, [_P, _P, c_int32, _P]),
    "mpm_add_sdf_grid": (c_int32, [_P, _P, _P, _P, _P, c_double, c_double, ctypes.POINTER(c_int32)]),
    "mpm_get_collider_poses": (c_int32, [_P, _P, _P]),
    "mpm_enable_cpic": (c_int32, [_P, c_int32, _P]),
    "mpm_set_coupled_particles": (c_int32, [_P, c_int32, c_int64, _P, _P, _P, _P, _P]),
    "mpm_version": (c_int32, []),
    "mpm_ctx_create_pool": (c_int32, [ctypes.c_void_p, c_int32, ctypes.POINTER(c_void_p)]),
    "mpm_scene_admit": (c_int32, [_P, c_int64, ctypes.c_void_p, ctypes.c_void_p, c_int32, c_int64, _P, _P, c_int32, _P]),
    "mpm_scene_retire": (c_int32, [_P, c_int64, _P]),
    "mpm_scene_steps_left": (c_int32, [_P, ctypes.POINTER(c_int32), _P]),
    "mpm_substeps_noalloc": (c_int32, [_P, _P, c_int32, c_int64, _P, _P, _P, _P, _P, _P, _P, c_int32, _P]),
    "mpm_noalloc_last_error": (ctypes.c_char_p, []),
    "mpm_diff_forward": (c_int32, [_P, c_double, c_int32, c_int64] + [_P] * 14),
    "mpm_diff_backward": (c_int32, [_P, c_double, c_int32, c_int64] + [_P] * 22),
}

_lib = None
_lock = threading.Lock()


def exported_symbols() -> list[str]:
    """Names the binding expects the library to export (also checked by the CPU tests)."""
    return sorted(_SIGNATURES)


def load(path: str | None = None):
    """Load libgbmpm.so once; raise GenesisException if it is missing (no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise GenesisException(
                f"libgbmpm.so not found at {p}. Build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the MPM solver has no CPU fallback)."
            )
        lib = ctypes.CDLL(p)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def check(ret: int, ctx=None, what: str = "") -> None:
    """Map a status code to GenesisException carrying the library's error text."""
    if ret == MPM_OK:
        return
    lib = load()
    msg = lib.mpm_last_error(ctx)
    msg = msg.decode() if msg else ""
    raise GenesisException(f"{what}: {STATUS_NAMES.get(ret, ret)}: {msg}")


def ptr(t) -> int | None:
    """Device pointer of a contiguous torch tensor (None for None)."""
    if t is None:
        return None
    if not t.is_contiguous():
        raise GenesisException("tensor must be contiguous")
    return t.data_ptr()
