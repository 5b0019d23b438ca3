"""C-ABI library: loads, exports every function include/gbmpm.h declares, validates arguments
on the host before touching CUDA (no compute calls here: this container has no GPU)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "gbmpm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(mpm_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from genesis_gb300 import _lib
    from genesis_gb300.build import build

    build()
    return _lib.load()


def test_header_declares_expected_api():
    fns = header_functions()
    for name in ("mpm_ctx_create", "mpm_substeps", "mpm_get_state", "mpm_set_state", "mpm_add_particles",
                 "mpm_status_word"):
        assert name in fns


def test_library_exports_every_header_function(lib):
    from genesis_gb300 import _lib

    for name in header_functions():
        assert hasattr(lib, name), name
    assert set(header_functions()) == set(_lib.exported_symbols())
    assert lib.mpm_version() == 1


def _cfg(**kw):
    from genesis_gb300 import _lib

    c = _lib.MpmSceneConfig()
    c.substep_dt = kw.get("dt", 2e-4)
    for d in range(3):
        c.gravity[d] = (0, 0, -9.81)[d]
        c.lower_bound[d] = kw.get("lb", (0, 0, 0))[d]
        c.upper_bound[d] = kw.get("ub", (1, 1, 1))[d]
    c.grid_density = kw.get("density", 64)
    c.particle_size = 0.01
    c.mass_eps = 1.19e-7
    c.n_particles = kw.get("n", 10)
    return c


def _mat(scene=0):
    from genesis_gb300 import _lib

    m = _lib.MpmMaterial()
    m.type = 0
    m.scene = scene
    m.mu, m.lam, m.rho, m.default_Jp = 1e5, 1e5, 1000, 1
    return m


def _create(lib, cfgs, mats):
    ctx = ctypes.c_void_p()
    C = (type(cfgs[0]) * len(cfgs))(*cfgs)
    M = (type(mats[0]) * len(mats))(*mats) if mats else None
    r = lib.mpm_ctx_create(C, len(cfgs), M, len(mats), 0, ctypes.byref(ctx))
    return r, ctx, lib.mpm_last_error(None).decode()


def test_create_rejects_bad_bounds(lib):
    r, ctx, msg = _create(lib, [_cfg(lb=(0, 0, 1), ub=(1, 1, 0))], [_mat()])
    assert r == 1 and "upper_bound" in msg and not ctx.value


def test_create_rejects_huge_grid(lib):
    r, _, msg = _create(lib, [_cfg(density=2000, lb=(-1, -1, -1), ub=(1, 1, 1))], [_mat()])
    assert r == 1 and "1e9" in msg


def test_create_rejects_unsorted_materials(lib):
    r, _, msg = _create(lib, [_cfg(), _cfg()], [_mat(1), _mat(0)])
    assert r == 1 and "grouped by scene" in msg


def test_create_rejects_particles_without_material(lib):
    r, _, msg = _create(lib, [_cfg(), _cfg()], [_mat(0)])
    assert r == 1 and "no material" in msg


def test_null_ctx_is_bad_arg(lib):
    assert lib.mpm_substeps(None, 1, None) == 1
    assert lib.mpm_get_state(None, 0, 1, None, None, None, None, None, None, None) == 1
    assert lib.mpm_ctx_destroy(None) == 0


def test_product_fails_loudly_without_library(tmp_path):
    from genesis_gb300 import _lib
    from genesis_gb300.exceptions import GenesisException

    with pytest.raises(GenesisException):
        _lib.load(str(tmp_path / "missing.so"))


def test_differentiable_extras_are_validated_on_the_host(lib):
    """mpm_diff_forward_seq_ex / mpm_diff_backward_seq_ex reject malformed extras records before any
    CUDA call: too many force fields or tools, an unknown field type, a tool-shaped or SDF collider
    without its context, and half-given Muscle or constraint inputs."""
    from genesis_gb300 import _lib

    cfg = _cfg(n=0)
    buf = (ctypes.c_float * 64)()  # stands in for the device arrays; never touched on rejection
    p = ctypes.cast(buf, ctypes.c_void_p)

    def fwd(ex):
        return lib.mpm_diff_forward_seq_ex(ctypes.byref(cfg), p, p, p, 0, 1, p, p, p, p, p, 2, p, p,
                                           ctypes.byref(ex), p, p, 0, p, None)

    def bwd(ex):
        return lib.mpm_diff_backward_seq_ex(ctypes.byref(cfg), p, p, p, 0, 1, p, p, p, p, p, p, p,
                                            ctypes.byref(ex), p, p, p, p, p, p, p, p, None)

    ff = (_lib.MpmForceField * 9)()
    col = (_lib.MpmCollider * 1)()
    cases = []
    ex = _lib.MpmDiffExtras()
    ex.force_fields, ex.n_force_fields = ctypes.addressof(ff), 9
    cases.append(ex)
    ex = _lib.MpmDiffExtras()
    ff[0].type = 99
    ex.force_fields, ex.n_force_fields = ctypes.addressof(ff), 1
    cases.append(ex)
    ex = _lib.MpmDiffExtras()
    ex.n_tools = _lib.DIFF_MAX_TOOLS + 1
    cases.append(ex)
    for ctype in (4, 3):  # MPM_COLLIDER_TOOL; MPM_COLLIDER_SDF with no context to hold its grid
        col[0].type = ctype
        ex = _lib.MpmDiffExtras()
        ex.colliders, ex.n_colliders = ctypes.addressof(col), 1
        cases.append(ex)
    ex = _lib.MpmDiffExtras()
    ex.colliders, ex.n_colliders = ctypes.addressof(col), _lib.DIFF_MAX_COLLIDERS + 1
    cases.append(ex)
    ex = _lib.MpmDiffExtras()
    ex.actu = p.value
    cases.append(ex)
    ex = _lib.MpmDiffExtras()
    ex.constraint_stiffness = p.value
    cases.append(ex)
    for i, ex in enumerate(cases):
        assert fwd(ex) == 1, i
        assert bwd(ex) == 1, i


def test_staged_differentiable_substep_arguments_are_validated_on_the_host(lib):
    """mpm_diff_substep_stage / _adj reject a phase or stage out of range, a field range outside the
    record and a stage adjoint without the velocity it began from, before any CUDA call."""
    from genesis_gb300 import _lib

    cfg = _cfg(n=0)
    buf = (ctypes.c_float * 64)()
    p = ctypes.cast(buf, ctypes.c_void_p)
    ex = _lib.MpmDiffExtras()

    def fwd(phase, stage, b=0, e=0):
        return lib.mpm_diff_substep_stage(ctypes.byref(cfg), p, p, p, 0, p, p, p, p, p, p, p, ctypes.byref(ex),
                                          phase, stage, b, e, p, p, p, p, p, p, p, p, None)

    def adj(phase, stage, vstage, b=0, e=0):
        return lib.mpm_diff_substep_stage_adj(ctypes.byref(cfg), p, p, p, 0, p, p, p, p, p, p, p, ctypes.byref(ex),
                                              phase, stage, b, e, vstage, p, p, p, p, p, p, p, p, p, p, p, p,
                                              p, p, p, p, p, None)

    assert fwd(3, 0) == 1 and fwd(-1, 0) == 1
    assert fwd(1, 0) == 1 and fwd(1, 4) == 1
    assert fwd(1, 1, 0, 1) == 1  # the record holds no field
    assert adj(1, 2, None) == 1 and adj(1, 3, None) == 1
    assert adj(1, 2, p, 2, 1) == 1
