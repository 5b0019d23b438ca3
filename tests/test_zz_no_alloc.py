"""mpm_substeps_noalloc: the entry point for callers that may not allocate device memory.

Such callers (plug-ins whose host application owns every device allocation through its own
pool, real-time loops that forbid allocator calls after start-up) pass their own particle
arrays; the grid the substep needs lives in a fixed device array inside the library.  The GPU
test checks it against the context entry point (mpm_substeps) and against the FP64 CPU oracle
on the same scene, over two calls in a row, within the position tolerance the other GPU tests
use (1e-4 of the 1 m domain).  This file is named to be collected last."""

import ctypes

import numpy as np
import pytest
import torch

POS_TOL = 1e-4


def _scene_and_materials(n):
    from genesis_gb300 import _lib
    from genesis_gb300.materials import Elastic, Sand
    from capi_helpers import scene_record

    sc = scene_record(_lib, 2e-4, n, density=64.0, p_size=1 / 128)
    mats = [Elastic(E=3e5, nu=0.2).to_c(0), Sand().to_c(0)]
    return sc, mats


def test_noalloc_rejects_grid_beyond_limit():
    """Host-side check (no GPU needed): a grid above 524288 nodes is refused before any CUDA call."""
    from genesis_gb300 import _lib
    from genesis_gb300.build import build
    from capi_helpers import scene_record

    build()
    lib = _lib.load()
    sc = scene_record(_lib, 2e-4, 10, density=128.0)  # 129^3 nodes
    m = (_lib.MpmMaterial * 1)(_scene_and_materials(10)[1][0])
    r = lib.mpm_substeps_noalloc(ctypes.byref(sc), m, 1, 0, None, None, None, None, None, None, None, 1, None)
    assert r == 1
    assert b"524288" in lib.mpm_noalloc_last_error()


@pytest.mark.gpu
def test_noalloc_matches_context_entry_point_on_two_calls(oracle):
    import __graft_entry__ as g

    g.build()
    from genesis_gb300 import _lib
    from capi_helpers import Ctx

    rng = np.random.default_rng(11)
    ax = np.linspace(0.35, 0.45, 13)
    cube_a = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    cube_b = cube_a + np.array([0.2, 0.1, 0.05])
    pos = np.concatenate([cube_a, cube_b]) + rng.uniform(-0.004, 0.004, size=(2 * len(cube_a), 3))
    n = len(pos)
    mat = np.concatenate([np.zeros(len(cube_a), np.int32), np.ones(len(cube_b), np.int32)])
    sc, mats = _scene_and_materials(n)

    # existing entry point: a context
    c = Ctx([sc], mats)
    c.add(0, 1, 0, pos[: len(cube_a)], 0)
    c.add(0, 1, len(cube_a), pos[len(cube_a):], 1)

    # no-allocation entry point: caller-owned arrays
    lib = _lib.load()
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    P = dev(pos.astype(np.float32))
    V = torch.zeros((n, 3), device="cuda")
    Cm = torch.zeros((n, 3, 3), device="cuda")
    F = torch.eye(3, device="cuda").repeat(n, 1, 1).contiguous()
    Jp = dev(np.where(mat == 1, 0.0, 1.0).astype(np.float32))
    M = dev(mat)
    A = torch.ones(n, dtype=torch.uint8, device="cuda")
    mat_arr = (_lib.MpmMaterial * 2)(*mats)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    host = dict(pos=pos.astype(np.float32).astype(np.float64), vel=np.zeros((n, 3)), C=np.zeros((n, 3, 3)),
                F=np.tile(np.eye(3), (n, 1, 1)), Jp=np.where(mat == 1, 0.0, 1.0), mat=mat, active=np.ones(n, bool))
    osc = oracle.make_scene(2e-4, grid_density=64.0, particle_size=1 / 128)
    omats = [oracle.from_c_material(m) for m in mats]
    for call in range(2):
        c.substeps(25)
        ref = c.get_state(0, 1, n)
        host, _, _ = oracle.run(osc, omats, host, 25)
        r = lib.mpm_substeps_noalloc(ctypes.byref(sc), mat_arr, 2, n, P.data_ptr(), V.data_ptr(), Cm.data_ptr(),
                                     F.data_ptr(), Jp.data_ptr(), M.data_ptr(), A.data_ptr(), 25, stream)
        assert r == 0, lib.mpm_noalloc_last_error()
        torch.cuda.synchronize()
        err = np.abs(P.cpu().numpy() - ref["pos"]).max()
        assert err <= POS_TOL, (call, err)
        assert np.abs(V.cpu().numpy() - ref["vel"]).max() <= 1e-2, call
        assert np.abs(F.cpu().numpy() - ref["F"]).max() <= 1e-4, call
        oerr = np.abs(P.cpu().numpy() - host["pos"]).max()
        assert oerr <= POS_TOL, (call, oerr)
        assert np.abs(V.cpu().numpy() - host["vel"]).max() <= 1e-2, call
    c.close()


@pytest.mark.gpu
def test_noalloc_reports_a_particle_outside_the_grid():
    """A particle whose stencil would leave the grid is skipped and reported as MPM_ERR_OOB (the
    kernel range-checks it and touches no memory for it); the next call starts from a clear
    status and succeeds on particles inside the grid."""
    import __graft_entry__ as g

    g.build()
    from genesis_gb300 import _lib

    lib = _lib.load()
    sc, mats = _scene_and_materials(3)
    pos = torch.tensor([[0.5, 0.5, 0.5], [0.45, 0.5, 0.5], [1.5, 0.5, 0.5]], device="cuda")
    n = 3
    V = torch.zeros((n, 3), device="cuda")
    Cm = torch.zeros((n, 3, 3), device="cuda")
    F = torch.eye(3, device="cuda").repeat(n, 1, 1).contiguous()
    Jp = torch.ones(n, device="cuda")
    mat_arr = (_lib.MpmMaterial * 1)(mats[0])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    r = lib.mpm_substeps_noalloc(ctypes.byref(sc), mat_arr, 1, n, pos.data_ptr(), V.data_ptr(), Cm.data_ptr(),
                                 F.data_ptr(), Jp.data_ptr(), None, None, 2, stream)
    assert _lib.STATUS_NAMES.get(r) == "MPM_ERR_OOB", (r, lib.mpm_noalloc_last_error())
    assert b"left the grid" in lib.mpm_noalloc_last_error()
    inside = pos[:2].contiguous()
    r = lib.mpm_substeps_noalloc(ctypes.byref(sc), mat_arr, 1, 2, inside.data_ptr(), V.data_ptr(), Cm.data_ptr(),
                                 F.data_ptr(), Jp.data_ptr(), None, None, 2, stream)
    assert r == 0, lib.mpm_noalloc_last_error()
    assert torch.isfinite(inside).all()
