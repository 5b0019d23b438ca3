"""The CUDA substep against golden vectors from the reference's own MPM code (tests/golden/).

Float32 kernels vs float64 reference execution, same inputs: grid mass/momentum after the
first P2G within 1e-5 relative (L2); particle state after 1 and 10 substeps, after 5 substeps
with force fields, after 3 with rigid coupling (with and without CPIC) and after 4 with a tool
within the float32 tolerances stated below."""

import os

import numpy as np
import pytest
import torch

from capi_helpers import Ctx, material_record, scene_record

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# after several substeps, relative to the largest entry: float32 accumulation against float64 (the
# measured errors are about 10x smaller: pos 4e-8, vel 2e-6, C 3e-6, F 2e-6, Jp 4e-6)
GOLDEN_STATE_TOL = (("pos", 1e-6), ("vel", 2e-5), ("C", 3e-5), ("F", 2e-5), ("Jp", 5e-5))


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__ as g

    g.build()
    from genesis_gb300 import _lib

    gd = np.load(os.path.join(GOLDEN, "substep_small.npz"))
    dt, density, p_size, lx, ly, lz, ux, uy, uz, eps = gd["scene"]
    n = len(gd["in/pos"])
    mats = [material_record(_lib, 0, p[0], p[1], p[2], p[3], p[9], None, p[4], p[5], p[6], p[7], p[8])
            for p in gd["material_params"]]
    c = Ctx([scene_record(_lib, dt, n, (lx, ly, lz), (ux, uy, uz), density, p_size, eps)], mats)
    mat = gd["in/mat"]
    for m in range(len(mats)):
        idx = np.nonzero(mat == m)[0]
        assert np.all(np.diff(idx) == 1)
        c.add(0, 1, int(idx[0]), gd["in/pos"][idx], m)
    yield c, gd, n
    c.close()


def _load(c, gd, n):
    from genesis_gb300 import _lib

    c.set_state(0, 1, pos=gd["in/pos"], vel=gd["in/vel"], C=gd["in/C"], F=gd["in/F"], Jp=gd["in/Jp"],
                active=np.ones(n, np.uint8))
    c.set_field(_lib.FIELD_ACTU, 0, 1, 0, gd["in/actu"][None, :, None])
    c.set_field(_lib.FIELD_MUSCLE_DIR, 0, 1, 0, gd["in/mdir"][None])


def test_first_p2g_grid_matches_reference(ctx):
    c, gd, n = ctx
    _load(c, gd, n)
    c.call("mpm_substep_pre", c.stream)
    g = c.grid(0)
    ref = gd["grid1"]
    assert np.linalg.norm(g[..., 3] - ref[..., 3]) <= 1e-5 * np.linalg.norm(ref[..., 3])
    assert np.linalg.norm(g[..., :3] - ref[..., :3]) <= 1e-5 * np.linalg.norm(ref[..., :3])
    c.call("mpm_substep_grid_op", c.stream)
    c.call("mpm_substep_post", c.stream)
    s = c.get_state(0, 1, n)
    for k, tol in (("pos", 1e-6), ("vel", 1e-4), ("C", 1e-3), ("F", 1e-5), ("Jp", 1e-5)):
        ref = gd["out1/" + k]
        err = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
        assert err <= tol, (k, err)
    assert c.status()[0] == 0


def test_ten_substeps_match_reference(ctx):
    c, gd, n = ctx
    _load(c, gd, n)
    c.substeps(10)
    s = c.get_state(0, 1, n)
    errs = {}
    for k, tol in GOLDEN_STATE_TOL:
        ref = gd["out10/" + k]
        errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
        assert errs[k] <= tol, (k, errs[k])
    print("ten-substep golden errors (relative to max):", {k: f"{v:.2e}" for k, v in errs.items()})
    assert c.status()[0] == 0


def test_force_fields_match_reference(ctx):
    """Constant, Wind, Point, Drag, Vortex and Turbulence fields in the CUDA grid op against five
    substeps of the reference's own grid-op and force-field code (tests/golden/force_fields.npz)."""
    from genesis_gb300 import _lib
    from test_golden_oracle import _golden_fields

    c, _, n = ctx
    gf = np.load(os.path.join(GOLDEN, "force_fields.npz"))
    fields = _golden_fields(gf)
    recs = (_lib.MpmForceField * len(fields))(*[f.to_c() for f in fields])
    c.call("mpm_set_force_fields", len(fields), recs)
    try:
        _load(c, gf, n)
        c.substeps(5)
        s = c.get_state(0, 1, n)
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gf["out5/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        print("force-field golden errors (relative to max):", {k: f"{v:.2e}" for k, v in errs.items()})
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_force_fields", 0, None)


def test_rigid_coupling_matches_reference(ctx, oracle):
    """The CUDA grid op's rigid coupling (sphere, tilted plane, voxel-SDF box) against three substeps
    of the reference's own rigid-collision, SDF and geometry code (tests/golden/rigid_coupling.npz):
    particle state, and the reaction on each geom (the reference accumulates it into the link's
    cfrc_coupling with the opposite sign)."""
    _check_rigid_golden(ctx, oracle, "rigid_coupling.npz", cpic=False)


def test_cpic_matches_reference(ctx, oracle):
    """CPIC in the CUDA P2G and G2P (particle-side normals, cells across a geom skipped, their
    velocity replaced by the particle's own rigid collision) against three substeps of the
    reference's own p2g/g2p with enable_CPIC (tests/golden/cpic_coupling.npz: a sphere, a tilted
    plane and a thin tilted plate through one of the blocks)."""
    _check_rigid_golden(ctx, oracle, "cpic_coupling.npz", cpic=True)


def _check_rigid_golden(ctx, oracle, fixture, cpic):
    import ctypes

    from genesis_gb300 import _lib
    from test_golden_oracle import _golden_colliders

    c, _, n = ctx
    gr = np.load(os.path.join(GOLDEN, fixture))
    oracle.clear_sdf_grids()
    cols = _golden_colliders(oracle, gr)
    oracle.clear_sdf_grids()
    recs = []
    for col, sid in cols:
        if col.sdf is not None:
            g = col.sdf
            vals = np.ascontiguousarray(g.values, np.float32)
            grads = np.ascontiguousarray(g.grads, np.float32)
            res = np.asarray(vals.shape, np.int32)
            T = np.ascontiguousarray(g.T_mesh_to_sdf, np.float64)
            out = ctypes.c_int32()
            c.call("mpm_add_sdf_grid", res.ctypes.data, vals.ctypes.data, grads.ctypes.data, T.ctypes.data,
                   float(g.cell_size), float(g.sdf_max), ctypes.byref(out))
            sid = out.value
        recs.append(col.to_c(sid))
    if cpic:
        c.call("mpm_enable_cpic", len(recs), c.stream)
    arr = (_lib.MpmCollider * len(recs))(*recs)
    c.call("mpm_set_colliders", len(recs), arr)
    try:
        _load(c, gr, n)
        c.substeps(3)
        s = c.get_state(0, 1, n)
        forces = np.zeros((len(recs), 6))
        c.call("mpm_get_collider_forces", forces.ctypes.data, 1, c.stream)
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gr["out3/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        ferr = np.abs(forces[:, :3] + gr["link_force"]).max() / np.abs(gr["link_force"]).max()
        terr = np.abs(forces[:, 3:] + gr["link_torque"]).max() / np.abs(gr["link_torque"]).max()
        print(fixture, "golden errors:", {k: f"{v:.2e}" for k, v in errs.items()}, f"force {ferr:.2e}",
              f"torque {terr:.2e}")
        assert ferr <= 1e-5 and terr <= 5e-5, (ferr, terr)
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_colliders", 0, None)
        if cpic:
            c.call("mpm_enable_cpic", 0, c.stream)


def test_tool_coupling_matches_reference(ctx, oracle):
    """The CUDA grid op's tool coupling and the library's tool motion (advect onto the floor
    height) against substeps of the reference's own Mesh, ToolEntity and geometry code
    (tests/golden/tool_coupling.npz): particle state and the tool's final pose."""
    import ctypes

    from genesis_gb300 import _lib
    from test_golden_oracle import _golden_tool

    c, _, n = ctx
    gt = np.load(os.path.join(GOLDEN, "tool_coupling.npz"))
    n_steps = int(gt["n_steps"])
    oracle.clear_sdf_grids()
    col, _ = _golden_tool(oracle, gt)
    oracle.clear_sdf_grids()
    g = col.sdf
    vals = np.ascontiguousarray(g.values, np.float32)
    res = np.asarray(vals.shape, np.int32)
    T = np.ascontiguousarray(g.T_mesh_to_sdf, np.float64)
    out = ctypes.c_int32()
    c.call("mpm_add_sdf_grid", res.ctypes.data, vals.ctypes.data, None, T.ctypes.data, float(g.cell_size),
           float(g.sdf_max), ctypes.byref(out))
    arr = (_lib.MpmCollider * 1)(col.to_c(out.value))
    c.call("mpm_set_colliders", 1, arr)
    try:
        _load(c, gt, n)
        c.substeps(n_steps)
        s = c.get_state(0, 1, n)
        pose = np.zeros((1, 7))
        c.call("mpm_get_collider_poses", pose.ctypes.data, c.stream)
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gt[f"out{n_steps}/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        perr = np.abs(pose[0] - np.r_[gt["tool/pos_out"], gt["tool/quat_out"]]).max()
        print("tool-coupling golden errors:", {k: f"{v:.2e}" for k, v in errs.items()}, f"pose {perr:.2e}")
        assert perr <= 1e-6, perr
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_colliders", 0, None)


def test_particle_coupling_matches_reference(ctx):
    """The CUDA grid op's SPH and PBD coupling (mean velocity of the other solver's particles in a
    node's cell, momentum change given back, PBD free particles only) against substeps of the
    reference's own grid op and SpatialHasher (tests/golden/particle_coupling.npz): particle state
    and both sets' velocities."""
    c, _, n = ctx
    gp = np.load(os.path.join(GOLDEN, "particle_coupling.npz"))
    n_steps = int(gp["n_steps"])
    dev = lambda a, dt=torch.float32: torch.tensor(np.asarray(a), dtype=dt, device="cuda").contiguous()  # noqa: E731
    sets = {}
    for kind, name in ((0, "sph"), (1, "pbd")):
        sets[name] = (dev(gp[f"{name}/pos"]), dev(gp[f"{name}/vel"]), dev(gp[f"{name}/mass"]),
                      dev(gp[f"{name}/free"], torch.uint8) if name == "pbd" else None)
    torch.cuda.synchronize()
    try:
        for kind, name in ((0, "sph"), (1, "pbd")):
            p, v, m, f = sets[name]
            c.call("mpm_set_coupled_particles", kind, len(p), p.data_ptr(), v.data_ptr(), m.data_ptr(),
                   None if f is None else f.data_ptr(), c.stream)
        _load(c, gp, n)
        c.substeps(n_steps)
        s = c.get_state(0, 1, n)
        torch.cuda.synchronize()
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gp[f"out{n_steps}/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        verr = {name: np.abs(sets[name][1].double().cpu().numpy() - gp[f"{name}/vel_out"]).max() for name in sets}
        print("particle-coupling golden errors:", {k: f"{v:.2e}" for k, v in errs.items()},
              {k: f"{v:.2e}" for k, v in verr.items()})
        assert max(verr.values()) <= 2e-5, verr
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_coupled_particles", 0, 0, None, None, None, None, c.stream)
        c.call("mpm_set_coupled_particles", 1, 0, None, None, None, None, c.stream)


def test_particle_constraints_match_reference(ctx):
    """The CUDA spring update after G2P (particles attached to two moving links and to their start
    positions, some released midway) against substeps of the reference's own constraint kernels
    (tests/golden/particle_constraints.npz)."""
    c, _, n = ctx
    gc = np.load(os.path.join(GOLDEN, "particle_constraints.npz"))
    n_steps = int(gc["n_steps"])
    dev = lambda a, dt=torch.float32: torch.tensor(np.asarray(a), dtype=dt, device="cuda").contiguous()  # noqa: E731

    def poses(k):
        return np.ascontiguousarray(np.concatenate([gc["link_pos"][k], gc["link_quat"][k]], -1)[None], np.float32)

    _load(c, gc, n)
    p0 = poses(0)
    c.call("mpm_set_link_poses", p0.shape[1], p0.ctypes.data)
    keep = []
    for i in range(3):
        start, mask = int(gc[f"set{i}/start"]), dev(gc[f"set{i}/mask"], torch.uint8)
        li = int(gc[f"set{i}/link"])
        lp, lq = dev(gc["link_pos"][0, max(li, 0)][None]), dev(gc["link_quat"][0, max(li, 0)][None])
        keep += [mask, lp, lq]
        torch.cuda.synchronize()
        c.call("mpm_set_particle_constraints", 0, 1, start, mask.numel(), mask.data_ptr(),
               float(gc[f"set{i}/stiffness"]), li, lp.data_ptr(), lq.data_ptr(), c.stream)
    rm = dev(gc["remove/mask"], torch.uint8)
    torch.cuda.synchronize()
    try:
        for step in range(n_steps):
            pk = poses(step + 1)
            c.call("mpm_set_link_poses", pk.shape[1], pk.ctypes.data)
            if step == int(gc["remove/before"]):
                c.call("mpm_remove_particle_constraints", 0, 1, int(gc["remove/start"]), rm.numel(), rm.data_ptr(),
                       c.stream)
            c.substeps(1)
        s = c.get_state(0, 1, n)
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gc[f"out{n_steps}/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        print("particle-constraint golden errors:", {k: f"{v:.2e}" for k, v in errs.items()})
        assert c.status()[0] == 0
    finally:
        ones = dev(np.ones(n), torch.uint8)
        torch.cuda.synchronize()
        c.call("mpm_remove_particle_constraints", 0, 1, 0, n, ones.data_ptr(), c.stream)


def _custom_acc_batched(pos, vel, t, i):
    """tests/golden/make_golden.py custom_acc, batched over nodes (torch [M, 3])."""
    return torch.stack([-3.0 * (pos[:, 1] - 0.125) - 0.5 * vel[:, 0] + 2.0 * t,
                        3.0 * (pos[:, 0] - 0.125) - 0.5 * vel[:, 1],
                        -1.0 + 0.3 * pos[:, 2] * (1.0 + t)], 1)


def test_custom_force_field_matches_reference(ctx):
    """A Custom force field between Drag and Constant, applied through the staged grid op
    (mpm_substep_grid_stage: stage 1 gravity + Drag, the user function on the node velocities of
    the buffer mpm_grid_nodes exposes, stage 2 Constant, stage 3 boundary) against five substeps of
    the reference's grid op calling the same function (tests/golden/custom_field.npz)."""
    import ctypes

    from genesis_gb300 import _lib
    from genesis_gb300 import force_fields as ff
    from genesis_gb300.solver import _DeviceArray

    c, _, n = ctx
    gc = np.load(os.path.join(GOLDEN, "custom_field.npz"))
    n_steps = int(gc["n_steps"])
    fields = [ff.Drag(linear=0.8, quadratic=0.4), ff.Constant(direction=(0.0, 1.0, 0.5), strength=1.5)]
    for f in fields:
        f.activate()
    recs = (_lib.MpmForceField * 2)(*[f.to_c() for f in fields])
    c.call("mpm_set_force_fields", 2, recs)
    dt = float(gc["scene"][0])
    eps = float(np.finfo(np.float32).eps)
    try:
        _load(c, gc, n)
        ptr, count = ctypes.c_void_p(), ctypes.c_int64()
        for step in range(n_steps):
            c.call("mpm_substep_pre", c.stream)
            c.call("mpm_substep_grid_stage", 1, 0, 1, c.stream)
            c.call("mpm_grid_nodes", ctypes.byref(ptr), ctypes.byref(count))
            nn = int(count.value)
            if step == 0:
                pos = torch.empty((nn, 3), dtype=torch.float32, device="cuda")
                scene = torch.empty((nn,), dtype=torch.int32, device="cuda")
                c.call("mpm_grid_node_positions", pos.data_ptr(), scene.data_ptr(), c.stream)
            torch.cuda.synchronize()
            nodes = torch.as_tensor(_DeviceArray(ptr.value, (nn, 4)), device="cuda")
            sel = torch.nonzero((scene >= 0) & (nodes[:, 3] > eps)).squeeze(1)
            v = nodes.index_select(0, sel)[:, :3]
            nodes[sel, :3] = v + _custom_acc_batched(pos.index_select(0, sel), v, step * dt, -1) * dt
            torch.cuda.synchronize()
            c.call("mpm_substep_grid_stage", 2, 1, 2, c.stream)
            c.call("mpm_substep_grid_stage", 3, 0, 0, c.stream)
            c.call("mpm_substep_post", c.stream)
        s = c.get_state(0, 1, n)
        errs = {}
        for k, tol in GOLDEN_STATE_TOL:
            ref = gc[f"out{n_steps}/" + k]
            errs[k] = np.abs(s[k] - ref).max() / max(1.0, np.abs(ref).max())
            assert errs[k] <= tol, (k, errs[k])
        print("custom-field golden errors:", {k: f"{v:.2e}" for k, v in errs.items()})
        assert c.status()[0] == 0
    finally:
        c.call("mpm_set_force_fields", 0, None)
