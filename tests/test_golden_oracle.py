"""Pin the CPU oracle against golden vectors produced by executing the reference's own MPM code
(tests/golden/make_golden.py): material updates and full substeps (P2G grid, G2P state)."""

import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _mat(O, p, rho=1000.0):
    t, fl, mu, lam, alpha, yl, yh, vm, st = p[:9]
    return O.make_material(int(t), mu, lam, rho, 0.0 if int(t) == 2 else 1.0, alpha, yl, yh, vm, st, int(fl))


def test_materials_match_reference_functions(oracle):
    g = np.load(os.path.join(GOLDEN, "materials.npz"))
    names = sorted({k.split("/")[0] for k in g.files})
    assert len(names) == 9
    for name in names:
        m = _mat(oracle, g[f"{name}/params"])
        moduli = abs(m.lam) + 2 * abs(m.mu) + m.stiffness
        for i in range(len(g[f"{name}/F_tmp"])):
            Fn, jn, P = oracle.material_update(m, g[f"{name}/F_tmp"][i], g[f"{name}/Jp"][i], g[f"{name}/actu"][i],
                                               g[f"{name}/mdir"][i])
            assert np.allclose(Fn, g[f"{name}/F_new"][i], rtol=1e-9, atol=1e-10), (name, i)
            assert abs(jn - g[f"{name}/Jp_new"][i]) <= 1e-9 * max(1, abs(jn)), (name, i)
            assert np.abs(P - g[f"{name}/stress"][i]).max() <= 1e-9 * moduli, (name, i)


@pytest.fixture(scope="module")
def small():
    return np.load(os.path.join(GOLDEN, "substep_small.npz"))


def _oracle_inputs(O, g):
    dt, density, p_size, lx, ly, lz, ux, uy, uz, eps = g["scene"]
    sc = O.make_scene(dt, lower_bound=(lx, ly, lz), upper_bound=(ux, uy, uz), grid_density=density,
                      particle_size=p_size, eps=eps)
    mats = [_mat(O, p, p[9]) for p in g["material_params"]]
    n = len(g["in/pos"])
    st = dict(pos=g["in/pos"], vel=g["in/vel"], C=g["in/C"], F=g["in/F"], Jp=g["in/Jp"], mat=g["in/mat"],
              active=np.ones(n, bool), actu=g["in/actu"], mdir=g["in/mdir"])
    return sc, mats, st


def test_one_substep_grid_and_state(oracle, small):
    sc, mats, st = _oracle_inputs(oracle, small)
    out, grid, _ = oracle.run(sc, mats, st, 1, want_grid=True)
    g1 = small["grid1"]
    assert np.linalg.norm(grid[..., 3] - g1[..., 3]) <= 1e-12 * np.linalg.norm(g1[..., 3])
    assert np.linalg.norm(grid[..., :3] - g1[..., :3]) <= 1e-10 * np.linalg.norm(g1[..., :3])
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = small["out1/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), k


def test_ten_substeps_state(oracle, small):
    sc, mats, st = _oracle_inputs(oracle, small)
    out, _, _ = oracle.run(sc, mats, st, 10)
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = small["out10/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max()), k


def _golden_fields(g):
    """The facade's force fields built with the fixture's parameters (genesis_gb300.force_fields
    mirrors the constructors of genesis/engine/force_fields.py)."""
    import genesis_gb300.force_fields as ff

    out = []
    for i, name in enumerate(g["fields"]):
        kw = {k.split("/")[1]: g[k] for k in g.files if k.startswith(f"field{i}/")}
        kw = {k: (tuple(v.tolist()) if v.ndim else (int(v) if k == "seed" else float(v))) for k, v in kw.items()}
        f = getattr(ff, str(name))(**kw)
        f.activate()
        out.append(f)
    return out


def test_force_fields_match_reference_code(oracle):
    """The oracle's force fields (Constant, Wind, Point, Drag, Vortex, Turbulence, applied in order
    after gravity in the grid op) against five substeps of the reference's own grid op and field
    code (tests/golden/force_fields.npz)."""
    g = np.load(os.path.join(GOLDEN, "force_fields.npz"))
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.set_force_fields([f.to_c() for f in _golden_fields(g)])
    try:
        out, grid, _ = oracle.run(sc, mats, st, 1, want_grid=True)
        for k in ("pos", "vel", "C", "F", "Jp"):
            ref = g["out1/" + k]
            assert np.abs(out[k] - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), k
        out5, _, _ = oracle.run(sc, mats, st, 5)
    finally:
        oracle.set_force_fields([])
    plain, _, _ = oracle.run(sc, mats, st, 5)
    assert np.abs(plain["vel"] - g["out5/vel"]).max() > 1e-3  # the fields act on this scene
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g["out5/" + k]
        assert np.abs(out5[k] - ref).max() <= 1e-8 * max(1.0, np.abs(ref).max()), k


def _golden_colliders(O, g):
    """The facade's colliders for the reference geoms of tests/golden/rigid_coupling.npz (sphere,
    tilted plane, rotated box given by its SDF grid), the box grid registered with the oracle."""
    from genesis_gb300.coupling import Collider, SDFGrid

    out = []
    for i, t in enumerate(g["geom_types"]):
        pos, quat, data = g[f"geom{i}/pos"], g[f"geom{i}/quat"], g[f"geom{i}/data"]
        fr, so, re = g[f"geom{i}/coup"]
        kw = dict(pos=tuple(pos), quat=tuple(quat), lin_vel=tuple(g[f"geom{i}/lin_vel"]),
                  ang_vel=tuple(g[f"geom{i}/ang_vel"]), com=tuple(pos), coup_friction=fr, coup_softness=so,
                  coup_restitution=re)
        sid = -1
        if t == "sphere":
            c = Collider("sphere", radius=float(data[0]), **kw)
        elif t == "plane":
            c = Collider("plane", normal=tuple(data), **kw)
        else:
            grid = SDFGrid(values=g["sdf_grid/values"], T_mesh_to_sdf=g["sdf_grid/T"], grads=g["sdf_grid/grads"],
                           cell_size=float(g["sdf_grid/cell_size"]), sdf_max=float(g["sdf_grid/sdf_max"]))
            c = Collider("sdf", sdf=grid, **kw)
            sid = O.add_sdf_grid(grid.values, grid.grads, grid.T_mesh_to_sdf, grid.cell_size, grid.sdf_max)
        out.append((c, sid))
    return out


def test_rigid_coupling_matches_reference_code(oracle):
    """The oracle's rigid coupling (SDF of a sphere, a plane and a voxel-SDF box, influence,
    relative-velocity projection with friction and restitution, reaction on the link) against three
    substeps of the reference's own grid op with its rigid-collision, SDF and geometry code
    (tests/golden/rigid_coupling.npz).  The reference accumulates the reaction into the link's
    cfrc_coupling with the opposite sign of the force the oracle reports."""
    g = np.load(os.path.join(GOLDEN, "rigid_coupling.npz"))
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.clear_sdf_grids()
    cols = _golden_colliders(oracle, g)
    oracle.set_colliders([c.to_c(sid) for c, sid in cols])
    try:
        out, _, _ = oracle.run(sc, mats, st, 3)
        forces = oracle.collider_forces(len(cols))
    finally:
        oracle.set_colliders([])
        oracle.clear_sdf_grids()
    plain, _, _ = oracle.run(sc, mats, st, 3)
    assert np.abs(plain["vel"] - g["out3/vel"]).max() > 1e-3  # the geoms act on this scene
    # both sides run in float64; the remaining differences come from the order of operations
    # (quaternion rotations, normalisations), amplified in C by 4 / dx
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g["out3/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max()), k
    assert np.all(np.abs(g["link_force"]).max(1) > 0)
    assert np.abs(forces[:, :3] + g["link_force"]).max() <= 1e-6 * np.abs(g["link_force"]).max()
    assert np.abs(forces[:, 3:] + g["link_torque"]).max() <= 1e-6 * np.abs(g["link_torque"]).max()


def _golden_tool(O, g):
    """The facade's tool collider for tests/golden/tool_coupling.npz (a rotated box given by a
    values-only SDF grid), the grid registered with the oracle."""
    from genesis_gb300.coupling import SDFGrid, tool

    grid = SDFGrid(values=g["tool_sdf/values"], T_mesh_to_sdf=g["tool_sdf/T"], cell_size=float(g["tool_sdf/cell_size"]),
                   sdf_max=float(g["tool_sdf/sdf_max"]))
    c = tool(grid, pos=tuple(g["tool/pos"]), quat=tuple(g["tool/quat"]), vel=tuple(g["tool/vel"]),
             ang=tuple(g["tool/ang"]), friction=float(g["tool/friction"]), coup_softness=float(g["tool/coup_softness"]),
             floor_height=float(g["tool/floor_height"]))
    return c, O.add_sdf_grid(grid.values, None, grid.T_mesh_to_sdf, grid.cell_size, grid.sdf_max)


def test_tool_coupling_matches_reference_code(oracle):
    """The oracle's tool coupling (voxel-SDF trilinear value, finite-difference normal, collider
    velocity from the next pose, friction and influence) and tool motion (advect with the floor
    boundary) against substeps of the reference's own Mesh, ToolEntity and geometry code
    (tests/golden/tool_coupling.npz): particle state and the tool's final pose."""
    g = np.load(os.path.join(GOLDEN, "tool_coupling.npz"))
    n_steps = int(g["n_steps"])
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.clear_sdf_grids()
    c, sid = _golden_tool(oracle, g)
    oracle.set_colliders([c.to_c(sid)])
    try:
        out, _, _ = oracle.run(sc, mats, st, n_steps)
        pose = oracle.collider_poses(1)[0]
    finally:
        oracle.set_colliders([])
        oracle.clear_sdf_grids()
    plain, _, _ = oracle.run(sc, mats, st, n_steps)
    assert np.abs(plain["vel"] - g[f"out{n_steps}/vel"]).max() > 1e-3  # the tool acts on this scene
    assert g["tool/pos_out"][2] == g["tool/floor_height"]  # the floor stopped the tool
    assert np.abs(pose[:3] - g["tool/pos_out"]).max() <= 1e-12
    assert np.abs(pose[3:] - g["tool/quat_out"]).max() <= 1e-12
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g[f"out{n_steps}/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max()), (k, np.abs(out[k] - ref).max())


def test_cpic_matches_reference_code(oracle):
    """The oracle's CPIC (particle-side normals updated before P2G, cells across a geom skipped in
    P2G, their velocity replaced by the particle's own rigid collision in G2P, with its reaction on
    the link) against three substeps of the reference's own p2g/g2p with enable_CPIC and the
    coupler's mpm_surface_to_particle (tests/golden/cpic_coupling.npz, the rigid-coupling geoms)."""
    g = np.load(os.path.join(GOLDEN, "cpic_coupling.npz"))
    sc, mats, st = _oracle_inputs(oracle, g)
    oracle.clear_sdf_grids()
    cols = _golden_colliders(oracle, g)
    oracle.set_colliders([c.to_c(sid) for c, sid in cols])
    try:
        plain, _, _ = oracle.run(sc, mats, st, 3)
        oracle.set_colliders([c.to_c(sid) for c, sid in cols])
        oracle.set_cpic(True)
        out, _, _ = oracle.run(sc, mats, st, 3)
        forces = oracle.collider_forces(len(cols))
    finally:
        oracle.set_cpic(False)
        oracle.set_colliders([])
        oracle.clear_sdf_grids()
    assert np.abs(plain["vel"] - g["out3/vel"]).max() > 1e-3  # CPIC acts on this scene
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g["out3/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-7 * max(1.0, np.abs(ref).max()), (k, np.abs(out[k] - ref).max())
    assert np.abs(forces[:, :3] + g["link_force"]).max() <= 1e-6 * np.abs(g["link_force"]).max()
    assert np.abs(forces[:, 3:] + g["link_torque"]).max() <= 1e-6 * np.abs(g["link_torque"]).max()


def test_particle_coupling_matches_reference_code(oracle):
    """The oracle's SPH and PBD grid coupling (a node takes the mean velocity of the other solver's
    particles within dx/2 and gives the momentum change back to them; PBD: free particles only)
    against substeps of the reference's own grid op, with the particle sets ordered and looked up
    through the reference's SpatialHasher (tests/golden/particle_coupling.npz)."""
    g = np.load(os.path.join(GOLDEN, "particle_coupling.npz"))
    n_steps = int(g["n_steps"])
    sc, mats, st = _oracle_inputs(oracle, g)
    try:
        oracle.set_coupled(0, g["sph/pos"], g["sph/vel"], g["sph/mass"])
        oracle.set_coupled(1, g["pbd/pos"], g["pbd/vel"], g["pbd/mass"], free=g["pbd/free"])
        out, _, _ = oracle.run(sc, mats, st, n_steps)
        v_sph, v_pbd = oracle.coupled_velocities(0), oracle.coupled_velocities(1)
    finally:
        oracle.set_coupled(0)
        oracle.set_coupled(1)
    plain, _, _ = oracle.run(sc, mats, st, n_steps)
    assert np.abs(plain["vel"] - g[f"out{n_steps}/vel"]).max() > 1e-3  # the sets act on this scene
    assert np.abs(g["sph/vel_out"] - g["sph/vel"]).max() > 1e-2 and np.abs(g["pbd/vel_out"] - g["pbd/vel"]).max() > 1e-2
    for k in ("pos", "vel", "C", "F", "Jp"):
        ref = g[f"out{n_steps}/" + k]
        assert np.abs(out[k] - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max()), (k, np.abs(out[k] - ref).max())
    assert np.abs(v_sph - g["sph/vel_out"]).max() <= 1e-12
    assert np.abs(v_pbd - g["pbd/vel_out"]).max() <= 1e-12


def _quat_rot(q, v):
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    return v @ R.T


def test_particle_constraints_restatement_matches_reference_code(oracle):
    """The spring update the GPU parity tests check against (attachment offset kept in the link
    frame, target following the link, dv = dt (-k (x - target) - 2 sqrt(k m) v) / m after G2P,
    link -1: the start position, released particles untouched), applied between single oracle
    substeps, against the reference's own constraint kernels (tests/golden/particle_constraints.npz)."""
    g = np.load(os.path.join(GOLDEN, "particle_constraints.npz"))
    n_steps = int(g["n_steps"])
    sc, mats, st = _oracle_inputs(oracle, g)
    dt, p_size = g["scene"][0], g["scene"][2]
    m = p_size ** 3 * g["material_params"][:, 9][g["in/mat"]]
    n = len(st["pos"])
    k = np.zeros(n)
    link = np.full(n, -2)
    local = np.zeros((n, 3))
    target = np.zeros((n, 3))
    for i in range(3):
        start, mask = int(g[f"set{i}/start"]), g[f"set{i}/mask"].astype(bool)
        idx = start + np.nonzero(mask)[0]
        li = int(g[f"set{i}/link"])
        k[idx], link[idx], target[idx] = g[f"set{i}/stiffness"], li, st["pos"][idx]
        lp, lq = g["link_pos"][0, max(li, 0)], g["link_quat"][0, max(li, 0)]
        local[idx] = _quat_rot(lq * np.array([1, -1, -1, -1]), st["pos"][idx] - lp)
    st = dict(st)
    for step in range(n_steps):
        if step == int(g["remove/before"]):
            idx = int(g["remove/start"]) + np.nonzero(g["remove/mask"])[0]
            link[idx] = -2
        out, _, _ = oracle.run(sc, mats, st, 1)
        for li in (0, 1):
            sel = link == li
            target[sel] = _quat_rot(g["link_quat"][step + 1, li], local[sel]) + g["link_pos"][step + 1, li]
        sel = link >= -1
        v = out["vel"]
        v[sel] += dt * (-k[sel, None] * (out["pos"][sel] - target[sel]) - 2 * np.sqrt(k[sel] * m[sel])[:, None]
                        * v[sel]) / m[sel, None]
        st.update({key: out[key] for key in ("pos", "vel", "C", "F", "Jp")})
    plain, _, _ = oracle.run(sc, mats, _oracle_inputs(oracle, g)[2], n_steps)
    assert np.abs(plain["vel"] - g[f"out{n_steps}/vel"]).max() > 1e-2  # the springs act on this scene
    for key in ("pos", "vel", "C", "F", "Jp"):
        ref = g[f"out{n_steps}/" + key]
        assert np.abs(st[key] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max()), (key, np.abs(st[key] - ref).max())
