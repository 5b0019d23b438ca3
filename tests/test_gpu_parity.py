"""GPU parity: the CUDA substep (through the Genesis-style API / C ABI) against the FP64 CPU oracle.

Tolerances: grid mass and momentum per substep within 1e-5 relative
(L2 over the grid) of the FP64 oracle started from the same state; particle positions within
1e-4 * domain (domain = 1 m) after 100 substeps.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GRID_RTOL = 1e-5
POS_TOL = 1e-4


@pytest.fixture(scope="module")
def gs():
    import __graft_entry__ as g

    g.build()
    import genesis_gb300 as gs

    gs.init(backend=gs.gpu, seed=0)
    return gs


def jittered_lattice(center, size, spacing, dx, seed):
    n = [max(1, round(size / spacing))] * 3
    lo = np.asarray(center) - size / 2 + 0.5 * spacing
    axes = [np.linspace(lo[d], lo[d] + (n[d] - 1) * spacing, n[d]) for d in range(3)]
    p = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    return p + rng.uniform(-0.25 * dx, 0.25 * dx, size=p.shape)


def c1_scene(gs, n_envs=0, seed=7, size=0.2, cpic=False):
    """Config 1: grid 64^3 over the unit cube, elastic cube of side 0.2 at (0.5,0.5,0.4),
    2 particles per cell per axis, jitter +-0.25 dx, E=3e5 nu=0.2 rho=1000, dt=2e-4."""
    dx = 1 / 64
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4, substeps=1),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                          particle_size=1 / 128, enable_CPIC=cpic),
    )
    mat = gs.materials.MPM.Elastic(E=3e5, nu=0.2, rho=1000, sampler="regular")
    cube = scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.5, 0.5, 0.4), size=(size,) * 3))
    scene.build(n_envs=n_envs)
    pos = jittered_lattice((0.5, 0.5, 0.4), size, 1 / 128, dx, seed)
    assert len(pos) == cube.n_particles
    cube.set_particles_pos(torch.tensor(pos, dtype=torch.float32, device="cuda"))
    return scene, cube, mat


def oracle_state(st, b=0, mats_idx=None):
    n = st.pos.shape[1]
    d = lambda t: t[b].detach().double().cpu().numpy()  # noqa: E731
    return dict(pos=d(st.pos), vel=d(st.vel), C=d(st.C), F=d(st.F), Jp=d(st.Jp),
                mat=np.zeros(n, np.int32) if mats_idx is None else mats_idx,
                active=st.active[b].cpu().numpy().astype(bool))


def oracle_scene_for(O, solver):
    return O.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                        upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                        particle_size=solver.particle_size)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a)


def test_c1_grid_mass_momentum_per_substep(gs, oracle):
    scene, cube, mat = c1_scene(gs)
    solver = scene.sim.mpm_solver
    sc = oracle_scene_for(oracle, solver)
    om = oracle.from_c_material(mat.to_c(0))
    checked = 0
    for k in range(1, 31):
        st = solver.get_state()
        solver.substep_pre_coupling()
        g = solver.get_grid(0).double().cpu().numpy()
        _, og, _ = oracle.run(sc, [om], oracle_state(st), 1, want_grid=True)
        assert rel_l2(g[..., 3], og[..., 3]) <= GRID_RTOL, k
        if np.linalg.norm(og[..., :3]) > 0:
            assert rel_l2(g[..., :3], og[..., :3]) <= GRID_RTOL, k
            checked += 1
        else:
            assert np.abs(g[..., :3]).max() < 1e-6
        solver.couple()
        solver.substep_post_coupling()
    assert checked >= 25
    solver.check_state()


def test_c1_positions_after_100_substeps(gs, oracle):
    scene, cube, mat = c1_scene(gs)
    solver = scene.sim.mpm_solver
    st0 = solver.get_state()
    for _ in range(100):
        scene.step()
    st = solver.get_state()
    ref, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))],
                           oracle_state(st0), 100)
    err = np.abs(st.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st.vel[0].double().cpu().numpy() - ref["vel"]).max() < 1e-3
    assert np.abs(st.F[0].double().cpu().numpy() - ref["F"]).max() < 1e-4


MULTI = [
    ("Liquid", {"E": 1e5, "nu": 0.3}, (0.3, 0.3, 0.25)),
    ("Sand", {}, (0.7, 0.3, 0.25)),
    ("Snow", {}, (0.3, 0.7, 0.25)),
    ("ElastoPlastic", {}, (0.7, 0.7, 0.25)),
    ("Muscle", {}, (0.5, 0.5, 0.6)),
    ("Elastic", {"model": "neohooken"}, (0.5, 0.5, 0.25)),
]


def test_multimaterial_scene(gs, oracle):
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4, substeps=5),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                          particle_size=1 / 128),
    )
    ents = []
    for name, kw, c in MULTI:
        m = getattr(gs.materials.MPM, name)(sampler="regular", **kw)
        ents.append((scene.add_entity(material=m, morph=gs.morphs.Box(pos=c, size=(0.1, 0.1, 0.1))), m))
    scene.build()
    muscle = ents[4][0]
    muscle.set_actuation(0.5)
    solver = scene.sim.mpm_solver
    st0 = solver.get_state()
    for _ in range(20):
        scene.step()
    st = solver.get_state()
    mats = solver._unique_materials()
    oms = [oracle.from_c_material(m.to_c(0)) for m in mats]
    mat_idx = np.concatenate([np.full(e.n_particles, m.idx, np.int32) for e, m in ents])
    s = oracle_state(st0, mats_idx=mat_idx)
    s["actu"] = np.concatenate([np.full(e.n_particles, 0.5 if e is muscle else 0.0) for e, _ in ents])
    ref, _, _ = oracle.run(oracle_scene_for(oracle, solver), oms, s, 100)
    err = np.abs(st.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    jp_err = np.abs(st.Jp[0].double().cpu().numpy() - ref["Jp"]).max()
    assert jp_err < 1e-3, jp_err


def test_envs_are_independent_copies(gs):
    scene, cube, _ = c1_scene(gs, n_envs=3, size=0.1)
    for _ in range(20):
        scene.step()
    p = cube.get_particles_pos()
    assert p.shape == (3, cube.n_particles, 3)
    assert (p[1] - p[0]).abs().max().item() < 1e-6
    assert (p[2] - p[0]).abs().max().item() < 1e-6


def test_state_roundtrip_and_reset(gs):
    scene, cube, _ = c1_scene(gs, size=0.1)
    for _ in range(5):
        scene.step()
    s = scene.get_state()
    for _ in range(5):
        scene.step()
    after = cube.get_particles_pos().clone()
    scene.reset(s)
    for _ in range(5):
        scene.step()
    assert (cube.get_particles_pos() - after).abs().max().item() < 1e-6
    scene.reset()
    s0 = scene.get_state()
    assert torch.equal(s0.solvers_state[0].pos, scene._init_state.pos)


def test_inactive_entity_is_frozen(gs):
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)),
    )
    a = scene.add_entity(material=gs.materials.MPM.Elastic(), morph=gs.morphs.Box(pos=(0.3, 0.5, 0.5), size=(0.1,) * 3))
    b = scene.add_entity(material=gs.materials.MPM.Elastic(), morph=gs.morphs.Box(pos=(0.7, 0.5, 0.5), size=(0.1,) * 3))
    scene.build()
    b.deactivate()
    pb = None
    for i in range(10):
        scene.step()
        if i == 0:
            pb = b.get_particles_pos().clone()
    assert torch.equal(b.get_particles_pos(), pb)
    assert not b.get_particles_active().any()
    assert (a.get_particles_vel()[:, 2] < 0).all()


def test_nan_position_raises(gs):
    scene, cube, _ = c1_scene(gs, size=0.1)
    pos = cube.get_particles_pos().clone()
    pos[0, 0] = float("nan")
    cube.set_particles_pos(pos)
    with pytest.raises(gs.GenesisException, match="NaN"):
        scene.step()


def test_particle_outside_the_grid_raises_and_the_context_recovers(gs):
    """A particle put outside the grid (its stencil would leave it) is never scattered or gathered:
    the keying's bounds check flags it, scene.step() raises, and once it is back inside the scene
    steps on and matches a scene that never left (the status word is read and cleared)."""
    scene, cube, _ = c1_scene(gs, size=0.1)
    ref, ref_cube, _ = c1_scene(gs, size=0.1)
    pos0 = cube.get_particles_pos().clone()
    bad = pos0.clone()
    bad[3] = torch.tensor([1.5, 0.5, 0.5], device="cuda")
    cube.set_particles_pos(bad)
    with pytest.raises(gs.GenesisException, match="left the simulation grid"):
        scene.step()
    cube.set_particles_pos(pos0)
    for _ in range(5):
        scene.step()
        ref.step()
    assert (cube.get_particles_pos() - ref_cube.get_particles_pos()).abs().max().item() < 1e-6


def test_graph_and_split_paths_agree(gs):
    sa, ca, _ = c1_scene(gs, size=0.1)
    sb, cb, _ = c1_scene(gs, size=0.1)
    sa.sim.mpm_solver.substeps(16)
    for _ in range(16):
        sb.sim.substep()
    assert (ca.get_particles_pos() - cb.get_particles_pos()).abs().max().item() < 1e-6


def test_mass_conservation_and_touched_nodes(gs):
    scene, cube, mat = c1_scene(gs)
    solver = scene.sim.mpm_solver
    solver.substep_pre_coupling()
    g = solver.get_grid(0)
    m_expected = cube.n_particles * np.float32(np.float32(solver.particle_volume) * np.float32(mat.rho))
    assert abs(g[..., 3].double().sum().item() - m_expected) <= 1e-5 * m_expected
    solver.couple()
    solver.substep_post_coupling()


def test_render_fields_and_visual_vertices(gs):
    """update_render_fields (mpm_solver.py:780-803): positions / velocities / active flags in the
    reference order, the nowhere point for inactive particles, and visual vertices as the
    support-weighted sum of the current particle positions."""
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)),
        vis_options=gs.options.VisOptions(n_support_neighbors=6),
    )
    a = scene.add_entity(material=gs.materials.MPM.Elastic(), morph=gs.morphs.Box(pos=(0.3, 0.5, 0.5), size=(0.1,) * 3))
    b = scene.add_entity(material=gs.materials.MPM.Elastic(), morph=gs.morphs.Box(pos=(0.7, 0.5, 0.5), size=(0.1,) * 3))
    rng = np.random.default_rng(1)
    va = 0.3 + rng.uniform(-0.04, 0.04, size=(50, 3)) + np.array([0.0, 0.2, 0.2])
    a.set_vverts(va)
    b.set_vverts(np.array([0.7, 0.5, 0.5]) + rng.uniform(-0.04, 0.04, size=(20, 3)))
    scene.build()
    solver = scene.sim.mpm_solver
    solver.update_render_fields()
    vr = solver.vverts_render["pos"][0].cpu().numpy()
    assert np.abs(vr[:50] - va).max() < 1e-5  # at rest the supports reproduce the vertices
    b.deactivate()
    for _ in range(5):
        scene.step()
    solver.update_render_fields()
    st = solver.get_state()
    pr = solver.particles_render
    na = a.n_particles
    assert torch.equal(pr["pos"][0, :na], st.pos[0, :na])
    assert torch.equal(pr["vel"][0], st.vel[0])
    assert torch.equal(pr["active"][0], st.active[0])
    nowhere = torch.tensor([-2333333.0, -6666666.0, -5201314.0], device="cuda")
    assert torch.equal(pr["pos"][0, na:], nowhere.expand(b.n_particles, 3))
    idx = torch.as_tensor(np.concatenate([a._vvert_support_idx, b._vvert_support_idx]), device="cuda").long()
    w = torch.as_tensor(np.concatenate([a._vvert_support_w, b._vvert_support_w]), device="cuda")
    want = (st.pos[0][idx] * w[..., None]).sum(1)
    assert torch.allclose(solver.vverts_render["pos"][0], want, atol=1e-6)
    act = solver.vverts_render["active"][0]
    assert act[:50].all() and not act[50:].any()


def _quat_rotate(q, v):
    w, x, y, z = q
    R = np.array([[x * x + w * w - y * y - z * z, 2 * x * y - 2 * w * z, 2 * x * z + 2 * w * y],
                  [2 * w * z + 2 * x * y, w * w - x * x + y * y - z * z, -2 * w * x + 2 * y * z],
                  [-2 * w * y + 2 * x * z, 2 * w * x + 2 * y * z, w * w - x * x - y * y + z * z]])
    return v @ R.T


def test_particle_constraints_match_spring_update(gs, oracle):
    """apply_particle_constraints (mpm_solver.py:1099-1128) after G2P: the target follows the link
    (attachment offset in the link frame), dv = dt (-k (x - target) - 2 sqrt(k m) v) / m."""
    scene, cube, mat = c1_scene(gs, size=0.1)
    solver = scene.sim.mpm_solver
    n = cube.n_particles
    q0 = np.array([np.cos(0.2), 0.0, 0.0, np.sin(0.2)])  # rotation about z
    p0 = np.array([0.5, 0.5, 0.4])
    solver.set_link_poses(p0[None], q0[None])
    mask = torch.zeros(n, dtype=torch.bool)
    mask[::3] = True
    k = 2e3
    cube.set_particle_constraints(mask, 0, k)
    st0 = solver.get_state()
    x0 = st0.pos[0].double().cpu().numpy()
    local = _quat_rotate(q0 * np.array([1, -1, -1, -1]), x0 - p0)
    # move the link, then one substep
    q1 = np.array([np.cos(0.25), 0.0, np.sin(0.25) * 0.6, np.sin(0.25) * 0.8])
    p1 = np.array([0.52, 0.49, 0.41])
    solver.set_link_poses(p1[None], q1[None])
    scene.step()
    st1 = solver.get_state()
    ref, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))], oracle_state(st0), 1)
    m_real = np.float32(np.float32(solver.particle_volume) * np.float32(mat.rho)) / 1e3
    target = _quat_rotate(q1, local) + p1
    v = ref["vel"].copy()
    sel = mask.numpy()
    dv = 2e-4 * (-k * (ref["pos"][sel] - target[sel]) - 2 * np.sqrt(k * m_real) * v[sel]) / m_real
    v[sel] += dv
    got = st1.vel[0].double().cpu().numpy()
    assert np.abs(got - v).max() <= 1e-4 * max(1.0, np.abs(v).max()), np.abs(got - v).max()
    assert np.abs(dv).max() > 1e-3  # the spring acted
    cube.remove_particle_constraints()
    st1b = solver.get_state()
    scene.step()
    st2 = solver.get_state()
    ref2, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))],
                            oracle_state(st1b), 1)
    assert np.abs(st2.vel[0].double().cpu().numpy() - ref2["vel"]).max() <= 1e-4


def test_emitter_activates_droplets_and_recycles(gs):
    """Emitter.emit (emitter.py:56-194): the next pool particles take the droplet's positions and
    the emission velocity and become active; the pool index wraps when it would overflow."""
    from genesis_gb300.emitter import z_up_frame

    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=4e-3, substeps=10),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)),
    )
    em = scene.add_emitter(material=gs.materials.MPM.Liquid(), max_particles=3000)
    scene.build()
    ent = em.entity
    assert not ent.get_particles_active().any()
    # the droplet length from speed * dt (1.5 * 4e-3 = 6 mm) is below the particle size: the first
    # call only accumulates it (emitter.py:110-116), the second emits
    em.emit("sphere", 0.08, pos=(0.5, 0.5, 0.6), direction=(0.0, 0.0, -1.0), speed=1.5)
    assert not ent.get_particles_active().any()
    em.emit("sphere", 0.08, pos=(0.5, 0.5, 0.6), direction=(0.0, 0.0, -1.0), speed=1.5)
    act = ent.get_particles_active()
    n1 = int(act.sum())
    assert n1 > 100 and act[:n1].all()
    vel = ent.get_particles_vel()[:n1]
    assert torch.allclose(vel, torch.tensor([0.0, 0.0, -1.5], device="cuda").expand(n1, 3))
    pos = ent.get_particles_pos()[:n1].cpu().numpy()
    assert np.linalg.norm(pos - np.array([0.5, 0.5, 0.6]), axis=1).max() <= 0.04 + 1e-6
    for _ in range(3):
        scene.step()
    assert (ent.get_particles_pos()[:n1, 2] < 0.6 - 0.04).any()
    # square nozzle along +x with a rotation: positions sit in the rotated frame
    em.emit("square", 0.05, droplet_length=0.03, pos=(0.3, 0.5, 0.5), direction=(1.0, 0.0, 0.0), theta=0.3,
            speed=0.5)
    n2 = int(ent.get_particles_active().sum()) - n1
    assert n2 > 0
    p2 = ent.get_particles_pos()[n1:n1 + n2].double().cpu().numpy()
    R = z_up_frame(np.array([1.0, 0.0, 0.0]), gs.EPS)
    local = (p2 - np.array([0.3, 0.5, 0.5])) @ R
    assert np.abs(local[:, 2]).max() <= 0.015 + 1e-6  # droplet length along the direction
    while em._next_particle != 0:  # keep emitting until the pool wraps
        em.emit("sphere", 0.08, droplet_length=0.05, pos=(0.5, 0.5, 0.6), direction=(0.0, 0.0, -1.0), speed=1.5)
    assert int(ent.get_particles_active().sum()) <= 3000


def test_rigid_colliders_match_oracle(gs, oracle):
    """MPM <-> rigid coupling in the grid op (legacy_coupler.py:166-218, 284-347) with kinematic
    sphere / rotated box / tilted plane colliders, one of them moving and spinning: particle state
    and the reaction force on each collider against the FP64 oracle."""
    from genesis_gb300.coupling import Collider

    scene, cube, mat = c1_scene(gs, size=0.12)
    solver = scene.sim.mpm_solver
    st = solver.get_state()
    vel = st.vel.clone()
    vel[..., 2] = -2.0
    st.vel = vel
    solver.set_state(0, st)
    cols = [
        Collider("sphere", pos=(0.46, 0.5, 0.30), radius=0.04, lin_vel=(0.2, 0.0, 0.1), ang_vel=(0.0, 3.0, 0.0),
                 coup_friction=0.4),
        Collider("box", pos=(0.55, 0.52, 0.30), quat=(np.cos(0.3), 0.0, np.sin(0.3), 0.0),
                 half_extents=(0.03, 0.04, 0.015), coup_restitution=0.3, coup_softness=0.004),
        Collider("plane", pos=(0.5, 0.5, 0.325), quat=(np.cos(0.1), np.sin(0.1), 0.0, 0.0), normal=(0.0, 0.0, 1.0)),
    ]
    solver.set_colliders(cols)
    st0 = solver.get_state()
    n_sub = 60
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    f_gpu = solver.get_collider_forces()
    oracle.set_colliders([c.to_c() for c in cols])
    try:
        ref, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))],
                               oracle_state(st0), n_sub)
        f_ref = oracle.collider_forces(len(cols))
    finally:
        oracle.set_colliders([])
    assert np.abs(f_ref[:, :3]).max(axis=1).min() > 1.0, f_ref  # every collider was hit
    err = np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() < 5e-3
    assert np.allclose(f_gpu, f_ref, rtol=2e-3, atol=2e-3 * np.abs(f_ref).max()), (f_gpu, f_ref)
    solver.set_colliders([])


def _box_sdf(half):
    half = np.asarray(half)

    def f(p):
        q = np.abs(p) - half
        return np.linalg.norm(np.maximum(q, 0.0), axis=-1) + np.minimum(q.max(axis=-1), 0.0)

    return f


def test_sdf_grid_and_tool_colliders_match_oracle(gs, oracle):
    """A rigid geom given by an SDF grid (utils/sdf.py: trilinear value and gradient, proxy outside
    the grid) and a moving, spinning tool entity (tool_entity/mesh.py: voxel SDF, central-difference
    normal, friction and softness, pose advanced every substep) in the grid op: particle state,
    the rigid geom's reaction and the tool's pose after 60 substeps against the FP64 oracle."""
    from genesis_gb300.coupling import Collider, SDFGrid, tool

    scene, cube, mat = c1_scene(gs, size=0.12)
    solver = scene.sim.mpm_solver
    st = solver.get_state()
    vel = st.vel.clone()
    vel[..., 2] = -2.0
    st.vel = vel
    solver.set_state(0, st)
    box = SDFGrid.from_function(_box_sdf((0.03, 0.04, 0.015)), (-0.06,) * 3, (0.06,) * 3, 33)
    knob = SDFGrid.from_function(lambda p: np.linalg.norm(p, axis=-1) - 0.025, (-0.05,) * 3, (0.05,) * 3, 25,
                                 grads=False)
    cols = [
        tool(knob, pos=(0.45, 0.5, 0.31), vel=(0.0, 0.0, 0.5), ang=(0.0, 0.0, 4.0), friction=0.3,
             coup_softness=0.002),
        Collider("sdf", sdf=box, pos=(0.56, 0.52, 0.30), quat=(np.cos(0.3), 0.0, np.sin(0.3), 0.0),
                 coup_friction=0.2, coup_restitution=0.3, coup_softness=0.004),
    ]
    solver.set_colliders(cols)
    st0 = solver.get_state()
    n_sub = 60
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    f_gpu = solver.get_collider_forces()
    pose_gpu = solver.get_collider_poses()
    oracle.clear_sdf_grids()
    ids = [oracle.add_sdf_grid(g.values, g.grads, g.T_mesh_to_sdf, g.cell_size, g.sdf_max) for g in (knob, box)]
    recs = [c.to_c(i) for c, i in zip(cols, ids)]
    o_scene, o_mat = oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))]
    oracle.set_colliders(recs)
    try:
        ref, _, _ = oracle.run(o_scene, o_mat, oracle_state(st0), n_sub)
        f_ref = oracle.collider_forces(len(cols))
        pose_ref = oracle.collider_poses(len(cols))
    finally:
        oracle.set_colliders([])
    free, _, _ = oracle.run(o_scene, o_mat, oracle_state(st0), n_sub)
    oracle.clear_sdf_grids()
    assert np.abs(free["pos"] - ref["pos"]).max() > 5e-3  # both colliders pushed particles
    assert np.abs(f_ref[1, :3]).max() > 1.0, f_ref
    assert np.all(f_ref[0] == 0.0)  # a tool takes no reaction
    err = np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() < 5e-3
    assert np.allclose(f_gpu, f_ref, rtol=2e-3, atol=2e-3 * np.abs(f_ref).max()), (f_gpu, f_ref)
    assert np.abs(pose_gpu - pose_ref).max() < 1e-5, (pose_gpu, pose_ref)
    assert abs(pose_ref[0, 2] - (0.31 + 0.5 * n_sub * solver.substep_dt)) < 1e-9
    solver.set_colliders([])


def test_cpic_thin_blade_matches_oracle(gs, oracle):
    """CPIC (mpm_solver.py:389-411, 445-459; legacy_coupler.py:503-529): a thin static blade through
    an elastic cube that moves into it.  Nodes behind the blade take nothing from a particle in
    P2G and give it its own collided velocity in G2P.  Particle state and the blade's reaction
    against the FP64 oracle; the oracle without CPIC must end elsewhere (CPIC did something)."""
    from genesis_gb300.coupling import Collider

    scene, cube, mat = c1_scene(gs, size=0.12, cpic=True)
    solver = scene.sim.mpm_solver
    st = solver.get_state()
    vel = st.vel.clone()
    vel[..., 0] = 1.0
    vel[..., 2] = -0.5
    st.vel = vel
    solver.set_state(0, st)
    # mid-plane exact in fp32 and 4.9 mm from the nearest node column: every side test is clear-cut
    bx = 0.5 + 5 / 1024
    blade = Collider("box", pos=(bx, 0.5, 0.4), half_extents=(0.0015, 0.15, 0.15), coup_friction=0.3)
    solver.set_colliders([blade])
    st0 = solver.get_state()
    n_sub = 40
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    f_gpu = solver.get_collider_forces()
    sc = oracle_scene_for(oracle, solver)
    om = [oracle.from_c_material(mat.to_c(0))]
    try:
        oracle.set_cpic(True)
        oracle.set_colliders([blade.to_c()])
        ref, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
        f_ref = oracle.collider_forces(1)
        oracle.set_cpic(False)
        oracle.set_colliders([blade.to_c()])
        plain, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
    finally:
        oracle.set_cpic(False)
        oracle.set_colliders([])
    assert f_ref[0, 0] > 100.0, f_ref  # the cube pushes the blade along +x
    assert np.abs(plain["pos"] - ref["pos"]).max() > 20 * POS_TOL
    err = np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() < 5e-3
    assert np.allclose(f_gpu, f_ref, rtol=2e-3, atol=2e-3 * np.abs(f_ref).max()), (f_gpu, f_ref)
    solver.set_colliders([])


def test_sph_pbd_grid_coupling_matches_oracle(gs, oracle):
    """MPM <-> SPH and MPM <-> PBD coupling in the grid op (legacy_coupler.py:404-498) with two
    caller-held particle sets: an SPH slab under an elastic cube moving down and left, a PBD slab
    beside it with every other particle not free.  MPM particle state and both sets' velocities
    after 40 substeps against the FP64 oracle (which finds each node's particles by the cell test
    itself); not-free PBD particles keep their velocity; the uncoupled oracle ends elsewhere."""
    scene, cube, mat = c1_scene(gs, size=0.12)
    solver = scene.sim.mpm_solver
    st = solver.get_state()
    vel = st.vel.clone()
    vel[..., 0] = -0.5
    vel[..., 2] = -1.0
    st.vel = vel
    solver.set_state(0, st)
    dx = 1 / 64
    rng = np.random.default_rng(3)

    def slab(ix, iy, iz, dup_every):  # one particle per node cell (some two), 0.35 dx from the node at most
        g = np.stack(np.meshgrid(ix, iy, iz, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
        g = np.concatenate([g, g[::dup_every]])
        return ((g + rng.uniform(-0.35, 0.35, g.shape)) * dx).astype(np.float32)

    sph = slab(np.arange(28, 37), np.arange(28, 37), np.arange(20, 22), 2)
    pbd = slab(np.arange(26, 28), np.arange(28, 37), np.arange(22, 30), 3)
    free = (np.arange(len(pbd)) % 2).astype(np.uint8)
    dev = lambda a, dt=torch.float32: torch.tensor(a, dtype=dt, device="cuda").contiguous()  # noqa: E731
    sph_pos, sph_vel, sph_m = dev(sph), dev(np.zeros_like(sph)), dev(np.full(len(sph), 2e-3))
    pbd_pos, pbd_vel, pbd_m = dev(pbd), dev(np.tile([0.2, 0.0, 0.0], (len(pbd), 1))), dev(np.full(len(pbd), 1e-3))
    pbd_free = dev(free, torch.uint8)
    solver.set_coupled_particles("sph", sph_pos, sph_vel, sph_m)
    solver.set_coupled_particles("pbd", pbd_pos, pbd_vel, pbd_m, pbd_free)
    st0 = solver.get_state()
    n_sub = 40
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    v_sph, v_pbd = sph_vel.double().cpu().numpy(), pbd_vel.double().cpu().numpy()
    solver.set_coupled_particles("sph")
    solver.set_coupled_particles("pbd")
    sc = oracle_scene_for(oracle, solver)
    om = [oracle.from_c_material(mat.to_c(0))]
    try:
        oracle.set_coupled(0, sph.astype(np.float64), np.zeros((len(sph), 3)), np.full(len(sph), np.float32(2e-3)))
        oracle.set_coupled(1, pbd.astype(np.float64), np.tile([0.2, 0.0, 0.0], (len(pbd), 1)),
                           np.full(len(pbd), np.float32(1e-3)), free)
        ref, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
        r_sph, r_pbd = oracle.coupled_velocities(0), oracle.coupled_velocities(1)
    finally:
        oracle.set_coupled(0)
        oracle.set_coupled(1)
    plain, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
    assert np.abs(plain["pos"] - ref["pos"]).max() > 10 * POS_TOL
    assert np.abs(r_sph).max() > 0.5 and np.abs(r_pbd[free == 1] - [0.2, 0.0, 0.0]).max() > 0.5
    err = np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() < 5e-3
    assert np.abs(v_sph - r_sph).max() < 5e-3, np.abs(v_sph - r_sph).max()
    assert np.abs(v_pbd - r_pbd).max() < 5e-3, np.abs(v_pbd - r_pbd).max()
    assert np.array_equal(v_pbd[free == 0], np.tile([0.2, 0.0, 0.0], ((free == 0).sum(), 1)).astype(np.float32))


def test_force_fields_match_oracle(gs, oracle):
    """Force fields in the grid op (legacy_coupler.py:381-383, engine/force_fields.py): constant,
    wind, point, drag and vortex fields (one left inactive) against the FP64 oracle."""
    ff = gs.force_fields
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4, substeps=1),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                          particle_size=1 / 128),
    )
    mat = gs.materials.MPM.Elastic(E=3e5, nu=0.2, rho=1000, sampler="regular")
    cube = scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.5, 0.5, 0.4), size=(0.12,) * 3))
    fields = [
        ff.Constant(direction=(1.0, 0.5, 0.0), strength=3.0),
        ff.Wind(direction=(0.0, 1.0, 0.0), strength=4.0, radius=0.04, center=(0.5, 0.5, 0.4)),
        ff.Point(strength=-2.0, position=(0.45, 0.55, 0.35), falloff_pow=1.0, flow=0.5),
        ff.Drag(linear=0.8, quadratic=0.3),
        ff.Vortex(center=(0.52, 0.48, 0.0), strength_perpendicular=6.0, strength_radial=1.0, falloff_min=0.02,
                  falloff_max=0.3, damping=0.2),
        ff.Constant(direction=(0.0, 0.0, 1.0), strength=50.0),  # stays inactive
    ]
    for f in fields:
        scene.add_force_field(f)
    scene.build()
    for f in fields[:5]:
        f.activate()
    solver = scene.sim.mpm_solver
    st0 = solver.get_state()
    n_sub = 40
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    oracle.set_force_fields([f.to_c() for f in fields])
    try:
        ref, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))],
                               oracle_state(st0), n_sub)
    finally:
        oracle.set_force_fields([])
    ref_plain, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))],
                                 oracle_state(st0), n_sub)
    assert np.abs(ref["vel"] - ref_plain["vel"]).max() > 1e-2  # the fields act
    assert np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max() <= POS_TOL
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() <= 1e-3
    fields[0].deactivate()
    for f in fields[1:5]:
        f.deactivate()
    st2 = solver.get_state()
    scene.step()
    ref2, _, _ = oracle.run(oracle_scene_for(oracle, solver), [oracle.from_c_material(mat.to_c(0))], oracle_state(st2), 1)
    assert np.abs(solver.get_state().vel[0].double().cpu().numpy() - ref2["vel"]).max() <= 1e-4


def test_noise_and_turbulence_fields_match_oracle(gs, oracle):
    """Turbulence (Perlin noise over numpy-shuffled permutations, force_fields.py:372-421,
    441-544) and Noise (uniform draws per node, component and substep from a counter-based hash,
    force_fields.py:232-259) in the grid op against the FP64 oracle, which restates both (the same
    draws); the fields change the motion, and two noise seeds give different motion."""
    ff = gs.force_fields
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-4, substeps=1),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                          particle_size=1 / 128),
    )
    mat = gs.materials.MPM.Elastic(E=3e5, nu=0.2, rho=1000, sampler="regular")
    scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.5, 0.5, 0.4), size=(0.12,) * 3))
    fields = [ff.Turbulence(strength=30.0, frequency=5, flow=0.3, seed=11), ff.Noise(strength=20.0, seed=7)]
    for f in fields:
        scene.add_force_field(f)
    scene.build()
    for f in fields:
        f.activate()
    solver = scene.sim.mpm_solver
    st0 = solver.get_state()
    n_sub = 40
    for _ in range(n_sub):
        scene.step()
    st1 = solver.get_state()
    sc = oracle_scene_for(oracle, solver)
    om = [oracle.from_c_material(mat.to_c(0))]
    other = [fields[0].to_c(), ff.Noise(strength=20.0, seed=8).to_c()]
    other[1].active = 1
    try:
        oracle.set_force_fields([f.to_c() for f in fields])
        ref, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
        oracle.set_force_fields(other)
        ref_seed, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
    finally:
        oracle.set_force_fields([])
    ref_plain, _, _ = oracle.run(sc, om, oracle_state(st0), n_sub)
    assert np.abs(ref["vel"] - ref_plain["vel"]).max() > 1e-2  # the fields act
    assert np.abs(ref["vel"] - ref_seed["vel"]).max() > 1e-3   # the noise seed matters
    assert np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max() <= POS_TOL
    assert np.abs(st1.vel[0].double().cpu().numpy() - ref["vel"]).max() <= 1e-3


def test_full_size_conservation_properties(gs):
    """The ~1M-particle three-material scene of the benchmark (too large for the oracle in a test):
    size-independent properties.  Without gravity and away from the walls, total mass on the grid
    equals the particles' mass every substep, total linear momentum is conserved (APIC transfers
    and internal stresses exchange momentum only), and the re-sort keeps every particle (the state
    is a permutation: ids and positions round-trip)."""
    import bench

    scene, ents, spacing = bench.build_c2_scene(gs)
    solver = scene.sim.mpm_solver
    solver.set_gravity((0.0, 0.0, 0.0))
    st = solver.get_state()
    n = st.pos.shape[1]
    rng = np.random.default_rng(5)
    vel = torch.tensor(rng.normal(scale=0.05, size=(1, n, 3)), dtype=torch.float32, device="cuda")
    st.vel = vel
    solver.set_state(0, st)
    masses = []
    for e in ents:
        masses += [np.float32(np.float32(solver.particle_volume) * np.float32(e.material.rho))] * e.n_particles
    m = torch.tensor(np.array(masses, dtype=np.float64), device="cuda")
    p0 = (m[:, None] * st.vel[0].double()).sum(0)
    for k in range(20):
        solver.substeps(5)
        s = solver.get_state()
        p = (m[:, None] * s.vel[0].double()).sum(0)
        assert torch.linalg.norm(p - p0).item() <= 2e-4 * (m.sum().item() * 0.05), (k, p, p0)
    solver.substep_pre_coupling()
    g = solver.get_grid(0)
    assert abs(g[..., 3].double().sum().item() - m.sum().item()) <= 1e-5 * m.sum().item()
    solver.couple()
    solver.substep_post_coupling()
    s = solver.get_state()
    assert s.active[0].all() and torch.isfinite(s.pos).all()


@pytest.mark.parametrize("shape,size,p_size", [
    ("box", (0.2, 0.13, 0.07), 0.01), ("box", (0.3, 0.3, 0.3), 1.0 / 128), ("sphere", 0.1, 0.0034),
    ("sphere", 0.045, 0.01), ("cylinder", (0.05, 0.2), 0.0071)])
def test_device_regular_sampling_equals_host(gs, shape, size, p_size):
    """mpm_sample_regular reproduces the host 'regular' samplers (utils/particle.py:180-278)
    bit for bit after the float32 rounding every particle position goes through."""
    from genesis_gb300 import morphs

    pos = (0.5, 0.47, 0.52)
    if shape == "box":
        host = morphs.box_to_particles(p_size, pos, size, "regular")
    elif shape == "sphere":
        host = morphs.sphere_to_particles(p_size, pos, size, "regular")
    else:
        host = morphs.cylinder_to_particles(p_size, pos, size[0], size[1], "regular")
    dev = morphs.sample_regular_on_device(shape, pos, size, p_size).cpu().numpy()
    assert dev.shape == host.shape
    assert np.array_equal(dev, host.astype(np.float32))


def test_reference_scenario_cube_settles_on_coupled_plane(gs):
    """The MPM part of the reference's tests/test_deformable_physics.py::test_deformable_parallel,
    through the drop-in API: an Elastic(rho=200) cube in MPMOptions(lower_bound=(0.5, -0.1, -0.05),
    upper_bound=(0.7, 0.1, 0.3)) dropped on the coupled ground plane (Rigid needs_coup,
    coup_friction=0; a kinematic plane collider here), 2 envs, dt 2e-3 x 10 substeps, 1500 steps:
    the cube moved, stays above the ground (z > -1e-5) and comes to rest (|v| <= 1e-4)."""
    from genesis_gb300.coupling import Collider

    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-3, substeps=10),
        mpm_options=gs.options.MPMOptions(lower_bound=(0.5, -0.1, -0.05), upper_bound=(0.7, 0.1, 0.3)),
    )
    cube = scene.add_entity(material=gs.materials.MPM.Elastic(rho=200),
                            morph=gs.morphs.Box(pos=(0.6, 0.0, 0.1), size=(0.1, 0.1, 0.1)))
    scene.build(n_envs=2)
    scene.sim.mpm_solver.set_colliders([Collider("plane", pos=(0.0, 0.0, 0.0), normal=(0.0, 0.0, 1.0),
                                                 coup_friction=0.0)])
    init = cube.get_particles_pos().clone()
    for _ in range(1500):
        scene.step()
    final = cube.get_particles_pos()
    assert (init - final).abs().sum().item() > 0.1
    assert final[..., 2].min().item() > -1e-5
    assert cube.get_particles_vel().abs().max().item() <= 1e-4
    scene.sim.mpm_solver.set_colliders([])


def test_reference_scenario_particle_constraints_follow_link(gs):
    """The reference's tests/test_deformable_physics.py::test_mpm_particle_constraints through the
    drop-in API, with the fixed rigid box as a kinematic link (its pose given by set_link_poses):
    bbox selection gives an (n_envs, n_particles) mask that selects some but not all particles; the
    attached particles follow the link moved by +0.2 m in x over 30 steps of 20 substeps.

    Stiffness 1e4 instead of the reference test's 1e5: with particle mass 1e-3 kg and substep 1e-4 s,
    k = 1e5 gives dt * sqrt(k / m) = 1, where the explicit critically damped update of
    apply_particle_constraints has an eigenvalue of magnitude 1.62 for a lone particle; this run then
    diverges (NaN), so only the grid coupling of the reference's own sampling can keep it bounded.
    At k = 1e4 (dt * sqrt(k / m) = 0.32) the update is stable."""
    from genesis_gb300.coupling import Collider

    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-3, substeps=20),
        mpm_options=gs.options.MPMOptions(lower_bound=(-1.0, -1.0, 0.0), upper_bound=(1.0, 1.0, 1.0),
                                          grid_density=64),
    )
    cube = scene.add_entity(material=gs.materials.MPM.Elastic(E=5e4, nu=0.3, rho=1000),
                            morph=gs.morphs.Box(pos=(0.0, 0.0, 0.35), size=(0.15, 0.15, 0.15)))
    scene.build(n_envs=2)
    solver = scene.sim.mpm_solver
    solver.set_colliders([Collider("plane", normal=(0.0, 0.0, 1.0))])  # gs.morphs.Plane()
    box_pos = np.array([0.0, 0.0, 0.55])
    solver.set_link_poses(box_pos[None], np.array([[1.0, 0.0, 0.0, 0.0]]))
    mask = cube.get_particles_in_bbox((-0.08, -0.08, 0.41), (0.08, 0.08, 0.44))
    assert tuple(mask.shape) == (2, cube.n_particles)
    assert mask.any() and not mask.all()
    cube.set_particle_constraints(mask, 0, stiffness=1e4)
    x0 = cube.get_particles_pos()[:, mask[0], 0].mean()
    solver.set_link_poses((box_pos + np.array([0.2, 0.0, 0.0]))[None], np.array([[1.0, 0.0, 0.0, 0.0]]))
    for _ in range(30):
        scene.step()
    moved = cube.get_particles_pos()[:, mask[0], 0].mean() - x0
    assert moved.item() > 0.2 * 0.3, moved.item()
    solver.set_colliders([])


@pytest.mark.parametrize("material", ["Liquid", "Sand", "Snow", "Elastic"])
def test_reference_scenario_fluid_emitter(gs, material):
    """The MPM cases of the reference's tests/test_hybrid.py::test_fluid_emitter through the drop-in
    API (2 envs; the ground plane as a coupled plane collider, the URDF wheel left out: no URDF
    parser on this path): emit_omni, then five circular droplets with a step after each, then one
    more step.  The reference checks that this runs; here also that particles were emitted, every
    active one is finite and inside the domain, and no NaN was flagged."""
    from genesis_gb300.coupling import Collider

    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=4e-3, substeps=10),
        mpm_options=gs.options.MPMOptions(lower_bound=(0.0, -1.5, 0.0), upper_bound=(1.0, 1.5, 4.0)),
    )
    emitter = scene.add_emitter(material=getattr(gs.materials.MPM, material)(), max_particles=5000)
    scene.build(n_envs=2)
    scene.sim.mpm_solver.set_colliders([Collider("plane", normal=(0.0, 0.0, 1.0))])
    emitter.emit_omni()
    for _ in range(5):
        emitter.emit(droplet_shape="circle", droplet_size=0.25)
        scene.step()
    scene.step()
    ent = emitter.entity
    act = ent.get_particles_active()
    assert act.shape[0] == 2 and int(act[0].sum()) > 0
    pos = ent.get_particles_pos()[act]
    assert torch.isfinite(pos).all()
    lo = torch.tensor([0.0, -1.5, 0.0], device="cuda")
    hi = torch.tensor([1.0, 1.5, 4.0], device="cuda")
    assert ((pos >= lo) & (pos <= hi)).all()
    scene.sim.mpm_solver.set_colliders([])


@pytest.mark.parametrize("n_envs", [0, 2])
def test_reference_scenario_muscle_groups(gs, n_envs):
    """The MPM case of the reference's tests/test_deformable_physics.py::test_muscle through the
    drop-in API, with a box for the worm mesh (no mesh loader on this path): Muscle(E=5e5, nu=0.45,
    rho=1e4, n_groups=4) split into the reference's four groups (upper/lower x fore/hind), fiber
    direction +y, a coupled ground plane with coup_friction 5, 200 steps of sinusoidal actuation of
    group 3.  Every particle carries its group's actuation; the actuated body ends elsewhere than
    an unactuated one; no NaN."""
    from genesis_gb300.coupling import Collider

    def run(actuate):
        scene = gs.Scene(
            sim_options=gs.options.SimOptions(dt=5e-4, substeps=10, gravity=(0, 0, -9.8)),
            mpm_options=gs.options.MPMOptions(lower_bound=(-1.0, -1.0, -0.2), upper_bound=(1.0, 1.0, 1.0)),
        )
        worm = scene.add_entity(material=gs.materials.MPM.Muscle(E=5e5, nu=0.45, rho=10000.0, n_groups=4),
                                morph=gs.morphs.Box(pos=(0.3, 0.3, 0.03), size=(0.06, 0.3, 0.05)))
        scene.build(n_envs=n_envs) if n_envs > 0 else scene.build()
        scene.sim.mpm_solver.set_colliders([Collider("plane", normal=(0.0, 0.0, 1.0), coup_friction=5.0)])
        pos = worm.get_state().pos[0].cpu().numpy()
        lo, hi = pos.min(0), pos.max(0)
        rng_ = hi - lo
        upper = pos[:, 2] > lo[2] + rng_[2] * 0.3
        fore = pos[:, 1] < lo[1] + rng_[1] * 0.6
        group = np.zeros(len(pos), dtype=np.int64)
        group[upper & ~fore] = 1
        group[~upper & fore] = 2
        group[~upper & ~fore] = 3
        worm.set_muscle(muscle_group=group, muscle_direction=np.tile([0.0, 1.0, 0.0], (len(pos), 1)))
        scene.reset()
        for i in range(200):
            a = np.array([0.0, 0.0, 0.0, (1.0 if actuate else 0.0) * (0.5 + np.sin(0.005 * np.pi * i))])
            worm.set_actuation(np.tile(a, (n_envs, 1)) if n_envs > 1 else a)
            if i == 0:
                actu = worm.get_particles_actu()
                actu = actu[0] if n_envs > 1 else actu
                want = np.where(group == 3, a[3], 0.0)
                assert np.allclose(actu.cpu().numpy(), want), "each particle takes its group's actuation"
            scene.step()
        out = worm.get_particles_pos()
        scene.sim.mpm_solver.set_colliders([])
        return out[0] if n_envs > 1 else out

    act = run(True)
    rest = run(False)
    assert torch.isfinite(act).all() and torch.isfinite(rest).all()
    assert (act - rest).abs().max().item() > 1e-3
    assert act[:, 2].min().item() > -1e-3


def test_entity_queries_frame_and_checkpoints(gs):
    """find_closest_particle (particle_entity.py:716-743), get_frame (mpm_entity.py:305-352),
    visual index ranges and the entity checkpoints of pending targets (particle_entity.py:371-403)."""
    scene, cube, _ = c1_scene(gs, n_envs=2, size=0.1)
    for _ in range(3):
        scene.step()
    pos = cube.get_particles_pos()
    idx = cube.find_closest_particle(pos[:, 7])
    assert idx.shape == (2,) and (idx == 7).all()
    B, n = 2, cube.n_particles
    bufs = [torch.empty((B, n, 3), device="cuda"), torch.empty((B, n, 3), device="cuda"),
            torch.empty((B, n, 3, 3), device="cuda"), torch.empty((B, n, 3, 3), device="cuda"),
            torch.empty((B, n), device="cuda"), torch.empty((B, n), dtype=torch.int64, device="cuda")]
    cube.get_frame(None, *bufs)
    st = cube.get_state()
    for got, want in zip(bufs, (st.pos, st.vel, st.C, st.F, st.Jp, st.active)):
        assert torch.equal(got, want.reshape(got.shape).to(got.dtype))
    assert cube.vvert_start == 0 and cube.vvert_end == cube.n_vverts and cube.n_vfaces == 0
    cube.init_ckpt()
    cube.set_velocity(torch.tensor([0.0, 0.0, 1.0], device="cuda"))
    cube.save_ckpt("a")
    scene.step()  # applies and clears the pending target
    cube.load_ckpt("a")
    scene.step()  # applies it again
    v = cube.get_particles_vel()
    assert v[..., 2].mean().item() > 0.5


def test_scene_checkpoint_roundtrip_and_lookup(gs, tmp_path):
    """Scene.save_checkpoint / load_checkpoint (scene.py:1402-1446) through the numpy dump of the
    solver (base_solver.py:63-126): a run continued from a loaded checkpoint follows the run that
    wrote it; entity lookup by name; the gradient members of the Solver protocol need a scene
    built with requires_grad."""
    scene, cube, _ = c1_scene(gs, n_envs=2, size=0.1)
    for _ in range(5):
        scene.step()
    path = tmp_path / "ckpt.pkl"
    scene.save_checkpoint(path)
    t_saved = scene.t
    for _ in range(5):
        scene.step()
    after = cube.get_particles_pos().clone()
    for _ in range(3):
        scene.step()
    scene.load_checkpoint(path)
    assert scene.t == t_saved
    for _ in range(5):
        scene.step()
    assert (cube.get_particles_pos() - after).abs().max().item() < 1e-5
    assert scene.get_entity(cube.name) is cube and cube.name in scene.entity_names
    assert np.allclose(scene.gravity[0], (0.0, 0.0, -9.81))
    with pytest.raises(gs.GenesisException, match="requires_grad"):
        scene.sim.mpm_solver.reset_grad()


def test_mesh_morph_entity_steps(gs, tmp_path):
    """An MPM entity from a mesh file (gs.morphs.Mesh) samples like the Box of the same cube, steps,
    and takes the mesh vertices as its visual vertices."""
    from test_api_host import _cube_obj

    obj = tmp_path / "cube.obj"
    _cube_obj(obj, half=0.05)
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-4),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1)))
    mat = gs.materials.MPM.Elastic(sampler="regular")
    ent = scene.add_entity(material=mat, morph=gs.morphs.Mesh(file=str(obj), pos=(0.5, 0.5, 0.4), euler=(0, 0, 30)))
    ref = gs.morphs.Box(size=(0.1, 0.1, 0.1), pos=(0.5, 0.5, 0.4), euler=(0, 0, 30)).sample(ent.particle_size, "regular")
    assert ent.n_particles == len(ref)
    ent.set_vverts(ent.morph.visual_vertices())
    scene.build()
    for _ in range(10):
        scene.step()
    p = ent.get_particles_pos()
    assert torch.isfinite(p).all() and (p[:, 2] < 0.4).any()
    assert ent.n_vverts == 8


@pytest.mark.parametrize("substeps", [1, 10])
def test_reference_scenario_rigid_mpm_legacy_coupling(gs, substeps):
    """tests/test_hybrid.py::test_rigid_mpm_legacy_coupling through the collider API: a light rigid
    box (rho = 1, 0.2 m, resting on the ground at y = -0.25) beside a 0.3 m liquid block; 100 substeps
    of 4e-4 s as 100 steps of 1 substep or 10 steps of 10.  The box is the host's rigid body: after
    every step its velocity takes the particles' reaction force (get_collider_forces, summed over the
    step's substeps) with gravity balanced by the ground and Coulomb friction against it (mu = 1, the
    rigid material default); the MPM side sees it as a moving box collider.  As in the reference, the
    liquid pushes the box towards -y, with either step size."""
    from genesis_gb300.coupling import Collider

    dt = 4e-4
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=dt * substeps, substeps=substeps),
        mpm_options=gs.options.MPMOptions(lower_bound=(-0.5, -1.0, 0.0), upper_bound=(0.5, 1.0, 1.0)),
    )
    scene.add_entity(material=gs.materials.MPM.Liquid(), morph=gs.morphs.Box(pos=(0.0, 0.0, 0.2), size=(0.3, 0.3, 0.3)))
    scene.build()
    solver = scene.sim.mpm_solver
    mass, mu_ground, g = 1.0 * 0.2 ** 3, 1.0, 9.81
    pos = np.array([0.0, -0.25, 0.1])
    vel = np.zeros(3)
    pushed = 0.0
    for _ in range(100 // substeps):
        solver.set_colliders([Collider("box", pos=tuple(pos), half_extents=(0.1, 0.1, 0.1), lin_vel=tuple(vel))])
        scene.step()
        f = solver.get_collider_forces()[0, :3] / substeps  # mean force over the step's substeps
        pushed = min(pushed, f[1])
        h = dt * substeps
        fh = f[:2].copy()
        vh = vel[:2] + h * fh / mass
        speed = np.linalg.norm(vh)
        dv_fric = h * mu_ground * g  # ground friction (normal force m g) brakes the sliding speed
        vel[:2] = 0.0 if speed <= dv_fric else vh * (1.0 - dv_fric / speed)
        pos[:2] += h * vel[:2]
    solver.check_state()
    assert pushed < 0.0  # the liquid pushed the box towards -y
    assert pos[1] + 0.25 < 0.0, pos


def test_custom_force_field_through_scene_api(gs):
    """force_fields.Custom through scene.add_force_field: a Custom field returning the Constant
    field's acceleration reproduces the run with that Constant field (same trajectory within float
    rounding: the library adds acc dt with a fused multiply-add, torch in two steps), both between
    the same Drag fields; the user function sees the simulation time of each substep; a scene with
    a Custom field also steps through the split phases (scene.sim.substep)."""
    ff = gs.force_fields
    direction, strength = np.array([1.0, 0.5, 0.0]) / np.linalg.norm([1.0, 0.5, 0.0]), 3.0
    seen_t = []

    def as_constant(pos, vel, t, i):
        seen_t.append(t)
        assert i == -1 and pos.shape == vel.shape and pos.shape[1] == 3
        return torch.tensor(direction * strength, dtype=torch.float32, device=pos.device).expand_as(pos)

    def run(middle):
        scene = gs.Scene(
            sim_options=gs.options.SimOptions(dt=2e-3, substeps=10),
            mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                              particle_size=1 / 128),
        )
        mat = gs.materials.MPM.Elastic(E=3e5, nu=0.2, rho=1000, sampler="regular")
        cube = scene.add_entity(material=mat, morph=gs.morphs.Box(pos=(0.5, 0.5, 0.4), size=(0.12,) * 3))
        fields = [ff.Drag(linear=0.8, quadratic=0.3), middle, ff.Drag(linear=0.2, quadratic=0.0)]
        for f in fields:
            scene.add_force_field(f)
        scene.build()
        for f in fields:
            f.activate()
        for _ in range(4):
            scene.step()
        return scene, cube.get_particles_pos().double().cpu().numpy()

    _, ref = run(ff.Constant(direction=tuple(direction), strength=strength))
    scene, got = run(ff.Custom(as_constant))
    assert np.abs(got - ref).max() <= 1e-6, np.abs(got - ref).max()
    assert len(seen_t) == 40 and np.allclose(seen_t, np.arange(40) * 2e-4)
    z0 = got[:, 2].mean()
    scene.sim.substep()  # split phases: pre, the staged grid op, post
    assert len(seen_t) == 41 and abs(seen_t[-1] - 40 * 2e-4) < 1e-12
    assert np.isfinite(z0)


def test_tool_entity_through_scene_api(gs, tmp_path):
    """A tool entity through the reference's API (scene.add_entity(morph=gs.morphs.Mesh(...),
    material=gs.materials.Tool(...)), set_velocity / set_position before a step, get_state) pushing
    an elastic block: the same run as the tool given through the collider API with the entity's
    SDF grid; the pose advances by vel * dt every substep and stops at ToolOptions.floor_height;
    with two environments, tools moving apart leave the two blocks in different places."""
    from test_api_host import _cube_obj

    from genesis_gb300 import coupling

    obj = tmp_path / "cube.obj"
    _cube_obj(obj, half=1.0)
    n_steps, dt, substeps = 6, 2e-3, 10

    def make(n_envs=0, tool=True):
        scene = gs.Scene(sim_options=gs.options.SimOptions(dt=dt, substeps=substeps),
                         mpm_options=gs.options.MPMOptions(lower_bound=(0.0, -0.5, 0.0), upper_bound=(1.0, 1.0, 0.55)),
                         tool_options=gs.options.ToolOptions(floor_height=0.02))
        t = None
        if tool:
            t = scene.add_entity(morph=gs.morphs.Mesh(file=str(obj), scale=0.1, pos=(0.3, 0.16, 0.1)),
                                 material=gs.materials.Tool(friction=2.0))
        block = scene.add_entity(morph=gs.morphs.Box(lower=(0.2, 0.2, 0.05), upper=(0.4, 0.35, 0.15)),
                                 material=gs.materials.MPM.Elastic(rho=500, sampler="regular"))
        scene.build(n_envs=n_envs)
        return scene, t, block

    scene, tool, block = make()
    tool.set_velocity(vel=(0.0, 1.0, -0.5))
    for _ in range(n_steps):
        scene.step()
    got = block.get_particles_pos().double().cpu().numpy()
    st = tool.get_state()
    t_end = n_steps * dt
    want = np.array([0.3, 0.16 + t_end, max(0.1 - 0.5 * t_end, 0.02)])
    assert np.abs(st.pos[0].double().cpu().numpy() - want).max() < 1e-5, st.pos
    assert np.allclose(st.vel[0].cpu().numpy(), (0.0, 1.0, -0.5))

    ref_scene, _, ref_block = make(tool=False)
    ref_scene.sim.mpm_solver.set_colliders([coupling.tool(tool.sdf, pos=(0.3, 0.16, 0.1), vel=(0.0, 1.0, -0.5),
                                                         friction=2.0, coup_softness=0.01, floor_height=0.02)])
    for _ in range(n_steps):
        ref_scene.step()
    ref = ref_block.get_particles_pos().double().cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-6, np.abs(got - ref).max()
    moved = np.abs(got - block.init_particles).max()
    assert moved > 1e-3  # the tool pushed the block

    # the floor stops it: 0.1 - 50 * t > 0.02 fails after 1.6 ms
    tool.set_velocity(vel=(0.0, 0.0, -50.0))
    scene.step()
    assert abs(tool.get_state().pos[0, 2].item() - 0.02) < 1e-6

    scene2, tool2, block2 = make(n_envs=2)
    tool2.set_velocity(vel=[[0.0, 1.0, 0.0], [0.0, -1.0, 0.0]])
    for _ in range(n_steps):
        scene2.step()
    p = block2.get_particles_pos().double().cpu().numpy()
    assert np.abs(p[0] - p[1]).max() > 1e-3
    s2 = tool2.get_state().pos.double().cpu().numpy()
    assert abs(s2[0, 1] - (0.16 + t_end)) < 1e-5 and abs(s2[1, 1] - (0.16 - t_end)) < 1e-5
