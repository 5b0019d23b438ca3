"""Differentiable mode through the scene API (SimOptions(requires_grad=True)): entity inputs that
require grad, scene.step(), scene.get_state() / entity.get_state(), loss.backward().

* The gradient of a loss on the final centre of mass w.r.t. the initial velocity set through
  entity.set_velocity (a scene of an Elastic and a Liquid entity, and one of a Sand and a Snow
  entity, 4 steps x 10 substeps each, with floor contact) against FP64 central differences of the
  CPU oracle (eps = 1e-4), tolerance 2e-2 relative.
* The input pattern of the reference's tests/test_grad.py::test_differentiable_push (two envs, a
  position and a velocity set before the first step, a velocity input every step, a loss on the
  solver state at step 5 and one on the entity state at step 8): inputs that reach a loss get a
  non-zero gradient and the last step's input gets none, here with the liquid entity's velocity
  as the per-step input, and (test_reference_scenario_differentiable_push_with_tool) with the
  reference's own inputs: a tool entity's velocity every step.
* Tool entities in differentiable mode: gradients w.r.t. a tool's start position and velocity
  against FP64 central differences of the oracle; likewise dL/dv0 of a box falling onto kinematic
  rigid colliders (sphere, tilted moving box, SDF grid), and of a box hung on a moving link by
  particle constraints.
* Force fields in differentiable mode: dL/dv0 through seven active built-in fields (Drag, Point,
  Vortex, Turbulence, Noise, Wind, Constant) against FP64 central differences of the oracle running
  the same fields; the forward with fields (two envs, a field switched off mid-run) equals the
  product path; the solver-protocol walk equals autograd with fields.
* The forward of differentiable mode equals the product path on the same scene (1e-4 m).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GRAD_RTOL = 2e-2


@pytest.fixture(scope="module")
def gs():
    import __graft_entry__ as g

    g.build()
    import genesis_gb300 as gs

    gs.init(backend=gs.gpu, seed=0)
    return gs


def _scene(gs, requires_grad=True, n_envs=0, box_z=0.35, fields=()):
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-3, substeps=10, requires_grad=requires_grad),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=32,
                                          particle_size=1.0 / 64),
    )
    box = scene.add_entity(material=gs.materials.MPM.Elastic(E=2e5, nu=0.25, rho=800, sampler="regular"),
                           morph=gs.morphs.Box(pos=(0.45, 0.5, box_z), size=(0.12, 0.12, 0.12)))
    water = scene.add_entity(material=gs.materials.MPM.Liquid(E=1e5, nu=0.3, sampler="regular"),
                             morph=gs.morphs.Box(pos=(0.6, 0.5, 0.22), size=(0.1, 0.1, 0.1)))
    for f in fields:
        scene.add_force_field(f)
    scene.build(n_envs=n_envs)
    return scene, box, water


def _field_set(gs):
    """Every built-in field type, all but the last active; the velocity-dependent ones (Drag, Point
    with flow, Vortex damping, Turbulence with flow) strong enough to change dL/dv0 by tens of %."""
    ff = gs.force_fields
    fields = [
        ff.Drag(linear=10.0, quadratic=10.0),
        ff.Point(strength=-3.0, position=(0.5, 0.5, 0.25), falloff_pow=1.0, flow=2.0),
        ff.Vortex(center=(0.5, 0.5, 0.0), strength_perpendicular=4.0, strength_radial=1.0, falloff_min=0.02,
                  falloff_max=0.5, damping=3.0),
        ff.Turbulence(strength=3.0, frequency=4, flow=1.5, seed=5),
        ff.Noise(strength=2.0, seed=3),
        ff.Wind(direction=(0.0, 1.0, 0.0), strength=2.0, radius=0.1, center=(0.5, 0.5, 0.2)),
        ff.Constant(direction=(1.0, 0.0, 0.0), strength=1.0),
        ff.Constant(direction=(0.0, 0.0, 1.0), strength=40.0),  # stays inactive
    ]
    for f in fields[:-1]:
        f.activate()
    return fields


def _oracle_com_loss(O, scene, ents, v_box, target, n_sub, fields=()):
    solver = scene.sim.mpm_solver
    mats = solver._unique_materials()
    oms = [O.from_c_material(m.to_c(0)) for m in mats]
    pos = np.concatenate([e.init_particles.astype(np.float32).astype(np.float64) for e in ents])
    n = len(pos)
    vel = np.zeros((n, 3))
    nb = ents[0].n_particles
    vel[:nb] = v_box
    st = dict(pos=pos, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
              Jp=np.concatenate([np.full(e.n_particles, float(e.material._default_Jp)) for e in ents]),
              mat=np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents]),
              active=np.ones(n, bool))
    sc = O.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                      upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                      particle_size=solver.particle_size)
    O.set_force_fields([f.to_c() for f in fields])  # also restarts the noise draws' substep counter
    try:
        out, _, _ = O.run(sc, oms, st, n_sub)
    finally:
        O.set_force_fields([])
    com = out["pos"][:nb].mean(0)
    return float(((com - target) ** 2).sum())


def test_grad_of_initial_velocity_matches_fp64_central_differences(gs, oracle):
    """The box starts 1 cm above the floor boundary moving down at 1.5 m/s, so its lower layers hit
    the boundary during the 40 substeps: the gradient goes through the contact, not only through
    free flight."""
    scene, box, water = _scene(gs, box_z=0.165)
    v0 = np.array([0.4, -0.3, -1.5])
    target = np.array([0.52, 0.47, 0.3])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    box.set_velocity(v)
    steps = 4
    for _ in range(steps):
        scene.step()
    st = box.get_state()
    loss = ((st.pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    n_sub = steps * scene.substeps
    ref_loss = _oracle_com_loss(oracle, scene, [box, water], v0, target, n_sub)
    assert abs(loss.item() - ref_loss) <= 1e-4 * max(ref_loss, 1e-6) + 1e-8, (loss.item(), ref_loss)
    eps = 1e-4
    fd = np.zeros(3)
    for k in range(3):
        e = np.zeros(3)
        e[k] = eps
        fd[k] = (_oracle_com_loss(oracle, scene, [box, water], v0 + e, target, n_sub)
                 - _oracle_com_loss(oracle, scene, [box, water], v0 - e, target, n_sub)) / (2 * eps)
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)


def test_force_field_gradients_match_fp64_central_differences(gs, oracle):
    """dL/dv0 of the box thrown onto the floor through seven active force fields (and one inactive)
    against FP64 central differences of the oracle with the same fields; without the fields the
    differences move by more than 10%, so the fields' Jacobians are what the check resolves."""
    fields = _field_set(gs)
    scene, box, water = _scene(gs, box_z=0.165, fields=fields)
    v0 = np.array([0.4, -0.3, -1.5])
    target = np.array([0.52, 0.47, 0.3])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    box.set_velocity(v)
    steps = 4
    for _ in range(steps):
        scene.step()
    loss = ((box.get_state().pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    n_sub = steps * scene.substeps
    ents = [box, water]
    ref_loss = _oracle_com_loss(oracle, scene, ents, v0, target, n_sub, fields)
    assert abs(loss.item() - ref_loss) <= 1e-4 * max(ref_loss, 1e-6) + 1e-8, (loss.item(), ref_loss)

    def fd(fs):
        eps = 1e-4
        return np.array([(_oracle_com_loss(oracle, scene, ents, v0 + eps * np.eye(3)[k], target, n_sub, fs)
                          - _oracle_com_loss(oracle, scene, ents, v0 - eps * np.eye(3)[k], target, n_sub, fs))
                         / (2 * eps) for k in range(3)])

    fd_ff, fd_plain = fd(fields), fd(())
    assert np.linalg.norm(fd_ff - fd_plain) > 0.1 * np.linalg.norm(fd_ff), (fd_ff, fd_plain)
    assert np.linalg.norm(g - fd_ff) <= GRAD_RTOL * np.linalg.norm(fd_ff), (g, fd_ff)


def test_differentiable_forward_with_force_fields_equals_product_path(gs):
    """Two envs (the noise draws differ per env), every field type, Drag switched off after two
    steps (the fields' substep counter restarts in both forms): the differentiable forward equals
    the product path (1e-4 m), and the backward through it gives a finite gradient."""
    fg, fp = _field_set(gs), _field_set(gs)
    sg, box_g, _ = _scene(gs, requires_grad=True, n_envs=2, fields=fg)
    sp, box_p, _ = _scene(gs, requires_grad=False, n_envs=2, fields=fp)
    v0 = torch.tensor([0.3, 0.1, -0.4], device="cuda", requires_grad=True)
    box_g.set_velocity(v0)
    box_p.set_velocity(v0.detach())
    for k in range(5):
        if k == 2:
            fg[0].deactivate()
            fp[0].deactivate()
        sg.step()
        sp.step()
    a = sg.get_state().solvers_state[0].pos
    b = sp.get_state().solvers_state[0].pos
    assert (a.detach() - b).abs().max().item() <= 1e-4
    assert (a.detach()[0] - a.detach()[1]).abs().max().item() > 1e-6  # the envs' noise differs
    a.mean().backward()
    assert torch.isfinite(v0.grad).all() and v0.grad.abs().max().item() > 0
    sp.sim.mpm_solver.destroy()


def test_plastic_materials_grad_matches_fp64_central_differences(gs, oracle):
    """Sand (Drucker-Prager) and Snow (clamped, hardening) boxes thrown onto the floor boundary, 40
    substeps: the impact deforms them past their yield limits (sand Jp leaves 0, snow Jp leaves 1), so
    the gradient goes through the plastic return mappings and their Jp updates.  dL/dv0 of the sand box against FP64 central
    differences of the oracle (2e-2)."""
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=2e-3, substeps=10, requires_grad=True),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=32,
                                          particle_size=1.0 / 64),
    )
    sand = scene.add_entity(material=gs.materials.MPM.Sand(sampler="regular"),
                            morph=gs.morphs.Box(pos=(0.4, 0.5, 0.16), size=(0.1, 0.1, 0.1)))
    snow = scene.add_entity(material=gs.materials.MPM.Snow(sampler="regular"),
                            morph=gs.morphs.Box(pos=(0.62, 0.5, 0.16), size=(0.1, 0.1, 0.1)))
    scene.build()
    v0 = np.array([0.3, 0.2, -2.0])
    target = np.array([0.45, 0.5, 0.1])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    sand.set_velocity(v)
    snow.set_velocity(torch.tensor([-0.2, 0.0, -2.5], device="cuda"))
    steps = 4
    for _ in range(steps):
        scene.step()
    st = sand.get_state()
    assert (st.Jp[0].abs() > 1e-3).any(), "the sand never flowed plastically"  # Jp != 0: projected
    assert (snow.get_state().Jp[0] != 1.0).any(), "the snow never reached a clamp bound"
    loss = ((st.pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    n_sub = steps * scene.substeps

    def oracle_loss(vb):
        solver = scene.sim.mpm_solver
        ents = [sand, snow]
        oms = [oracle.from_c_material(m.to_c(0)) for m in solver._unique_materials()]
        pos = np.concatenate([e.init_particles.astype(np.float32).astype(np.float64) for e in ents])
        n, ns = len(pos), sand.n_particles
        vel = np.zeros((n, 3))
        vel[:ns] = vb
        vel[ns:] = np.array([-0.2, 0.0, -2.5], np.float32)
        s0 = dict(pos=pos, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
                  Jp=np.concatenate([np.zeros(ns), np.ones(n - ns)]),
                  mat=np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents]),
                  active=np.ones(n, bool))
        sc = oracle.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]),
                               lower_bound=tuple(solver.lower_bound), upper_bound=tuple(solver.upper_bound),
                               grid_density=solver.grid_density, particle_size=solver.particle_size)
        out, _, _ = oracle.run(sc, oms, s0, n_sub)
        return float(((out["pos"][:ns].mean(0) - target) ** 2).sum())

    assert abs(loss.item() - oracle_loss(v0)) <= 1e-3 * loss.item() + 1e-8
    eps = 1e-4
    fd = np.array([(oracle_loss(v0 + eps * np.eye(3)[k]) - oracle_loss(v0 - eps * np.eye(3)[k])) / (2 * eps)
                   for k in range(3)])
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)


def test_reference_push_pattern_gradients(gs):
    """The inputs and losses of test_differentiable_push without its tool entity."""
    scene, box, water = _scene(gs, n_envs=2)
    horizon = 10
    pos_init = torch.tensor([0.45, 0.5, 0.35], device="cuda", requires_grad=True)
    box.set_position(pos_init)
    v_init = torch.tensor([0.0, -1.0, 0.0], device="cuda", requires_grad=True)
    box.set_velocity(v_init)
    goal = torch.tensor([0.5, 0.8, 0.05], device="cuda")
    loss = 0.0
    v_list = []
    for i in range(horizon):
        v_i = torch.tensor([[0.0, 1.0, 0.0], [0.0, 1.0, 0.0]], device="cuda", requires_grad=True)
        water.set_velocity(v_i[:, None, :])
        v_list.append(v_i)
        scene.step()
        if i == horizon // 2:
            mpm = scene.get_state().solvers_state[0]
            loss = loss + torch.pow(mpm.pos[mpm.active == 1] - goal, 2).sum()
        if i == horizon - 2:
            st = box.get_state()
            loss = loss + torch.pow(st.pos - goal, 2).sum()
    loss.backward()
    assert pos_init.grad is not None and (pos_init.grad.abs() > 1e-6).any()
    assert v_init.grad is not None and (v_init.grad.abs() > 1e-6).any()
    for v_i in v_list[: horizon // 2 + 1]:  # the liquid is part of the solver-state loss at step 5
        assert v_i.grad is not None and (v_i.grad.abs() > 1e-7).any()
    assert v_list[-1].grad is None or (v_list[-1].grad.abs() < 1e-7).all()


def test_differentiable_forward_equals_product_path(gs):
    sg, box_g, _ = _scene(gs, requires_grad=True)
    sp, box_p, _ = _scene(gs, requires_grad=False)
    v0 = torch.tensor([0.3, 0.1, -0.4], device="cuda")
    box_g.set_velocity(v0)
    box_p.set_velocity(v0)
    for _ in range(5):
        sg.step()
        sp.step()
    a = sg.get_state().solvers_state[0].pos.detach()
    b = sp.get_state().solvers_state[0].pos
    assert (a - b).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()


@pytest.mark.parametrize("with_fields", [False, True, "custom"])
def test_solver_protocol_gradient_walk_equals_autograd(gs, with_fields):
    """The reference's imperative walk (Scene._backward: add_grad_from_state, then per step in reverse
    substep_post_coupling_grad / substep_pre_coupling_grad per substep and process_input_grad) through
    the solver's protocol members gives the same input gradient as loss.backward()."""
    target = torch.tensor([0.5, 0.5, 0.3], device="cuda")
    steps = 3

    def run(imperative):
        if with_fields == "custom":  # a Custom field between two built-in ones: the staged substeps
            fs = _field_set(gs)[:2] + [gs.force_fields.Custom(lambda p, u, t, i: -2.0 * u + 0.5 * p)]
        else:
            fs = _field_set(gs) if with_fields else ()
        scene, box, water = _scene(gs, box_z=0.165, fields=fs)
        v = torch.tensor([0.2, 0.1, -1.0], device="cuda", requires_grad=True)
        box.set_velocity(v)
        for _ in range(steps):
            scene.step()
        solver = scene.sim.mpm_solver
        st = solver.get_state()
        if not imperative:
            ((st.pos[0].mean(0) - target) ** 2).sum().backward()
            return v.grad.clone()
        leaf = type(st)(1, solver.n_particles, "cuda")
        for k in ("pos", "vel", "C", "F"):
            setattr(leaf, k, getattr(st, k).detach().clone().requires_grad_(True))
        ((leaf.pos[0].mean(0) - target) ** 2).sum().backward()
        solver.reset_grad()
        solver.add_grad_from_state(leaf)
        for _ in range(steps):
            for f in range(scene.substeps - 1, -1, -1):
                solver.substep_post_coupling_grad(f)
                solver.substep_pre_coupling_grad(f)
            solver.process_input_grad()
        return v.grad.clone()

    a = run(False)
    b = run(True)
    assert torch.allclose(a, b, rtol=1e-4, atol=1e-7), (a, b)


def _rod_obj(path, hx=0.05, hy=0.05, hz=0.5):
    """A closed box mesh (a rod along z, 0.1 x 0.1 x 1 before the tool's normalisation)."""
    v = [(x, y, z) for x in (-hx, hx) for y in (-hy, hy) for z in (-hz, hz)]
    quads = [(1, 2, 4, 3), (5, 7, 8, 6), (1, 5, 6, 2), (3, 4, 8, 7), (1, 3, 7, 5), (2, 6, 8, 4)]
    with open(path, "w") as f:
        for p in v:
            f.write("v %f %f %f\n" % p)
        for q in quads:
            f.write("f " + " ".join(str(i) for i in q) + "\n")


def _tool_scene(gs, obj, requires_grad=True, n_envs=0):
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-3, substeps=10, requires_grad=requires_grad),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0.0, 0.0, 0.0), upper_bound=(1.0, 1.0, 0.55)))
    tool = scene.add_entity(morph=gs.morphs.Mesh(file=str(obj), scale=0.08, pos=(0.275, 0.16, 0.1)),
                            material=gs.materials.Tool(friction=1.0, sdf_res=48))
    block = scene.add_entity(morph=gs.morphs.Box(lower=(0.2, 0.2, 0.05), upper=(0.35, 0.35, 0.15)),
                             material=gs.materials.MPM.Elastic(rho=500, sampler="regular"))
    scene.build(n_envs=n_envs)
    return scene, tool, block


def test_tool_gradients_match_fp64_central_differences(gs, oracle, tmp_path):
    """A tool entity (a cube mesh) pushed into an Elastic block through the scene API in
    differentiable mode: d loss / d (tool velocity) along a random direction and d loss / d (tool
    start position) along x and z, through Mesh.collide in the grid op and ToolEntity.advect (loss:
    a fixed random projection of the block's final particle positions), against FP64 central
    differences of the oracle running the same tool as a collider, tolerance 5e-2 relative; the
    forward of differentiable mode follows the oracle (1e-4 m).  The start position is not checked
    along y, the push direction: there a shift moves the tool's influence front across grid nodes,
    whose velocity jumps where the influence passes 0.1 (mesh.py:156-157), and the central
    differences follow those jumps (they change by 2x between eps = 1e-4 and 1e-5 m) while the
    adjoint, like the reference's autodiff, differentiates the smooth part."""
    from test_api_host import _cube_obj

    from genesis_gb300.coupling import tool as tool_collider

    obj = tmp_path / "cube.obj"
    _cube_obj(obj, half=1.0)
    scene, tool, block = _tool_scene(gs, obj)
    n = block.n_particles
    w = torch.tensor(np.random.default_rng(3).normal(size=(n, 3)), dtype=torch.float32, device="cuda")
    p0 = np.array([0.275, 0.16, 0.1])  # the cube's face at the block's (y = 0.2)
    u0 = np.array([0.0, 1.0, -0.2])
    p = torch.tensor(p0, dtype=torch.float32, device="cuda", requires_grad=True)
    u = torch.tensor(u0, dtype=torch.float32, device="cuda", requires_grad=True)
    tool.set_position(p)
    tool.set_velocity(vel=u)
    steps = 8
    for _ in range(steps):
        scene.step()
    x = block.get_state().pos[0]
    loss = (x * w).sum() / n
    loss.backward()
    gp, gu = p.grad.double().cpu().numpy(), u.grad.double().cpu().numpy()
    assert np.abs(gu).max() > 0 and np.abs(gp).max() > 0

    solver = scene.sim.mpm_solver
    sc = oracle.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                           upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                           particle_size=solver.particle_size)
    om = [oracle.from_c_material(block.material.to_c(0))]
    x0 = block.init_particles.astype(np.float32).astype(np.float64)
    st = dict(pos=x0, vel=np.zeros((n, 3)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)), Jp=np.ones(n),
              mat=np.zeros(n, np.int32), active=np.ones(n, bool))
    wn = w.double().cpu().numpy()
    g = tool.sdf

    def L(pos, vel):
        oracle.clear_sdf_grids()
        sid = oracle.add_sdf_grid(g.values, None, g.T_mesh_to_sdf, g.cell_size, g.sdf_max)
        c = tool_collider(g, pos=tuple(pos), vel=tuple(vel), friction=1.0, coup_softness=0.01, floor_height=0.0)
        oracle.set_colliders([c.to_c(sid)])
        try:
            out, _, _ = oracle.run(sc, om, st, steps * 10)
        finally:
            oracle.set_colliders([])
            oracle.clear_sdf_grids()
        return float((out["pos"] * wn).sum() / n), out["pos"]

    base, xo = L(p0, u0)
    assert np.abs(x.detach().double().cpu().numpy() - xo).max() < 1e-4
    assert np.abs(xo - L(p0 + np.array([0.0, -0.2, 0.0]), u0)[1]).max() > 5e-3  # the tool acts on the block
    rng = np.random.default_rng(11)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    checks = [("vel", gu, d, 1e-4), ("pos x", gp, np.array([1.0, 0.0, 0.0]), 1e-5),
              ("pos z", gp, np.array([0.0, 0.0, 1.0]), 1e-5)]
    for which, grad, dirn, eps in checks:
        if which == "vel":
            fd = (L(p0, u0 + eps * dirn)[0] - L(p0, u0 - eps * dirn)[0]) / (2 * eps)
        else:
            fd = (L(p0 + eps * dirn, u0)[0] - L(p0 - eps * dirn, u0)[0]) / (2 * eps)
        ad = float(grad @ dirn)
        print(f"tool d loss / d {which}: adjoint {ad:.6e} fd {fd:.6e}")
        assert abs(fd) > 1e-6, (which, fd)
        assert abs(ad - fd) <= 5e-2 * abs(fd), (which, ad, fd)


def test_reference_scenario_differentiable_push_with_tool(gs, tmp_path):
    """tests/test_grad.py::test_differentiable_push with its tool entity: two envs, a rod-shaped tool
    (set_position with a tensor that requires grad, then a velocity input every step), an Elastic
    box (position and velocity inputs), losses on the solver state at step 5 and on the entity
    state at step 8; after loss.backward() every velocity input but the last has a non-zero
    gradient and the last one none, as the reference asserts; the tool's start positions get
    gradients too.  The stirrer asset is replaced by a 0.6 m rod turned along y (euler (90, 0, 0)
    as in the reference) that lies on the box in env 0 (z = 0.16) and clear of it in env 1; the
    rod slides along its axis, dragging the box's top layer by friction."""
    obj = tmp_path / "rod.obj"
    _rod_obj(obj)
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-3, substeps=10, requires_grad=True),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0.0, -1.0, 0.0), upper_bound=(1.0, 1.0, 0.55)))
    stick = scene.add_entity(morph=gs.morphs.Mesh(file=str(obj), scale=0.6, pos=(0.5, 0.5, 0.05),
                                                  euler=(90.0, 0.0, 0.0)),
                             material=gs.materials.Tool(friction=8.0, sdf_res=64))
    obj_e = scene.add_entity(morph=gs.morphs.Box(lower=(0.2, 0.1, 0.05), upper=(0.4, 0.3, 0.15)),
                             material=gs.materials.MPM.Elastic(rho=500))
    scene.build(n_envs=2)
    init_pos = torch.tensor([[0.3, 0.1, 0.16], [0.3, 0.1, 0.5]], device="cuda", requires_grad=True)
    stick.set_position(init_pos)
    pos_obj_init = torch.tensor([0.3, 0.3, 0.1], device="cuda", requires_grad=True)
    obj_e.set_position(pos_obj_init)
    v_obj_init = torch.tensor([0.0, -1.0, 0.0], device="cuda", requires_grad=True)
    obj_e.set_velocity(v_obj_init)
    goal = torch.tensor([0.5, 0.8, 0.05], device="cuda")
    horizon = 10
    loss = 0.0
    v_list = []
    for i in range(horizon):
        v_i = torch.tensor([[0.0, 1.0, 0.0], [0.0, 1.0, 0.0]], device="cuda", requires_grad=True)
        stick.set_velocity(vel=v_i)
        v_list.append(v_i)
        scene.step()
        if i == horizon // 2:
            mpm = scene.get_state().solvers_state[0]
            loss = loss + torch.pow(mpm.pos[mpm.active == 1] - goal, 2).sum()
        if i == horizon - 2:
            state = obj_e.get_state()
            loss = loss + torch.pow(state.pos - goal, 2).sum()
    loss.backward()
    eps = float(np.finfo(np.float32).eps)
    for v_i in v_list[:-1]:
        assert (v_i.grad.abs() > eps).any()
    # the last input never reaches a loss: torch leaves its grad None where the reference's
    # backward walk writes zeros
    assert v_list[-1].grad is None or (v_list[-1].grad.abs() < eps).all()
    assert init_pos.grad is not None and (init_pos.grad.abs() > eps).any()
    assert (pos_obj_init.grad.abs() > eps).any() and (v_obj_init.grad.abs() > eps).any()


def test_couplings_outside_the_differentiable_form_raise(gs):
    """Tool-shaped colliders (tool entities are the differentiable form), reaction forces and SPH /
    PBD coupling have no differentiable form here: differentiable mode refuses them instead of
    stepping without them."""
    from genesis_gb300.coupling import Collider, SDFGrid
    from genesis_gb300.exceptions import GenesisException

    scene, box, _ = _scene(gs)
    solver = scene.sim.mpm_solver
    knob = SDFGrid.from_function(lambda p: np.linalg.norm(p, axis=-1) - 0.03, (-0.06,) * 3, (0.06,) * 3, 17,
                                 grads=False)
    with pytest.raises(GenesisException, match="differentiable mode"):
        solver.set_colliders([Collider("tool", pos=(0.5, 0.5, 0.1), sdf=knob)])
    solver.set_colliders([Collider("sphere", pos=(0.5, 0.5, 0.1), radius=0.05)])
    with pytest.raises(GenesisException, match="differentiable mode"):
        solver.get_collider_forces()
    p = torch.zeros((4, 3), device="cuda")
    with pytest.raises(GenesisException, match="differentiable mode"):
        solver.set_coupled_particles("sph", pos=p, vel=p.clone(), mass=torch.ones(4, device="cuda"))
    solver.set_colliders([])  # an empty list stays allowed



def _collider_set():
    from genesis_gb300.coupling import Collider, SDFGrid

    knob = SDFGrid.from_function(lambda p: np.linalg.norm(p, axis=-1) - 0.03, (-0.06,) * 3, (0.06,) * 3, 25)
    cols = [
        Collider("sphere", pos=(0.42, 0.5, 0.10), radius=0.06, coup_friction=0.4, coup_softness=0.002),
        Collider("box", pos=(0.49, 0.47, 0.13), quat=(np.cos(0.2), np.sin(0.2), 0.0, 0.0),
                 half_extents=(0.03, 0.05, 0.02), lin_vel=(0.3, 0.0, 0.1), ang_vel=(0.0, 0.0, 2.0),
                 coup_friction=0.2, coup_restitution=0.2, coup_softness=0.004),
        Collider("sdf", sdf=knob, pos=(0.40, 0.56, 0.12), coup_friction=0.3, coup_softness=0.003),
    ]
    return cols, knob


def test_rigid_collider_gradients_match_fp64_central_differences(gs, oracle):
    """The box falls onto a sphere, a tilted moving box and an SDF-grid geom (legacy_coupler.py:134-218,
    284-347 in the differentiable grid op): dL/dv0 against FP64 central differences of the oracle
    with the same colliders (2%); the colliders move the differences by more than 10%, and the
    forward equals the product path (1e-4 m)."""
    cols, knob = _collider_set()
    scene, box, water = _scene(gs, box_z=0.215)
    scene.sim.mpm_solver.set_colliders(cols)
    v0 = np.array([0.1, 0.05, -2.0])
    target = np.array([0.5, 0.5, 0.2])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    box.set_velocity(v)
    steps = 4
    for _ in range(steps):
        scene.step()
    pos = box.get_state().pos
    loss = ((pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    sp, bp, _ = _scene(gs, requires_grad=False, box_z=0.215)
    sp.sim.mpm_solver.set_colliders(cols)
    bp.set_velocity(torch.tensor(v0, dtype=torch.float32, device="cuda"))
    for _ in range(steps):
        sp.step()
    assert (bp.get_state().pos[0] - pos[0].detach()).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()
    n_sub = steps * scene.substeps
    ents = [box, water]

    def L(vb, with_colliders=True):
        oracle.clear_sdf_grids()
        ids = [oracle.add_sdf_grid(knob.values, knob.grads, knob.T_mesh_to_sdf, knob.cell_size, knob.sdf_max)]
        oracle.set_colliders([c.to_c(ids[0] if c.sdf is not None else -1) for c in cols] if with_colliders else [])
        try:
            return _oracle_com_loss(oracle, scene, ents, vb, target, n_sub)
        finally:
            oracle.set_colliders([])
            oracle.clear_sdf_grids()

    assert abs(loss.item() - L(v0.astype(np.float32).astype(np.float64))) <= 1e-4 * loss.item() + 1e-8
    eps = 1e-4

    def fd(wc):
        return np.array([(L(v0 + eps * np.eye(3)[k], wc) - L(v0 - eps * np.eye(3)[k], wc)) / (2 * eps)
                         for k in range(3)])

    fd_c, fd_free = fd(True), fd(False)
    assert np.linalg.norm(fd_c - fd_free) > 0.1 * np.linalg.norm(fd_c), (fd_c, fd_free)
    assert np.linalg.norm(g - fd_c) <= GRAD_RTOL * np.linalg.norm(fd_c), (g, fd_c)


def _qrot(q, v):
    w, u = q[0], np.asarray(q[1:])
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def test_particle_constraint_gradients_match_fp64_central_differences(gs, oracle):
    """A quarter of the box's particles hang on a link that moves and turns between steps
    (apply_particle_constraints after G2P, mpm_solver.py:1099-1128): dL/dv0 against FP64 central
    differences of the oracle's substeps with the same spring applied after each (2%); the springs
    move the differences by more than 10%, and the forward equals the product path (1e-4 m)."""
    steps, k = 4, 300.0
    p0, q0 = np.array([0.45, 0.5, 0.35]), np.array([1.0, 0.0, 0.0, 0.0])
    poses = [(p0 + np.array([0.01, 0.0, 0.005]) * (s + 1),
              np.array([np.cos(0.05 * (s + 1)), 0.0, 0.0, np.sin(0.05 * (s + 1))])) for s in range(steps)]
    v0 = np.array([0.3, -0.2, 0.5])
    target = np.array([0.47, 0.5, 0.37])

    def run(requires_grad, vel):
        scene, box, water = _scene(gs, requires_grad=requires_grad)
        solver = scene.sim.mpm_solver
        solver.set_link_poses(p0[None], q0[None])
        mask = np.zeros(box.n_particles, bool)
        mask[::4] = True
        box.set_particle_constraints(mask, 0, k)
        box.set_velocity(vel)
        for p, q in poses:
            solver.set_link_poses(p[None], q[None])
            scene.step()
        return scene, box, water, mask

    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    scene, box, water, mask = run(True, v)
    pos = box.get_state().pos[0]
    loss = ((pos.mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    sp, bp, _, _ = run(False, torch.tensor(v0, dtype=torch.float32, device="cuda"))
    assert (bp.get_state().pos[0] - pos.detach()).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()

    solver = scene.sim.mpm_solver
    ents = [box, water]
    oms = [oracle.from_c_material(m.to_c(0)) for m in solver._unique_materials()]
    x0 = np.concatenate([e.init_particles.astype(np.float32).astype(np.float64) for e in ents])
    n, nb = len(x0), box.n_particles
    sel = np.zeros(n, bool)
    sel[:nb] = mask
    local = np.array([_qrot(q0 * np.array([1, -1, -1, -1]), x - p0) for x in x0[sel]])
    m_real = float(np.float32(np.float32(solver.particle_volume) * np.float32(box.material.rho))) / 1e3
    sc = oracle.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                           upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                           particle_size=solver.particle_size)

    def L(vb, springs=True):
        vel = np.zeros((n, 3))
        vel[:nb] = vb
        st = dict(pos=x0, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
                  Jp=np.concatenate([np.full(e.n_particles, float(e.material._default_Jp)) for e in ents]),
                  mat=np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents]),
                  active=np.ones(n, bool))
        for p, q in poses:
            tgt = np.array([_qrot(q, l) for l in local]) + p
            for _ in range(scene.substeps):
                st, _, _ = oracle.run(sc, oms, st, 1)
                if springs:
                    vv = st["vel"][sel]
                    st["vel"][sel] = vv + solver.substep_dt * (-k * (st["pos"][sel] - tgt)
                                                                - 2.0 * np.sqrt(k * m_real) * vv) / m_real
        return float(((st["pos"][:nb].mean(0) - target) ** 2).sum())

    assert abs(loss.item() - L(v0.astype(np.float32).astype(np.float64))) <= 1e-4 * loss.item() + 1e-8
    eps = 1e-4

    def fd(springs):
        return np.array([(L(v0 + eps * np.eye(3)[j], springs) - L(v0 - eps * np.eye(3)[j], springs)) / (2 * eps)
                         for j in range(3)])

    fd_s, fd_free = fd(True), fd(False)
    assert np.linalg.norm(fd_s - fd_free) > 0.1 * np.linalg.norm(fd_s), (fd_s, fd_free)
    assert np.linalg.norm(g - fd_s) <= GRAD_RTOL * np.linalg.norm(fd_s), (g, fd_s)


def test_reset_in_differentiable_mode_restores_tools_and_restarts(gs, tmp_path):
    """scene.reset() in differentiable mode puts the particles and the tool back at their initial
    state and restarts the step count (simulator.py:223-232): the same inputs then give the same
    trajectory and the same gradient as the first run."""
    from test_api_host import _cube_obj

    obj = tmp_path / "cube.obj"
    _cube_obj(obj, half=1.0)
    scene, tool, block = _tool_scene(gs, obj)
    w = torch.tensor(np.random.default_rng(4).normal(size=(block.n_particles, 3)), dtype=torch.float32,
                     device="cuda")

    def run():
        u = torch.tensor([0.0, 1.0, -0.2], device="cuda", requires_grad=True)
        tool.set_velocity(vel=u)
        for _ in range(6):
            scene.step()
        x = block.get_state().pos[0]
        (x * w).sum().backward()
        return x.detach().clone(), tool.get_state().pos.detach().clone(), u.grad.clone()

    x1, t1, g1 = run()
    assert g1.abs().max().item() > 0
    scene.reset()
    assert scene.sim.mpm_solver._diff.substeps_taken == 0
    x2, t2, g2 = run()
    assert (x1 - x2).abs().max().item() < 1e-6
    assert (t1 - t2).abs().max().item() < 1e-6
    assert torch.allclose(g1, g2, rtol=1e-4, atol=1e-7), (g1, g2)


def test_env_specific_collider_in_differentiable_mode(gs):
    """A collider given to one env only (Collider.env) acts in that env's differentiable grid op and
    not in the other's, as in the product path (two envs, 1e-4 m), and the gradient reaches both
    envs' inputs."""
    from genesis_gb300.coupling import Collider

    col = [Collider("sphere", pos=(0.45, 0.5, 0.22), radius=0.06, coup_friction=0.3, env=1)]
    sg, bg, _ = _scene(gs, requires_grad=True, n_envs=2, box_z=0.33)
    sp, bp, _ = _scene(gs, requires_grad=False, n_envs=2, box_z=0.33)
    sg.sim.mpm_solver.set_colliders(col)
    sp.sim.mpm_solver.set_colliders(col)
    v = torch.tensor([0.0, 0.0, -2.0], device="cuda", requires_grad=True)
    bg.set_velocity(v)
    bp.set_velocity(v.detach())
    for _ in range(4):
        sg.step()
        sp.step()
    a = bg.get_state().pos
    b = bp.get_state().pos
    assert (a.detach() - b).abs().max().item() <= 1e-4
    assert (a.detach()[0] - a.detach()[1]).abs().max().item() > 1e-3  # the sphere met env 1's box only
    a[1].mean(0)[2].backward()
    assert torch.isfinite(v.grad).all() and v.grad.abs().max().item() > 0
    sp.sim.mpm_solver.destroy()


def test_custom_force_field_gradients_match_fp64_central_differences(gs, oracle):
    """A Custom force field (a torch function of the node velocities, between a built-in field before
    it and one after it) in differentiable mode: the substeps run in stages with the function applied
    between them and its Jacobian taken by torch autograd in the adjoint.  The function is a drag with a
    learnable coefficient k, so the oracle can run the same field as a built-in Drag: dL/dv0 and dL/dk
    against FP64 central differences of the oracle (2%), and the forward equals the product path."""
    ff = gs.force_fields
    k0 = 3.0
    k = torch.tensor(k0, device="cuda", requires_grad=True)

    def drag(pos, vel, t, i):
        return -k * vel - 1.5 * vel.norm(dim=1, keepdim=True) * vel

    def fields(custom_k):
        fs = [ff.Constant(direction=(1.0, 0.0, 0.0), strength=2.0), ff.Custom(custom_k),
              ff.Point(strength=-3.0, position=(0.5, 0.5, 0.25), falloff_pow=1.0, flow=2.0)]
        for f in (fs[0], fs[2]):
            f.activate()
        return fs

    scene, box, water = _scene(gs, box_z=0.165, fields=fields(drag))
    v0 = np.array([0.4, -0.3, -1.5])
    target = np.array([0.52, 0.47, 0.3])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    box.set_velocity(v)
    steps = 3
    for _ in range(steps):
        scene.step()
    pos = box.get_state().pos
    loss = ((pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g_v = v.grad.detach().cpu().numpy().astype(np.float64)
    g_k = float(k.grad)

    sp, bp, _ = _scene(gs, requires_grad=False, box_z=0.165,
                       fields=fields(lambda p, u, t, i: -k0 * u - 1.5 * u.norm(dim=1, keepdim=True) * u))
    bp.set_velocity(torch.tensor(v0, dtype=torch.float32, device="cuda"))
    for _ in range(steps):
        sp.step()
    assert (bp.get_state().pos[0] - pos[0].detach()).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()

    n_sub = steps * scene.substeps
    ents = [box, water]

    def L(vb, kv):
        fs = [ff.Constant(direction=(1.0, 0.0, 0.0), strength=2.0), ff.Drag(linear=kv, quadratic=1.5),
              ff.Point(strength=-3.0, position=(0.5, 0.5, 0.25), falloff_pow=1.0, flow=2.0)]
        for f in fs:
            f.activate()
        return _oracle_com_loss(oracle, scene, ents, vb, target, n_sub, fs)

    assert abs(loss.item() - L(v0.astype(np.float32).astype(np.float64), k0)) <= 1e-4 * loss.item() + 1e-8
    eps = 1e-4
    fd_v = np.array([(L(v0 + eps * np.eye(3)[j], k0) - L(v0 - eps * np.eye(3)[j], k0)) / (2 * eps) for j in range(3)])
    fd_k = (L(v0, k0 + 1e-3) - L(v0, k0 - 1e-3)) / 2e-3
    assert np.linalg.norm(g_v - fd_v) <= GRAD_RTOL * np.linalg.norm(fd_v), (g_v, fd_v)
    assert abs(fd_k) > 1e-6 and abs(g_k - fd_k) <= GRAD_RTOL * abs(fd_k), (g_k, fd_k)


def test_activity_changes_in_differentiable_mode(gs, oracle):
    """entity.deactivate() between steps in differentiable mode: the Liquid block stops taking part
    (mpm_solver.py p2g / g2p skip an inactive particle and keep its state), the forward equals the
    product path with the same activity (1e-4 m), and dL/dv0 of the box matches FP64 central
    differences of the oracle with the same activity per substep (2%)."""
    v0 = np.array([0.4, -0.3, -1.5])
    target = np.array([0.52, 0.47, 0.3])
    steps = 4

    def run(requires_grad, vel):
        scene, box, water = _scene(gs, requires_grad=requires_grad, box_z=0.165)
        box.set_velocity(vel)
        water.set_velocity(torch.tensor([-2.0, 0.0, 0.0], device="cuda"))
        for s_i in range(steps):
            if s_i == 1:
                water.deactivate()
            scene.step()
        return scene, box, water

    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    scene, box, water = run(True, v)
    pos = box.get_state().pos
    wpos = water.get_state().pos
    loss = ((pos[0].mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    sp, bp, wp = run(False, torch.tensor(v0, dtype=torch.float32, device="cuda"))
    assert (bp.get_state().pos[0] - pos[0].detach()).abs().max().item() <= 1e-4
    assert (wp.get_state().pos[0] - wpos[0].detach()).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()

    solver = scene.sim.mpm_solver
    ents = [box, water]
    oms = [oracle.from_c_material(m.to_c(0)) for m in solver._unique_materials()]
    x0 = np.concatenate([e.init_particles.astype(np.float32).astype(np.float64) for e in ents])
    n, nb = len(x0), box.n_particles
    sc = oracle.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                           upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                           particle_size=solver.particle_size)

    def L(vb):
        vel = np.zeros((n, 3))
        vel[:nb] = vb
        vel[nb:] = (-2.0, 0.0, 0.0)
        st = dict(pos=x0, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
                  Jp=np.concatenate([np.full(e.n_particles, float(e.material._default_Jp)) for e in ents]),
                  mat=np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents]),
                  active=np.ones(n, bool))
        st, _, _ = oracle.run(sc, oms, st, scene.substeps)
        st["active"] = np.concatenate([np.ones(nb, bool), np.zeros(n - nb, bool)])
        st, _, _ = oracle.run(sc, oms, st, (steps - 1) * scene.substeps)
        return float(((st["pos"][:nb].mean(0) - target) ** 2).sum())

    assert abs(loss.item() - L(v0.astype(np.float32).astype(np.float64))) <= 1e-4 * loss.item() + 1e-8
    eps = 1e-4
    fd = np.array([(L(v0 + eps * np.eye(3)[j]) - L(v0 - eps * np.eye(3)[j])) / (2 * eps) for j in range(3)])
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)
