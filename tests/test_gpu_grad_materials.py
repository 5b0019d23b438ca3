"""Differentiable mode with the ElastoPlastic and Muscle materials (the reference differentiates every
MPM material through its autodiff; mpm_entity.py process_input_grad delivers dL/dactuation).

* dL/d(actuation of two muscle groups) set with entity.set_actuation before every step, for a loss
  on the final particle positions, against FP64 central differences of the oracle with the same
  per-particle actuation and fibre directions (2%).
* dL/dv0 of a von Mises ElastoPlastic box and a clamped ElastoPlastic box thrown onto the floor
  (both past their yield limits) against FP64 central differences of the oracle (2%).
* The differentiable forward of such a scene equals the product path (1e-4 m).
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


def _opts(gs, requires_grad):
    return dict(sim_options=gs.options.SimOptions(dt=2e-3, substeps=10, requires_grad=requires_grad),
                mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=32,
                                                  particle_size=1.0 / 64))


def _oracle_scene(oracle, solver):
    return oracle.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                             upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                             particle_size=solver.particle_size)


def _muscle_scene(gs, requires_grad):
    scene = gs.Scene(**_opts(gs, requires_grad))
    worm = scene.add_entity(material=gs.materials.MPM.Muscle(E=1e5, nu=0.3, rho=800, n_groups=2, sampler="regular"),
                            morph=gs.morphs.Box(pos=(0.5, 0.5, 0.3), size=(0.2, 0.06, 0.06)))
    scene.build()
    pos = worm.init_particles
    group = (pos[:, 0] > 0.5).astype(np.int64)
    d = np.array([1.0, 0.0, 0.3]) / np.linalg.norm([1.0, 0.0, 0.3])
    worm.set_muscle(muscle_group=group, muscle_direction=np.tile(d, (len(pos), 1)))
    return scene, worm, group, d


def test_muscle_actuation_gradient_matches_fp64_central_differences(gs, oracle):
    scene, worm, group, d = _muscle_scene(gs, True)
    a0 = np.array([0.2, -0.1])
    a = torch.tensor(a0, dtype=torch.float32, device="cuda", requires_grad=True)
    steps = 4
    for _ in range(steps):
        worm.set_actuation(a)
        scene.step()
    n = worm.n_particles
    W = np.random.default_rng(5).normal(size=(n, 3))
    pos = worm.get_state().pos[0]
    loss = (pos * torch.tensor(W, dtype=torch.float32, device="cuda")).sum()
    loss.backward()
    g = a.grad.detach().cpu().numpy().astype(np.float64)
    solver = scene.sim.mpm_solver
    om = [oracle.from_c_material(worm.material.to_c(0))]
    x0 = worm.init_particles.astype(np.float32).astype(np.float64)
    mdir = np.tile(d.astype(np.float32).astype(np.float64), (n, 1))

    def L(av):
        st = dict(pos=x0, vel=np.zeros((n, 3)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)), Jp=np.ones(n),
                  mat=np.zeros(n, np.int32), active=np.ones(n, bool), actu=np.asarray(av)[group], mdir=mdir)
        out, _, _ = oracle.run(_oracle_scene(oracle, solver), om, st, steps * scene.substeps)
        return float((out["pos"] * W).sum())

    assert abs(loss.item() - L(a0.astype(np.float32).astype(np.float64))) <= 1e-4 * abs(loss.item()) + 1e-4
    eps = 1e-4
    fd = np.array([(L(a0 + eps * np.eye(2)[k]) - L(a0 - eps * np.eye(2)[k])) / (2 * eps) for k in range(2)])
    assert np.abs(fd).min() > 1e-3, fd  # both groups' actuation moves the loss
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)


def _ep_scene(gs, requires_grad):
    scene = gs.Scene(**_opts(gs, requires_grad))
    vm = scene.add_entity(material=gs.materials.MPM.ElastoPlastic(E=2e5, nu=0.3, use_von_mises=True,
                                                                   von_mises_yield_stress=2e3, sampler="regular"),
                          morph=gs.morphs.Box(pos=(0.4, 0.5, 0.16), size=(0.1, 0.1, 0.1)))
    cl = scene.add_entity(material=gs.materials.MPM.ElastoPlastic(E=2e5, nu=0.3, use_von_mises=False,
                                                                   sampler="regular"),
                          morph=gs.morphs.Box(pos=(0.62, 0.5, 0.16), size=(0.1, 0.1, 0.1)))
    scene.build()
    return scene, vm, cl


def test_elastoplastic_grad_matches_fp64_central_differences(gs, oracle):
    """Both boxes take the same initial velocity v (2.5 m/s down): the loss on their joint centre of
    mass goes through the von Mises return mapping and through the clamped stretches."""
    scene, vm, cl = _ep_scene(gs, True)
    v0 = np.array([0.3, 0.2, -2.5])
    target = np.array([0.5, 0.52, 0.1])
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    vm.set_velocity(v)
    cl.set_velocity(v)
    steps = 4
    for _ in range(steps):
        scene.step()
    pos = scene.sim.mpm_solver.get_state().pos[0]
    loss = ((pos.mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    g = v.grad.detach().cpu().numpy().astype(np.float64)
    solver = scene.sim.mpm_solver
    ents = [vm, cl]
    oms = [oracle.from_c_material(m.to_c(0)) for m in solver._unique_materials()]
    x0 = np.concatenate([e.init_particles.astype(np.float32).astype(np.float64) for e in ents])
    n = len(x0)
    mat = np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents])

    def L(vb, materials=oms):
        st = dict(pos=x0, vel=np.tile(vb, (n, 1)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
                  Jp=np.ones(n), mat=mat, active=np.ones(n, bool))
        out, _, _ = oracle.run(_oracle_scene(oracle, solver), materials, st, steps * scene.substeps)
        return float(((out["pos"].mean(0) - target) ** 2).sum())

    assert abs(loss.item() - L(v0.astype(np.float32).astype(np.float64))) <= 1e-4 * loss.item() + 1e-8
    # both boxes yield: as purely elastic bodies they would end elsewhere
    elastic = [oracle.from_c_material(gs.materials.MPM.Elastic(E=2e5, nu=0.3).to_c(0)) for _ in oms]
    assert abs(L(v0, elastic) - L(v0)) > 1e-3 * L(v0)
    eps = 1e-4
    fd = np.array([(L(v0 + eps * np.eye(3)[k]) - L(v0 - eps * np.eye(3)[k])) / (2 * eps) for k in range(3)])
    assert np.linalg.norm(g - fd) <= GRAD_RTOL * np.linalg.norm(fd), (g, fd)


def test_muscle_and_elastoplastic_forward_equals_product_path(gs):
    sg, wg, _, _ = _muscle_scene(gs, True)
    sp, wp, _, _ = _muscle_scene(gs, False)
    for k in range(5):
        act = torch.tensor([0.3 * np.sin(k), 0.2], device="cuda")
        wg.set_actuation(act)
        wp.set_actuation(act)
        sg.step()
        sp.step()
    a = sg.get_state().solvers_state[0].pos.detach()
    b = sp.get_state().solvers_state[0].pos
    assert (a - b).abs().max().item() <= 1e-4
    sp.sim.mpm_solver.destroy()
    eg, vg, cg = _ep_scene(gs, True)
    ep, vp, cp = _ep_scene(gs, False)
    v0 = torch.tensor([0.3, 0.2, -2.5], device="cuda")
    for e in (vg, cg, vp, cp):
        e.set_velocity(v0)
    for _ in range(5):
        eg.step()
        ep.step()
    a = eg.get_state().solvers_state[0].pos.detach()
    b = ep.get_state().solvers_state[0].pos
    assert (a - b).abs().max().item() <= 1e-4
    ep.sim.mpm_solver.destroy()


def test_solver_protocol_walk_delivers_actuation_gradients(gs):
    """The reference's imperative walk (reset_grad, add_grad_from_state, substep_post_coupling_grad /
    substep_pre_coupling_grad per substep, process_input_grad per step) gives the actuation tensor
    the same gradient as loss.backward()."""
    steps = 3

    def run(imperative):
        scene, worm, _, _ = _muscle_scene(gs, True)
        a = torch.tensor([0.25, -0.15], device="cuda", requires_grad=True)
        for _ in range(steps):
            worm.set_actuation(a)
            scene.step()
        solver = scene.sim.mpm_solver
        st = solver.get_state()
        W = torch.linspace(-1.0, 1.0, st.pos[0].numel(), device="cuda").reshape(st.pos[0].shape)
        if not imperative:
            (st.pos[0] * W).sum().backward()
            return a.grad.clone()
        leaf = type(st)(1, solver.n_particles, "cuda")
        for k in ("pos", "vel", "C", "F"):
            setattr(leaf, k, getattr(st, k).detach().clone().requires_grad_(True))
        (leaf.pos[0] * W).sum().backward()
        solver.reset_grad()
        solver.add_grad_from_state(leaf)
        for _ in range(steps):
            for f in range(scene.substeps - 1, -1, -1):
                solver.substep_post_coupling_grad(f)
                solver.substep_pre_coupling_grad(f)
            solver.process_input_grad()
        return a.grad.clone()

    g_auto = run(False)
    g_walk = run(True)
    assert g_auto.abs().min().item() > 0
    assert torch.allclose(g_auto, g_walk, rtol=1e-4, atol=1e-7), (g_auto, g_walk)
