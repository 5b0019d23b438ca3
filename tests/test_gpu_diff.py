"""Differentiation form: hand-written adjoint substeps checked against FP64 central differences
of the CPU oracle (eps = 1e-4), for d loss / d v0 and a directional derivative d loss / d E.

d/dv0 uses the differentiation config's loss ||centre of mass - target||^2.  Without contact a
centre of mass does not depend on E (internal stresses exert no net force), so the E checks
use a loss that sees the deformation: a fixed random projection of every final position, with
an initial shear velocity so the elastic forces matter.  The reference's own (Quadrants
autodiff) gradient cannot run here; FP64 finite differences of the reference algorithm are the
ground truth.  Tolerance: 2e-2 relative (float32 adjoint against float64 differences)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GRAD_RTOL = 2e-2


def _scene(n_sub_dt=2e-4):
    from genesis_gb300 import _lib
    from capi_helpers import scene_record

    return scene_record(_lib, n_sub_dt, 0, density=32.0, p_size=1.0 / 64)


def _setup(seed=4, n_side=8):
    rng = np.random.default_rng(seed)
    ax = 0.5 + (np.arange(n_side) - (n_side - 1) / 2) / 64.0
    x0 = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    x0 = x0 + rng.uniform(-0.002, 0.002, size=x0.shape)
    E = 3e5 * np.exp(0.2 * rng.normal(size=len(x0)))
    v0 = np.array([0.3, -0.2, 0.5])
    target = rng.uniform(0.3, 0.7, size=3)
    return x0, v0, E, target


def _shear(x0):
    """Fixed initial velocity field (shear + stretch), added to the uniform v0."""
    d = x0 - x0.mean(0)
    return np.stack([20.0 * d[:, 2], -15.0 * d[:, 0], 25.0 * d[:, 1]], -1)


def _proj(n, seed=12):
    return np.random.default_rng(seed).normal(size=(n, 3))


def _oracle_loss(O, x0, v0, E, target, n_sub, nu=0.2, dt=2e-4, vfield=None, proj=None):
    n = len(x0)
    sc = O.make_scene(dt, grid_density=32.0, particle_size=1.0 / 64)
    mats = []
    for e in E:
        mu = e / (2 * (1 + nu))
        lam = e * nu / ((1 + nu) * (1 - 2 * nu))
        mats.append(O.make_material(0, mu, lam, 1000.0))
    vel = np.tile(v0, (n, 1)) + (0.0 if vfield is None else vfield)
    st = dict(pos=x0, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
              Jp=np.ones(n), mat=np.arange(n, dtype=np.int32), active=np.ones(n, bool))
    out, _, _ = O.run(sc, mats, st, n_sub)
    if proj is not None:
        return float((out["pos"] * proj).sum() / n), out["pos"]
    com = out["pos"].mean(0)
    return float(((com - target) ** 2).sum()), out["pos"]


@pytest.fixture(scope="module")
def sim():
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    return DifferentiableMPM(_scene(), nu=0.2, rho=1000.0, ckpt_every=16)


def _gpu_loss_and_grads(sim, x0, v0, E, target, n_sub, vfield=None, proj=None):
    x = torch.tensor(x0, dtype=torch.float32, device="cuda")
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    e = torch.tensor(E, dtype=torch.float32, device="cuda", requires_grad=True)
    vv = v.expand(len(x0), 3)
    if vfield is not None:
        vv = vv + torch.tensor(vfield, dtype=torch.float32, device="cuda")
    xf = sim.rollout(x, vv, e, n_sub)
    if proj is not None:
        loss = (xf * torch.tensor(proj, dtype=torch.float32, device="cuda")).sum() / len(x0)
    else:
        loss = ((xf.mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    return loss.item(), xf.detach().cpu().numpy(), v.grad.cpu().numpy().astype(np.float64), e.grad.cpu().numpy().astype(np.float64)


def test_forward_matches_oracle(sim, oracle):
    x0, v0, E, target = _setup()
    _, xf, _, _ = _gpu_loss_and_grads(sim, x0, v0, E, target, 40)
    _, ref = _oracle_loss(oracle, x0, v0, E, target, 40)
    assert np.abs(xf - ref).max() < 1e-5


def test_grad_v0_and_E_match_fp64_central_differences(sim, oracle):
    x0, v0, E, target = _setup()
    n_sub = 40
    _, _, gv, gE = _gpu_loss_and_grads(sim, x0, v0, E, target, n_sub)
    eps = 1e-4
    fd_v = np.zeros(3)
    for k in range(3):
        dv = np.zeros(3)
        dv[k] = eps
        fd_v[k] = (_oracle_loss(oracle, x0, v0 + dv, E, target, n_sub)[0] -
                   _oracle_loss(oracle, x0, v0 - dv, E, target, n_sub)[0]) / (2 * eps)
    assert np.linalg.norm(gv - fd_v) <= GRAD_RTOL * np.linalg.norm(fd_v), (gv, fd_v)


def test_grad_E_matches_fp64_central_differences(sim, oracle):
    x0, v0, E, target = _setup()
    n_sub = 40
    vf, pj = _shear(x0), _proj(len(x0))
    _, _, _, gE = _gpu_loss_and_grads(sim, x0, v0, E, target, n_sub, vfield=vf, proj=pj)
    assert np.abs(gE).max() > 0
    rng = np.random.default_rng(8)
    for trial in range(2):
        d = rng.normal(size=len(E))
        d /= np.linalg.norm(d)
        eps = 1e-4
        h = eps * E  # relative step per particle: E (1 +- eps d)
        fd_E = (_oracle_loss(oracle, x0, v0, E + h * d, target, n_sub, vfield=vf, proj=pj)[0] -
                _oracle_loss(oracle, x0, v0, E - h * d, target, n_sub, vfield=vf, proj=pj)[0]) / (2 * eps)
        ad_E = float(np.dot(gE, E * d))
        assert abs(fd_E) > 1e-8, fd_E
        assert abs(ad_E - fd_E) <= GRAD_RTOL * abs(fd_E), (trial, ad_E, fd_E)


def test_checkpointing_does_not_change_gradients(oracle):
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    x0, v0, E, target = _setup(seed=6)
    a = DifferentiableMPM(_scene(), ckpt_every=8)
    b = DifferentiableMPM(_scene(), ckpt_every=1000)
    vf, pj = _shear(x0), _proj(len(x0))
    _, _, gva, gEa = _gpu_loss_and_grads(a, x0, v0, E, target, 32, vfield=vf, proj=pj)
    _, _, gvb, gEb = _gpu_loss_and_grads(b, x0, v0, E, target, 32, vfield=vf, proj=pj)
    assert np.allclose(gva, gvb, rtol=1e-3, atol=1e-9 + 1e-4 * np.abs(gvb).max())
    assert np.linalg.norm(gEa - gEb) <= 1e-2 * np.linalg.norm(gEb)
    # keeping every segment from the forward (no re-simulation in the backward) changes nothing
    c = DifferentiableMPM(_scene(), ckpt_every=8, keep_segments=True)
    _, _, gvc, gEc = _gpu_loss_and_grads(c, x0, v0, E, target, 32, vfield=vf, proj=pj)
    assert np.allclose(gvc, gva, rtol=1e-3, atol=1e-9 + 1e-4 * np.abs(gva).max())
    assert np.linalg.norm(gEc - gEa) <= 1e-2 * np.linalg.norm(gEa)


def test_memory_budget_fallbacks_do_not_change_gradients(oracle):
    """The backward's memory-bound modes give the default mode's gradients: a forward that keeps only
    some segments, a substep-by-substep backward that keeps each re-simulated substep's grid, and one
    that keeps none (every adjoint substep re-runs its forward).  The memory budget is overridden on
    the instance to reach each mode at this size."""
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    x0, v0, E, target = _setup(seed=6)
    n = len(x0)
    vf, pj = _shear(x0), _proj(n)
    ref = DifferentiableMPM(_scene(), ckpt_every=8)
    _, _, gv_ref, gE_ref = _gpu_loss_and_grads(ref, x0, v0, E, target, 32, vfield=vf, proj=pj)
    assert ref.last_backward == "segments" and ref.last_segments == (1, 4)

    def check(sim, mode):
        _, _, gv, gE = _gpu_loss_and_grads(sim, x0, v0, E, target, 32, vfield=vf, proj=pj)
        assert sim.last_backward == mode
        assert np.allclose(gv, gv_ref, rtol=1e-3, atol=1e-9 + 1e-4 * np.abs(gv_ref).max())
        assert np.linalg.norm(gE - gE_ref) <= 1e-2 * np.linalg.norm(gE_ref)

    # the forward asks once per segment (four), the backward once: segments 3 and 4 do not fit
    part = DifferentiableMPM(_scene(), ckpt_every=8, keep_segments=True)
    calls = []

    def budget():
        calls.append(1)
        return 0 if len(calls) in (3, 4) else 1 << 50

    part.grid_budget_bytes = budget
    check(part, "segments")
    assert part.last_segments == (2, 4)
    # a segment does not fit, its grids do
    sub = DifferentiableMPM(_scene(), ckpt_every=8)
    sub.grid_budget_bytes = lambda: sub.segment_bytes(n, 8) - 1
    assert sub.nodes * 32 * 8 <= sub.segment_bytes(n, 8) - 1
    check(sub, "substeps")
    assert sub.last_segments == (0, 4)
    # nothing fits
    bare = DifferentiableMPM(_scene(), ckpt_every=8)
    bare.grid_budget_bytes = lambda: 0
    check(bare, "substeps")


def _oracle_two_loss(O, x0, v0, E, target, n1, n2, nu=0.2, dt=2e-4, vfield=None, proj=None):
    """Loss on the state after n1 substeps plus the loss on the state after n1 + n2 (the oracle
    continues from its own intermediate state)."""
    n = len(x0)
    sc = O.make_scene(dt, grid_density=32.0, particle_size=1.0 / 64)
    mats = []
    for e in E:
        mu = e / (2 * (1 + nu))
        lam = e * nu / ((1 + nu) * (1 - 2 * nu))
        mats.append(O.make_material(0, mu, lam, 1000.0))
    vel = np.tile(v0, (n, 1)) + (0.0 if vfield is None else vfield)
    st = dict(pos=x0, vel=vel, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
              Jp=np.ones(n), mat=np.arange(n, dtype=np.int32), active=np.ones(n, bool))
    mid, _, _ = O.run(sc, mats, st, n1)
    st2 = dict(st, pos=mid["pos"], vel=mid["vel"], C=mid["C"], F=mid["F"], Jp=mid["Jp"])
    end, _, _ = O.run(sc, mats, st2, n2)
    f = lambda p: float((p * proj).sum() / n)  # noqa: E731
    return f(mid["pos"]) + f(end["pos"])


def test_intermediate_losses_through_chained_segments_match_fp64_differences(sim, oracle):
    """advance() chains: a loss on the state after 16 substeps plus one after 40 (as the reference's
    differentiable mode takes losses at several frames of an episode) gives dL/dv0 and dL/dE that
    match FP64 central differences of the oracle; and chaining 16 + 24 substeps gives the same
    gradient of a final-state loss as one 40-substep advance."""
    x0, v0, E, target = _setup(seed=5)
    n = len(x0)
    vf, pj = _shear(x0), _proj(n)
    cu = lambda a, g=False: torch.tensor(a, dtype=torch.float32, device="cuda", requires_grad=g)  # noqa: E731

    def grads(split):
        v = cu(v0, True)
        e = cu(E, True)
        s = (cu(x0), v.expand(n, 3) + cu(vf), torch.zeros((n, 3, 3), device="cuda"),
             torch.eye(3, device="cuda").repeat(n, 1, 1))
        P = cu(pj)
        if split:
            s1 = sim.advance(s, e, 16)
            s2 = sim.advance(s1, e, 24)
            loss = (s1[0] * P).sum() / n + (s2[0] * P).sum() / n
        else:
            s2 = sim.advance(s, e, 40)
            loss = (s2[0] * P).sum() / n
        loss.backward()
        return v.grad.cpu().numpy().astype(np.float64), e.grad.cpu().numpy().astype(np.float64), s2

    gv, gE, _ = grads(True)
    eps = 1e-4
    fd_v = np.zeros(3)
    for k in range(3):
        dv = np.zeros(3)
        dv[k] = eps
        fd_v[k] = (_oracle_two_loss(oracle, x0, v0 + dv, E, target, 16, 24, vfield=vf, proj=pj) -
                   _oracle_two_loss(oracle, x0, v0 - dv, E, target, 16, 24, vfield=vf, proj=pj)) / (2 * eps)
    assert np.linalg.norm(gv - fd_v) <= GRAD_RTOL * np.linalg.norm(fd_v), (gv, fd_v)
    d = np.random.default_rng(3).normal(size=n)
    d /= np.linalg.norm(d)
    h = eps * E
    fd_E = (_oracle_two_loss(oracle, x0, v0, E + h * d, target, 16, 24, vfield=vf, proj=pj) -
            _oracle_two_loss(oracle, x0, v0, E - h * d, target, 16, 24, vfield=vf, proj=pj)) / (2 * eps)
    ad_E = float(np.dot(gE, E * d))
    assert abs(ad_E - fd_E) <= GRAD_RTOL * abs(fd_E), (ad_E, fd_E)

    # one final-state loss: chained segments == one advance
    def final_grad(split):
        v = cu(v0, True)
        e = cu(E, True)
        s = (cu(x0), v.expand(n, 3) + cu(vf), torch.zeros((n, 3, 3), device="cuda"),
             torch.eye(3, device="cuda").repeat(n, 1, 1))
        out = sim.advance(sim.advance(s, e, 16), e, 24) if split else sim.advance(s, e, 40)
        ((out[0] * cu(pj)).sum() / n).backward()
        return v.grad.cpu().numpy(), e.grad.cpu().numpy()

    ga, gEa = final_grad(True)
    gb, gEb = final_grad(False)
    assert np.allclose(ga, gb, rtol=1e-3, atol=1e-9 + 1e-4 * np.abs(gb).max()), (ga, gb)
    assert np.linalg.norm(gEa - gEb) <= 1e-2 * np.linalg.norm(gEb)


def test_liquid_gradients_match_fp64_central_differences(oracle):
    """The differentiable form with Liquid (liquid.py: mu = 0, stress lam J (J - 1) I, F reset to
    J^(1/3) I every substep; E per particle through lam): dL/dv0 and a directional dL/dE of a
    projection loss after 40 substeps against FP64 central differences of the oracle."""
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    x0, v0, E, _ = _setup(seed=7)
    n = len(x0)
    # shear plus a uniform compression, so the pressure lam J (J - 1) shapes the motion
    vf, pj = _shear(x0) - 5.0 * (x0 - x0.mean(0)), _proj(n)
    nu, n_sub = 0.3, 40
    sim = DifferentiableMPM(_scene(), nu=nu, rho=1000.0, ckpt_every=16, material="liquid")

    def oracle_loss(v0_, E_):
        sc = oracle.make_scene(2e-4, grid_density=32.0, particle_size=1.0 / 64)
        mats = [oracle.make_material(1, 0.0, e * nu / ((1 + nu) * (1 - 2 * nu)), 1000.0) for e in E_]
        st = dict(pos=x0, vel=np.tile(v0_, (n, 1)) + vf, C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
                  Jp=np.ones(n), mat=np.arange(n, dtype=np.int32), active=np.ones(n, bool))
        out, _, _ = oracle.run(sc, mats, st, n_sub)
        return float((out["pos"] * pj).sum() / n), out["pos"]

    _, ref = oracle_loss(v0, E)
    _, xf, gv, gE = _gpu_loss_and_grads(sim, x0, v0, E, None, n_sub, vfield=vf, proj=pj)
    assert np.abs(xf - ref).max() < 1e-5
    eps = 1e-4
    fd_v = np.array([(oracle_loss(v0 + eps * e, E)[0] - oracle_loss(v0 - eps * e, E)[0]) / (2 * eps)
                     for e in np.eye(3)])
    assert np.linalg.norm(gv - fd_v) <= GRAD_RTOL * np.linalg.norm(fd_v), (gv, fd_v)
    d = np.random.default_rng(2).normal(size=n)
    d /= np.linalg.norm(d)
    fd_E = (oracle_loss(v0, E * (1 + eps * d))[0] - oracle_loss(v0, E * (1 - eps * d))[0]) / (2 * eps)
    ad_E = float(np.dot(gE, E * d))
    assert abs(fd_E) > 1e-8 and abs(ad_E - fd_E) <= GRAD_RTOL * abs(fd_E), (ad_E, fd_E)
