"""Differentiation form: hand-written adjoint substeps checked against FP64 central differences
of the CPU oracle (eps = 1e-4), for d loss / d v0 and a directional derivative d loss / d E.

loss = ||centre of mass of the final positions - target||^2 (the differentiation config).
The reference's own (Quadrants autodiff) gradient cannot run here; the FP64 finite
differences of the reference algorithm are the ground truth.  Tolerance: 2e-2 relative
(float32 adjoint against float64 differences of a float64 rollout)."""

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


def _oracle_loss(O, x0, v0, E, target, n_sub, nu=0.2, dt=2e-4):
    n = len(x0)
    sc = O.make_scene(dt, grid_density=32.0, particle_size=1.0 / 64)
    mats = []
    for e in E:
        mu = e / (2 * (1 + nu))
        lam = e * nu / ((1 + nu) * (1 - 2 * nu))
        mats.append(O.make_material(0, mu, lam, 1000.0))
    st = dict(pos=x0, vel=np.tile(v0, (n, 1)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
              Jp=np.ones(n), mat=np.arange(n, dtype=np.int32), active=np.ones(n, bool))
    out, _, _ = O.run(sc, mats, st, n_sub)
    com = out["pos"].mean(0)
    return float(((com - target) ** 2).sum()), out["pos"]


@pytest.fixture(scope="module")
def sim():
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    return DifferentiableMPM(_scene(), nu=0.2, rho=1000.0, ckpt_every=16)


def _gpu_loss_and_grads(sim, x0, v0, E, target, n_sub):
    x = torch.tensor(x0, dtype=torch.float32, device="cuda")
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    e = torch.tensor(E, dtype=torch.float32, device="cuda", requires_grad=True)
    xf = sim.rollout(x, v, e, n_sub)
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
    rng = np.random.default_rng(8)
    d = rng.normal(size=len(E))
    d /= np.linalg.norm(d)
    h = eps * E  # relative step per particle: E (1 +- eps d)
    fd_E = (_oracle_loss(oracle, x0, v0, E + h * d, target, n_sub)[0] -
            _oracle_loss(oracle, x0, v0, E - h * d, target, n_sub)[0]) / (2 * eps)
    ad_E = float(np.dot(gE, h * d)) / eps
    assert abs(ad_E - fd_E) <= GRAD_RTOL * max(abs(fd_E), 1e-12) + 1e-9, (ad_E, fd_E)


def test_checkpointing_does_not_change_gradients(oracle):
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.diff import DifferentiableMPM

    x0, v0, E, target = _setup(seed=6)
    a = DifferentiableMPM(_scene(), ckpt_every=8)
    b = DifferentiableMPM(_scene(), ckpt_every=1000)
    _, _, gva, gEa = _gpu_loss_and_grads(a, x0, v0, E, target, 32)
    _, _, gvb, gEb = _gpu_loss_and_grads(b, x0, v0, E, target, 32)
    assert np.allclose(gva, gvb, rtol=1e-3, atol=1e-9)
    assert np.allclose(gEa, gEb, rtol=1e-2, atol=1e-3 * np.abs(gEb).max())
