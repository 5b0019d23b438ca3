"""Differentiation at the size the benchmark runs it: the ~216k-particle elastic cube on the 97^3
grid, 640 substeps (64 steps x 10) with a checkpoint every 160, falling onto the floor boundary
(bench.diff_config).  The hand-written adjoint's directional derivatives of
L = ||COM - target||^2 along a random direction of the initial velocity and a random relative
direction of the per-particle Young's moduli against FP64 central differences of the oracle run
on every host core.  Tolerance: 2e-2 relative (float32 adjoint against float64 differences, as
for the small cases)."""

import os

import numpy as np
import pytest
import torch

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
GRAD_RTOL = 2e-2
N_SUB = 640


def _oracle_loss(O, cfg, x0, v0, E, target, nu=0.2):
    n = len(x0)
    sc = O.make_scene(cfg.substep_dt, gravity=tuple(cfg.gravity), lower_bound=tuple(cfg.lower_bound),
                      upper_bound=tuple(cfg.upper_bound), grid_density=cfg.grid_density,
                      particle_size=cfg.particle_size, eps=cfg.mass_eps)
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mats = [O.make_material(0, float(m), float(lm), 1000.0) for m, lm in zip(mu, lam)]
    st = dict(pos=x0, vel=np.tile(v0, (n, 1)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)),
              Jp=np.ones(n), mat=np.arange(n, dtype=np.int32), active=np.ones(n, bool))
    out, _, _ = O.run(sc, mats, st, N_SUB, threads=os.cpu_count() or 1)
    return float(((out["pos"].mean(0) - target) ** 2).sum())


def test_c4_directional_derivatives_match_fp64_central_differences(oracle):
    import __graft_entry__ as g

    g.build()
    import bench
    from genesis_gb300.diff import DifferentiableMPM

    cfg, x0, E, v0, target = bench.diff_config()
    sim = DifferentiableMPM(cfg, nu=0.2, rho=1000.0, ckpt_every=160)
    x = torch.tensor(x0, dtype=torch.float32, device="cuda")
    v = torch.tensor(v0, dtype=torch.float32, device="cuda", requires_grad=True)
    e = torch.tensor(E, dtype=torch.float32, device="cuda", requires_grad=True)
    loss = ((sim.rollout(x, v, e, N_SUB).mean(0) - torch.tensor(target, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    gv = v.grad.double().cpu().numpy()
    gE = e.grad.double().cpu().numpy()
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gE)) and np.abs(gE).max() > 0

    rng = np.random.default_rng(21)
    dv = rng.normal(size=3)
    dv /= np.linalg.norm(dv)
    eps = 1e-4
    fd_v = (_oracle_loss(oracle, cfg, x0, v0 + eps * dv, E, target) -
            _oracle_loss(oracle, cfg, x0, v0 - eps * dv, E, target)) / (2 * eps)
    ad_v = float(gv @ dv)
    dE = rng.normal(size=len(E))
    dE /= np.linalg.norm(dE)
    fd_E = (_oracle_loss(oracle, cfg, x0, v0, E * (1 + eps * dE), target) -
            _oracle_loss(oracle, cfg, x0, v0, E * (1 - eps * dE), target)) / (2 * eps)
    ad_E = float(gE @ (E * dE))
    print(f"C4 directional derivatives: v0 adjoint {ad_v:.6e} fd {fd_v:.6e}; E adjoint {ad_E:.6e} fd {fd_E:.6e}")
    assert abs(fd_v) > 1e-6 and abs(fd_E) > 1e-9, (fd_v, fd_E)
    assert abs(ad_v - fd_v) <= GRAD_RTOL * abs(fd_v), (ad_v, fd_v)
    assert abs(ad_E - fd_E) <= GRAD_RTOL * abs(fd_E), (ad_E, fd_E)
