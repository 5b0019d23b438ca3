"""GPU parity on the benchmark workload: the ~1M-particle three-material scene (liquid 0.3^3 block,
Drucker-Prager sand 0.2^3 block, elastic sphere r = 0.1, stacked in z; 129^3-node grid over the unit
cube; dt = 1e-4; gravity on), against the FP64 CPU oracle started from the same state.

Tolerances as in the other parity tests: grid mass and momentum per substep within 1e-5 relative
(L2 over the grid); particle positions within 1e-4 m (1e-4 of the 1 m domain) after 100 substeps.
At about 12 particles per touched cell this is the scene with the most float-atomic reordering per
node of all the parity cases.  The same boxes at 4 particles per cell per axis (5.27M particles)
are checked over two substeps.
"""

import numpy as np
import pytest

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


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / nb if nb > 0 else np.linalg.norm(a)


def _scene(gs, spacing=None):
    import bench

    scene, ents, _ = bench.build_c2_scene(gs, spacing=spacing)
    return scene, ents


def _oracle_inputs(O, scene, ents, st):
    solver = scene.sim.mpm_solver
    mats = solver._unique_materials()
    oms = [O.from_c_material(m.to_c(0)) for m in mats]
    mat_idx = np.concatenate([np.full(e.n_particles, e.material.idx, np.int32) for e in ents])
    d = lambda t: t[0].detach().double().cpu().numpy()  # noqa: E731
    state = dict(pos=d(st.pos), vel=d(st.vel), C=d(st.C), F=d(st.F), Jp=d(st.Jp), mat=mat_idx,
                 active=st.active[0].cpu().numpy().astype(bool))
    sc = O.make_scene(solver.substep_dt, gravity=tuple(solver.gravity[0]), lower_bound=tuple(solver.lower_bound),
                      upper_bound=tuple(solver.upper_bound), grid_density=solver.grid_density,
                      particle_size=solver.particle_size)
    return sc, oms, state


def _threads():
    import os

    return os.cpu_count() or 1


def _oracle_velocity_grid(sc, solver, og):
    """The grid op of the oracle's P2G grid (legacy_coupler.py:367-373, 501): v = p/m + dt g on nodes
    with mass > eps, then the free-slip separating boundary; the fused GPU path leaves this grid."""
    m = og[..., 3]
    v = np.zeros(og.shape[:3] + (3,))
    on = m > sc.eps
    v[on] = og[on][:, :3] / m[on][:, None] + np.asarray(sc.gravity) * sc.dt
    lo, hi = solver.boundary.lower, solver.boundary.upper
    off = np.asarray(solver.grid_offset)
    for d in range(3):
        pos = (np.arange(og.shape[d]) + off[d]) * solver.dx
        shape = [1, 1, 1]
        shape[d] = -1
        p = pos.reshape(shape)
        vd = v[..., d]
        out_hi = (p >= hi[d]) & (vd >= 0)
        out_lo = (p <= lo[d]) & (vd <= 0) & ~out_hi
        vd[out_hi | out_lo] = 0.0
    return v, m


def test_c2_grid_per_substep_split_path(gs, oracle):
    """Five substeps through the split phases (P2G, grid op, G2P): after each P2G the GPU grid's mass
    and momentum against the oracle's first substep from the same particle state."""
    scene, ents = _scene(gs)
    solver = scene.sim.mpm_solver
    for k in range(5):
        st = solver.get_state()
        solver.substep_pre_coupling()
        g = solver.get_grid(0).double().cpu().numpy()
        sc, oms, state = _oracle_inputs(oracle, scene, ents, st)
        _, og, touched = oracle.run(sc, oms, state, 1, want_grid=True, threads=_threads())
        assert touched > 100_000
        assert rel_l2(g[..., 3], og[..., 3]) <= GRID_RTOL, (k, rel_l2(g[..., 3], og[..., 3]))
        assert rel_l2(g[..., :3], og[..., :3]) <= GRID_RTOL, (k, rel_l2(g[..., :3], og[..., :3]))
        solver.couple()
        solver.substep_post_coupling()
    solver.check_state()
    solver.destroy()


def test_c2_grid_after_fused_graph_substeps(gs, oracle):
    """Substeps on the fused path (grid op inside G2P, two-substep CUDA graph): the last substep's
    grid (velocity after the grid op, and mass) against the oracle advanced by the same substeps."""
    scene, ents = _scene(gs)
    solver = scene.sim.mpm_solver
    solver.substeps(3)
    for n_sub in (4, 6):
        st = solver.get_state()
        solver.substeps(n_sub)
        g = solver.get_grid(0).double().cpu().numpy()
        sc, oms, state = _oracle_inputs(oracle, scene, ents, st)
        _, og, _ = oracle.run(sc, oms, state, n_sub, want_grid=True, threads=_threads())
        ov, om = _oracle_velocity_grid(sc, solver, og)
        assert rel_l2(g[..., 3], om) <= GRID_RTOL, (n_sub, rel_l2(g[..., 3], om))
        assert rel_l2(g[..., :3], ov) <= GRID_RTOL, (n_sub, rel_l2(g[..., :3], ov))
    solver.check_state()
    solver.destroy()


def test_c2_positions_after_100_substeps(gs, oracle):
    """Ten scene.step() calls of 10 substeps (the benchmark's step) against 100 oracle substeps."""
    scene, ents = _scene(gs)
    solver = scene.sim.mpm_solver
    st0 = solver.get_state()
    for _ in range(10):
        scene.step()
    st = solver.get_state()
    sc, oms, state = _oracle_inputs(oracle, scene, ents, st0)
    ref, _, _ = oracle.run(sc, oms, state, 100, threads=_threads())
    err = np.abs(st.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    assert np.abs(st.vel[0].double().cpu().numpy() - ref["vel"]).max() < 1e-3
    assert np.abs(st.Jp[0].double().cpu().numpy() - ref["Jp"]).max() < 1e-3
    solver.destroy()


def test_c2_dense_variant_two_substeps(gs, oracle):
    """The same boxes at 4 particles per cell per axis (5.27M particles, about 64 per touched cell):
    the grid after two fused substeps and the positions after them."""
    scene, ents = _scene(gs, spacing=1.0 / (4 * 128))
    solver = scene.sim.mpm_solver
    assert solver.n_particles > 5_000_000
    st = solver.get_state()
    solver.substeps(2)
    g = solver.get_grid(0).double().cpu().numpy()
    st1 = solver.get_state()
    sc, oms, state = _oracle_inputs(oracle, scene, ents, st)
    ref, og, _ = oracle.run(sc, oms, state, 2, want_grid=True, threads=_threads())
    ov, om = _oracle_velocity_grid(sc, solver, og)
    assert rel_l2(g[..., 3], om) <= GRID_RTOL, rel_l2(g[..., 3], om)
    assert rel_l2(g[..., :3], ov) <= GRID_RTOL, rel_l2(g[..., :3], ov)
    err = np.abs(st1.pos[0].double().cpu().numpy() - ref["pos"]).max()
    assert err <= POS_TOL, err
    solver.check_state()
    solver.destroy()
