"""Batched and served forms against the FP64 CPU oracle: every scene of a batch and every served
request, advanced on the GPU together with the others, is compared with the oracle running that
scene alone from the same initial particles.  Positions within 1e-4 m (1e-4 of the 1 m domain),
as in the other parity tests.

The batch covers the four materials of the batched workload (Elastic, Liquid, Sand, Snow) at box
extents 0.1 and 0.3 m and at 2,000 and 64,000 particles; the served requests use 33^3, 65^3 and
129^3-node grids.
"""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
POS_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


def _oracle_alone(O, spec, pos0, n_substeps):
    """The scene of `spec` alone on the oracle: particles at pos0 with v = 0, C = 0, F = I and the
    material's default Jp (what mpm_add_particles / mpm_scene_admit give them)."""
    n = len(pos0)
    cm = spec.material.to_c(0)
    state = dict(pos=np.asarray(pos0, np.float64), vel=np.zeros((n, 3)), C=np.zeros((n, 3, 3)),
                 F=np.tile(np.eye(3), (n, 1, 1)), Jp=np.full(n, cm.default_Jp), mat=np.zeros(n, np.int32),
                 active=np.ones(n, bool))
    sc = O.make_scene(spec.substep_dt, gravity=spec.gravity, lower_bound=spec.lower_bound,
                      upper_bound=spec.upper_bound, grid_density=spec.grid_density,
                      particle_size=spec.particle_size)
    ref, _, _ = O.run(sc, [O.from_c_material(cm)], state, n_substeps, threads=os.cpu_count() or 1)
    return ref


def _specs():
    from genesis_gb300.batched import SceneSpec
    from genesis_gb300.materials import Elastic, Liquid, Sand, Snow

    rows = [
        (Elastic, 2000, 0.1), (Liquid, 64000, 0.3), (Sand, 2000, 0.3), (Snow, 64000, 0.1),
        (Elastic, 64000, 0.3), (Liquid, 2000, 0.1), (Sand, 64000, 0.1), (Snow, 2000, 0.3),
        (Elastic, 9000, 0.2), (Sand, 20000, 0.25),
    ]
    return [SceneSpec(m(), n, ext, (0.5, 0.5, 0.06 + ext / 2 + 0.02), seed=100 + i)
            for i, (m, n, ext) in enumerate(rows)]


def test_batched_scenes_match_oracle(oracle):
    from genesis_gb300.batched import BatchedMPM

    specs = _specs()
    n_sub = 60
    b = BatchedMPM(specs, tune=False)
    st0 = b.get_state_all()
    b.step(n_sub)
    assert b.check() == 0
    st = b.get_state_all()
    for i, s in enumerate(specs):
        pos0 = b.scene_state(i, st0)["pos"].double().cpu().numpy()
        ref = _oracle_alone(oracle, s, pos0, n_sub)
        got = b.scene_state(i, st)
        err = np.abs(got["pos"].double().cpu().numpy() - ref["pos"]).max()
        assert err <= POS_TOL, (i, type(s.material).__name__, s.n_particles, s.extent, err)
        verr = np.abs(got["vel"].double().cpu().numpy() - ref["vel"]).max()
        assert verr <= 1e-2, (i, verr)
    b.close()


def test_served_requests_match_oracle(oracle):
    """Requests on 33^3, 65^3 and 129^3 grids served together (4 slots, so later requests join
    while earlier ones run); each result against the oracle running that request alone."""
    from genesis_gb300.serve import MPMServer, serving_workload

    reqs = serving_workload(n_requests=9, rate_hz=0, seed=31, n_range=(1000, 60000), grid_res=(33, 65, 129),
                            substep_range=(40, 120), with_payload=True)
    assert {int(r.spec.grid_density) + 1 for r in reqs} == {33, 65, 129}
    srv = MPMServer(max_slots=4, particle_capacity=400_000, max_grid_res=129, chunk=10)
    stats = srv.run(reqs, keep_results=True, realtime=False)
    assert stats["requests"] == len(reqs) and stats["status"] == 0
    for r in reqs:
        ref = _oracle_alone(oracle, r.spec, r.payload, r.spec.substeps)
        err = np.abs(r.result["pos"].double().cpu().numpy() - ref["pos"]).max()
        assert err <= POS_TOL, (r.rid, int(r.spec.grid_density) + 1, type(r.spec.material).__name__, err)
    srv.close()
