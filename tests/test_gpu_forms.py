"""Batched and serving forms: every scene's result in a batch / in the served mix equals the
same scene run alone, within the position tolerance of the parity tests (1e-4 m)."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
POS_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


def test_batched_uneven_scenes_equal_alone():
    from genesis_gb300.batched import BatchedMPM, batched_workload

    specs = batched_workload(n_scenes=8, seed=21, n_range=(2000, 12000))
    assert len({s.n_particles for s in specs}) > 1 and len({type(s.material) for s in specs}) > 1
    b = BatchedMPM(specs, tune=False)
    b.step(60)
    assert b.check() == 0
    st = b.get_state_all()
    for i, s in enumerate(specs):
        alone = BatchedMPM([s], tune=False)
        alone.step(60)
        ref = alone.scene_state(0)
        got = b.scene_state(i, st)
        err = (got["pos"] - ref["pos"]).abs().max().item()
        assert err <= POS_TOL, (i, type(s.material).__name__, err)
        alone.close()
    b.close()


def test_batched_autotune_keeps_state():
    from genesis_gb300.batched import BatchedMPM, batched_workload

    specs = batched_workload(n_scenes=4, seed=5, n_range=(2000, 6000))
    b = BatchedMPM(specs, tune=False)
    before = b.get_state_all()
    choice, timings = b.tune()
    after = b.get_state_all()
    assert torch.equal(before["pos"], after["pos"])
    assert f"{choice[0]}x{choice[1]}/{choice[2]}" in timings or timings == {}
    b.close()


def test_served_results_equal_alone_and_batching_is_continuous():
    from genesis_gb300.batched import BatchedMPM
    from genesis_gb300.serve import MPMServer, serving_workload

    reqs = serving_workload(n_requests=10, rate_hz=0, seed=3, n_range=(1000, 20000), grid_res=(33, 65),
                            substep_range=(20, 70))
    srv = MPMServer(max_slots=4, particle_capacity=200_000, max_grid_res=65, chunk=10)
    stats = srv.run(reqs, keep_results=True, realtime=False)
    assert stats["requests"] == len(reqs) and stats["status"] == 0
    # continuous batching: with 4 slots for 10 requests, later requests are admitted only after
    # earlier ones finish, and they then run alongside requests that are still in flight
    first_finish = min(r.finished for r in reqs)
    late = [r for r in reqs if r.admitted >= first_finish]
    assert late, "slots never turned over"
    assert any(o.admitted < r.admitted < o.finished for r in late for o in reqs if o is not r)
    for r in reqs:
        alone = BatchedMPM([r.spec], tune=False)
        alone.step(r.spec.substeps)
        ref = alone.scene_state(0)
        err = (r.result["pos"] - ref["pos"]).abs().max().item()
        assert err <= POS_TOL, (r.rid, err)
        alone.close()
    srv.close()


def test_pool_slot_reuse_after_retire():
    from genesis_gb300.batched import BatchedMPM
    from genesis_gb300.serve import MPMServer, Request, serving_workload

    reqs = serving_workload(n_requests=3, rate_hz=0, seed=9, n_range=(3000, 8000), grid_res=(65,),
                            substep_range=(40, 40))
    srv = MPMServer(max_slots=2, particle_capacity=50_000, max_grid_res=65, chunk=10)
    stats = srv.run(reqs, keep_results=True, realtime=False)
    assert stats["requests"] == 3
    for r in reqs:
        alone = BatchedMPM([r.spec], tune=False)
        alone.step(r.spec.substeps)
        err = (r.result["pos"] - alone.scene_state(0)["pos"]).abs().max().item()
        assert err <= POS_TOL, (r.rid, err)
        alone.close()
    srv.close()


def test_served_results_equal_alone_in_a_wide_pool():
    """A pool with many buckets (16 slots of 129^3 grids: 575k buckets, 1,123 scan tiles, several
    waves of scan CTAs in the look-back): each request's result is still the one it gets alone."""
    from genesis_gb300.batched import BatchedMPM
    from genesis_gb300.serve import MPMServer, serving_workload

    reqs = serving_workload(n_requests=6, rate_hz=0, seed=9, n_range=(2000, 30000), grid_res=(65, 129),
                            substep_range=(20, 60))
    srv = MPMServer(max_slots=16, particle_capacity=400_000, max_grid_res=129, chunk=10)
    stats = srv.run(reqs, keep_results=True, realtime=False)
    assert stats["requests"] == len(reqs) and stats["status"] == 0
    for r in reqs:
        alone = BatchedMPM([r.spec], tune=False)
        alone.step(r.spec.substeps)
        ref = alone.scene_state(0)
        err = (r.result["pos"] - ref["pos"]).abs().max().item()
        assert err <= POS_TOL, (r.rid, err)
        alone.close()
    srv.close()


def test_served_cancellation_and_unadmittable_request():
    """Host-side faults of the serving loop: a running request cancelled after its first chunk is
    retired without a result and frees its slot; a request cancelled while waiting is never
    admitted; the others still match their runs alone.  A request larger than the pool can never be
    admitted and raises, and the server keeps serving afterwards."""
    from genesis_gb300.batched import BatchedMPM
    from genesis_gb300.serve import MPMServer, serving_workload

    reqs = serving_workload(n_requests=6, rate_hz=0, seed=11, n_range=(1000, 8000), grid_res=(33, 65),
                            substep_range=(30, 60))
    srv = MPMServer(max_slots=2, particle_capacity=40_000, max_grid_res=65, chunk=10)
    srv.cancel(reqs[5].rid)  # before it is admitted

    def on_chunk(server, k):
        if k == 0:
            server.cancel(reqs[0].rid)  # running since the start

    stats = srv.run(reqs, keep_results=True, realtime=False, on_chunk=on_chunk)
    assert stats["cancelled"] == 2 and stats["requests"] == 4 and stats["status"] == 0
    assert reqs[0].cancelled and reqs[0].result is None and reqs[0].admitted is not None
    assert reqs[5].cancelled and reqs[5].admitted is None
    for r in reqs[1:5]:
        assert not r.cancelled
        alone = BatchedMPM([r.spec], tune=False)
        alone.step(r.spec.substeps)
        err = (r.result["pos"] - alone.scene_state(0)["pos"]).abs().max().item()
        assert err <= POS_TOL, (r.rid, err)
        alone.close()
    big = serving_workload(n_requests=1, rate_hz=0, seed=12, n_range=(60000, 60001), grid_res=(65,))
    with pytest.raises(RuntimeError, match="can never be admitted"):
        srv.run(big, realtime=False)
    again = serving_workload(n_requests=2, rate_hz=0, seed=13, n_range=(1000, 3000), grid_res=(33,),
                             substep_range=(20, 30))
    assert srv.run(again, realtime=False)["requests"] == 2
    srv.close()
