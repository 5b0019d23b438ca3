"""Serving form: continuous batching of MPM rollout requests on one GPU.

Requests (one single-material scene each, with its own particle count, grid resolution and
substep budget) arrive over time.  The server keeps every admitted scene's particle and grid
state resident in one pool context (libgbmpm pool mode), so all live scenes advance together
in the same P2G / grid-op / G2P launches (replayed as a CUDA graph between membership
changes).  Between chunks of substeps it:
  * admits waiting requests in arrival order while a slot, pool particles and the HBM budget
    (particle + grid bytes, capped at `mem_fraction` of device memory) allow;
  * retires scenes whose substep budget reached zero (a finished scene is frozen on the
    device, so overshooting the chunk does not change its result), after copying its state;
  * drops or retires cancelled requests (`cancel`), freeing their slot and memory.
Latency of a request = completion time - arrival time.  The reference has no serving mode;
the loop is the GB300 form of running many Genesis scenes.
"""

from __future__ import annotations

import ctypes
import dataclasses
import heapq
import math
import time

import numpy as np
import torch

from . import _lib
from .batched import SceneSpec, scene_config
from .materials import Elastic, Liquid, Sand, Snow

PARTICLE_BYTES = 2 * 27 * 4 + 3 * 4  # two particle buffers + key/rank/perm
BLOCK_BYTES = 2 * 64 * 16 + 4 * 4  # two grid buffers + flags/lists/bucket arrays


@dataclasses.dataclass
class Request:
    rid: int
    spec: SceneSpec
    arrival: float
    admitted: float | None = None
    finished: float | None = None
    result: dict | None = None
    payload: np.ndarray | None = None  # initial particle positions [n, 3] float32, sent with the request
    cancelled: bool = False

    @property
    def work(self) -> int:
        return self.spec.n_particles * self.spec.substeps


def grid_blocks(res: int) -> int:
    return ((res + 3) // 4) ** 3


def serving_workload(n_requests=64, rate_hz=200.0, seed=7, n_range=(1000, 500000), grid_res=(33, 65, 129),
                     substep_range=(50, 500), substep_dt=2e-4, with_payload=False):
    """Config 5: Poisson arrivals; N ~ logUniform[1k, 500k]; grid res from {33,65,129}^3 (the
    reference's +1 node convention for 32/64/128 cells over the unit cube); substeps ~ U[50, 500];
    material uniform over {Elastic, Liquid, Sand, Snow}.  The particle box is sized so particles
    sit about 2 per cell per axis, clipped to [0.05, 0.6] m.  With `with_payload` every request
    carries its initial positions (made by the client, before it arrives), so admission only
    copies them to the device."""
    rng = np.random.default_rng(seed)
    mats = (Elastic, Liquid, Sand, Snow)
    t = 0.0
    reqs = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate_hz) if rate_hz > 0 else 0.0
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        res = int(grid_res[int(rng.integers(0, len(grid_res)))])
        density = float(res - 1)
        ext = float(np.clip(n ** (1.0 / 3.0) * 0.5 / density, 0.05, 0.6))
        steps = int(rng.integers(substep_range[0], substep_range[1] + 1))
        m = mats[int(rng.integers(0, 4))]()
        center = (0.5, 0.5, 3.5 / density + ext / 2 + 0.01)
        spec = SceneSpec(m, n, ext, center, grid_density=density, substep_dt=substep_dt,
                         seed=int(rng.integers(0, 2**31)), substeps=steps)
        reqs.append(Request(i, spec, t))
    if with_payload:
        for r in reqs:
            r.payload = r.spec.positions().astype(np.float32)
    return reqs


class MPMServer:
    def __init__(self, max_slots=64, particle_capacity=None, max_grid_res=129, mem_fraction=0.8, chunk=20,
                 device=None):
        self.lib = _lib.load()
        dev = torch.cuda.current_device() if device is None else device
        free, total = torch.cuda.mem_get_info(dev)
        self.budget = int(mem_fraction * total)
        self.max_grid_res = max_grid_res
        self.slot_blocks = grid_blocks(max_grid_res)
        grid_bytes = max_slots * self.slot_blocks * BLOCK_BYTES
        if particle_capacity is None:
            particle_capacity = min(64_000_000, max(1, (min(self.budget, free) // 2 - grid_bytes) // PARTICLE_BYTES))
        self.capacity = int(particle_capacity)
        cfg = _lib.MpmPoolConfig()
        cfg.max_scenes = max_slots
        cfg.particle_capacity = self.capacity
        cfg.max_grid_res = max_grid_res
        cfg.max_materials_per_scene = 1
        cfg.with_muscle = 0
        self.ctx = ctypes.c_void_p()
        _lib.check(self.lib.mpm_ctx_create_pool(ctypes.byref(cfg), dev, ctypes.byref(self.ctx)), None, "create_pool")
        self.max_slots = max_slots
        self.free_slots = list(range(max_slots))
        self.live = {}  # slot -> Request
        self.chunk = chunk
        self.live_bytes = 0
        self.live_particles = 0
        self.fixed_bytes = grid_bytes
        self._cancel = set()  # request ids to drop (waiting) or retire (running) at the next check

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def request_bytes(self, r: Request) -> int:
        return r.spec.n_particles * PARTICLE_BYTES + grid_blocks(int(r.spec.grid_density) + 1) * BLOCK_BYTES

    def can_admit(self, r: Request) -> bool:
        return (bool(self.free_slots) and self.live_particles + r.spec.n_particles <= self.capacity
                and self.fixed_bytes + self.live_bytes + self.request_bytes(r) <= self.budget
                and int(r.spec.grid_density) + 1 <= self.max_grid_res)

    def admit(self, r: Request, now: float) -> None:
        slot = self.free_slots.pop(0)
        s = r.spec
        cfg = scene_config(s, float(np.finfo(np.float32).eps))
        mats = (_lib.MpmMaterial * 1)(s.material.to_c(slot))
        host = r.payload if r.payload is not None else s.positions().astype(np.float32)
        pos = torch.from_numpy(np.ascontiguousarray(host, dtype=np.float32)).to("cuda")
        _lib.check(self.lib.mpm_scene_admit(self.ctx, slot, ctypes.byref(cfg), mats, 1, s.n_particles, pos.data_ptr(),
                                            None, int(s.substeps), self._stream()), self.ctx, "mpm_scene_admit")
        r.admitted = now
        self.live[slot] = r
        self.live_bytes += self.request_bytes(r)
        self.live_particles += s.n_particles

    def retire(self, slot: int, now: float, keep_result: bool) -> None:
        r = self.live.pop(slot)
        if keep_result:
            n = r.spec.n_particles
            pos = torch.empty((n, 3), device="cuda")
            vel = torch.empty((n, 3), device="cuda")
            _lib.check(self.lib.mpm_get_state(self.ctx, slot, slot + 1, pos.data_ptr(), vel.data_ptr(), None, None,
                                              None, None, self._stream()), self.ctx, "mpm_get_state")
            r.result = {"pos": pos, "vel": vel}
        _lib.check(self.lib.mpm_scene_retire(self.ctx, slot, self._stream()), self.ctx, "mpm_scene_retire")
        r.finished = now
        self.free_slots.append(slot)
        self.live_bytes -= self.request_bytes(r)
        self.live_particles -= r.spec.n_particles

    def cancel(self, rid: int) -> None:
        """Cancel request `rid`: if it is waiting it is never admitted; if it is running it is
        retired after the current chunk of substeps, without a result, and its slot and memory go
        to the next admission.  Safe to call from `run`'s on_chunk callback."""
        self._cancel.add(int(rid))

    def run(self, requests, keep_results=False, realtime=True, on_chunk=None):
        """Serve `requests` (arrival times in seconds from the start).  Returns stats.
        on_chunk(server, chunk_index) is called after every chunk of substeps (e.g. to cancel)."""
        pending = sorted(requests, key=lambda r: r.arrival)
        cancelled = []
        queue = []  # arrived, waiting: (arrival, rid, request)
        steps_left = (ctypes.c_int32 * self.max_slots)()
        t0 = time.perf_counter()
        done = []
        i = 0
        chunks = 0
        while i < len(pending) or queue or self.live:
            now = time.perf_counter() - t0 if realtime else float("inf")
            while i < len(pending) and pending[i].arrival <= now:
                heapq.heappush(queue, (pending[i].arrival, pending[i].rid, pending[i]))
                i += 1
            while queue:
                r = queue[0][2]
                if r.rid in self._cancel:  # cancelled while waiting: never admitted
                    heapq.heappop(queue)
                    self._cancel.discard(r.rid)
                    r.cancelled, r.finished = True, time.perf_counter() - t0
                    cancelled.append(r)
                    continue
                if not self.can_admit(r):
                    break
                self.admit(heapq.heappop(queue)[2], time.perf_counter() - t0)
            if not self.live:
                if queue and not self.can_admit(queue[0][2]):
                    raise RuntimeError(f"request {queue[0][2].rid} can never be admitted")
                if i < len(pending):
                    time.sleep(max(0.0, min(pending[i].arrival - (time.perf_counter() - t0), 0.01)))
                continue
            _lib.check(self.lib.mpm_substeps(self.ctx, self.chunk, self._stream()), self.ctx, "mpm_substeps")
            chunks += 1
            _lib.check(self.lib.mpm_scene_steps_left(self.ctx, steps_left, self._stream()), self.ctx, "steps_left")
            if on_chunk is not None:
                on_chunk(self, chunks - 1)
            now = time.perf_counter() - t0
            for slot in [s for s, r in self.live.items() if r.rid in self._cancel]:  # cancelled while running
                r = self.live[slot]
                self._cancel.discard(r.rid)
                self.retire(slot, now, keep_result=False)
                r.cancelled = True
                cancelled.append(r)
            for slot in [s for s in self.live if steps_left[s] == 0]:
                r = self.live[slot]
                self.retire(slot, now, keep_results)
                done.append(r)
        wall = time.perf_counter() - t0
        st = ctypes.c_uint32()
        _lib.check(self.lib.mpm_status_word(self.ctx, ctypes.byref(st), None, 1, self._stream()), self.ctx, "status")
        lat = np.array([r.finished - r.arrival for r in done])
        work = sum(r.work for r in done)
        first = min(r.arrival for r in done) if done else 0.0
        return {
            "requests": len(done),
            "particle_substeps": work,
            "wall_s": wall,
            "throughput": work / max(1e-9, wall - (first if realtime else 0.0)),
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "chunks": chunks,
            "cancelled": len(cancelled),
            "status": st.value,
        }

    def close(self):
        if self.ctx:
            self.lib.mpm_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
