"""Benchmark of the MLS-MPM substep on one GB300 (metric: particle-substeps/s).

Workload (default, N=1): the single large multi-material scene - grid 128^3 cells (129^3
nodes) over the unit cube, ~1M particles: a liquid block 0.3^3 (E=1e5, nu=0.3), a
Drucker-Prager sand block 0.2^3 (friction angle 45 deg) and an elastic sphere of radius
0.1, stacked in z and dropped onto the ground; seed-jittered lattices (spacing chosen for
~1M particles: (V_total/1e6)^(1/3)); substep dt = 1e-4.  One bench step = one
`scene.step()` of 10 substeps.  Inputs are synthetic (seeded), generated here.

--impl reference times the CPU restatement of the reference algorithm (the oracle, fp32,
all host cores via OpenMP) on the same workload; the reference itself (Genesis on the
Quadrants JIT) cannot be installed on these machines.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SUBSTEPS_PER_STEP = 10
# kernels one substep of the benchmark launches (fused grid op: no pinned particles, colliders or
# force fields): k_p2g, k_g2p, k_scan_onepass, k_perm
KERNELS_PER_SUBSTEP = 4
SUBSTEP_DT = 1e-4
PREROLL_SUBSTEPS = 300  # substeps run before the warm-up steps (fixed start of the timed window)
GRID_DENSITY = 128
SEED = 2024
METRIC = "particle-substeps/s on 1 GB300 (plain, batched, served p50/p99) at stated tol"
# per-kernel algorithmic bytes (per particle, per touched node): what each kernel must move at least
ALG_BYTES = {
    "p2g": (144, 16),   # read pos,vel,C,F,Jp,material (104 B) + write F,Jp (40 B); grid write 16 B/node
    "grid_op": (0, 32),  # read (momentum,mass) 16 B + write velocity 16 B per touched node
    "g2p": (72, 16),    # read pos 12 B + write pos,vel,C 60 B; read node velocity 16 B/node
    "scan": (0, 0),
    "perm": (0, 0),
}
SUBSTEP_ALG = (204, 32)  # whole substep: 204 B/particle + 32 B/touched node


def workload_boxes():
    liquid = ((0.5, 0.5, 0.2), 0.3)
    sand = ((0.5, 0.5, 0.5), 0.2)
    sphere = ((0.5, 0.5, 0.75), 0.1)
    v_total = liquid[1] ** 3 + sand[1] ** 3 + 4.0 / 3.0 * np.pi * sphere[1] ** 3
    spacing = (v_total / 1e6) ** (1.0 / 3.0)
    return liquid, sand, sphere, spacing


def jitter(pos, spacing, rng):
    return pos + rng.uniform(-0.25 * spacing, 0.25 * spacing, size=pos.shape)


def build_c2_scene(gs, n_envs=0, spacing=None):
    """The ~1M-particle three-material scene through the Genesis-style API (or the same boxes at
    another particle spacing)."""
    import torch

    liquid, sand, sphere, sp = workload_boxes()
    spacing = sp if spacing is None else spacing
    scene = gs.Scene(
        sim_options=gs.options.SimOptions(dt=SUBSTEP_DT * SUBSTEPS_PER_STEP, substeps=SUBSTEPS_PER_STEP),
        mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=GRID_DENSITY,
                                          particle_size=spacing),
    )
    rng = np.random.default_rng(SEED)
    ents = [
        scene.add_entity(material=gs.materials.MPM.Liquid(E=1e5, nu=0.3, sampler="regular"),
                         morph=gs.morphs.Box(pos=liquid[0], size=(liquid[1],) * 3)),
        scene.add_entity(material=gs.materials.MPM.Sand(friction_angle=45.0, sampler="regular"),
                         morph=gs.morphs.Box(pos=sand[0], size=(sand[1],) * 3)),
        scene.add_entity(material=gs.materials.MPM.Elastic(sampler="regular"),
                         morph=gs.morphs.Sphere(pos=sphere[0], radius=sphere[1])),
    ]
    scene.build(n_envs=n_envs)
    for e in ents:
        p = jitter(e.init_particles, spacing, rng)
        e.set_particles_pos(torch.tensor(p, dtype=torch.float32, device="cuda"))
    return scene, ents, spacing


def oracle_c2_state():
    """Same workload on the host for the CPU baseline (fp32 oracle)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import genesis_gb300 as gs
    from genesis_gb300 import morphs

    liquid, sand, sphere, spacing = workload_boxes()
    rng = np.random.default_rng(SEED)
    mats = [gs.materials.MPM.Liquid(E=1e5, nu=0.3), gs.materials.MPM.Sand(friction_angle=45.0),
            gs.materials.MPM.Elastic()]
    parts = [
        morphs.Box(pos=liquid[0], size=(liquid[1],) * 3).sample(spacing, "regular"),
        morphs.Box(pos=sand[0], size=(sand[1],) * 3).sample(spacing, "regular"),
        morphs.Sphere(pos=sphere[0], radius=sphere[1]).sample(spacing, "regular"),
    ]
    pos = np.concatenate([jitter(p, spacing, rng) for p in parts])
    n = len(pos)
    mat_idx = np.concatenate([np.full(len(p), i, np.int32) for i, p in enumerate(parts)])
    jp = np.concatenate([np.full(len(p), m._default_Jp) for p, m in zip(parts, mats)])
    st = dict(pos=pos, vel=np.zeros((n, 3)), C=np.zeros((n, 3, 3)), F=np.tile(np.eye(3), (n, 1, 1)), Jp=jp,
              mat=mat_idx, active=np.ones(n, bool))
    sc = O.make_scene(SUBSTEP_DT, grid_density=GRID_DENSITY, particle_size=spacing)
    oms = [O.from_c_material(m.to_c(0)) for m in mats]
    return O, sc, oms, st


def cpu_baseline(target_s=10.0):
    """Oracle fp32 on all host cores, bounded sample of the workload (whole scene, a few substeps)."""
    O, sc, oms, st = oracle_c2_state()
    cores = os.cpu_count() or 1
    n = len(st["pos"])
    t0 = time.perf_counter()
    st, _, _ = O.run(sc, oms, st, 1, dtype=np.float32, threads=cores)
    t1 = time.perf_counter() - t0
    k = int(max(1, min(50, target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    O.run(sc, oms, st, k, dtype=np.float32, threads=cores)
    dt = time.perf_counter() - t0
    # the same restatement on one thread (one substep of the full scene)
    t0 = time.perf_counter()
    O.run(sc, oms, st, 1, dtype=np.float32, threads=1)
    dt1 = time.perf_counter() - t0
    return {
        "value": n * k / dt,
        "unit": "particle-substeps/s",
        "cores": cores,
        "kind": "port",
        "sample": f"full workload ({n} particles), {k} substeps after 1 warm-up substep, fp32 oracle, "
        f"OpenMP {cores} threads, {dt:.1f} s",
        "single_thread": {"value": n / dt1, "cores": 1, "sample": f"1 substep of the full workload, {dt1:.1f} s"},
    }


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0, period_ms=20):
        self.samples = []  # (host time when read, fields)
        self.proc = None
        self.dev = device_index
        self.period_ms = period_ms
        self.t_begin = self.t_end = None

    def start(self, wait_s=10.0):
        """Start nvidia-smi and wait for its first sample, so the timed region is covered."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", str(self.period_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while not self.samples and time.perf_counter() - t0 < wait_s and self.proc.poll() is None:
            time.sleep(0.01)

    def begin(self):
        self.t_begin = time.perf_counter()

    def end(self):
        self.t_end = time.perf_counter()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.perf_counter(), parts))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        inside = [p for t, p in self.samples
                  if self.t_begin is not None and self.t_end is not None and self.t_begin <= t <= self.t_end]
        # a sample is read up to one period after it was taken: also keep the one read just after the end
        after = [p for t, p in self.samples if self.t_end is not None and self.t_end < t <= self.t_end + self.period_ms / 1e3]
        use = inside + after[:1] if inside or after else [p for _, p in self.samples]
        sm = [float(s[1]) for s in use if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in use if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in use for i in range(4) if s[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(use), "period_ms": self.period_ms,
                "window": "timed region" if inside or after else "whole run (no sample inside the timed region)"}


class NvmlClockSampler:
    """Polls the SM clock, its maximum, the power draw and the clock-event reasons through NVML
    (libnvidia-ml, read-only queries) every `period_ms` from a thread, so a timed region of a few
    tens of milliseconds still gets many samples.  The device is found by its PCI address."""

    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, torch_device=0, period_ms=2.0):
        import ctypes

        import torch

        self.samples = []  # (host time, sm MHz, max MHz, power W, reasons bitmask)
        self.period = period_ms / 1e3
        self.t_begin = self.t_end = None
        self._stop = threading.Event()
        self.ok = False
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return
            p = torch.cuda.get_device_properties(torch_device)
            bus = f"{p.pci_domain_id:08x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0".encode()
            h = ctypes.c_void_p()
            if nv.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(h)) != 0:
                return
            self.reason_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
        except (OSError, AttributeError, RuntimeError):
            return
        self.nv, self.h, self.ct = nv, h, ctypes
        self.ok = True

    def _one(self):
        ct = self.ct
        sm, mx, mw, rs = ct.c_uint(), ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        self.nv.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(sm))  # NVML_CLOCK_SM
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(mx))
        self.nv.nvmlDeviceGetPowerUsage(self.h, ct.byref(mw))
        self.reason_fn(self.h, ct.byref(rs))
        return sm.value, mx.value, mw.value / 1e3, rs.value

    def _run(self):
        while not self._stop.is_set():
            self.samples.append((time.perf_counter(), *self._one()))
            time.sleep(self.period)

    def start(self, wait_s=0.0):
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()
        time.sleep(0.01)

    def begin(self):
        self.t_begin = time.perf_counter()

    def end(self):
        self.t_end = time.perf_counter()

    def stop(self):
        self._stop.set()
        self.thread.join(timeout=2)
        use = [s for s in self.samples if self.t_begin <= s[0] <= self.t_end]
        window = "timed region"
        if not use:
            use, window = self.samples, "whole run (no sample inside the timed region)"
        reasons = sorted({nm for s in use for bit, nm in self.REASONS.items() if s[4] & bit})
        return {"sm_mhz": statistics.median(s[1] for s in use) if use else None,
                "sm_max_mhz": max(s[2] for s in use) if use else None,
                "power_w_median": statistics.median(s[3] for s in use) if use else None,
                "reasons": reasons, "samples": len(use), "period_ms": self.period * 1e3, "window": window,
                "source": "NVML"}


def clock_sampler(torch_device):
    """NVML polling where the library loads, else the nvidia-smi loop."""
    s = NvmlClockSampler(torch_device)
    return s if s.ok else ClockSampler(torch_device)


def reduce_over_ranks(ms: float, units: float, device) -> tuple[float, float]:
    """Replicas: job time = max over ranks, work = sum over ranks (no collective on the data path)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return t.item(), u.item()


def load_traffic(kernel):
    p = os.path.join(ROOT, "profiles", f"{kernel}_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d
    return None


def run_ours(args, rank, world):
    import ctypes

    import torch

    import __graft_entry__ as g

    g.build()
    import genesis_gb300 as gs
    from genesis_gb300 import _lib

    gs.init(backend=gs.gpu, seed=SEED)
    scene, ents, spacing = build_c2_scene(gs)
    solver = scene.sim.mpm_solver
    n = solver.n_particles
    lib = _lib.load()
    stream = torch.cuda.current_stream()

    # launch-shape autotuning (P2G threads x particles per thread), then warm-up (captures the graph)
    from genesis_gb300.autotune import autotune

    if args.tuning:  # fixed launch shapes (profiling captures, where timings under the profiler mislead)
        t, pp, gt = (int(v) for v in args.tuning.split(","))
        _lib.check(lib.mpm_set_tuning(solver.ctx, t, pp, 1, gt), solver.ctx, "mpm_set_tuning")
        tuning, tune_ms = (t, pp, gt), {}
    else:
        tuning, tune_ms = autotune(solver.ctx, substeps=10, repeats=2, use_cache=False)
    # a fixed pre-roll before the warm-up steps: the timed window then starts at the same point of
    # the trajectory whatever --warmup is, past the particle order of the initial lattice (the
    # first ~60 substeps after a row-ordered state run a few percent faster)
    solver.substeps(PREROLL_SUBSTEPS)
    for _ in range(args.warmup):
        scene.step()
    torch.cuda.synchronize()
    start_state = solver.get_state()  # the per-kernel region below replays the same trajectory

    # --- timed region: K steps of 10 substeps, CUDA graph path, inputs resident in HBM
    clocks = clock_sampler(torch.cuda.current_device())
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.begin()
    e0.record(stream)
    for _ in range(args.steps):
        solver.substeps(SUBSTEPS_PER_STEP)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks.end()
    ms = e0.elapsed_time(e1)
    time.sleep(0.05)
    clk = clocks.stop()
    solver.check_state()
    total_units = n * SUBSTEPS_PER_STEP * args.steps
    if world > 1:
        ms, total_units = reduce_over_ranks(ms, total_units, "cuda")
    value = total_units / (ms / 1e3)

    # --- per-kernel durations over a second timed region: the same K steps from the same state
    # (events around every kernel, no graph)
    solver.set_state(0, start_state)
    solver.substeps(2)
    torch.cuda.synchronize()
    lib.mpm_set_profiling(solver.ctx, 1)
    lib.mpm_kernel_times(solver.ctx, None, None, 1)
    mid_state = None
    for k in range(args.steps):
        solver.substeps(SUBSTEPS_PER_STEP)
        if k == args.steps // 2 - 1:  # the e2e below replays the step from the middle of the trajectory
            mid_state = solver.get_state()
    kms = (ctypes.c_double * 5)()
    kcnt = (ctypes.c_int64 * 5)()
    lib.mpm_kernel_times(solver.ctx, kms, kcnt, 1)
    lib.mpm_set_profiling(solver.ctx, 0)
    touched = ctypes.c_int64()
    _lib.check(lib.mpm_count_touched_nodes(solver.ctx, ctypes.byref(touched), ctypes.c_void_p(stream.cuda_stream)))
    names = ["p2g", "grid_op", "g2p", "scan", "perm"]
    per_kernel = {nm: {"ms_avg": kms[i] / max(1, kcnt[i]), "launches": int(kcnt[i])} for i, nm in enumerate(names)}
    total_k = sum(kms[i] for i in range(5))
    for i, nm in enumerate(names):
        per_kernel[nm]["share"] = kms[i] / total_k if total_k else None
    dom = max(names, key=lambda nm: per_kernel[nm]["ms_avg"] * per_kernel[nm]["launches"])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    bp, bn = ALG_BYTES[dom]
    alg = bp * n + bn * touched.value
    achieved = alg / (per_kernel[dom]["ms_avg"] / 1e3) / 1e9
    substep_ms = total_k / max(1, kcnt[0])
    sub_alg = SUBSTEP_ALG[0] * n + SUBSTEP_ALG[1] * touched.value
    tr = load_traffic(dom)
    roofline = {
        "bound": "hbm",
        "kernel": dom,
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "peak_source": peak_src,
        "traffic": (tr["bytes_per_particle"] * n + tr.get("bytes_per_touched_node", 0) * touched.value) if tr else None,
        "algorithmic_bytes": alg,
        "substep": {"algorithmic_bytes": sub_alg, "ms": substep_ms,
                    "achieved": sub_alg / (substep_ms / 1e3) / 1e9,
                    "frac": sub_alg / (substep_ms / 1e3) / 1e9 / peak},
    }
    if tr and "warp_instructions_per_particle" in tr:
        # the dominant kernel is bound by instruction issue, not HBM: its warp-instruction rate
        # (ncu count per particle x particles / event-timed duration) against the SM issue peak
        # (4 schedulers x SMs x SM clock under load)
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        sm_hz = (clk.get("sm_mhz") or 2070.0) * 1e6
        issue_peak = 4 * props.multi_processor_count * sm_hz
        inst = tr["warp_instructions_per_particle"] * n
        rate = inst / (per_kernel[dom]["ms_avg"] / 1e3)
        roofline["issue"] = {"kernel": dom, "warp_instructions": inst, "achieved": rate / 1e9,
                             "peak": issue_peak / 1e9, "unit": "G warp-instructions/s", "frac": rate / issue_peak}

    # --- e2e: through the public C API with host buffers: every step uploads the full particle
    # state from pinned host memory (mpm_set_state), runs 10 substeps (mpm_substeps) and reads the
    # positions back (mpm_get_state); the copies run on their own streams with double-buffered
    # device staging, so step k's uploads overlap step k-1's substeps and its read-back overlaps
    # step k+1's.  The uploaded state is the one from the middle of the timed trajectory, so the
    # e2e steps simulate the same kind of substeps as the device-timed region.
    st = mid_state if mid_state is not None else solver.get_state()
    keys = ("pos", "vel", "C", "F", "Jp", "active")
    host = {k: (getattr(st, k).to(torch.uint8) if k == "active" else getattr(st, k)).cpu().pin_memory() for k in keys}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    stage = [{k: torch.empty_like(v, device="cuda") for k, v in host.items()} for _ in range(2)]
    dev_out = [torch.empty_like(host["pos"], device="cuda") for _ in range(2)]
    out_host = [torch.empty_like(host["pos"]).pin_memory() for _ in range(2)]
    d2h = out_host[0].numel() * out_host[0].element_size()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    staged = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    produced = [torch.cuda.Event() for _ in range(2)]
    read = [torch.cuda.Event() for _ in range(2)]
    h = ctypes.c_void_p(stream.cuda_stream)
    B = solver._B

    def e2e_step(k):
        b = k % 2
        with torch.cuda.stream(up):  # upload step k's state once step k-2 has consumed the buffer
            up.wait_event(consumed[b])
            for key in keys:
                stage[b][key].copy_(host[key], non_blocking=True)
            staged[b].record(up)
        stream.wait_event(staged[b])
        stream.wait_event(read[b])  # step k-2's positions have left dev_out[b]
        sb = stage[b]
        _lib.check(lib.mpm_set_state(solver.ctx, 0, B, sb["pos"].data_ptr(), sb["vel"].data_ptr(), sb["C"].data_ptr(),
                                     sb["F"].data_ptr(), sb["Jp"].data_ptr(), sb["active"].data_ptr(), h), solver.ctx,
                   "mpm_set_state")
        consumed[b].record(stream)
        _lib.check(lib.mpm_substeps(solver.ctx, SUBSTEPS_PER_STEP, h), solver.ctx, "mpm_substeps")
        _lib.check(lib.mpm_get_state(solver.ctx, 0, B, dev_out[b].data_ptr(), None, None, None, None, None, h),
                   solver.ctx, "mpm_get_state")
        produced[b].record(stream)
        with torch.cuda.stream(down):
            down.wait_event(produced[b])
            out_host[b].copy_(dev_out[b], non_blocking=True)
            read[b].record(down)

    for k in range(2):
        e2e_step(k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": n * SUBSTEPS_PER_STEP * args.steps * world / e2e_s, "unit": "particle-substeps/s",
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    result = {
        "metric": METRIC,
        "value": value,
        "unit": "particle-substeps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded jittered lattices)",
        "config": {
            "workload": "plain large: 129^3-node grid, ~1M particles (liquid 0.3^3 + sand 0.2^3 + elastic sphere "
                        "r=0.1), dt=1e-4, step = 10 substeps",
            "n_particles": n,
            "substeps_per_step": SUBSTEPS_PER_STEP,
            "touched_nodes": touched.value,
            "parallelism": "replicas only" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (particle state double buffer 2 x 108 MB)",
            "path": "CUDA graph of 2 substeps",
            "timed_window": f"substeps {PREROLL_SUBSTEPS + SUBSTEPS_PER_STEP * args.warmup} to "
                            f"{PREROLL_SUBSTEPS + SUBSTEPS_PER_STEP * (args.warmup + args.steps)} of the trajectory "
                            f"(after a {PREROLL_SUBSTEPS}-substep pre-roll and the warm-up steps)",
            "p2g_tuning": {"threads": tuning[0], "particles_per_thread": tuning[1], "g2p_threads": tuning[2],
                           "ms_per_substep": {k: round(v, 4) for k, v in tune_ms.items()}},
        },
        "roofline": roofline,
        "kernels": per_kernel,
        "e2e": e2e,
        "gpu_launches": KERNELS_PER_SUBSTEP * SUBSTEPS_PER_STEP * args.steps,
        "clocks": clk,
    }
    if rank == 0 and not args.skip_forms:
        result["forms"] = run_forms()
        result["forms"]["differentiation"] = run_diff()
        result["forms"]["differentiation"]["scene_api"] = run_diff_scene()
    if rank == 0 and not args.skip_cpu:
        result["cpu_baseline"] = cpu_baseline()
    return result


def validate_line(d: dict) -> None:
    """Checks the shape of the JSON line (keys and types the consumers read); raises ValueError
    naming the first key that is missing or of the wrong type."""
    num = (int, float)

    def need(obj, key, typ, where):
        if key not in obj or isinstance(obj[key], bool) != (typ is bool) or not isinstance(obj[key], typ):
            raise ValueError(f"{where}{key}: expected {typ}, got {obj.get(key)!r}")

    if d.get("impl") == "reference":
        if "unavailable" in d:
            need(d, "unavailable", str, "")
            return
        for k, t in (("metric", str), ("value", num), ("unit", str), ("cpu_baseline", dict), ("e2e", dict)):
            need(d, k, t, "")
    else:
        for k, t in (("metric", str), ("value", num), ("unit", str), ("n_gpus", int), ("steps", int),
                     ("warmup", int), ("ms_per_step", num), ("higher_is_better", bool), ("scaling", str),
                     ("dtype", str), ("data", str), ("config", dict), ("roofline", dict), ("e2e", dict),
                     ("gpu_launches", int), ("clocks", dict)):
            need(d, k, t, "")
        need(d["config"], "workload", str, "config.")
        for k, t in (("bound", str), ("achieved", num), ("peak", num), ("unit", str), ("frac", num)):
            need(d["roofline"], k, t, "roofline.")
        if "traffic" not in d["roofline"] or not (d["roofline"]["traffic"] is None
                                                   or isinstance(d["roofline"]["traffic"], num)):
            raise ValueError("roofline.traffic: expected a number or null")
        need(d["clocks"], "reasons", list, "clocks.")
        for k in ("sm_mhz", "sm_max_mhz"):
            if k not in d["clocks"] or not (d["clocks"][k] is None or isinstance(d["clocks"][k], num)):
                raise ValueError(f"clocks.{k}: expected a number or null")
    for k, t in (("value", num), ("unit", str), ("h2d_bytes_per_step", int), ("d2h_bytes_per_step", int)):
        need(d["e2e"], k, t, "e2e.")
    if "cpu_baseline" in d:
        for k, t in (("value", num), ("unit", str), ("cores", int), ("kind", str), ("sample", str)):
            need(d["cpu_baseline"], k, t, "cpu_baseline.")
        if d["cpu_baseline"]["kind"] not in ("reference", "port"):
            raise ValueError("cpu_baseline.kind: expected 'reference' or 'port'")


def _timed(fn):
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def run_c1(substeps=100, repeats=5):
    """The small plain case: 17,576-particle elastic cube (side 0.2 at (0.5, 0.5, 0.4), regular
    sampler at particle size 1/128, jitter +-0.25 dx) on a 65^3 grid, dt = 2e-4, 100 substeps.
    Its particle state (~4 MB) is L2-resident and the substep is launch-bound."""
    import torch

    import genesis_gb300 as gs

    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=2e-4, substeps=1),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=64,
                                                       particle_size=1.0 / 128))
    cube = scene.add_entity(material=gs.materials.MPM.Elastic(sampler="regular"),
                            morph=gs.morphs.Box(pos=(0.5, 0.5, 0.4), size=(0.2, 0.2, 0.2)))
    scene.build()
    rng = np.random.default_rng(SEED)
    p = cube.init_particles + rng.uniform(-0.25 / 64, 0.25 / 64, size=cube.init_particles.shape)
    cube.set_particles_pos(torch.tensor(p, dtype=torch.float32, device="cuda"))
    solver = scene.sim.mpm_solver
    n = solver.n_particles
    solver.substeps(substeps)
    t = min(_timed(lambda: solver.substeps(substeps)) for _ in range(repeats))
    solver.check_state()
    return {"workload": "17,576-particle elastic cube, 65^3 grid, dt 2e-4, 100 substeps (L2-resident)",
            "n_particles": n, "value": n * substeps / t, "us_per_substep": t / substeps * 1e6,
            "unit": "particle-substeps/s"}


def run_dense(steps=20):
    """The same three-material scene at 4 particles per cell per axis (spacing dx / 4, ~5.3M
    particles, the density the config names literally), graph path, 10 substeps per step."""
    import genesis_gb300 as gs

    scene, ents, spacing = build_c2_scene(gs, spacing=1.0 / (4 * GRID_DENSITY))
    solver = scene.sim.mpm_solver
    n = solver.n_particles
    solver.substeps(2 * SUBSTEPS_PER_STEP)
    t = _timed(lambda: [solver.substeps(SUBSTEPS_PER_STEP) for _ in range(steps)])
    solver.check_state()
    out = {"workload": f"three-material scene at 4 particles per cell per axis ({n} particles), 129^3, "
                       f"{steps} steps x {SUBSTEPS_PER_STEP} substeps", "n_particles": n,
           "value": n * SUBSTEPS_PER_STEP * steps / t, "unit": "particle-substeps/s"}
    solver.destroy()
    return out


def run_forms(batched_substeps=200, n_requests=48):
    """Batched (256 uneven scenes, one context) and served (continuous batching) forms, each
    against the plain form run scene by scene (one context per scene) on the same workload."""
    from genesis_gb300 import _lib
    from genesis_gb300.batched import BatchedMPM, batched_workload
    from genesis_gb300.serve import MPMServer, serving_workload

    out = {"plain_small": run_c1(), "plain_dense": run_dense()}
    specs = batched_workload(n_scenes=256, seed=1234)
    b = BatchedMPM(specs, tune=True)
    b.step(2)
    t = _timed(lambda: b.step(batched_substeps))
    st = b.check()
    n_b = b.n_particles
    tuning = b.tuning[0] if b.tuning else None
    b.close()
    t_plain = 0.0
    for sp in specs:
        one = BatchedMPM([sp], tune=False)
        one.step(2)
        t_plain += _timed(lambda: one.step(batched_substeps))
        one.close()
    out["batched"] = {
        "workload": "256 scenes, 65^3 grids each, N ~ logU[2k,64k], Elastic/Liquid/Sand/Snow, extent U[0.1,0.3], "
                    f"dt 2e-4, {batched_substeps} substeps",
        "n_scenes": len(specs), "n_particles": n_b, "value": n_b * batched_substeps / t,
        "plain_scene_by_scene": n_b * batched_substeps / t_plain, "speedup_vs_plain": t_plain / t,
        "p2g_tuning": tuning, "status": st, "unit": "particle-substeps/s",
    }
    # served: the same request set (a) saturated (all arrive at once) for throughput, against each
    # request run alone in turn; (b) Poisson arrivals at half the saturated rate for p50/p99 latency
    reqs = serving_workload(n_requests=n_requests, rate_hz=0, seed=77, with_payload=True)
    work = sum(r.work for r in reqs)
    srv = MPMServer(max_slots=64, particle_capacity=40_000_000, max_grid_res=129, chunk=10)
    sat = srv.run(reqs, realtime=False)
    t_alone = 0.0
    for r in reqs:  # GPU time of each request's substeps alone (the plain form, setup excluded)
        one = BatchedMPM([r.spec], tune=False, positions=[r.payload])
        one.step(2)
        t_alone += _timed(lambda: one.step(r.spec.substeps))
        one.close()
    # each request end to end through the plain form, one after another: context creation, upload
    # of its payload, its substeps, read-back of its positions, teardown (wall clock, as the served
    # run is timed)
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        one = BatchedMPM([r.spec], tune=False, positions=[r.payload])
        one.step(r.spec.substeps)
        pos = torch.empty((r.spec.n_particles, 3), device="cuda")
        _lib.check(one.lib.mpm_get_state(one.ctx, 0, 1, pos.data_ptr(), None, None, None, None, None,
                                         one._stream()), one.ctx, "mpm_get_state")
        pos.cpu()
        one.close()
    t_alone_wall = time.perf_counter() - t0
    mean_work = work / len(reqs)
    rate = 0.5 * sat["throughput"] / mean_work
    reqs2 = serving_workload(n_requests=n_requests, rate_hz=rate, seed=77, with_payload=True)
    live = srv.run(reqs2, realtime=True)
    srv.close()
    out["served"] = {
        "workload": f"{n_requests} requests, N ~ logU[1k,500k], grid 33^3/65^3/129^3, substeps U[50,500], "
                    "4 materials; continuous batching in one pool context",
        "throughput_saturated": sat["throughput"], "plain_alone_sequential": work / t_alone,
        "speedup_vs_plain": sat["throughput"] / (work / t_alone),
        "plain_alone_end_to_end": work / t_alone_wall,
        "speedup_vs_plain_end_to_end": sat["throughput"] / (work / t_alone_wall),
        "poisson_rate_hz": rate, "throughput_poisson": live["throughput"],
        "p50_latency_s": live["p50_s"], "p99_latency_s": live["p99_s"], "status": sat["status"] | live["status"],
        "unit": "particle-substeps/s",
    }
    return out


def run_served_only(n_requests=48):
    """The served form's saturated run alone (one warm-up run, then the measured one): the
    workload of run_forms, for profiling captures of the pool's kernels."""
    import __graft_entry__ as g

    g.build()
    from genesis_gb300.serve import MPMServer, serving_workload

    srv = MPMServer(max_slots=64, particle_capacity=40_000_000, max_grid_res=129, chunk=10)
    srv.run(serving_workload(n_requests=n_requests, rate_hz=0, seed=77, with_payload=True), realtime=False)
    sat = srv.run(serving_workload(n_requests=n_requests, rate_hz=0, seed=77, with_payload=True), realtime=False)
    srv.close()
    return {"form": "served (saturated)", "throughput": sat["throughput"], "wall_s": sat["wall_s"],
            "chunks": sat["chunks"], "status": sat["status"]}


def diff_config(seed=99):
    """The differentiation workload: a ~216k-particle elastic cube (60^3 lattice at 1/240 m, jittered)
    2 cm above the floor boundary of a 97^3 grid (density 96, dt 1e-4, gravity on), per-particle
    E ~ LogNormal(ln 3e5, 0.2), nu 0.2, rho 1000, v0 = (0.1, 0, -1), a random COM target.
    Returns (scene config, x0 [n, 3], E [n], v0 [3], target [3]) as numpy arrays."""
    from genesis_gb300 import _lib

    rng = np.random.default_rng(seed)
    cfg = _lib.MpmSceneConfig()
    cfg.substep_dt = 1e-4
    for d in range(3):
        cfg.gravity[d] = (0.0, 0.0, -9.81)[d]
        cfg.lower_bound[d], cfg.upper_bound[d] = 0.0, 1.0
    cfg.grid_density = 96.0
    cfg.particle_size = 1.0 / 240
    cfg.mass_eps = float(np.finfo(np.float32).eps)
    side = 60
    ax = 0.5 + (np.arange(side) - (side - 1) / 2) / 240.0
    x0 = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
    x0[:, 2] += 0.18 - 0.5  # 2 cm above the floor boundary: the fall ends in contact, so E shapes the COM
    x0 = x0 + rng.uniform(-0.25 / 240, 0.25 / 240, size=x0.shape)
    E = 3e5 * np.exp(0.2 * rng.normal(size=len(x0)))
    v0 = np.array([0.1, 0.0, -1.0])
    target = rng.uniform(0.3, 0.7, size=3)
    return cfg, x0, E, v0, target


def run_diff(steps=64, substeps_per_step=10, ckpt_steps=16, seed=99):
    """Differentiation config (diff_config): 64 steps x 10 substeps, checkpoint every 16 steps;
    loss = ||COM - target||^2; gradients w.r.t. the initial velocity and every particle's E.
    Reports forward+backward particle-substeps/s (forward substeps counted once)."""
    import torch

    from genesis_gb300.diff import DifferentiableMPM

    cfg, x0, E_np, v0_np, target_np = diff_config(seed)
    n = len(x0)
    E = torch.tensor(E_np, dtype=torch.float32, device="cuda", requires_grad=True)
    v0 = torch.tensor(v0_np, dtype=torch.float32, device="cuda", requires_grad=True)
    target = torch.tensor(target_np, dtype=torch.float32, device="cuda")
    sim = DifferentiableMPM(cfg, nu=0.2, rho=1000.0, ckpt_every=ckpt_steps * substeps_per_step)
    x = torch.tensor(x0, dtype=torch.float32, device="cuda")
    n_sub = steps * substeps_per_step

    def fwd_bwd():
        loss = ((sim.rollout(x, v0, E, n_sub).mean(0) - target) ** 2).sum()
        loss.backward()
        return loss

    torch.cuda.empty_cache()  # the earlier forms' cached blocks: the backward sizes its segments by free memory
    free_gb = torch.cuda.mem_get_info()[0] / 1e9
    # warm-up: one whole forward + backward (the first one also pays the allocation of the ~8 GB of
    # segment states and grids, several seconds on some boxes), then the timed one
    fwd_bwd()
    v0.grad = None
    E.grad = None
    t = _timed(fwd_bwd)
    g_v0, g_E = v0.grad.tolist(), float(E.grad.norm())
    # the same rollout keeping every segment's states and grids (the backward re-simulates none)
    sim.keep_segments = True
    fwd_bwd()
    v0.grad = None
    E.grad = None
    t_keep = _timed(fwd_bwd)
    keep_mode = getattr(sim, "last_backward", None)
    kept, total = getattr(sim, "last_segments", (None, None))
    return {
        "workload": f"elastic cube {n} particles, 97^3 grid, {steps} steps x {substeps_per_step} substeps, "
                    f"checkpoint every {ckpt_steps} steps, grads w.r.t. v0 and per-particle E",
        "n_particles": n, "seconds_fwd_bwd": t, "value": n * n_sub / t, "unit": "particle-substeps/s (fwd+bwd)",
        "grad_v0": g_v0, "grad_E_norm": g_E, "backward_mode": getattr(sim, "last_backward", None),
        "free_device_gb": free_gb,
        "keep_segments": {"seconds_fwd_bwd": t_keep, "value": n * n_sub / t_keep, "backward_mode": keep_mode,
                          "segments_kept": kept, "segments": total,
                          "grad_v0": v0.grad.tolist(), "grad_E_norm": float(E.grad.norm())},
    }


def run_diff_scene(steps=64, substeps_per_step=10, seed=99):
    """The differentiation rollout through the reference's own API: SimOptions(requires_grad=True),
    the cube as one Elastic entity (E = 3e5, nu 0.2, rho 1000: one material per entity, as that API
    gives it; a 0.25 m box at particle size 1/240 on the same 97^3 grid, dt 1e-4), a v0 tensor
    through entity.set_velocity, `steps` scene.step() calls, the COM loss on get_state().pos and
    loss.backward().  Each step is a checkpoint, re-simulated in the backward.  Timed: scene.reset()
    through the backward, host loop included."""
    import torch

    import genesis_gb300 as gs

    if not gs._initialized:
        gs.init(backend=gs.gpu, seed=SEED)
    _, _, _, v0_np, target_np = diff_config(seed)
    scene = gs.Scene(sim_options=gs.options.SimOptions(dt=substeps_per_step * 1e-4, substeps=substeps_per_step,
                                                       requires_grad=True),
                     mpm_options=gs.options.MPMOptions(lower_bound=(0, 0, 0), upper_bound=(1, 1, 1), grid_density=96,
                                                       particle_size=1.0 / 240))
    cube = scene.add_entity(material=gs.materials.MPM.Elastic(E=3e5, nu=0.2, rho=1000.0, sampler="regular"),
                            morph=gs.morphs.Box(pos=(0.5, 0.5, 0.18), size=(0.25, 0.25, 0.25)))
    scene.build()
    target = torch.tensor(target_np, dtype=torch.float32, device="cuda")
    out = {}

    def fwd_bwd():
        scene.reset()
        v0 = torch.tensor(v0_np, dtype=torch.float32, device="cuda", requires_grad=True)
        cube.set_velocity(v0)
        for _ in range(steps):
            scene.step()
        loss = ((cube.get_state().pos[0].mean(0) - target) ** 2).sum()
        loss.backward()
        out["v0"] = v0

    fwd_bwd()
    t = _timed(fwd_bwd)
    n = cube.n_particles
    res = {"n_particles": n, "seconds_fwd_bwd": t, "value": n * steps * substeps_per_step / t,
           "grad_v0": out["v0"].grad.tolist()}
    scene.sim.mpm_solver.destroy()
    return res


def run_reference(args):
    """The CPU implementation of the path (oracle restatement), all host cores, same metric."""
    O, sc, oms, st = oracle_c2_state()
    cores = os.cpu_count() or 1
    n = len(st["pos"])
    for _ in range(args.warmup):
        st, _, _ = O.run(sc, oms, st, 1, dtype=np.float32, threads=cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st, _, _ = O.run(sc, oms, st, 1, dtype=np.float32, threads=cores)
    dt = time.perf_counter() - t0
    v = n * args.steps / dt
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": "particle-substeps/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded jittered lattices)",
        "config": {"workload": "plain large: 129^3-node grid, ~1M particles (liquid 0.3^3 + sand 0.2^3 + elastic sphere "
                               "r=0.1), dt=1e-4, step = 10 substeps",
                   "n_particles": n, "reference_step": "1 substep of the whole scene on the host cores (bounded "
                                                        "sample; the metric is per particle-substep)"},
        "cpu_baseline": {"value": v, "unit": "particle-substeps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} substeps of the full {n}-particle scene, fp32, OpenMP {cores} threads"},
        "e2e": {"value": v, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "The reference (Genesis + Quadrants JIT) is not installable here; this is the oracle restatement "
                "of its algorithm on the host cores.",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-forms", action="store_true", help="skip the batched/served form measurements")
    ap.add_argument("--tuning", default="", help="fixed P2G threads,particles per thread,G2P threads (no autotune)")
    ap.add_argument("--form", default="", choices=["", "served", "differentiation"],
                    help="diagnostic: run only the saturated served workload or the differentiation rollout "
                         "(for profiling captures)")
    ap.add_argument("--diff-steps", type=int, default=64, help="steps of the differentiation rollout (--form)")
    args = ap.parse_args()
    if args.form == "served":
        print(json.dumps(run_served_only()))
        return
    if args.form == "differentiation":
        d = run_diff(steps=args.diff_steps)
        d["scene_api"] = run_diff_scene(steps=args.diff_steps)
        print(json.dumps(d))
        return
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            line = run_reference(args)
            validate_line(line)
            print(json.dumps(line))
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    if rank == 0:
        validate_line(res)
        print(json.dumps(res))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
