"""Autotuner of the launch shapes (P2G threads per CTA x particles per thread, G2P threads).

The work chunk of one P2G CTA is threads * particles_per_thread particles of one grid
block's bucket.  Larger chunks amortise the shared-tile clear/flush over more particles;
smaller chunks spread sparse or uneven scenes over more SMs.  The tuner times each
candidate with CUDA events over a few substeps of the caller's own context, keeps the
fastest, and caches the choice per workload signature (particle count, grid blocks, scene
count, rounded to powers of two) in a JSON file.
"""

from __future__ import annotations

import ctypes
import json
import math
import os

import torch

from . import _lib

# (P2G threads, particles per thread, G2P threads); P2G threads * ppt <= 1024
CANDIDATES = ((64, 1, 128), (64, 2, 128), (128, 1, 128), (128, 2, 128), (128, 4, 128), (256, 1, 128),
              (256, 2, 128), (256, 4, 128), (128, 2, 64), (128, 2, 256))
DEFAULT = (128, 2, 128)  # a new context's launch shapes (libgbmpm) ...
DEFAULT_SMALL = (64, 1, 128)  # ... below SMALL_PARTICLES particles
SMALL_PARTICLES = 65536
# another candidate replaces DEFAULT only when it is faster by more than this fraction: short
# timing windows on the starting state cannot resolve smaller differences, which later states of
# the same run can reverse
MARGIN = 0.01
CACHE_PATH = os.environ.get(
    "GBMPM_AUTOTUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "genesis_gb300", "autotune.json")
)


def signature(ctx) -> str:
    lib = _lib.load()
    n, k, s = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    lib.mpm_get_info(ctx, ctypes.byref(n), ctypes.byref(k), ctypes.byref(s))
    r = lambda v: 2 ** int(round(math.log2(max(1, v))))  # noqa: E731
    return f"n{r(n.value)}_k{r(k.value)}_s{r(s.value)}"


def _load_cache() -> dict:
    try:
        with open(CACHE_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(c: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        with open(CACHE_PATH, "w") as f:
            json.dump(c, f, indent=1)
    except OSError:
        pass


def choose(timings: dict, candidates=CANDIDATES, default=DEFAULT) -> tuple:
    """Fastest candidate of `timings` ({"TxP/G": ms}); `default` unless beaten by more than MARGIN."""
    key = lambda c: timings[f"{c[0]}x{c[1]}/{c[2]}"]  # noqa: E731
    best = min(candidates, key=key)
    if default in candidates and key(best) > (1.0 - MARGIN) * key(default):
        return default
    return best


def autotune(ctx, substeps: int = 10, repeats: int = 2, use_cache: bool = True, candidates=CANDIDATES):
    """Pick (threads, ppt) for `ctx`; returns (choice, {candidate: ms_per_substep}).

    The timing substeps advance the context's state: callers tune on a scratch copy of the
    state or reset it afterwards."""
    lib = _lib.load()
    sig = signature(ctx)
    cache = _load_cache() if use_cache else {}
    if sig in cache and len(cache[sig]["choice"]) == 3:
        t, p, g = cache[sig]["choice"]
        _lib.check(lib.mpm_set_tuning(ctx, t, p, 1, g), ctx, "mpm_set_tuning")
        return (t, p, g), cache[sig].get("timings", {})
    stream = torch.cuda.current_stream()
    h = ctypes.c_void_p(stream.cuda_stream)
    timings = {}
    for t, p, g in candidates:
        _lib.check(lib.mpm_set_tuning(ctx, t, p, 1, g), ctx, "mpm_set_tuning")
        _lib.check(lib.mpm_substeps(ctx, 2, h), ctx, "mpm_substeps")  # warm-up + graph capture
        best = float("inf")
        for _ in range(repeats):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(lib.mpm_substeps(ctx, substeps, h), ctx, "mpm_substeps")
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / substeps)
        timings[f"{t}x{p}/{g}"] = best
    n = ctypes.c_int64()
    lib.mpm_get_info(ctx, ctypes.byref(n), None, None)
    choice = choose(timings, candidates, DEFAULT_SMALL if n.value < SMALL_PARTICLES else DEFAULT)
    _lib.check(lib.mpm_set_tuning(ctx, choice[0], choice[1], 1, choice[2]), ctx, "mpm_set_tuning")
    cache[sig] = {"choice": list(choice), "timings": timings}
    if use_cache:
        _save_cache(cache)
    return choice, timings
