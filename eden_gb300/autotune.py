"""Autotuner of the batched path's launch shape.

Three knobs decide how the windowed kernels cover a network
(`EdenGpuOptions`, include/eden_gpu.h):

* steps_per_launch -- the window length K, the steps one launch advances
  (at most the exact bound min(31, min delay / dt));
* segments_per_warp -- the most compartments one warp's forest of cells
  holds (its shared-memory slice and its share of the work);
* segments_per_depth -- the most compartments of a forest at one depth
  (the width of each step of the depth-by-depth cable solve).

`tune()` times the batched path on the network itself for candidate values,
one knob at a time starting from the built-in choice (coordinate descent),
keeps the fastest, and caches the result per network and device so that the
search runs once.  Every candidate computes the same network: the packing
changes neither a compartment's operations nor a cell's elimination order,
and a window is exact for any length up to the bound, so the tuned run
differs from the default only by the rounding of the synapses' closed-form
decay across window boundaries.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

import numpy as np

KNOBS = ("segments_per_depth", "segments_per_warp", "steps_per_launch")
MAX_WINDOW = 31


def window_bound(low) -> int:
    """The longest exact window: every connection delay covers it."""
    if len(low.syn_delay) == 0:
        return MAX_WINDOW
    k = int(np.floor(float(np.min(low.syn_delay)) / float(low.dt)))
    return max(1, min(MAX_WINDOW, k))


def candidates(low) -> dict:
    """Values tried for each knob; 0 is the built-in choice."""
    kmax = window_bound(low)
    steps = sorted({0, max(1, kmax // 2), max(1, kmax // 4)}, key=lambda k: (k != 0, -k))
    if low.n_comp == 0:
        return {"segments_per_depth": [0], "segments_per_warp": [0], "steps_per_launch": steps}
    return {"segments_per_depth": [0, 32, 128],
            "segments_per_warp": [0, 512, 384, 256, 192, 64, 1023],
            "steps_per_launch": steps}


def fingerprint(low, device_name: str = "") -> str:
    """Digest of what the launch shape depends on: sizes, cell structure,
    channel layout, input placement and delays."""
    h = hashlib.sha1()
    h.update(device_name.encode())
    h.update(np.float32(low.dt).tobytes())
    for a in (low.phys_comp_off, low.comp_parent, low.comp_chan_off, low.chan_type, low.syn_target,
              low.syn_type, low.pois_target, low.pulse_target):
        arr = np.ascontiguousarray(a)
        h.update(str(arr.shape).encode())
        h.update(arr.tobytes())
    h.update(np.float32(np.min(low.syn_delay) if len(low.syn_delay) else 0).tobytes())
    h.update(str(low.n_izh).encode())
    return h.hexdigest()


def _cache_path(path: str | None) -> str:
    if path:
        return path
    env = os.environ.get("EDEN_GB300_TUNE_CACHE")
    if env:
        return env
    return os.path.join(os.path.expanduser("~"), ".cache", "eden_gb300", "autotune.json")


def measure_gpu(low, config: dict, device: int = 0, steps: int = 320, repeats: int = 3) -> float:
    """Device ms per simulation step of the batched path with `config`
    (the best of `repeats` timed runs of `steps` steps after a warm-up)."""
    from .engine import MODE_BATCHED, Simulation
    sim = Simulation(low, mode=MODE_BATCHED, device=device, record_capacity_steps=steps + 64,
                     spike_capacity=1 << 24, **config)
    try:
        sim.initialize()
        sim.run_steps(steps)
        sim.fetch()
        best = float("inf")
        for _ in range(repeats):
            ms = sim.run_steps(steps)
            sim.fetch()
            best = min(best, ms / steps)
        return best
    finally:
        sim.close()


def search(low, measure) -> tuple[dict, list]:
    """Coordinate descent over the knobs; `measure(config) -> ms per step`."""
    cands = candidates(low)
    best = {k: 0 for k in KNOBS}
    seen = {}

    def cost(cfg):
        key = tuple(cfg[k] for k in KNOBS)
        if key not in seen:
            seen[key] = measure(dict(cfg))
        return seen[key]

    best_ms = cost(best)
    for knob in KNOBS:
        for v in cands[knob]:
            trial = dict(best, **{knob: v})
            ms = cost(trial)
            if ms < best_ms:
                best, best_ms = trial, ms
    tried = [dict(zip(KNOBS, k), ms_per_step=v) for k, v in seen.items()]
    return dict(best, ms_per_step=best_ms), tried


def tune(low, device: int = 0, cache: str | None = None, measure=None, device_name: str | None = None) -> dict:
    """The fastest launch shape for `low` on `device`: a dict of the three
    knobs (0 = built-in choice) plus ms_per_step, the search time and the
    candidates tried (empty when the result came from the cache)."""
    if device_name is None:
        try:
            import torch
            device_name = torch.cuda.get_device_name(device)
        except Exception:
            device_name = "unknown"
    key = fingerprint(low, device_name)
    path = _cache_path(cache)
    store = {}
    if os.path.exists(path):
        try:
            with open(path) as f:
                store = json.load(f)
        except (OSError, ValueError):
            store = {}
    if key in store:
        return dict(store[key], search_s=0.0, tried=[], cached=True)
    if measure is None:
        def measure(cfg):
            return measure_gpu(low, cfg, device)
    t0 = time.perf_counter()
    best, tried = search(low, measure)
    out = dict(best, search_s=time.perf_counter() - t0, tried=tried, cached=False)
    store[key] = {k: best[k] for k in list(KNOBS) + ["ms_per_step"]}
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        with open(path + ".tmp", "w") as f:
            json.dump(store, f)
        os.replace(path + ".tmp", path)
    except OSError:
        pass
    return out


def options(result: dict) -> dict:
    """The Simulation keyword arguments of a tune() result."""
    return {k: int(result[k]) for k in KNOBS}
