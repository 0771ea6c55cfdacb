"""Launch-shape tuner of the batched step, with an on-disk cache.

Candidates: threads per block x tile size (cells per tile) x grid (persistent
blocks walking the tile table, or one block per tile). Each candidate
is timed with CUDA events over a few steps of the actual batch (the pools
are saved before and restored after, so tuning does not advance the
simulation). The fastest is stored under a key made of the device name,
stencil, storage, collision and the sorted domain sizes, in
``$LGB_AUTOTUNE_CACHE`` (default ``~/.cache/lettuce_gb300/autotune.json``).
"""
from __future__ import annotations

import hashlib
import json
import os

import torch

THREADS = (128, 256, 512)
TILE_CELLS = (1024, 2048, 4096, 8192, 16384)


def cache_path() -> str:
    return os.environ.get("LGB_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "lettuce_gb300",
                                       "autotune.json"))


def _key(sim) -> str:
    sizes = sorted(tuple(int(v) for v in d["res"]) for d in sim.domains)
    h = hashlib.sha1(json.dumps(sizes).encode()).hexdigest()[:16]
    name = torch.cuda.get_device_name(sim.context.device)
    return f"{name}|{sim.stencil.lgb_id}|{sim.context.storage}|{sim.collision_id}|{h}"


def _load() -> dict:
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def lookup(sim):
    return _load().get(_key(sim))


def time_config(sim, threads: int, tile_cells: int, persistent: bool = True, steps: int = 10,
                warmup: int = 3) -> float:
    """milliseconds per step of one launch shape (eager launches)"""
    sim._configure(threads, tile_cells, persistent)
    stream = torch.cuda.current_stream(sim.context.device)
    for _ in range(warmup):
        sim.step_once()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        sim.step_once()
    end.record(stream)
    torch.cuda.synchronize(sim.context.device)
    return start.elapsed_time(end) / steps


def tune(sim, save: bool = True) -> dict:
    saved = [p.clone() for p in sim._pools]
    cur = sim._cur
    best = None
    results = {}
    try:
        for t in THREADS:
            for c in TILE_CELLS:
                for pers in (True, False):
                    ms = time_config(sim, t, c, pers)
                    results[f"{t}x{c}{'' if pers else 'x1'}"] = ms
                    if best is None or ms < best[0]:
                        best = (ms, t, c, pers)
    finally:
        for p, s in zip(sim._pools, saved):
            p.copy_(s)
        sim._cur = cur
        torch.cuda.synchronize(sim.context.device)
    cfg = {"threads": best[1], "tile_cells": best[2], "persistent": best[3],
           "ms_per_step": best[0]}
    if save:
        data = _load()
        data[_key(sim)] = cfg
        path = cache_path()
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(data, fh, indent=1)
            os.replace(tmp, path)
        except OSError:
            pass
    sim.tuning_results = results
    return cfg
