"""Autotuner for the launch shape of a workload.

The reference fixes its workgroup sizes at compile time
(runners/bevy/src/compute/builder.rs:16, 01_integration.rs:36-40,
assets/shaders/prefix_sum.wgsl:9-15) and lists changing them as a TODO
(README.md:28).  Here the launch shape is a per-context setting, and `tune`
picks it by timing candidates on the workload itself:

  solve_block       threads per block of the solve kernels
  solve_per_thread  particles each thread of the extended solve takes in
                    turn (32 x this = particles per warp); the grid shrinks
                    by the same factor
  rebin_blocks      the grid of the rebin's large-cell sort (its blocks loop
                    over the cells of more than 64 particles; default 8 per SM)
  cell_size      only when the caller passes `cell_sizes`: it is a physics
                 change, not a launch shape -- it changes which particles
                 share a cell, hence the capacity rule and the summation order
                 (results stay deterministic but are not those of another cell
                 size)

A launch shape never changes results: every candidate steps the same frames
bit for bit.

Results are cached as JSON, keyed by GPU name and the workload's shape, so
later runs skip the timing.
"""
import dataclasses
import json
import math
import os
import time

import numpy as np

from . import api


def cache_path():
    return os.environ.get("WRACH_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "wrach_gb300",
                                       "autotune.json"))


def workload_key(gpu, config, nworlds, particles, cells, tune_cell_size):
    """Cache key: the GPU and the workload's shape (sizes rounded to powers
    of two), not its contents."""
    return "|".join([
        gpu, "mode%d" % config.mode, "it%d" % config.iterations, "cap%d" % config.cell_capacity,
        "w%d" % nworlds, "p2^%d" % round(math.log2(max(particles, 1))),
        "c2^%d" % round(math.log2(max(cells, 1))),
        "cs*" if tune_cell_size else "cs%d" % config.cell_size,
    ])


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0).replace("|", "/")
    except Exception:
        return "unknown-gpu"


def _upload(sim, positions, velocities, worlds):
    if worlds is None:
        sim.set_particles(positions, velocities)
    else:
        for w, (p, v) in enumerate(zip(positions, velocities)):
            sim.set_particles(p, v, world=w)


def _time_frames(sim, frames):
    sim.step(2)
    sim.sync()
    t0 = time.perf_counter()
    sim.step(frames)
    sim.sync()
    return (time.perf_counter() - t0) * 1000.0 / frames


LAUNCH_KNOBS = ("solve_block", "solve_per_thread", "rebin_blocks")


def launch_shape(config):
    """The tuned knobs of a config (cell size included)."""
    return {k: getattr(config, k) for k in ("cell_size",) + LAUNCH_KNOBS}


def tune(config, positions, velocities, worlds=None, frames=10, rebin_blocks=None,
         solve_blocks=(128, 256, 512), per_thread=(1, 2, 4), cell_sizes=None, use_cache=True,
         path=None):
    """Returns (tuned config, {candidate: ms per frame}).  `positions` and
    `velocities` are one (n, 2) array each, or one per world when `worlds`
    (a list of (width, height)) is given.  For each cell size, the solve's
    block size and particles per thread are tuned together, then the
    rebin's large-cell grid (`rebin_blocks`, default 4, 8 and 16 blocks per
    SM) for the best of those.  `cell_sizes` (e.g. (1, 2)) lets the tuner
    change the cell size, which changes the physics."""
    tune_cs = bool(cell_sizes)
    cell_sizes = tuple(cell_sizes) if cell_sizes else (config.cell_size,)
    probe = api.Simulation(dataclasses.replace(config), worlds=worlds)
    try:
        stats = probe.stats()
        particles = sum(len(p) for p in positions) if worlds is not None else len(positions)
        per_sm8 = stats["rebin_blocks"]  # the default: 8 blocks per SM
        key = workload_key(_gpu_name(), config, probe.num_worlds, particles, stats["cells"], tune_cs)
    finally:
        probe.close()
    cache = load_cache(path) if use_cache else {}
    if use_cache and key in cache:
        return dataclasses.replace(config, **cache[key]["choice"]), cache[key]["ms"]
    if rebin_blocks is None:
        rebin_blocks = (per_sm8 // 2, per_sm8, per_sm8 * 2)
    timings = {}

    def run(**knobs):
        cand = dataclasses.replace(config, **knobs)
        with api.Simulation(cand, worlds=worlds) as sim:
            _upload(sim, positions, velocities, worlds)
            ms = _time_frames(sim, frames)
        label = ",".join("%s=%d" % (k, knobs[k]) for k in ("cell_size",) + LAUNCH_KNOBS)
        timings[label] = ms
        return ms

    best, best_ms = None, float("inf")
    for cs in cell_sizes:
        shape, shape_ms = None, float("inf")
        for sb in solve_blocks:
            for pt in per_thread:
                ms = run(cell_size=cs, solve_block=sb, solve_per_thread=pt, rebin_blocks=per_sm8)
                if ms < shape_ms:
                    shape_ms, shape = ms, dict(cell_size=cs, solve_block=sb, solve_per_thread=pt)
        for rb in rebin_blocks:
            ms = shape_ms if rb == per_sm8 else run(rebin_blocks=rb, **shape)
            if ms < best_ms:
                best_ms, best = ms, dict(shape, rebin_blocks=rb)
    if use_cache:
        cache[key] = {"choice": best, "ms": timings}
        save_cache(cache, path)
    return dataclasses.replace(config, **best), timings
