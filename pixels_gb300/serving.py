"""Serving subtract-edits on a resident world (continuous batching).

The game's carve, expressed as the rasteriser expresses it: ``Builder.carve``
of a sphere or capsule (shapes.ts:65-72, 114-128, 423-426), appended to the
world's op history.  ``serve`` runs the native serving loop
(``px_serve_run``): requests are released at their arrival times, admitted in
arrival order by free-pool memory, batched (up to ``max_batch`` per build step)
and applied by incremental builds on the resident world.

``edit_stream`` draws the benchmark's request stream: centres uniform on
occupied bricks, radii log-uniform 1-40 cm, 70% spheres / 30% capsules,
Poisson arrivals.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib, config as _config
from .ir import Program
from .shapes import capsule, sphere

SPHERE, CAPSULE = 0, 1


def edit_stream(grid: np.ndarray, bricks, vpm: float, n: int, rate: float, seed: int = 0,
                r_min: float = 0.01, r_max: float = 0.4, p_sphere: float = 0.7):
    """``n`` edits ``(shape, a, b, r)`` and their arrival times (seconds)."""
    rng = np.random.default_rng(seed)
    bx, by, bz = bricks
    occ = np.nonzero(grid != 0)[0]
    if len(occ) == 0:
        raise ValueError("the world has no occupied brick")
    vs = 1.0 / vpm
    edits = []
    for _ in range(n):
        ci = int(occ[rng.integers(len(occ))])
        x, y, z = ci % bx, (ci // bx) % by, ci // (bx * by)
        c = np.array([(x * 8 + rng.uniform(0, 8)) * vs, (y * 8 + rng.uniform(0, 8)) * vs, (z * 8 + rng.uniform(0, 8)) * vs])
        r = math.exp(rng.uniform(math.log(r_min), math.log(r_max)))
        if rng.random() < p_sphere:
            edits.append((SPHERE, tuple(c), tuple(c), r))
        else:
            d = rng.normal(size=3)
            d = d / max(np.linalg.norm(d), 1e-9) * r * rng.uniform(0.5, 2.0)
            edits.append((CAPSULE, tuple(c - d), tuple(c + d), r))
    gaps = rng.exponential(1.0 / rate, size=n) if rate > 0 else np.zeros(n)
    return edits, np.cumsum(gaps) - (gaps[0] if n else 0.0)


def carve_program(edits, order, vpm: float) -> Program:
    """The edits as Builder.carve ops (the reference's view), in the applied order."""
    prog = Program()
    with _config.using(vpm):
        for i in order:
            shape, a, b, r = edits[int(i)]
            s = sphere(a, r) if shape == SPHERE else capsule(a, b, r)
            prog.add_op(1, s, 0)
    return prog


def serve(world, edits, arrivals, max_batch: int = 256, pool_budget: int | None = None, stream: int = 0):
    """Run the edits through the serving loop on ``world`` (a VoxelWorld)."""
    world._ensure()
    if pool_budget is None:
        pool_budget = 1 << 40
    return _lib.serve_run(world._h, edits, arrivals, max_batch, pool_budget, world.mode, stream)


def step_overlap(results) -> float | None:
    """Fraction of consecutive build steps whose device work overlapped: the
    next step's first kernel started before the previous step's last ended."""
    ok = results[results["status"] == 0]
    if len(ok) == 0:
        return None
    steps = {}
    for b, s0, s1 in zip(ok["batch"], ok["dev_start_ms"], ok["dev_end_ms"]):
        steps[int(b)] = (float(s0), float(s1))
    ids = sorted(steps)
    pairs = list(zip(ids, ids[1:]))
    if not pairs:
        return None
    return sum(steps[b][0] < steps[a][1] for a, b in pairs) / len(pairs)


def latency_stats(results) -> dict:
    ok = results[results["status"] == 0]
    lat = (ok["done_s"] - ok["arrival_s"]) * 1e3
    span = (ok["done_s"].max() - ok["arrival_s"].min()) if len(ok) else 0.0
    return {
        "requests": int(len(results)), "admitted": int(len(ok)),
        "p50_ms": float(np.percentile(lat, 50)) if len(ok) else None,
        "p99_ms": float(np.percentile(lat, 99)) if len(ok) else None,
        "max_ms": float(lat.max()) if len(ok) else None,
        "edits_per_s": float(len(ok) / span) if span > 0 else None,
        "batches": int(len(np.unique(ok["batch"]))) if len(ok) else 0,
        "max_step_ms": float(((ok["done_s"] - ok["start_s"]) * 1e3).max()) if len(ok) else None,
        "mean_batch": float(len(ok) / max(len(np.unique(ok["batch"])), 1)) if len(ok) else 0.0,
        "steps_overlapping_on_device": step_overlap(results),
    }
