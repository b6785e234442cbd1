"""Benchmark: the penthouse world build at 80 voxels per metre on one GB300.

A step is one complete build of the penthouse scene (2,429 ops) into an empty
1280x352x960 world (432,537,600 cells): brick / sub-block / voxel
classification, paint, pool allocation replay, the pool / grid write-out and
the derived upload buffers (super-grid counts, density, the GPU free list).
``value`` is Gvoxels/s (grid cells per second of device time, ops already
resident in HBM); ``e2e`` is the same metric through the public C ABI with the
op list uploaded from host memory and grid, pool, super counts, density and
free list read back every step (``e2e.with_host_flatten`` also runs the scene
program and flattens it to PXIR on the host every step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank builds its own replica (the scene does not
shard across GPUs here); value = all ranks' cells / the slowest rank's time.
``--impl reference`` times the reference's CPU algorithm (the float64 oracle
restatement, all host threads) on rank 0 only.
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
import types

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gvoxels/s at vpm=80 (mixed vs all-FP64 GPU, 0 mismatches); edit p50/p99 ms"
UNIT = "Gvoxels/s"
VPM = 80.0


def node_runtime() -> dict:
    """The JavaScript runtime the reference would run under on this host, if any."""
    import shutil
    path = shutil.which("node")
    if not path:
        return {"node": "absent"}
    try:
        v = subprocess.run([path, "--version"], capture_output=True, text=True, timeout=10).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        v = "unknown"
    return {"node": v, "node_path": path}


def world_mismatches(h, o, cfg, max_bricks=1 << 31) -> dict:
    """Every output of a built world against the oracle's: grid entries, live pool
    voxels, poolUsed, holes, super counts, density bytes and the GPU free list."""
    import numpy as np
    from pixels_gb300 import _lib
    n = cfg.bricks[0] * cfg.bricks[1] * cfg.bricks[2]
    grid = _lib.read_grid(h, n)
    pool = _lib.read_pool(h)
    st = _lib.stats(h)
    n_super = ((cfg.bricks[0] + 3) // 4) * ((cfg.bricks[1] + 3) // 4) * ((cfg.bricks[2] + 3) // 4)
    d = _lib.read_derived(h, max_bricks, n, n_super)
    holes = _lib.read_holes(h)
    out = {"grid_cells": int(np.count_nonzero(grid != o.grid)),
           "pool_used": int(st["pool_used"]) - int(o.pool_used),
           "holes": 0 if np.array_equal(holes, o.free_holes) else max(1, len(holes) ^ len(o.free_holes)),
           "super": int(np.count_nonzero(d["super"] != o.super)),
           "density": int(np.count_nonzero(d["density"] != o.density))}
    fl = o.free_list(max_bricks)
    out["free_list"] = (int(np.count_nonzero(d["free_list"] != fl)) if len(fl) == len(d["free_list"])
                        else abs(len(fl) - len(d["free_list"])))
    if out["grid_cells"] == 0 and out["pool_used"] == 0:
        live = np.nonzero((o.grid != 0) & ((o.grid & 0x80000000) == 0))[0]
        idx = o.grid[live].astype(np.int64) - 1
        out["pool_voxels"] = int(np.count_nonzero(pool.reshape(-1, 512)[idx] != o.pool.reshape(-1, 512)[idx]))
    else:
        out["pool_voxels"] = -1
    out["total"] = sum(abs(v) for v in out.values())
    return out


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(values, dist=None, device=None):
    """Element-wise maximum of per-rank timings (the slowest rank sets the job time)."""
    if dist is None:
        return list(values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def job_value(world_size: int, cells_per_rank: int, seconds: float) -> float:
    """Whole-job Gvoxels/s: every rank builds its own replica (weak scaling)."""
    return world_size * cells_per_rank / seconds / 1e9


def reference_arm(args):
    """The reference's CPU algorithm (float64 oracle restatement) on the host cores."""
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from pixels_gb300 import config
    from pixels_gb300.scenes.penthouse import penthouse_program
    cfg = config.Config(VPM)
    prog, _ = penthouse_program(VPM)
    ir = prog.to_bytes()
    threads = os.cpu_count() or 1
    for _ in range(max(args.warmup, 0) and 1):
        pyoracle.OracleWorld(ir, VPM, cfg.dims, threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o = pyoracle.OracleWorld(ir, VPM, cfg.dims, threads=threads)  # build + super counts + density
        o.free_list()                                                  # GpuWorld.ts:103-109
        times.append(time.perf_counter() - t0)
    t = statistics.mean(times)
    v = cfg.cells / t / 1e9
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (deterministic scene program)",
        "config": {"workload": "penthouse scene, vpm=80, 1280x352x960 cells, one full world build per step",
                   "cells": cfg.cells, "ops": len(prog)},
        "cpu_baseline": {"value": round(v, 6), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full penthouse builds at vpm=80 (float64 restatement of "
                                   f"shapes.ts apply + VoxelWorld + GpuWorld derived buffers and free list)",
                         **node_runtime()},
        "e2e": {"value": round(v, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def _device_ms(build_fn, steps, warmup):
    import torch
    for _ in range(warmup):
        build_fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        build_fn()
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    return statistics.mean(ms)


def synthetic_section(args, pyoracle):
    """Seeded synthetic scene: 4,096 primitives (box, rounded box, cylinder, capsule,
    torus, 8-point lathe, extruded hexagon; 30% subtract, 10% intersect; 25% noise
    paint) in the 16 x 4.4 x 12 m volume at vpm=80, both forms, each checked
    against the oracle right after it is timed (every output of the world)."""
    from pixels_gb300 import _lib, config
    from pixels_gb300.scenes.synthetic import synthetic_program
    from pixels_gb300.world import MODE_FP64, MODE_MIXED
    vpm = 80.0
    cfg = config.Config(vpm)
    prog = synthetic_program(1, 4096, vpm)
    ir = prog.to_bytes()
    o = pyoracle.OracleWorld(ir, vpm, cfg.dims, threads=os.cpu_count() or 1)
    h = _lib.world_create(*cfg.dims, vpm, 1 << 15)
    _lib.set_derive_on_build(h, 1 << 31)
    _lib.submit_ops(h, ir)
    _lib.build(h, MODE_MIXED)
    res = {"workload": "synthetic seed 1, 4096 primitives, vpm=80", "ops": len(prog), "cells": cfg.cells}
    for name, mode in (("mixed", MODE_MIXED), ("fp64", MODE_FP64)):
        def one():
            _lib.world_reset(h, True)
            _lib.build(h, mode)
        t = _device_ms(one, max(2, args.steps // 2), 2)
        st = _lib.stats(h)
        res[name] = {"ms_per_step": round(t, 4), "value": round(cfg.cells / (t * 1e-3) / 1e9, 3),
                     "mismatches": world_mismatches(h, o, cfg), "voxel_evals": st["voxel_evals"]}
        if mode == MODE_MIXED:
            res[name]["rescued_voxels"] = st["rescued_voxel"]
            res[name]["rescued"] = st["rescued"]
            res[name]["max_abs_d32_minus_d64"] = st["max_abs_err32"]
    res["speedup_mixed_vs_fp64"] = round(res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"], 3)
    _lib.world_destroy(h)
    return res


def batched_section(args, pyoracle, n_scenes: int = 256, check: int = 32):
    """256 independent seeded scenes of uneven size (volumes log-uniform 0.5-64 m^3,
    aspect up to 4:1, 16-2048 primitives, vpm 40/80/160) rebuilt by one CUDA graph
    launch; the autotuner picks the launch shape; `check` scenes (every n/check-th)
    are compared with the oracle bit for bit: grid, pool, poolUsed, holes, super
    counts, density and the GPU free list."""
    from pixels_gb300.batch import Batch, tune
    from pixels_gb300.scenes.synthetic import batch_specs, synthetic_program
    from pixels_gb300.world import MODE_FP64, MODE_MIXED, VoxelWorld
    specs = batch_specs(seed=7, n=n_scenes)
    t0 = time.perf_counter()
    progs = [synthetic_program(s["seed"], s["n_prims"], s["vpm"], s["volume"]) for s in specs]
    t_gen = time.perf_counter() - t0
    worlds = []
    for s, prog in zip(specs, progs):
        w = VoxelWorld(*s["dims"], initialPoolBricks=256, vpm=s["vpm"], mode=MODE_MIXED)
        w._pending = prog
        w.build()
        worlds.append(w)
    cells = int(sum(s["dims"][0] * s["dims"][1] * s["dims"][2] for s in specs))
    shape, ms, table = tune(worlds, MODE_MIXED)
    out = {"workload": f"{n_scenes} synthetic scenes (batch seed 7), one graph launch per step",
           "cells": cells, "prims": int(sum(s["n_prims"] for s in specs)), "host_generation_s": round(t_gen, 2),
           "autotune": table, "shape": {"streams": shape[0], "pairs_per_block": shape[1]}}
    with Batch(worlds, MODE_MIXED, *shape) as b:
        for _ in range(2):
            b.run()
        ts = [b.run() for _ in range(max(3, args.steps))]
    t = statistics.median(ts)
    out["mixed"] = {"ms_per_launch": round(t, 4), "value": round(cells / (t * 1e-3) / 1e9, 3),
                    "scenes_per_s": round(n_scenes / (t * 1e-3), 1)}
    with Batch(worlds, MODE_FP64, *shape) as b:
        b.run()
        ts = [b.run() for _ in range(3)]
    t64 = statistics.median(ts)
    out["fp64"] = {"ms_per_launch": round(t64, 4), "value": round(cells / (t64 * 1e-3) / 1e9, 3)}
    # sequential builds of the same scenes, one after another on one stream (no graph)
    from pixels_gb300 import _lib
    t0 = time.perf_counter()
    for w in worlds:
        _lib.world_reset(w._h, True)
        _lib.build(w._h, MODE_MIXED)
    out["sequential_ms"] = round((time.perf_counter() - t0) * 1e3, 3)
    mism = {}
    checked = []
    for i in range(0, n_scenes, max(1, n_scenes // check)):
        s, w = specs[i], worlds[i]
        o = pyoracle.OracleWorld(progs[i].to_bytes(), s["vpm"], s["dims"], threads=os.cpu_count() or 1)
        cfg = types.SimpleNamespace(bricks=tuple(d // 8 for d in s["dims"]))
        for k, v in world_mismatches(w._h, o, cfg).items():
            mism[k] = mism.get(k, 0) + abs(v)
        checked.append(i)
    out["oracle_checked_scenes"] = checked
    out["mismatches"] = mism
    for w in worlds:
        w.close()
    return out


def serving_section(args, pyoracle):
    """Subtract-edits (70% spheres, 30% capsules, radii 1-40 cm, centres on occupied
    bricks, Poisson arrivals) served on a resident synthetic map at vpm=160
    (2560x704x1920 = 3.46 G cells), continuous batching up to 512 edits per step."""
    import numpy as np
    from pixels_gb300 import config, serving
    from pixels_gb300.scenes.synthetic import synthetic_program
    from pixels_gb300.world import MODE_MIXED, VoxelWorld
    vpm = 160.0
    cfg = config.Config(vpm)
    prog = synthetic_program(1, 4096, vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 20, vpm=vpm, mode=MODE_MIXED)
    w._pending = prog
    w.build()
    grid = w.grid
    out = {"workload": "resident synthetic map (seed 1, 4096 primitives) at vpm=160", "cells": cfg.cells,
           "max_batch": 512, "rates": []}
    for rate in (1000.0, 20000.0, 100000.0, 200000.0):
        edits, arr = serving.edit_stream(grid, cfg.bricks, vpm, 2000, rate=rate, seed=int(rate))
        res, order = serving.serve(w, edits, arr, max_batch=512)
        st = serving.latency_stats(res)
        st["rate_offered"] = rate
        out["rates"].append(st)
    # 256 concurrent requests: bursts of 256 edits arriving together, 4 ms apart
    edits, _ = serving.edit_stream(grid, cfg.bricks, vpm, 256 * 16, rate=0, seed=7)
    arr = np.repeat(np.arange(16) * 0.004, 256)
    res, order = serving.serve(w, edits, arr, max_batch=512)
    st = serving.latency_stats(res)
    st["burst"] = 256
    out["concurrent_256"] = st
    w.close()
    return out


# DRAM bytes per build from one ncu capture on the penthouse at vpm=80 (the
# bench cannot run ncu itself): dram__bytes_read.sum + dram__bytes_write.sum of
# the evaluation kernels (classify, sub-block, the four voxel kernels, paint,
# apply) with caches flushed before each kernel, and of all 15 kernels of the
# build, flushed before each and left alone (the run's first build)
EVAL_TRAFFIC_BYTES = 33_314_048
BUILD_TRAFFIC_COLD_BYTES = 91_652_352
BUILD_TRAFFIC_WARM_BYTES = 65_374_208


def hbm_line(cfg, pool_used, ir_bytes, ms, derived_bytes=0):
    """Algorithmic HBM bytes of one build (outputs written -- grid, pool, and the
    derived super counts, density and free list -- plus the op list read once)
    over the build time, against the measured copy bandwidth."""
    peak = None
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        pass
    n_bricks = cfg.bricks[0] * cfg.bricks[1] * cfg.bricks[2]
    alg = 4 * n_bricks + 1024 * int(pool_used) + int(ir_bytes) + int(derived_bytes)
    gbs = alg / (ms * 1e-3) / 1e9
    return {"alg_bytes_per_build": alg, "achieved_gbs": round(gbs, 2), "peak_gbs": peak,
            "frac": round(gbs / peak, 5) if peak else None, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--vpm", type=float, default=VPM)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", choices=("both", "mixed", "fp64"), default="both",
                    help="forms to time (profiling runs time one)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the synthetic-scene and serving sections")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    import numpy as np
    import torch

    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from pixels_gb300 import _lib, build as pxbuild, config
    from pixels_gb300.scenes.penthouse import penthouse_program
    from pixels_gb300.world import MODE_FP64, MODE_MIXED
    pxbuild.build()
    L = _lib.load()
    vpm = args.vpm
    cfg = config.Config(vpm)
    t_flat = time.perf_counter()
    prog, _ = penthouse_program(vpm)
    ir = prog.to_bytes()
    t_flat = time.perf_counter() - t_flat  # host: run the scene program and flatten it to PXIR
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    s_ptr = stream.cuda_stream
    h = _lib.world_create(*cfg.dims, vpm, 1 << 15)
    MAX_BRICKS = 1 << 31
    _lib.set_derive_on_build(h, MAX_BRICKS)  # every build ends with super counts, density and free list
    _lib.submit_ops(h, ir)
    _lib.build(h, MODE_FP64 if args.mode == "fp64" else MODE_MIXED, s_ptr)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # 256 MB > L2 (129 MB)

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed_builds(mode, steps, warmup):
        for _ in range(warmup):
            _lib.world_reset(h, True, s_ptr)
            _lib.build(h, mode, s_ptr)
        ms, fold_ms, cls_ms = [], [], []
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier()
        torch.cuda.synchronize()
        for i in range(steps):
            flush.fill_(i & 0xFF)                      # L2 flush between timed iterations
            ev[i][0].record(stream)
            _lib.world_reset(h, True, s_ptr)
            _lib.build_enqueue(h, mode, s_ptr)
            ev[i][1].record(stream)
            _lib.build_finish(h)
            st_ = _lib.stats(h)
            fold_ms.append(st_["fold_ms"])
            cls_ms.append(st_["classify_ms"])
        torch.cuda.synchronize()
        barrier()
        ms = [a.elapsed_time(b) for a, b in ev]
        timed_builds.cls = statistics.mean(cls_ms)
        return ms, fold_ms

    def graph_builds(mode, steps, warmup):
        """The same build relaunched as the world's captured CUDA graph (px_batch of one
        world): all of a build's launches submitted at once; device time per launch."""
        b = _lib.batch_create([h], mode, 1, 0)
        try:
            for _ in range(warmup):
                _lib.batch_run(b, s_ptr)
            barrier()
            torch.cuda.synchronize()
            ms = []
            for i in range(steps):
                flush.fill_(i & 0xFF)                  # L2 flush between timed iterations
                ms.append(_lib.batch_run(b, s_ptr))
            torch.cuda.synchronize()
            barrier()
        finally:
            _lib.batch_destroy(b)
        return ms

    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.start()
    ms64 = fold64 = ms_mx = fold_mx = None
    cls64 = cls_mx = None
    stream_ms = {}
    if args.mode in ("both", "fp64"):
        s64, fold64 = timed_builds(MODE_FP64, args.steps, args.warmup)
        cls64 = timed_builds.cls
        ms64 = graph_builds(MODE_FP64, args.steps, args.warmup)
        stream_ms["fp64"] = statistics.mean(s64)
    if args.mode in ("both", "mixed"):
        smx, fold_mx = timed_builds(MODE_MIXED, args.steps, args.warmup)
        cls_mx = timed_builds.cls
        ms_mx = graph_builds(MODE_MIXED, args.steps, args.warmup)
        stream_ms["mixed"] = statistics.mean(smx)
    have64 = ms64 is not None
    if ms_mx is None:
        ms_mx, fold_mx = ms64, fold64
    if ms64 is None:
        ms64, fold64 = ms_mx, fold_mx
    clocks = sampler.stop() if sampler else None
    st = _lib.stats(h)

    # max over ranks
    t_mx, t_64 = max_over_ranks([statistics.mean(ms_mx), statistics.mean(ms64)], dist, dev)
    cells = cfg.cells
    value = job_value(world, cells, t_mx * 1e-3)
    value64 = job_value(world, cells, t_64 * 1e-3)

    # end to end through the C ABI: op list from host memory; grid, pool, super counts,
    # density and free list back to pinned host memory
    import ctypes
    n_bricks = cfg.bricks[0] * cfg.bricks[1] * cfg.bricks[2]
    n_super = ((cfg.bricks[0] + 3) // 4) * ((cfg.bricks[1] + 3) // 4) * ((cfg.bricks[2] + 3) // 4)
    grid_h = torch.empty(n_bricks, dtype=torch.int32, pin_memory=True)
    pool_h = torch.empty(max(st["pool_used"], 1) * 512, dtype=torch.int16, pin_memory=True)
    super_h = torch.empty(n_super, dtype=torch.int32, pin_memory=True)
    dens_h = torch.empty(n_bricks, dtype=torch.uint8, pin_memory=True)
    free_len = ctypes.c_uint32()
    assert L.px_read_free_list(h, MAX_BRICKS, None, 0, ctypes.byref(free_len)) == 0
    free_h = torch.empty(free_len.value + 4096, dtype=torch.int32, pin_memory=True)
    ir_buf = ctypes.create_string_buffer(ir, len(ir))

    def e2e_step(flatten: bool):
        t0 = time.perf_counter()
        if flatten:  # the scene program and its flattening to PXIR on the host
            p_, _ = penthouse_program(vpm)
            ir_ = p_.to_bytes()
            buf = ctypes.create_string_buffer(ir_, len(ir_))
        else:
            buf, ir_ = ir_buf, ir
        tf = time.perf_counter()
        _lib.world_reset(h, False, s_ptr)
        assert L.px_submit_ops(h, buf, len(ir_)) == 0
        ta = time.perf_counter()
        _lib.build(h, MODE_MIXED, s_ptr)
        used_ = _lib.stats(h)["pool_used"]
        tb = time.perf_counter()
        assert L.px_read_grid(h, grid_h.data_ptr(), grid_h.numel()) == 0
        assert L.px_read_pool(h, pool_h.data_ptr(), pool_h.numel()) == 0
        assert L.px_read_super(h, super_h.data_ptr(), super_h.numel()) == 0
        assert L.px_read_density(h, dens_h.data_ptr(), dens_h.numel()) == 0
        assert L.px_read_free_list(h, MAX_BRICKS, free_h.data_ptr(), free_h.numel(), ctypes.byref(free_len)) == 0
        t1 = time.perf_counter()
        return used_, (tf - t0, ta - tf, tb - ta, t1 - tb)

    # pipelined end to end: two worlds on two streams, so that step i's readback
    # (host-blocking copies) overlaps step i+1's build on the GPU; every step still
    # submits its op list from host memory and reads all of its outputs back
    h2 = None
    if not args.no_e2e:
        h2 = _lib.world_create(*cfg.dims, vpm, 1 << 15)
        _lib.set_derive_on_build(h2, MAX_BRICKS)
        _lib.submit_ops(h2, ir)
        _lib.build(h2, MODE_MIXED, s_ptr)
    pipe_streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]

    class _DeviceArray:  # a world's device buffer seen through the CUDA array interface (no copy)
        def __init__(self, ptr, n, typestr):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3}

    def dev_tensor(ptr, n, typestr):
        return torch.as_tensor(_DeviceArray(ptr, n, typestr), device=dev)

    # per world: pinned host copies of its outputs, and an event after their copies
    outs = [{"grid": torch.empty_like(grid_h).pin_memory(), "pool": torch.empty_like(pool_h).pin_memory(),
             "super": torch.empty_like(super_h).pin_memory(), "dens": torch.empty_like(dens_h).pin_memory(),
             "free": torch.empty_like(free_h).pin_memory()} for _ in range(2)]
    copy_stream = torch.cuda.Stream(dev)
    copied = [torch.cuda.Event(), torch.cuda.Event()]

    def copy_outputs(hh, k):
        """Device-to-host copies of every output of world hh on the copy stream (the
        device view of the public API), not waited for by the host."""
        v = _lib.device_view(hh)
        used_k = _lib.stats(hh)["pool_used"]
        o = outs[k]
        with torch.cuda.stream(copy_stream):
            o["grid"].copy_(dev_tensor(v.grid, n_bricks, "<i4"), non_blocking=True)
            o["pool"][:used_k * 512].copy_(dev_tensor(v.pool, used_k * 512, "<i2"), non_blocking=True)
            o["super"].copy_(dev_tensor(v.super_counts, n_super, "<i4"), non_blocking=True)
            o["dens"].copy_(dev_tensor(v.density, n_bricks, "|u1"), non_blocking=True)
            o["free"][:v.free_len].copy_(dev_tensor(v.free_list, v.free_len, "<i4"), non_blocking=True)
            copied[k].record(copy_stream)

    def e2e_pipelined(n: int) -> float:
        hs = (h, h2)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        busy = [False, False]  # the world's outputs are still being copied out
        for i in range(n + 1):
            if i < n:
                k = i % 2
                hh, st = hs[k], pipe_streams[k]
                if busy[k]:
                    st.wait_event(copied[k])  # on the device: its readback first, then its reset
                _lib.world_reset(hh, False, st.cuda_stream)
                assert L.px_submit_ops(hh, ir_buf, len(ir)) == 0
                _lib.build_enqueue(hh, MODE_MIXED, st.cuda_stream)
            if i > 0:
                k = (i - 1) % 2
                _lib.build_finish(hs[k])
                copy_outputs(hs[k], k)
                busy[k] = True
        copy_stream.synchronize()
        return (time.perf_counter() - t0) / n

    t_pipe = None
    if not args.no_e2e:
        e2e_pipelined(max(args.warmup, 1))
        t_pipe = max_over_ranks([e2e_pipelined(max(args.steps, 2))], dist, dev)[0]

    e2e, e2e_parts, e2e_fl = [], [], []
    used = st["pool_used"]
    for flatten in (False, True):
        for i in range(0 if args.no_e2e else args.warmup + args.steps):
            torch.cuda.synchronize()
            barrier()
            used, parts = e2e_step(flatten)
            if i >= args.warmup:
                (e2e_fl if flatten else e2e).append(sum(parts))
                if not flatten:
                    e2e_parts.append(parts[1:])
    if not e2e:  # profiling run: one readback for the mismatch check
        used, _ = e2e_step(False)
        e2e = e2e_fl = [float("nan")]
    t_e2e_serial, t_e2e_fl = max_over_ranks([statistics.mean(e2e), statistics.mean(e2e_fl)], dist, dev)
    t_e2e = t_pipe if t_pipe is not None else t_e2e_serial
    e2e_value = job_value(world, cells, t_e2e)
    if h2 is not None:
        _lib.world_destroy(h2)
    d2h = int(grid_h.numel() * 4 + used * 1024 + super_h.numel() * 4 + dens_h.numel() + free_len.value * 4)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # mismatches against the float64 oracle at the full size (outside the timed region):
    # the world the last e2e step built (mixed form), every output
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    t0 = time.perf_counter()
    o = pyoracle.OracleWorld(ir, vpm, cfg.dims, count_flops=True)
    t_cpu1 = time.perf_counter() - t0
    mism = world_mismatches(h, o, cfg, MAX_BRICKS)
    mism64 = None
    if have64:  # the float64 form's world, rebuilt once
        _lib.world_reset(h, True, s_ptr)
        _lib.build(h, MODE_FP64, s_ptr)
        mism64 = world_mismatches(h, o, cfg, MAX_BRICKS)

    # CPU baseline: the oracle, one thread, a bounded sample
    cpu = None
    if not args.no_cpu_baseline:
        times = [t_cpu1]
        t_end = time.perf_counter() + 10.0
        while time.perf_counter() < t_end and len(times) < 8:
            t0 = time.perf_counter()
            pyoracle.OracleWorld(ir, vpm, cfg.dims)
            times.append(time.perf_counter() - t0)
        tc = statistics.mean(times[1:] or times)
        cpu = {"value": round(cells / tc / 1e9, 6), "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{len(times)} full penthouse builds at vpm=80, single thread", **node_runtime()}

    # roofline of the dominant kernel (fold): algorithmic float ops from the oracle ledger
    alg_ops = o.stats["flops"] + o.stats["divs"] + o.stats["sqrts"]
    fold_s = statistics.mean(fold_mx) * 1e-3
    peak32 = _lib.probe_peak(False)
    peak64 = _lib.probe_peak(True)
    achieved = alg_ops / fold_s / 1e12
    fold64_s = statistics.mean(fold64) * 1e-3
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_mx, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (deterministic scene program, no dataset)",
        "config": {"workload": "penthouse scene (2,429 ops), vpm=80, 1280x352x960 = 432,537,600 cells, "
                               "one full world build per step",
                   "cells": cells, "ops": len(prog), "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "fp64_form": ({"value": round(value64, 4), "ms_per_step": round(t_64, 4),
                       "stream_ms_per_step": round(stream_ms["fp64"], 4),
                       "fold_ms": round(fold64_s * 1e3, 4), "classify_ms": cls64} if have64 else None),
        "stream_ms_per_step": round(stream_ms["mixed"], 4) if "mixed" in stream_ms else None,
        "timing": "device time per build: the world's build graph relaunched (px_batch_run of one world); "
                  "stream_ms_per_step: the same build launched kernel by kernel (px_build_enqueue)",
        "classify_ms": cls_mx,
        "speedup_mixed_vs_fp64": round(t_64 / t_mx, 3) if have64 else None,
        "mismatches": mism,
        "mismatches_fp64_form": mism64,
        "rescued": {"total": st["rescued"], "brick": st["rescued_brick"], "sub": st["rescued_sub"],
                    "voxel": st["rescued_voxel"], "polygon_test": st["rescued_polygon"],
                    "paint": st["rescued_paint"],
                    "fraction_of_voxel_evals": round(st["rescued_voxel"] / max(st["voxel_evals"], 1), 6)},
        "max_abs_d32_minus_d64": st["max_abs_err32"],
        "e2e": {"value": round(e2e_value, 4), "unit": UNIT, "h2d_bytes_per_step": len(ir),
                "d2h_bytes_per_step": d2h,
                "ms_per_step": round(t_e2e * 1e3, 3),
                "reads": "grid, pool, super counts, density, free list",
                "pipelined": t_pipe is not None,
                "how": "two worlds built alternately on two CUDA streams; every step resets its world, submits "
                       "the op list from host memory, builds, and copies every output (the public device view) "
                       "to pinned host memory on a third stream, overlapping the next step's build; the timed "
                       "region ends when the last copy has landed",
                "serial": {"value": round(job_value(world, cells, t_e2e_serial), 4),
                           "ms_per_step": round(t_e2e_serial * 1e3, 3)},
                "split_ms": ({k: round(statistics.mean(p[j] for p in e2e_parts) * 1e3, 3)
                              for j, k in enumerate(("reset_and_submit", "build_and_derive", "read_outputs"))}
                             if e2e_parts else None),
                "with_host_flatten": {"value": round(job_value(world, cells, t_e2e_fl), 4),
                                      "ms_per_step": round(t_e2e_fl * 1e3, 3),
                                      "what": "the scene program run and flattened to PXIR on the host "
                                              "(Python) every step, then the same C ABI calls"}},
        "roofline": {"bound": "fp32-alu", "achieved": round(achieved, 4), "peak": round(peak32, 2),
                     "unit": "TFLOP/s", "frac": round(achieved / peak32, 5), "traffic": EVAL_TRAFFIC_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the classify, sub-block, "
                                       "voxel (4), paint and apply kernels of one build of this workload "
                                       "(one capture, caches flushed before each kernel, --clock-control none)",
                     "build_traffic": {"cold": BUILD_TRAFFIC_COLD_BYTES, "warm": BUILD_TRAFFIC_WARM_BYTES,
                                       "what": "all 15 kernels of one build: caches flushed before each kernel "
                                               "(cold), or left alone (warm, the run's first build)"},
                     "kernel": "classify_kernel + sub_kernel + voxel_lean_kernel x3 + voxel_kernel + paint_kernel "
                               "+ fold_kernel (every SDF and paint evaluation)",
                     "alg_ops_per_launch": int(alg_ops),
                     "fold_ms": round(fold_s * 1e3, 4),
                     "peak_source": "measured here: dependent FFMA chains on all SMs (px_probe_peak)",
                     "fp64": ({"achieved": round(alg_ops / fold64_s / 1e12, 5), "peak": round(peak64, 3),
                               "frac": round(alg_ops / fold64_s / 1e12 / peak64, 5)} if have64 else None)},
        "hbm": hbm_line(cfg, used, len(ir), t_mx, super_h.numel() * 4 + dens_h.numel() + free_len.value * 4),
        "host_flatten_ms": round(t_flat * 1e3, 2),
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": int(st["kernel_launches"]) * args.steps,
    }
    if not args.no_extra:
        _lib.world_destroy(h)
        out["synthetic"] = synthetic_section(args, pyoracle)
        out["serving"] = serving_section(args, pyoracle)
        out["batched"] = batched_section(args, pyoracle)
    print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
