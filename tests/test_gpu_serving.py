"""Serving subtract-edits on a resident world: batched results equal one-at-a-time
results and the float64 oracle rebuilt with the edits appended as carves."""
import numpy as np
import pytest

import pyoracle
from pixels_gb300 import config, serving
from pixels_gb300.scenes.penthouse import penthouse_program
from pixels_gb300.world import MODE_MIXED, VoxelWorld

from test_gpu_parity import assert_same_world


def resident(vpm, prog):
    w = VoxelWorld(*config.Config(vpm).dims, vpm=vpm, mode=MODE_MIXED)
    w._pending = prog
    w.build()
    return w


@pytest.mark.gpu
def test_batched_edits_equal_sequential_and_oracle(built_lib):
    vpm = 40.0
    prog, _ = penthouse_program(vpm)
    base_ir = prog.to_bytes()
    w_batch = resident(vpm, prog)
    cfg = config.Config(vpm)
    edits, _ = serving.edit_stream(w_batch.grid, cfg.bricks, vpm, 160, rate=0, seed=3)
    arrivals = np.zeros(len(edits))
    res_b, order_b = serving.serve(w_batch, edits, arrivals, max_batch=64)
    assert (res_b["status"] == 0).all()
    assert len(np.unique(res_b["batch"])) == 3            # 64 + 64 + 32, all arrived at once
    prog2, _ = penthouse_program(vpm)
    w_seq = resident(vpm, prog2)
    res_s, order_s = serving.serve(w_seq, edits, arrivals, max_batch=1)
    assert list(order_b) == list(order_s) == list(range(len(edits)))
    np.testing.assert_array_equal(w_batch.grid, w_seq.grid)
    assert w_batch.poolUsed == w_seq.poolUsed
    np.testing.assert_array_equal(w_batch.freeBricks(), w_seq.freeBricks())
    # the reference: the scene followed by the carves, one op after the other
    carves = serving.carve_program(edits, order_b, vpm)
    o = pyoracle.OracleWorld(_concat_ir(prog2, carves), vpm, cfg.dims)
    assert_same_world(w_batch, o)


def _concat_ir(a, b):
    from pixels_gb300.ir import Program
    p = Program()
    code_off, par_off = len(a.code), len(a.params)
    p.ops = list(a.ops)
    p.code = list(a.code)
    p.params = list(a.params)
    for op in b.ops:
        op = list(op)
        op[5] += code_off
        op[4] = op[4] + par_off if op[2] else op[4]
        p.ops.append(tuple(op))
    p.code += [(w0, off + par_off) for (w0, off) in b.code]
    p.params += list(b.params)
    return p.to_bytes()


@pytest.mark.gpu
def test_resident_synthetic_vpm160_after_served_stream_matches_oracle(built_lib):
    """The serving benchmark's world: the seeded 4,096-primitive synthetic map at
    160 voxels per metre (2560 x 704 x 1920 = 3.46 G cells), then a Poisson
    stream of 2,000 sphere/capsule subtract-edits served in batches of up to 512.
    The result must equal the oracle's build of the scene followed by the
    carves in the order they were applied (shapes.ts:423-426)."""
    import os
    from pixels_gb300.scenes.synthetic import synthetic_program
    vpm = 160.0
    cfg = config.Config(vpm)
    prog = synthetic_program(1, 4096, vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 20, vpm=vpm, mode=MODE_MIXED)
    w._pending = prog
    w.build()
    edits, arrivals = serving.edit_stream(w.grid, cfg.bricks, vpm, 2000, rate=100000.0, seed=100000)
    res, order = serving.serve(w, edits, arrivals, max_batch=512)
    assert (res["status"] == 0).all() and len(order) == len(edits)
    assert len(np.unique(res["batch"])) > 1
    carves = serving.carve_program(edits, order, vpm)
    o = pyoracle.OracleWorld(_concat_ir(synthetic_program(1, 4096, vpm), carves), vpm, cfg.dims,
                             threads=os.cpu_count() or 1)
    assert_same_world(w, o)
    w.close()


@pytest.mark.gpu
def test_steps_overlap_on_the_device_and_commit_in_order(built_lib):
    """256 edits arriving together, at most 16 per step: while one step's apply
    pass runs, the next step's evaluation passes run on another stream.  The
    device timestamps of consecutive steps overlap, and the world still equals
    the oracle's build followed by the carves in the order applied."""
    vpm = 40.0
    cfg = config.Config(vpm)
    prog, _ = penthouse_program(vpm)
    w = resident(vpm, prog)
    edits, _ = serving.edit_stream(w.grid, cfg.bricks, vpm, 256, rate=0, seed=11)
    res, order = serving.serve(w, edits, np.zeros(len(edits)), max_batch=16)
    assert (res["status"] == 0).all() and len(order) == len(edits)
    assert len(np.unique(res["batch"])) >= 16
    assert (res["dev_end_ms"] > res["dev_start_ms"]).all()
    frac = serving.step_overlap(res)
    assert frac is not None and frac > 0.5, frac
    prog2, _ = penthouse_program(vpm)
    o = pyoracle.OracleWorld(_concat_ir(prog2, serving.carve_program(edits, order, vpm)), vpm, cfg.dims)
    assert_same_world(w, o)


@pytest.mark.gpu
def test_poisson_stream_latency(built_lib):
    vpm = 40.0
    prog, _ = penthouse_program(vpm)
    w = resident(vpm, prog)
    cfg = config.Config(vpm)
    edits, arrivals = serving.edit_stream(w.grid, cfg.bricks, vpm, 400, rate=20000.0, seed=5)
    res, order = serving.serve(w, edits, arrivals, max_batch=256)
    st = serving.latency_stats(res)
    assert st["admitted"] == 400
    assert st["p99_ms"] is not None and st["p99_ms"] < 1000


@pytest.mark.gpu
def test_pool_budget_admission(built_lib):
    vpm = 40.0
    prog, _ = penthouse_program(vpm)
    w = resident(vpm, prog)
    cfg = config.Config(vpm)
    live = w.liveBricks
    edits, _ = serving.edit_stream(w.grid, cfg.bricks, vpm, 50, rate=0, seed=9, r_min=0.3, r_max=0.4)
    res, order = serving.serve(w, edits, np.zeros(len(edits)), max_batch=50, pool_budget=live + 8)
    # a 30-40 cm edit spans at least 3 x 3 x 3 bricks of 20 cm: none fits in 8
    assert (res["status"] == 3).all() and len(order) == 0


@pytest.mark.gpu
def test_derive_on_build_after_carves(built_lib):
    """Derive on build over two builds: the penthouse, then 96 carves built on top
    of it (no reset). The second build's super counts, density and GPU free list
    come from the opaque counts finalize kept for the bricks the carves left
    alone and recounted for the ones they rewrote; all must equal the oracle's
    for the scene followed by the carves."""
    vpm = 40.0
    cfg = config.Config(vpm)
    prog, _ = penthouse_program(vpm)
    w = VoxelWorld(*cfg.dims, vpm=vpm, mode=MODE_MIXED, derive_on_build=True)
    w._pending = prog
    w.build()
    edits, _ = serving.edit_stream(w.grid, cfg.bricks, vpm, 96, rate=0, seed=11)
    carves = serving.carve_program(edits, range(len(edits)), vpm)
    w._pending = carves
    w.build()
    o = pyoracle.OracleWorld(_concat_ir(prog, carves), vpm, cfg.dims)
    assert_same_world(w, o)
