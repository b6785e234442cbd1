"""GPU parity: the CUDA voxeliser against the float64 oracle, bit for bit.

Compares every product of the world build: grid entries (including pool
indices), the contents of every live pool brick, poolUsed, the free-list
holes, super-grid counts, density bytes and the full GPU free list.
"""
import numpy as np
import pytest

from pixels_gb300 import config
from pixels_gb300.scenes.penthouse import build_penthouse, penthouse_program
from pixels_gb300.world import MODE_FP64, MODE_MIXED, VoxelWorld

import pyoracle


def build_gpu(vpm, mode, program=None):
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 14, vpm=vpm, mode=mode)
    if program is None:
        build_penthouse(w)
    else:
        w._pending = program
    w.build()
    return w


def assert_same_world(w, o):
    grid = w.grid
    np.testing.assert_array_equal(grid, o.grid, err_msg="grid differs")
    assert w.poolUsed == o.pool_used
    np.testing.assert_array_equal(w.freeBricks(), o.free_holes)
    pool = w.pool
    live = np.nonzero((grid != 0) & ((grid & 0x80000000) == 0))[0]
    for ci in live:
        p = int(grid[ci]) - 1
        np.testing.assert_array_equal(pool[p * 512:(p + 1) * 512], o.pool[p * 512:(p + 1) * 512],
                                      err_msg=f"pool brick {p} of cell {ci} differs")
    d = w.derived()
    np.testing.assert_array_equal(d["super"], o.super)
    np.testing.assert_array_equal(d["density"], o.density)
    np.testing.assert_array_equal(d["free_list"], o.free_list())


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [MODE_FP64, MODE_MIXED])
def test_penthouse_vpm20_bit_exact(built_lib, mode):
    prog, _ = penthouse_program(20.0)
    o = pyoracle.OracleWorld(prog.to_bytes(), 20.0, config.Config(20.0).dims)
    w = build_gpu(20.0, mode)
    assert_same_world(w, o)
    s = w.stats()
    assert s["voxel_evals"] == o.stats["voxel_evals"]
    assert s["brick_evals"] == o.stats["brick_evals"]


@pytest.mark.gpu
@pytest.mark.parametrize("vpm", [20.0, 40.0])
def test_mixed_enclosures_hold_everywhere(built_lib, vpm):
    """Validation mode: every float32 interval must enclose the float64 value
    (within the certified margin), every certified float32 paint decision and
    every filtered Math.hypot decision must equal the correctly rounded float64
    one; the build must still be bit-exact."""
    from pixels_gb300 import _lib
    prog, _ = penthouse_program(vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims)
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, vpm=vpm, mode=MODE_MIXED)
    _lib.set_validation(w._h, True)
    w._pending = prog
    w.build()
    s = w.stats()
    assert s["violations"] == 0
    assert_same_world(w, o)


@pytest.mark.gpu
@pytest.mark.parametrize("vpm", [40.0])
def test_penthouse_vpm40_mixed_bit_exact(built_lib, vpm):
    prog, _ = penthouse_program(vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims)
    w = build_gpu(vpm, MODE_MIXED, program=prog)
    assert_same_world(w, o)
    s = w.stats()
    assert s["rescued"] < 0.01 * s["voxel_evals"]


@pytest.mark.gpu
def test_op_uploads_by_kernel_and_by_copy_agree(built_lib, monkeypatch):
    """Where the GPU reads pageable host memory, a build's op tables are copied
    by one kernel reading the host arrays; with that switched off they go by
    cudaMemcpyAsync.  Both builds must give the same world."""
    prog, _ = penthouse_program(20.0)
    w_kernel = build_gpu(20.0, MODE_MIXED, program=prog)
    monkeypatch.setenv("PIXELS_GB300_NO_HOST_READS", "1")
    w_copy = build_gpu(20.0, MODE_MIXED, program=prog)
    np.testing.assert_array_equal(w_kernel.grid, w_copy.grid)
    assert w_kernel.poolUsed == w_copy.poolUsed
    np.testing.assert_array_equal(w_kernel.pool, w_copy.pool)
