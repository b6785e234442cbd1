"""GPU parity: the CUDA voxeliser against the float64 oracle, bit for bit.

Compares every product of the world build: grid entries (including pool
indices), the contents of every live pool brick, poolUsed, the free-list
holes, super-grid counts, density bytes and the full GPU free list.  Covered
at the penthouse's 20, 40 and 80 voxels per metre (the last is the benchmark's
432.5 M-cell world) and on the seeded 4,096-primitive synthetic scene at 80
voxels per metre, in both the float64 and the mixed form; the mixed form's
float32 enclosures are also checked everywhere (validation mode).
"""
import os

import numpy as np
import pytest

from pixels_gb300 import config
from pixels_gb300.scenes.penthouse import build_penthouse, penthouse_program
from pixels_gb300.world import MODE_FP64, MODE_MIXED, VoxelWorld

import pyoracle

THREADS = os.cpu_count() or 1


def build_gpu(vpm, mode, program=None, derive_on_build=False, validate=False):
    from pixels_gb300 import _lib
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 14, vpm=vpm, mode=mode, derive_on_build=derive_on_build)
    if validate:
        _lib.set_validation(w._h, True)
    if program is None:
        build_penthouse(w)
    else:
        w._pending = program
    w.build()
    return w


def live_pool_mismatches(grid, pool, o) -> int:
    """Voxels of live pool bricks that differ from the oracle's (grids equal)."""
    live = np.nonzero((grid != 0) & ((grid & 0x80000000) == 0))[0]
    idx = grid[live].astype(np.int64) - 1
    return int(np.count_nonzero(pool.reshape(-1, 512)[idx] != o.pool.reshape(-1, 512)[idx]))


def assert_same_world(w, o):
    grid = w.grid
    np.testing.assert_array_equal(grid, o.grid, err_msg="grid differs")
    assert w.poolUsed == o.pool_used
    np.testing.assert_array_equal(w.freeBricks(), o.free_holes)
    assert live_pool_mismatches(grid, w.pool, o) == 0, "live pool bricks differ"
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
@pytest.mark.parametrize("vpm", [20.0, 40.0, 80.0])
def test_mixed_enclosures_hold_everywhere(built_lib, vpm):
    """Validation mode: every float32 interval must enclose the float64 value
    (within the certified margin), every certified float32 paint decision and
    every filtered Math.hypot decision must equal the correctly rounded float64
    one; the build must still be bit-exact."""
    prog, _ = penthouse_program(vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims, threads=THREADS)
    w = build_gpu(vpm, MODE_MIXED, program=prog, validate=True)
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
@pytest.mark.parametrize("mode", [MODE_FP64, MODE_MIXED])
def test_penthouse_vpm80_bit_exact(built_lib, mode):
    """The benchmark's world: 1280 x 352 x 960 cells, 2,429 ops, with the derived
    buffers and the GPU free list made by the build itself (derive on build)."""
    vpm = 80.0
    prog, _ = penthouse_program(vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims, threads=THREADS)
    w = build_gpu(vpm, mode, program=prog, derive_on_build=True)
    assert_same_world(w, o)
    s = w.stats()
    assert s["voxel_evals"] == o.stats["voxel_evals"]
    if mode == MODE_MIXED:
        assert s["rescued_voxel"] < 1e-3 * s["voxel_evals"]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [MODE_FP64, MODE_MIXED])
def test_synthetic_4096_vpm80_bit_exact(built_lib, mode):
    """The seeded synthetic scene (seed 1): 4,096 primitives of every kind,
    rotated uniformly on SO(3), 30% subtract / 10% intersect, 25% noise paint,
    in the 16 x 4.4 x 12 m volume at 80 voxels per metre."""
    from pixels_gb300.scenes.synthetic import synthetic_program
    vpm = 80.0
    prog = synthetic_program(1, 4096, vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims, threads=THREADS)
    w = build_gpu(vpm, mode, program=prog, derive_on_build=True)
    assert_same_world(w, o)


@pytest.mark.gpu
@pytest.mark.parametrize("seed,n,vpm", [(2, 1024, 40.0), (3, 256, 80.0)])
def test_synthetic_validation_mode(built_lib, seed, n, vpm):
    """Validation mode on synthetic scenes: every float32 enclosure of the rotated
    and composed programs, and every float32 noise-paint value (cells from
    enclosed products, coordinates from the axis tables), must agree with the
    float64 evaluation; the build must be bit-exact."""
    from pixels_gb300.scenes.synthetic import synthetic_program
    prog = synthetic_program(seed, n, vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims, threads=THREADS)
    w = build_gpu(vpm, MODE_MIXED, program=prog, validate=True)
    assert w.stats()["violations"] == 0
    assert_same_world(w, o)


@pytest.mark.gpu
def test_derive_on_build_matches_derive_on_read(built_lib):
    """The derived buffers the build leaves on the device equal those px_derive
    computes from the built world, and survive a rebuild."""
    from pixels_gb300 import _lib
    prog, _ = penthouse_program(20.0)
    a = build_gpu(20.0, MODE_MIXED, program=prog, derive_on_build=True)
    b = build_gpu(20.0, MODE_MIXED, program=prog)
    da, db = a.derived(), b.derived()
    for k in ("super", "density", "free_list"):
        np.testing.assert_array_equal(da[k], db[k], err_msg=k)
    view = _lib.device_view(a._h)
    assert view.free_len == len(da["free_list"]) and view.free_list
    _lib.world_reset(a._h, True)
    _lib.build(a._h, MODE_MIXED)
    np.testing.assert_array_equal(a.derived()["free_list"], db["free_list"])


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
