"""px_derive_noalloc: derived buffers into caller-held device memory, no allocation.

Some callers fix their device memory before they start working (a renderer
that sizes its buffers once, a frame loop where an allocation could stall a
frame, a process under a hard device-memory cap) and cannot let the library
allocate.  This entry point serves them with a fixed scratch array inside the
library.  Called through the C ABI on device buffers the test owns, it must
give the same super-grid counts and density bytes as px_derive (through the
world handle), or as the reference's formulas restated below for grids no
world produced, on two calls in a row: the fixed scratch is shared by both
calls and keeps the first call's contents.
"""
import ctypes

import numpy as np
import pytest

from pixels_gb300 import _lib, config
from pixels_gb300.scenes.penthouse import build_penthouse
from pixels_gb300.world import MODE_MIXED, VoxelWorld


def _tables():
    from pixels_gb300.materials import opaque_table, uniform_density_table
    return np.array(opaque_table(), np.uint8), np.array(uniform_density_table(), np.uint8)


def test_pool_beyond_the_fixed_scratch_is_refused(built_lib):
    """The size check comes before any GPU work (the pointers are never used)."""
    op, ud = _tables()
    dummy = ctypes.c_void_p(16)
    rc = built_lib.px_derive_noalloc(dummy, dummy, 8, 8, 8, _lib.PX_NOALLOC_MAX_POOL_BRICKS + 1, op.ctypes.data,
                                     ud.ctypes.data, dummy, dummy, None)
    assert rc == 9  # PX_E_TOO_LARGE


def test_misaligned_pool_is_refused(built_lib):
    """The pool is read as 32-bit voxel pairs: a pool that starts at an odd
    uint16 element is refused before any GPU work (the pointers are never used)."""
    op, ud = _tables()
    al = ctypes.c_void_p(256)
    rc = built_lib.px_derive_noalloc(al, ctypes.c_void_p(258), 8, 8, 8, 4, op.ctypes.data, ud.ctypes.data, al, al, None)
    assert rc == 1  # PX_E_INVALID_ARG
    rc = built_lib.px_derive_noalloc(ctypes.c_void_p(254), al, 8, 8, 8, 4, op.ctypes.data, ud.ctypes.data, al, al, None)
    assert rc == 1


def _expected(grid: np.ndarray, pool: np.ndarray, bricks):
    """GpuWorld.ts:90-101 / VoxelWorld.ts:159-170 restated in numpy: super counts
    (non-zero grid cells per 4^3 bricks) and density bytes."""
    op, ud = _tables()
    bx, by, bz = bricks
    g = grid.reshape(bz, by, bx)
    sx, sy, sz = (bx + 3) // 4, (by + 3) // 4, (bz + 3) // 4
    pad = np.zeros((sz * 4, sy * 4, sx * 4), np.uint32)
    pad[:bz, :by, :bx] = g != 0
    sup = pad.reshape(sz, 4, sy, 4, sx, 4).sum(axis=(1, 3, 5)).astype(np.uint32).ravel()
    den = np.zeros(grid.size, np.uint8)
    uni = (grid & 0x80000000) != 0
    den[uni] = ud[grid[uni] & 0xFF]
    pl = (grid != 0) & ~uni
    if pl.any():
        vox = pool.reshape(-1, 512)[grid[pl].astype(np.int64) - 1]
        n = ((vox != 0) & (op[vox & 0xFF] != 0)).sum(axis=1)
        den[pl] = np.floor((n / 512.0) * 255.0 + 0.5).astype(np.uint8)  # Math.round, half up
    return sup, den


def _run_twice(grid_ptr, pool_ptr, bricks, n_pool, exp_sup, exp_den):
    import torch
    sup = torch.empty(exp_sup.size, dtype=torch.int32, device="cuda:0")
    den = torch.empty(exp_den.size, dtype=torch.uint8, device="cuda:0")
    for call in range(2):
        sup.fill_(-0x21524111)  # 0xdeadbeef: stale values must not survive
        den.fill_(0xAB)
        torch.cuda.synchronize()
        _lib.derive_noalloc(grid_ptr, pool_ptr, bricks, n_pool, sup.data_ptr(), den.data_ptr())
        np.testing.assert_array_equal(sup.cpu().numpy().view(np.uint32), exp_sup, err_msg=f"super, call {call}")
        np.testing.assert_array_equal(den.cpu().numpy(), exp_den, err_msg=f"density, call {call}")
    return sup, den


@pytest.mark.gpu
@pytest.mark.parametrize("vpm", [20.0, 80.0])
def test_derive_noalloc_matches_px_derive(built_lib, vpm):
    """The penthouse at vpm=20 (2.6k pool bricks) and vpm=80 (46k pool bricks,
    13,200 super cells: several grid-stride passes of both kernels)."""
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 12, vpm=vpm, mode=MODE_MIXED)
    build_penthouse(w)
    w.build()
    ref = w.derived()  # px_derive through the world handle
    view = _lib.device_view(w._h)
    n_pool = w.poolUsed
    bricks = (w.bx, w.by, w.bz)
    sup, den = _run_twice(view.grid, view.pool, bricks, n_pool, ref["super"], ref["density"])
    # a pool shorter than the grid's references is reported (nothing is read past it)
    with pytest.raises(_lib.PxError) as e:
        _lib.derive_noalloc(view.grid, view.pool, bricks, n_pool // 2, sup.data_ptr(), den.data_ptr())
    assert e.value.code == 1
    w.close()


@pytest.mark.gpu
def test_derive_noalloc_partial_super_cells_and_empty_pool(built_lib):
    """5x3x7 bricks (no axis a multiple of 4: every super cell on the far faces is
    partial) mixing air, uniform and pool bricks; then an all-uniform grid with
    no pool at all (the pool pass is skipped)."""
    import torch
    rng = np.random.default_rng(5)
    bricks = (5, 3, 7)
    n = 5 * 3 * 7
    n_pool = 40
    kind = rng.integers(0, 3, n)
    grid = np.zeros(n, np.uint32)
    mats = rng.integers(1, 64, n).astype(np.uint32)
    grid[kind == 1] = 0x80000000 | mats[kind == 1]
    pool_cells = np.nonzero(kind == 2)[0][:n_pool]
    grid[kind == 2] = 0x80000000 | 3
    grid[pool_cells] = rng.permutation(n_pool)[: pool_cells.size].astype(np.uint32) + 1
    pool = rng.integers(0, 70, n_pool * 512).astype(np.uint16)
    pool[rng.random(pool.size) < 0.3] = 0
    g_d = torch.from_numpy(grid.view(np.int32)).cuda()
    p_d = torch.from_numpy(pool.view(np.int16)).cuda()
    exp_sup, exp_den = _expected(grid, pool, bricks)
    _run_twice(g_d.data_ptr(), p_d.data_ptr(), bricks, n_pool, exp_sup, exp_den)

    grid_u = (0x80000000 | rng.integers(0, 64, n)).astype(np.uint32)
    grid_u[rng.random(n) < 0.25] = 0
    g_u = torch.from_numpy(grid_u.view(np.int32)).cuda()
    exp_sup, exp_den = _expected(grid_u, np.zeros(0, np.uint16), bricks)
    _run_twice(g_u.data_ptr(), 0, bricks, 0, exp_sup, exp_den)
