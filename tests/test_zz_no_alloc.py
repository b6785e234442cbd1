"""px_derive_noalloc: derived buffers into caller-held device memory, no allocation.

Called through the C ABI on device buffers the test owns, it must give the
same super-grid counts and density bytes as px_derive (through the world
handle) on two calls in a row; the fixed scratch is shared by both calls.
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


@pytest.mark.gpu
def test_derive_noalloc_matches_px_derive(built_lib):
    import torch
    vpm = 20.0
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 12, vpm=vpm, mode=MODE_MIXED)
    build_penthouse(w)
    w.build()
    ref = w.derived()  # px_derive through the world handle
    view = _lib.device_view(w._h)
    n_pool = w.poolUsed
    bricks = (w.bx, w.by, w.bz)
    n_super = ref["super"].size
    sup = torch.empty(n_super, dtype=torch.int32, device="cuda:0")
    den = torch.empty(w.bx * w.by * w.bz, dtype=torch.uint8, device="cuda:0")
    torch.cuda.synchronize()
    for call in range(2):
        sup.fill_(-0x21524111)  # 0xdeadbeef: stale values must not survive
        den.fill_(0xAB)
        torch.cuda.synchronize()
        _lib.derive_noalloc(view.grid, view.pool, bricks, n_pool, sup.data_ptr(), den.data_ptr())
        np.testing.assert_array_equal(sup.cpu().numpy().view(np.uint32), ref["super"], err_msg=f"super, call {call}")
        np.testing.assert_array_equal(den.cpu().numpy(), ref["density"], err_msg=f"density, call {call}")
    # a pool shorter than the grid's references is reported (nothing is read past it)
    with pytest.raises(_lib.PxError) as e:
        _lib.derive_noalloc(view.grid, view.pool, bricks, n_pool // 2, sup.data_ptr(), den.data_ptr())
    assert e.value.code == 1
    w.close()
