"""``VoxelWorld``: the sparse voxel store, built on the GPU through the C ABI.

Drop-in for ``src/world/VoxelWorld.ts`` as the scene builder and the GPU
upload see it (``VoxelWorld.ts:15-187``, ``GpuWorld.ts:50-136``):

* ``grid``: u32 per 8^3 brick: 0 = air, ``0x80000000 | v`` = uniform brick,
  ``n > 0`` = pool brick ``n - 1``;
* ``pool``: 512 u16 voxels per pool brick (x fastest, then y, then z);
* ``poolUsed`` / ``freeBricks()``: the LIFO allocator state;
* the derived upload buffers: super-grid counts, density, free list.

Ops queued through ``shapes.apply``/``Builder`` run on the GPU, in order, at
the next ``build()`` (or at the first read).  The result is bit-identical to
the reference's op-by-op rasteriser, pool indices included.
"""
from __future__ import annotations

import numpy as np

from . import config as _config
from .ir import Program

UNIFORM = 0x80000000   # VoxelWorld.ts:13

MODE_FP64 = 0     # all-float64 evaluation, mirrors JavaScript numbers
MODE_MIXED = 1    # float32 bulk evaluation + certified float64 rescue


class OpRecorder:
    """Collects a scene's ops into a ``Program`` without building anything."""

    def __init__(self, vpm: float):
        self.vpm = float(vpm)
        cfg = _config.Config(self.vpm)
        self.dx, self.dy, self.dz = cfg.dims
        self.program = Program()

    def submit(self, kind: int, shape, paint) -> None:
        self.program.add_op(kind, shape, paint)


class VoxelWorld:
    """A world handle owned by the CUDA library (one GPU)."""

    def __init__(self, dx: int, dy: int, dz: int, initialPoolBricks: int = 1 << 14,
                 vpm: float | None = None, mode: int = MODE_MIXED, max_bricks: int = 1 << 31,
                 derive_on_build: bool = False):
        from . import _lib
        if vpm is None:
            vpm = _config.current().vpm
        self.vpm = float(vpm)
        self.dx, self.dy, self.dz = int(dx), int(dy), int(dz)
        self.bx, self.by, self.bz = self.dx // 8, self.dy // 8, self.dz // 8
        self.mode = mode
        self.max_bricks = int(max_bricks)
        self._lib = _lib
        self._h = _lib.world_create(self.dx, self.dy, self.dz, self.vpm, int(initialPoolBricks))
        if derive_on_build:  # every build also leaves the upload buffers of GpuWorld.ts:90-111 on the device
            _lib.set_derive_on_build(self._h, self.max_bricks)
        self._pending = Program()

    # -- op submission (shapes.apply) ---------------------------------------
    def submit(self, kind: int, shape, paint) -> None:
        self._pending.add_op(kind, shape, paint)

    def build(self, stream: int = 0) -> None:
        """Run every queued op on the GPU (synchronous on ``stream``)."""
        if len(self._pending):
            self._lib.submit_ops(self._h, self._pending.to_bytes())
            self._pending = Program()
        self._lib.build(self._h, self.mode, stream)

    def _ensure(self):
        if len(self._pending):
            self.build()

    # -- reads ------------------------------------------------------------
    @property
    def poolUsed(self) -> int:
        self._ensure()
        return self._lib.stats(self._h)["pool_used"]

    @property
    def liveBricks(self) -> int:
        """``poolUsed - freeList.length`` (VoxelWorld.ts:139-141)."""
        self._ensure()
        s = self._lib.stats(self._h)
        return s["pool_used"] - s["n_holes"]

    @property
    def grid(self) -> np.ndarray:
        self._ensure()
        return self._lib.read_grid(self._h, self.bx * self.by * self.bz)

    @property
    def pool(self) -> np.ndarray:
        self._ensure()
        return self._lib.read_pool(self._h)

    def freeBricks(self) -> np.ndarray:
        """Pool bricks allocated but unused, in push order (VoxelWorld.ts:173-175)."""
        self._ensure()
        return self._lib.read_holes(self._h)

    def cellIndex(self, bx: int, by: int, bz: int) -> int:
        return bx + self.bx * (by + self.by * bz)

    def get(self, x: int, y: int, z: int) -> int:
        """VoxelWorld.ts:55-61."""
        if x < 0 or y < 0 or z < 0 or x >= self.dx or y >= self.dy or z >= self.dz:
            return 0
        g = int(self.grid[(x >> 3) + self.bx * ((y >> 3) + self.by * (z >> 3))])
        if g == 0:
            return 0
        if g & UNIFORM:
            return g & 0xFFFF
        return int(self.pool[(g - 1) * 512 + ((x & 7) | ((y & 7) << 3) | ((z & 7) << 6))])

    def derived(self) -> dict:
        """The upload products of GpuWorld.ts:90-113 (super counts, density, free list)."""
        self._ensure()
        n_super = ((self.bx + 3) // 4) * ((self.by + 3) // 4) * ((self.bz + 3) // 4)
        return self._lib.read_derived(self._h, self.max_bricks, self.bx * self.by * self.bz, n_super)

    def stats(self) -> dict:
        return self._lib.stats(self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
