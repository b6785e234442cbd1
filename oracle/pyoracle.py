"""ctypes wrapper of the oracle library (test infrastructure only).

Used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` to check and time the CUDA voxeliser.  The product never imports
this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


class OracleResult(ctypes.Structure):
    _fields_ = [
        ("dx", ctypes.c_int32), ("dy", ctypes.c_int32), ("dz", ctypes.c_int32),
        ("bx", ctypes.c_int32), ("by", ctypes.c_int32), ("bz", ctypes.c_int32),
        ("pool_used", ctypes.c_uint32), ("n_free", ctypes.c_uint32),
        ("grid", ctypes.POINTER(ctypes.c_uint32)),
        ("pool", ctypes.POINTER(ctypes.c_uint16)),
        ("free_list", ctypes.POINTER(ctypes.c_uint32)),
        ("pairs", ctypes.c_uint64), ("contains_tests", ctypes.c_uint64),
        ("brick_evals", ctypes.c_uint64), ("sub_evals", ctypes.c_uint64),
        ("voxel_evals", ctypes.c_uint64), ("paint_evals", ctypes.c_uint64),
        ("flops", ctypes.c_uint64), ("divs", ctypes.c_uint64), ("sqrts", ctypes.c_uint64),
        ("trans", ctypes.c_uint64), ("allocs", ctypes.c_uint64), ("frees", ctypes.c_uint64),
        ("error", ctypes.c_char * 256),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.oracle_build.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                   ctypes.POINTER(OracleResult)]
        L.oracle_build.restype = ctypes.c_int
        L.oracle_build_mt.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OracleResult)]
        L.oracle_build_mt.restype = ctypes.c_int
        L.oracle_free.argtypes = [ctypes.POINTER(OracleResult)]
        L.oracle_derive.argtypes = [ctypes.POINTER(OracleResult), ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


class OracleWorld:
    """The world the reference would build from an op list, plus derived buffers."""

    def __init__(self, ir_bytes: bytes, vpm: float, dims, initial_pool_bricks: int = 1 << 15,
                 count_flops: bool = False, threads: int = 1):
        from pixels_gb300.materials import opaque_table, uniform_density_table
        L = lib()
        res = OracleResult()
        buf = ctypes.create_string_buffer(ir_bytes, len(ir_bytes))
        if threads > 1:
            rc = L.oracle_build_mt(buf, len(ir_bytes), float(vpm), int(dims[0]), int(dims[1]), int(dims[2]),
                                   int(threads), ctypes.byref(res))
        else:
            rc = L.oracle_build(buf, len(ir_bytes), float(vpm), int(dims[0]), int(dims[1]), int(dims[2]),
                                int(initial_pool_bricks), int(count_flops), ctypes.byref(res))
        if rc != 0:
            raise ValueError(res.error.decode())
        try:
            self.dims = (res.dx, res.dy, res.dz)
            self.bricks = (res.bx, res.by, res.bz)
            n = res.bx * res.by * res.bz
            self.grid = np.ctypeslib.as_array(res.grid, (n,)).copy()
            self.pool_used = res.pool_used
            self.pool = (np.ctypeslib.as_array(res.pool, (res.pool_used * 512,)).copy()
                         if res.pool_used else np.zeros(0, np.uint16))
            self.free_holes = (np.ctypeslib.as_array(res.free_list, (res.n_free,)).copy()
                               if res.n_free else np.zeros(0, np.uint32))
            self.stats = {k: getattr(res, k) for k in ("pairs", "contains_tests", "brick_evals", "sub_evals",
                                                        "voxel_evals", "paint_evals", "flops", "divs",
                                                        "sqrts", "trans", "allocs", "frees")}
            sx, sy, sz = ((b + 3) // 4 for b in self.bricks)
            self.super_dims = (sx, sy, sz)
            self.super = np.zeros(sx * sy * sz, np.uint32)
            self.density = np.zeros(n, np.uint8)
            op = np.array(opaque_table(), np.uint8)
            ud = np.array(uniform_density_table(), np.uint8)
            L.oracle_derive(ctypes.byref(res), op.ctypes.data, ud.ctypes.data,
                            self.super.ctypes.data, self.density.ctypes.data)
        finally:
            L.oracle_free(ctypes.byref(res))

    @property
    def live_bricks(self) -> int:
        """``poolUsed - freeList.length`` (VoxelWorld.ts:139-141)."""
        return int(self.pool_used - len(self.free_holes))

    def pool_capacity(self, max_bricks: int = 1 << 31) -> int:
        """GpuWorld.ts:55-60."""
        used = self.pool_used
        return min(max_bricks, max(used + 98304, used * 2))

    def free_list(self, max_bricks: int = 1 << 31) -> np.ndarray:
        """GpuWorld.ts:103-108: holes in push order, then ``cap-1 .. used``."""
        cap = self.pool_capacity(max_bricks)
        tail = np.arange(cap - 1, self.pool_used - 1, -1, dtype=np.int64).astype(np.uint32)
        return np.concatenate([self.free_holes.astype(np.uint32), tail])

    def get(self, x: int, y: int, z: int) -> int:
        """VoxelWorld.get (VoxelWorld.ts:55-61)."""
        dx, dy, dz = self.dims
        if x < 0 or y < 0 or z < 0 or x >= dx or y >= dy or z >= dz:
            return 0
        bx, by, _ = self.bricks
        g = int(self.grid[(x >> 3) + bx * ((y >> 3) + by * (z >> 3))])
        if g == 0:
            return 0
        if g & 0x80000000:
            return g & 0xFFFF
        return int(self.pool[(g - 1) * 512 + ((x & 7) | ((y & 7) << 3) | ((z & 7) << 6))])

    def snap_to_emissive(self, emits, x: int, y: int, z: int):
        """snapToEmissive (GpuWorld.ts:165-174): the first emissive voxel of the
        cubes of radius 0..2 around (x, y, z), z then y then x outermost first.
        ``emits(material_byte)`` is True/False, or raises for an unknown material."""
        for r in range(3):
            for oz in range(-r, r + 1):
                for oy in range(-r, r + 1):
                    for ox in range(-r, r + 1):
                        v = self.get(x + ox, y + oy, z + oz)
                        if v and emits(v & 0xFF):
                            return (x + ox, y + oy, z + oz)
        return (x, y, z)

    def live_pool_bricks(self) -> dict:
        """{cell index: brick voxels} for every cell that references the pool."""
        g = self.grid
        cells = np.nonzero((g != 0) & ((g & 0x80000000) == 0))[0]
        return {int(c): self.pool[(int(g[c]) - 1) * 512:int(g[c]) * 512] for c in cells}
