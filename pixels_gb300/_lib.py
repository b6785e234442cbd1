"""ctypes binding of ``libpixels_gb300.so`` (include/pixels_gb300.h).

The library is the only compute path: if it is missing or cannot find a GPU,
every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PIXELS_GB300_LIB selects another in-tree build of the library (kernel variants)
LIB_PATH = os.environ.get("PIXELS_GB300_LIB", os.path.join(HERE, "libpixels_gb300.so"))

PX_OK = 0
ERRORS = {1: "PX_E_INVALID_ARG", 2: "PX_E_INVALID_IR", 3: "PX_E_OOM", 4: "PX_E_QUEUE_OVERFLOW",
          5: "PX_E_TIMEOUT", 6: "PX_E_CUDA", 7: "PX_E_RANGE", 8: "PX_E_NO_DEVICE", 9: "PX_E_TOO_LARGE"}
PX_NOALLOC_MAX_POOL_BRICKS = 1 << 20

# Every symbol include/pixels_gb300.h declares.
EXPORTS = [
    "px_world_create", "px_world_destroy", "px_world_reset", "px_submit_ops", "px_build", "px_build_enqueue",
    "px_build_finish", "px_read_grid", "px_read_pool", "px_read_holes", "px_derive", "px_read_super",
    "px_read_density", "px_read_free_list", "px_set_material_tables", "px_set_validation", "px_get_stats",
    "px_device_view_get", "px_last_error", "px_probe_peak", "px_world_info", "px_serve_run", "px_derive_noalloc",
    "px_batch_create", "px_batch_run", "px_batch_destroy", "px_batch_last_error", "px_snap_anchors",
    "px_reserve_pool", "px_set_derive_on_build", "px_check_sqrt_bounds",
]


class PxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class DeviceView(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_void_p), ("pool", ctypes.c_void_p), ("holes", ctypes.c_void_p),
                ("super_counts", ctypes.c_void_p), ("density", ctypes.c_void_p), ("free_list", ctypes.c_void_p),
                ("free_len", ctypes.c_uint32), ("pad", ctypes.c_uint32)]


class Edit(ctypes.Structure):
    _fields_ = [("shape", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("a", ctypes.c_double * 3),
                ("b", ctypes.c_double * 3), ("r", ctypes.c_double)]


class EditResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_uint32), ("batch", ctypes.c_uint32),
                ("arrival_s", ctypes.c_double), ("start_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("dev_start_ms", ctypes.c_double), ("dev_end_ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("ops_applied", ctypes.c_uint64), ("pairs", ctypes.c_uint64), ("brick_evals", ctypes.c_uint64),
        ("sub_evals", ctypes.c_uint64), ("voxel_evals", ctypes.c_uint64), ("paint_evals", ctypes.c_uint64),
        ("rescued", ctypes.c_uint64), ("alloc_events", ctypes.c_uint64), ("free_events", ctypes.c_uint64),
        ("pool_used", ctypes.c_uint32), ("n_holes", ctypes.c_uint32), ("pool_capacity", ctypes.c_uint32),
        ("status", ctypes.c_uint32), ("max_abs_err32", ctypes.c_double), ("build_ms", ctypes.c_float),
        ("fold_ms", ctypes.c_float), ("kernel_launches", ctypes.c_uint32), ("pad", ctypes.c_uint32),
        ("violations", ctypes.c_uint64), ("rescued_brick", ctypes.c_uint64), ("rescued_sub", ctypes.c_uint64),
        ("rescued_voxel", ctypes.c_uint64), ("rescued_polygon", ctypes.c_uint64),
        ("classify_ms", ctypes.c_float), ("rescued_paint", ctypes.c_uint32),
    ]


_L = None


def load(path: str = LIB_PATH):
    """Load the library (raises if it was not built)."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m pixels_gb300.build`")
    L = ctypes.CDLL(path)
    vp, sz, u32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32
    L.px_world_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, u32, ctypes.POINTER(vp)]
    L.px_world_destroy.argtypes = [vp]
    L.px_world_reset.argtypes = [vp, ctypes.c_int, vp]
    L.px_world_destroy.restype = None
    L.px_submit_ops.argtypes = [vp, vp, sz]
    L.px_build.argtypes = [vp, ctypes.c_int, vp]
    L.px_build_enqueue.argtypes = [vp, ctypes.c_int, vp]
    L.px_build_finish.argtypes = [vp]
    for f in ("px_read_grid", "px_read_pool", "px_read_holes", "px_read_super", "px_read_density"):
        getattr(L, f).argtypes = [vp, vp, sz]
    L.px_derive.argtypes = [vp]
    L.px_read_free_list.argtypes = [vp, u32, vp, sz, ctypes.POINTER(u32)]
    L.px_set_material_tables.argtypes = [vp, vp, vp]
    L.px_set_validation.argtypes = [vp, ctypes.c_int]
    L.px_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.px_device_view_get.argtypes = [vp, vp]
    L.px_last_error.argtypes = [vp]
    L.px_last_error.restype = ctypes.c_char_p
    L.px_probe_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_float)]
    L.px_world_info.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.px_serve_run.argtypes = [vp, ctypes.POINTER(Edit), ctypes.POINTER(ctypes.c_double), sz, u32, ctypes.c_uint64,
                               ctypes.c_int, vp, ctypes.POINTER(EditResult), ctypes.POINTER(ctypes.c_uint64),
                               ctypes.POINTER(sz)]
    L.px_batch_create.argtypes = [ctypes.POINTER(vp), sz, ctypes.c_int, u32, u32, ctypes.POINTER(vp)]
    L.px_batch_run.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float)]
    L.px_batch_destroy.argtypes = [vp]
    L.px_batch_destroy.restype = None
    L.px_batch_last_error.argtypes = [vp]
    L.px_batch_last_error.restype = ctypes.c_char_p
    L.px_snap_anchors.argtypes = [vp, vp, sz, vp, vp]
    L.px_reserve_pool.argtypes = [vp, ctypes.c_uint64]
    L.px_derive_noalloc.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, u32, vp, vp, vp, vp, vp]
    L.px_set_derive_on_build.argtypes = [vp, u32]
    L.px_check_sqrt_bounds.argtypes = [u32, u32, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(u32)]
    _L = L
    return L


def _check(h, rc: int):
    if rc != PX_OK:
        msg = load().px_last_error(h) if h else b""
        raise PxError(rc, (msg or b"").decode())


def world_create(dx, dy, dz, vpm, initial_pool_bricks):
    from .materials import opaque_table, uniform_density_table
    L = load()
    h = ctypes.c_void_p()
    _check(None, L.px_world_create(dx, dy, dz, vpm, initial_pool_bricks, ctypes.byref(h)))
    op = np.array(opaque_table(), np.uint8)
    ud = np.array(uniform_density_table(), np.uint8)
    _check(h, L.px_set_material_tables(h, op.ctypes.data, ud.ctypes.data))
    return h


def set_derive_on_build(h, max_bricks: int):
    """Every later build ends with super counts, density and the GPU free list
    on the device (0: off)."""
    _check(h, load().px_set_derive_on_build(h, int(max_bricks)))


def set_validation(h, on: bool):
    _check(h, load().px_set_validation(h, int(on)))


def world_destroy(h):
    load().px_world_destroy(h)


def submit_ops(h, ir: bytes):
    buf = ctypes.create_string_buffer(ir, len(ir))
    _check(h, load().px_submit_ops(h, buf, len(ir)))


def build(h, mode: int, stream: int = 0):
    _check(h, load().px_build(h, mode, ctypes.c_void_p(stream)))


def build_enqueue(h, mode: int, stream: int = 0):
    _check(h, load().px_build_enqueue(h, mode, ctypes.c_void_p(stream)))


def build_finish(h):
    _check(h, load().px_build_finish(h))


def world_reset(h, requeue_last_ops: bool = False, stream: int = 0):
    _check(h, load().px_world_reset(h, int(requeue_last_ops), ctypes.c_void_p(stream)))


def stats(h) -> dict:
    s = Stats()
    _check(h, load().px_get_stats(h, ctypes.byref(s)))
    return {k: getattr(s, k) for k, _ in Stats._fields_}


def read_grid(h, n: int) -> np.ndarray:
    out = np.empty(n, np.uint32)
    _check(h, load().px_read_grid(h, out.ctypes.data, n))
    return out


def read_pool(h) -> np.ndarray:
    used = stats(h)["pool_used"]
    out = np.empty(used * 512, np.uint16)
    _check(h, load().px_read_pool(h, out.ctypes.data if used else None, out.size))
    return out


def read_holes(h) -> np.ndarray:
    n = stats(h)["n_holes"]
    out = np.empty(n, np.uint32)
    _check(h, load().px_read_holes(h, out.ctypes.data if n else None, n))
    return out


def read_derived(h, max_bricks: int, n_cells: int, n_super: int) -> dict:
    L = load()
    sup = np.empty(n_super, np.uint32)
    den = np.empty(n_cells, np.uint8)
    _check(h, L.px_read_super(h, sup.ctypes.data, n_super))
    _check(h, L.px_read_density(h, den.ctypes.data, n_cells))
    ln = ctypes.c_uint32()
    _check(h, L.px_read_free_list(h, max_bricks, None, 0, ctypes.byref(ln)))
    fl = np.empty(ln.value, np.uint32)
    _check(h, L.px_read_free_list(h, max_bricks, fl.ctypes.data, fl.size, ctypes.byref(ln)))
    return {"super": sup, "density": den, "free_list": fl}


def probe_peak(fp64: bool) -> float:
    """Measured FMA throughput of the CUDA cores (TFLOP/s)."""
    v = ctypes.c_float()
    _check(None, load().px_probe_peak(int(fp64), ctypes.byref(v)))
    return float(v.value)


def check_sqrt_bounds(lo_bits: int, hi_bits: int):
    """(failures, smallest failing bit pattern) of the float32 evaluator's
    square-root bounds against the IEEE directed square roots."""
    n = ctypes.c_uint64()
    first = ctypes.c_uint32()
    _check(None, load().px_check_sqrt_bounds(int(lo_bits), int(hi_bits), ctypes.byref(n), ctypes.byref(first)))
    return int(n.value), int(first.value)


def serve_run(h, edits, arrivals, max_batch: int, pool_budget: int, mode: int, stream: int = 0):
    """Run the continuous-batching edit server; returns (results array, applied order).

    ``edits``: sequence of (shape, a, b, r) with shape 0 sphere / 1 capsule.
    """
    n = len(edits)
    arr = (Edit * max(n, 1))()
    for i, (shape, a, b, r) in enumerate(edits):
        arr[i].shape = int(shape)
        arr[i].a[:] = [float(v) for v in a]
        arr[i].b[:] = [float(v) for v in b]
        arr[i].r = float(r)
    t = (ctypes.c_double * max(n, 1))(*[float(v) for v in arrivals])
    res = (EditResult * max(n, 1))()
    order = (ctypes.c_uint64 * max(n, 1))()
    n_app = ctypes.c_size_t()
    _check(h, load().px_serve_run(h, arr, t, n, max_batch, pool_budget, mode, ctypes.c_void_p(stream), res, order,
                                  ctypes.byref(n_app)))
    out = np.array([(r.id, r.status, r.batch, r.arrival_s, r.start_s, r.done_s, r.dev_start_ms, r.dev_end_ms)
                    for r in res[:n]],
                   dtype=[("id", "u8"), ("status", "u4"), ("batch", "u4"), ("arrival_s", "f8"), ("start_s", "f8"),
                          ("done_s", "f8"), ("dev_start_ms", "f8"), ("dev_end_ms", "f8")])
    return out, np.array(order[:n_app.value], dtype=np.int64)


def device_view(h) -> DeviceView:
    """Device addresses of a world's buffers (valid until its next build)."""
    v = DeviceView()
    _check(h, load().px_device_view_get(h, ctypes.byref(v)))
    return v


def derive_noalloc(grid_ptr: int, pool_ptr: int, bricks, n_pool_bricks: int, super_ptr: int, density_ptr: int,
                   stream: int = 0) -> None:
    """px_derive_noalloc on caller-held device buffers (addresses as ints)."""
    from .materials import opaque_table, uniform_density_table
    op = np.array(opaque_table(), np.uint8)
    ud = np.array(uniform_density_table(), np.uint8)
    bx, by, bz = bricks
    rc = load().px_derive_noalloc(ctypes.c_void_p(grid_ptr), ctypes.c_void_p(pool_ptr), int(bx), int(by), int(bz),
                                  int(n_pool_bricks), op.ctypes.data, ud.ctypes.data, ctypes.c_void_p(super_ptr),
                                  ctypes.c_void_p(density_ptr), ctypes.c_void_p(stream))
    if rc == 9:
        raise PxError(rc, f"a pool of {n_pool_bricks} bricks exceeds the fixed scratch of px_derive_noalloc "
                          f"({PX_NOALLOC_MAX_POOL_BRICKS} bricks)")
    if rc == 1:
        raise PxError(rc, "bad argument, or the grid names a pool brick beyond n_pool_bricks")
    if rc != PX_OK:
        raise PxError(rc, "px_derive_noalloc failed")


def batch_create(handles, mode: int, n_streams: int, pairs_per_block: int):
    """px_batch_create over world handles; returns the batch handle."""
    L = load()
    arr = (ctypes.c_void_p * len(handles))(*[h.value if isinstance(h, ctypes.c_void_p) else h for h in handles])
    b = ctypes.c_void_p()
    rc = L.px_batch_create(arr, len(handles), mode, n_streams, pairs_per_block, ctypes.byref(b))
    if rc != PX_OK:
        msgs = [(L.px_last_error(h) or b"").decode() for h in handles]
        raise PxError(rc, "; ".join(m for m in msgs if m) or "px_batch_create failed")
    return b


def batch_run(b, stream: int = 0) -> float:
    """Launch the batch's graph and wait; returns its device time in ms."""
    L = load()
    ms = ctypes.c_float()
    rc = L.px_batch_run(b, ctypes.c_void_p(stream), ctypes.byref(ms))
    if rc != PX_OK:
        raise PxError(rc, (L.px_batch_last_error(b) or b"").decode())
    return float(ms.value)


def batch_destroy(b):
    load().px_batch_destroy(b)


def snap_anchors(h, xyz: np.ndarray, emission: np.ndarray) -> np.ndarray:
    """px_snap_anchors: (n, 3) int32 voxel coordinates -> snapped coordinates."""
    xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    out = np.empty_like(xyz)
    em = np.ascontiguousarray(emission, dtype=np.uint8)
    if em.size != 256:
        raise ValueError("emission table must have 256 entries")
    _check(h, load().px_snap_anchors(h, xyz.ctypes.data, xyz.shape[0], em.ctypes.data, out.ctypes.data))
    return out
