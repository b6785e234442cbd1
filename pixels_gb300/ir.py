"""Op-list IR: the byte format the C-ABI library (and the oracle) consume.

A scene is an ordered list of ops, each ``(kind, shape, paint)`` exactly as
``Builder.add/carve/paint`` receives them (``shapes.ts:417-431``).  The shape's
SDF closure tree is flattened into postfix bytecode whose parameters are the
constants the reference's closures capture (already clamped / derived by the
constructors, so both consumers evaluate the same float64 expressions).

Layout (little endian)::

    header  : 8 x u32   magic 'PXIR', version, n_ops, n_code, n_params, 0, 0, 0
    ops     : n_ops x 128 bytes (see OP_DTYPE)
    code    : n_code x 2 u32   (opcode | n << 8, parameter offset)
    params  : n_params x f64

The layout is mirrored by ``include/pixels_gb300.h`` (``px_ir_op``).
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = 0x52495850  # 'PXIR'
VERSION = 1

# op kinds (shapes.ts:325-330)
ADD, CARVE, PAINT = 0, 1, 2

# SDF opcodes
OP_BOX = 1
OP_ROUNDBOX = 2
OP_SPHERE = 3
OP_ELLIPSOID = 4
OP_CYL_X, OP_CYL_Y, OP_CYL_Z = 5, 6, 7
OP_CAPSULE = 8
OP_TORUS_X, OP_TORUS_Y, OP_TORUS_Z = 9, 10, 11
OP_LATHE_SOLID = 12
OP_LATHE_SHELL = 13
OP_PRISM = 14
OP_STADIUM = 15
OP_ROT_X, OP_ROT_Y, OP_ROT_Z = 20, 21, 22
OP_ROT_END = 23
OP_OFFSET = 24
OP_NEGMAX = 25   # subtract step: d = max(d, -b)
OP_MAX = 26      # intersect
OP_MIN = 27      # union

PRIM_NPARAMS = {
    OP_BOX: 6, OP_ROUNDBOX: 7, OP_SPHERE: 4, OP_ELLIPSOID: 7,
    OP_CYL_X: 5, OP_CYL_Y: 5, OP_CYL_Z: 5, OP_CAPSULE: 8,
    OP_TORUS_X: 5, OP_TORUS_Y: 5, OP_TORUS_Z: 5,
    OP_STADIUM: 6,
}
# polygon opcodes: fixed head + 2n point coordinates
POLY_HEAD = {OP_LATHE_SOLID: 3, OP_LATHE_SHELL: 4, OP_PRISM: 4}

# paint kinds (registered device counterparts of the reference's paint closures)
PAINT_CONST = 0
PAINT_CHIP_STACK = 1     # penthouse.ts:371-377
PAINT_TUFTED = 2         # penthouse.ts:495-501
PAINT_CARD = 3           # penthouse.ts:597-600
PAINT_WHITE_KEYS = 4     # penthouse.ts:744-748
PAINT_BLACK_KEYS = 5     # penthouse.ts:749-756
PAINT_VASE = 6           # penthouse.ts:810-816
PAINT_PAINTING = 7       # penthouse.ts:840-845
PAINT_NOISE = 8          # synthetic scenes: integer hash + float32 sine noise
PAINT_NPARAMS = {
    PAINT_CHIP_STACK: 5, PAINT_TUFTED: 3, PAINT_CARD: 4, PAINT_WHITE_KEYS: 2,
    PAINT_BLACK_KEYS: 2, PAINT_VASE: 5, PAINT_PAINTING: 1 + 9 * 4, PAINT_NOISE: 8,
}

OPF_CONTAINS = 1      # shape has the exact AABB ``contains`` test (boxes, shapes.ts:47-48)
OPF_HAS_SLACK = 2     # shape.slack defined (else 1 is used, shapes.ts:336)
OPF_PAINT_FRAME = 4   # paint sees coordinates through a rotateY frame (penthouse.ts:85-92)

OP_DTYPE = np.dtype([
    ("kind", "<u1"), ("flags", "<u1"), ("paint_kind", "<u2"),
    ("paint_value", "<u4"), ("paint_param", "<u4"), ("code_begin", "<u4"),
    ("code_len", "<u4"), ("pad0", "<u4"),
    ("min", "<f8", 3), ("max", "<f8", 3), ("slack", "<f8"),
    ("frame", "<f8", 4),     # px, pz, cos, sin of the paint frame
    ("pad1", "<f8", 2),
])
assert OP_DTYPE.itemsize == 128, OP_DTYPE.itemsize


class Program:
    """Accumulates ops into IR arrays."""

    def __init__(self):
        self.ops: list[tuple] = []
        self.code: list[tuple[int, int]] = []
        self.params: list[float] = []

    def __len__(self):
        return len(self.ops)

    # -- shape flattening -------------------------------------------------
    def _emit(self, node):
        tag = node[0]
        if tag == "prim":
            _, opcode, params, n = node
            off = len(self.params)
            self.params.extend(float(p) for p in params)
            self.code.append((opcode | (n << 8), off))
        elif tag == "rot":
            _, opcode, params, child = node
            off = len(self.params)
            self.params.extend(float(p) for p in params)
            self.code.append((opcode, off))
            self._emit(child)
            self.code.append((OP_ROT_END, 0))
        elif tag == "offset":
            _, child, k = node
            self._emit(child)
            off = len(self.params)
            self.params.append(float(k))
            self.code.append((OP_OFFSET, off))
        elif tag == "sub":
            _, a, bs = node
            self._emit(a)
            for b in bs:
                self._emit(b)
                self.code.append((OP_NEGMAX, 0))
        elif tag == "inter":
            _, a, b = node
            self._emit(a)
            self._emit(b)
            self.code.append((OP_MAX, 0))
        elif tag == "union":
            _, children = node
            for i, c in enumerate(children):
                self._emit(c)
                if i:
                    self.code.append((OP_MIN, 0))
        else:
            raise ValueError(f"unknown shape node {tag!r}")

    def add_op(self, kind: int, shape, paint) -> None:
        from .paints import PaintFn  # local import: paints imports ir
        code_begin = len(self.code)
        self._emit(shape.node)
        code_len = len(self.code) - code_begin
        flags = 0
        if shape.contains:
            flags |= OPF_CONTAINS
        if shape.slack is not None:
            flags |= OPF_HAS_SLACK
        frame = (0.0, 0.0, 1.0, 0.0)
        if isinstance(paint, PaintFn):
            pk = paint.kind
            pv = 0
            pp = len(self.params)
            self.params.extend(float(v) for v in paint.params)
            if paint.frame is not None:
                flags |= OPF_PAINT_FRAME
                frame = tuple(float(v) for v in paint.frame)
        else:
            pk = PAINT_CONST
            pv = int(paint)
            if pv < 0 or pv > 0xFFFF:
                raise ValueError("constant paint must be a u16 voxel value")
            pp = 0
        slack = float(shape.slack) if shape.slack is not None else 1.0
        self.ops.append((kind, flags, pk, pv, pp, code_begin, code_len, 0,
                         tuple(map(float, shape.min)), tuple(map(float, shape.max)), slack,
                         frame, (0.0, 0.0)))

    # -- serialisation ----------------------------------------------------
    def arrays(self):
        ops = np.zeros(len(self.ops), dtype=OP_DTYPE)
        for i, o in enumerate(self.ops):
            ops[i] = o
        code = np.array(self.code, dtype="<u4").reshape(-1, 2) if self.code else np.zeros((0, 2), "<u4")
        params = np.array(self.params, dtype="<f8")
        return ops, code, params

    def to_bytes(self) -> bytes:
        ops, code, params = self.arrays()
        hdr = struct.pack("<8I", MAGIC, VERSION, len(ops), len(code), len(params), 0, 0, 0)
        return hdr + ops.tobytes() + code.tobytes() + params.tobytes()


def decode(buf: bytes):
    """Inverse of ``Program.to_bytes`` (for tests and tools)."""
    magic, version, n_ops, n_code, n_params = struct.unpack_from("<5I", buf, 0)
    if magic != MAGIC or version != VERSION:
        raise ValueError("not a PXIR v1 buffer")
    o = 32
    ops = np.frombuffer(buf, dtype=OP_DTYPE, count=n_ops, offset=o)
    o += n_ops * OP_DTYPE.itemsize
    code = np.frombuffer(buf, dtype="<u4", count=2 * n_code, offset=o).reshape(-1, 2)
    o += 8 * n_code
    params = np.frombuffer(buf, dtype="<f8", count=n_params, offset=o)
    return ops, code, params
