"""Paint kinds: registered counterparts of the reference's paint closures.

The reference paints with arbitrary closures ``(x, y, z) => number``
(``shapes.ts:21-22``).  A closure cannot cross the C ABI, so each paint the
scene uses is a *kind* with a parameter block; the CUDA library holds one
device function per kind (``csrc/paints.cuh``).  Each kind here also has a
Python evaluation (``__call__``) that follows the reference closure line by
line; tests compare it with the device on dense point sets.
"""
from __future__ import annotations

import math
from typing import Sequence

from . import config as _config
from . import ir
from .jsmath import PI, js_hypot, js_round
from .materials import vox


class PaintFn:
    """A paint kind with its parameters and an optional rotateY frame."""

    __slots__ = ("kind", "params", "frame")

    def __init__(self, kind: int, params: Sequence[float], frame=None):
        if len(params) != ir.PAINT_NPARAMS[kind]:
            raise ValueError(f"paint kind {kind} takes {ir.PAINT_NPARAMS[kind]} parameters")
        self.kind = kind
        self.params = tuple(float(p) for p in params)
        self.frame = None if frame is None else tuple(float(v) for v in frame)

    def __call__(self, x: float, y: float, z: float) -> int:
        if self.frame is not None:
            px, pz, c, sn = self.frame
            dx, dz = x - px, z - pz
            x, z = px + c * dx + sn * dz, pz - sn * dx + c * dz
        return _EVAL[self.kind](self.params, x, y, z)

    def __repr__(self):
        return f"PaintFn(kind={self.kind}, frame={self.frame is not None})"


def local_paint(fn: PaintFn, angle: float, pivot) -> PaintFn:
    """``localPaint`` (penthouse.ts:85-92): evaluate ``fn`` in a rotateY frame."""
    if fn.frame is not None:
        raise ValueError("paint already has a frame")
    px, _, pz = map(float, pivot)
    return PaintFn(fn.kind, fn.params, (px, pz, math.cos(angle), math.sin(angle)))


# ---------------------------------------------------------------------------
# Constructors (parameter blocks hold the closure's captured values)

def chip_stack(x, y, z, r, mat) -> PaintFn:
    """penthouse.ts:371-377: striped chip edges on alternate layers."""
    vs = _config.current().voxel_size
    return PaintFn(ir.PAINT_CHIP_STACK, (x, y, z, r - vs * 1.2, mat))


def tufted(z0, floor, mat) -> PaintFn:
    """penthouse.ts:495-501: darker buttons on a diamond grid."""
    return PaintFn(ir.PAINT_TUFTED, (z0, floor, mat))


def card(px, pz, off, mat) -> PaintFn:
    """penthouse.ts:597-600 (inner function; wrap with ``local_paint``)."""
    return PaintFn(ir.PAINT_CARD, (px, pz, off, mat))


def white_keys(x0, mat) -> PaintFn:
    """penthouse.ts:744-748 (inner function; ``x0 = cx - 0.66``)."""
    return PaintFn(ir.PAINT_WHITE_KEYS, (x0, mat))


def black_keys(x0, mat) -> PaintFn:
    """penthouse.ts:749-756 (inner function): returns 0 (air) between keys."""
    return PaintFn(ir.PAINT_BLACK_KEYS, (x0, mat))


def vase(x, y, z, s, mat) -> PaintFn:
    """penthouse.ts:810-816: bands and a sine motif."""
    return PaintFn(ir.PAINT_VASE, (x, y, z, s, mat))


def painting(blobs, mat) -> PaintFn:
    """penthouse.ts:840-845: nine blobs (last hit wins) and a sine stripe."""
    if len(blobs) != 9:
        raise ValueError("painting takes nine blobs")
    flat = []
    for b in blobs:
        flat.extend((b["x"], b["y"], b["r"], b["s"]))
    return PaintFn(ir.PAINT_PAINTING, (mat, *flat))


def noise(seed, scale, fx, fy, fz, thresh, va, vb) -> PaintFn:
    """Procedural paint of the synthetic scenes: integer hash + float32 sine noise.

    Not in the reference (its scenes are fixed); defined here for the
    seeded synthetic workloads, with the same definition on host and device.
    ``va``/``vb`` are full voxel values (``vox(mat, shade)``).
    """
    return PaintFn(ir.PAINT_NOISE, (seed, scale, fx, fy, fz, thresh, va, vb))


# ---------------------------------------------------------------------------
# Python evaluation (mirrors the reference closures; used by tests)

def _chip(p, px, py, pz):
    x, y, z, edge_r, mat = p
    a = math.atan2(pz - z, px - x)
    edge = js_hypot(px - x, pz - z) > edge_r
    stripe = math.fmod(math.floor(((a + PI) / (2 * PI)) * 8), 2) == 0
    layer = math.fmod(math.floor((py - y) / 0.0045), 2)
    return vox(int(mat), 255 if (edge and stripe and layer == 0) else 0)


def _tufted(p, x, y, z):
    z0, floor, mat = p
    u = (z - z0) / 0.16
    v = (y - floor) / 0.16
    du = u - js_round(u)
    dv = v - js_round(v)
    odd = math.fmod(js_round(u) + js_round(v), 2) == 0
    return vox(int(mat), 200 if (odd and js_hypot(du, dv) < 0.12) else 0)


def _card(p, x, y, z):
    px, pz, off, mat = p
    edge = abs(x - px - off) > 0.022 or abs(z - pz) > 0.034
    return vox(int(mat), 0 if edge else 255)


def _white(p, x, y, z):
    x0, mat = p
    k = math.floor((x - x0) / 0.0254)
    f = (x - x0) / 0.0254 - k
    return vox(int(mat), 120 if f < 0.12 else 0)


def _black(p, x, y, z):
    x0, mat = p
    u = (x - x0) / 0.0254
    k = math.floor(u + 0.5)
    f = u + 0.5 - k
    n = math.fmod(math.fmod(k - 1, 7) + 7, 7)
    has = n in (0, 1, 3, 4, 5)
    return vox(int(mat)) if (has and abs(f - 0.5) < 0.3) else 0


def _vase(p, px, py, pz):
    x, y, z, s, mat = p
    a = math.atan2(pz - z, px - x)
    h = (py - y) / s
    band = (0.04 < h < 0.06) or (0.36 < h < 0.38) or (0.47 < h < 0.49)
    motif = 0.08 < h < 0.33 and math.sin(a * 5 + math.sin(h * 30) * 2) > 0.55
    return vox(int(mat), 255 if (band or motif) else 0)


def _painting(p, x, y, z):
    mat = p[0]
    shade = 0
    for i in range(9):
        bx, by, br, bs = p[1 + 4 * i: 5 + 4 * i]
        if js_hypot(x - bx, (y - by) * 1.3) < br:
            shade = bs
    stripe = abs(math.sin(x * 9 + y * 3)) < 0.06
    return vox(int(mat), 255 if stripe else int(shade))


def _f32(v: float) -> float:
    import struct as _s
    return _s.unpack("<f", _s.pack("<f", v))[0]


def noise_hash(ix: int, iy: int, iz: int, seed: int) -> int:
    """32-bit integer hash of a cell (multiply-xorshift mixing, all mod 2^32)."""
    h = (seed ^ (ix * 0x8DA6B343) ^ (iy * 0xD8163841) ^ (iz * 0xCB1AB31F)) & 0xFFFFFFFF
    h ^= h >> 16
    h = (h * 0x7FEB352D) & 0xFFFFFFFF
    h ^= h >> 15
    h = (h * 0x846CA68B) & 0xFFFFFFFF
    h ^= h >> 16
    return h


_C1, _C2, _C3 = _f32(0.0751), _f32(0.6432), _f32(1.5708)


def sin_poly_f32(t: float) -> float:
    """A float32 sine-like wave of a phase ``t`` in turns, in [-1, 1].

    Fold the phase to a triangle wave ``w`` in [-1, 1] and shape it with the
    odd quintic ``w * (1.5708 + w^2 * (-0.6432 + 0.0751 w^2))`` (close to
    ``sin(pi/2 w)``).  Every step is one float32 operation, so host and device
    agree bit for bit.
    """
    f = _f32
    u = f(t - float(math.floor(t)))               # [0, 1)
    v = f(f(u * 4.0) - 2.0)                        # [-2, 2)
    w = f(abs(v) - 1.0)                            # [-1, 1]
    w2 = f(w * w)
    p = f(f(w2 * _C1) - _C2)
    p = f(f(p * w2) + _C3)
    r = f(p * w)
    return r if v >= 0 else -r


def _noise(p, x, y, z):
    seed, scale, fx, fy, fz, thresh, va, vb = p
    ix = math.floor(x * scale)
    iy = math.floor(y * scale)
    iz = math.floor(z * scale)
    h = noise_hash(int(ix) & 0xFFFFFFFF, int(iy) & 0xFFFFFFFF, int(iz) & 0xFFFFFFFF, int(seed) & 0xFFFFFFFF)
    jitter = _f32((h & 0xFFFF) * (1.0 / 65536.0))
    f = _f32
    t = f(f(f(f(x) * f(fx)) + f(f(y) * f(fy))) + f(f(z) * f(fz)))
    t = f(t + jitter)
    s = sin_poly_f32(t)
    return int(va) if s > f(thresh) else int(vb)


_EVAL = {
    ir.PAINT_CHIP_STACK: _chip, ir.PAINT_TUFTED: _tufted, ir.PAINT_CARD: _card,
    ir.PAINT_WHITE_KEYS: _white, ir.PAINT_BLACK_KEYS: _black, ir.PAINT_VASE: _vase,
    ir.PAINT_PAINTING: _painting, ir.PAINT_NOISE: _noise,
}
