"""SDF shape constructors, CSG, rotations and the ``Builder`` / ``apply`` API.

Drop-in for ``src/world/shapes.ts``.  Every constructor computes the same
float64 constants as the reference closure captures (same expressions, same
operation order) plus the shape's ``min``/``max``/``slack``/``contains``
(``shapes.ts:11-19``).  Instead of a JavaScript closure each shape carries a
descriptor node that ``pixels_gb300.ir`` flattens into SDF bytecode; the
CUDA library evaluates that bytecode on the GPU.

``apply`` does not rasterise immediately: it appends the op to the world's
pending op list; ``VoxelWorld.build()`` (or any read of the world) runs all
pending ops on the GPU in order, with the same result as the reference's
one-op-at-a-time loop (``shapes.ts:334-414``).
"""
from __future__ import annotations

import math
from enum import IntEnum
from typing import Optional, Sequence

from . import config as _config
from . import ir
from .jsmath import js_max, js_min, js_or_eps


class Shape:
    """``interface Shape`` (shapes.ts:11-19) with an SDF descriptor instead of a closure."""

    __slots__ = ("node", "min", "max", "slack", "contains")

    def __init__(self, node, mn, mx, slack: Optional[float] = None, contains: bool = False):
        self.node = node
        self.min = tuple(float(v) for v in mn)
        self.max = tuple(float(v) for v in mx)
        self.slack = None if slack is None else float(slack)
        self.contains = bool(contains)

    def contains_box(self, x0, y0, z0, x1, y1, z1) -> bool:
        """``contains`` of a box (shapes.ts:47-48); only boxes have it."""
        if not self.contains:
            raise AttributeError("shape has no exact contains test")
        n, m = self.min, self.max
        return x0 >= n[0] and x1 <= m[0] and y0 >= n[1] and y1 <= m[1] and z0 >= n[2] and z1 <= m[2]

    def __repr__(self):
        return f"Shape({self.node[0]}, min={self.min}, max={self.max}, slack={self.slack})"


def _prim(opcode, params, n=0):
    return ("prim", opcode, tuple(float(p) for p in params), n)


def _cfg():
    return _config.current()


# ---------------------------------------------------------------------------
# Primitives (shapes.ts:30-222)

def boxMinMax(x0, y0, z0, x1, y1, z1) -> Shape:
    """shapes.ts:30-34."""
    cx, cy, cz = (x0 + x1) / 2, (y0 + y1) / 2, (z0 + z1) / 2
    hx, hy, hz = abs(x1 - x0) / 2, abs(y1 - y0) / 2, abs(z1 - z0) / 2
    return box((cx, cy, cz), (hx, hy, hz))


def box(c, h) -> Shape:
    """shapes.ts:36-50; the only primitive with ``contains``."""
    cx, cy, cz = map(float, c)
    hx, hy, hz = map(float, h)
    return Shape(_prim(ir.OP_BOX, (cx, cy, cz, hx, hy, hz)),
                 (cx - hx, cy - hy, cz - hz), (cx + hx, cy + hy, cz + hz), None, True)


def roundBox(c, h, r) -> Shape:
    """shapes.ts:52-63."""
    cx, cy, cz = map(float, c)
    r = float(r)
    hx, hy, hz = h[0] - r, h[1] - r, h[2] - r
    return Shape(_prim(ir.OP_ROUNDBOX, (cx, cy, cz, hx, hy, hz, r)),
                 (cx - h[0], cy - h[1], cz - h[2]), (cx + h[0], cy + h[1], cz + h[2]))


def sphere(c, r) -> Shape:
    """shapes.ts:65-72."""
    cx, cy, cz = map(float, c)
    r = float(r)
    return Shape(_prim(ir.OP_SPHERE, (cx, cy, cz, r)),
                 (cx - r, cy - r, cz - r), (cx + r, cy + r, cz + r))


def ellipsoid(c, r) -> Shape:
    """shapes.ts:74-84; ``slack = max(r)/min(r)`` widens the classify thresholds."""
    cx, cy, cz = map(float, c)
    rx, ry, rz = map(float, r)
    rmin = js_min(rx, ry, rz)
    return Shape(_prim(ir.OP_ELLIPSOID, (cx, cy, cz, rx, ry, rz, rmin)),
                 (cx - rx, cy - ry, cz - rz), (cx + rx, cy + ry, cz + rz),
                 js_max(rx, ry, rz) / rmin)


_AXIS_CYL = {"x": ir.OP_CYL_X, "y": ir.OP_CYL_Y, "z": ir.OP_CYL_Z}
_AXIS_TORUS = {"x": ir.OP_TORUS_X, "y": ir.OP_TORUS_Y, "z": ir.OP_TORUS_Z}


def cylinder(c, r, halfHeight, axis: str = "y") -> Shape:
    """Capped cylinder (shapes.ts:89-103); radius and height clamped to the voxel size."""
    cfg = _cfg()
    r = js_max(float(r), cfg.min_column_r)
    halfHeight = js_max(float(halfHeight), cfg.voxel_size * 0.5)
    cx, cy, cz = map(float, c)
    if axis == "y":
        ext = (r, halfHeight, r)
    elif axis == "x":
        ext = (halfHeight, r, r)
    else:
        ext = (r, r, halfHeight)
    return Shape(_prim(_AXIS_CYL[axis], (cx, cy, cz, r, halfHeight)),
                 (cx - ext[0], cy - ext[1], cz - ext[2]), (cx + ext[0], cy + ext[1], cz + ext[2]))


def capsule(a, b, r) -> Shape:
    """shapes.ts:114-128; ``bb || 1e-12`` guards a zero-length segment."""
    cfg = _cfg()
    r = js_max(float(r), cfg.min_line_r)
    ax, ay, az = map(float, a)
    b = tuple(map(float, b))
    bax, bay, baz = b[0] - ax, b[1] - ay, b[2] - az
    bb = js_or_eps(bax * bax + bay * bay + baz * baz)
    return Shape(_prim(ir.OP_CAPSULE, (ax, ay, az, bax, bay, baz, bb, r)),
                 (js_min(ax, b[0]) - r, js_min(ay, b[1]) - r, js_min(az, b[2]) - r),
                 (js_max(ax, b[0]) + r, js_max(ay, b[1]) + r, js_max(az, b[2]) + r))


def torus(c, R, r, axis: str = "y") -> Shape:
    """shapes.ts:130-143."""
    cfg = _cfg()
    r = js_max(float(r), cfg.min_line_r)
    R = float(R)
    cx, cy, cz = map(float, c)
    e = R + r
    if axis == "y":
        ext = (e, r, e)
    elif axis == "x":
        ext = (r, e, e)
    else:
        ext = (e, e, r)
    return Shape(_prim(_AXIS_TORUS[axis], (cx, cy, cz, R, r)),
                 (cx - ext[0], cy - ext[1], cz - ext[2]), (cx + ext[0], cy + ext[1], cz + ext[2]))


def lathe(c, profile: Sequence[float], shell: float = 0) -> Shape:
    """Surface of revolution around the vertical axis through ``c`` (shapes.ts:180-202).

    Solid lathes close the profile against the axis (``poly``, ``:194``);
    shell lathes are a wall of thickness ``shell`` around the open polyline.
    """
    cfg = _cfg()
    shell = float(shell)
    profile = [float(v) for v in profile]
    if len(profile) < 4 or len(profile) % 2:
        raise ValueError("lathe profile needs at least two (r, y) points")
    if shell > 0:
        shell = js_max(shell, cfg.min_shell)
    cx, cy, cz = map(float, c)
    rmax, ymin, ymax = 0.0, math.inf, -math.inf
    for i in range(0, len(profile), 2):
        rmax = js_max(rmax, profile[i])
        ymin = js_min(ymin, profile[i + 1])
        ymax = js_max(ymax, profile[i + 1])
    pad = shell / 2
    if shell > 0:
        node = _prim(ir.OP_LATHE_SHELL, (cx, cy, cz, shell / 2, *profile), len(profile) // 2)
    else:
        poly = [0.0, profile[1], *profile, 0.0, profile[-1]]
        node = _prim(ir.OP_LATHE_SOLID, (cx, cy, cz, *poly), len(poly) // 2)
    return Shape(node,
                 (cx - rmax - pad, cy + ymin - pad, cz - rmax - pad),
                 (cx + rmax + pad, cy + ymax + pad, cz + rmax + pad))


def prism(c, pts: Sequence[float], y0, y1) -> Shape:
    """Closed xz polygon (relative to ``c``) extruded over ``[y0, y1]`` (shapes.ts:205-222)."""
    cx, _, cz = map(float, c)
    pts = [float(v) for v in pts]
    if len(pts) < 6 or len(pts) % 2:
        raise ValueError("prism needs a polygon of at least three points")
    y0, y1 = float(y0), float(y1)
    x0, x1, z0, z1 = math.inf, -math.inf, math.inf, -math.inf
    for i in range(0, len(pts), 2):
        x0 = js_min(x0, pts[i]); x1 = js_max(x1, pts[i])
        z0 = js_min(z0, pts[i + 1]); z1 = js_max(z1, pts[i + 1])
    ym, hy = (y0 + y1) / 2, (y1 - y0) / 2
    return Shape(_prim(ir.OP_PRISM, (cx, cz, ym, hy, *pts), len(pts) // 2),
                 (cx + x0, y0, cz + z0), (cx + x1, y1, cz + z1))


def stadium(c, hl, r, y0, y1) -> Shape:
    """Rounded-rectangle slab (the reference's scene-local ``stadium``, penthouse.ts:69-82).

    A library constructor here because a closure literal cannot cross the
    C ABI; the SDF uses ``Math.hypot`` twice.
    """
    cx, _, cz = map(float, c)
    hl, r, y0, y1 = float(hl), float(r), float(y0), float(y1)
    ym, hy = (y0 + y1) / 2, (y1 - y0) / 2
    return Shape(_prim(ir.OP_STADIUM, (cx, cz, hl, r, ym, hy)),
                 (cx - hl - r, y0, cz - r), (cx + hl + r, y1, cz + r))


def offset(s: Shape, k: float) -> Shape:
    """``{sdf: s.sdf + k, min, max, slack}`` (the foam core of penthouse.ts:250).

    Keeps the bounds and slack, drops ``contains`` like the literal does.
    """
    return Shape(("offset", s.node, float(k)), s.min, s.max, s.slack, False)


# ---------------------------------------------------------------------------
# Combinators (shapes.ts:227-320)

def _slack_or_1(s: Shape) -> float:
    return 1.0 if s.slack is None else s.slack


def union(*shapes: Shape) -> Shape:
    """shapes.ts:227-238."""
    if not shapes:
        raise ValueError("union of nothing")
    mn = tuple(js_min(*(s.min[i] for s in shapes)) for i in range(3))
    mx = tuple(js_max(*(s.max[i] for s in shapes)) for i in range(3))
    return Shape(("union", tuple(s.node for s in shapes)), mn, mx,
                 js_max(1.0, *(_slack_or_1(s) for s in shapes)))


def subtract(a: Shape, *b: Shape) -> Shape:
    """shapes.ts:240-251: keeps ``a``'s bounds."""
    return Shape(("sub", a.node, tuple(s.node for s in b)), a.min, a.max,
                 js_max(_slack_or_1(a), *(_slack_or_1(s) for s in b)))


def intersect(a: Shape, b: Shape) -> Shape:
    """shapes.ts:253-260: bounds are the box intersection."""
    mn = tuple(js_max(a.min[i], b.min[i]) for i in range(3))
    mx = tuple(js_min(a.max[i], b.max[i]) for i in range(3))
    return Shape(("inter", a.node, b.node), mn, mx, js_max(_slack_or_1(a), _slack_or_1(b)))


def rotateY(s: Shape, angle: float, pivot) -> Shape:
    """Rotate about the vertical axis through ``pivot`` (shapes.ts:263-280)."""
    c, sn = math.cos(angle), math.sin(angle)
    px, _, pz = map(float, pivot)
    corners = []
    for x in (s.min[0], s.max[0]):
        for z in (s.min[2], s.max[2]):
            dx, dz = x - px, z - pz
            corners.append((px + c * dx - sn * dz, 0.0, pz + sn * dx + c * dz))
    mn = (js_min(*(k[0] for k in corners)), s.min[1], js_min(*(k[2] for k in corners)))
    mx = (js_max(*(k[0] for k in corners)), s.max[1], js_max(*(k[2] for k in corners)))
    return Shape(("rot", ir.OP_ROT_Y, (px, pz, c, sn), s.node), mn, mx, s.slack)


def rotateX(s: Shape, angle: float, pivot) -> Shape:
    """Rotate about the x axis through ``pivot`` (shapes.ts:283-300)."""
    c, sn = math.cos(angle), math.sin(angle)
    _, py, pz = map(float, pivot)
    corners = []
    for y in (s.min[1], s.max[1]):
        for z in (s.min[2], s.max[2]):
            dy, dz = y - py, z - pz
            corners.append((0.0, py + c * dy - sn * dz, pz + sn * dy + c * dz))
    mn = (s.min[0], js_min(*(k[1] for k in corners)), js_min(*(k[2] for k in corners)))
    mx = (s.max[0], js_max(*(k[1] for k in corners)), js_max(*(k[2] for k in corners)))
    return Shape(("rot", ir.OP_ROT_X, (py, pz, c, sn), s.node), mn, mx, s.slack)


def rotateZ(s: Shape, angle: float, pivot) -> Shape:
    """Rotate about the z axis through ``pivot`` (shapes.ts:303-320)."""
    c, sn = math.cos(angle), math.sin(angle)
    px, py = float(pivot[0]), float(pivot[1])
    corners = []
    for x in (s.min[0], s.max[0]):
        for y in (s.min[1], s.max[1]):
            dx, dy = x - px, y - py
            corners.append((px + c * dx - sn * dy, py + sn * dx + c * dy, 0.0))
    mn = (js_min(*(k[0] for k in corners)), js_min(*(k[1] for k in corners)), s.min[2])
    mx = (js_max(*(k[0] for k in corners)), js_max(*(k[1] for k in corners)), s.max[2])
    return Shape(("rot", ir.OP_ROT_Z, (px, py, c, sn), s.node), mn, mx, s.slack)


# ---------------------------------------------------------------------------
# Rasteriser API (shapes.ts:325-431)

class Op(IntEnum):
    """shapes.ts:325-330."""
    Add = ir.ADD
    Carve = ir.CARVE
    Paint = ir.PAINT


def apply(world, shape: Shape, op: Op, paint=0) -> None:
    """Rasterise ``shape`` into ``world`` (shapes.ts:334-414).

    The op is queued on the world and executed, in order with every other
    queued op, by the GPU build the next time the world is built or read.
    """
    world.submit(int(op), shape, paint)


class Builder:
    """Convenience wrapper that collects scene operations (shapes.ts:416-431)."""

    def __init__(self, world):
        self.world = world

    def add(self, shape: Shape, paint) -> "Builder":
        apply(self.world, shape, Op.Add, paint)
        return self

    def carve(self, shape: Shape) -> "Builder":
        apply(self.world, shape, Op.Carve)
        return self

    def paint(self, shape: Shape, paint) -> "Builder":
        apply(self.world, shape, Op.Paint, paint)
        return self
