"""The penthouse scene program (restates ``src/scene/penthouse.ts``).

A deterministic list of ``Builder.add/carve/paint`` calls (seeded with the
reference's mulberry32 ``rng(1337)`` and ``rng(5)``).  Every constant and
every expression keeps the reference's float64 operation order, because the
scene itself depends on the voxel density (``snap``, ``VS``) and on the exact
placement values.  Host transcendentals (``cos``/``sin``/``atan2``) come from
the C library; ``Math.hypot`` uses the engine's scaled compensated method
(``jsmath.js_hypot``).  Lights are returned as plain records (they are not
part of the world build).
"""
from __future__ import annotations

import math

from .. import config as _config
from ..jsmath import js_hypot, js_max, js_round, mulberry32
from ..materials import M, vox
from ..paints import (black_keys, card, chip_stack, local_paint, painting, tufted,
                      vase as vase_paint, white_keys)
from ..shapes import (Builder, box, boxMinMax, capsule, cylinder, ellipsoid, intersect, lathe,
                      offset, prism, rotateX, rotateY, rotateZ, roundBox, sphere, stadium,
                      subtract, torus)
from .font import layout_text

PI = math.pi
RW = 16   # room width (x), penthouse.ts:52
RD = 12   # room depth (z), penthouse.ts:53


class _Ctx:
    """The module-level constants of penthouse.ts:47-51 at one voxel density."""

    def __init__(self, vpm: float):
        from ..config import BRICK
        self.vpm = vpm
        self.VS = 1 / vpm
        self.BRICK_M = BRICK / vpm

        def snap(m):
            return (js_round((m * vpm) / BRICK) * BRICK) / vpm

        self.snap = snap
        self.FLOOR = snap(0.2)
        self.CEIL = snap(4.1)
        self.WALL = snap(0.25)


def build_penthouse(world, progress=None) -> dict:
    """``buildPenthouse`` (penthouse.ts:94-170): queue every op of the scene on ``world``."""
    with _config.using(world.vpm):
        return _build(world, _Ctx(world.vpm), progress)


def penthouse_program(vpm: float):
    """The scene as an op program (no world needed): returns ``(Program, scene)``."""
    from ..world import OpRecorder
    rec = OpRecorder(vpm)
    scene = build_penthouse(rec)
    return rec.program, scene


def _build(world, C: _Ctx, progress):
    B = Builder(world)
    lights = []
    R = mulberry32(1337)
    steps = 16
    step = [0]

    def stage(msg):
        if progress:
            progress(msg, step[0] / steps)
        step[0] += 1

    FLOOR, CEIL, VS = C.FLOOR, C.CEIL, C.VS

    stage("Pouring the floor slab")
    _shell(B, C)
    stage("Glazing the Strip view")
    _windows(B, C)
    stage("Rolling out the casino carpet")
    B.add(boxMinMax(4.3, FLOOR - VS * 0.5, 6.3, 11.6, FLOOR + 2 * VS, 11.3), vox(M.carpet))
    _column(B, C, 4.1, 5.6)
    _column(B, C, 12.1, 5.9)
    stage("Upholstering the sectional")
    _sofa(B, C)
    stage("Setting the coffee table")
    _coffee_table(B, C, 7.9, 8.85, R)
    stage("Hanging the chandelier")
    lights.append(_chandelier(B, C, 7.9, 8.85, R))
    lights.append(dict(pos=(7.9, CEIL + 0.05, 8.85), radius=4, color=(1.0, 0.7, 0.4), shadow=False, anchors=[]))
    stage("Plugging in the lamps")
    lights.append(_floor_lamp(B, C, 10.85, 6.95))
    lights.append(_floor_lamp(B, C, 5.25, 10.55))
    stage("Stocking the bar")
    lights.extend(_bar(B, C, R))
    stage("Shuffling the cards")
    lights.extend(_poker_table(B, C, 11.4, 3.5, R))
    stage("Loading the slots")
    for i in range(4):
        lights.append(_slot_machine(B, C, 12.75 + i * 0.78, 0.25, i, R))
    stage("Tuning the piano")
    _piano(B, C, 13.45, 8.7, -0.55)
    stage("Building the champagne tower")
    _champagne_tower(B, C, 10.75, 10.45)
    stage("Mounting the TV")
    lights.append(_tv(B, C))
    stage("Lighting the neon")
    lights.extend(_neon_signs(B, C))
    stage("Placing priceless art")
    _decor(B, C, R)
    stage("Watering the palms")
    _palm(B, C, 0.85, 11.05, R)
    _palm(B, C, 15.1, 5.0, R)
    _palm(B, C, 0.85, 0.85, R)
    lights.append(dict(pos=(3.0, CEIL - 0.2, 10.0), radius=5, color=(0.9, 0.7, 0.5), shadow=False, anchors=[]))
    lights.append(dict(pos=(6.0, CEIL - 0.2, 2.5), radius=5, color=(0.9, 0.7, 0.5), shadow=False, anchors=[]))
    lights.append(dict(pos=(14.0, CEIL - 0.2, 11.0), radius=4.5, color=(0.8, 0.65, 0.5), shadow=False, anchors=[]))
    if progress:
        progress("Done", 1)
    return dict(lights=lights, spawn=dict(pos=(7.6, FLOOR, 4.6), yaw=PI * 0.82, pitch=-0.08))


# ---------------------------------------------------------------------------

def _shell(B, C):
    """penthouse.ts:174-206."""
    FLOOR, CEIL, WALL, BRICK_M, snap = C.FLOOR, C.CEIL, C.WALL, C.BRICK_M, C.snap
    B.add(boxMinMax(0, 0, 0, RW, FLOOR, RD), vox(M.floor))
    B.add(boxMinMax(0, CEIL, 0, RW, 4.4, RD), vox(M.ceiling))
    B.carve(cylinder((7.9, CEIL + 0.07, 8.85), 2.4, 0.08))
    B.add(torus((7.9, CEIL + 0.005, 8.85), 2.42, 0.03), vox(M.gold))
    B.add(torus((7.9, CEIL + 0.11, 8.85), 2.32, 0.012), vox(M.lampshade))
    B.add(boxMinMax(WALL, CEIL - 0.06, WALL, RW - WALL, CEIL, WALL + 0.03), vox(M.gold))
    B.add(boxMinMax(WALL, CEIL - 0.06, WALL, WALL + 0.03, CEIL, RD - WALL), vox(M.gold))
    B.add(boxMinMax(0, FLOOR, 0, WALL, CEIL, RD), vox(M.concrete))
    B.add(boxMinMax(0, FLOOR, 0, RW, CEIL, WALL), vox(M.concrete))
    B.add(boxMinMax(WALL - BRICK_M, FLOOR, WALL, WALL, CEIL, RD), vox(M.wall))
    B.add(boxMinMax(WALL, FLOOR, WALL - BRICK_M, RW, CEIL, WALL), vox(M.wall))
    B.add(boxMinMax(WALL - BRICK_M, FLOOR, snap(2.1), WALL, CEIL, snap(7.9)), vox(M.wallDark))
    B.add(boxMinMax(WALL, FLOOR, WALL, WALL + 0.02, FLOOR + 0.12, RD - WALL), vox(M.marbleBlack))
    B.add(boxMinMax(WALL, FLOOR, WALL, RW - WALL, FLOOR + 0.12, WALL + 0.02), vox(M.marbleBlack))
    B.add(boxMinMax(1.2, FLOOR, WALL - 0.02, 3.0, FLOOR + 2.55, WALL + 0.04), vox(M.marbleBlack))
    B.add(boxMinMax(1.3, FLOOR, WALL, 2.9, FLOOR + 2.45, WALL + 0.05), vox(M.walnutY))
    B.carve(boxMinMax(2.095, FLOOR, WALL + 0.035, 2.105, FLOOR + 2.45, WALL + 0.06))
    for x in (1.98, 2.22):
        B.add(capsule((x, FLOOR + 0.9, WALL + 0.09), (x, FLOOR + 1.3, WALL + 0.09), 0.012), vox(M.gold))
    for x in (1.98, 2.22):
        B.add(capsule((x, FLOOR + 0.95, WALL + 0.04), (x, FLOOR + 0.95, WALL + 0.09), 0.008), vox(M.gold))
        B.add(capsule((x, FLOOR + 1.25, WALL + 0.04), (x, FLOOR + 1.25, WALL + 0.09), 0.008), vox(M.gold))


def _windows(B, C):
    """penthouse.ts:208-233."""
    FLOOR, CEIL, WALL, VS = C.FLOOR, C.CEIL, C.WALL, C.VS
    g = 2 * VS
    B.add(boxMinMax(WALL, FLOOR, 11.8, RW - WALL, CEIL, 11.8 + g), vox(M.windowGlass))
    B.add(boxMinMax(15.8 - g, FLOOR, WALL, 15.8, CEIL, 11.8 + g), vox(M.windowGlass))
    frame = vox(M.frame)
    B.add(boxMinMax(WALL, FLOOR, 11.72, RW - WALL + 0.2, FLOOR + 0.06, 11.92), frame)
    B.add(boxMinMax(WALL, CEIL - 0.14, 11.72, RW - WALL + 0.2, CEIL, 11.92), frame)
    B.add(boxMinMax(15.65, FLOOR, WALL, 15.88, FLOOR + 0.06, 11.92), frame)
    B.add(boxMinMax(15.65, CEIL - 0.14, WALL, 15.88, CEIL, 11.92), frame)
    n = 8
    for i in range(n + 1):
        x = WALL + ((RW - 2 * WALL) * i) / n
        B.add(boxMinMax(x - 0.04, FLOOR, 11.72, x + 0.04, CEIL, 11.92), frame)
    m = 6
    for i in range(m + 1):
        z = WALL + ((11.8 - WALL) * i) / m
        B.add(boxMinMax(15.65, FLOOR, z - 0.04, 15.88, CEIL, z + 0.04), frame)
    B.add(boxMinMax(15.62, FLOOR, 11.7, 15.9, CEIL, 11.95), frame)


def _column(B, C, x, z):
    """penthouse.ts:235-242."""
    FLOOR, CEIL = C.FLOOR, C.CEIL
    B.add(box((x, FLOOR + 0.08, z), (0.32, 0.08, 0.32)), vox(M.marbleBlack))
    B.add(cylinder((x, (FLOOR + CEIL) / 2, z), 0.24, (CEIL - FLOOR) / 2 - 0.1), vox(M.marble))
    B.add(torus((x, FLOOR + 0.2, z), 0.25, 0.035), vox(M.gold))
    B.add(torus((x, CEIL - 0.3, z), 0.25, 0.03), vox(M.gold))
    B.add(lathe((x, CEIL - 0.28, z), (0.24, 0, 0.3, 0.12, 0.34, 0.18), 0), vox(M.gold))
    B.add(box((x, CEIL - 0.05, z), (0.36, 0.05, 0.36)), vox(M.marbleBlack))


def _upholstered(B, s, cover, inset, inner=M.foam):
    """penthouse.ts:247-252: cover, then a foam core ``{sdf: s.sdf + inset}``."""
    B.add(s, vox(cover))
    B.add(offset(s, inset), vox(inner))


def _sofa(B, C):
    """penthouse.ts:254-294."""
    FLOOR, VS = C.FLOOR, C.VS
    y0 = FLOOR + 2 * VS
    legH = 0.07
    v = M.velvet
    lx0, lx1, lz0, lz1 = 4.75, 10.45, 6.45, 7.4
    sx0, sx1, sz1 = 4.75, 5.7, 10.1
    for x, z in ((lx0 + 0.06, lz0 + 0.06), (lx1 - 0.06, lz0 + 0.06), (lx1 - 0.06, lz1 - 0.06),
                 (sx0 + 0.06, sz1 - 0.06), (sx1 - 0.06, sz1 - 0.06), (sx1 - 0.06, lz1 + 0.3)):
        B.add(cylinder((x, y0 + legH / 2, z), 0.025, legH / 2 + VS), vox(M.gold))
    base = y0 + legH
    _upholstered(B, roundBox(((lx0 + lx1) / 2, base + 0.16, (lz0 + lz1) / 2), ((lx1 - lx0) / 2, 0.16, (lz1 - lz0) / 2), 0.03), v, 0.03)
    _upholstered(B, roundBox(((sx0 + sx1) / 2, base + 0.16, (lz1 + sz1) / 2), ((sx1 - sx0) / 2, 0.16, (sz1 - lz1) / 2 + 0.02), 0.03), v, 0.03)
    _upholstered(B, roundBox(((lx0 + lx1) / 2, base + 0.42, lz0 + 0.12), ((lx1 - lx0) / 2, 0.42, 0.12), 0.06), v, 0.04)
    _upholstered(B, roundBox((sx0 + 0.12, base + 0.42, (lz0 + sz1) / 2), (0.12, 0.42, (sz1 - lz0) / 2), 0.06), v, 0.04)
    _upholstered(B, roundBox((lx1 - 0.11, base + 0.3, (lz0 + lz1) / 2), (0.11, 0.3, (lz1 - lz0) / 2), 0.05), v, 0.04)
    _upholstered(B, roundBox(((sx0 + sx1) / 2, base + 0.3, sz1 - 0.11), ((sx1 - sx0) / 2, 0.3, 0.11), 0.05), v, 0.04)
    seatY = base + 0.32 + 0.07
    n = 4
    cx0, cx1 = lx0 + 0.24, lx1 - 0.22
    for i in range(n):
        a = cx0 + ((cx1 - cx0) * i) / n + 0.008
        b = cx0 + ((cx1 - cx0) * (i + 1)) / n - 0.008
        _upholstered(B, roundBox(((a + b) / 2, seatY, (lz0 + 0.24 + lz1) / 2), ((b - a) / 2, 0.075, (lz1 - lz0 - 0.24) / 2), 0.05), v, 0.035)
    for i in range(2):
        a = lz1 + (i * (sz1 - 0.22 - lz1)) / 2 + 0.008
        b = lz1 + ((i + 1) * (sz1 - 0.22 - lz1)) / 2 - 0.008
        _upholstered(B, roundBox(((sx0 + 0.24 + sx1) / 2, seatY, (a + b) / 2), ((sx1 - sx0 - 0.24) / 2, 0.075, (b - a) / 2), 0.05), v, 0.035)
    _upholstered(B, roundBox(((sx0 + 0.24 + sx1) / 2, seatY, (lz0 + 0.24 + lz1) / 2), ((sx1 - sx0 - 0.24) / 2 - 0.008, 0.075, (lz1 - lz0 - 0.24) / 2), 0.05), v, 0.035)

    def pil(c, yaw, mat):
        _upholstered(B, rotateY(rotateX(ellipsoid(c, (0.2, 0.18, 0.07)), -0.35, c), yaw, c), mat, 0.03, M.foam)

    pil((6.2, seatY + 0.22, lz0 + 0.33), 0, M.velvetGold)
    pil((8.9, seatY + 0.22, lz0 + 0.33), 0.15, M.velvetRed)
    pil((sx0 + 0.33, seatY + 0.22, 9.2), PI / 2, M.velvetGold)


def _coupe(B, C, x, y, z, fill):
    """penthouse.ts:296-302."""
    VS = C.VS
    t = 1.4 * VS
    B.add(lathe((x, y, z), (0, t / 2, 0.034, t / 2), t), vox(M.glassClear))
    B.add(cylinder((x, y + 0.045, z), js_max(0.006, VS * 0.6), 0.04), vox(M.glassClear))
    B.add(lathe((x, y, z), (0.006, 0.085, 0.03, 0.09, 0.048, 0.105, 0.056, 0.125), t), vox(M.glassClear))
    if fill:
        B.add(intersect(lathe((x, y, z), (0.006, 0.088, 0.028, 0.093, 0.045, 0.106, 0.05, 0.116), 0),
                        box((x, y + 0.1, z), (0.06, 0.016, 0.06))), vox(M.champagne))


def _bottle(B, C, x, y, z, R, kind=None):
    """penthouse.ts:304-340."""
    VS = C.VS
    k = kind if kind is not None else math.floor(R() * 4)
    t = 1.5 * VS
    glasses = (M.glassGreen, M.glassAmber, M.glassSmoke, M.glassBlue, M.glassRed, M.glassClear)
    liquids = (M.wine, M.whiskey, M.absinthe, M.champagne, M.water)
    g = glasses[math.floor(R() * len(glasses))]
    liq = liquids[math.floor(R() * len(liquids))]
    fill = 0.5 + R() * 0.45
    c = (x, y, z)
    if k == 0:
        r = 0.034
        B.add(lathe(c, (0, t / 2, r, t / 2, r, 0.2, 0.016, 0.25, 0.013, 0.31), t), vox(g))
        B.add(intersect(cylinder((x, y + 0.11, z), r - t, 0.1), box((x, y + t + 0.1 * fill, z), (r, 0.1 * fill, r))), vox(liq))
        shp = subtract(cylinder((x, y + 0.11, z), r + VS, 0.045), cylinder((x, y + 0.11, z), r - t * 0.7, 0.05))
        B.paint(shp, vox(M.label, 1 + math.floor(R() * 200)))
        shp = cylinder((x, y + 0.305, z), 0.015, 0.012)
        B.add(shp, vox(M.gold if R() < 0.5 else M.cork))
    elif k == 1:
        h = 0.17
        B.add(subtract(roundBox((x, y + h / 2, z), (0.04, h / 2, 0.04), 0.01),
                       roundBox((x, y + h / 2 + t, z), (0.04 - t, h / 2, 0.04 - t), 0.008)), vox(g))
        B.add(box((x, y + t + (h * fill) / 2, z), (0.04 - t - VS * 0.2, (h * fill) / 2, 0.04 - t - VS * 0.2)), vox(M.whiskey))
        B.add(cylinder((x, y + h + 0.02, z), 0.014, 0.025), vox(g))
        B.add(sphere((x, y + h + 0.06, z), 0.022), vox(M.glassClear))
    elif k == 2:
        B.add(lathe(c, (0, t / 2, 0.03, t / 2, 0.052, 0.06, 0.05, 0.12, 0.02, 0.18, 0.012, 0.24), t), vox(g))
        B.add(intersect(lathe(c, (0, t, 0.026, t, 0.046, 0.06, 0.044, 0.12, 0.015, 0.18), 0),
                        box((x, y + 0.1 * fill, z), (0.06, 0.1 * fill, 0.06))), vox(liq))
        B.add(cylinder((x, y + 0.245, z), 0.013, 0.012), vox(M.cork))
    else:
        r = 0.042
        B.add(lathe(c, (0, t / 2, r, t / 2, r, 0.2, 0.02, 0.27, 0.016, 0.33), t), vox(M.glassGreen))
        B.add(intersect(cylinder((x, y + 0.11, z), r - t, 0.1), box((x, y + t + 0.1 * fill, z), (r, 0.1 * fill, r))), vox(M.champagne))
        B.add(lathe(c, (0.022, 0.26, 0.018, 0.3, 0.018, 0.34), 1.2 * VS), vox(M.gold))
        B.paint(subtract(cylinder((x, y + 0.1, z), r + VS, 0.04), cylinder((x, y + 0.1, z), r - t * 0.7, 0.05)), vox(M.label, 1))


_PIP_LAYOUTS = {
    1: ((0, 0),),
    2: ((-1, -1), (1, 1)),
    3: ((-1, -1), (0, 0), (1, 1)),
    4: ((-1, -1), (1, 1), (-1, 1), (1, -1)),
    5: ((-1, -1), (1, 1), (-1, 1), (1, -1), (0, 0)),
    6: ((-1, -1), (1, 1), (-1, 1), (1, -1), (-1, 0), (1, 0)),
}


def _dice(B, C, c, s, yaw):
    """penthouse.ts:342-366."""
    h = s / 2
    die = roundBox(c, (h, h, h), s * 0.12)
    B.add(rotateY(die, yaw, c), vox(M.dieRed))
    pr = s * 0.09
    off = s * 0.27

    def pips_on(n, face):
        for u, v in _PIP_LAYOUTS[n]:
            B.add(rotateY(sphere(face(u * off, v * off), pr), yaw, c), vox(M.pip))

    x, y, z = c
    e = h - pr * 0.35
    pips_on(5, lambda u, v: (x + u, y + e, z + v))
    pips_on(3, lambda u, v: (x + u, y + v, z + e))
    pips_on(4, lambda u, v: (x + u, y + v, z - e))
    pips_on(2, lambda u, v: (x + e, y + v, z + u))
    pips_on(6, lambda u, v: (x - e, y + v, z + u))


def _chip_stack(B, C, x, y, z, n, mat):
    """penthouse.ts:368-378."""
    h = n * 0.0045
    r = 0.022
    B.add(cylinder((x, y + h / 2, z), r, h / 2), chip_stack(x, y, z, r, mat))


def _coffee_table(B, C, cx, cz, R):
    """penthouse.ts:380-418."""
    FLOOR, VS = C.FLOOR, C.VS
    y0 = FLOOR + 2 * VS
    top = FLOOR + 0.44
    hx, hz = 0.8, 0.45
    for sx in (-1, 1):
        for sz in (-1, 1):
            B.add(box((cx + sx * (hx - 0.03), (y0 + top) / 2, cz + sz * (hz - 0.03)), (0.02, (top - y0) / 2, 0.02)), vox(M.gold))
    B.add(subtract(box((cx, top - 0.035, cz), (hx, 0.015, hz)), box((cx, top - 0.035, cz), (hx - 0.04, 0.02, hz - 0.04))), vox(M.gold))
    B.add(box((cx, top - 0.01, cz), (hx - 0.01, 0.012, hz - 0.01)), vox(M.glassTable))
    B.add(box((cx, y0 + 0.13, cz), (hx - 0.04, 0.015, hz - 0.04)), vox(M.marbleBlack))
    ty = top + 0.002
    bx, bz = cx - 0.42, cz - 0.05
    B.add(lathe((bx, ty, bz), (0, VS, 0.085, VS, 0.105, 0.2, 0.112, 0.21), 1.6 * VS), vox(M.chrome))
    for _ in range(22):
        a = R() * PI * 2
        r = R() * 0.06
        px = bx + math.cos(a) * r
        py = ty + 0.03 + R() * 0.13
        B.add(roundBox((px, py, bz + math.sin(a) * r), (0.018, 0.016, 0.018), 0.005), vox(M.ice))
    bc = (bx, ty + 0.03, bz)
    r, t = 0.04, 1.5 * VS
    B.add(rotateZ(lathe(bc, (0, t / 2, r, t / 2, r, 0.2, 0.02, 0.27, 0.016, 0.33), t), -0.32, bc), vox(M.glassGreen))
    B.add(rotateZ(cylinder((bx, ty + 0.03 + 0.1, bz), r - t, 0.08), -0.32, bc), vox(M.champagne))
    B.add(rotateZ(lathe(bc, (0.022, 0.26, 0.018, 0.3, 0.018, 0.34), 1.2 * VS), -0.32, bc), vox(M.gold))
    _coupe(B, C, cx - 0.12, ty, cz + 0.18, True)
    _coupe(B, C, cx + 0.02, ty, cz + 0.24, True)
    _dice(B, C, (cx + 0.25, ty + 0.06, cz - 0.12), 0.12, 0.3)
    _dice(B, C, (cx + 0.43, ty + 0.06, cz + 0.02), 0.12, -0.6)
    _chip_stack(B, C, cx + 0.55, ty, cz + 0.28, 12, M.chipBlack)
    _chip_stack(B, C, cx + 0.6, ty, cz + 0.22, 8, M.chipPurple)
    _chip_stack(B, C, cx + 0.5, ty, cz + 0.2, 15, M.chipRed)
    B.add(lathe((cx + 0.15, ty, cz + 0.22), (0, VS, 0.05, VS, 0.1, 0.06, 0.11, 0.075), 1.5 * VS), vox(M.crystal))
    for _ in range(7):
        a = R() * PI * 2
        rr = R() * 0.05
        px = cx + 0.15 + math.cos(a) * rr
        py = ty + 0.05 + R() * 0.02
        shp = sphere((px, py, cz + 0.22 + math.sin(a) * rr), 0.025)
        B.add(shp, vox(M.porcelainRed if R() < 0.5 else M.gold))


def _chandelier(B, C, cx, cz, R):
    """penthouse.ts:420-471."""
    CEIL, VS = C.CEIL, C.VS
    top = CEIL + 0.15
    bodyY = 3.05
    gold = vox(M.gold)
    B.add(lathe((cx, top, cz), (0.14, 0, 0.1, -0.06, 0.02, -0.09), 0), gold)
    B.add(cylinder((cx, (top + bodyY + 0.3) / 2, cz), 0.012, (top - bodyY - 0.3) / 2), gold)
    y = bodyY + 0.4
    while y < top - 0.1:
        B.add(torus((cx, y, cz), 0.022, 0.007), gold)
        y += 0.12
    B.add(lathe((cx, bodyY, cz), (0, -0.12, 0.06, -0.1, 0.1, 0.0, 0.07, 0.12, 0.04, 0.25, 0.02, 0.32), 0), gold)
    B.add(sphere((cx, bodyY - 0.17, cz), 0.075), vox(M.crystal))
    rings = (dict(r=0.72, y=bodyY - 0.02, drops=40, arms=12), dict(r=0.46, y=bodyY + 0.2, drops=24, arms=8))
    anchors = []
    for ring in rings:
        B.add(torus((cx, ring["y"], cz), ring["r"], 0.016), gold)
        for i in range(ring["arms"]):
            a = (i / ring["arms"]) * PI * 2
            ex, ez = cx + math.cos(a) * ring["r"], cz + math.sin(a) * ring["r"]
            B.add(capsule((cx + math.cos(a) * 0.06, ring["y"] + 0.06, cz + math.sin(a) * 0.06), (ex, ring["y"], ez), 0.009), gold)
            B.add(cylinder((ex, ring["y"] + 0.035, ez), 0.022, 0.025), gold)
            B.add(ellipsoid((ex, ring["y"] + 0.09, ez), (0.018, 0.035, 0.018)), vox(M.bulb))
            anchors.append((ex, ring["y"] + 0.09, ez))
        for i in range(ring["drops"]):
            a = ((i + 0.5) / ring["drops"]) * PI * 2
            ex, ez = cx + math.cos(a) * ring["r"], cz + math.sin(a) * ring["r"]
            ln = 0.05 + R() * 0.08
            B.add(capsule((ex, ring["y"] - 0.01, ez), (ex, ring["y"] - ln, ez), VS * 0.55), vox(M.crystal))
            B.add(ellipsoid((ex, ring["y"] - ln - 0.03, ez), (0.016, 0.035, 0.016)), vox(M.crystal))
    for i in range(16):
        a = (i / 16) * PI * 2
        prev = None
        for k in range(7):
            f = k / 6
            r = rings[1]["r"] + (rings[0]["r"] - rings[1]["r"]) * f
            yy = rings[1]["y"] + (rings[0]["y"] - rings[1]["y"]) * f - math.sin(f * PI) * 0.08
            p = (cx + math.cos(a) * r, yy, cz + math.sin(a) * r)
            B.add(sphere(p, 0.011), vox(M.crystal))
            if prev is not None:
                B.add(capsule(prev, p, VS * 0.55), vox(M.crystal))
            prev = p
    return dict(pos=(cx, bodyY - 0.34, cz), radius=11, color=(3.2, 2.2, 1.25), shadow=True, anchors=anchors)


def _floor_lamp(B, C, x, z):
    """penthouse.ts:473-484."""
    FLOOR, VS = C.FLOOR, C.VS
    y0 = FLOOR + 2 * VS
    B.add(lathe((x, y0, z), (0.18, 0, 0.18, 0.025, 0.04, 0.05, 0.02, 0.06), 0), vox(M.gold))
    B.add(cylinder((x, y0 + 0.8, z), 0.014, 0.78), vox(M.gold))
    B.add(lathe((x, y0, z), (0.23, 1.42, 0.17, 1.75), 1.6 * VS), vox(M.lampshade))
    for i in range(3):
        a = (i / 3) * PI * 2
        B.add(capsule((x, y0 + 1.6, z), (x + math.cos(a) * 0.18, y0 + 1.72, z + math.sin(a) * 0.18), 0.006), vox(M.gold))
    B.add(ellipsoid((x, y0 + 1.6, z), (0.035, 0.05, 0.035)), vox(M.bulb))
    return dict(pos=(x, y0 + 1.5, z), radius=5.5, color=(1.6, 1.1, 0.6), shadow=False, anchors=[(x, y0 + 1.6, z)])


def _bar(B, C, R):
    """penthouse.ts:489-564."""
    FLOOR, WALL, VS = C.FLOOR, C.WALL, C.VS
    z0, z1 = 2.4, 7.6
    lights = []
    B.add(boxMinMax(2.35, FLOOR, z0, 2.86, FLOOR + 1.02, z1), vox(M.walnutZ))
    B.add(boxMinMax(2.33, FLOOR, z0 - 0.02, 2.9, FLOOR + 0.12, z1 + 0.02), vox(M.marbleBlack))
    B.add(boxMinMax(2.86, FLOOR + 0.13, z0, 2.9, FLOOR + 0.94, z1), tufted(z0, FLOOR, M.leather))
    B.add(boxMinMax(2.86, FLOOR + 0.94, z0, 2.92, FLOOR + 0.97, z1), vox(M.gold))
    B.add(boxMinMax(2.86, FLOOR + 0.12, z0, 2.92, FLOOR + 0.14, z1), vox(M.gold))
    B.add(boxMinMax(2.22, FLOOR + 1.02, z0 - 0.08, 3.0, FLOOR + 1.08, z1 + 0.08), vox(M.marbleBlack))
    B.add(capsule((2.97, FLOOR + 1.008, z0), (2.97, FLOOR + 1.008, z1), 0.008), vox(M.neonPink))
    B.add(capsule((3.06, FLOOR + 0.2, z0 + 0.05), (3.06, FLOOR + 0.2, z1 - 0.05), 0.022), vox(M.gold))
    z = z0 + 0.3
    while z < z1:
        B.add(capsule((2.9, FLOOR + 0.2, z), (3.06, FLOOR + 0.2, z), 0.015), vox(M.gold))
        z += 1.2
    lights.append(dict(pos=(3.25, FLOOR + 0.75, 3.5), radius=1.8, color=(1.6, 0.25, 0.9), shadow=False, anchors=[(2.97, FLOOR + 1.008, 3.5)]))
    lights.append(dict(pos=(3.25, FLOOR + 0.75, 6.4), radius=1.8, color=(1.6, 0.25, 0.9), shadow=False, anchors=[(2.97, FLOOR + 1.008, 6.4)]))
    B.add(boxMinMax(WALL, FLOOR, z0, 0.72, FLOOR + 0.9, z1), vox(M.walnutZ))
    B.add(boxMinMax(WALL, FLOOR + 0.9, z0 - 0.02, 0.76, FLOOR + 0.94, z1 + 0.02), vox(M.marbleBlack))
    B.add(boxMinMax(WALL, FLOOR + 0.94, z0 + 0.05, WALL + 0.02, FLOOR + 2.65, z1 - 0.05), vox(M.mirror))
    B.add(boxMinMax(WALL, FLOOR + 2.65, z0 + 0.03, WALL + 0.04, FLOOR + 2.69, z1 - 0.03), vox(M.gold))
    shelves = (FLOOR + 1.36, FLOOR + 1.8, FLOOR + 2.24)
    for sy in shelves:
        B.add(boxMinMax(WALL + 0.02, sy - 2 * VS, z0 + 0.1, 0.62, sy, z1 - 0.1), vox(M.glassTable))
        z = z0 + 0.3
        while z < z1 - 0.1:
            B.add(capsule((WALL + 0.01, sy - 2.5 * VS, z), (0.58, sy - 2.5 * VS, z), VS * 0.8), vox(M.gold))
            z += 1.15
        B.add(capsule((WALL + 0.035, sy + VS, z0 + 0.12), (WALL + 0.035, sy + VS, z1 - 0.12), VS * 0.7), vox(M.neonCyan))
    lights.append(dict(pos=(0.75, FLOOR + 1.85, 3.6), radius=2.6, color=(0.2, 1.1, 1.3), shadow=False, anchors=[(WALL + 0.035, shelves[1] + VS, 3.6)]))
    lights.append(dict(pos=(0.75, FLOOR + 1.85, 6.4), radius=2.6, color=(0.2, 1.1, 1.3), shadow=False, anchors=[(WALL + 0.035, shelves[1] + VS, 6.4)]))
    for sy in (FLOOR + 0.94, *shelves):
        z = z0 + 0.18
        while z < z1 - 0.15:
            bx = 0.45 + (R() - 0.5) * 0.08
            _bottle(B, C, bx, sy, z, R)
            z += 0.1 + R() * 0.06
    for i in range(6):
        z = z0 + 0.4 + i * 0.85 + R() * 0.2
        if i % 2 == 0:
            _coupe(B, C, 2.62, FLOOR + 1.08, z, True)
        else:
            _bottle(B, C, 2.55, FLOOR + 1.08, z, R)
    for z in (3.1, 5.15, 6.9):
        B.add(lathe((2.7, FLOOR + 1.08, z), (0, VS, 0.035, VS, 0.037, 0.085), 1.4 * VS), vox(M.glassClear))
        B.add(cylinder((2.7, FLOOR + 1.08 + 0.03, z), 0.03, 0.02), vox(M.whiskey))
        B.add(roundBox((2.7, FLOOR + 1.08 + 0.05, z), (0.015, 0.015, 0.015), 0.004), vox(M.ice))
    B.add(lathe((2.5, FLOOR + 1.08, 4.0), (0, 0, 0.04, 0, 0.045, 0.14, 0.035, 0.18, 0.02, 0.22, 0.02, 0.24), 0), vox(M.chrome))
    for z in (3.25, 4.45, 5.65, 6.85):
        x = 3.5
        B.add(lathe((x, FLOOR, z), (0.2, 0, 0.2, 0.02, 0.05, 0.04, 0.03, 0.05), 0), vox(M.chrome))
        B.add(cylinder((x, FLOOR + 0.4, z), 0.024, 0.36), vox(M.chrome))
        B.add(torus((x, FLOOR + 0.32, z), 0.17, 0.012), vox(M.chrome))
        for i in range(4):
            a = (i / 4) * PI * 2 + 0.4
            B.add(capsule((x, FLOOR + 0.32, z), (x + math.cos(a) * 0.17, FLOOR + 0.32, z + math.sin(a) * 0.17), 0.009), vox(M.chrome))
        B.add(cylinder((x, FLOOR + 0.77, z), 0.075, 0.015), vox(M.chrome))
        _upholstered(B, roundBox((x, FLOOR + 0.82, z), (0.2, 0.045, 0.2), 0.04), M.leather, 0.025)
        B.add(torus((x, FLOOR + 0.8, z), 0.19, 0.012), vox(M.gold))
    return lights


def _poker_table(B, C, cx, cz, R):
    """penthouse.ts:569-620."""
    FLOOR, CEIL, VS = C.FLOOR, C.CEIL, C.VS
    hl, rr = 0.62, 0.68
    top = FLOOR + 0.76
    for sx in (-1, 1):
        B.add(lathe((cx + sx * 0.55, FLOOR, cz), (0.42, 0, 0.42, 0.04, 0.16, 0.1, 0.12, 0.2, 0.12, 0.6), 0), vox(M.walnutY))
    B.add(stadium((cx, 0, cz), hl, rr - 0.04, top - 0.16, top - 0.02), vox(M.walnut))
    B.add(stadium((cx, 0, cz), hl, rr - 0.17, top - 0.04, top), vox(M.felt))
    B.add(subtract(stadium((cx, 0, cz), hl, rr, top - 0.04, top + 0.06), stadium((cx, 0, cz), hl, rr - 0.17, top - 0.1, top + 0.1)), vox(M.leather))
    B.add(subtract(stadium((cx, 0, cz), hl, rr - 0.165, top - 0.01, top + 0.012), stadium((cx, 0, cz), hl, rr - 0.18, top - 0.1, top + 0.1)), vox(M.gold))
    B.add(box((cx, top + 0.012, cz - rr + 0.27), (0.25, 0.012, 0.06)), vox(M.chrome))
    chip_mats = (M.chipRed, M.chipBlue, M.chipGreen, M.chipBlack, M.chipPurple)
    for i in range(10):
        n = 3 + math.floor(R() * 4)
        _chip_stack(B, C, cx - 0.2 + i * 0.045, top + 0.006, cz - rr + 0.27, n, chip_mats[i % 5])
    seats = []
    for sx in (-1, 0, 1):
        seats.append((cx + sx * 0.6, cz + rr + 0.38, PI))
    seats.append((cx - hl - rr - 0.38, cz, -PI / 2))
    seats.append((cx + hl + rr + 0.38, cz, PI / 2))
    for sxp, szp, syaw in seats:
        dx, dz = cx - sxp, cz - szp
        dl = js_hypot(dx, dz)
        px, pz = sxp + (dx / dl) * 0.62, szp + (dz / dl) * 0.62
        for c in range(2):
            ang = syaw + c * 0.25
            crd = rotateY(box((px + c * 0.03, top + VS * 0.5, pz), (0.032, VS * 0.5, 0.045)), ang, (px, top, pz))
            B.add(crd, local_paint(card(px, pz, c * 0.03, M.card), ang, (px, top, pz)))
        for k in range(3):
            a = math.atan2(dz, dx) + PI / 2
            n = 4 + math.floor(R() * 10)
            mat = chip_mats[math.floor(R() * 5)]
            _chip_stack(B, C, px + math.cos(a) * (0.12 + k * 0.05), top, pz + math.sin(a) * (0.12 + k * 0.05), n, mat)
        _chair(B, C, sxp, szp, syaw)
    ly = 2.15
    B.add(cylinder((cx, (ly + CEIL) / 2 + 0.1, cz), 0.006, (CEIL - ly) / 2 - 0.08), vox(M.steelDark))
    B.add(subtract(stadium((cx, 0, cz), 0.5, 0.2, ly, ly + 0.16), stadium((cx, 0, cz), 0.5, 0.2 - 1.6 * VS, ly - 0.01, ly + 0.16 - 1.6 * VS)), vox(M.glassGreen))
    B.add(stadium((cx, 0, cz), 0.5, 0.21, ly + 0.14, ly + 0.18), vox(M.gold))
    anchors = []
    for sx in (-0.4, 0, 0.4):
        B.add(sphere((cx + sx, ly + 0.08, cz), 0.035), vox(M.bulb))
        anchors.append((cx + sx, ly + 0.08, cz))
    return [dict(pos=(cx, ly - 0.02, cz), radius=6, color=(2.2, 1.9, 1.3), shadow=True, anchors=anchors)]


def _chair(B, C, x, z, yaw):
    """penthouse.ts:622-632."""
    FLOOR = C.FLOOR
    c = (x, 0, z)

    def rot(s):
        return rotateY(s, yaw, c)

    for sx, sz in ((-1, -1), (1, -1), (-1, 1), (1, 1)):
        B.add(rot(cylinder((x + sx * 0.19, FLOOR + 0.22, z + sz * 0.19), 0.018, 0.22)), vox(M.gold))
    _upholstered(B, rot(roundBox((x, FLOOR + 0.48, z), (0.24, 0.05, 0.24), 0.04)), M.velvetRed, 0.025)
    _upholstered(B, rot(roundBox((x, FLOOR + 0.8, z - 0.21), (0.23, 0.3, 0.04), 0.035)), M.velvetRed, 0.02)
    B.add(rot(torus((x, FLOOR + 1.1, z - 0.21), 0.2, 0.012, "z")), vox(M.gold))


def _slot_machine(B, C, x, zBack, i, R):
    """penthouse.ts:634-667."""
    FLOOR, VS = C.FLOOR, C.VS
    z0, z1 = zBack + 0.02, zBack + 0.62
    zc = (z0 + z1) / 2
    w = 0.32
    cab = vox(M.slotRed, 1 + ((i * 37) % 60))
    B.add(roundBox((x, FLOOR + 0.66, zc), (w, 0.66, (z1 - z0) / 2), 0.03), cab)
    B.add(cylinder((x, FLOOR + 1.32, zc), w, (z1 - z0) / 2 - 0.02, "z"), cab)
    B.add(boxMinMax(x - w - 0.01, FLOOR, z0, x + w + 0.01, FLOOR + 0.1, z1 + 0.01), vox(M.chrome))
    B.carve(boxMinMax(x - 0.24, FLOOR + 0.78, z1 - 0.05, x + 0.24, FLOOR + 1.16, z1 + 0.01))
    B.add(boxMinMax(x - 0.24, FLOOR + 0.78, z1 - 0.05, x + 0.24, FLOOR + 1.16, z1 - 0.05 + 2 * VS), vox(M.screen))
    B.add(subtract(boxMinMax(x - 0.27, FLOOR + 0.75, z1 - 0.01, x + 0.27, FLOOR + 1.19, z1 + 0.02),
                   boxMinMax(x - 0.24, FLOOR + 0.78, z1 - 0.05, x + 0.24, FLOOR + 1.16, z1 + 0.05)), vox(M.chrome))
    deck = rotateX(box((x, FLOOR + 0.66, z1 + 0.06), (w - 0.02, 0.025, 0.08)), -0.25, (x, FLOOR + 0.66, z1))
    B.add(deck, vox(M.chrome))
    for b in range(4):
        B.add(cylinder((x - 0.18 + b * 0.12, FLOOR + 0.7, z1 + 0.07), 0.022, 0.012), vox(M.neonCyan if b % 2 else M.neonPink))
    B.add(subtract(box((x, FLOOR + 0.26, z1 + 0.04), (0.2, 0.04, 0.05)), box((x, FLOOR + 0.29, z1 + 0.04), (0.18, 0.04, 0.04))), vox(M.chrome))
    _neon_text(B, C, "777", (x, FLOOR + 1.33, z1 - 0.01), 0.13, "south", M.neonGold, 0.008)
    B.add(torus((x, FLOOR + 1.32, z1 - 0.03), w - 0.02, 0.012, "z"), vox(M.neonPink))
    B.add(box((x + w + 0.03, FLOOR + 0.9, zc + 0.1), (0.03, 0.06, 0.06)), vox(M.chrome))
    B.add(capsule((x + w + 0.07, FLOOR + 0.9, zc + 0.1), (x + w + 0.07, FLOOR + 1.3, zc + 0.12), 0.012), vox(M.chrome))
    B.add(sphere((x + w + 0.07, FLOOR + 1.33, zc + 0.12), 0.035), vox(M.glassRed))
    sz = z1 + 0.42
    B.add(lathe((x, FLOOR, sz), (0.17, 0, 0.17, 0.02, 0.03, 0.04), 0), vox(M.chrome))
    B.add(cylinder((x, FLOOR + 0.33, sz), 0.022, 0.3), vox(M.chrome))
    _upholstered(B, cylinder((x, FLOOR + 0.66, sz), 0.18, 0.045), M.leather, 0.025)
    hue = R()
    color = (1.5, 0.3, 0.8) if hue < 0.33 else (0.3, 1.0, 1.5) if hue < 0.66 else (1.6, 1.0, 0.2)
    return dict(pos=(x, FLOOR + 1.0, z1 + 0.4), radius=2.0, color=color, shadow=False, anchors=[(x, FLOOR + 0.97, z1 - 0.05 + VS)])


def _neon_text(B, C, text, at, height, facing, mat, tube=0.016):
    """penthouse.ts:675-695."""
    VS = C.VS
    strokes, width = layout_text(text)
    s = height / 6
    ax, ay, az = at

    def mp(u, v):
        if facing == "south":
            return (ax + (u - width / 2) * s, ay + (v - 3) * s, az)
        return (ax, ay + (v - 3) * s, az - (u - width / 2) * s)

    pts = []
    for sa, sb in strokes:
        a = mp(*sa)
        b = mp(*sb)
        B.add(capsule(a, b, tube), vox(mat))
        pts.append(a)
    for i in range(0, len(pts), 3):
        p = pts[i]
        back = (p[0], p[1], p[2] - 0.05) if facing == "south" else (p[0] - 0.05, p[1], p[2])
        B.add(capsule(p, back, VS * 0.6), vox(M.steelDark))
    return pts


def _neon_signs(B, C):
    """penthouse.ts:697-717."""
    WALL = C.WALL
    lights = []
    vy, vz = 2.95, WALL + 0.06
    p = _neon_text(B, C, "VEGAS", (9.6, vy, vz), 0.62, "south", M.neonPink, 0.02)
    _neon_text(B, C, "*", (7.85, vy, vz), 0.5, "south", M.neonGold, 0.016)
    _neon_text(B, C, "*", (11.35, vy, vz), 0.5, "south", M.neonGold, 0.016)
    B.add(boxMinMax(7.5, vy - 0.48, WALL, 11.7, vy - 0.45, WALL + 0.03), vox(M.neonCyan))
    lights.append(dict(pos=(8.8, vy, 0.8), radius=3.6, color=(2.2, 0.35, 1.2), shadow=False, anchors=[p[0]]))
    lights.append(dict(pos=(10.4, vy, 0.8), radius=3.6, color=(2.2, 0.35, 1.2), shadow=False, anchors=[p[-1]]))
    b = _neon_text(B, C, "BAR", (WALL + 0.06, 3.2, 5.0), 0.5, "west", M.neonCyan, 0.018)
    lights.append(dict(pos=(0.9, 3.2, 5.0), radius=3.0, color=(0.3, 1.6, 2.0), shadow=False, anchors=[b[0]]))
    mx, my, mz = WALL + 0.06, 3.2, 6.6
    ms = ((-0.18, 0.2, 0, 0), (0.18, 0.2, 0, 0), (-0.18, 0.2, 0.18, 0.2), (0, 0, 0, -0.22), (-0.1, -0.22, 0.1, -0.22))
    for u0, v0, u1, v1 in ms:
        B.add(capsule((mx, my + v0, mz - u0), (mx, my + v1, mz - u1), 0.014), vox(M.neonPink))
    B.add(sphere((mx, my + 0.12, mz - 0.05), 0.03), vox(M.absinthe))
    B.add(capsule((mx, my + 0.08, mz), (mx, my + 0.24, mz - 0.12), 0.006), vox(M.neonGold))
    return lights


def _piano(B, C, cx, cz, yaw):
    """penthouse.ts:721-772."""
    FLOOR, VS = C.FLOOR, C.VS
    c = (cx, 0, cz)

    def rot(s):
        return rotateY(s, yaw, c)

    outline = (-0.75, 0, 0.75, 0, 0.75, 0.5, 0.68, 0.75, 0.5, 0.95, 0.25, 1.15, 0.1, 1.35, 0.0, 1.6, -0.15, 1.8, -0.35, 1.92, -0.6, 1.95, -0.75, 1.9)
    inner = (-0.71, 0.04, 0.71, 0.04, 0.71, 0.5, 0.64, 0.73, 0.47, 0.92, 0.22, 1.12, 0.06, 1.33, -0.04, 1.58, -0.18, 1.76, -0.36, 1.87, -0.6, 1.9, -0.71, 1.86)
    zOff = -0.9

    def at(pts):
        return [v + zOff if i % 2 else v for i, v in enumerate(pts)]

    y0, y1 = FLOOR + 0.62, FLOOR + 0.95
    B.add(rot(subtract(prism(c, at(outline), y0, y1), prism(c, at(inner), y0 + 0.14, y1 + 0.01))), vox(M.lacquer))
    B.add(rot(prism(c, at(inner), y0 + 0.14, y0 + 0.17)), vox(M.gold))
    for i in range(-6, 7):
        x = cx + i * 0.09
        B.add(rot(capsule((x, y0 + 0.18, cz + zOff + 0.1), (x - 0.04, y0 + 0.18, cz + zOff + 1.55 - abs(i) * 0.06), VS * 0.45)), vox(M.chrome))
    hinge = (cx - 0.75, y1 + 0.01, cz)
    B.add(rot(rotateZ(prism(c, at(outline), y1, y1 + 0.022), 0.62, hinge)), vox(M.lacquer))
    lx, ly = cx - 0.75 + 1.15 * math.cos(0.62), y1 + 1.15 * math.sin(0.62)
    B.add(rot(capsule((cx + 0.35, y1 - 0.02, cz + zOff + 0.9), (lx - 0.02, ly - 0.03, cz + zOff + 0.9), 0.012)), vox(M.lacquer))
    kz0 = cz + zOff - 0.24
    B.add(rot(boxMinMax(cx - 0.75, y0 - 0.04, kz0, cx + 0.75, y0 + 0.07, cz + zOff + 0.02)), vox(M.lacquer))
    B.add(rot(boxMinMax(cx - 0.66, y0 + 0.07, kz0 + 0.02, cx + 0.66, y0 + 0.09, cz + zOff - 0.02)),
          local_paint(white_keys(cx - 0.66, M.ivory), yaw, c))
    B.add(rot(boxMinMax(cx - 0.66, y0 + 0.09, kz0 + 0.1, cx + 0.66, y0 + 0.105, cz + zOff - 0.02)),
          local_paint(black_keys(cx - 0.66, M.lacquer), yaw, c))
    B.add(rot(boxMinMax(cx - 0.75, y0 + 0.07, cz + zOff - 0.02, cx + 0.75, y0 + 0.2, cz + zOff + 0.03)), vox(M.lacquer))
    B.add(rot(box((cx, y0 + 0.24, cz + zOff + 0.06), (0.25, 0.1, 0.01))), vox(M.lacquer))
    for lx2, lz in ((-0.62, 0.15), (0.62, 0.15), (-0.45, 1.72)):
        B.add(rot(cylinder((cx + lx2, FLOOR + 0.33, cz + zOff + lz), 0.05, 0.3)), vox(M.lacquer))
        B.add(rot(sphere((cx + lx2, FLOOR + 0.03, cz + zOff + lz), 0.032)), vox(M.gold))
    B.add(rot(box((cx, FLOOR + 0.3, cz + zOff + 0.25), (0.08, 0.3, 0.03))), vox(M.lacquer))
    for px in (-0.05, 0, 0.05):
        B.add(rot(box((cx + px, FLOOR + 0.06, cz + zOff + 0.18), (0.012, 0.008, 0.05))), vox(M.gold))
    bz = cz + zOff - 0.62
    for sx, sz in ((-1, -1), (1, -1), (-1, 1), (1, 1)):
        B.add(rot(cylinder((cx + sx * 0.32, FLOOR + 0.24, bz + sz * 0.12), 0.02, 0.24)), vox(M.lacquer))
    B.add(rot(box((cx, FLOOR + 0.5, bz), (0.38, 0.03, 0.17))), vox(M.lacquer))
    _upholstered(B, rot(roundBox((cx, FLOOR + 0.55, bz), (0.36, 0.035, 0.15), 0.025)), M.leather, 0.02)


def _champagne_tower(B, C, cx, cz):
    """penthouse.ts:774-792."""
    FLOOR, VS = C.FLOOR, C.VS
    y0 = FLOOR + 2 * VS
    B.add(lathe((cx, y0, cz), (0.32, 0, 0.32, 0.03, 0.09, 0.07, 0.07, 0.66, 0.42, 0.7, 0.42, 0.75), 0), vox(M.marble))
    B.add(torus((cx, y0 + 0.725, cz), 0.42, 0.012), vox(M.gold))
    top = y0 + 0.75
    sp = 0.112
    levels = 5
    for L in range(levels):
        n = levels - L
        y = top + L * 0.125 - L * VS * 0.5
        for i in range(n):
            for j in range(n):
                x = cx + (i - (n - 1) / 2) * sp
                z = cz + (j - (n - 1) / 2) * sp
                _coupe(B, C, x, y, z, True)
    _bottle(B, C, cx + 0.33, top, cz - 0.2, mulberry32(5), 3)


def _tv(B, C):
    """penthouse.ts:794-804."""
    FLOOR, WALL, VS = C.FLOOR, C.WALL, C.VS
    z0, z1, y0, y1 = 8.55, 11.05, FLOOR + 1.15, FLOOR + 2.55
    B.add(boxMinMax(WALL, FLOOR, z0 - 0.15, 0.7, FLOOR + 0.48, z1 + 0.15), vox(M.walnutZ))
    B.add(boxMinMax(WALL, FLOOR + 0.48, z0 - 0.17, 0.73, FLOOR + 0.52, z1 + 0.17), vox(M.marbleBlack))
    B.add(boxMinMax(WALL, y0, z0, WALL + 0.06, y1, z1), vox(M.plasticBlack))
    B.add(boxMinMax(WALL + 0.06, y0 + 0.03, z0 + 0.03, WALL + 0.06 + VS, y1 - 0.03, z1 - 0.03), vox(M.tv))
    _vase(B, C, 0.48, FLOOR + 0.52, z0 + 0.1, 0.6, M.porcelain)
    _vase(B, C, 0.48, FLOOR + 0.52, z1 - 0.1, 0.6, M.porcelainRed)
    return dict(pos=(1.2, (y0 + y1) / 2, (z0 + z1) / 2), radius=4.2, color=(0.5, 0.45, 1.6), shadow=False,
                anchors=[(WALL + 0.06 + VS * 0.5, (y0 + y1) / 2, (z0 + z1) / 2)])


def _vase(B, C, x, y, z, scale, mat):
    """penthouse.ts:806-817."""
    VS = C.VS
    s = scale
    prof = [v * s for v in (0, 0, 0.07, 0, 0.12, 0.05, 0.16, 0.17, 0.14, 0.3, 0.07, 0.4, 0.055, 0.46, 0.075, 0.5)]
    for i in range(1, len(prof), 2):
        prof[i] += VS * 0.4
    B.add(lathe((x, y, z), prof, 1.7 * VS), vase_paint(x, y, z, s, mat))


def _decor(B, C, R):
    """penthouse.ts:819-846."""
    FLOOR, WALL, VS = C.FLOOR, C.WALL, C.VS
    pz = 0.62

    def trophy(x, y):
        B.add(lathe((x, y, pz), (0.09, 0, 0.09, 0.03, 0.03, 0.06, 0.02, 0.14, 0.05, 0.16, 0.14, 0.24, 0.16, 0.4), 2 * VS), vox(M.gold))
        B.add(torus((x - 0.17, y + 0.3, pz), 0.06, 0.012, "z"), vox(M.gold))
        B.add(torus((x + 0.17, y + 0.3, pz), 0.06, 0.012, "z"), vox(M.gold))

    items = (
        (4.4, lambda x, y: _vase(B, C, x, y, pz, 1.0, M.porcelain)),
        (5.8, lambda x, y: _vase(B, C, x, y, pz, 1.15, M.porcelainRed)),
        (7.0, trophy),
    )
    for x, place in items:
        B.add(box((x, FLOOR + 0.5, pz), (0.2, 0.5, 0.2)), vox(M.marbleBlack))
        B.add(box((x, FLOOR + 1.01, pz), (0.23, 0.02, 0.23)), vox(M.gold))
        place(x, FLOOR + 1.03)
    ax0, ax1, ay0, ay1 = 3.9, 7.5, 1.75, 3.25
    B.add(boxMinMax(ax0 - 0.08, ay0 - 0.08, WALL, ax1 + 0.08, ay1 + 0.08, WALL + 0.05), vox(M.gold))
    blobs = []
    for _ in range(9):
        bx = ax0 + R() * (ax1 - ax0)
        by = ay0 + R() * (ay1 - ay0)
        br = 0.15 + R() * 0.4
        bs = 1 + math.floor(R() * 254)
        blobs.append(dict(x=bx, y=by, r=br, s=bs))
    B.add(boxMinMax(ax0, ay0, WALL, ax1, ay1, WALL + 0.06), painting(blobs, M.paperArt))


def _palm(B, C, x, z, R):
    """penthouse.ts:848-881."""
    FLOOR, VS = C.FLOOR, C.VS
    y0 = FLOOR
    B.add(lathe((x, y0, z), (0, 0, 0.16, 0, 0.21, 0.42, 0.23, 0.46), 2 * VS), vox(M.terracotta))
    B.add(cylinder((x, y0 + 0.38, z), 0.19, 0.04), vox(M.soil))
    px, py, pz = x, y0 + 0.4, z
    lean = R() * PI * 2
    for i in range(8):
        nx, ny, nz = px + math.cos(lean) * 0.025, py + 0.17, pz + math.sin(lean) * 0.025
        B.add(capsule((px, py, pz), (nx, ny, nz), 0.045 - i * 0.002), vox(M.trunk))
        B.add(torus((nx, ny - 0.02, nz), 0.04 - i * 0.002, 0.008), vox(M.trunk, 200))
        px, py, pz = nx, ny, nz
    n = 9
    for i in range(n):
        a = (i / n) * PI * 2 + R() * 0.3
        lift = 0.5 + R() * 0.5
        fx, fy, fz = px, py, pz
        for k in range(1, 10):
            t = k / 9
            dist = t * 0.85
            nx = px + math.cos(a) * dist
            nz = pz + math.sin(a) * dist
            ny = py + math.sin(t * PI * 0.9) * 0.28 * lift - t * t * 0.45
            w = 0.07 * math.sin(t * PI) + 0.015
            seg = capsule((fx, fy, fz), (nx, ny, nz), 0.012)
            B.add(seg, vox(M.leaf, 1))
            c = ((fx + nx) / 2, (fy + ny) / 2, (fz + nz) / 2)
            B.add(rotateY(ellipsoid(c, (0.05, 0.012, w)), a, c), vox(M.leaf))
            fx, fy, fz = nx, ny, nz
