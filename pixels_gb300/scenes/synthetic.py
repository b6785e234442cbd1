"""Seeded synthetic scenes (not in the reference, whose only scene is the
penthouse): many primitives of every kind the reference's shape library has,
with CSG, rotations and a procedural paint, written through the same Builder
API so the GPU build and the oracle see ordinary op lists.

``synthetic_program(seed, n_prims=4096, vpm=80)`` follows the distributions of
the benchmark's synthetic configuration:

* a 16 x 4.4 x 12 m volume; centres uniform in it;
* primitives uniform over {box, rounded box (radius 0.1-0.4 of the smallest
  half extent), cylinder, capsule, torus, lathe with an 8-point profile,
  extruded hexagon (prism)}; sizes log-uniform 2 cm - 1.5 m;
* rotations uniform on SO(3), composed as rotateZ(rotateY(rotateZ(shape)))
  about the centre (the reference API rotates about one axis at a time);
* CSG: 30% of primitives are subtracted from the next one, 10% intersected
  with it; 10% of the remaining single primitives are carved;
* 64 materials, random shades; 25% of the ops paint with the procedural
  noise kind (integer hash + float32 sine);
* every parameter is a float32-representable double.
"""
from __future__ import annotations

import math

import numpy as np

from .. import config as _config
from ..materials import vox
from ..paints import noise
from ..shapes import (Builder, box, capsule, cylinder, intersect, lathe, prism, rotateY, rotateZ, roundBox,
                      subtract, torus)

VOLUME = (16.0, 4.4, 12.0)
KINDS = ("box", "roundbox", "cylinder", "capsule", "torus", "lathe", "prism")


def _f32(v) -> float:
    return float(np.float32(v))


def _prim(rng: np.random.Generator, volume=VOLUME):
    kind = KINDS[int(rng.integers(len(KINDS)))]
    c = tuple(_f32(rng.uniform(0, volume[i])) for i in range(3))
    size = _f32(math.exp(rng.uniform(math.log(0.02), math.log(1.5))))
    half = size / 2
    ext = tuple(_f32(half * rng.uniform(0.3, 1.0)) for _ in range(3))
    if kind == "box":
        s = box(c, ext)
    elif kind == "roundbox":
        r = _f32(min(ext) * rng.uniform(0.1, 0.4))
        s = roundBox(c, ext, r)
    elif kind == "cylinder":
        s = cylinder(c, _f32(half * rng.uniform(0.2, 0.6)), _f32(half * rng.uniform(0.3, 1.0)),
                     "xyz"[int(rng.integers(3))])
    elif kind == "capsule":
        d = rng.normal(size=3)
        d = d / max(np.linalg.norm(d), 1e-9) * half
        a = tuple(_f32(c[i] - d[i]) for i in range(3))
        b = tuple(_f32(c[i] + d[i]) for i in range(3))
        s = capsule(a, b, _f32(half * rng.uniform(0.05, 0.3)))
    elif kind == "torus":
        R = _f32(half * rng.uniform(0.5, 0.8))
        s = torus(c, R, _f32(R * rng.uniform(0.1, 0.4)), "xyz"[int(rng.integers(3))])
    elif kind == "lathe":
        ys = np.sort(rng.uniform(0, 2 * half, size=8))
        rs = rng.uniform(0.2, 1.0, size=8) * half * 0.6
        prof = []
        for r_, y_ in zip(rs, ys):
            prof.extend((_f32(r_), _f32(y_ - half)))
        shell = 0 if rng.random() < 0.7 else _f32(half * rng.uniform(0.05, 0.15))
        s = lathe(c, prof, shell)
    else:  # extruded hexagon
        pts = []
        for k in range(6):
            a = k * math.pi / 3 + rng.uniform(-0.3, 0.3)
            r_ = half * rng.uniform(0.6, 1.0)
            pts.extend((_f32(r_ * math.cos(a)), _f32(r_ * math.sin(a))))
        y0 = _f32(c[1] - ext[1])
        y1 = _f32(c[1] + ext[1])
        s = prism(c, pts, y0, y1)
    # uniform rotation on SO(3): Rz(alpha) Ry(beta) Rz(gamma), cos(beta) uniform
    alpha = _f32(rng.uniform(0, 2 * math.pi))
    beta = _f32(math.acos(rng.uniform(-1, 1)))
    gamma = _f32(rng.uniform(0, 2 * math.pi))
    s = rotateZ(rotateY(rotateZ(s, gamma, c), beta, c), alpha, c)
    return s


def _paint(rng: np.random.Generator):
    mat = 1 + int(rng.integers(64))
    v = vox(mat, int(rng.integers(256)))
    if rng.random() < 0.25:
        vb = vox(1 + int(rng.integers(64)), int(rng.integers(256)))
        return noise(int(rng.integers(1 << 31)), _f32(rng.uniform(10, 80)), _f32(rng.uniform(0.5, 4)),
                     _f32(rng.uniform(0.5, 4)), _f32(rng.uniform(0.5, 4)), _f32(rng.uniform(-0.5, 0.5)), v, vb)
    return v


def build_synthetic(world, seed: int = 1, n_prims: int = 4096, volume=VOLUME) -> int:
    """Queue a seeded synthetic scene on ``world`` (centres uniform in
    ``volume``, metres); returns the number of ops."""
    rng = np.random.default_rng(seed)
    B = Builder(world)
    ops = 0
    i = 0
    with _config.using(world.vpm):
        while i < n_prims:
            u = rng.random()
            if u < 0.3 and i + 1 < n_prims:
                s = subtract(_prim(rng, volume), _prim(rng, volume))
                i += 2
                B.add(s, _paint(rng))
            elif u < 0.4 and i + 1 < n_prims:
                s = intersect(_prim(rng, volume), _prim(rng, volume))
                i += 2
                B.add(s, _paint(rng))
            else:
                s = _prim(rng, volume)
                i += 1
                if rng.random() < 0.1:
                    B.carve(s)
                else:
                    B.add(s, _paint(rng))
            ops += 1
    return ops


def synthetic_program(seed: int = 1, n_prims: int = 4096, vpm: float = 80.0, volume=VOLUME):
    from ..world import OpRecorder
    rec = OpRecorder(vpm)
    build_synthetic(rec, seed, n_prims, volume)
    return rec.program


def dims_for(volume, vpm: float):
    """World dims (voxels) of a volume: ceil(m * vpm / 8) * 8 per axis, as config.ts sizes the world."""
    return tuple(int(math.ceil(m * vpm / 8)) * 8 for m in volume)


def batch_specs(seed: int = 7, n: int = 256):
    """The batched workload: ``n`` independent scenes of uneven size.

    Volumes log-uniform 0.5-64 m^3 with aspect ratios up to 4:1 (two axes
    1-4x the third, in random order), primitive counts log-uniform 16-2048,
    voxel density uniform over {40, 80, 160} per metre; each scene is a
    synthetic scene (same distributions as above) with its own seed.
    """
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        vol = math.exp(rng.uniform(math.log(0.5), math.log(64.0)))
        ratios = [1.0, float(rng.uniform(1.0, 4.0)), float(rng.uniform(1.0, 4.0))]
        rng.shuffle(ratios)
        k = (vol / (ratios[0] * ratios[1] * ratios[2])) ** (1.0 / 3.0)
        volume = tuple(_f32(k * r) for r in ratios)
        n_prims = int(round(math.exp(rng.uniform(math.log(16), math.log(2048)))))
        vpm = float((40, 80, 160)[int(rng.integers(3))])
        specs.append({"seed": seed * 100003 + i, "volume": volume, "n_prims": n_prims, "vpm": vpm,
                      "dims": dims_for(volume, vpm)})
    return specs
