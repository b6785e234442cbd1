"""Light records and anchors of the upload (packLights, GpuWorld.ts:141-162).

``pack_lights(world, lights)`` returns the two word arrays the renderer's
light pass reads: 16 words per light (position, radius, colour, shadow flag,
1.0 as float32; first anchor and anchor count as u32; a phase of i * 7.31 as
float32) and 8 words per anchor (snapped voxel x, y, z, 0, y, 0, 0, 0).  At
most 32 lights and 256 anchors are kept (layout.ts LIMITS).  The anchors are
snapped to emissive voxels on the GPU, all in one launch (px_snap_anchors);
``snap`` may replace that step (tests pass the oracle's).
"""
from __future__ import annotations

import math

import numpy as np

MAX_LIGHTS = 32    # layout.ts LIMITS.maxLights
MAX_ANCHORS = 256  # layout.ts LIMITS.maxAnchors


def anchor_voxels(lights, vpm: float):
    """The anchors packLights snaps, in order, as voxel coordinates
    (Math.floor(a / VOXEL_SIZE), VOXEL_SIZE = 1 / vpm), with their light index."""
    vs = 1.0 / vpm
    out, owner = [], []
    for i, light in enumerate(lights[:MAX_LIGHTS]):
        for a in light["anchors"]:
            if len(out) >= MAX_ANCHORS:
                break
            out.append([math.floor(a[0] / vs), math.floor(a[1] / vs), math.floor(a[2] / vs)])
            owner.append(i)
    return np.array(out, dtype=np.int64).reshape(-1, 3), owner


def pack_lights(world, lights, snap=None):
    """(lights u32[n * 16], anchors u32[max(8 * anchors, 1)]) for a built world."""
    xyz, owner = anchor_voxels(lights, world.vpm)
    if snap is None:
        from . import _lib
        from .materials import emission_table
        world._ensure()
        snapped = _lib.snap_anchors(world._h, xyz, np.array(emission_table(), np.uint8)) if len(xyz) else xyz
    else:
        snapped = snap(xyz)
    snapped = np.asarray(snapped, dtype=np.int64).reshape(-1, 3)
    n = min(len(lights), MAX_LIGHTS)
    words = np.zeros(n * 16, dtype=np.uint32)
    fl = words.view(np.float32)
    anchors = []
    k = 0
    for i in range(n):
        light = lights[i]
        start = len(anchors) // 8
        while k < len(owner) and owner[k] == i:
            x, y, z = (int(v) for v in snapped[k])
            anchors.extend((x, y, z, 0, y, 0, 0, 0))
            k += 1
        count = len(anchors) // 8 - start
        o = i * 16
        fl[o:o + 9] = np.array([*light["pos"], light["radius"], *light["color"], 1 if light["shadow"] else 0, 1],
                               dtype=np.float64).astype(np.float32)
        words[o + 9] = start
        words[o + 10] = count
        fl[o + 11] = np.float32(i * 7.31)
    anc = np.array(anchors if anchors else [0], dtype=np.int64).astype(np.uint32)  # Uint32Array wraps negatives
    return words, anc
