"""World constants: voxel density, brick size and world dimensions.

Restates ``src/config.ts:10-30`` of the reference.  The reference reads ``vpm``
from the page URL once at import (``config.ts:3-12``), so a process can only
ever hold one voxel density.  Here the density is a value the caller sets
(``set_vpm``) before building shapes, because the shape constructors clamp
radii against the voxel size (``shapes.ts:110-112``) exactly like the
reference does at construction time.
"""
from __future__ import annotations

import math

BRICK = 8                      # config.ts:16
BRICK_VOXELS = BRICK * BRICK * BRICK   # config.ts:17
WORLD_METERS = (16.0, 4.4, 12.0)       # config.ts:20
VPM_MIN, VPM_MAX, VPM_DEFAULT = 16.0, 160.0, 80.0   # config.ts:12


def clamp_vpm(v) -> float:
    """``num('vpm', 80, 16, 160)`` of config.ts:5-8: non-finite -> default, else clamp."""
    try:
        v = float(v)
    except (TypeError, ValueError):
        return VPM_DEFAULT
    if not math.isfinite(v):
        return VPM_DEFAULT
    return min(VPM_MAX, max(VPM_MIN, v))


def round_to_brick(m: float, vpm: float) -> int:
    """``Math.ceil((m * VOXELS_PER_METER) / BRICK) * BRICK`` (config.ts:22-24)."""
    return int(math.ceil((m * vpm) / BRICK) * BRICK)


class Config:
    """One voxel density and everything derived from it."""

    def __init__(self, vpm: float = VPM_DEFAULT):
        self.vpm = float(vpm)
        self.voxel_size = 1 / self.vpm                       # config.ts:13
        self.dims = tuple(round_to_brick(m, self.vpm) for m in WORLD_METERS)  # config.ts:26-30
        # shapes.ts:110-112: minimum radii that keep thin features 6-connected.
        self.min_line_r = 0.9 * self.voxel_size
        self.min_column_r = 0.6 * self.voxel_size
        self.min_shell = 1.75 * self.voxel_size

    @property
    def bricks(self):
        return tuple(d // BRICK for d in self.dims)

    @property
    def cells(self) -> int:
        dx, dy, dz = self.dims
        return dx * dy * dz

    def __repr__(self):
        return f"Config(vpm={self.vpm:g}, dims={self.dims})"


_current = Config(VPM_DEFAULT)


def current() -> Config:
    return _current


def set_vpm(vpm: float) -> Config:
    """Make ``vpm`` the density that shape constructors and ``apply`` use."""
    global _current
    _current = Config(vpm)
    return _current


class using:
    """``with using(20): ...`` builds shapes at another density, then restores."""

    def __init__(self, vpm: float):
        self.vpm = vpm

    def __enter__(self):
        global _current
        self.prev = _current
        _current = Config(self.vpm)
        return _current

    def __exit__(self, *exc):
        global _current
        _current = self.prev
        return False
