"""Material ids and the opacity flag the voxeliser needs.

Restates the parts of ``src/world/materials.ts`` the world build reads:
the voxel encoding (``:1-5``), ``vox`` (``:108-110``), material ids in
definition order (``define``, ``:68-95``; palette ``M``, ``:115-190``) and the
``glass`` value that decides opacity (``VoxelWorld.ts:159-170,190-196``).
Shading fields (colours, patterns, prices) are not needed by the build and
are left out.
"""
from __future__ import annotations

RUBBLE = 128   # materials.ts:63

# (name, glass) in definition order; id = position + 1 (materials.ts:69).
_PALETTE = [
    ("concrete", 0), ("wall", 0), ("wallDark", 0), ("ceiling", 0), ("floor", 0),
    ("marble", 0), ("marbleBlack", 0), ("frame", 0), ("windowGlass", 0.82),
    ("gold", 0), ("chrome", 0), ("steelDark", 0), ("lacquer", 0), ("ivory", 0),
    ("walnut", 0), ("walnutZ", 0), ("walnutY", 0), ("oak", 0),
    ("velvet", 0), ("velvetRed", 0), ("leather", 0), ("foam", 0), ("felt", 0), ("carpet", 0),
    ("crystal", 0.9), ("glassClear", 0.9), ("glassTable", 0.75), ("glassGreen", 0.7),
    ("glassAmber", 0.7), ("glassBlue", 0.7), ("glassRed", 0.7), ("glassSmoke", 0.65),
    ("champagne", 0.7), ("wine", 0.55), ("whiskey", 0.65), ("absinthe", 0.65),
    ("ice", 0.75), ("water", 0.8),
    ("porcelain", 0), ("porcelainRed", 0), ("terracotta", 0), ("soil", 0), ("leaf", 0), ("trunk", 0),
    ("dieRed", 0.35), ("pip", 0), ("chip", 0), ("card", 0),
    ("neonPink", 0), ("neonCyan", 0), ("neonGold", 0), ("bulb", 0), ("lampshade", 0),
    ("screen", 0), ("tv", 0), ("plasticBlack", 0), ("slotRed", 0), ("paperArt", 0),
    ("mirror", 0), ("label", 0), ("cork", 0), ("velvetGold", 0),
    ("chipRed", 0), ("chipBlue", 0), ("chipGreen", 0), ("chipBlack", 0), ("chipPurple", 0),
]

GLASS = {i + 1: g for i, (_, g) in enumerate(_PALETTE)}
# emission (materials.ts:34,80; nonzero only for these, :171-177)
EMISSION = {"neonPink": 6, "neonCyan": 6, "neonGold": 6, "bulb": 8, "lampshade": 1.3, "screen": 2.5, "tv": 1.6}
NUM_MATERIALS = len(_PALETTE)


class _Palette:
    pass


M = _Palette()
for _i, (_name, _g) in enumerate(_PALETTE):
    setattr(M, _name, _i + 1)


def vox(material_id: int, shade: int = 0) -> int:
    """``vox`` (materials.ts:108-110): low byte material, high byte shade."""
    return (int(material_id) & 0xFF) | ((int(shade) & 0xFF) << 8)


def opaque_table() -> list[int]:
    """``initOpaqueTable`` (VoxelWorld.ts:190-196).

    Entry 0 stays 0; ids without a material (the reference's ``mat(i)`` is
    undefined) count as opaque, glass materials as see-through.
    """
    t = [0] * 256
    for i in range(1, 256):
        g = GLASS.get(i)
        t[i] = 1 if (g is None or g == 0) else 0
    return t


def uniform_density_table() -> list[int]:
    """Density of a uniform brick per material id (VoxelWorld.ts:162).

    ``mat(g & 0xff).glass > 0 ? 0 : 255``.  For ids with no material the
    reference would throw; the table treats them as opaque (255), matching
    the opacity table above.
    """
    t = [255] * 256
    for i in range(256):
        g = GLASS.get(i)
        if g is not None and g > 0:
            t[i] = 0
    return t


def emission_table() -> list:
    """Per material byte: 1 if the material emits (mat(id).emission > 0), 0 if not,
    2 if no material has that id (mat(id) is undefined in the reference)."""
    t = [2] * 256
    for i, (name, _) in enumerate(_PALETTE):
        t[i + 1] = 1 if EMISSION.get(name, 0) > 0 else 0
    return t
