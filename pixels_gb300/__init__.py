"""GB300-native scene voxeliser (drop-in for the reference's world builder)."""
from . import config, ir, jsmath, materials, paints, shapes  # noqa: F401
from .config import set_vpm  # noqa: F401
from .shapes import Builder, Op, Shape, apply  # noqa: F401
