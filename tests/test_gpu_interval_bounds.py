"""The float32 interval evaluator's square-root bounds, checked exhaustively.

The mixed form encloses sqrt(v) with the hardware reciprocal square root
(csrc/sdf32.cuh, sqrt_lo / sqrt_hi) instead of the IEEE directed square roots.
For every float32 v in [2^-100, 2^100] -- the range where those bounds are
used -- they must enclose the directed square roots of this GPU; below and
above that range the evaluator takes constant bounds or the directed roots.
"""
import struct

import pytest

from pixels_gb300 import _lib


def bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


@pytest.mark.gpu
def test_sqrt_bounds_enclose_the_directed_roots_everywhere_they_are_used(built_lib):
    lo, hi = bits(2.0 ** -100), bits(2.0 ** 100)
    n_bad, first = _lib.check_sqrt_bounds(lo, hi)
    assert n_bad == 0, f"{n_bad} failures, first at bit pattern {first:#x}"


@pytest.mark.gpu
def test_sqrt_bounds_at_the_range_edges(built_lib):
    """The constant and fallback branches: 0, the smallest subnormal, up to the
    fast range, and the largest finite floats."""
    for lo, hi in ((0, bits(2.0 ** -100) + 1024), (bits(2.0 ** 100) - 1024, 0x7f7fffff)):
        n_bad, first = _lib.check_sqrt_bounds(lo, hi)
        assert n_bad == 0, f"{n_bad} failures in [{lo:#x}, {hi:#x}], first {first:#x}"
