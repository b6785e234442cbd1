"""JavaScript number semantics that differ from Python's defaults.

Host-side helpers used while building ops (scene placement, constructor
constants).  Only the arithmetic the reference's host code uses is covered.
"""
from __future__ import annotations

import math

PI = math.pi   # Math.PI


def js_round(x: float) -> float:
    """``Math.round``: round half toward +infinity.

    ``floor(x + 0.5)`` is wrong for 0.49999999999999994, so compare the exact
    fractional part instead (``x - floor(x)`` is exact for finite doubles).
    """
    if not math.isfinite(x):
        return x
    r = math.floor(x)
    if x - r >= 0.5:
        r += 1
    return float(r)


def js_hypot(*args: float) -> float:
    """``Math.hypot`` as engines that follow the scaled, compensated method do.

    Published method: scale every operand by the largest magnitude, sum the
    squares with Kahan compensated summation, and return ``sqrt(sum) * max``.
    This is not ``sqrt(x*x + y*y)`` and not C's ``hypot``; results differ in
    the last bit for some inputs.
    """
    vals = [abs(float(a)) for a in args]
    if any(math.isinf(v) for v in vals):
        return math.inf
    if any(math.isnan(v) for v in vals):
        return math.nan
    m = max(vals) if vals else 0.0
    if m == 0:
        return 0.0
    s = 0.0
    comp = 0.0
    for v in vals:
        n = v / m
        summand = n * n - comp
        prelim = s + summand
        comp = (prelim - s) - summand
        s = prelim
    return math.sqrt(s) * m


def js_max(*args: float) -> float:
    """``Math.max`` (NaN-propagating)."""
    r = -math.inf
    for a in args:
        if a != a:
            return math.nan
        if a > r:
            r = a
    return r


def js_min(*args: float) -> float:
    """``Math.min`` (NaN-propagating)."""
    r = math.inf
    for a in args:
        if a != a:
            return math.nan
        if a < r:
            r = a
    return r


def js_or_eps(v: float, eps: float = 1e-12) -> float:
    """``v || eps``: 0 and NaN are falsy in JavaScript."""
    return eps if (v == 0 or v != v) else v


def u32(x: int) -> int:
    return x & 0xFFFFFFFF


def imul(a: int, b: int) -> int:
    """``Math.imul`` viewed as an unsigned 32-bit result."""
    return (a * b) & 0xFFFFFFFF


def mulberry32(seed: int):
    """``rng(seed)`` of penthouse.ts:55-64 (mulberry32), returning doubles in [0, 1)."""
    state = [seed & 0xFFFFFFFF]

    def nxt() -> float:
        a = u32(state[0] + 0x6D2B79F5)
        state[0] = a
        t = a
        t = imul(t ^ (t >> 15), t | 1)
        t = t ^ u32(t + imul(t ^ (t >> 7), t | 61))
        return u32(t ^ (t >> 14)) / 4294967296

    return nxt
