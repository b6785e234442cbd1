"""Stroke font for neon signs (restates ``src/scene/font.ts``).

Glyphs live on a 4 x 6 grid (y up); each glyph is a list of polylines.
"""
from __future__ import annotations

import math


def _star() -> list[float]:
    """font.ts:6-14: a five-pointed star polyline (cos/sin from the host libm)."""
    pts: list[float] = []
    for i in range(11):
        a = math.pi / 2 + (i * math.pi) / 5
        r = 3 if i % 2 == 0 else 1.25
        pts.extend((2 + math.cos(a) * r, 3 + math.sin(a) * r))
    return pts


GLYPHS = {   # font.ts:16-39
    "A": [[0, 0, 2, 6, 4, 0], [0.9, 2.4, 3.1, 2.4]],
    "B": [[0, 0, 0, 6, 3, 6, 4, 5, 4, 4, 3, 3, 0, 3], [3, 3, 4, 2, 4, 1, 3, 0, 0, 0]],
    "C": [[4, 5, 3, 6, 1, 6, 0, 5, 0, 1, 1, 0, 3, 0, 4, 1]],
    "E": [[4, 6, 0, 6, 0, 0, 4, 0], [0, 3, 3, 3]],
    "G": [[4, 5, 3, 6, 1, 6, 0, 5, 0, 1, 1, 0, 3, 0, 4, 1, 4, 3, 2, 3]],
    "I": [[2, 0, 2, 6], [1, 0, 3, 0], [1, 6, 3, 6]],
    "J": [[1, 6, 4, 6], [3, 6, 3, 1, 2, 0, 1, 0, 0, 1]],
    "K": [[0, 0, 0, 6], [4, 6, 0, 2.5], [1.2, 3.4, 4, 0]],
    "L": [[0, 6, 0, 0, 4, 0]],
    "N": [[0, 0, 0, 6, 4, 0, 4, 6]],
    "O": [[1, 0, 0, 1, 0, 5, 1, 6, 3, 6, 4, 5, 4, 1, 3, 0, 1, 0]],
    "P": [[0, 0, 0, 6, 3, 6, 4, 5, 4, 4, 3, 3, 0, 3]],
    "R": [[0, 0, 0, 6, 3, 6, 4, 5, 4, 4, 3, 3, 0, 3], [2, 3, 4, 0]],
    "S": [[4, 5, 3, 6, 1, 6, 0, 5, 0, 4, 1, 3, 3, 3, 4, 2, 4, 1, 3, 0, 1, 0, 0, 1]],
    "T": [[0, 6, 4, 6], [2, 6, 2, 0]],
    "U": [[0, 6, 0, 1, 1, 0, 3, 0, 4, 1, 4, 6]],
    "V": [[0, 6, 2, 0, 4, 6]],
    "X": [[0, 0, 4, 6], [0, 6, 4, 0]],
    "Y": [[0, 6, 2, 3, 4, 6], [2, 3, 2, 0]],
    "7": [[0, 6, 4, 6, 1.5, 0]],
    "*": [_star()],
    " ": [],
}


def layout_text(text: str):
    """``layoutText`` (font.ts:47-60): strokes in glyph units (height 6, advance 5.5)."""
    strokes = []
    x = 0.0
    for ch in text.upper():
        g = GLYPHS.get(ch, [])
        for line in g:
            i = 0
            while i + 3 < len(line):
                strokes.append(((x + line[i], float(line[i + 1])), (x + line[i + 2], float(line[i + 3]))))
                i += 2
        x += 5.5
    return strokes, max(0.0, x - 1.5)
