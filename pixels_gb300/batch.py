"""Batched builds: many independent scenes rebuilt by one CUDA graph launch.

``Batch(worlds)`` captures the rebuild of every world (each from the op list
of its last build) into one graph over several streams (``px_batch_create``);
``run()`` relaunches it.  Each world's result is its scene's build, the same
bits as building it alone.

``tune()`` is the autotuner of the batched path: it sweeps the launch shape —
streams the scenes are dealt over, and (op, brick) pairs per block of each
scene's persistent grids (0 = every kernel takes the whole GPU) — times each
shape's graph on the device, and returns the fastest.
"""
from __future__ import annotations

import statistics

from . import _lib

# launch shapes the autotuner tries: (streams, pairs per block)
SHAPES = ((1, 0), (8, 0), (32, 0), (8, 256), (32, 128), (32, 256), (32, 2048), (64, 256), (64, 1024), (128, 256))


class Batch:
    def __init__(self, worlds, mode: int | None = None, n_streams: int = 32, pairs_per_block: int = 256):
        for w in worlds:
            w._ensure()
        self.worlds = list(worlds)
        self.mode = self.worlds[0].mode if mode is None else mode
        self.shape = (int(n_streams), int(pairs_per_block))
        self._b = _lib.batch_create([w._h for w in self.worlds], self.mode, self.shape[0], self.shape[1])

    def run(self, stream: int = 0) -> float:
        """Launch the graph and wait; returns its device time (ms)."""
        return _lib.batch_run(self._b, stream)

    def close(self) -> None:
        if getattr(self, "_b", None) is not None:
            _lib.batch_destroy(self._b)
            self._b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune(worlds, mode: int | None = None, shapes=SHAPES, repeats: int = 3, warmup: int = 1):
    """Time every launch shape; returns ((streams, pairs_per_block), ms, table)."""
    table = []
    for n_streams, ppb in shapes:
        with Batch(worlds, mode, n_streams, ppb) as b:
            for _ in range(warmup):
                b.run()
            ms = statistics.median(b.run() for _ in range(repeats))
        table.append({"streams": n_streams, "pairs_per_block": ppb, "ms": round(ms, 4)})
    best = min(table, key=lambda r: r["ms"])
    return (best["streams"], best["pairs_per_block"]), best["ms"], table
