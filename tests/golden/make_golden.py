"""Generate tests/golden/penthouse.json: digests of the world the float64
oracle builds from the penthouse scene at small densities.

The reference repository ships no tests or fixtures; its README table
(vpm -> grid dims, live bricks) is the only published pin and is checked by
tests/test_oracle_pins.py.  These digests freeze the oracle's full output
(grid with pool indices, live pool bricks, free-list holes, super-grid
counts, density) so that any change to the oracle or the scene program shows
up, and so the GPU tests on a machine without this repository's history can
compare against them.

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
from pixels_gb300 import config  # noqa: E402
from pixels_gb300.scenes.penthouse import penthouse_program  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def world_digests(o) -> dict:
    g = o.grid
    live = np.nonzero((g != 0) & ((g & 0x80000000) == 0))[0]
    idx = g[live].astype(np.int64) - 1
    live_pool = o.pool.reshape(-1, 512)[idx] if len(idx) else np.zeros((0, 512), np.uint16)
    return {
        "dims": list(o.dims), "pool_used": int(o.pool_used), "n_holes": int(len(o.free_holes)),
        "live_bricks": int(o.live_bricks),
        "grid": digest(g), "live_pool": digest(live_pool), "holes": digest(o.free_holes),
        "super": digest(o.super), "density": digest(o.density),
        "uniform_cells": int(np.count_nonzero(g & 0x80000000)), "pool_cells": int(len(live)),
        "stats": {k: int(v) for k, v in o.stats.items()},
    }


def main():
    out = {}
    for vpm in (20.0, 40.0):
        prog, _ = penthouse_program(vpm)
        ir = prog.to_bytes()
        o = pyoracle.OracleWorld(ir, vpm, config.Config(vpm).dims, count_flops=True)
        d = world_digests(o)
        d["ops"] = len(prog)
        d["ir_sha256"] = hashlib.sha256(ir).hexdigest()
        out[f"{vpm:g}"] = d
    with open(os.path.join(HERE, "penthouse.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps({k: (v["pool_used"], v["grid"][:12]) for k, v in out.items()}))


if __name__ == "__main__":
    main()
