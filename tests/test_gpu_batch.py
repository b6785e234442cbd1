"""Batched builds (many scenes in one CUDA graph) against the oracle, scene by scene."""
import math

import numpy as np
import pytest

from pixels_gb300 import _lib
from pixels_gb300.batch import Batch, tune
from pixels_gb300.scenes.synthetic import batch_specs, dims_for, synthetic_program
from pixels_gb300.world import MODE_FP64, MODE_MIXED, VoxelWorld

import pyoracle


def test_batch_specs_follow_the_workload():
    specs = batch_specs(seed=7, n=256)
    assert len(specs) == 256 and specs == batch_specs(seed=7, n=256)
    for s in specs:
        v = math.prod(s["volume"])
        assert 0.5 * 0.999 <= v <= 64 * 1.001
        assert max(s["volume"]) / min(s["volume"]) <= 4.0 + 1e-6
        assert 16 <= s["n_prims"] <= 2048
        assert s["vpm"] in (40.0, 80.0, 160.0)
        assert s["dims"] == dims_for(s["volume"], s["vpm"]) and all(d % 8 == 0 for d in s["dims"])
    assert len({s["vpm"] for s in specs}) == 3


def small_specs():
    """Uneven scenes small enough for the oracle: 0.05-1.5 m^3, 16-300 primitives."""
    rng = np.random.default_rng(3)
    out = []
    for i in range(7):
        vol = tuple(float(np.float32(x)) for x in rng.uniform(0.3, 1.4, size=3))
        vpm = (40.0, 80.0)[i % 2]
        out.append({"seed": 500 + i, "volume": vol, "n_prims": int(rng.integers(16, 300)), "vpm": vpm,
                    "dims": dims_for(vol, vpm)})
    return out


def make_worlds(specs, mode):
    worlds, progs = [], []
    for s in specs:
        prog = synthetic_program(s["seed"], s["n_prims"], s["vpm"], s["volume"])
        w = VoxelWorld(*s["dims"], initialPoolBricks=64, vpm=s["vpm"], mode=mode)
        w._pending = prog
        w.build()
        worlds.append(w)
        progs.append(prog)
    return worlds, progs


def same_as_oracle(w, prog, vpm, dims):
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, dims)
    np.testing.assert_array_equal(w.grid, o.grid)
    assert w.poolUsed == o.pool_used
    np.testing.assert_array_equal(w.freeBricks(), o.free_holes)
    live = np.nonzero((o.grid != 0) & ((o.grid & 0x80000000) == 0))[0]
    idx = o.grid[live].astype(np.int64) - 1
    pool = w.pool.reshape(-1, 512)
    np.testing.assert_array_equal(pool[idx], o.pool.reshape(-1, 512)[idx])
    d = w.derived()
    np.testing.assert_array_equal(d["super"], o.super)
    np.testing.assert_array_equal(d["density"], o.density)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [MODE_MIXED, MODE_FP64])
def test_batch_matches_each_scene_alone(built_lib, mode):
    specs = small_specs()
    worlds, progs = make_worlds(specs, mode)
    alone = [(w.grid.copy(), w.pool.copy()) for w in worlds]
    with Batch(worlds, n_streams=4, pairs_per_block=64) as b:
        for _ in range(2):  # the graph relaunches: the same worlds again
            ms = b.run()
            assert ms > 0
            for w, (g, p) in zip(worlds, alone):
                np.testing.assert_array_equal(w.grid, g)
                np.testing.assert_array_equal(w.pool, p)
        for w, prog, s in zip(worlds, progs, specs):
            same_as_oracle(w, prog, s["vpm"], s["dims"])
        # a world in a batch cannot be rebuilt
        with pytest.raises(_lib.PxError):
            worlds[0].build()
    for w in worlds:
        w.close()


@pytest.mark.gpu
def test_autotuner_picks_a_measured_shape(built_lib):
    specs = small_specs()[:4]
    worlds, _ = make_worlds(specs, MODE_MIXED)
    shape, ms, table = tune(worlds, shapes=((1, 0), (4, 64)), repeats=2)
    assert shape in {(1, 0), (4, 64)} and len(table) == 2
    assert ms == min(r["ms"] for r in table) and ms > 0
    for w in worlds:
        w.close()
