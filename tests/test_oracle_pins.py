"""The oracle pinned against the only published figures of the reference
(README.md:168-173: grid dims and live bricks per voxel density) and against
the committed golden digests of its own output."""
import json
import os

import numpy as np
import pytest

import pyoracle
from pixels_gb300 import config
from pixels_gb300.scenes.penthouse import penthouse_program

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("vpm,dims", [(64, (1024, 288, 768)), (80, (1280, 352, 960)),
                                      (100, (1600, 448, 1200)), (128, (2048, 568, 1536))])
def test_dims_match_readme(vpm, dims):
    # 4.4 * 100 = 440.00000000000006 in float64 -> ceil(55.000000000000007) * 8 = 448
    assert config.Config(vpm).dims == dims


@pytest.mark.parametrize("vpm,live_k", [(64, 42), (80, 46), (100, 75)])
def test_live_bricks_match_readme(vpm, live_k):
    prog, _ = penthouse_program(float(vpm))
    o = pyoracle.OracleWorld(prog.to_bytes(), float(vpm), config.Config(vpm).dims)
    assert round(o.live_bricks / 1000) == live_k, o.live_bricks


def test_golden_digests():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    gold = json.load(open(os.path.join(HERE, "golden", "penthouse.json")))
    for key in ("20", "40"):
        vpm = float(key)
        prog, _ = penthouse_program(vpm)
        o = pyoracle.OracleWorld(prog.to_bytes(), vpm, config.Config(vpm).dims, count_flops=True)
        d = mg.world_digests(o)
        for k in ("grid", "live_pool", "holes", "super", "density", "pool_used", "live_bricks"):
            assert d[k] == gold[key][k], (key, k)


def test_multithreaded_oracle_equals_sequential():
    vpm = 40.0
    prog, _ = penthouse_program(vpm)
    ir = prog.to_bytes()
    dims = config.Config(vpm).dims
    a = pyoracle.OracleWorld(ir, vpm, dims)
    b = pyoracle.OracleWorld(ir, vpm, dims, threads=4)
    assert np.array_equal(a.grid, b.grid)
    assert a.pool_used == b.pool_used
    assert np.array_equal(a.pool, b.pool)
    assert np.array_equal(a.free_holes, b.free_holes)
    assert np.array_equal(a.density, b.density)
