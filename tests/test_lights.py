"""Light anchors and light records (packLights / snapToEmissive, GpuWorld.ts:141-174)."""
import numpy as np
import pytest

from pixels_gb300 import config, materials
from pixels_gb300.ir import Program
from pixels_gb300.lights import MAX_ANCHORS, MAX_LIGHTS, anchor_voxels, pack_lights
from pixels_gb300.scenes.penthouse import build_penthouse, penthouse_program
from pixels_gb300.shapes import box
from pixels_gb300.world import MODE_MIXED, VoxelWorld

import pyoracle


class _FakeWorld:
    vpm = 40.0


def _emits(table):
    def f(m):
        if table[m] == 2:
            raise KeyError(m)
        return table[m] == 1
    return f


def test_pack_lights_layout_and_limits():
    lights = [dict(pos=(1.0, 2.0, 3.0), radius=4.5, color=(0.1, 0.2, 0.3), shadow=(i % 2 == 0),
                   anchors=[(0.5 + 0.1 * k, 1.0, 2.0) for k in range(20)]) for i in range(MAX_LIGHTS + 3)]
    words, anchors = pack_lights(_FakeWorld(), lights, snap=lambda xyz: xyz)
    assert words.size == MAX_LIGHTS * 16
    fl = words.view(np.float32)
    assert anchors.size == MAX_ANCHORS * 8
    for i in range(MAX_LIGHTS):
        o = i * 16
        np.testing.assert_array_equal(fl[o:o + 9], np.array([1, 2, 3, 4.5, 0.1, 0.2, 0.3, 1 if i % 2 == 0 else 0, 1],
                                                            dtype=np.float32))
        start, count = int(words[o + 9]), int(words[o + 10])
        assert start == min(20 * i, MAX_ANCHORS)
        assert count == max(0, min(20, MAX_ANCHORS - 20 * i))
        assert fl[o + 11] == np.float32(i * 7.31)
    # anchor words: x, y, z, 0, y, 0, 0, 0 with x = floor(a / (1 / vpm))
    assert tuple(anchors[:8]) == (20, 40, 80, 0, 40, 0, 0, 0)
    xyz, owner = anchor_voxels(lights, 40.0)
    assert len(xyz) == MAX_ANCHORS and owner[-1] == MAX_ANCHORS // 20


def test_oracle_snap_finds_the_nearest_shell_in_scan_order():
    """A 1-voxel emissive box: anchors 0, 1 and 2 voxels away snap onto it; 3 away stays."""
    vpm = 40.0
    vs = 1.0 / vpm
    prog = Program()
    with config.using(vpm):
        bulb = materials.vox(materials.M.bulb)
        prog.add_op(0, box((10.5 * vs, 10.5 * vs, 10.5 * vs), (0.4 * vs, 0.4 * vs, 0.4 * vs)), bulb)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, (32, 32, 32))
    assert o.get(10, 10, 10) == bulb
    emits = _emits(materials.emission_table())
    assert o.snap_to_emissive(emits, 10, 10, 10) == (10, 10, 10)
    assert o.snap_to_emissive(emits, 11, 11, 9) == (10, 10, 10)
    assert o.snap_to_emissive(emits, 12, 10, 8) == (10, 10, 10)
    assert o.snap_to_emissive(emits, 13, 10, 10) == (13, 10, 10)


def test_emission_table():
    t = materials.emission_table()
    assert t[0] == 2 and t[materials.M.bulb] == 1 and t[materials.M.neonPink] == 1 and t[materials.M.wall] == 0
    assert sum(1 for v in t if v == 1) == 7


@pytest.mark.gpu
@pytest.mark.parametrize("vpm", [20.0, 40.0])
def test_penthouse_lights_match_the_oracle(built_lib, vpm):
    cfg = config.Config(vpm)
    w = VoxelWorld(*cfg.dims, initialPoolBricks=1 << 14, vpm=vpm, mode=MODE_MIXED)
    scene = build_penthouse(w)
    w.build()
    words, anchors = pack_lights(w, scene["lights"])
    prog, scene_o = penthouse_program(vpm)
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, cfg.dims)
    emits = _emits(materials.emission_table())
    words_o, anchors_o = pack_lights(w, scene_o["lights"],
                                     snap=lambda xyz: [o.snap_to_emissive(emits, *map(int, a)) for a in xyz])
    np.testing.assert_array_equal(words, words_o)
    np.testing.assert_array_equal(anchors, anchors_o)
    xyz, _ = anchor_voxels(scene["lights"], vpm)
    moved = np.count_nonzero(np.any(anchors.reshape(-1, 8)[:len(xyz), :3].astype(np.int64) != xyz, axis=1))
    assert len(xyz) > 0 and moved > 0  # some anchors land just off their tube and are snapped
    w.close()
