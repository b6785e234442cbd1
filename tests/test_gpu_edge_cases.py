"""Edge cases of the rasteriser against the oracle, bit for bit, in both forms.

Empty op lists, ops wholly outside the world, degenerate shapes (zero-size
boxes, capsules with equal ends, lathe profiles with repeated points,
collinear prisms), paints on air and paints that return air, carve/re-add
sequences that reuse freed pool bricks in LIFO order, a world wider than
the float32 path certifies (every op then runs in float64), unions, and CSG /
rotation trees deeper than the register evaluators hold (shapes.ts:227-320
put no limit on nesting), and allocator churn (bricks freed and reallocated
many times in one build, then a build that starts with holes).
"""
import numpy as np
import pytest

from pixels_gb300 import config
from pixels_gb300.ir import Program
from pixels_gb300.materials import M, vox
from pixels_gb300.paints import black_keys, tufted
from pixels_gb300.shapes import (box, boxMinMax, capsule, cylinder, ellipsoid, intersect, lathe, prism, rotateX,
                                 rotateY, rotateZ, roundBox, sphere, subtract, torus, union)
from pixels_gb300.world import MODE_FP64, MODE_MIXED, VoxelWorld

import pyoracle


def run_both(prog: Program, vpm: float, dims):
    """Build the op list on the GPU in both forms (and in validation mode) and the oracle."""
    o = pyoracle.OracleWorld(prog.to_bytes(), vpm, dims)
    out = []
    for mode, validate in ((MODE_FP64, False), (MODE_MIXED, False), (MODE_MIXED, True)):
        w = VoxelWorld(*dims, initialPoolBricks=4, vpm=vpm, mode=mode)
        if validate:
            from pixels_gb300 import _lib
            _lib.set_validation(w._h, True)
        w._pending = prog
        w.build()
        grid = w.grid
        np.testing.assert_array_equal(grid, o.grid, err_msg=f"grid, mode {mode} validate {validate}")
        assert w.poolUsed == o.pool_used
        np.testing.assert_array_equal(w.freeBricks(), o.free_holes)
        live = np.nonzero((o.grid != 0) & ((o.grid & 0x80000000) == 0))[0]
        idx = o.grid[live].astype(np.int64) - 1
        np.testing.assert_array_equal(w.pool.reshape(-1, 512)[idx], o.pool.reshape(-1, 512)[idx])
        d = w.derived()
        np.testing.assert_array_equal(d["super"], o.super)
        np.testing.assert_array_equal(d["density"], o.density)
        if validate:
            assert w.stats()["violations"] == 0
        out.append(w.stats())
        w.close()
    return o, out


def program(vpm, ops):
    prog = Program()
    with config.using(vpm):
        for kind, shape, paint in ops():
            prog.add_op(kind, shape, paint)
    return prog


@pytest.mark.gpu
def test_empty_op_list(built_lib):
    o, _ = run_both(Program(), 40.0, (64, 32, 48))
    assert o.pool_used == 0 and not o.grid.any()


@pytest.mark.gpu
def test_ops_outside_the_world_and_degenerate_shapes(built_lib):
    vpm = 40.0
    vs = 1 / vpm

    def ops():
        yield 0, box((-5.0, -5.0, -5.0), (0.5, 0.5, 0.5)), vox(M.wall)           # wholly outside
        yield 0, box((0.5, 0.4, 0.5), (0.0, 0.0, 0.0)), vox(M.marble)            # zero-size box
        yield 0, capsule((0.3, 0.3, 0.3), (0.3, 0.3, 0.3), 0.1), vox(M.gold)      # equal ends: bb || 1e-12
        yield 0, lathe((0.8, 0.2, 0.8), [0.1, 0.0, 0.1, 0.0, 0.15, 0.2, 0.0, 0.3], 0), vox(M.porcelain)  # repeated point
        yield 0, lathe((0.2, 0.2, 0.9), [0.05, 0.0, 0.05, 0.0, 0.08, 0.25], vs * 2), vox(M.glassClear)
        yield 0, prism((0.6, 0.1, 0.3), [0.0, 0.0, 0.1, 0.0, 0.2, 0.0, 0.1, 0.1], 0.1, 0.3), vox(M.oak)  # collinear
        yield 0, torus((0.4, 0.5, 0.6), 0.15, 0.0, "x"), vox(M.chrome)          # radius clamped to the minimum
        yield 0, cylinder((1.0, 0.3, 0.2), 0.0, 0.0, "z"), vox(M.steelDark)      # clamped radius and height
        yield 0, rotateY(roundBox((0.9, 0.5, 0.5), (0.2, 0.1, 0.15), 0.05), 0.7, (0.9, 0.5, 0.5)), vox(M.velvet)
        yield 0, subtract(sphere((0.5, 0.5, 0.5), 0.3), box((0.5, 0.5, 0.5), (0.1, 0.4, 0.1))), vox(M.felt)
    o, _ = run_both(program(vpm, ops), vpm, (48, 32, 48))
    assert o.pool_used > 0


@pytest.mark.gpu
def test_paints_on_air_paints_returning_air_and_pool_reuse(built_lib):
    vpm = 40.0

    def ops():
        yield 2, box((0.4, 0.4, 0.4), (0.3, 0.3, 0.3)), vox(M.gold)             # paint on air: nothing
        yield 0, boxMinMax(0.1, 0.1, 0.1, 0.9, 0.6, 0.9), vox(M.wall)
        yield 0, boxMinMax(0.2, 0.2, 0.2, 0.7, 0.5, 0.7), black_keys(0.2, M.lacquer)  # returns 0 between keys
        yield 1, sphere((0.5, 0.35, 0.5), 0.25), 0                                # carve: frees bricks
        yield 2, boxMinMax(0.0, 0.0, 0.0, 1.0, 0.7, 1.0), tufted(0.1, 0.1, M.leather)
        yield 0, sphere((0.45, 0.4, 0.45), 0.12), vox(M.bulb)                     # re-add: pops freed bricks
        yield 1, boxMinMax(0.0, 0.0, 0.0, 1.0, 1.0, 0.35), 0                      # frees more
        yield 0, capsule((0.1, 0.2, 0.1), (0.9, 0.5, 0.3), 0.08), vox(M.chrome)
    o, stats = run_both(program(vpm, ops), vpm, (48, 32, 48))
    assert o.free_holes.size > 0 or o.stats["frees"] > 0
    assert all(s["free_events"] > 0 for s in stats)


@pytest.mark.gpu
def test_world_wider_than_the_float32_range(built_lib):
    """1,104 m along z at 1 voxel per metre: every op runs in float64 in the mixed form."""
    vpm = 1.0

    def ops():
        yield 0, boxMinMax(0.0, 0.0, 1000.0, 8.0, 8.0, 1100.0), vox(M.concrete)
        yield 0, sphere((4.0, 4.0, 1050.0), 3.5), vox(M.marble)
        yield 1, capsule((1.0, 1.0, 1010.0), (7.0, 7.0, 1090.0), 1.2), 0
    o, stats = run_both(program(vpm, ops), vpm, (8, 8, 1104))
    assert o.pool_used > 0
    assert stats[1]["rescued"] == 0  # nothing to rescue: no float32 evaluation at all


@pytest.mark.gpu
def test_union_and_deep_csg_and_rotation_trees(built_lib):
    """union (shapes.ts:227-238) of six overlapping shapes; a subtract chain six
    deep, subtract(a, subtract(b, subtract(c, ...))); rotations nested five deep
    (rotateY(rotateX(rotateZ(rotateY(rotateX(...)))))); and a union of
    intersections of rotated subtracts.  Programs deeper than four stack values
    or three rotation frames run on the deep float64 evaluator in both forms."""
    vpm = 40.0

    def chain(depth, c):
        s = sphere(c, 0.05 + 0.03 * depth)
        for k in range(depth):
            r = 0.08 + 0.03 * (depth - k)
            outer = box(c, (r, r * 0.8, r * 0.9)) if k % 2 else sphere(c, r)
            s = subtract(outer, s)
        return s

    def nested_rot(shape, c, depth):
        for k in range(depth):
            rot = (rotateY, rotateX, rotateZ)[k % 3]
            shape = rot(shape, 0.3 + 0.41 * k, c)
        return shape

    def ops():
        u = union(sphere((0.3, 0.3, 0.3), 0.12), box((0.4, 0.3, 0.3), (0.1, 0.05, 0.08)),
                  capsule((0.2, 0.2, 0.4), (0.5, 0.4, 0.4), 0.04), torus((0.35, 0.35, 0.25), 0.1, 0.03, "z"),
                  cylinder((0.3, 0.45, 0.3), 0.05, 0.1, "y"), ellipsoid((0.45, 0.3, 0.45), (0.08, 0.05, 0.12)))
        yield 0, u, vox(M.marble)
        yield 0, chain(6, (0.9, 0.4, 0.4)), vox(M.gold)                        # stack depth 7
        c = (0.6, 0.45, 0.9)
        yield 0, nested_rot(roundBox(c, (0.15, 0.05, 0.1), 0.02), c, 5), vox(M.oak)   # 5 rotation frames
        d = (1.0, 0.3, 1.0)
        deep = union(*[intersect(nested_rot(subtract(box(d, (0.2, 0.2, 0.2)), sphere(d, 0.1 + 0.02 * k)), d, 4),
                                 sphere(d, 0.22 + 0.01 * k)) for k in range(3)])
        yield 0, deep, vox(M.velvet)
        yield 1, union(sphere((0.3, 0.3, 0.3), 0.06), chain(5, (0.35, 0.32, 0.3))), 0   # carve with a deep union
        yield 2, nested_rot(chain(4, (0.9, 0.4, 0.4)), (0.9, 0.4, 0.4), 4), tufted(0.05, 0.05, M.leather)
    o, stats = run_both(program(vpm, ops), vpm, (64, 32, 64))
    assert o.pool_used > 0


@pytest.mark.gpu
def test_allocator_churn_across_scan_tiles_and_builds(built_lib):
    """The pool allocator under churn (VoxelWorld.ts:112-127): the same bricks
    allocated, freed and allocated again many times in one build, so that pool
    indices pass along long chains of pushes and pops, over enough (op, brick)
    pairs for many tiles of the replay's scan; then a second build that starts
    with holes.  The world after both builds must equal the oracle's after the
    concatenated op list, bit for bit, in both forms."""
    vpm = 40.0
    dims = (96, 48, 96)
    rng = np.random.default_rng(7)
    centres = [tuple(float(v) for v in (rng.uniform(0.5, 1.9), rng.uniform(0.4, 0.8), rng.uniform(0.5, 1.9)))
               for _ in range(16)]

    def first():
        for k, c in enumerate(centres):
            yield 0, sphere(c, 0.35), vox(M.marble)                                   # allocates mixed bricks
            yield 0, capsule((c[0] - 0.3, c[1], c[2]), (c[0] + 0.3, c[1] + 0.1, c[2]), 0.12), vox(M.gold)
            yield 1, box(c, (0.45, 0.45, 0.45)), 0                                    # frees them all again
            yield 0, sphere((c[0] + 0.05, c[1], c[2] - 0.05), 0.3), vox(M.oak)       # pops the freed bricks
            if k % 3 == 2:
                yield 1, boxMinMax(c[0] - 0.2, 0.0, c[2] - 0.2, c[0] + 0.5, 1.2, c[2] + 0.5), 0
        yield 1, boxMinMax(0.0, 0.0, 0.0, 2.4, 1.2, 1.2), 0                           # leaves holes behind

    def second():
        for c in centres[::2]:
            yield 0, roundBox(c, (0.3, 0.2, 0.25), 0.05), vox(M.velvet)               # pops the holes first
            yield 1, sphere(c, 0.15), 0
        yield 2, boxMinMax(0.0, 0.0, 0.0, 2.4, 1.2, 2.4), tufted(0.1, 0.1, M.leather)

    def both():
        yield from first()
        yield from second()

    o = pyoracle.OracleWorld(program(vpm, both).to_bytes(), vpm, dims)
    assert o.stats["frees"] > 1000
    for mode in (MODE_FP64, MODE_MIXED):
        w = VoxelWorld(*dims, initialPoolBricks=4, vpm=vpm, mode=mode)
        w._pending = program(vpm, first)
        w.build()
        assert w.freeBricks().size > 0  # the second build starts with holes
        w._pending = program(vpm, second)
        w.build()
        np.testing.assert_array_equal(w.grid, o.grid, err_msg=f"grid, mode {mode}")
        assert w.poolUsed == o.pool_used
        np.testing.assert_array_equal(w.freeBricks(), o.free_holes)
        live = np.nonzero((o.grid != 0) & ((o.grid & 0x80000000) == 0))[0]
        idx = o.grid[live].astype(np.int64) - 1
        np.testing.assert_array_equal(w.pool.reshape(-1, 512)[idx], o.pool.reshape(-1, 512)[idx])
        d = w.derived()
        np.testing.assert_array_equal(d["super"], o.super)
        np.testing.assert_array_equal(d["density"], o.density)
        w.close()
