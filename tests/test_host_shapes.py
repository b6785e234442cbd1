"""Host-side constructors (shapes.ts restated): bounds, clamps, captured
constants, and the op IR round trip."""
import math

import numpy as np
import pytest

from pixels_gb300 import config, ir
from pixels_gb300.paints import chip_stack, local_paint, card
from pixels_gb300.shapes import (box, boxMinMax, capsule, cylinder, ellipsoid, intersect, lathe, offset, prism,
                                 rotateX, rotateY, rotateZ, roundBox, sphere, stadium, subtract, torus, union)
from pixels_gb300.world import OpRecorder


def test_box_min_max_and_contains():
    s = boxMinMax(1.0, 2.0, 3.0, 0.0, 5.0, 4.0)
    assert s.min == (0.0, 2.0, 3.0) and s.max == (1.0, 5.0, 4.0) and s.contains
    assert s.contains_box(0.0, 2.0, 3.0, 1.0, 5.0, 4.0)
    assert not s.contains_box(-0.1, 2.0, 3.0, 1.0, 5.0, 4.0)
    assert not roundBox((0, 0, 0), (1, 1, 1), 0.1).contains


def test_radius_clamps_follow_voxel_size():
    with config.using(20):
        vs = 1 / 20
        c = capsule((0, 0, 0), (1, 0, 0), 0.001)
        assert c.node[2][-1] == 0.9 * vs
        cy = cylinder((0, 0, 0), 0.001, 0.001)
        assert cy.node[2][3] == 0.6 * vs and cy.node[2][4] == vs * 0.5
        t = torus((0, 0, 0), 1.0, 0.0)
        assert t.node[2][4] == 0.9 * vs
        la = lathe((0, 0, 0), (0.1, 0, 0.1, 1), 0.001)
        assert la.node[2][3] == (1.75 * vs) / 2


def test_capsule_degenerate_segment_uses_epsilon():
    c = capsule((1, 2, 3), (1, 2, 3), 0.1)
    assert c.node[2][6] == 1e-12


def test_ellipsoid_slack_and_combinator_slack():
    e = ellipsoid((0, 0, 0), (0.2, 0.1, 0.05))
    assert e.slack == 0.2 / 0.05
    assert subtract(box((0, 0, 0), (1, 1, 1)), e).slack == e.slack
    assert intersect(e, box((0, 0, 0), (1, 1, 1))).slack == e.slack
    assert union(box((0, 0, 0), (1, 1, 1))).slack == 1.0
    assert offset(e, 0.01).slack == e.slack and not offset(box((0, 0, 0), (1, 1, 1)), 0.1).contains


def test_rotate_bounds_are_rotated_corners():
    b = box((1.0, 0.5, 2.0), (0.5, 0.5, 0.25))
    r = rotateY(b, math.pi / 2, (1.0, 0.0, 2.0))
    assert r.min[1] == b.min[1] and r.max[1] == b.max[1]
    assert abs(r.min[0] - 0.75) < 1e-12 and abs(r.max[0] - 1.25) < 1e-12
    assert abs(r.min[2] - 1.5) < 1e-12 and abs(r.max[2] - 2.5) < 1e-12
    rx = rotateX(b, 0.3, (0, 0.5, 2.0))
    assert rx.min[0] == b.min[0]
    rz = rotateZ(b, 0.3, (1.0, 0.5, 0))
    assert rz.min[2] == b.min[2]


def test_lathe_solid_closes_profile_against_axis():
    la = lathe((1, 2, 3), (0.3, 0.0, 0.2, 0.5), 0)
    params = la.node[2]
    assert list(params[3:]) == [0.0, 0.0, 0.3, 0.0, 0.2, 0.5, 0.0, 0.5]
    assert la.min == (1 - 0.3, 2.0, 3 - 0.3) and la.max == (1.3, 2.5, 3.3)


def test_prism_and_stadium_bounds():
    p = prism((1, 0, 1), (-0.5, -0.5, 0.5, -0.5, 0.0, 0.5), 0.2, 0.4)
    assert p.min == (0.5, 0.2, 0.5) and p.max == (1.5, 0.4, 1.5)
    s = stadium((2, 0, 3), 0.6, 0.5, 0.1, 0.3)
    assert s.min == (2 - 0.6 - 0.5, 0.1, 2.5) and s.max == (3.1, 0.3, 3.5)


def test_ir_round_trip_and_postfix():
    rec = OpRecorder(20.0)
    with config.using(20):
        sh = rotateY(subtract(box((1, 1, 1), (0.5, 0.5, 0.5)), sphere((1, 1, 1), 0.4), sphere((1, 1.5, 1), 0.2)),
                     0.5, (1, 0, 1))
        rec.submit(ir.ADD, sh, 0x0105)
        rec.submit(ir.PAINT, box((1, 1, 1), (0.1, 0.1, 0.1)), local_paint(card(1, 1, 0.0, 48), 0.3, (1, 0, 1)))
        rec.submit(ir.CARVE, sphere((2, 2, 2), 0.3), 0)
    ops, code, params = ir.decode(rec.program.to_bytes())
    assert len(ops) == 3
    ops0 = code[ops[0]["code_begin"]:ops[0]["code_begin"] + ops[0]["code_len"], 0] & 0xFF
    assert list(ops0) == [ir.OP_ROT_Y, ir.OP_BOX, ir.OP_SPHERE, ir.OP_NEGMAX, ir.OP_SPHERE, ir.OP_NEGMAX, ir.OP_ROT_END]
    assert ops[1]["paint_kind"] == ir.PAINT_CARD and ops[1]["flags"] & ir.OPF_PAINT_FRAME
    assert ops[0]["paint_value"] == 0x0105 and ops[2]["kind"] == ir.CARVE
    with pytest.raises(ValueError):
        rec.submit(ir.ADD, box((0, 0, 0), (1, 1, 1)), 0x10000)


def test_chip_stack_paint_matches_closure():
    with config.using(80):
        p = chip_stack(1.0, 0.5, 2.0, 0.022, 66)
        # a voxel on the stripe edge of layer 0
        v = p(1.0 + 0.021, 0.5 + 0.001, 2.0 + 0.0005)
        assert v & 0xFF == 66
        assert p(1.0, 0.5 + 0.001, 2.0) == 66  # the axis is not on the edge
