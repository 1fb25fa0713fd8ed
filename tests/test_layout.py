"""Layout member operators and anchor symbols (no device needed).

The expected positions are worked by hand from the reference's rules
(crates/forgedthoughts/src/eval.rs: attach_object E:4934-4986,
align_object_axis E:4988-5019, place_object_relative E:5021-5039,
object_bounds E:4784-4916, face_object_to E:4679-4713) and compared with the
centre and rotation of the lowered primitive.
"""
import math

import numpy as np
import pytest

import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native

FLOOR = "var floor = Box { size: vec3(20.0, 0.5, 20.0) };\nfloor.pos.y = -1.15;\n"  # top face at y = -0.9


def _placed(src, kinds=(_native.FT_NODE_SPHERE, _native.FT_NODE_BOX)):
    """(centre, rotation) of each primitive of the scene, in node order."""
    d = ft.parse_and_eval(src).desc
    out = []
    for i in range(d.n_nodes):
        n = d.nodes[i]
        if n.kind in kinds:
            out.append((np.array(n.center[:]), np.array(n.rot_deg[:])))
    return out


def _pos(src, index=-1):
    return _placed(src)[index][0]


def test_attach_to_faces_with_offsets_and_gaps():
    s = "let a = Sphere { radius: 0.82 }.attach(floor, Top);\nlet scene = floor + a;\n"
    assert np.allclose(_pos(FLOOR + s), [0.0, -0.9 + 0.82, 0.0], atol=1e-6)
    # `Top + 0.3` offsets the face; a number as third argument is a gap.
    s = "let a = Sphere { radius: 0.5 }.attach(floor, Top + 0.3);\nlet scene = floor + a;\n"
    assert np.allclose(_pos(FLOOR + s), [0.0, -0.9 + 0.3 + 0.5, 0.0], atol=1e-6)
    s = "let a = Sphere { radius: 0.5 }.attach(floor, Top, 0.25);\nlet scene = floor + a;\n"
    assert np.allclose(_pos(FLOOR + s), [0.0, -0.9 + 0.25 + 0.5, 0.0], atol=1e-6)
    s = "let a = Sphere { radius: 0.5 }.attach(floor, Bottom - 0.1);\nlet scene = floor + a;\n"
    assert np.allclose(_pos(FLOOR + s), [0.0, -1.4 + 0.1 - 0.5, 0.0], atol=1e-6)
    box = "let b = Box { size: vec3(2.0, 2.0, 2.0) };\n"
    for face, expect in [("Left", [-1.5, 0, 0]), ("Right", [1.5, 0, 0]), ("Front", [0, 0, 1.5]),
                         ("Back", [0, 0, -1.5])]:
        s = box + f"let a = Sphere {{ radius: 0.5 }}.attach(b, {face});\nlet scene = b + a;\n"
        assert np.allclose(_pos(s), expect, atol=1e-6), face


def test_attach_by_corner_and_by_own_anchor():
    box = "let b = Box { size: vec3(2.0, 2.0, 2.0) };\n"
    # A corner moves the object's same corner onto the other's: the sphere's
    # back-right-bottom corner (r, -r, -r) lands on (1, -1, -1).
    s = box + "let a = Sphere { radius: 0.5 }.attach(b, BackRightCorner);\nlet scene = b + a;\n"
    assert np.allclose(_pos(s), [0.5, -0.5, -0.5], atol=1e-6)
    # attach(other, Top, Bottom): the sphere's bottom point onto the box's top.
    s = box + "let a = Sphere { radius: 0.5 }.attach(b, Top, Bottom);\nlet scene = b + a;\n"
    assert np.allclose(_pos(s), [0.0, 1.5, 0.0], atol=1e-6)


def test_align_and_relative_placement():
    box = "let b = Box { size: vec3(2.0, 2.0, 2.0), pos: vec3(3.0, 1.0, -2.0) };\n"
    cases = {
        "align_x(b, Center)": [3.0, 0, 0], "align_y(b, Top)": [0, 1.5, 0], "align_z(b, Back)": [0, 0, -2.5],
        "align_x(b, Left + 0.2)": [2.7, 0, 0],
        "right_of(b, 0.1)": [4.6, 0, 0], "left_of(b, 0.1)": [1.4, 0, 0],
        "on_top_of(b, 0.0)": [0, 2.5, 0], "below(b, 0.0)": [0, -0.5, 0],
        "in_front_of(b, 0.2)": [0, 0, -0.3], "behind(b, 0.2)": [0, 0, -3.7],
    }
    for call, expect in cases.items():
        s = box + f"let a = Sphere {{ radius: 0.5 }}.{call};\nlet scene = b + a;\n"
        assert np.allclose(_pos(s), expect, atol=1e-5), call


def test_offset_and_rotate_set_fields():
    s = "let a = Sphere { radius: 0.5, pos: vec3(1.0, 2.0, 3.0) }.offset_x(0.5).offset_z(-1.0);\nlet scene = a;\n"
    assert np.allclose(_pos(s), [1.5, 2.0, 2.0], atol=1e-6)
    # rotate_* sets one angle (it does not add to it).
    s = "let a = Box { size: vec3(1.0), rot: vec3(5.0, 6.0, 7.0) }.rotate_z(10.0).rotate_z(30.0);\nlet scene = a;\n"
    (c, r), = _placed(s)
    assert np.allclose(r, [5.0, 6.0, 30.0], atol=1e-6)


def test_rotated_box_bounds_use_its_turned_corners():
    """A 2x1x1 box turned 90 degrees about z spans 1 in x and 2 in y."""
    s = ("let b = Box { size: vec3(2.0, 1.0, 1.0), rot: vec3(0.0, 0.0, 90.0) };\n"
         "let a = Sphere { radius: 0.25 }.on_top_of(b, 0.0).right_of(b, 0.0);\nlet scene = b + a;\n")
    assert np.allclose(_pos(s), [0.75, 1.25, 0.0], atol=1e-5)


def test_composite_bounds():
    pair = ("let l = Sphere { radius: 1.0, pos: vec3(-2.0, 0.0, 0.0) };\n"
            "let r = Sphere { radius: 0.5, pos: vec3(3.0, 1.0, 0.0) };\n")
    for expr, top in [("l + r", 1.5), ("l.union_round(r, 0.2)", 1.5), ("l - r", 1.0), ("l.mirror_x()", 1.0),
                      ("l.repeat_y(4.0, 3)", 5.0), ("l.slice_y(-0.5, 0.25)", 0.25), ("l.smooth(2.0)", 1.2)]:
        s = pair + f"let g = {expr};\nlet a = Sphere {{ radius: 0.1 }}.attach(g, Top);\nlet scene = g + a;\n"
        assert abs(_pos(s)[1] - (top + 0.1)) < 1e-5, expr


CUSTOM = """
sdf Shelf {
  let depth = 0.4;
  let anchors = { TopSurface: vec3(0.0, 0.5, 0.0) };
  fn bounds() {
    return vec3(1.0, 0.5, depth);
  }
  fn distance(p) {
    let q = abs(p) - vec3(1.0, 0.5, depth);
    return length(max(q, vec3(0.0))) + min(max(q.x, max(q.y, q.z)), 0.0);
  }
};
"""


def test_custom_sdf_bounds_and_anchors():
    """A custom sdf instance carries its bounds() (with instance overrides)
    and its `anchors` binding for layout."""
    s = CUSTOM + ("let shelf = Shelf { pos: vec3(0.0, 1.0, 0.0), depth: 0.8 };\n"
                  "let a = Sphere { radius: 0.25 }.attach(shelf, \"TopSurface\", Bottom);\n"
                  "let c = Sphere { radius: 0.25 }.attach(shelf, Front);\n"
                  "let scene = shelf + a + c;\n")
    (pa, _), (pc, _) = _placed(s, kinds=(_native.FT_NODE_SPHERE,))
    assert np.allclose(pa, [0.0, 1.75, 0.0], atol=1e-6)
    assert np.allclose(pc, [0.0, 0.0, 0.8 + 0.25], atol=1e-6)  # a face moves one axis only


def test_face_to_sets_pitch_and_yaw():
    s = ("let t = Sphere { radius: 0.5, pos: vec3(3.0, 4.0, 3.0) };\n"
         "let a = Box { size: vec3(1.0) }.face_to(t);\nlet scene = a + t;\n")
    (c, r), _ = _placed(s)
    assert abs(r[1] - 45.0) < 1e-4
    assert abs(r[0] - math.degrees(math.atan2(-4.0, math.hypot(3.0, 3.0)))) < 1e-4


def test_layout_errors():
    with pytest.raises(ft.EvalError, match="layout operation requires bounded object values"):
        ft.parse_and_eval("let a = Sphere { radius: 0.5 }.attach(Cylinder { radius: 1.0 }, Top);\nlet scene = a;\n")
    with pytest.raises(ft.EvalError, match="call on unsupported callee"):
        ft.parse_and_eval("let b = Sphere {};\nlet a = Sphere { radius: 0.5 }.right_of(b, Top);\nlet scene = a;\n")
    with pytest.raises(ft.RenderError) as e:
        ft.parse_and_eval("let b = Sphere {};\nlet a = Sphere { radius: 0.5 }.bind(b);\nlet scene = a;\n")
    assert e.value.status == _native.FT_ERR_UNSUPPORTED


def test_boolean_example_layout():
    """The layout of the reference's boolean examples' base scene: a sphere
    set on the floor, a box placed right of it, lifted 0.3 above the floor
    and turned."""
    s = FLOOR + ("var a = Sphere { radius: 0.82 }\n  .attach(floor, Top)\n  .align_z(floor, Center)\n"
                 "  .offset_x(-0.28);\n"
                 "var b = Box { size: vec3(1.15, 1.15, 1.15) }\n  .right_of(a, -0.8)\n  .align_z(a, Center)\n"
                 "  .attach(floor, Top + 0.3)\n  .rotate_z(10.0);\nlet scene = floor + (a + b);\n")
    (_, _), (pa, _), (pb, rb) = _placed(s)
    assert np.allclose(pa, [-0.28, -0.08, 0.0], atol=1e-6)
    assert np.allclose(pb, [-0.28 + 0.82 - 0.8 + 0.575, -0.9 + 0.3 + 0.575, 0.0], atol=1e-6)
    assert np.allclose(rb, [0.0, 0.0, 10.0])
