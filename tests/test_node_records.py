"""A scene handed over as `ft_node` records instead of `.ft` source: the form
a host that already holds the reference's evaluated scene (`EvalState` with
its `SdfNode` tree, renderer.rs:171-355) would pass, lowering each node to one
record.  The records here are written by hand from the scene's meaning; the
library must build and render them exactly as it does the same scene parsed
from source."""
import ctypes

import numpy as np
import pytest

import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native

SOURCE = """let camera = Camera { origin: vec3(0, 1, -5), target: vec3(0, 0, 0), fov_y: 45.0 };
var ground = Box { size: vec3(220, 1, 220) };
ground.pos.y = -0.5;
let a = Sphere { radius: 0.5, pos: vec3(-0.6, 0.5, 0.2) };
var b = Box { size: vec3(0.6, 0.6, 0.6), pos: vec3(0.6, 0.4, 0.0) };
b.rot.y = 30.0;
let light = PointLight { position: vec3(3, 6, -3), intensity: 60.0 };
let scene = ground + a.union_round(b, 0.2);
"""


def _node(kind, a=-1, b=-1, obj=0, center=(0, 0, 0), rot=(0, 0, 0), f=()):
    n = _native.NodeC()
    n.kind, n.a, n.b, n.program, n.object_id, n.material_id = kind, a, b, -1, obj, 0
    n.center[:] = [float(x) for x in center]
    n.rot_deg[:] = [float(x) for x in rot]
    n.f[:] = [float(x) for x in f] + [0.0] * (6 - len(f))
    return n


def hand_built_desc():
    """SdfNode -> ft_node by hand: Box (half size), Sphere (radius), Box with a
    y rotation in degrees, UnionRound(r), Union; one default material, one
    point light, the camera."""
    nodes = (_native.NodeC * 5)(
        _node(_native.FT_NODE_BOX, obj=1, center=(0, -0.5, 0), f=(110, 0.5, 110)),
        _node(_native.FT_NODE_SPHERE, obj=2, center=(-0.6, 0.5, 0.2), f=(0.5,)),
        _node(_native.FT_NODE_BOX, obj=3, center=(0.6, 0.4, 0.0), rot=(0, 30, 0), f=(0.3, 0.3, 0.3)),
        _node(_native.FT_NODE_UNION_ROUND, a=1, b=2, f=(0.2,)),
        _node(_native.FT_NODE_UNION, a=0, b=3))
    mats = (_native.MaterialC * 1)()
    m = mats[0]
    # the default material (Standard, MaterialParams defaults)
    m.kind, m.color[:], m.roughness, m.ior, m.specular, m.specular_weight = (
        _native.FT_MAT_STANDARD, [0.8, 0.8, 0.8], 0.5, 1.5, 0.5, 1.0)
    m.specular_color[:] = [1.0, 1.0, 1.0]
    m.clearcoat_roughness = 0.1
    m.color_program = m.roughness_program = m.ior_program = m.thin_walled_program = -1
    m.hook_program[:] = [-1] * _native.FT_MATERIAL_HOOK_SLOTS
    lights = (_native.LightC * 1)()
    lights[0].kind, lights[0].samples = _native.FT_LIGHT_POINT, 1
    lights[0].position[:] = [3.0, 6.0, -3.0]
    lights[0].intensity[:] = [60.0, 60.0, 60.0]
    d = _native.SceneDescC()
    d.abi_version = _native.FT_ABI_VERSION
    d.root, d.nodes, d.n_nodes = 4, ctypes.cast(nodes, ctypes.POINTER(_native.NodeC)), 5
    d.materials, d.n_materials = ctypes.cast(mats, ctypes.POINTER(_native.MaterialC)), 1
    d.lights, d.n_lights = ctypes.cast(lights, ctypes.POINTER(_native.LightC)), 1
    d.environment_program = -1
    d.camera.origin[:], d.camera.target[:], d.camera.up[:] = [0.0, 1.0, -5.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0]
    d.camera.fov_y_degrees, d.has_camera = 45.0, 1
    d.settings_accel = -1
    return d, (nodes, mats, lights)  # keep the arrays alive


def test_hand_built_records_build_like_source():
    d, keep = hand_built_desc()
    info = _native.BuildInfoC()
    assert _native.lib().ft_scene_build_info(ctypes.byref(d), ctypes.byref(info)) == 0, _native.last_error()
    st = ft.parse_and_eval(SOURCE)
    ref = _native.BuildInfoC()
    assert _native.lib().ft_scene_build_info(st.desc_ptr, ctypes.byref(ref)) == 0
    for f in ("leaves", "primitive_leaves", "union_round_leaves", "generic_leaves", "bvh_nodes"):
        assert getattr(info, f) == getattr(ref, f), f


@pytest.mark.gpu
def test_hand_built_records_render_like_source():
    d, keep = hand_built_desc()
    lib = _native.lib()
    h = ctypes.c_void_p()
    assert lib.ft_scene_create(ctypes.byref(d), ctypes.byref(h)) == 0, _native.last_error()
    st = ft.parse_and_eval(SOURCE)
    opts = ft.RenderOptions(width=128, height=96, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    o = opts.to_c()
    w, hh = opts.width, opts.height
    t = np.empty(w * hh, np.float32)
    mask = np.empty(w * hh, np.uint8)
    rgb = np.empty(w * hh * 3, np.float32)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    assert lib.ft_render_depth(h, ctypes.byref(o), 1, 1, p(t), p(mask), None, None, None, 0, None) == 0
    assert lib.ft_render_trace(h, ctypes.byref(o), 1, 1, 3, p(rgb), None, 0, None) == 0
    lib.ft_scene_destroy(h)
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 3)
    assert 0.2 < mask.mean() < 0.95
    assert np.array_equal(mask.reshape(hh, w), img.mask[..., 0])
    assert np.array_equal(t.reshape(hh, w), img.t[..., 0])
    # radiance sums with float atomics in a varying order: last bits only
    assert np.allclose(rgb.reshape(hh, w, 3), lin, rtol=1e-5, atol=1e-6)
