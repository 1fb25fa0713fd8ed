"""The reference renderer's own unit tests (crates/forgedthoughts/src/renderer.rs,
`mod tests`), and those of crates/forgedthoughts/src/lib.rs whose values reach
the scene description, one by one under their names, on the CPU.  Where the reference
builds an `EvalState` by hand the same bindings are written as `.ft` source.
Renders go through the oracle, on the scene description the GPU library
consumes; material resolution goes through the lowered materials and hook
programs.  The GPU renders of these descriptions are covered by the parity
tests against the oracle."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import _native


def _depth_rgb8(st, width, height, accel=ft.AccelMode.Naive):
    _, _, _, rgb, _ = oracle.render_depth(st, ft.RenderOptions(width=width, height=height), accel, 1, 32)
    return rgb


def _root_material(st):
    d = st.desc
    return _native.MaterialC.from_buffer_copy(d.materials[d.nodes[d.root].material_id])


def _hook_args(position, local_position, normal=(0.0, 1.0, 0.0), view=(0.0, 0.0, 1.0)):
    a = np.zeros((1, 7, 3), np.float32)
    a[0, 0], a[0, 1], a[0, 2], a[0, 3] = position, local_position, normal, view
    a[0, 4] = a[0, 5] = a[0, 6] = 1  # front_face, object_id, material_id
    return a


def test_renders_depth_png_for_simple_sphere_scene(tmp_path):
    st = ft.parse_and_eval("var s = Sphere { x: 0.0, y: 0.0, z: 0.0 };")
    rgb = _depth_rgb8(st, 64, 64)
    out = tmp_path / "forgedthoughts-render-test.png"
    ft.write_png(out, rgb)
    assert out.stat().st_size > 0
    assert np.array_equal(ft.read_png(out), rgb)


def test_renders_non_black_for_offset_sphere():
    st = ft.parse_and_eval("var s = Sphere { x: 10.0, y: 0.0, z: 0.0 };")
    assert (_depth_rgb8(st, 64, 64) > 0).any()


def test_renders_with_all_accel_modes():
    st = ft.parse_and_eval("var s = Sphere { x: 1.0, y: 0.0, z: 0.0 };")
    images = [_depth_rgb8(st, 32, 32, mode) for mode in ft.AccelMode]
    assert (images[0] > 0).any()
    assert all(np.array_equal(images[0], im) for im in images[1:])


def test_uses_camera_and_lights_from_bindings():
    st = ft.parse_and_eval("""
        var s = Sphere {};
        let camera = Camera { origin: vec3(0.0, 0.0, 7.0), target: vec3(0.0, 0.0, 0.0), fov_y: 40.0 };
        let light_key = PointLight { position: vec3(2.0, 2.0, 4.0), color: vec3(1.0, 0.5, 0.25), intensity: 6.0 };
        let light_env = EnvLight { color: vec3(0.5, 0.5, 1.0), intensity: 0.08 };
    """)
    d = st.desc
    assert d.has_camera == 1 and list(d.camera.origin) == [0.0, 0.0, 7.0] and d.camera.fov_y_degrees == 40.0
    # lights in binding-name order, radiance = colour * intensity (render_api.rs:172-205)
    assert d.n_lights == 2
    env, key = d.lights[0], d.lights[1]
    assert env.kind == _native.FT_LIGHT_ENV and np.allclose(list(env.intensity), [0.04, 0.04, 0.08])
    assert key.kind == _native.FT_LIGHT_POINT and list(key.position) == [2.0, 2.0, 4.0]
    assert np.allclose(list(key.intensity), [6.0, 3.0, 1.5])
    assert (_depth_rgb8(st, 64, 64) > 0).any()


def test_traces_with_sphere_light():
    st = ft.parse_and_eval("""
        let scene = Sphere { radius: 0.9 };
        let camera = Camera { origin: vec3(0.0, 0.8, 5.0), target: vec3(0.0, 0.2, 0.0), fov_y: 35.0 };
        let key = SphereLight { position: vec3(2.0, 3.0, 3.5), radius: 0.7, color: vec3(1.0, 0.94, 0.86),
                                intensity: 40.0, samples: 4.0 };
    """)
    d = st.desc
    light = d.lights[0]
    assert d.n_lights == 1 and light.kind == _native.FT_LIGHT_SPHERE and light.samples == 4
    assert abs(light.radius - 0.7) < 1e-6
    opts = ft.RenderOptions(width=48, height=48, max_steps=320, max_dist=30.0, epsilon=0.0002, step_scale=0.7,
                            camera_z=6.0, fov_y_degrees=35.0)
    _, rgb8, _ = oracle.render_trace(st, opts, ft.AccelMode.Naive, 1, 2, 32)
    assert (rgb8 != 0).any()


def test_extracts_render_settings_from_bindings():
    """The path-tracer settings of the same binding (spp, bounces, min_spp,
    noise_threshold) belong to the progressive path tracer, which this
    library does not provide, and are not extracted."""
    st = ft.parse_and_eval("""
        let render = RenderSettings { width: 640, height: 360, max_steps: 180, max_dist: 60.0, epsilon: 0.0005,
          step_scale: 0.7, camera_z: 9.0, fov_y: 50.0, spp: 64, bounces: 8, min_spp: 12, noise_threshold: 0.025,
          accel: Bvh {} };
        let scene = Sphere {};
    """)
    s = ft.extract_scene_render_settings(st)
    assert (s.width, s.height, s.max_steps) == (640, 360, 180)
    assert s.max_dist == 60.0 and s.epsilon == np.float32(0.0005) and s.step_scale == np.float32(0.7)
    assert s.camera_z == 9.0 and s.fov_y_degrees == 50.0 and s.accel == ft.AccelMode.Bvh


def test_extracts_legacy_material_as_dielectric_from_scene_object():
    m = _root_material(ft.parse_and_eval("""
        var s = Sphere { material: Material {
          roughness: 0.2, metallic: 0.7, specular: 0.9, specular_weight: 0.8, specular_color: vec3(0.7, 0.8, 0.9),
          ior: 1.65, clearcoat: 0.3, clearcoat_roughness: 0.12, transmission: 0.55, thin_walled: 1.0,
          anisotropy: -0.25, anisotropy_rotation: 0.33, emission_color: vec3(0.1, 0.2, 0.3),
          emission_strength: 3.0, base_color: vec3(0.9, 0.5, 0.2) } };
    """))
    assert m.kind == _native.FT_MAT_STANDARD
    assert abs(m.roughness - 0.2) < 1e-6 and abs(m.ior - 1.65) < 1e-6 and m.thin_walled == 1
    assert abs(m.transmission - 0.55) < 1e-6 and abs(m.clearcoat - 0.3) < 1e-6
    assert abs(m.emission_color[1] - 0.2) < 1e-6 and abs(m.emission_strength - 3.0) < 1e-6
    assert abs(m.color[0] - 0.9) < 1e-6


def test_parses_lambert_material_constructor():
    m = _root_material(ft.parse_and_eval("""
        let scene = Sphere { material: Lambert { color: vec3(0.6, 0.4, 0.2), emission_color: vec3(0.0, 0.1, 0.0),
                                                 emission_strength: 2.0 } };
    """))
    assert m.kind == _native.FT_MAT_LAMBERT and abs(m.color[0] - 0.6) < 1e-6
    assert abs(m.emission_color[1] - 0.1) < 1e-6 and abs(m.emission_strength - 2.0) < 1e-6


def test_parses_metal_material_constructor():
    m = _root_material(ft.parse_and_eval(
        "let scene = Sphere { material: Metal { color: vec3(0.8, 0.7, 0.6), roughness: 0.35 } };"))
    assert m.kind == _native.FT_MAT_METAL and abs(m.color[0] - 0.8) < 1e-6 and abs(m.roughness - 0.35) < 1e-6


def test_parses_dielectric_material_constructor():
    m = _root_material(ft.parse_and_eval("""
        let scene = Sphere { material: Dielectric { color: vec3(0.95, 0.97, 1.0), ior: 1.52, roughness: 0.02,
                                                    thin_walled: 1.0 } };
    """))
    assert m.kind == _native.FT_MAT_DIELECTRIC and abs(m.color[0] - 0.95) < 1e-6
    assert abs(m.ior - 1.52) < 1e-6 and abs(m.roughness - 0.02) < 1e-6 and m.thin_walled == 1


def test_parses_material_fields_computed_from_ft_expressions():
    m = _root_material(ft.parse_and_eval("""
        let tint = mix(vec3(0.9, 0.7, 0.25), vec3(1.0), 0.2);
        let polish = clamp(0.08 + 0.04 * 2.0, 0.0, 1.0);
        let glow = max(0.5, 0.2 * 4.0);
        let material = Metal {
          color: tint,
          roughness: polish,
          emission_color: vec3(glow * 0.1, glow * 0.08, glow * 0.04),
          emission_strength: glow - 0.5
        };
        let scene = Sphere { material: material };
    """))
    assert m.kind == _native.FT_MAT_METAL
    assert np.allclose(list(m.color), [0.92, 0.76, 0.4], atol=1e-6) and abs(m.roughness - 0.16) < 1e-6
    assert np.allclose(list(m.emission_color), [0.08, 0.064, 0.032], atol=1e-6)
    assert abs(m.emission_strength - 0.3) < 1e-6


def test_resolves_material_local_helper_functions_across_hooks():
    """Colour and roughness hooks sharing a helper function.  The
    definition's `fn normal(ctx)` hook is not lowered."""
    st = ft.parse_and_eval("""
        material Brick {
          model: Lambert;
          let brick = vec3(0.68, 0.24, 0.16);
          let mortar = vec3(0.8, 0.77, 0.72);
          fn mortar_mask(ctx) {
            let band_x = smoothstep(-0.12, 0.12, sin(ctx.local_position.x * 11.0));
            let band_y = smoothstep(-0.12, 0.12, sin(ctx.local_position.y * 7.0));
            return max(band_x, band_y);
          }
          fn color(ctx) { return mix(brick, mortar, mortar_mask(ctx)); }
          fn roughness(ctx) { return mix(0.7, 0.95, mortar_mask(ctx)); }
          fn normal(ctx) {
            let m = mortar_mask(ctx);
            return normalize(ctx.normal + vec3(m * 0.2, 0.0, 0.0));
          }
        };
        let scene = Sphere { material: Brick {} };
    """)
    m = _root_material(st)
    assert m.kind == _native.FT_MAT_STANDARD and m.color_program >= 0 and m.roughness_program >= 0
    args = _hook_args((0.1, 0.1, 1.0), (0.1, 0.1, 1.0), normal=(0.0, 0.0, 1.0))
    assert oracle.eval_program(st, m.color_program, args)[0, 0] > 0.7
    assert oracle.eval_program(st, m.roughness_program, args)[0, 0] > 0.8


def test_resolves_dynamic_material_instance_overrides():
    st = ft.parse_and_eval("""
        material CheckerFloor {
          model: Lambert;
          roughness = 1.0;
          let color_a = #f1f3f6;
          let color_b = #6f7784;
          let scale = 3.4;
          fn checker(p, scale) {
            let sx = step(0.0, sin(p.x * scale));
            let sz = step(0.0, sin(p.z * scale));
            return abs(sx - sz);
          }
          fn color(ctx) {
            let m = checker(ctx.local_position, scale);
            return mix(color_a, color_b, m);
          }
        };
        let scene = Box { size: vec3(4.0, 0.5, 4.0),
                          material: CheckerFloor { color_a: #ff0000, color_b: #0000ff, scale: 3.1415926535 } };
    """)
    m = _root_material(st)
    assert m.kind == _native.FT_MAT_STANDARD and m.color_program >= 0
    a = oracle.eval_program(st, m.color_program, _hook_args((0.25, 0.25, 0.0), (0.25, 0.25, 0.0)))[0]
    b = oracle.eval_program(st, m.color_program, _hook_args((1.25, 0.25, 0.0), (1.25, 0.25, 0.0)))[0]
    assert a[0] > b[0] and b[2] > a[2]
    assert abs(a[0] - b[0]) > 0.2 and abs(b[2] - a[2]) > 0.2


def test_renders_cylinder_torus_and_extruded_polygon_with_rotation():
    st = ft.parse_and_eval("""
        let cylinder = Cylinder { radius: 0.7, height: 2.2, rot: vec3(20.0, 0.0, 15.0) };
        let torus = Torus { major_radius: 1.6, minor_radius: 0.25, y: 0.4 };
        let polygon = ExtrudePolygon { sides: 6.0, radius: 0.75, height: 0.6, x: -1.2, y: -0.2 };
        let scene = cylinder + torus + polygon;
    """)
    d = st.desc
    kinds = {d.nodes[i].kind for i in range(d.n_nodes)}
    assert {_native.FT_NODE_CYLINDER, _native.FT_NODE_TORUS, _native.FT_NODE_EXTRUDE_POLYGON} <= kinds
    assert (_depth_rgb8(st, 96, 96) > 0).any()


def test_resolves_environment_color_on_miss():
    st = ft.parse_and_eval("""
        environment Sky {
          let zenith = #4d74c7;
          let horizon = #d8e7ff;
          fn color(dir) {
            let t = clamp(dir.y * 0.5 + 0.5, 0.0, 1.0);
            return mix(horizon, zenith, t);
          }
        };
        let scene = Sphere { radius: 1.0 };
    """)
    d = st.desc
    assert d.environment_program >= 0
    sky = oracle.eval_program(st, d.environment_program, np.array([[[0.0, 1.0, 0.0]]], np.float32))[0]
    assert sky[2] > sky[0]


# ---- crates/forgedthoughts/src/lib.rs tests whose values reach the scene description

def test_supports_primitive_round_fields():
    st = ft.parse_and_eval("let b = Box { size: vec3(1.0, 2.0, 3.0), round: 0.1 };")  # owns the description
    d = st.desc
    n = d.nodes[d.root]
    assert n.kind == _native.FT_NODE_BOX and list(n.f[:3]) == [0.5, 1.0, 1.5] and abs(n.f[3] - 0.1) < 1e-7


def test_supports_nested_transform_assignments():
    st = ft.parse_and_eval("var s = Sphere{}; s.pos.x = 1.5; s.pos.y = -0.25; s.rot.z = 30.0;")
    d = st.desc
    n = d.nodes[d.root]
    assert list(n.center) == [1.5, -0.25, 0.0] and list(n.rot_deg) == [0.0, 0.0, 30.0]


@pytest.mark.parametrize("expr,kind,params", [
    ("a & b", 9, ()),                        # FT_NODE_INTERSECT
    ("a.union_round(b, 0.2)", 11, (0.2,)),   # FT_NODE_UNION_ROUND, r
    ("a.diff_stairs(b, 0.3, 5.0)", 23, (0.3, 5.0)),  # FT_NODE_DIFF_STAIRS, r and n
])
def test_supports_intersection_and_boolean_variant_calls(expr, kind, params):
    st = ft.parse_and_eval(f"var a = Sphere{{}}; var b = Box {{ size: vec3(1.0) }}; let scene = {expr};")
    d = st.desc
    n = d.nodes[d.root]
    assert n.kind == kind and np.allclose(list(n.f[:len(params)]), params, atol=1e-7)
    assert d.nodes[n.a].kind == _native.FT_NODE_SPHERE and d.nodes[n.b].kind == _native.FT_NODE_BOX


def test_material_properties_accept_instance_overrides():
    m = _root_material(ft.parse_and_eval("""
        material Checker {
          model: Lambert;
          let color_a = #ffffff;
          let scale = 3.4;
          color = color_a;
          roughness = scale / 10.0;
        };
        let scene = Sphere { material: Checker { color_a: vec3(0.2, 0.4, 0.6), scale: 6.0 } };
    """))
    assert np.allclose(list(m.color), [0.2, 0.4, 0.6], atol=1e-6) and abs(m.roughness - 0.6) < 1e-6


def test_sdf_functions_accept_instance_overrides():
    st = ft.parse_and_eval("""
        sdf SoftBlob {
          let radius = 1.0;
          let warp_frequency = 4.0;
          let warp_amount = 0.16;
          fn bounds() {
            return vec3(radius + 0.2, radius + warp_amount + 0.2, radius + 0.1);
          }
          fn warp(p) {
            return vec3(p.x, p.y + sin(p.x * warp_frequency) * warp_amount, p.z);
          }
          fn distance(p) {
            let q = warp(p);
            return length(q) - radius;
          }
        };
        let scene = SoftBlob { radius: 2.0, warp_frequency: 3.1415926535, warp_amount: 0.0 };
    """)
    d = st.desc
    n = d.nodes[d.root]
    assert n.kind == _native.FT_NODE_CUSTOM
    assert abs(n.f[0] - 2.2) < 1e-6 and abs(n.f[1] - 2.2) < 1e-6
    dist = oracle.eval_program(st, n.program, np.array([[[2.0, 0.0, 0.0]]], np.float32))[0, 0]
    assert abs(dist) < 1e-6


def test_supports_object_level_modifier_function_assignments():
    """Assigned `domain` / `distance_post` functions become modifier nodes
    with their hook programs (the F8 double transform keeps both)."""
    st = ft.parse_and_eval("""
        var statue = Box { size: vec3(1.0, 2.0, 1.0) };
        statue.domain = fn(p) {
          return rotate_y(p, p.y * 10.0);
        };
        statue.distance_post = fn(d, p) {
          return abs(d + sin(p.y * 20.0) * 0.01) - 0.02;
        };
        let scene = statue;
    """)
    d = st.desc
    kinds = {d.nodes[i].kind: d.nodes[i] for i in range(d.n_nodes)}
    assert 5 in kinds and 6 in kinds  # FT_NODE_DOMAIN, FT_NODE_DISTANCE_POST
    assert kinds[5].program >= 0 and kinds[6].program >= 0
    post = oracle.eval_program(st, kinds[6].program, np.array([[[0.2, 0.0, 0.0], [0.0, 0.0, 0.0]]], np.float32))
    assert abs(post[0, 0] - 0.18) < 1e-6  # abs(0.2 + sin(0) * 0.01) - 0.02


def test_jits_scalar_material_hook_with_ctx_members():
    """The reference checks the value is finite; it is also the closed form
    mix(0.08, 0.32, smoothstep(-0.2, 0.2, sin(3)))."""
    st = ft.parse_and_eval("""
        material Stripe {
          model: Metal;
          fn roughness(ctx) {
            let phase = sin(ctx.local_position.y * 12.0);
            let mask = smoothstep(-0.2, 0.2, phase);
            return mix(0.08, 0.32, mask);
          }
        };
        let scene = Sphere { material: Stripe {} };
    """)
    m = _root_material(st)
    assert m.kind == _native.FT_MAT_METAL and m.roughness_program >= 0
    v = oracle.eval_program(st, m.roughness_program, _hook_args((0.0, 0.25, 0.0), (0.0, 0.25, 0.0)))[0, 0]
    t = min(max((np.sin(3.0) + 0.2) / 0.4, 0.0), 1.0)
    assert np.isfinite(v) and abs(v - (0.08 + 0.24 * t * t * (3 - 2 * t))) < 1e-5


def test_material_functions_accept_instance_overrides():
    st = ft.parse_and_eval("""
        material Checker {
          model: Lambert;
          let color_a = #ffffff;
          let color_b = #000000;
          let scale = 3.4;
          fn checker(p, scale) {
            let sx = step(0.0, sin(p.x * scale));
            let sz = step(0.0, sin(p.z * scale));
            return abs(sx - sz);
          }
          fn color(ctx) {
            let m = checker(ctx.local_position, scale);
            return mix(color_a, color_b, m);
          }
        };
        let scene = Sphere { material: Checker { color_a: vec3(1.0, 0.0, 0.0), color_b: vec3(0.0, 0.0, 1.0),
                                                 scale: 3.1415926535 } };
    """)
    m = _root_material(st)
    a = oracle.eval_program(st, m.color_program, _hook_args((0.5, 0.0, 0.0), (0.5, 0.0, 0.0)))[0]
    b = oracle.eval_program(st, m.color_program, _hook_args((1.5, 0.0, 0.0), (1.5, 0.0, 0.0)))[0]
    assert a[0] > 0.9 and a[2] < 0.1 and b[2] > 0.9 and b[0] < 0.1


def test_evaluates_environment_function():
    """The environment colour straight up is the zenith colour: the reference
    checks blue > 0.7; the hex literal #4d74c7 is (77, 116, 199) / 255."""
    st = ft.parse_and_eval("""
        environment Sky {
          let zenith = #4d74c7;
          let horizon = #d8e7ff;
          fn color(dir) {
            let t = clamp(dir.y * 0.5 + 0.5, 0.0, 1.0);
            return mix(horizon, zenith, t);
          }
        };
        let scene = Sphere {};
    """)
    d = st.desc
    c = oracle.eval_program(st, d.environment_program, np.array([[[0.0, 1.0, 0.0]]], np.float32))[0]
    assert c[2] > 0.7
    assert np.allclose(c, np.array([77, 116, 199], np.float32) / np.float32(255), atol=1e-6)
