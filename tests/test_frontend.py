"""`.ft` front-end: the reference's own parse/eval error fixtures, hook KATs,
scene lowering details (lights, camera, settings, modifiers)."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from conftest import FIXTURES
from forgedthoughts_gb300 import _native, workloads


@pytest.mark.parametrize("name", sorted(p.stem for p in (FIXTURES / "parse_err").glob("*.ft")))
def test_parse_error_fixtures(name):
    src = (FIXTURES / "parse_err" / f"{name}.ft").read_text()
    want = (FIXTURES / "parse_err" / f"{name}.err").read_text().strip()
    with pytest.raises(ft.ParseError) as e:
        ft.parse_and_eval(src)
    assert str(e.value) == want


@pytest.mark.parametrize("name", sorted(p.stem for p in (FIXTURES / "eval_err").glob("*.ft")))
def test_eval_error_fixtures(name):
    src = (FIXTURES / "eval_err" / f"{name}.ft").read_text()
    want = (FIXTURES / "eval_err" / f"{name}.err").read_text().strip()
    with pytest.raises(ft.RenderError) as e:
        ft.parse_and_eval(src + "\nlet scene = Sphere {};\n")
    assert str(e.value) == want


def test_missing_scene_root():
    with pytest.raises(ft.MissingSceneRoot):
        ft.parse_and_eval("let a = Sphere {};")


def test_unsupported_object_type():
    with pytest.raises(ft.UnsupportedObjectType):
        ft.parse_and_eval("let scene = Teapot {};")


def test_expected_object():
    with pytest.raises(ft.ExpectedObject):
        ft.parse_and_eval("let scene = 3.0;")


def test_distance_post_kat():
    # crates/forgedthoughts/src/lib.rs:1919: abs(d) - 0.05 at d = 0.2 is 0.15
    st = ft.parse_and_eval("let scene = Sphere { radius: 1.0, distance_post: fn(d, p) { return abs(d) - 0.05; } };")
    assert st.desc.n_programs == 1
    out = oracle.eval_program(st, 0, np.array([[[0.2, 0.2, 0.2], [0.0, 0.0, 0.0]]], np.float32))
    assert np.float32(out[0, 0]) == np.float32(0.15)


def test_hook_program_matches_builtin_semantics():
    src = ("let k = 3.0;\n"
           "let scene = Sphere { radius: 1.0, domain: fn(p) {\n"
           "  let q = rotate_y(p, p.y * 18.0);\n"
           "  return vec3(clamp(q.x, -1.0, 1.0), mix(q.y, k, 0.25), smoothstep(0.0, 1.0, q.z)) + normalize(p) * 0.5;\n"
           "} };")
    st = ft.parse_and_eval(src)
    rng = np.random.default_rng(3)
    p = rng.uniform(-2, 2, (64, 3)).astype(np.float32)
    got = oracle.eval_program(st, 0, p[:, None, :], precision=64)
    for i in range(len(p)):
        x, y, z = map(float, p[i])
        a = np.radians(y * 18.0)
        q = (np.cos(a) * x + np.sin(a) * z, y, -np.sin(a) * x + np.cos(a) * z)
        t = min(max(q[2], 0.0), 1.0)
        n = np.array([x, y, z]) / np.linalg.norm([x, y, z])
        want = np.array([min(max(q[0], -1), 1), q[1] * 0.75 + 3.0 * 0.25, t * t * (3 - 2 * t)]) + n * 0.5
        np.testing.assert_allclose(got[i], want, rtol=1e-6, atol=1e-6)


def test_scene_lowering_records_lights_camera_settings():
    src = (FIXTURES / "render_regression" / "ray_boolean_union_round.ft").read_text()
    src += "\nlet render = RenderSettings { width: 64, height: 48, max_steps: 99, accel: Bricks {} };\n"
    st = ft.parse_and_eval(src)
    d = st.desc
    assert d.n_lights == 2  # fill, key: ordered by binding name
    assert d.lights[0].kind == 0 and abs(d.lights[0].intensity[0] - 34.0 * 0xc9 / 255.0) < 1e-4
    assert d.has_camera == 1 and abs(d.camera.fov_y_degrees - 25.0) < 1e-6
    s = ft.extract_scene_render_settings(st)
    assert (s.width, s.height, s.max_steps, s.accel) == (64, 48, 99, ft.AccelMode.Bricks)
    assert d.environment_program >= 0


def test_union_round_tree_and_modifiers_lower():
    st = ft.parse_and_eval(workloads.union_round_field(n=16, width=8, height=8).source)
    kinds = [st.desc.nodes[i].kind for i in range(st.desc.n_nodes)]
    assert kinds.count(11) == 15  # union_round nodes
    st2 = ft.parse_and_eval(workloads.twisted_shells(n=4, width=8, height=8).source)
    kinds2 = [st2.desc.nodes[i].kind for i in range(st2.desc.n_nodes)]
    # one DOMAIN and one DISTANCE_POST wrapper per sphere, hooks compiled once
    assert kinds2.count(5) == 4 and kinds2.count(6) == 4 and st2.desc.n_programs == 2


def test_double_transform_of_domain_plus_distance_post():
    # Both hooks keep the primitive's transform (split_modifier_base, R:1750-1780).
    st = ft.parse_and_eval("let scene = Sphere { radius: 0.5, pos: vec3(1, 0, 0), "
                           "domain: fn(p) { return p; }, distance_post: fn(d, p) { return d; } };")
    d, _, _ = oracle.distance(st, np.array([[2.0, 0.0, 0.0]]), accel=0)
    # p - c applied twice: |2 - 1 - 1| - 0.5 = -0.5
    assert abs(d[0] + 0.5) < 1e-6


def test_mirror_and_repeat_expand():
    st = ft.parse_and_eval("let b = Sphere { radius: 0.25, pos: vec3(1, 0, 0) };\n"
                           "let scene = b.mirror_x().repeat_z(2.0, 3);")
    prims = [n for n in (st.desc.nodes[i] for i in range(st.desc.n_nodes)) if n.kind == 0]
    centers = sorted((round(p.center[0], 3), round(p.center[2], 3)) for p in prims)
    # the final copies are the remapped ones; each compile also leaves its base node
    assert (-1.0, -2.0) in centers and (1.0, 2.0) in centers and (-1.0, 0.0) in centers


def test_workload_generators_are_deterministic():
    a = workloads.union_round_field(n=32, width=16, height=16).source
    b = workloads.union_round_field(n=32, width=16, height=16).source
    assert a == b
    assert "e-" not in a and "e+" not in a  # the lexer has no exponent syntax


def _sphere_material(source: str):
    st = ft.parse_and_eval(source)
    d = st.desc
    sph = [d.nodes[i] for i in range(d.n_nodes) if d.nodes[i].kind == 0]
    assert len(sph) == 1
    return _native.MaterialC.from_buffer_copy(d.materials[sph[0].material_id])  # outlives the description


def test_material_definition_static_color_property():
    """The reference's resolves_ft_material_static_color_property
    (renderer.rs tests): a Lambert-model definition assigning `color` from a
    binding is a Standard material with that colour and the Lambert
    parameters (material_from_dynamic_def, R:6633-6690)."""
    m = _sphere_material("""
        material Solid {
          model: Lambert;
          let tint = vec3(0.24, 0.5, 0.82);
          color = tint;
        };
        let scene = Sphere { material: Solid {} };
    """)
    assert m.kind == _native.FT_MAT_STANDARD
    assert abs(m.color[0] - 0.24) < 1e-6 and abs(m.color[1] - 0.5) < 1e-6 and abs(m.color[2] - 0.82) < 1e-6
    assert m.roughness == 1.0 and m.metallic == 0.0 and abs(m.specular - 0.5) < 1e-7


def test_material_definition_properties_clamps_and_overrides():
    """Metal and Dielectric definitions keep their kind; properties are
    clamped as apply_dynamic_material_properties (R:6692-6770); an instance
    field replaces the binding of the same name (material_override_value,
    eval.rs:3761-3766)."""
    metal = _sphere_material("""
        material Brushed {
          model: Metal;
          color = vec3(0.8, 0.72, 0.3);
          roughness = 1.7;
        };
        let scene = Sphere { material: Brushed {} };
    """)
    assert metal.kind == _native.FT_MAT_METAL and metal.metallic == 1.0
    assert abs(metal.color[1] - 0.72) < 1e-6 and metal.roughness == 1.0
    glass = _sphere_material("""
        material Glass {
          model: Dielectric;
          ior = 5.0;
        };
        let scene = Sphere { material: Glass {} };
    """)
    assert glass.kind == _native.FT_MAT_DIELECTRIC and glass.ior == 3.0 and glass.transmission == 1.0
    over = _sphere_material("""
        material Solid {
          model: Standard;
          let tint = vec3(0.24, 0.5, 0.82);
          color = tint;
          metallic = 0.25;
        };
        let scene = Sphere { material: Solid { tint: vec3(0.1, 0.2, 0.3) } };
    """)
    assert over.kind == _native.FT_MAT_STANDARD and over.roughness == 0.5 and over.metallic == 0.25
    assert abs(over.color[0] - 0.1) < 1e-6 and abs(over.color[2] - 0.3) < 1e-6
    # Standard-model definitions get the coat of resolve_leaf_material
    # (R:7396-7470): IOR 1.33 and clearcoat roughness 0.08 by default
    assert abs(over.ior - 1.33) < 1e-6 and abs(over.clearcoat_roughness - 0.08) < 1e-6 and over.clearcoat == 0.0
    coat = _sphere_material("""
        material Coated {
          model: Standard;
          ior = 1.7;
          coat_ior = 1.5;
          coat_weight = 0.6;
          coat_color = vec3(0.9, 0.95, 1.0);
        };
        let scene = Sphere { material: Coated {} };
    """)
    assert abs(coat.ior - 1.5) < 1e-6 and abs(coat.clearcoat - 0.6) < 1e-6 and abs(coat.specular_color[1] - 0.95) < 1e-6


def test_material_medium_field():
    """The reference's parses_medium_and_subsurface_material_fields: a
    Dielectric's `medium: Medium {...}` field (medium_from_value,
    R:6834-6845) gives IOR 1.33, absorption blue 1.0 and density 0.35."""
    m = _sphere_material("""
        let scene = Sphere {
          material: Dielectric {
            color: vec3(0.96, 0.98, 1.0),
            ior: 1.52,
            medium: Medium {
              ior: 1.33,
              absorption_color: vec3(0.82, 0.91, 1.0),
              density: 0.35
            },
            subsurface: Subsurface {
              color: vec3(1.0, 0.58, 0.44),
              radius: vec3(0.8, 0.4, 0.22),
              anisotropy: 0.15,
              scale: 1.25
            }
          }
        };
    """)
    assert m.kind == _native.FT_MAT_DIELECTRIC and m.has_medium == 1
    assert abs(m.medium_ior - 1.33) < 1e-6 and abs(m.medium_absorption[2] - 1.0) < 1e-6
    assert abs(m.medium_absorption[0] - 0.82) < 1e-6 and abs(m.medium_density - 0.35) < 1e-6
    assert abs(m.ior - 1.52) < 1e-6


def test_material_medium_defaults_clamps_and_definitions():
    """Missing medium fields take medium_from_value's defaults and clamps
    (IOR 1 within [1, 3], white absorption, density >= 0); any model reads
    the field; a definition's `medium = ...` property is its static medium
    (apply_dynamic_material_properties, R:6761-6763); no field, no medium."""
    m = _sphere_material("let scene = Sphere { material: Lambert { medium: Medium { ior: 7.0, density: -2.0 } } };")
    assert m.kind == _native.FT_MAT_LAMBERT and m.has_medium == 1
    assert m.medium_ior == 3.0 and m.medium_density == 0.0 and list(m.medium_absorption) == [1.0, 1.0, 1.0]
    m = _sphere_material("let scene = Sphere { material: Metal { medium: Fog {} } };")
    assert m.kind == _native.FT_MAT_METAL and m.has_medium == 1 and m.medium_ior == 1.0
    m = _sphere_material("let scene = Sphere { material: Dielectric { medium: 0.5 } };")
    assert m.has_medium == 0
    m = _sphere_material("""
        material WaxedGlass {
          model: Dielectric;
          color = vec3(1.0);
          medium = Medium {
            ior: 1.33,
            absorption_color: vec3(0.9, 0.95, 1.0),
            density: 0.05
          };
        };
        let scene = Sphere { material: WaxedGlass {} };
    """)
    assert m.kind == _native.FT_MAT_DIELECTRIC and m.has_medium == 1
    assert abs(m.medium_ior - 1.33) < 1e-6 and abs(m.medium_absorption[1] - 0.95) < 1e-6
    assert abs(m.medium_density - 0.05) < 1e-6


def _hook_args(local_positions):
    a = np.zeros((len(local_positions), 7, 3), np.float32)
    for i, lp in enumerate(local_positions):
        a[i, 0] = a[i, 1] = lp            # position, local_position
        a[i, 2] = (0.0, 1.0, 0.0)         # normal
        a[i, 3] = (0.0, 0.0, 1.0)         # view_dir
        a[i, 4] = a[i, 5] = a[i, 6] = 1   # front_face, object_id, material_id
    return a


def test_checker_pattern_reference_known_answer():
    """The reference's resolves_checker_pattern_from_local_hit_position: a
    Lambert with a Checker3d pattern (scale 2) is colour_a at local
    (0.1, 0.1, 0.1) and colour_b at (0.6, 0.1, 0.1).  The pattern is lowered
    as the material's colour hook; its static colour stays the given one."""
    st = ft.parse_and_eval("""
        let material = Lambert {
          color: vec3(0.5),
          pattern: Checker3d { color_a: vec3(0.1, 0.2, 0.3), color_b: vec3(0.9, 0.8, 0.7), scale: 2.0 }
        };
        let scene = Sphere { material: material };
    """)
    d = st.desc
    m = d.materials[d.nodes[d.root].material_id]
    assert m.kind == _native.FT_MAT_LAMBERT and m.color_program >= 0 and list(m.color) == [0.5, 0.5, 0.5]
    c = oracle.eval_program(st, m.color_program, _hook_args([(0.1, 0.1, 0.1), (0.6, 0.1, 0.1)]))
    assert np.allclose(c[0], [0.1, 0.2, 0.3], atol=1e-6) and np.allclose(c[1], [0.9, 0.8, 0.7], atol=1e-6)
    # negative cells follow the integer parity of the floors: floor(-0.2) = -1 is odd
    c = oracle.eval_program(st, m.color_program, _hook_args([(-0.1, 0.1, 0.1), (-0.6, -0.6, 0.2)]))
    assert np.allclose(c[0], [0.9, 0.8, 0.7], atol=1e-6) and np.allclose(c[1], [0.1, 0.2, 0.3], atol=1e-6)
    # colours are exactly the given constants (a select, not a blend)
    assert np.array_equal(c.astype(np.float32)[1], np.array([0.1, 0.2, 0.3], np.float32))


def test_checker_pattern_defaults_aliases_and_sharing():
    """read_pattern_field's aliases (color1/color2, frequency) and defaults
    (0.15 / 0.85 grey, scale 4); every model takes a pattern; another pattern
    type is ignored; primitives with the same pattern share one program."""
    st = ft.parse_and_eval("""
        let a = Sphere { material: Metal { pattern: Checker { } } };
        let b = Sphere { pos: vec3(3, 0, 0), material: Dielectric { pattern: checker3d { color1: vec3(1, 0, 0),
                                                                               color2: vec3(0, 0, 1), frequency: 1.0 } } };
        let c = Sphere { pos: vec3(6, 0, 0), material: Metal { pattern: Checker { } } };
        let d = Sphere { pos: vec3(9, 0, 0), material: Lambert { pattern: Stripes { } } };
        let scene = a + b + c + d;
    """)
    d = st.desc
    sph = [d.nodes[i] for i in range(d.n_nodes) if d.nodes[i].kind == 0]
    mats = [d.materials[n.material_id] for n in sph]
    assert mats[0].kind == _native.FT_MAT_METAL and mats[0].color_program >= 0
    assert mats[2].color_program == mats[0].color_program and d.n_programs == 2
    assert mats[3].color_program == -1
    c = oracle.eval_program(st, mats[0].color_program, _hook_args([(0.1, 0.1, 0.1), (0.3, 0.1, 0.1)]))
    assert np.allclose(c, [[0.15] * 3, [0.85] * 3], atol=1e-6)  # scale 4: floor(1.2) = 1 is odd
    c = oracle.eval_program(st, mats[1].color_program, _hook_args([(0.5, 0.5, 0.5), (1.5, 0.5, 0.5)]))
    assert np.allclose(c, [[1, 0, 0], [0, 0, 1]], atol=1e-6)


def test_checker_pattern_renders_both_colours():
    """Traced through the oracle, a checkered sphere under a white sky shows
    pixels of both colours."""
    st = ft.parse_and_eval("""
        environment Sky { fn color(dir) { return vec3(1.0, 1.0, 1.0); } };
        let scene = Sphere { radius: 1.0, material: Lambert {
          pattern: Checker3d { color_a: vec3(1.0, 0.0, 0.0), color_b: vec3(0.0, 0.0, 1.0), scale: 3.0 } } };
    """)
    opts = ft.RenderOptions(width=32, height=32, max_steps=200, max_dist=20.0, epsilon=1e-4, camera_z=4.0)
    rgb, _, _ = oracle.render_trace(st, opts, 1, 1, 2, 32)
    hit = rgb[8:24, 8:24].reshape(-1, 3)
    reds = (hit[:, 0] > 0.05) & (hit[:, 2] < 0.01)
    blues = (hit[:, 2] > 0.05) & (hit[:, 0] < 0.01)
    assert reds.sum() > 20 and blues.sum() > 20, (reds.sum(), blues.sum())


HOOK_MATERIALS = """
material Stripe {
  model: Lambert;
  let warm = vec3(0.9, 0.72, 0.3);
  let dark = vec3(0.12, 0.14, 0.18);
  fn color(ctx) {
    let phase = sin(ctx.local_position.x * 8.0);
    let mask = step(0.0, phase);
    return mix(warm, dark, mask);
  }
};
material RoughStripe {
  model: Metal;
  color = vec3(0.8, 0.72, 0.3);
  roughness = 0.15;
  fn roughness(ctx) {
    let phase = sin(ctx.local_position.x * 6.0);
    let mask = step(0.0, phase);
    return mix(0.12, 0.48, mask);
  }
};
material RippleGlass {
  model: Dielectric;
  color = vec3(1.0);
  ior = 1.52;
  roughness = 0.02;
  thin_walled = 0.0;
  fn ior(ctx) {
    let phase = sin(ctx.local_position.x * 6.0);
    let mask = step(0.0, phase);
    return mix(1.45, 1.6, mask);
  }
  fn thin_walled(ctx) {
    let phase = sin(ctx.local_position.y * 6.0);
    return step(0.0, phase);
  }
};
"""


def _hook_ctx(pos):
    a = np.zeros((1, _native.FT_MATERIAL_HOOK_PARAMS, 3), np.float32)
    a[0, 0] = a[0, 1] = pos          # position; local_position (sphere at the origin)
    a[0, 2] = (0.0, 1.0, 0.0)        # normal
    a[0, 3] = (0.0, 0.0, 1.0)        # view_dir
    a[0, 4] = a[0, 5] = a[0, 6] = 1  # front_face, object_id, material_id
    return a


def _materials_of(st):
    d = st.desc
    return {int(d.materials[i].kind): _native.MaterialC.from_buffer_copy(d.materials[i])
            for i in range(d.n_materials)}


@pytest.mark.parametrize("material,kind", [("Stripe", "FT_MAT_STANDARD"), ("RoughStripe", "FT_MAT_METAL"),
                                           ("RippleGlass", "FT_MAT_DIELECTRIC")])
def test_material_hooks_reference_known_answers(material, kind):
    """The reference's resolves_ft_material_color_from_local_hit_position,
    resolves_ft_material_dynamic_roughness_hook and
    resolves_ft_material_dynamic_dielectric_hooks (renderer.rs tests): the
    lowered hook programs evaluated on the same hits."""
    st = ft.parse_and_eval(HOOK_MATERIALS + f"let scene = Sphere {{ material: {material} {{}} }};\n")
    m = _materials_of(st)[getattr(_native, kind)]
    if material == "Stripe":
        assert m.roughness_program < 0 and m.ior_program < 0
        warm = oracle.eval_program(st, m.color_program, _hook_ctx((-0.1, 0.0, 0.0)))[0]
        dark = oracle.eval_program(st, m.color_program, _hook_ctx((0.1, 0.0, 0.0)))[0]
        assert np.allclose(warm, (0.9, 0.72, 0.3), atol=1e-6) and np.allclose(dark, (0.12, 0.14, 0.18), atol=1e-6)
    elif material == "RoughStripe":
        assert m.color_program < 0 and abs(m.color[0] - 0.8) < 1e-6
        smooth = oracle.eval_program(st, m.roughness_program, _hook_ctx((-0.1, 0.0, 0.0)))[0, 0]
        rough = oracle.eval_program(st, m.roughness_program, _hook_ctx((0.1, 0.0, 0.0)))[0, 0]
        assert abs(smooth - 0.12) < 1e-6 and abs(rough - 0.48) < 1e-6
    else:
        solid, thin = _hook_ctx((-0.1, -0.1, 0.0)), _hook_ctx((0.1, 0.1, 0.0))
        assert abs(oracle.eval_program(st, m.ior_program, solid)[0, 0] - 1.45) < 1e-6
        assert abs(oracle.eval_program(st, m.ior_program, thin)[0, 0] - 1.6) < 1e-6
        assert oracle.eval_program(st, m.thin_walled_program, solid)[0, 0] < 0.5
        assert oracle.eval_program(st, m.thin_walled_program, thin)[0, 0] >= 0.5


# The reference's custom sdf test sources (lib.rs tests
# evaluates_custom_sdf_distance_with_helper_functions,
# supports_programmable_sdf_domain_and_distance_post_hooks,
# jits_vec3_box_style_sdf_distance), with bounds() added where they have none.
CUSTOM_SDFS = """
sdf SoftBlob {
  let warp_scale = 0.25;
  fn bounds() {
    return vec3(1.2, 1.2, 1.2);
  }
  fn warp(p) {
    return vec3(p.x, p.y + sin(p.x * 3.0) * warp_scale, p.z);
  }
  fn distance(p) {
    let q = warp(p);
    return length(q) - 1.0;
  }
};
sdf TwistedShell {
  let radius = 0.5;
  let thickness = 0.05;
  fn bounds() {
    return 0.6;
  }
  fn domain(p) {
    return rotate_y(p, p.y * 90.0);
  }
  fn distance(p) {
    return length(p) - radius;
  }
  fn distance_post(d, p) {
    return abs(d) - thickness;
  }
};
sdf ShellBox {
  let width = 1.6;
  let height = 2.0;
  let depth = 0.6;
  let wall_thickness = 0.05;
  fn bounds() {
    return vec3(0.8, 1.0, 0.3);
  }
  fn sd_box(p, half_size) {
    let q = abs(p) - half_size;
    let outside = length(max(q, vec3(0.0)));
    let inside = min(max(q.x, max(q.y, q.z)), 0.0);
    return outside + inside;
  }
  fn distance(p) {
    let half_outer = vec3(width * 0.5, height * 0.5, depth * 0.5);
    let outer = sd_box(p, half_outer);
    let inner_half = max(half_outer - vec3(wall_thickness, wall_thickness, wall_thickness), vec3(0.001));
    let cavity = sd_box(vec3(p.x, p.y, p.z - wall_thickness), inner_half);
    return max(outer, -cavity);
  }
};
"""

CUSTOM_SCENE = CUSTOM_SDFS + """
let camera = Camera { origin: vec3(0.0, 1.5, -6.0), target: vec3(0.0, 0.8, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0) };
let blob = SoftBlob { pos: vec3(-1.8, 1.2, 0.0), material: Lambert { color: vec3(0.8, 0.3, 0.2) } };
let shell = TwistedShell { pos: vec3(0.0, 0.6, -0.5), rot: vec3(0.0, 30.0, 0.0), material: Metal { roughness: 0.1 } };
let box = ShellBox { pos: vec3(1.8, 1.0, 0.5), rot: vec3(0.0, -20.0, 0.0) };
let scene = ground + blob + shell + box;
"""


def test_custom_sdf_definitions_lower_to_programs():
    """User `sdf` definitions become Custom leaves (R:1528-1550): the
    reference's known answer (lib.rs, evaluates_custom_sdf_distance_with_
    helper_functions: distance(0, 1, 0) is exactly 0, bounds x is 1.2), the
    domain and distance_post hooks, vec3 helper functions, and the world box
    of the rotated half extents (sdf_bounds, R:5304-5326)."""
    st = ft.parse_and_eval(CUSTOM_SCENE)
    d = st.desc
    custom = [_native.NodeC.from_buffer_copy(d.nodes[i]) for i in range(d.n_nodes) if d.nodes[i].kind == 30]
    assert len(custom) == 3
    blob, shell, box = custom
    assert oracle.eval_program(st, blob.program, np.array([[[0.0, 1.0, 0.0]]], np.float32))[0, 0] == 0.0
    assert blob.f[0] == np.float32(1.2) and blob.ival < 0 and blob.reserved < 0
    assert shell.ival >= 0 and shell.reserved >= 0 and shell.f[0] == np.float32(0.6)
    # TwistedShell at its local point (0.5, 0, 0): |p| - 0.5 = 0, post abs(0) - 0.05
    q = oracle.eval_program(st, shell.ival, np.array([[[0.5, 0.0, 0.0]]], np.float32))[0]
    assert np.allclose(q, (0.5, 0.0, 0.0), atol=1e-6)
    post = oracle.eval_program(st, shell.reserved, np.array([[[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]]], np.float32))
    assert abs(post[0, 0] + 0.05) < 1e-7
    # ShellBox wall: 0.05 inside the outer x face, well inside the cavity's z
    assert abs(oracle.eval_program(st, box.program, np.array([[[0.75, 0.0, 0.0]]], np.float32))[0, 0]) < 1e-6
    # rotated by -20 degrees about y: the world box holds the rotated corners
    c, s = np.cos(np.radians(20.0)), np.sin(np.radians(20.0))
    half_x = 0.8 * c + 0.3 * s
    assert abs((box.bounds_max[0] - box.bounds_min[0]) / 2 - half_x) < 1e-5
    # an sdf without distance(p) is refused
    with pytest.raises(ft.RenderError, match="distance"):
        ft.parse_and_eval("sdf Empty { fn bounds() { return 1.0; } };\nlet scene = Empty {};\n")
