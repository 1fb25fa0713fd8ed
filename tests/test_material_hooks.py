"""The further material hooks on the CPU: the reference's unit tests of the
BSDF hooks (eval / pdf / sample), the dynamic normal and bump hooks and
helper functions shared across hooks (renderer.rs tests
resolves_ft_custom_bsdf_hooks, resolves_ft_material_dynamic_normal_hook,
resolves_ft_material_dynamic_bump_hook,
resolves_material_local_helper_functions_across_hooks), restated with the
same sources, hits and expected values through the oracle; and the lowering
of the property hooks into ft_material.hook_program."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import _native

CUSTOM_BSDF = """
material CustomBsdf {
  model: Lambert;
  color = vec3(0.2);
  fn eval(ctx) {
    return vec3(0.25, 0.5, 0.75);
  }
  fn pdf(ctx) {
    return 0.42;
  }
  fn sample(ctx) {
    return BsdfSample {
      wi: ctx.normal,
      f: vec3(0.6, 0.4, 0.2),
      pdf: 0.35,
      delta: 0.0,
      apply_cos: 1.0,
      transmission: 0.0,
      thin_walled: 0.0,
      next_ior: ctx.current_ior
    };
  }
};

let scene = Sphere {
  material: CustomBsdf {}
};
"""


def test_custom_bsdf_hooks():
    """resolves_ft_custom_bsdf_hooks: hit (0, 0, 1) with normal +z, view +z,
    current IOR 1.1, wi +z."""
    st = ft.parse_and_eval(CUSTOM_BSDF)
    r = oracle.bsdf_hit(st, (0.0, 0.0, 1.0), (0.0, 0.0, 1.0), True, 1, 1, (0.0, 0.0, 1.0), 1.1, (0.0, 0.0, 1.0))
    assert np.allclose(r["eval"], [0.25, 0.5, 0.75], atol=1e-6)
    assert abs(r["pdf"] - 0.42) < 1e-6
    assert abs(r["sample_wi"][2] - 1.0) < 1e-6
    assert abs(r["sample_f"][0] - 0.6) < 1e-6 and abs(r["sample_f"][1] - 0.4) < 1e-6
    assert abs(r["sample_pdf"] - 0.35) < 1e-6
    assert abs(r["sample_next_ior"] - 1.1) < 1e-6
    assert r["sample_apply_cos"] and not r["sample_delta"] and not r["sample_transmission"]
    # every field of the record is one program; eval and pdf take the BSDF context
    d = st.desc
    m = d.materials[1]
    for slot in range(_native.FT_HOOK_EVAL, _native.FT_HOOK_SAMPLE_NEXT_IOR + 1):
        prog = m.hook_program[slot]
        assert prog >= 0, slot
        assert d.programs[prog].n_params == _native.FT_BSDF_HOOK_PARAMS
    for slot in range(_native.FT_HOOK_EVAL):
        assert m.hook_program[slot] == -1


def test_bsdf_hooks_fall_back_to_the_builtin_model():
    """Without hooks eval / pdf / sample are the material model's (Lambert:
    albedo / pi, cos / pi)."""
    st = ft.parse_and_eval("let scene = Sphere { material: Lambert { color: vec3(0.5, 0.25, 1.0) } };\n")
    r = oracle.bsdf_hit(st, (0.0, 0.0, 1.0), (0.0, 0.0, 1.0), True, 1, 1, (0.0, 0.0, 1.0), 1.0, (0.0, 0.0, 1.0))
    assert np.allclose(r["eval"], np.array([0.5, 0.25, 1.0]) / np.pi, rtol=1e-6)
    assert abs(r["pdf"] - 1.0 / np.pi) < 1e-6
    assert r["sample_wi"][2] > 0.0 and r["sample_apply_cos"]


def test_dynamic_normal_hook():
    """resolves_ft_material_dynamic_normal_hook: the normal hook tilts the
    shading normal of a hit at (0, 0, 1) towards +x."""
    src = """
material Bumped {
  model: Lambert;
  fn normal(ctx) {
    return normalize(vec3(ctx.normal.x + 0.35, ctx.normal.y, ctx.normal.z));
  }
};

let scene = Sphere {
  material: Bumped {}
};
"""
    st = ft.parse_and_eval(src)
    r = oracle.bsdf_hit(st, (0.0, 0.0, 1.0), (0.0, 0.0, 1.0), True, 1, 1, (0.0, 0.0, 1.0), 1.0, (0.0, 0.0, 1.0))
    assert r["normal"][0] > 0.2 and r["normal"][2] > 0.9


def test_dynamic_bump_hook():
    """resolves_ft_material_dynamic_bump_hook: a height field in the local
    position bends the normal of a hit at (0.1, 0, 0.995)."""
    src = """
material Bumpy {
  fn bump(ctx) {
    return sin(ctx.local_position.x * 10.0) * 0.2;
  }
};

let scene = Sphere {
  material: Bumpy {}
};
"""
    st = ft.parse_and_eval(src)
    n = np.array([0.1, 0.0, 0.995], np.float32)
    n /= np.linalg.norm(n)
    r = oracle.bsdf_hit(st, (0.1, 0.0, 0.995), tuple(n), True, 1, 1, (0.0, 0.0, 1.0), 1.0, (0.0, 0.0, 1.0))
    assert float(np.dot(r["normal"], n)) < 0.9999
    assert abs(float(np.linalg.norm(r["normal"])) - 1.0) < 1e-5


def test_helper_functions_across_hooks_normal():
    """resolves_material_local_helper_functions_across_hooks: the normal hook
    shares the definition's helper with the colour and roughness hooks."""
    src = """
material Brick {
  model: Lambert;
  let brick = vec3(0.68, 0.24, 0.16);
  let mortar = vec3(0.8, 0.77, 0.72);

  fn mortar_mask(ctx) {
    let band_x = smoothstep(-0.12, 0.12, sin(ctx.local_position.x * 11.0));
    let band_y = smoothstep(-0.12, 0.12, sin(ctx.local_position.y * 7.0));
    return max(band_x, band_y);
  }

  fn color(ctx) {
    return mix(brick, mortar, mortar_mask(ctx));
  }

  fn roughness(ctx) {
    return mix(0.7, 0.95, mortar_mask(ctx));
  }

  fn normal(ctx) {
    let m = mortar_mask(ctx);
    return normalize(ctx.normal + vec3(m * 0.2, 0.0, 0.0));
  }
};

let scene = Sphere {
  material: Brick {}
};
"""
    st = ft.parse_and_eval(src)
    r = oracle.bsdf_hit(st, (0.1, 0.1, 1.0), (0.0, 0.0, 1.0), True, 1, 1, (0.0, 0.0, 1.0), 1.0, (0.0, 0.0, 1.0))
    assert r["normal"][0] > 0.05


PROPERTY_HOOKS = """
material Glow {
  model: Lambert;
  fn emission_color(ctx) { return vec3(1.0, 0.5, 0.25); }
  fn emission_strength(ctx) { return ctx.position.y * 2.0 - 10.0; }
  fn metallic(ctx) { return 0.5; }
};
material Coated {
  model: Standard;
  coat_weight = 0.8;
  fn metallic(ctx) { return ctx.local_position.x * 4.0; }
  fn specular(ctx) { return 0.25; }
  fn specular_weight(ctx) { return 0.5; }
  fn transmission(ctx) { return -1.0; }
  fn coat_color(ctx) { return 0.5; }
  fn coat_roughness(ctx) { return 0.3; }
  fn coat_ior(ctx) { return 9.0; }
  fn coat_mask(ctx) { return 0.5; }
  fn clearcoat(ctx) { return 1.0; }
};
let scene = Sphere { material: Glow {} } + Sphere { pos: vec3(2.0, 0.0, 0.0), material: Coated {} };
"""


def test_property_hooks_are_lowered_per_model():
    """Emission hooks for every definition; metallic, specular,
    specular_weight, transmission and the coat hooks for Standard / Layered
    definitions only; a coated definition's own clearcoat hook is replaced by
    the coat (R:7258-7470) and is not lowered."""
    st = ft.parse_and_eval(PROPERTY_HOOKS)
    d = st.desc
    mats = [d.materials[i] for i in range(d.n_materials)]
    glow = next(m for m in mats if m.hook_program[_native.FT_HOOK_EMISSION_COLOR] >= 0)
    assert glow.hook_program[_native.FT_HOOK_EMISSION_STRENGTH] >= 0
    assert glow.hook_program[_native.FT_HOOK_METALLIC] == -1  # a Lambert-model definition
    coated = next(m for m in mats if m.hook_program[_native.FT_HOOK_COAT_IOR] >= 0)
    for slot in (_native.FT_HOOK_METALLIC, _native.FT_HOOK_SPECULAR, _native.FT_HOOK_SPECULAR_WEIGHT,
                 _native.FT_HOOK_TRANSMISSION, _native.FT_HOOK_COAT_COLOR, _native.FT_HOOK_COAT_ROUGHNESS,
                 _native.FT_HOOK_COAT_MASK):
        assert coated.hook_program[slot] >= 0, slot
    assert coated.hook_program[_native.FT_HOOK_COAT_WEIGHT] == -1  # a static property, folded
    assert abs(coated.clearcoat - 0.8) < 1e-6
    args = np.zeros((1, _native.FT_MATERIAL_HOOK_PARAMS, 3), np.float32)
    args[0, 1] = (0.1, 0.0, 0.0)  # local position
    assert abs(oracle.eval_program(st, coated.hook_program[_native.FT_HOOK_METALLIC], args)[0, 0] - 0.4) < 1e-6
    assert oracle.eval_program(st, coated.hook_program[_native.FT_HOOK_COAT_IOR], args)[0, 0] == pytest.approx(9.0)


def test_bsdf_and_property_hook_programs_are_validated():
    """A BSDF hook must take the 13-parameter BSDF context and a property
    hook the 7-parameter shading context; the reserved slot stays empty."""
    import ctypes

    from test_scene_build import _with_materials

    st = ft.parse_and_eval(CUSTOM_BSDF)

    def eval_as_property(mats, d):
        for i in range(d.n_materials):
            mats[i].hook_program[_native.FT_HOOK_EMISSION_COLOR] = mats[i].hook_program[_native.FT_HOOK_EVAL]

    rc, _ = _with_materials(st, eval_as_property)
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "shading context" in _native.last_error()

    def reserved(mats, d):
        mats[0].hook_program[_native.FT_MATERIAL_HOOK_SLOTS - 1] = 0

    rc, _ = _with_materials(st, reserved)
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "reserved" in _native.last_error()


MEDIUM_HOOK = """
material Smoky {
  model: Dielectric;
  ior = 1.5;
  fn medium(ctx) {
    return Medium {
      ior: 1.4 + ctx.local_position.y * 0.2,
      absorption_color: vec3(0.9, 0.5 + ctx.local_position.x, 0.3),
      density: 2.0 + ctx.local_position.z
    };
  }
};
material Partial {
  model: Dielectric;
  fn medium(ctx) { return Medium { density: 5.0 }; }
};
let scene = Sphere { material: Smoky {} } + Sphere { pos: vec3(2.0, 0.0, 0.0), material: Partial {} };
"""


def test_medium_hook_is_lowered_field_by_field():
    """`fn medium(ctx)` returns a Medium record: each of ior,
    absorption_color and density is one program over the shading context,
    and a field the record lacks is left to medium_from_value's default."""
    st = ft.parse_and_eval(MEDIUM_HOOK)
    d = st.desc
    mats = [d.materials[i] for i in range(d.n_materials)]
    smoky = next(m for m in mats if m.hook_program[_native.FT_HOOK_MEDIUM_ABSORPTION] >= 0)
    partial = next(m for m in mats if m.hook_program[_native.FT_HOOK_MEDIUM_DENSITY] >= 0
                   and m.hook_program[_native.FT_HOOK_MEDIUM_ABSORPTION] < 0)
    assert partial.hook_program[_native.FT_HOOK_MEDIUM_IOR] == -1
    args = np.zeros((1, _native.FT_MATERIAL_HOOK_PARAMS, 3), np.float32)
    args[0, 1] = (0.1, 0.5, -0.25)  # local position
    ev = lambda slot: oracle.eval_program(st, smoky.hook_program[slot], args)[0]
    assert ev(_native.FT_HOOK_MEDIUM_IOR)[0] == pytest.approx(1.5, abs=1e-6)
    assert np.allclose(ev(_native.FT_HOOK_MEDIUM_ABSORPTION), [0.9, 0.6, 0.3], atol=1e-6)
    assert ev(_native.FT_HOOK_MEDIUM_DENSITY)[0] == pytest.approx(1.75, abs=1e-6)
    assert d.programs[smoky.hook_program[_native.FT_HOOK_MEDIUM_IOR]].n_params == _native.FT_MATERIAL_HOOK_PARAMS
