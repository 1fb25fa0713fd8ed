"""The further material hooks on the GPU against the f32 oracle, through the
C ABI: bump and normal hooks (the shading normal), the BSDF eval / pdf /
sample hooks, the emission hooks and a Standard definition's metallic and
coat hooks, in the Whitted trace (interpreted and NVRTC-compiled) and the MIS
path tracer."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from parity import radiance_rmse

pytestmark = pytest.mark.gpu

HOOK_SCENE = """
environment Sky { fn color(dir) { return mix(vec3(0.9, 0.85, 0.8), vec3(0.3, 0.5, 1.0), clamp(dir.y, 0.0, 1.0)); } };
let camera = Camera { origin: vec3(0.0, 1.3, -4.8), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let fill = EnvLight { color: vec3(1.0, 1.0, 1.0), intensity: 0.2 };
material Bumpy {
  model: Lambert;
  color = vec3(0.7, 0.6, 0.5);
  fn bump(ctx) { return sin(ctx.local_position.x * 6.0) * sin(ctx.local_position.z * 6.0) * 0.05; }
};
material Tilted {
  model: Metal;
  color = vec3(0.8, 0.7, 0.4);
  roughness = 0.2;
  fn normal(ctx) { return normalize(ctx.normal + vec3(0.25, 0.0, 0.0)); }
};
material Toon {
  model: Lambert;
  fn eval(ctx) { return vec3(0.3, 0.2, 0.1) * smoothstep(0.2, 0.8, dot(ctx.normal, ctx.wi)) + vec3(0.02, 0.02, 0.05); }
  fn pdf(ctx) { return max(dot(ctx.normal, ctx.wi), 0.0) * 0.3183; }
};
material Lamp {
  model: Lambert;
  color = vec3(0.2, 0.2, 0.2);
  fn emission_color(ctx) { return vec3(1.0, 0.6, 0.2); }
  fn emission_strength(ctx) { return 0.5 + 0.5 * sin(ctx.local_position.y * 20.0); }
};
material Lacquer {
  model: Standard;
  color = vec3(0.1, 0.3, 0.8);
  fn metallic(ctx) { return clamp(ctx.local_position.y + 0.5, 0.0, 1.0); }
  fn coat_weight(ctx) { return 0.9; }
  fn coat_mask(ctx) { return smoothstep(-0.2, 0.2, ctx.local_position.x); }
  fn coat_roughness(ctx) { return 0.35; }
};
material Mirror {
  model: Lambert;
  fn sample(ctx) {
    return BsdfSample {
      wi: ctx.normal * (2.0 * dot(ctx.normal, ctx.wo)) - ctx.wo,
      f: vec3(0.8, 0.85, 0.9),
      pdf: 1.0,
      delta: 1.0,
      apply_cos: 0.0
    };
  }
};
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Bumpy {} };
let a = Sphere { radius: 0.45, pos: vec3(-1.5, 0.45, 0.0), material: Tilted {} };
let b = Sphere { radius: 0.45, pos: vec3(-0.5, 0.45, 0.3), material: Toon {} };
let c = Sphere { radius: 0.45, pos: vec3(0.5, 0.45, 0.0), material: Lamp {} };
let d = Box { size: vec3(0.7, 0.7, 0.7), pos: vec3(1.5, 0.35, 0.2), rot: vec3(0.0, 30.0, 0.0), material: Lacquer {} };
let e = Sphere { radius: 0.35, pos: vec3(0.0, 0.35, -1.2), material: Mirror {} };
let scene = ground + a + b + c + d + e;
"""

OPTS = dict(width=160, height=96, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)


def _check(lin, ref32, ref64, what):
    # 99 % of the pixels within 1e-3, and an RMSE within 1e-3 or within the
    # oracle's own f32-vs-f64 gap: the metallic hook on the rotated box makes a
    # handful of its edge and highlight pixels sensitive to the last bit (the
    # oracle's f32 and f64 traces differ by RMSE 8e-4 there, 4e-5 without
    # the hooks)
    within = float((np.abs(lin.astype(np.float64) - ref32).max(axis=-1) <= 1e-3).mean())
    assert within >= 0.99, (what, within)
    bar = max(1e-3, radiance_rmse(ref32, ref64))
    assert radiance_rmse(lin, ref32) <= bar, (what, radiance_rmse(lin, ref32), bar)


def test_gpu_trace_with_material_hooks():
    """Whitted depth 1 and 2: GPU (interpreted, then NVRTC-compiled) against
    the f32 oracle; and the hooks change the image against the same scene
    with the hooks' definitions replaced by plain materials."""
    opts = ft.RenderOptions(**OPTS)
    st = ft.parse_and_eval(HOOK_SCENE)
    refs = {}
    for depth in (1, 2):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        refs[depth] = oracle.render_trace(st, opts, 1, 1, depth, 32)[0], oracle.render_trace(st, opts, 1, 1, depth, 64)[0]
        _check(lin, *refs[depth], f"interpreted depth {depth}")
    st.gpu().jit()
    lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 2)
    _check(lin, *refs[2], "compiled depth 2")
    plain = ft.parse_and_eval(HOOK_SCENE.replace("fn bump(", "fn unused_bump(").replace("fn normal(", "fn unused_normal(")
                              .replace("fn eval(", "fn unused_eval(").replace("fn emission_", "fn unused_emission_")
                              .replace("fn metallic(", "fn unused_metallic(").replace("fn coat_", "fn unused_coat_"))
    lin_p, _ = ft.render_trace(plain, opts, ft.AccelMode.Bvh, 1, 2)
    assert radiance_rmse(lin_p, refs[2][0]) > 1e-2


def test_gpu_path_tracer_with_bsdf_hooks():
    """The MIS path tracer with the eval, pdf and sample hooks (and the
    normal / bump / property hooks): GPU against the f32 oracle on the same
    samples, with the path test's per-pixel bar."""
    opts = ft.RenderOptions(**OPTS)
    st = ft.parse_and_eval(HOOK_SCENE)
    s = ft.PathtraceSettings(spp=8, max_bounces=4, min_spp=8, noise_threshold=0.0)
    lin, _, n = ft.render_pathtrace(st, opts, ft.AccelMode.Bvh, s)
    ref, _, nref, _ = oracle.render_path(st, opts, 1, spp=8, max_bounces=4, min_spp=8, noise_threshold=0.0)
    assert (n == nref).all()
    diff = np.abs(lin.astype(np.float64) - ref).max(axis=-1)
    assert (diff <= 1e-3).mean() >= 0.99, (diff <= 1e-3).mean()
    assert radiance_rmse(lin, ref) <= 2e-2, radiance_rmse(lin, ref)


MEDIUM_SCENE = """
environment Sky { fn color(dir) { return mix(vec3(0.9, 0.85, 0.8), vec3(0.3, 0.5, 1.0), clamp(dir.y, 0.0, 1.0)); } };
let camera = Camera { origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
material Smoky {
  model: Dielectric;
  ior = 1.5;
  fn medium(ctx) {
    return Medium {
      ior: 1.45,
      absorption_color: vec3(0.9, 0.4 + 0.3 * clamp(ctx.local_position.y + 0.5, 0.0, 1.0), 0.3),
      density: 1.5
    };
  }
};
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Lambert { color: vec3(0.7, 0.7, 0.7) } };
let ball = Sphere { radius: 0.55, pos: vec3(0.0, 0.55, 0.0), material: Smoky {} };
let scene = ground + ball;
"""


def test_gpu_trace_with_medium_hook():
    """A glass sphere whose `fn medium(ctx)` gives a height-dependent
    absorption: Whitted depth 4 (the refracted rays travel through the
    hooked medium) against the f32 oracle, and the hook visibly changes the
    image against the same glass without it."""
    opts = ft.RenderOptions(**OPTS)
    st = ft.parse_and_eval(MEDIUM_SCENE)
    lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 4)
    ref32, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 32)
    ref64, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 64)
    _check(lin, ref32, ref64, "medium hook depth 4")
    plain = ft.parse_and_eval(MEDIUM_SCENE.replace("fn medium(", "fn unused_medium("))
    lin_p, _ = ft.render_trace(plain, opts, ft.AccelMode.Bvh, 1, 4)
    assert radiance_rmse(lin_p, ref32) > 1e-2
