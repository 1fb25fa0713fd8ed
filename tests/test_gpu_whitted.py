"""Whitted trace on the GPU against the CPU oracle: explicit media inside
dielectrics.  Calls go through the C ABI; radiance is linear RGB, compared
by RMSE (the bar is 1e-3)."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle

pytestmark = pytest.mark.gpu


def radiance_rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)))


MEDIA_SCENE = """
environment Sky {{ fn color(dir) {{ return mix(vec3(0.9, 0.95, 1.0), vec3(0.4, 0.6, 1.0), clamp(dir.y, 0.0, 1.0)); }} }};
let camera = Camera {{ origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 }};
let light = PointLight {{ position: vec3(3.0, 6.0, -3.0), intensity: 60.0 }};
let ground = Box {{ size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0) }};
let a = Sphere {{ radius: 0.55, pos: vec3(-0.7, 0.6, 0.0),
  material: Dielectric {{ ior: 1.45, medium: Medium {{ absorption_color: vec3(0.95, 0.6, 0.2), density: 1.5 }} }} }};
let b = Sphere {{ radius: 0.55, pos: vec3(0.7, 0.6, 0.0),
  material: Dielectric {{ ior: 1.3, medium: Medium {{ ior: 1.2, absorption_color: vec3(0.3, 0.9, 0.9), density: 0.8 }} }} }};
let scene = ground + {join};
"""


@pytest.mark.parametrize("join", ["a + b", "a.union_round(b, 0.4)"])
def test_gpu_trace_explicit_media(join):
    """Absorbing media inside dielectrics (transition into the material's
    explicit medium, Beer-Lambert transmittance per segment), apart and
    blended by a union_round (blend_medium): GPU against the f32 oracle, and
    the media visibly change the image."""
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    src = MEDIA_SCENE.format(join=join)
    st = ft.parse_and_eval(src)
    assert sum(st.desc.materials[i].has_medium for i in range(st.desc.n_materials)) == 2
    for depth in (2, 4):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (join, depth, radiance_rmse(lin, ref))
    clear = ft.parse_and_eval(src.replace("density: 1.5", "density: 0.0").replace("density: 0.8", "density: 0.0"))
    lin_clear, _ = ft.render_trace(clear, opts, ft.AccelMode.Bvh, 1, 4)
    assert radiance_rmse(lin, lin_clear) > 5e-3


ROUGH_SCENE = """
environment Sky { fn color(dir) { return mix(vec3(0.95, 0.9, 0.8), vec3(0.3, 0.5, 1.0), clamp(dir.y, 0.0, 1.0)); } };
let camera = Camera { origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Lambert { color: vec3(0.7, 0.3, 0.2) } };
let a = Sphere { radius: 0.5, pos: vec3(-1.1, 0.55, 0.0), material: Dielectric { ior: 1.5, roughness: 0.09 } };
let b = Sphere { radius: 0.5, pos: vec3(0.0, 0.55, 0.2), material: Dielectric { ior: 1.45, roughness: 0.2 } };
let c = Sphere { radius: 0.5, pos: vec3(1.1, 0.55, 0.0), material: Dielectric { ior: 1.4, roughness: 0.35 } };
let scene = ground + a + b + c;
"""


def test_gpu_trace_rough_dielectric_lobes():
    """Dielectrics with roughness above 0.06 average a lobe of reflected and
    refracted rays (trace_rough_dielectric_reflection / _refraction,
    ray.rs:296-435): 1 to 3 reflection and 2 to 4 refraction rays by
    roughness.  GPU against the f32 oracle, and the lobes visibly change the
    image against the same spheres made smooth."""
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    st = ft.parse_and_eval(ROUGH_SCENE)
    for depth in (2, 3):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))
    smooth = ft.parse_and_eval(ROUGH_SCENE.replace("roughness: 0.09", "roughness: 0.0")
                               .replace("roughness: 0.2", "roughness: 0.0").replace("roughness: 0.35", "roughness: 0.0"))
    lin_s, _ = ft.render_trace(smooth, opts, ft.AccelMode.Bvh, 1, 3)
    assert radiance_rmse(lin, lin_s) > 5e-3


def test_gpu_path_tracer_matches_oracle():
    """The MIS path tracer (trace_path with estimate_direct_mis, every pixel
    sample seeded by seed_pixel_sample): GPU against the f32 oracle on the
    same samples, with and without adaptive stopping.  Lambert, Metal,
    Dielectric and the default Standard material, a point and an environment
    light, a sky environment."""
    import sys
    sys.path.insert(0, __file__.rsplit("/", 1)[0])
    from test_oracle import PATH_SCENE

    st = ft.parse_and_eval(PATH_SCENE)
    opts = ft.RenderOptions(width=96, height=72, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    for spp, min_spp, thr in ((8, 8, 0.0), (16, 4, 0.05)):
        s = ft.PathtraceSettings(spp=spp, max_bounces=4, min_spp=min_spp, noise_threshold=thr)
        lin, rgb8, n = ft.render_pathtrace(st, opts, ft.AccelMode.Bvh, s)
        ref, ref8, nref, _ = oracle.render_path(st, opts, 1, spp=spp, max_bounces=4, min_spp=min_spp,
                                                noise_threshold=thr)
        # the sample counts follow the same per-pixel statistics
        assert (n == nref).mean() >= 0.99, (n != nref).sum()
        same = n == nref
        # a path is a chain of random decisions: a last-bit difference can
        # send one sample elsewhere, so compare per pixel with the Whitted
        # chaotic bar
        diff = np.abs(lin[same].astype(np.float64) - ref[same]).max(axis=-1)
        assert (diff <= 1e-3).mean() >= 0.99, (diff <= 1e-3).mean()
        assert radiance_rmse(lin[same], ref[same]) <= 2e-2, radiance_rmse(lin[same], ref[same])
