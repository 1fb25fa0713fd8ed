"""The CPU oracle against the reference's own regression goldens, and its
f32/f64 forms against each other."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from conftest import FIXTURES
from forgedthoughts_gb300 import workloads

# crates/forgedthoughts/tests/render_regression.rs:34-107
PREVIEW_OPTS = dict(width=96, height=96, max_steps=320, max_dist=40.0, epsilon=0.0002, step_scale=0.7,
                    camera_z=6.0, fov_y_degrees=35.0)


@pytest.mark.parametrize("name", ["preview_lambert", "preview_material_hook"])
@pytest.mark.parametrize("precision", [32, 64])
def test_oracle_matches_reference_depth_golden(name, precision):
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / f"{name}.ft")
    _, _, _, rgb, _ = oracle.render_depth(st, ft.RenderOptions(**PREVIEW_OPTS), ft.AccelMode.Bvh, 1, precision)
    gold = ft.read_png(FIXTURES / "render_regression" / f"{name}.png")
    diff = np.abs(rgb.astype(int) - gold.astype(int))
    # reference tolerance (render_regression.rs:139-145) ...
    assert diff.max() <= 8 and diff.mean() <= 0.35
    # ... and in fact the restatement reproduces the goldens exactly.
    assert diff.max() == 0


@pytest.mark.parametrize("accel", [0, 1, 2])
def test_accel_modes_agree_on_primitive_leaves(accel):
    w = workloads.spheres_on_ground(width=64, height=64)
    st = ft.parse_and_eval(w.source)
    t0, m0, _, _, _ = oracle.render_depth(st, w.options, 1, 1, 32)
    t, m, _, _, _ = oracle.render_depth(st, w.options, accel, 1, 32)
    assert np.array_equal(m, m0)
    assert np.array_equal(t, t0)


def test_f32_march_tracks_f64_march():
    w = workloads.spheres_on_ground(width=128, height=128)
    st = ft.parse_and_eval(w.source)
    t32, m32, _, _, _ = oracle.render_depth(st, w.options, 0, 1, 32)
    t64, m64, _, _, _ = oracle.render_depth(st, w.options, 0, 1, 64)
    assert (m32 == m64).mean() >= 0.999
    both = (m32 == 1) & (m64 == 1)
    err = np.abs(t32[both].astype(np.float64) - t64[both])
    assert np.quantile(err, 0.999) <= 1e-4


def test_empty_sample_rows_are_untouched():
    w = workloads.spheres_on_ground(width=32, height=32)
    st = ft.parse_and_eval(w.source)
    t, m, _, _, _ = oracle.render_depth(st, w.options, 1, 1, 32, rows=(0, 32, 8))
    rendered = np.zeros(32, bool)
    rendered[::8] = True
    assert not m[~rendered].any()


# crates/forgedthoughts/tests/render_regression.rs:48-90 (Whitted, depth 4, aa 1, Bvh)
TRACE_CASES = {
    "ray_metal": dict(width=96, height=96, max_steps=360, max_dist=50.0, epsilon=0.0002, step_scale=0.7,
                      camera_z=6.0, fov_y_degrees=35.0),
    "ray_boolean_union_round": dict(width=96, height=96, max_steps=520, max_dist=60.0, epsilon=0.0002,
                                    step_scale=0.7, camera_z=6.0, fov_y_degrees=25.0),
}


@pytest.mark.parametrize("name", sorted(TRACE_CASES))
@pytest.mark.parametrize("precision", [32, 64])
def test_oracle_matches_reference_trace_golden(name, precision):
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / f"{name}.ft")
    _, rgb8, _ = oracle.render_trace(st, ft.RenderOptions(**TRACE_CASES[name]), ft.AccelMode.Bvh, 1, 4, precision)
    gold = ft.read_png(FIXTURES / "render_regression" / f"{name}.png")
    diff = np.abs(rgb8.astype(int) - gold.astype(int))
    # the reference's own regression tolerance (render_regression.rs:139-145)
    assert diff.max() <= 8 and diff.mean() <= 0.35, (diff.max(), diff.mean())


def _sphere_material(source):
    from forgedthoughts_gb300 import _native

    st = ft.parse_and_eval(source)
    d = st.desc
    sph = [d.nodes[i] for i in range(d.n_nodes) if d.nodes[i].kind == 0]  # FT_NODE_SPHERE
    return _native.MaterialC.from_buffer_copy(d.materials[sph[0].material_id])  # outlives the description


def test_medium_transmittance_known_answer():
    """The reference's applies_medium_transmittance_per_segment: absorption
    (0.5, 0.8, 1.0) at density 2 over 1.5 units gives (0.125, 0.512, 1)."""
    t = oracle.medium_transmittance(1.33, (0.5, 0.8, 1.0), 2.0, 1.5)
    assert np.allclose(t, [0.125, 0.512, 1.0], atol=1e-6), t
    # no density or no distance: no attenuation
    assert np.array_equal(oracle.medium_transmittance(1.33, (0.5, 0.8, 1.0), 0.0, 1.5), [1, 1, 1])
    assert np.array_equal(oracle.medium_transmittance(1.33, (0.5, 0.8, 1.0), 2.0, 0.0), [1, 1, 1])


def test_transition_medium_known_answer():
    """The reference's transitions_medium_when_crossing_dielectric: entering
    a Dielectric (IOR 1.52) with an explicit medium takes that medium, leaving
    it returns to air.  The material comes through the `.ft` lowering."""
    m = _sphere_material("""
        let scene = Sphere { material: Dielectric { ior: 1.52,
          medium: Medium { ior: 1.33, absorption_color: vec3(0.9, 0.8, 0.7), density: 0.25 } } };
    """)
    air = [1.0, 1.0, 1.0, 1.0, 0.0]
    entered = oracle.transition_medium(m, True, air)
    assert abs(entered[0] - 1.33) < 1e-6 and abs(entered[2] - 0.8) < 1e-6 and abs(entered[4] - 0.25) < 1e-6
    exited = oracle.transition_medium(m, False, entered)
    assert abs(exited[0] - 1.0) < 1e-6 and abs(exited[1] - 1.0) < 1e-6 and abs(exited[4]) < 1e-6
    # without an explicit medium the material's IOR is entered, with no absorption
    plain = _sphere_material("let scene = Sphere { material: Dielectric { ior: 1.52 } };")
    assert np.allclose(oracle.transition_medium(plain, True, air), [1.52, 1, 1, 1, 0], atol=1e-6)
    # an opaque material keeps the current medium
    lam = _sphere_material("let scene = Sphere { material: Lambert { medium: Medium { density: 3.0 } } };")
    assert np.array_equal(oracle.transition_medium(lam, True, entered), entered)


def test_trace_absorbing_medium_darkens_the_refraction():
    """A glass sphere with a dense blue-absorbing medium in front of a white
    sky: the pixels seen through it lose blue relative to the same sphere
    without the medium, and nothing else changes."""
    base = """
        environment Sky {{ fn color(dir) {{ return vec3(1.0, 1.0, 1.0); }} }};
        let scene = Sphere {{ radius: 1.0, material: Dielectric {{ ior: 1.3{medium} }} }};
    """
    opts = ft.RenderOptions(width=24, height=24, max_steps=200, max_dist=20.0, epsilon=1e-4, camera_z=4.0)
    plain = ft.parse_and_eval(base.format(medium=""))
    dense = ft.parse_and_eval(base.format(
        medium=", medium: Medium { absorption_color: vec3(0.9, 0.9, 0.2), density: 2.0 }"))
    a, _, _ = oracle.render_trace(plain, opts, 1, 1, 4, 32)
    b, _, _ = oracle.render_trace(dense, opts, 1, 1, 4, 32)
    centre = (slice(9, 15), slice(9, 15))
    assert (b[centre][..., 2] < 0.5 * a[centre][..., 2]).all()
    assert (b[centre][..., 0] > 0.5 * a[centre][..., 0]).all()
    assert np.array_equal(a[0, 0], b[0, 0])  # a corner ray misses the sphere


def test_trace_f32_tracks_f64():
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / "ray_boolean_union_round.ft")
    opts = ft.RenderOptions(**TRACE_CASES["ray_boolean_union_round"])
    a, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 32)
    b, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 64)
    assert np.sqrt(np.mean((a - b) ** 2)) <= 1e-3


def test_rough_dielectric_lobes_average_traced_rays():
    """A roughness-0.35 glass sphere (2 reflection and 4 refraction lobe rays
    per hit) traces more rays than the same sphere smooth, and its image is
    a blur of the smooth one: the sky seen through it keeps its mean."""
    src = """
        environment Sky {{ fn color(dir) {{ return mix(vec3(1.0, 0.9, 0.8), vec3(0.2, 0.4, 1.0), clamp(dir.y, 0.0, 1.0)); }} }};
        let scene = Sphere {{ radius: 1.0, material: Dielectric {{ ior: 1.4, roughness: {r} }} }};
    """
    opts = ft.RenderOptions(width=24, height=24, max_steps=200, max_dist=20.0, epsilon=1e-4, camera_z=4.0)
    smooth = ft.parse_and_eval(src.format(r="0.0"))
    rough = ft.parse_and_eval(src.format(r="0.35"))
    a, _, ea = oracle.render_trace(smooth, opts, 1, 1, 3, 32)
    b, _, eb = oracle.render_trace(rough, opts, 1, 1, 3, 32)
    assert eb > 2 * ea
    centre = (slice(8, 16), slice(8, 16))
    assert np.abs(b[centre] - a[centre]).max() > 1e-3
    assert abs(b[centre].mean() - a[centre].mean()) < 0.1 * a[centre].mean()


PATH_SCENE = """
environment Sky { fn color(dir) { return mix(vec3(0.9, 0.9, 0.95), vec3(0.3, 0.5, 1.0), clamp(dir.y, 0.0, 1.0)); } };
let camera = Camera { origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 40.0 };
let env = EnvLight { radiance: 0.3 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Lambert { color: vec3(0.6, 0.6, 0.6) } };
let a = Sphere { radius: 0.5, pos: vec3(-1.1, 0.5, 0.0), material: Metal { roughness: 0.3 } };
let b = Sphere { radius: 0.5, pos: vec3(0.0, 0.5, 0.3), material: Dielectric { ior: 1.5 } };
let c = Sphere { radius: 0.5, pos: vec3(1.1, 0.5, 0.0) };
let scene = ground + a + b + c;
"""


def test_path_tracer_is_deterministic_and_adaptive():
    """The MIS path tracer seeds every pixel sample's generator from the pixel
    and sample index: two runs are identical; with a noise threshold, pixels
    stop between min_spp and spp samples and a pixel of the flat sky stops
    at min_spp; more samples move the image less than fewer do."""
    st = ft.parse_and_eval(PATH_SCENE)
    opts = ft.RenderOptions(width=32, height=24, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    a, a8, na, _ = oracle.render_path(st, opts, 1, spp=16, max_bounces=4, min_spp=4, noise_threshold=0.05)
    b, b8, nb, _ = oracle.render_path(st, opts, 1, spp=16, max_bounces=4, min_spp=4, noise_threshold=0.05)
    assert np.array_equal(a, b) and np.array_equal(na, nb)
    assert na.min() >= 4 and na.max() <= 16 and (na < 16).any() and (na == 16).any()
    assert na[0, 0] == 4  # sky corner: the environment only, no variance
    full, _, nf, _ = oracle.render_path(st, opts, 1, spp=16, max_bounces=4, min_spp=16, noise_threshold=0.0)
    assert (nf == 16).all()
    assert np.isfinite(full).all() and full.mean() > 0.05
    few, _, _, _ = oracle.render_path(st, opts, 1, spp=4, max_bounces=4, min_spp=4, noise_threshold=0.0)
    more, _, _, _ = oracle.render_path(st, opts, 1, spp=64, max_bounces=4, min_spp=64, noise_threshold=0.0)
    assert np.abs(more - full).mean() < np.abs(few - full).mean()
    f64, _, _, _ = oracle.render_path(st, opts, 1, spp=16, max_bounces=4, min_spp=16, noise_threshold=0.0,
                                      precision=64)
    assert np.abs(f64 - full).mean() < 0.02
