"""GPU depth path against the CPU oracle (f32 restatement and f64 march) and
the reference's regression goldens.  Calls go through the C ABI."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from conftest import FIXTURES
from forgedthoughts_gb300 import _native, workloads
from parity import DEPTH_TOL, assert_depth_parity, compare_depth

pytestmark = pytest.mark.gpu

PREVIEW_OPTS = dict(width=96, height=96, max_steps=320, max_dist=40.0, epsilon=0.0002, step_scale=0.7,
                    camera_z=6.0, fov_y_degrees=35.0)


@pytest.mark.parametrize("name", ["preview_lambert", "preview_material_hook"])
def test_gpu_matches_reference_depth_golden(name):
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / f"{name}.ft")
    img = ft.render_depth(st, ft.RenderOptions(**PREVIEW_OPTS), ft.AccelMode.Bvh, 1)
    gold = ft.read_png(FIXTURES / "render_regression" / f"{name}.png")
    diff = np.abs(img.rgb8.astype(int) - gold.astype(int))
    assert diff.max() <= 8 and diff.mean() <= 0.35, (diff.max(), diff.mean())
    t, m, _, rgb, _ = oracle.render_depth(st, ft.RenderOptions(**PREVIEW_OPTS), 1, 1, 32)
    assert_depth_parity(img.t, img.mask, t, m, name)


@pytest.mark.parametrize("precision", [32, 64])
def test_spheres_on_ground_full_size(precision):
    w = workloads.spheres_on_ground()  # 256x256, 8 spheres, Naive
    st = ft.parse_and_eval(w.source)
    img = ft.render_depth(st, w.options, w.accel, w.aa, want_material=True, want_normal=True)
    t, m, mat, rgb, _, nrm = oracle.render_depth(st, w.options, w.accel, w.aa, precision, normals=True)
    r = assert_depth_parity(img.t, img.mask, t, m, f"spheres f{precision}")
    both = (img.mask == 1) & (m == 1)
    assert (img.material[both] == mat[both]).mean() >= 0.999
    cos = (img.normal[both] * nrm[both]).sum(-1)
    assert np.quantile(cos, 0.001) > 0.999
    if precision == 32:
        assert np.abs(img.rgb8.astype(int) - rgb.astype(int)).max() <= 1
    print(r)


@pytest.mark.parametrize("accel", [ft.AccelMode.Naive, ft.AccelMode.Bvh, ft.AccelMode.Bricks])
def test_union_round_field_reduced(accel):
    w = workloads.union_round_field(width=256, height=144, aa=1, accel=accel)
    st = ft.parse_and_eval(w.source)
    img = ft.render_depth(st, w.options, accel, 1, want_material=True)
    t, m, mat, _, _ = oracle.render_depth(st, w.options, int(accel), 1, 32)
    assert_depth_parity(img.t, img.mask, t, m, f"union_round {accel.name}")
    both = (img.mask == 1) & (m == 1)
    assert (img.material[both] == mat[both]).mean() >= 0.999


def test_union_round_distance_in_every_grid_region():
    """The union_round tree's value at points inside its fine candidate grid,
    in the coarser outer grid around it and beyond both (the tree BVH): the
    GPU's exact FP32 distance against the f32 oracle, which folds all 512
    primitives at every point."""
    import ctypes

    w = workloads.union_round_field(width=64, height=36, aa=1)
    st = ft.parse_and_eval(w.source)
    info = _native.BuildInfoC()
    assert _native.lib().ft_scene_build_info(st.desc_ptr, ctypes.byref(info)) == 0
    assert info.grid_cells > 0 and info.outer_grid_cells > 0
    g = st.gpu()
    g.build_bricks()
    rng = np.random.default_rng(11)
    inner = rng.uniform([-7.0, -0.5, -7.0], [7.0, 4.0, 7.0], size=(40_000, 3))
    outer = rng.uniform([-13.0, -0.5, -13.0], [13.0, 10.0, 13.0], size=(40_000, 3))
    beyond = rng.uniform([-40.0, -0.5, -40.0], [40.0, 30.0, 40.0], size=(20_000, 3))
    pts = np.concatenate([inner, outer, beyond]).astype(np.float32)
    _, exact = g.brick_bounds(pts)
    ref, _, _ = oracle.distance(st, pts, accel=1, precision=32)
    err = np.abs(exact.astype(np.float64) - ref)
    assert (err <= 1e-5 * np.maximum(1.0, np.abs(ref))).all(), float(err.max())


def test_union_round_field_full_size_rows():
    """1920x1080 with the 2x2 AA grid: GPU frame against oracle rows."""
    w = workloads.union_round_field()
    st = ft.parse_and_eval(w.source)
    img = ft.render_depth(st, w.options, w.accel, w.aa)
    rows = (3, w.options.height, 135)
    t, m, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, 32, rows=rows)
    sel = np.arange(*rows)
    assert_depth_parity(img.t[sel], img.mask[sel], t[sel], m[sel], "union_round 1080p rows")
    t64, m64, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, 64, rows=rows)
    r = compare_depth(img.t[sel], img.mask[sel], t64[sel], m64[sel])
    assert r["mask_agreement"] >= 0.999 and r["depth_within_tol"] >= 0.999, r
    # frames are deterministic
    img2 = ft.render_depth(st, w.options, w.accel, w.aa)
    assert np.array_equal(img.t, img2.t) and np.array_equal(img.mask, img2.mask)


def test_twisted_shells_hooks():
    w = workloads.twisted_shells(n=256, width=160, height=90)
    st = ft.parse_and_eval(w.source)
    img = ft.render_depth(st, w.options, ft.AccelMode.Bvh, 1)
    t, m, _, _, _ = oracle.render_depth(st, w.options, 1, 1, 32)
    assert_depth_parity(img.t, img.mask, t, m, "twisted shells")


ALL_KINDS = """
let camera = Camera { origin: vec3(0.0, 2.5, -7.0), target: vec3(0.0, 0.5, 0.0), fov_y: 40.0 };
var ground = Box { size: vec3(40, 1, 40) };
ground.pos.y = -0.5;
var a = Box { size: vec3(1.2, 1.0, 0.8), round: 0.1 }; a.pos.x = -2.2; a.pos.y = 0.6; a.rot.y = 25.0;
var b = Sphere { radius: 0.7, shell: 0.05 }; b.pos.x = -1.8; b.pos.y = 0.9;
var c = Cylinder { radius: 0.4, height: 1.2, round: 0.05 }; c.pos.x = 0.0; c.pos.y = 0.6; c.rot.z = 20.0;
var d = Torus { major_radius: 0.5, minor_radius: 0.15 }; d.pos.x = 1.5; d.pos.y = 0.5; d.rot.x = 60.0;
var e = ExtrudePolygon { sides: 6, radius: 0.45, height: 0.5 }; e.pos.x = 2.6; e.pos.y = 0.3;
var f = Sphere { radius: 0.5 }; f.pos.x = 0.4; f.pos.y = 0.9; f.pos.z = -0.6;
let g = a.diff_round(b, 0.1);
let h = c.union_chamfer(f, 0.15);
let i = d.intersect_round(Sphere { radius: 0.6, pos: vec3(1.5, 0.5, 0.0) }, 0.05);
let j = e.union_stairs(Box { size: vec3(0.6, 0.3, 0.6), pos: vec3(2.6, 0.6, 0.0) }, 0.2, 3.0);
let k = c.union_columns(Sphere { radius: 0.3, pos: vec3(0.0, 1.3, 0.0) }, 0.2, 4.0);
let l = (a & b).smooth(0.2);
let m = Sphere { radius: 0.4, pos: vec3(-0.8, 1.8, 0.5) }.pipe(Box { size: vec3(0.5, 0.5, 0.5), pos: vec3(-0.8, 1.8, 0.5) }, 0.05);
let n = Box { size: vec3(0.8, 0.8, 0.8), pos: vec3(1.0, 1.8, 0.5) }.engrave(Sphere { radius: 0.45, pos: vec3(1.0, 1.8, 0.5) }, 0.05);
let o = Sphere { radius: 0.5, pos: vec3(-2.5, 1.8, 1.0) }.slice_y(1.6, 2.2);
let q = Box { size: vec3(0.5, 0.5, 0.5), pos: vec3(2.4, 1.8, 1.0) }.groove(Sphere { radius: 0.3, pos: vec3(2.4, 2.0, 1.0) }, 0.05, 0.05);
let r = Sphere { radius: 0.4, pos: vec3(0.0, 2.6, 1.5) }.union_soft(Sphere { radius: 0.3, pos: vec3(0.4, 2.6, 1.5) }, 0.2);
let s = Sphere { radius: 0.35, pos: vec3(-1.5, 2.6, 1.5) }.mirror_x();
let u = Box { size: vec3(0.2, 0.2, 0.2), pos: vec3(0.0, 0.15, -1.5) }.repeat_x(0.5, 5);
let v = Sphere { radius: 0.3, pos: vec3(1.5, 2.6, 1.5) }.tongue(Box { size: vec3(0.3, 0.3, 0.3), pos: vec3(1.5, 2.6, 1.5) }, 0.05, 0.05);
let x = Box { size: vec3(0.6, 0.6, 0.6), pos: vec3(-0.5, 0.3, 1.8) }.diff_stairs(Sphere { radius: 0.4, pos: vec3(-0.5, 0.6, 1.8) }, 0.1, 2.0);
let y = Sphere { radius: 0.4, pos: vec3(0.6, 0.4, 1.8) }.noise(3.0, 2.0, 2.0);
let scene = ground + g + h + i + j + k + l + m + n + o + q + r + s + u + v + x + y;
"""


@pytest.mark.parametrize("accel", [ft.AccelMode.Naive, ft.AccelMode.Bvh])
def test_every_node_kind(accel):
    st = ft.parse_and_eval(ALL_KINDS)
    opts = ft.RenderOptions(width=200, height=150, max_steps=256, max_dist=60.0, epsilon=0.0002)
    img = ft.render_depth(st, opts, accel, 1, want_material=True)
    t, m, mat, _, _ = oracle.render_depth(st, opts, int(accel), 1, 32)
    r = assert_depth_parity(img.t, img.mask, t, m, f"all kinds {accel.name}")
    assert r["hits"] > 10000


def test_edge_cases():
    w = workloads.spheres_on_ground(width=1, height=1)
    st = ft.parse_and_eval(w.source)
    img = ft.render_depth(st, w.options, w.accel, 1)
    t, m, _, _, _ = oracle.render_depth(st, w.options, w.accel, 1, 32)
    assert img.mask[0, 0, 0] == m[0, 0, 0]
    # non-square AA sample count (pixel_sample_offsets with a ragged grid)
    w = workloads.spheres_on_ground(width=48, height=40)
    img = ft.render_depth(st, w.options, w.accel, 3)
    t, m, _, rgb, _ = oracle.render_depth(st, w.options, w.accel, 3, 32)
    assert_depth_parity(img.t, img.mask, t, m, "aa3")
    assert np.abs(img.rgb8.astype(int) - rgb.astype(int)).max() <= 1
    # zero step budget: every ray misses
    opts = ft.RenderOptions(width=16, height=16, max_steps=0)
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    assert not img.mask.any() and not img.rgb8.any()
    # camera looking away from the scene
    away = ft.parse_and_eval("let camera = Camera { origin: vec3(0, 50, 0), target: vec3(0, 100, 0) };\n"
                             "let scene = Sphere { radius: 1.0 };")
    img = ft.render_depth(away, ft.RenderOptions(width=32, height=32), ft.AccelMode.Bvh, 1)
    assert not img.mask.any()
    # invalid options are rejected before any launch
    with pytest.raises(ft.RenderError):
        ft.render_depth(st, ft.RenderOptions(width=0, height=8), ft.AccelMode.Bvh, 1)
    with pytest.raises(ft.RenderError):
        ft.render_depth(st, ft.RenderOptions(width=8, height=8, epsilon=0.0), ft.AccelMode.Bvh, 1)


# crates/forgedthoughts/tests/render_regression.rs:48-90 (Whitted, depth 4, aa 1, Bvh)
TRACE_CASES = {
    "ray_metal": dict(width=96, height=96, max_steps=360, max_dist=50.0, epsilon=0.0002, step_scale=0.7,
                      camera_z=6.0, fov_y_degrees=35.0),
    "ray_boolean_union_round": dict(width=96, height=96, max_steps=520, max_dist=60.0, epsilon=0.0002,
                                    step_scale=0.7, camera_z=6.0, fov_y_degrees=25.0),
}


def radiance_rmse(a, b):
    return float(np.sqrt(np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)))


@pytest.mark.parametrize("name", sorted(TRACE_CASES))
def test_gpu_trace_matches_reference_golden(name):
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / f"{name}.ft")
    opts = ft.RenderOptions(**TRACE_CASES[name])
    lin, rgb8 = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 4)
    gold = ft.read_png(FIXTURES / "render_regression" / f"{name}.png")
    diff = np.abs(rgb8.astype(int) - gold.astype(int))
    assert diff.max() <= 8 and diff.mean() <= 0.35, (diff.max(), diff.mean())
    ref, ref8, _ = oracle.render_trace(st, opts, 1, 1, 4, 32)
    assert radiance_rmse(lin, ref) <= 1e-3
    assert np.abs(rgb8.astype(int) - ref8.astype(int)).max() <= 2


def test_gpu_trace_union_round_field_reduced():
    """512-primitive union_round field, Bricks accel, 160x90.

    Up to two bounces the GPU matches the f32 oracle to radiance RMSE <= 1e-3.
    At six bounces reflections and refractions through 15 % dielectrics make
    ray paths sensitive to the last bit: the oracle's own f32 and f64 forms of
    the reference path differ there by more than 1e-3 RMSE.  The bar is then
    99 % of pixels within 1e-3 and an RMSE no larger than that f32-vs-f64 gap.
    """
    w = workloads.union_round_field(width=160, height=90, aa=1)
    st = ft.parse_and_eval(w.source)
    for depth in (1, 2):
        lin, _ = ft.render_trace(st, w.options, w.accel, 1, depth)
        ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))
    lin, _ = ft.render_trace(st, w.options, w.accel, 1, w.max_depth)
    ref32, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, w.max_depth, 32)
    ref64, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, w.max_depth, 64)
    within = (np.abs(lin.astype(np.float64) - ref32).max(axis=2) <= 1e-3).mean()
    assert within >= 0.99, within
    assert radiance_rmse(lin, ref32) <= max(1e-3, radiance_rmse(ref32, ref64)), (
        radiance_rmse(lin, ref32), radiance_rmse(ref32, ref64))


MATERIAL_DEFS_SCENE = """
material Solid {
  model: Lambert;
  let tint = vec3(0.24, 0.5, 0.82);
  color = tint;
};
material Brushed {
  model: Metal;
  color = vec3(0.8, 0.72, 0.3);
  roughness = 0.15;
};
material Glass {
  model: Dielectric;
  ior = 1.45;
};
let camera = Camera { origin: vec3(0.0, 1.2, -4.5), target: vec3(0.0, 0.4, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Solid { tint: vec3(0.7, 0.7, 0.68) } };
let a = Sphere { radius: 0.5, pos: vec3(-1.1, 0.5, 0.0), material: Solid {} };
let b = Sphere { radius: 0.5, pos: vec3(0.0, 0.5, 0.3), material: Brushed {} };
let c = Sphere { radius: 0.5, pos: vec3(1.1, 0.5, 0.0), material: Glass {} };
let scene = ground + a + b + c;
"""


def test_gpu_trace_material_definitions():
    """User material definitions (Lambert-model definitions become Standard
    materials, Metal and Dielectric keep their kind, properties and instance
    overrides applied): Whitted radiance against the f32 oracle."""
    st = ft.parse_and_eval(MATERIAL_DEFS_SCENE)
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    kinds = sorted({st.desc.materials[i].kind for i in range(st.desc.n_materials)})
    assert kinds == [_native.FT_MAT_STANDARD, _native.FT_MAT_METAL, _native.FT_MAT_DIELECTRIC]
    for depth in (1, 3):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))


def test_gpu_trace_material_hooks():
    """Per-hit material hooks (colour, roughness, IOR, thin_walled, evaluated
    on the hit's shading context in the primitive's frame): Whitted radiance
    against the f32 oracle, with the interpreter and with the run-time
    compiled kernels."""
    from test_frontend import HOOK_MATERIALS

    src = HOOK_MATERIALS + """
let camera = Camera { origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.4, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0), material: Stripe {} };
let a = Sphere { radius: 0.5, pos: vec3(-1.1, 0.5, 0.0), material: Stripe {} };
let b = Sphere { radius: 0.5, pos: vec3(0.0, 0.5, 0.3), material: RoughStripe {} };
let c = Sphere { radius: 0.5, pos: vec3(1.1, 0.5, 0.0), material: RippleGlass {} };
let scene = ground + a + b + c;
"""
    st = ft.parse_and_eval(src)
    d = st.desc
    assert any(d.materials[i].color_program >= 0 for i in range(d.n_materials))
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    interp = {}
    for depth in (1, 3):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))
        interp[depth] = lin
    # the stripes are visible: the hooked colours differ from the static ones
    flat = ft.parse_and_eval(src.replace("fn color(ctx)", "fn unused_color(ctx)"))
    lin_flat, _ = ft.render_trace(flat, opts, ft.AccelMode.Bvh, 1, 1)
    assert radiance_rmse(interp[1], lin_flat) > 1e-2
    st.gpu().jit()
    for depth in (1, 3):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        assert radiance_rmse(lin, interp[depth]) <= 1e-3, (depth, radiance_rmse(lin, interp[depth]))


@pytest.mark.parametrize("accel", [ft.AccelMode.Naive, ft.AccelMode.Bvh, ft.AccelMode.Bricks])
def test_gpu_custom_sdf_depth(accel):
    """User `sdf` definitions (helper functions, domain and distance_post
    hooks, vec3 helpers, rotated bounds, the far-box rule of Custom leaves):
    depth against the f32 and f64 oracle."""
    from test_frontend import CUSTOM_SCENE

    st = ft.parse_and_eval(CUSTOM_SCENE)
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    img = ft.render_depth(st, opts, accel, 1, want_material=True)
    assert 0.3 < img.mask.mean() < 0.95
    for prec in (32, 64):
        t, m, mat, _, _ = oracle.render_depth(st, opts, int(accel), 1, prec)
        assert_depth_parity(img.t, img.mask, t, m, f"custom sdf f{prec}")
    both = (img.mask == 1) & (m == 1)
    assert (img.material[both] == mat[both]).mean() >= 0.999


def test_gpu_trace_custom_sdf():
    """Whitted radiance of the custom sdf scene against the f32 oracle, with
    the interpreter and with the run-time compiled kernels."""
    from test_frontend import CUSTOM_SCENE

    st = ft.parse_and_eval(CUSTOM_SCENE)
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    interp = {}
    for depth in (1, 2):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))
        interp[depth] = lin
    st.gpu().jit()
    depth_jit = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    t, m, _, _, _ = oracle.render_depth(st, opts, 1, 1, 32)
    assert_depth_parity(depth_jit.t, depth_jit.mask, t, m, "custom sdf, compiled kernels")
    for depth in (1, 2):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        assert radiance_rmse(lin, interp[depth]) <= 1e-3, (depth, radiance_rmse(lin, interp[depth]))


def test_gpu_trace_material_hooks_in_union_round():
    """Hooked materials blended by a union_round tree (the tree resolve walk
    evaluates each primitive's hooks in its own frame; an instance field
    overrides a binding): Whitted radiance against the f32 oracle."""
    from test_frontend import HOOK_MATERIALS

    src = HOOK_MATERIALS + """
let camera = Camera { origin: vec3(0.0, 1.0, -4.0), target: vec3(0.0, 0.5, 0.0), fov_y: 45.0 };
let light = PointLight { position: vec3(3.0, 6.0, -3.0), intensity: 60.0 };
let ground = Box { size: vec3(20.0, 1.0, 20.0), pos: vec3(0.0, -0.5, 0.0) };
let s0 = Sphere { radius: 0.45, pos: vec3(-0.9, 0.5, 0.0), material: Stripe {} };
let s1 = Sphere { radius: 0.45, pos: vec3(-0.3, 0.6, 0.1), material: RoughStripe {} };
let s2 = Sphere { radius: 0.45, pos: vec3(0.3, 0.5, 0.0), material: Stripe { warm: vec3(0.2, 0.8, 0.3) } };
let s3 = Sphere { radius: 0.45, pos: vec3(0.9, 0.6, -0.1), material: RoughStripe {} };
let blob = s0.union_round(s1, 0.3).union_round(s2.union_round(s3, 0.3), 0.3);
let scene = ground + blob;
"""
    st = ft.parse_and_eval(src)
    opts = ft.RenderOptions(width=160, height=120, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7)
    for depth in (1, 2):
        lin, _ = ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, depth)
        ref, _, _ = oracle.render_trace(st, opts, 1, 1, depth, 32)
        assert radiance_rmse(lin, ref) <= 1e-3, (depth, radiance_rmse(lin, ref))
