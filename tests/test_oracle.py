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


def test_trace_f32_tracks_f64():
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / "ray_boolean_union_round.ft")
    opts = ft.RenderOptions(**TRACE_CASES["ray_boolean_union_round"])
    a, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 32)
    b, _, _ = oracle.render_trace(st, opts, 1, 1, 4, 64)
    assert np.sqrt(np.mean((a - b) ** 2)) <= 1e-3
