"""The work counters behind the FP32 roofline, against counts derived by hand
from the march's structure (raymarch_hit R:4091-4139: every hit takes its
march steps, then 10 bisections, 6 normal taps and one final lookup).

* One sphere: the scene is a single primitive leaf, so every distance
  evaluation is exactly one primitive and no culling box is tested.
* A ground box and one sphere: the two-leaf BVH tests both child boxes on
  every evaluation, and the second leaf is evaluated only when its box bound
  is not above the first leaf's distance.
* The Whitted trace's wavefront march counts the same way per ray job.
Calls go through the C ABI."""
import ctypes

import numpy as np
import pytest

import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native

pytestmark = pytest.mark.gpu

CAM = "let camera = Camera { origin: vec3(0.3, 0.7, -4), target: vec3(0, 0.4, 0), fov_y: 40.0 };\n"


def _opts(w=64, h=48):
    return ft.RenderOptions(width=w, height=h, max_steps=256, max_dist=50.0, epsilon=1e-4, step_scale=0.7,
                            camera_z=6.0, fov_y_degrees=40.0)


def _depth_stats(st, opts, accel):
    s = _native.RenderStatsC()
    rc = _native.lib().ft_render_depth_stats(st.gpu().handle, ctypes.byref(opts.to_c()), int(accel), 1, 0,
                                             ctypes.byref(s))
    assert rc == 0, _native.last_error()
    return s


@pytest.mark.parametrize("accel", [ft.AccelMode.Naive, ft.AccelMode.Bvh])
def test_single_sphere_counts(accel):
    st = ft.parse_and_eval(CAM + "let scene = Sphere { radius: 0.6, pos: vec3(0, 0.4, 0) };\n")
    opts = _opts()
    img = ft.render_depth(st, opts, accel, 1)
    hits = int(img.mask.sum())
    assert 0 < hits < img.mask.size
    s = _depth_stats(st, opts, accel)
    assert s.rays == opts.width * opts.height
    assert s.distance_evals == s.march_steps + 17 * hits
    assert s.primitive_evals == s.distance_evals
    assert s.box_tests == 0 and s.blend_ops == 0 and s.candidate_entries == 0


def test_ground_and_sphere_counts():
    src = CAM + ft_ground() + "let ball = Sphere { radius: 0.5, pos: vec3(0, 0.5, 0) };\nlet scene = ground + ball;\n"
    st = ft.parse_and_eval(src)
    opts = _opts()
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    hits = int(img.mask.sum())
    s = _depth_stats(st, opts, ft.AccelMode.Bvh)
    assert s.distance_evals == s.march_steps + 17 * hits
    assert s.box_tests == 2 * s.distance_evals
    assert s.distance_evals <= s.primitive_evals <= 2 * s.distance_evals


def test_union_round_counts_bounded_by_structure():
    # four spheres in a balanced union_round tree (three inner nodes): the
    # restricted fold of a point combines at most once per inner node, and
    # not at all where no primitive is within the blend radius
    src = CAM + "".join(f"let s{i} = Sphere {{ radius: 0.35, pos: vec3({-0.75 + 0.5 * i}, 0.4, 0) }};\n"
                        for i in range(4))
    src += "let scene = s0.union_round(s1, 0.2).union_round(s2.union_round(s3, 0.2), 0.2);\n"
    st = ft.parse_and_eval(src)
    opts = _opts()
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    hits = int(img.mask.sum())
    s = _depth_stats(st, opts, ft.AccelMode.Bvh)
    assert s.distance_evals == s.march_steps + 17 * hits
    assert 0 < s.blend_ops <= 3 * s.distance_evals
    assert s.primitive_evals <= 4 * s.distance_evals


def test_trace_kernel_counts_sum_to_the_trace_counts():
    src = CAM + ft_ground() + ("let ball = Sphere { radius: 0.5, pos: vec3(0, 0.5, 0) };\n"
                               "let scene = ground + ball;\n"
                               "let light = PointLight { position: vec3(2, 4, -2), intensity: 20.0 };\n")
    st = ft.parse_and_eval(src)
    opts = _opts()
    lib = _native.lib()
    k = [_native.RenderStatsC() for _ in range(3)]
    rc = lib.ft_render_trace_kernel_stats(st.gpu().handle, ctypes.byref(opts.to_c()), 1, 1, 2,
                                          *[ctypes.byref(x) for x in k])
    assert rc == 0, _native.last_error()
    tot = _native.RenderStatsC()
    assert lib.ft_render_trace_stats(st.gpu().handle, ctypes.byref(opts.to_c()), 1, 1, 2, ctypes.byref(tot)) == 0
    for f in ("distance_evals", "primitive_evals", "box_tests", "march_steps"):
        assert getattr(tot, f) == sum(getattr(x, f) for x in k), f
    march = k[0]
    # every march job: its steps, plus 17 evaluations when it hits; the primary
    # level alone hits on the depth march's hit samples
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    extra = march.distance_evals - march.march_steps
    hit_jobs = extra // 17
    assert extra % 17 == 0 and hit_jobs >= int(img.mask.sum())
    # the final lookup of a hit walks the leaf BVH for the hit leaf without
    # the two-box test of the other evaluations
    assert march.box_tests == 2 * (march.distance_evals - hit_jobs)
    # shadow jobs step on the leaf-box lower bound first
    assert k[2].box_tests > 0


def test_kernel_times_cover_every_launch():
    st = ft.parse_and_eval(CAM + ft_ground() + "let scene = ground + Sphere { radius: 0.5, pos: vec3(0, 0.5, 0) };\n")
    opts = _opts(96, 64)
    lib = _native.lib()
    g = st.gpu()
    assert lib.ft_scene_profile(g.handle, 1) == 0
    for _ in range(2):
        ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 3)
    n = ctypes.c_uint32(0)
    lib.ft_scene_last_launches(g.handle, ctypes.byref(n))
    kt = _native.KernelTimesC()
    assert lib.ft_scene_kernel_times(g.handle, ctypes.byref(kt)) == 0
    assert sum(kt.launches) == 2 * n.value
    assert kt.launches[_native.FT_KERNEL_PRIMARY] == 2 and kt.launches[_native.FT_KERNEL_PIXELS] == 2
    assert all(kt.ms[i] > 0 for i in range(_native.FT_KERNEL_KINDS) if kt.launches[i])
    assert lib.ft_scene_profile(g.handle, 0) == 0
    ft.render_trace(st, opts, ft.AccelMode.Bvh, 1, 3)
    kt2 = _native.KernelTimesC()
    assert lib.ft_scene_kernel_times(g.handle, ctypes.byref(kt2)) == 0
    assert sum(kt2.launches) == 0


def ft_ground():
    from forgedthoughts_gb300 import workloads

    return workloads.GROUND
