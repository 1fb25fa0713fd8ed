"""FP16 brick precision form of the depth march against the plain FP32 march
on the GPU and against the FP64 CPU oracle (through the C ABI)."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import workloads
from parity import DEPTH_TOL, MASK_AGREEMENT, compare_depth, radiance_rmse

pytestmark = pytest.mark.gpu


def _both(st, w, accel):
    plain = ft.render_depth(st, w.options, accel, w.aa, want_material=True, want_normal=True)
    fp16 = ft.render_depth(st, w.options, accel, w.aa, want_material=True, want_normal=True, fp16_bricks=True)
    return plain, fp16


def _check_against(plain, fp16, t_ref, m_ref, what):
    r_plain = compare_depth(plain.t, plain.mask, t_ref, m_ref)
    r_fp16 = compare_depth(fp16.t, fp16.mask, t_ref, m_ref)
    # the precision form meets the plain method's bar against the same reference
    assert r_fp16["mask_agreement"] >= MASK_AGREEMENT, (what, r_fp16, r_plain)
    assert r_fp16["depth_within_tol"] >= MASK_AGREEMENT, (what, r_fp16, r_plain)
    return r_fp16


def test_brick_build_info_and_errors():
    w = workloads.spheres_on_ground()
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    with pytest.raises(ft.RenderError, match="ft_scene_build_bricks"):
        ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    with pytest.raises(ft.RenderError):
        g.build_bricks(voxel_size=1e-6)
    with pytest.raises(ft.RenderError, match="max_lattice_points"):
        g.build_bricks(voxel_size=0.02, max_lattice_points=1000)
    info = g.build_bricks()
    assert info.exact_leaves == 1  # the ground slab
    assert info.near_bricks > 0 and info.device_bytes > 0
    assert 1.0 <= info.max_lipschitz < 2.0
    for a in range(3):
        assert info.region_max[a] > info.region_min[a]
    # rebuilding replaces the cache
    info2 = g.build_bricks(voxel_size=0.04)
    assert info2.near_bricks < info.near_bricks


@pytest.mark.parametrize("wl", ["spheres", "union_round"])
def test_far_field_is_a_lower_bound(wl):
    if wl == "spheres":
        w = workloads.spheres_on_ground()
    else:
        w = workloads.union_round_field(width=64, height=36, aa=1)
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    info = g.build_bricks()
    rng = np.random.default_rng(5)
    lo, hi = np.array(info.region_min), np.array(info.region_max)
    pts = rng.uniform(lo, hi, size=(200_000, 3)).astype(np.float32)
    bound, exact = g.brick_bounds(pts)
    assert not np.isnan(bound).any()  # all points inside the region
    over = bound - exact
    # a lower bound wherever the march can use it: outside solids (inside
    # overlapping solids the reference's culled field jumps)
    outside = exact >= 0.0
    assert (over[outside] <= 1e-5).all(), float(over[outside].max())
    # and a useful one: within a brick diagonal (0.28) plus the error bound
    far = exact > 0.5
    assert np.median(exact[far] - bound[far]) < 0.35
    # outside the region there is no bound (the march is exact there)
    b2, _ = g.brick_bounds((np.array(info.region_max) + 1.0)[None, :].astype(np.float32))
    assert np.isnan(b2[0])


def test_spheres_on_ground_fp16_vs_oracle():
    w = workloads.spheres_on_ground()  # 256x256, 8 spheres, Naive
    st = ft.parse_and_eval(w.source)
    st.gpu().build_bricks()
    plain, fp16 = _both(st, w, w.accel)
    for precision in (32, 64):
        t, m, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, precision)
        r = _check_against(plain, fp16, t, m, f"spheres f{precision}")
        print(precision, r)
    both = (plain.mask == 1) & (fp16.mask == 1)
    assert (plain.material[both] == fp16.material[both]).mean() >= 0.999
    cos = (plain.normal[both] * fp16.normal[both]).sum(-1)
    assert np.quantile(cos, 0.001) > 0.999


def test_union_round_field_fp16_vs_plain_and_oracle():
    w = workloads.union_round_field(width=320, height=180, aa=1)
    st = ft.parse_and_eval(w.source)
    info = st.gpu().build_bricks()
    assert info.exact_leaves == 1
    plain, fp16 = _both(st, w, w.accel)
    r = compare_depth(fp16.t, fp16.mask, plain.t, plain.mask)
    assert r["mask_agreement"] >= MASK_AGREEMENT and r["depth_within_tol"] >= MASK_AGREEMENT, r
    t64, m64, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), 1, 64)
    r64 = _check_against(plain, fp16, t64, m64, "union_round f64")
    assert r64["depth_err_q"] <= DEPTH_TOL, r64
    both = (plain.mask == 1) & (fp16.mask == 1)
    assert (plain.material[both] == fp16.material[both]).mean() >= 0.999


def test_union_round_field_fp16_full_frame_against_plain():
    """1920x1080 with the 2x2 AA grid: the whole frame against the plain march."""
    w = workloads.union_round_field()
    st = ft.parse_and_eval(w.source)
    st.gpu().build_bricks()
    plain, fp16 = _both(st, w, w.accel)
    r = compare_depth(fp16.t, fp16.mask, plain.t, plain.mask)
    assert r["mask_agreement"] >= MASK_AGREEMENT and r["depth_within_tol"] >= MASK_AGREEMENT, r
    assert r["depth_err_q"] <= DEPTH_TOL, r
    # deterministic
    again = ft.render_depth(st, w.options, w.accel, w.aa, fp16_bricks=True)
    assert np.array_equal(again.t, fp16.t) and np.array_equal(again.mask, fp16.mask)


def test_twisted_shells_fp16_vs_plain_and_oracle():
    w = workloads.twisted_shells(n=512, width=192, height=108)
    st = ft.parse_and_eval(w.source)
    info = st.gpu().build_bricks()
    assert info.exact_leaves == 1
    plain, fp16 = _both(st, w, w.accel)
    r = compare_depth(fp16.t, fp16.mask, plain.t, plain.mask)
    assert r["mask_agreement"] >= MASK_AGREEMENT, r
    t64, m64, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), 1, 64)
    r64 = compare_depth(fp16.t, fp16.mask, t64, m64)
    p64 = compare_depth(plain.t, plain.mask, t64, m64)
    # no worse than the plain FP32 march against the FP64 oracle
    assert r64["mask_agreement"] >= min(MASK_AGREEMENT, p64["mask_agreement"]), (r64, p64)
    assert r64["depth_within_tol"] >= min(MASK_AGREEMENT, p64["depth_within_tol"]), (r64, p64)


def test_trace_primary_hits_from_bricks():
    """A Whitted trace (depth 2) whose primary hits come from the FP16 brick
    march: where its primary hit agrees with the plain march's, the radiance
    is the plain trace's, and against the f32 oracle its radiance RMSE is
    <= 1e-3 and no worse than the plain trace's on those pixels.  The primary
    hits themselves agree on >= 99.9 % of the pixels (the precision form's
    depth bar).  A pixel whose hit flips at a silhouette changes its radiance
    by up to the whole sky-to-surface contrast, so the radiance bar is taken
    where the hits agree.  The frame is 160x90: at 320x180 the oracle's own
    f32 and f64 traces differ by RMSE 2.3e-3 at depth 2 (six pixels whose
    reflected ray lands elsewhere), against 1.2e-4 at 160x90."""
    w = workloads.union_round_field(width=160, height=90, aa=1)
    st = ft.parse_and_eval(w.source)
    st.gpu().build_bricks()
    plain, fp16 = _both(st, w, w.accel)
    lin_p, _ = ft.render_trace(st, w.options, w.accel, 1, 2)
    lin_b, rgb8_b = ft.render_trace(st, w.options, w.accel, 1, 2, fp16_bricks=True)
    same = (plain.mask[..., 0] == fp16.mask[..., 0]) & (plain.t[..., 0] == fp16.t[..., 0])
    close = (plain.mask[..., 0] == fp16.mask[..., 0]) & (np.abs(plain.t[..., 0] - fp16.t[..., 0]) <= 1e-4)
    assert close.mean() >= MASK_AGREEMENT
    # identical primary hit: identical shading up to FMA contraction
    assert np.abs(lin_b[same] - lin_p[same]).max() <= 1e-4
    ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, 2, 32)
    rm_close = radiance_rmse(lin_b[close], ref[close])
    assert rm_close <= 1e-3, (rm_close, radiance_rmse(lin_b, ref), int((~close).sum()))
    assert rm_close <= radiance_rmse(lin_p[close], ref[close]) + 1e-4
    # repeatable up to the order of the radiance atomics, and the 8-bit image
    # is the linear one's tone map
    again, _ = ft.render_trace(st, w.options, w.accel, 1, 2, fp16_bricks=True)
    assert np.allclose(again, lin_b, rtol=1e-5, atol=1e-6)
    assert rgb8_b.shape == (w.options.height, w.options.width, 3)


def test_trace_bricks_flag_needs_a_brick_cache():
    w = workloads.spheres_on_ground(8, 0, 64, 64)
    st = ft.parse_and_eval(w.source)
    with pytest.raises(ft.RenderError, match="ft_scene_build_bricks"):
        ft.render_trace(st, w.options, w.accel, 1, 2, fp16_bricks=True)


def test_brick_stats_count_far_steps():
    w = workloads.union_round_field(width=160, height=90, aa=1)
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    g.build_bricks()
    import ctypes

    from forgedthoughts_gb300 import _native

    lib = _native.lib()
    opts = w.options.to_c()
    s_plain, s_fp16 = _native.RenderStatsC(), _native.RenderStatsC()
    assert lib.ft_render_depth_stats(g.handle, ctypes.byref(opts), int(w.accel), 1, 0, ctypes.byref(s_plain)) == 0
    assert lib.ft_render_depth_stats(g.handle, ctypes.byref(opts), int(w.accel), 1, _native.FT_FLAG_FP16_BRICKS,
                                     ctypes.byref(s_fp16)) == 0
    assert s_plain.far_steps == 0 and s_plain.brick_fetches == 0
    assert s_fp16.far_steps > 0 and s_fp16.brick_fetches > 0
    # the precision form replaces most exact evaluations by far-field steps
    assert s_fp16.distance_evals < s_plain.distance_evals


def _limited(max_steps):
    import dataclasses

    w = workloads.union_round_field(width=480, height=270, aa=1)
    return w, dataclasses.replace(w.options, max_steps=max_steps)


def test_counted_form_keeps_the_plain_step_limit():
    """With a step limit of 96 the plain march gives up on the grazing ground
    rays (a band below the horizon).  The counted brick form follows the plain
    samples and counts the ground descent in closed form, so it gives up on
    the same rays and agrees with the plain march and the FP64 oracle."""
    w, opts = _limited(96)
    st = ft.parse_and_eval(w.source)
    st.gpu().build_bricks()
    plain = ft.render_depth(st, opts, w.accel, 1)
    full = ft.render_depth(st, w.options, w.accel, 1)
    assert plain.mask.mean() < full.mask.mean() - 0.01  # the limit bites
    fp16 = ft.render_depth(st, opts, w.accel, 1, fp16_bricks=True)
    r = compare_depth(fp16.t, fp16.mask, plain.t, plain.mask)
    assert r["mask_agreement"] >= MASK_AGREEMENT and r["depth_within_tol"] >= MASK_AGREEMENT, r
    t64, m64, _, _, _ = oracle.render_depth(st, opts, int(w.accel), 1, 64)
    r64 = compare_depth(fp16.t, fp16.mask, t64, m64)
    p64 = compare_depth(plain.t, plain.mask, t64, m64)
    assert r64["mask_agreement"] >= min(MASK_AGREEMENT, p64["mask_agreement"]), (r64, p64)
    assert r64["depth_within_tol"] >= min(MASK_AGREEMENT, p64["depth_within_tol"]), (r64, p64)


def test_counted_form_skips_most_evaluations():
    """On the 512-primitive field the ground descents taken in closed form
    (and secant hit refinement) leave far fewer evaluations than the plain
    march, and the free far-field form keeps working beside it."""
    import ctypes

    from forgedthoughts_gb300 import _native

    w = workloads.union_round_field(width=320, height=180, aa=1)
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    g.build_bricks()
    lib = _native.lib()
    opts = w.options.to_c()
    s_plain, s_fp16 = _native.RenderStatsC(), _native.RenderStatsC()
    assert lib.ft_render_depth_stats(g.handle, ctypes.byref(opts), int(w.accel), 1, 0, ctypes.byref(s_plain)) == 0
    assert lib.ft_render_depth_stats(g.handle, ctypes.byref(opts), int(w.accel), 1, _native.FT_FLAG_FP16_BRICKS,
                                     ctypes.byref(s_fp16)) == 0
    assert s_fp16.far_steps > 0  # ground descents taken in closed form
    assert s_fp16.distance_evals < 0.75 * s_plain.distance_evals, (s_fp16.distance_evals, s_plain.distance_evals)
    plain = ft.render_depth(st, w.options, w.accel, 1)
    g.build_bricks(free_far_steps=True)
    free = ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    r = compare_depth(free.t, free.mask, plain.t, plain.mask)
    assert r["mask_agreement"] >= MASK_AGREEMENT and r["depth_within_tol"] >= MASK_AGREEMENT, r
