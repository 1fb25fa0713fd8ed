"""Parity at the benchmark's own configurations, through the C ABI, against
the CPU oracle on strided bands of the full frames (the oracle would take
hours on a whole 1080p frame; every 45th row and 16th column takes seconds).

* C2, the headline: 512-primitive union_round field, 1920x1080, 2x2 AA,
  Whitted depth 2 and 6, and the jittered-AA variant (seed 1).
* C3: 4096 hooked shells, 1920x1080 depth (interpreter, run-time compiled
  kernels and FP16 bricks) against the FP64 oracle; the 1-bounce shaded pass
  at 1920x1080 with 256 shells (the reference's normal and material walks
  visit both children of every hard union, so a shaded 4096-leaf union costs
  the oracle O(n^2) per hit).
* C4: eight items of the 256-scene batch (depth and Whitted) against the
  oracle.
* C5: the adjoint at the full inverse-fitting configuration (64 primitives,
  449 parameters, 64 views at 256x256) against FP64 central differences on
  32 random parameters (seed 7).
"""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import workloads
from parity import assert_depth_parity, compare_depth, radiance_rmse

pytestmark = pytest.mark.gpu

ROWS = (22, 1080, 45)  # 24 rows of the 1080
COLS = (8, 16)         # 120 columns of the 1920
COLS6 = (8, 32)        # 60 columns: the depth-6 tree costs the oracle about 3x a depth-2 one


def _band(a, rows=ROWS, cols=COLS):
    return a[rows[0]:rows[1]:rows[2], cols[0]::cols[1]]


@pytest.fixture(scope="module")
def field():
    w = workloads.union_round_field()
    return w, ft.parse_and_eval(w.source)


def test_c2_trace_full_frame_depth2(field):
    """1-bounce Whitted (depth 2) of the full 1080p frame: radiance RMSE <= 1e-3
    against the f32 oracle."""
    w, st = field
    lin, _ = ft.render_trace(st, w.options, w.accel, w.aa, 2)
    ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 2, 32, rows=ROWS, cols=COLS)
    e = radiance_rmse(_band(lin), _band(ref))
    assert e <= 1e-3, e


def _chaotic_bar(lin, ref32, ref64):
    """Depth 6 through 15 % dielectrics: a tie in a refraction chain flips a
    whole sub-tree, so the f32 and f64 oracle already differ.  Bar: 99 % of
    pixels within 1e-3, RMSE no larger than max(1e-3, oracle f32-vs-f64)."""
    gap = radiance_rmse(ref32, ref64)
    e = radiance_rmse(lin, ref32)
    within = float((np.abs(lin.astype(np.float64) - ref32).max(axis=-1) <= 1e-3).mean())
    assert within >= 0.99, (within, e, gap)
    assert e <= max(1e-3, gap), (e, gap)
    return e, gap


def test_c2_trace_full_frame_depth6(field):
    """The headline configuration itself: 1920x1080, 2x2 AA, depth 6."""
    w, st = field
    lin, _ = ft.render_trace(st, w.options, w.accel, w.aa, 6)
    ref32, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 6, 32, rows=ROWS, cols=COLS6)
    ref64, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 6, 64, rows=ROWS, cols=COLS6)
    e, gap = _chaotic_bar(_band(lin, cols=COLS6), _band(ref32, cols=COLS6), _band(ref64, cols=COLS6))
    print(f"C2 depth 6: RMSE vs f32 oracle {e:.2e}, oracle f32 vs f64 {gap:.2e}")


def test_c2_jittered_seed1(field):
    """The jittered 4-spp variant (XorShift64 per pixel sample, seed 1): the
    depth march and the Whitted trace against the oracle's own jittered
    samples."""
    w, st = field
    img = ft.render_depth(st, w.options, w.accel, w.aa, jitter_seed=1)
    t, m, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, 32, rows=ROWS, cols=COLS, jitter_seed=1)
    assert_depth_parity(_band(img.t), _band(img.mask), _band(t), _band(m), "C2 jittered depth")
    grid = ft.render_depth(st, w.options, w.accel, w.aa)
    assert (grid.t != img.t).mean() > 0.5  # the offsets differ from the grid's
    lin, _ = ft.render_trace(st, w.options, w.accel, w.aa, 2, jitter_seed=1)
    ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 2, 32, rows=ROWS, cols=COLS, jitter_seed=1)
    assert radiance_rmse(_band(lin), _band(ref)) <= 1e-3
    lin6, _ = ft.render_trace(st, w.options, w.accel, w.aa, 6, jitter_seed=1)
    ref32, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 6, 32, rows=ROWS, cols=COLS6, jitter_seed=1)
    ref64, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, 6, 64, rows=ROWS, cols=COLS6, jitter_seed=1)
    _chaotic_bar(_band(lin6, cols=COLS6), _band(ref32, cols=COLS6), _band(ref64, cols=COLS6))


def test_c3_hooked_shells_full_frame_depth():
    """4096 shells with domain and distance_post hooks at 1920x1080: mask and
    depth against the FP64 oracle (and f32), for the interpreted hooks, the
    run-time compiled kernels and the FP16 brick form."""
    w = workloads.twisted_shells()
    st = ft.parse_and_eval(w.source)
    t64, m64, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), 1, 64, rows=ROWS, cols=COLS)
    t32, m32, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), 1, 32, rows=ROWS, cols=COLS)
    assert _band(m64).mean() > 0.05
    imgs = {"interpreter": ft.render_depth(st, w.options, w.accel, 1)}
    st.gpu().jit()
    imgs["compiled"] = ft.render_depth(st, w.options, w.accel, 1)
    st.gpu().build_bricks()
    imgs["fp16_bricks"] = ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    for name, img in imgs.items():
        r = assert_depth_parity(_band(img.t), _band(img.mask), _band(t64), _band(m64), f"C3 {name} vs f64")
        assert r["depth_err_q"] <= 1e-4, (name, r)
        assert_depth_parity(_band(img.t), _band(img.mask), _band(t32), _band(m32), f"C3 {name} vs f32")


def test_c3_shaded_full_frame():
    """C3's 1-bounce shading (Whitted depth 2) at 1920x1080, with 256 of the
    hooked shells, interpreted, compiled, and compiled with the primary hits
    from the FP16 brick march.

    The reference resolves a hit's normal and material by walking the scene
    root's hard unions with sdf_distance_info, whose union culling trusts each
    subtree's box lower bound.  A shell carries both hooks, so its transform
    applies twice and its surface lies partly outside its box: at a few hits
    that walk is culled away from the shell the march hit and takes another
    shell's normal.  The GPU resolves at the leaf its accelerator hit.  So:
    against the f32 oracle resolving at that leaf, radiance RMSE <= 1e-3
    where the primary hits agree; against the reference-resolving oracle,
    98.5 % of the pixels within 1e-3 (4 of the 360 band pixels take the other
    shell's normal there)."""
    w = workloads.twisted_shells(n=256)
    st = ft.parse_and_eval(w.source)
    rows, cols = (22, 1080, 90), (8, 64)
    ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, 2, 32, rows=rows, cols=cols)
    with oracle.resolve_at_hit_leaf():
        ref_leaf, _, _ = oracle.render_trace(st, w.options, int(w.accel), 1, 2, 32, rows=rows, cols=cols)
    t, m, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), 1, 32, rows=rows, cols=cols)
    img = ft.render_depth(st, w.options, w.accel, 1)
    # the thin banded shells put a primary hit on another shell now and then
    # (within the depth bar's 0.1 %); radiance is compared where the primary
    # hits agree
    def agreement(img):
        return _band((img.mask[..., 0] == m[..., 0]) & (np.abs(img.t[..., 0] - t[..., 0]) <= 1e-4), rows, cols)

    agree = agreement(img)
    assert agree.mean() >= 0.99
    results = {"interpreter": (ft.render_trace(st, w.options, w.accel, 1, 2)[0], agree)}
    st.gpu().jit()
    results["compiled"] = (ft.render_trace(st, w.options, w.accel, 1, 2)[0], agree)
    st.gpu().build_bricks()
    bagree = agreement(ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True))
    assert bagree.mean() >= 0.99
    results["compiled_fp16_bricks"] = (ft.render_trace(st, w.options, w.accel, 1, 2, fp16_bricks=True)[0], bagree)
    b, bl = _band(ref, rows, cols), _band(ref_leaf, rows, cols)
    for label, (lin, ok) in results.items():
        a = _band(lin, rows, cols)
        assert radiance_rmse(a[ok], bl[ok]) <= 1e-3, (label, radiance_rmse(a[ok], bl[ok]))
        within = float((np.abs(a.astype(np.float64) - b).max(axis=-1) <= 1e-3).mean())
        assert within >= 0.985, (label, within, radiance_rmse(a[ok], b[ok]))


def _spheres(w):
    return int(w.name.split("_spheres")[1].split("_")[0])


def test_c4_batch_items_against_oracle():
    """Eight items of the 256-scene batch (four depth previews, four Whitted
    depth 2), rendered in one batch launch: each against the oracle.  The
    Whitted items are the batch's smallest hard unions: the oracle restates
    the reference's normal and material walks, which visit both children of
    every union, so a shaded hit on an n-sphere union costs it O(n^2)."""
    ws = workloads.batch_scenes()
    depth = [w for w in ws if w.max_depth == 0 and w.options.width <= 256][:4]
    trace = sorted((w for w in ws if w.max_depth > 0 and w.options.width <= 256), key=_spheres)[:4]
    assert max(_spheres(w) for w in trace) <= 64
    picked = depth + trace
    states = [ft.parse_and_eval(w.source) for w in picked]
    b = ft.Batch([(st, w.options, w.aa, w.max_depth) for st, w in zip(states, picked)])
    b.autotune()
    b.launch()
    for k, (st, w) in enumerate(zip(states, picked)):
        got = b.read(k)
        if w.max_depth == 0:
            t, m, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, 32)
            assert_depth_parity(got["t"], got["mask"], t, m, w.name)
            t64, m64, _, _, _ = oracle.render_depth(st, w.options, int(w.accel), w.aa, 64)
            r = compare_depth(got["t"], got["mask"], t64, m64)
            assert r["mask_agreement"] >= 0.999 and r["depth_within_tol"] >= 0.999, (w.name, r)
        else:
            ref, _, _ = oracle.render_trace(st, w.options, int(w.accel), w.aa, w.max_depth, 32)
            assert radiance_rmse(got["rgb"], ref) <= 1e-3, (w.name, radiance_rmse(got["rgb"], ref))
    b.close()


def test_c5_adjoint_against_finite_differences_full_config():
    """The inverse-fitting configuration itself: 64 primitives (449
    parameters), 64 views at 256x256, 32 random parameters (seed 7), FP64
    central differences with h = 1e-4 of the FP64 forward.  The loss is a
    random linear functional of depth and silhouette on every 16th pixel in x
    and y of every view (16,384 rays per forward), so the FP64 forwards of
    the 64 perturbed scenes take seconds.  Excluded pixels, as in the
    analytic-gradient test: misses passing within ~1e-3 of a surface
    (silhouette above exp(-0.02), ill-conditioned in FP32), pixels whose hit
    state flips under a step, and kinks: pixels whose forward and backward
    differences disagree, where central differences measure the kink rather
    than the derivative (the FP64 analytic gradient disagrees with them there
    exactly as the GPU's does: about 0.4 % of the depth pixels and 0.05 % of
    the silhouette pixels).  Bar: relative error <= 1e-3 on all 32."""
    ps = ft.ParamScene(workloads.shape_fit())
    opts = workloads.shape_fit_options(256)
    vs = ft.ring_views(64)
    assert ps.n_params == 449
    stride, off = 16, 7
    theta = ps.get_params()
    t, m, sil = oracle.render_views(ps.state, vs, opts, 0.05, 64, stride=stride, offset=off)
    tg, mg, _ = ps.render(vs, opts)
    sample = np.zeros(t.shape, bool)
    sample[:, off::stride, off::stride] = True
    rng = np.random.default_rng(7)
    same = (mg == m) & sample
    wt = rng.normal(size=t.shape) * (m == 1) * same
    ws = rng.normal(size=t.shape) * (m == 0) * same * (sil < np.exp(-0.02))
    idx = rng.choice(ps.n_params, size=32, replace=False)
    h = 1e-4
    keep = np.ones(t.shape, bool)
    runs = {}
    for k in idx:
        for sgn in (1, -1):
            th = theta.copy()
            th[k] = np.float32(theta[k] + sgn * h)
            ps.set_params(th)
            tt, mm, ss = oracle.render_views(ps.state, vs, opts, 0.05, 64, stride=stride, offset=off)
            runs[(k, sgn)] = (tt, ss, float(th[k]))
            keep &= mm == m
    # kinks: where a pixel's forward and backward differences disagree (by
    # more than 5 % of the central difference) its depth or silhouette is not
    # differentiable at the step's scale (an occlusion edge, a switch of the
    # nearest primitive or of the silhouette's minimum); central differences
    # there measure the kink, not the derivative, so the pixel leaves that
    # term for every parameter
    kink_t = np.zeros(t.shape, bool)
    kink_s = np.zeros(t.shape, bool)
    for k in idx:
        tp, tn = runs[(k, 1)][0], runs[(k, -1)][0]
        sp, sn = runs[(k, 1)][1], runs[(k, -1)][1]
        kink_t |= np.abs((tp - t) - (t - tn)) > 0.05 * np.abs(tp - tn) + 1e-9
        kink_s |= np.abs((sp - sil) - (sil - sn)) > 0.05 * np.abs(sp - sn) + 1e-9
    print("C5 kinks excluded: depth", int((kink_t & (wt != 0)).sum()), "of", int((wt != 0).sum()),
          "silhouette", int((kink_s & (ws != 0)).sum()), "of", int((ws != 0).sum()))
    wt = wt * keep * ~kink_t
    ws = ws * ~kink_s
    fd = np.array([((wt * runs[(k, 1)][0]).sum() + (ws * runs[(k, 1)][1]).sum() - (wt * runs[(k, -1)][0]).sum()
                    - (ws * runs[(k, -1)][1]).sum()) / (runs[(k, 1)][2] - runs[(k, -1)][2]) for k in idx])
    ps.set_params(theta)
    g = ps.backward(vs, opts, wt.astype(np.float32), ws.astype(np.float32))[idx]
    scale = np.abs(fd).max()
    assert scale > 0
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    print("C5 FD relative errors: max", rel.max(), "median", np.median(rel))
    assert np.all(rel <= 1e-3), (idx[rel > 1e-3], g[rel > 1e-3], fd[rel > 1e-3], rel[rel > 1e-3])
