"""Differentiation form on the CPU: the parameter layout, and the FP64
restatement's analytic adjoint against FP64 central finite differences."""
import ctypes

import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import _native, workloads


def test_layout_counts_and_roundtrip():
    ps = ft.ParamScene(workloads.shape_fit())
    assert ps.n_params == 64 * 7 + 1
    names = ps.names()
    assert names[-1].endswith(".radius")
    v = ps.get_params()
    assert abs(v[-1] - 0.15) < 1e-7
    w = v.copy()
    w[0] += 0.25
    w[-1] = 0.2
    ps.set_params(w)
    assert np.array_equal(ps.get_params(), w)
    # every union_round node now carries the new radius
    d = ps.state.desc
    radii = {d.nodes[i].f[0] for i in range(d.n_nodes) if d.nodes[i].kind == 11}
    assert radii == {np.float32(0.2)}


@pytest.mark.parametrize("src, msg", [
    ("let a = Sphere { radius: 0.5 }; let b = Sphere { radius: 0.3, pos: vec3(1, 0, 0), rot: vec3(10, 0, 0) };"
     " let scene = a.union_round(b, 0.1);", "rotation"),
    ("let a = Sphere { radius: 0.5 }; let b = Torus { major_radius: 0.5, minor_radius: 0.1 };"
     " let scene = a.union_round(b, 0.1);", "node kind"),
])
def test_layout_rejects_undifferentiable_trees(src, msg):
    with pytest.raises(ft.RenderError, match=msg):
        ft.ParamScene(src)


def test_layout_of_scene_without_trees_is_empty():
    ps = ft.ParamScene("let scene = Sphere { radius: 0.5 } + Box { size: vec3(1, 1, 1), pos: vec3(2, 0, 0) };")
    assert ps.n_params == 0


def test_set_params_validation():
    ps = ft.ParamScene(workloads.shape_fit(n=4))
    with pytest.raises(ValueError):
        ps.set_params(np.zeros(3))
    bad = ps.get_params()
    bad[0] = np.nan
    with pytest.raises(ft.RenderError):
        ps.set_params(bad)


def _fd_setup(n_prims=8, size=20, views=2):
    src = workloads.shape_fit(n=n_prims)
    ps = ft.ParamScene(src)
    opts = workloads.shape_fit_options(size)
    vs = ft.ring_views(views)
    return ps, opts, vs


def test_oracle_forward_definitions():
    ps, opts, vs = _fd_setup(size=24)
    t, m, sil = oracle.render_views(ps.state, vs, opts, 0.05, 64)
    assert m.any() and (~m.astype(bool)).any()
    assert np.all(sil[m == 1] == 1.0)
    miss = m == 0
    assert np.all((sil[miss] >= 0.0) & (sil[miss] < 1.0))
    # depth is the zero of f: the distance at the hit points is ~0
    vc = ft.views_c(vs)
    pts = []
    for v in range(len(vs)):
        o = np.array(vc[v].origin[:], np.float64)
        tg = np.array(vc[v].target[:], np.float64)
        f = (tg - o) / np.linalg.norm(tg - o)
        r = np.cross(f, [0, 1, 0]); r /= np.linalg.norm(r)
        u = np.cross(r, f); u /= np.linalg.norm(u)
        th = np.tan(0.5 * np.radians(vc[v].fov_y_degrees))
        ys, xs = np.nonzero(m[v])
        for y, x in zip(ys, xs):
            px = ((x + 0.5) / opts.width) * 2 - 1
            py = 1 - ((y + 0.5) / opts.height) * 2
            d = f + r * px * th + u * py * th
            d /= np.linalg.norm(d)
            pts.append(o + d * t[v, y, x])
    dist, _, _ = oracle.distance(ps.state, np.array(pts), 1, 64)
    assert np.abs(dist).max() < 2e-5


def test_oracle_adjoint_matches_fp64_finite_differences():
    """32 random parameters, FP64 central differences (h = 1e-4) of a fixed
    random weighting of depth (hit pixels) and silhouette (miss pixels)."""
    ps, opts, vs = _fd_setup()
    theta = ps.get_params()
    rng = np.random.default_rng(7)
    t, m, sil = oracle.render_views(ps.state, vs, opts, 0.05, 64)
    wt = rng.normal(size=t.shape) * (m == 1)
    ws = rng.normal(size=t.shape) * (m == 0)
    h = 1e-4
    idx = rng.choice(ps.n_params, size=min(32, ps.n_params), replace=False)
    keep_t = np.ones(t.shape, bool)
    runs = {}
    for k in idx:
        for sgn in (1, -1):
            th = theta.copy()
            th[k] = np.float32(theta[k] + sgn * h)  # parameters are stored as f32: use the stored step
            ps.set_params(th)
            tt, mm, ss = oracle.render_views(ps.state, vs, opts, 0.05, 64)
            runs[(k, sgn)] = (tt, ss, float(th[k]))
            keep_t &= (mm == m)
    # pixels whose hit state flips anywhere are left out of the depth term
    wt_k = wt * keep_t
    fd = []
    for k in idx:
        (tp, sp, vp), (tm, sm, vm) = runs[(k, 1)], runs[(k, -1)]
        fd.append(((wt_k * tp).sum() + (ws * sp).sum() - (wt_k * tm).sum() - (ws * sm).sum()) / (vp - vm))
    ps.set_params(theta)
    g = oracle.render_backward(ps.state, vs, opts, ps.layout, wt_k.astype(np.float32), ws.astype(np.float32),
                               0.05, 64)
    fd = np.array(fd)
    an = g[idx]
    scale = max(np.abs(fd).max(), 1e-6)
    err = np.abs(an - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    assert np.all(err <= 1e-3), (idx[err > 1e-3], an[err > 1e-3], fd[err > 1e-3])
    assert np.abs(fd).max() > 0
