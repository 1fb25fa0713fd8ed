"""Differentiation form on the GPU: forward views against the CPU
restatement, the adjoint against the FP64 analytic gradient and FP64 central
finite differences, and the torch.autograd.Function wrapper."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
import oracle
from forgedthoughts_gb300 import workloads
from parity import DEPTH_TOL

pytestmark = pytest.mark.gpu


def _setup(n_prims=64, size=48, views=4):
    ps = ft.ParamScene(workloads.shape_fit(n=n_prims))
    return ps, workloads.shape_fit_options(size), ft.ring_views(views)


def test_views_forward_matches_oracle():
    ps, opts, vs = _setup()
    t, m, sil = ps.render(vs, opts)
    for prec in (32, 64):
        to, mo, so = oracle.render_views(ps.state, vs, opts, 0.05, prec)
        assert (m == mo).mean() >= 0.999
        both = (m == 1) & (mo == 1)
        assert np.quantile(np.abs(t[both] - to[both]), 0.999) <= DEPTH_TOL
        miss = (m == 0) & (mo == 0)
        assert np.quantile(np.abs(sil[miss] - so[miss]), 0.999) <= 1e-3


def test_backward_matches_fp64_analytic_gradient():
    ps, opts, vs = _setup()
    t, m, sil = ps.render(vs, opts)
    rng = np.random.default_rng(3)
    wt = (rng.normal(size=t.shape) * (m == 1)).astype(np.float32)
    ws = (rng.normal(size=t.shape) * (m == 0)).astype(np.float32)
    g_gpu = ps.backward(vs, opts, wt, ws)
    g_ref = oracle.render_backward(ps.state, vs, opts, ps.layout, wt, ws, 0.05, 64)
    scale = np.abs(g_ref).max()
    err = np.abs(g_gpu - g_ref) / np.maximum(np.abs(g_ref), 1e-2 * scale)
    # FP32 march vs FP64: a handful of rays change hit / minimum; the bulk agrees
    assert np.quantile(err, 0.9) <= 1e-3, np.sort(err)[-10:]
    assert np.corrcoef(g_gpu, g_ref)[0, 1] > 0.9999


def test_backward_matches_fp64_finite_differences():
    """32 random parameters (seed 7): GPU adjoint vs FP64 central differences
    of the FP64 forward, h = 1e-4, relative error <= 1e-3."""
    ps, opts, vs = _setup(n_prims=16, size=32, views=2)
    theta = ps.get_params()
    t, m, sil = oracle.render_views(ps.state, vs, opts, 0.05, 64)
    rng = np.random.default_rng(7)
    wt = rng.normal(size=t.shape) * (m == 1)
    ws = rng.normal(size=t.shape) * (m == 0)
    idx = rng.choice(ps.n_params, size=32, replace=False)
    h = 1e-4
    keep = np.ones(t.shape, bool)
    runs = {}
    for k in idx:
        for sgn in (1, -1):
            th = theta.copy()
            th[k] = np.float32(theta[k] + sgn * h)
            ps.set_params(th)
            tt, mm, ss = oracle.render_views(ps.state, vs, opts, 0.05, 64)
            runs[(k, sgn)] = (tt, ss, float(th[k]))
            keep &= mm == m
    wt = wt * keep
    fd = np.array([((wt * runs[(k, 1)][0]).sum() + (ws * runs[(k, 1)][1]).sum() - (wt * runs[(k, -1)][0]).sum()
                    - (ws * runs[(k, -1)][1]).sum()) / (runs[(k, 1)][2] - runs[(k, -1)][2]) for k in idx])
    ps.set_params(theta)
    # the GPU forward must see the same hit set for the comparison to be fair
    tg, mg, _ = ps.render(vs, opts)
    same = (mg == m)
    g = ps.backward(vs, opts, (wt * same).astype(np.float32), (ws * same).astype(np.float32))[idx]
    g64 = oracle.render_backward(ps.state, vs, opts, ps.layout, (wt * same).astype(np.float32),
                                 (ws * same).astype(np.float32), 0.05, 64)[idx]
    fd_same = g64  # the FP64 adjoint restricted to the same pixels, itself checked against FD below
    scale = np.abs(fd).max()
    rel_ref = np.abs(g64 - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    if same.all():
        assert np.all(rel_ref <= 1e-3), rel_ref
    rel = np.abs(g - fd_same) / np.maximum(np.abs(fd_same), 1e-2 * scale)
    assert np.all(rel <= 1e-3), (idx[rel > 1e-3], g[rel > 1e-3], fd_same[rel > 1e-3])


def test_autograd_function_and_a_fitting_step():
    torch = pytest.importorskip("torch")
    ps, opts, vs = _setup(n_prims=16, size=32, views=4)
    theta0 = ps.get_params()
    target = ft.ParamScene(workloads.shape_fit(n=16))
    rng = np.random.default_rng(7)
    tgt_params = theta0 + rng.normal(0, 0.05, size=theta0.shape).astype(np.float32)
    target.set_params(tgt_params)
    tt, tm, ts = target.render(vs, opts)
    tt, ts = torch.from_numpy(tt), torch.from_numpy(ts)
    tm = torch.from_numpy(tm).bool()
    fn = ft.render_function()
    p = torch.tensor(theta0, requires_grad=True)

    def loss_of(params):
        t, m, s = fn.apply(params, ps, vs, opts, 0.05)
        both = m.bool() & tm
        return ((t - tt)[both] ** 2).sum() + ((s - ts) ** 2).sum()

    loss = loss_of(p)
    loss.backward()
    assert p.grad is not None and torch.isfinite(p.grad).all() and p.grad.abs().sum() > 0
    opt = torch.optim.Adam([p], lr=0.01)
    losses = []
    for _ in range(10):
        opt.zero_grad()
        l = loss_of(p)
        l.backward()
        opt.step()
        losses.append(float(l))
    assert losses[-1] < losses[0]
