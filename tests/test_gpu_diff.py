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

# Misses that pass within ~1e-3 of the surface (silhouette above exp(-0.02))
# are ill-conditioned in FP32: the FP32 CPU restatement reproduces the GPU
# there and differs from FP64 by a few percent, so the gradient comparisons
# leave them out of the silhouette term.
GRAZING_SIL = float(np.exp(-0.02))


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
    to, mo, so = oracle.render_views(ps.state, vs, opts, 0.05, 64)
    same = m == mo  # pixels the FP32 and FP64 marches classify alike
    rng = np.random.default_rng(3)
    wt = (rng.normal(size=t.shape) * (m == 1) * same).astype(np.float32)
    ws = (rng.normal(size=t.shape) * (m == 0) * same * (so < GRAZING_SIL)).astype(np.float32)
    g_gpu = ps.backward(vs, opts, wt, ws)
    g_ref = oracle.render_backward(ps.state, vs, opts, ps.layout, wt, ws, 0.05, 64)
    scale = np.abs(g_ref).max()
    err = np.abs(g_gpu - g_ref) / np.maximum(np.abs(g_ref), 1e-2 * scale)
    # FP32 vs FP64: the silhouette term's minimum positions carry FP32
    # rounding (the FP32 CPU restatement deviates from FP64 alike)
    assert np.quantile(err, 0.9) <= 1e-3, np.sort(err)[-10:]
    assert err.max() <= 2e-2, np.sort(err)[-10:]
    assert np.corrcoef(g_gpu, g_ref)[0, 1] > 0.9999


def test_backward_matches_fp64_finite_differences():
    """32 random parameters (seed 7): the GPU adjoint against FP64 central
    differences of the FP64 forward, h = 1e-4, relative error <= 1e-3."""
    ps, opts, vs = _setup(n_prims=16, size=32, views=2)
    theta = ps.get_params()
    t, m, sil = oracle.render_views(ps.state, vs, opts, 0.05, 64)
    tg, mg, _ = ps.render(vs, opts)
    rng = np.random.default_rng(7)
    same = mg == m
    wt = rng.normal(size=t.shape) * (m == 1) * same
    ws = rng.normal(size=t.shape) * (m == 0) * same * (sil < GRAZING_SIL)
    idx = rng.choice(ps.n_params, size=32, replace=False)
    h = 1e-4
    keep = np.ones(t.shape, bool)
    runs = {}
    for k in idx:
        for sgn in (1, -1):
            th = theta.copy()
            th[k] = np.float32(theta[k] + sgn * h)  # parameters are stored as f32: use the stored step
            ps.set_params(th)
            tt, mm, ss = oracle.render_views(ps.state, vs, opts, 0.05, 64)
            runs[(k, sgn)] = (tt, ss, float(th[k]))
            keep &= mm == m
    wt = wt * keep  # pixels whose hit state flips under a step leave the depth term
    fd = np.array([((wt * runs[(k, 1)][0]).sum() + (ws * runs[(k, 1)][1]).sum() - (wt * runs[(k, -1)][0]).sum()
                    - (ws * runs[(k, -1)][1]).sum()) / (runs[(k, 1)][2] - runs[(k, -1)][2]) for k in idx])
    ps.set_params(theta)
    g = ps.backward(vs, opts, wt.astype(np.float32), ws.astype(np.float32))[idx]
    scale = np.abs(fd).max()
    assert scale > 0
    rel = np.abs(g - fd) / np.maximum(np.abs(fd), 1e-2 * scale)
    # <= 1e-3 on at least 90 % of the parameters; the rest within the FP32
    # silhouette-term rounding (at most 2 %)
    assert (rel <= 1e-3).mean() >= 0.9, (idx[rel > 1e-3], g[rel > 1e-3], fd[rel > 1e-3])
    assert np.all(rel <= 2e-2), (idx[rel > 2e-2], g[rel > 2e-2], fd[rel > 2e-2])


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
        losses.append(float(l.detach()))
    assert losses[-1] < losses[0]
