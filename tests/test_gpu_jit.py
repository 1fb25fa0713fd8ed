"""Scene JIT (NVRTC): kernels compiled at run time with the hook programs as
native code give the interpreter's results."""
import numpy as np
import pytest

import forgedthoughts_gb300 as ft
from conftest import FIXTURES
from forgedthoughts_gb300 import workloads

pytestmark = pytest.mark.gpu


def _pair(w, **kw):
    """(interpreter image, compiled image, jit info) of one workload."""
    st_vm = ft.parse_and_eval(w.source)
    st_jit = ft.parse_and_eval(w.source)
    info = st_jit.gpu().jit()
    a = ft.render_depth(st_vm, w.options, w.accel, w.aa, want_material=True, **kw)
    b = ft.render_depth(st_jit, w.options, w.accel, w.aa, want_material=True, **kw)
    return a, b, info, st_vm, st_jit


def _same_depth(a, b):
    assert (a.mask == b.mask).mean() >= 0.9999
    both = (a.mask == 1) & (b.mask == 1)
    assert np.abs(a.t[both] - b.t[both]).max() <= 1e-4
    assert (a.material[both] == b.material[both]).mean() >= 0.9999


def test_jit_twisted_shells_matches_interpreter():
    w = workloads.twisted_shells(n=256, width=160, height=90)
    a, b, info, _, st_jit = _pair(w)
    assert info["programs"] >= 2 and info["cubin_bytes"] > 0
    _same_depth(a, b)
    # a second scene with the same hook programs reuses the compiled module
    again = ft.parse_and_eval(w.source)
    info2 = again.gpu().jit()
    assert info2["cached"] and info2["compile_ms"] == 0.0
    c = ft.render_depth(again, w.options, w.accel, w.aa)
    assert np.array_equal(c.t, b.t) and np.array_equal(c.mask, b.mask)


def test_jit_reference_material_hook_fixture():
    st = ft.load_and_eval_scene(FIXTURES / "render_regression" / "preview_material_hook.ft")
    st.gpu().jit()
    opts = ft.RenderOptions(width=96, height=96, max_steps=320, max_dist=40.0, epsilon=0.0002, step_scale=0.7,
                            camera_z=6.0, fov_y_degrees=35.0)
    img = ft.render_depth(st, opts, ft.AccelMode.Bvh, 1)
    gold = ft.read_png(FIXTURES / "render_regression" / "preview_material_hook.png")
    diff = np.abs(img.rgb8.astype(int) - gold.astype(int))
    assert diff.max() <= 8 and diff.mean() <= 0.35


def test_jit_trace_with_environment_program():
    w = workloads.union_round_field(n=64, width=96, height=54, aa=1, max_depth=3)
    st_vm = ft.parse_and_eval(w.source)
    st_jit = ft.parse_and_eval(w.source)
    st_jit.gpu().jit()
    la, _ = ft.render_trace(st_vm, w.options, w.accel, 1, 3)
    lb, _ = ft.render_trace(st_jit, w.options, w.accel, 1, 3)
    assert np.sqrt(np.mean((la - lb) ** 2)) <= 1e-4


def test_jit_with_fp16_bricks():
    w = workloads.twisted_shells(n=128, width=128, height=72)
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    g.build_bricks()
    a = ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    g.jit()
    b = ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    assert (a.mask == b.mask).mean() >= 0.9999
    both = (a.mask == 1) & (b.mask == 1)
    assert np.abs(a.t[both] - b.t[both]).max() <= 1e-4
