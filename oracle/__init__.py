"""CPU oracle for the sphere-tracing hot path — TEST INFRASTRUCTURE ONLY.

ctypes binding of ``oracle/_build/libftoracle.so`` (a C++ restatement of the
reference renderer's depth path, see ``oracle/oracle.cpp``).  Only the tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
package; the product never does.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libftoracle.so"
_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} missing; run `python -m forgedthoughts_gb300.build`")
        h = ctypes.CDLL(str(LIB_PATH))
        vp = ctypes.c_void_p
        h.oracle_render_depth.restype = ctypes.c_int
        h.oracle_render_depth.argtypes = [vp, vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp, vp, vp,
                                          ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_distance.restype = ctypes.c_int
        h.oracle_distance.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_size_t, vp, vp, vp]
        h.oracle_eval_program.restype = ctypes.c_int
        h.oracle_eval_program.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_size_t, vp]
        h.oracle_render_trace.restype = ctypes.c_int
        h.oracle_render_trace.argtypes = [vp, vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp, vp,
                                          ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_render_views.restype = ctypes.c_int
        h.oracle_render_views.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                          vp, vp, vp]
        h.oracle_render_backward_strided.restype = ctypes.c_int
        h.oracle_render_backward_strided.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_float, vp,
                                                     ctypes.c_uint32, vp, vp, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_uint32, ctypes.c_uint32, vp]
        h.oracle_render_backward.restype = ctypes.c_int
        h.oracle_render_backward.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_float, vp, ctypes.c_uint32, vp,
                                             vp, ctypes.c_int, ctypes.c_int, vp]
        u32, i64 = ctypes.c_uint32, ctypes.c_int64
        h.oracle_render_depth_strided.restype = ctypes.c_int
        h.oracle_render_depth_strided.argtypes = [vp, vp, ctypes.c_int, u32, ctypes.c_int, ctypes.c_int, u32, u32, u32,
                                                  u32, u32, i64, vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_render_trace_strided.restype = ctypes.c_int
        h.oracle_render_trace_strided.argtypes = [vp, vp, ctypes.c_int, u32, u32, ctypes.c_int, ctypes.c_int, u32,
                                                  u32, u32, u32, u32, i64, vp, vp, ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_render_views_strided.restype = ctypes.c_int
        h.oracle_render_views_strided.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_float, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, vp, vp, vp]
        h.oracle_render_path.restype = ctypes.c_int
        h.oracle_render_path.argtypes = [vp, vp, ctypes.c_int, u32, u32, u32, ctypes.c_float, ctypes.c_int,
                                         ctypes.c_int, u32, u32, u32, u32, u32, vp, vp, vp,
                                         ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_render_sample.restype = ctypes.c_int
        h.oracle_render_sample.argtypes = [vp, vp, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]
        h.oracle_last_error.restype = ctypes.c_char_p
        h.oracle_medium_transmittance.restype = None
        h.oracle_medium_transmittance.argtypes = [vp, ctypes.c_float, vp]
        h.oracle_transition_medium.restype = None
        h.oracle_transition_medium.argtypes = [vp, ctypes.c_int, vp, vp]
        h.oracle_set_resolve_mode.restype = None
        h.oracle_set_resolve_mode.argtypes = [ctypes.c_int]
        h.oracle_bsdf_hit.restype = ctypes.c_int
        h.oracle_bsdf_hit.argtypes = [vp, vp, vp, ctypes.c_float, vp, vp, vp]
        _lib = h
    return _lib


def _vp(x):
    return ctypes.cast(x, ctypes.c_void_p)


def _arr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError("oracle failed: " + (lib().oracle_last_error() or b"").decode())


def render_depth(state, options, accel: int, aa: int = 1, precision: int = 32, threads: int = 0,
                 rows: tuple[int, int, int] | None = None, normals: bool = False,
                 cols: tuple[int, int] | None = None, jitter_seed: int | None = None):
    """Oracle depth preview.  Returns (t, mask, material, rgb8, evals[, normal]).
    ``rows`` = (begin, end, step) and ``cols`` = (begin, step) restrict it to
    a strided band (only those pixels of the full-frame outputs are written);
    ``jitter_seed`` selects the jittered AA offsets."""
    from forgedthoughts_gb300 import _native  # scene description structs only

    aa = max(int(aa), 1)
    h, w = int(options.height), int(options.width)
    t = np.zeros((h, w, aa), np.float32)
    mask = np.zeros((h, w, aa), np.uint8)
    mat = np.zeros((h, w, aa), np.uint32)
    rgb = np.zeros((h, w, 3), np.uint8)
    nrm = np.zeros((h, w, aa, 3), np.float32) if normals else None
    opts = options.to_c() if hasattr(options, "to_c") else options
    assert isinstance(opts, _native.RenderOptionsC)
    r0, r1, rs = rows if rows is not None else (0, h, 1)
    c0, cs = cols if cols is not None else (0, 1)
    evals = ctypes.c_uint64(0)
    _check(lib().oracle_render_depth_strided(_vp(state.desc_ptr), ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p),
                                             int(accel), aa, int(precision), int(threads), r0, r1, rs, c0, cs,
                                             -1 if jitter_seed is None else int(jitter_seed),
                                             _arr(t), _arr(mask), _arr(mat), _arr(nrm), _arr(rgb),
                                             ctypes.byref(evals)))
    if normals:
        return t, mask, mat, rgb, int(evals.value), nrm
    return t, mask, mat, rgb, int(evals.value)


def render_trace(state, options, accel: int, aa: int = 1, max_depth: int = 8, precision: int = 32,
                 threads: int = 0, rows: tuple[int, int, int] | None = None, cols: tuple[int, int] | None = None,
                 jitter_seed: int | None = None):
    """Oracle Whitted trace.  Returns (rgb linear float (H, W, 3), rgb8, evals).
    ``rows`` / ``cols`` / ``jitter_seed`` as in render_depth."""
    from forgedthoughts_gb300 import _native

    h, w = int(options.height), int(options.width)
    rgb = np.zeros((h, w, 3), np.float32)
    rgb8 = np.zeros((h, w, 3), np.uint8)
    opts = options.to_c() if hasattr(options, "to_c") else options
    assert isinstance(opts, _native.RenderOptionsC)
    r0, r1, rs = rows if rows is not None else (0, h, 1)
    c0, cs = cols if cols is not None else (0, 1)
    evals = ctypes.c_uint64(0)
    _check(lib().oracle_render_trace_strided(_vp(state.desc_ptr), ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p),
                                             int(accel), max(int(aa), 1), int(max_depth), int(precision),
                                             int(threads), r0, r1, rs, c0, cs,
                                             -1 if jitter_seed is None else int(jitter_seed), _arr(rgb), _arr(rgb8),
                                             ctypes.byref(evals)))
    return rgb, rgb8, int(evals.value)


def render_sample(state, options, accel: int, aa: int, max_depth: int, mode: str, threads: int = 0,
                  rows: tuple[int, int] = (0, 1), cols: tuple[int, int] = (0, 1)) -> int:
    """Strided pixel sample of a full frame in f32 (outputs discarded): the
    timed CPU baseline.  ``rows`` / ``cols`` = (first, step).  Returns the
    distance evaluations it took."""
    from forgedthoughts_gb300 import _native

    opts = options.to_c() if hasattr(options, "to_c") else options
    assert isinstance(opts, _native.RenderOptionsC)
    evals = ctypes.c_uint64(0)
    _check(lib().oracle_render_sample(_vp(state.desc_ptr), ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p),
                                      int(accel), max(int(aa), 1), int(max_depth), 0 if mode == "depth" else 1,
                                      int(threads), int(rows[0]), int(rows[1]), int(cols[0]), int(cols[1]),
                                      ctypes.byref(evals)))
    return int(evals.value)


def render_path(state, options, accel: int, spp: int = 16, max_bounces: int = 4, min_spp: int = 8,
                noise_threshold: float = 0.03, precision: int = 32, threads: int = 0,
                rows: tuple[int, int, int] | None = None, cols: tuple[int, int] | None = None):
    """Oracle MIS path tracer (the progressive renderer with adaptive
    sampling).  Returns (rgb linear (H, W, 3), rgb8, samples per pixel (H, W),
    evals); ``rows`` / ``cols`` restrict it to a strided band."""
    from forgedthoughts_gb300 import _native

    h, w = int(options.height), int(options.width)
    rgb = np.zeros((h, w, 3), np.float32)
    rgb8 = np.zeros((h, w, 3), np.uint8)
    count = np.zeros((h, w), np.uint32)
    opts = options.to_c() if hasattr(options, "to_c") else options
    assert isinstance(opts, _native.RenderOptionsC)
    r0, r1, rs = rows if rows is not None else (0, h, 1)
    c0, cs = cols if cols is not None else (0, 1)
    evals = ctypes.c_uint64(0)
    _check(lib().oracle_render_path(_vp(state.desc_ptr), ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p),
                                    int(accel), int(spp), int(max_bounces), int(min_spp), float(noise_threshold),
                                    int(precision), int(threads), r0, r1, rs, c0, cs, _arr(rgb), _arr(rgb8),
                                    _arr(count), ctypes.byref(evals)))
    return rgb, rgb8, count, int(evals.value)


def distance(state, points: np.ndarray, accel: int = 1, precision: int = 32):
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = pts.shape[0]
    d = np.zeros(n, np.float64)
    obj = np.zeros(n, np.uint32)
    mat = np.zeros(n, np.uint32)
    _check(lib().oracle_distance(_vp(state.desc_ptr), int(accel), int(precision), _arr(pts), n, _arr(d), _arr(obj),
                                 _arr(mat)))
    return d, obj, mat


def medium_transmittance(ior: float, absorption, density: float, distance: float) -> np.ndarray:
    """medium_transmittance (renderer.rs:5109-5119) in f32: the (3,) transmittance."""
    m = np.array([ior, *absorption, density], np.float32)
    out = np.zeros(3, np.float32)
    lib().oracle_medium_transmittance(_arr(m), float(distance), _arr(out))
    return out


def transition_medium(material, front_face: bool, current) -> np.ndarray:
    """transition_medium (renderer.rs:5147-5166) in f32 for an ``ft_material``
    (a ctypes structure): the next medium as (ior, r, g, b, density)."""
    cur = np.ascontiguousarray(current, np.float32)
    out = np.zeros(5, np.float32)
    lib().oracle_transition_medium(ctypes.cast(ctypes.byref(material), ctypes.c_void_p), int(bool(front_face)),
                                   _arr(cur), _arr(out))
    return out


def bsdf_hit(state, position, normal, front_face: bool, object_id: int, material_id: int, view_dir,
             current_ior: float, wi, u=(0.5, 0.5, 0.5)) -> dict:
    """The BSDF context of one hit (build_bsdf_context, renderer.rs:4397-4449)
    and the BSDF of the material resolved there, hooks included (eval_bsdf,
    pdf_bsdf, sample_bsdf_lobe, renderer.rs:4869-4950), in f32: the shading
    normal, eval(wi), pdf(wi) and the sample drawn with the randoms ``u``."""
    hit = np.array(list(position) + list(normal) + [1.0 if front_face else 0.0, object_id, material_id], np.float32)
    out = np.zeros(19, np.float32)
    _check(lib().oracle_bsdf_hit(state.desc_ptr, _arr(hit), _arr(np.asarray(view_dir, np.float32)),
                                 float(current_ior), _arr(np.asarray(wi, np.float32)),
                                 _arr(np.asarray(u, np.float32)), _arr(out)))
    return {"normal": out[0:3], "eval": out[3:6], "pdf": float(out[6]), "sample_wi": out[7:10],
            "sample_f": out[10:13], "sample_pdf": float(out[13]), "sample_delta": bool(out[14]),
            "sample_apply_cos": bool(out[15]), "sample_transmission": bool(out[16]),
            "sample_thin_walled": bool(out[17]), "sample_next_ior": float(out[18])}


class resolve_at_hit_leaf:
    """Context manager: while active, the oracle resolves a hit's normal and
    material from the hard-union leaf holding the hit's object (the leaf its
    accelerator found, as the GPU does) instead of walking the scene root's
    unions as the reference does.  The two differ only where the reference's
    union culling skips the hit's leaf (an object with both domain and
    distance_post hooks, whose surface leaves its box)."""

    def __enter__(self):
        lib().oracle_set_resolve_mode(1)
        return self

    def __exit__(self, *exc):
        lib().oracle_set_resolve_mode(0)
        return False


def eval_program(state, program: int, args: np.ndarray, precision: int = 32) -> np.ndarray:
    """Run hook program ``program`` on ``args`` of shape (n, n_params, 3)."""
    a = np.ascontiguousarray(args, np.float32)
    n = a.shape[0]
    out = np.zeros((n, 3), np.float64)
    _check(lib().oracle_eval_program(_vp(state.desc_ptr), int(program), int(precision), _arr(a), n, _arr(out)))
    return out


def _views_c(views):
    from forgedthoughts_gb300 import _native

    arr = (_native.ViewC * len(views))()
    for k, v in enumerate(views):
        arr[k] = v if isinstance(v, _native.ViewC) else _native.ViewC(*v)
    return arr


def render_views(state, views, options, tau: float = 0.05, precision: int = 64, threads: int = 0,
                 stride: int = 1, offset: int = 0):
    """Multi-view depth / mask / soft silhouette (the definitions of
    ft_render_views).  ``views``: (origin, target, fov) triples or ViewC.
    Returns (t, mask, sil), each (n_views, H, W).  With ``stride`` > 1 only
    the pixels (offset + i * stride, offset + j * stride) are rendered (the
    others stay zero)."""
    from forgedthoughts_gb300 import _native

    varr = _views_c(views)
    n = len(views)
    h, w = int(options.height), int(options.width)
    t = np.zeros((n, h, w), np.float64)
    mask = np.zeros((n, h, w), np.uint8)
    sil = np.zeros((n, h, w), np.float64)
    opts = options.to_c() if hasattr(options, "to_c") else options
    assert isinstance(opts, _native.RenderOptionsC)
    _check(lib().oracle_render_views_strided(_vp(state.desc_ptr), ctypes.cast(varr, ctypes.c_void_p), n,
                                             ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p), float(tau),
                                             int(precision), int(threads), int(stride), int(offset), _arr(t),
                                             _arr(mask), _arr(sil)))
    return t, mask, sil


def render_backward(state, views, options, params, dl_dt=None, dl_dsil=None, tau: float = 0.05,
                    precision: int = 64, threads: int = 0, stride: int = 1, offset: int = 0) -> np.ndarray:
    """The adjoint of render_views: dL/dparams (float64) for the upstream
    gradients dl_dt / dl_dsil (each (n_views, H, W) or None)."""
    from forgedthoughts_gb300 import _native

    varr = _views_c(views)
    parr = params if isinstance(params, ctypes.Array) else (_native.ParamC * len(params))(*params)
    opts = options.to_c() if hasattr(options, "to_c") else options
    a = None if dl_dt is None else np.ascontiguousarray(dl_dt, np.float32)
    b = None if dl_dsil is None else np.ascontiguousarray(dl_dsil, np.float32)
    g = np.zeros(len(parr), np.float64)
    _check(lib().oracle_render_backward_strided(_vp(state.desc_ptr), ctypes.cast(varr, ctypes.c_void_p), len(views),
                                                ctypes.cast(ctypes.pointer(opts), ctypes.c_void_p), float(tau),
                                                ctypes.cast(parr, ctypes.c_void_p), len(parr), _arr(a), _arr(b),
                                                int(precision), int(threads), int(stride), int(offset), _arr(g)))
    return g
