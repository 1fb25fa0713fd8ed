"""GB300-native sphere tracing for ForgedThoughts scenes.

Python host layer over the C ABI (``include/forgedthoughts_gb300.h``).  Names
and argument meanings mirror the reference crate's public API
(crates/forgedthoughts/src/renderer.rs, "R"):

* :class:`RenderOptions`            -- ``struct RenderOptions`` (R:32-56)
* :class:`AccelMode`                -- ``enum AccelMode`` (R:58-63)
* :func:`parse_and_eval`            -- ``parse_program`` + ``eval_program``
* :func:`load_and_eval_scene`       -- ``load_and_eval_scene`` (lib.rs:280-284)
* :func:`extract_scene_render_settings` -- R:1316-1354
* :func:`render_depth_png_with_accel`   -- R:1139-1156
* :func:`render_preview_progressive_with_accel` -- R:1238-1277
* :class:`RenderError` and subclasses -- ``enum RenderError`` (R:159-168)

All rendering runs in the sm_103a kernels of the native library; there is no
CPU path in this package.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import os
import struct
import zlib
from pathlib import Path
from typing import Callable, Optional

import numpy as np

from . import _native

__all__ = [
    "AccelMode", "RenderOptions", "SceneState", "GpuScene", "DepthImage", "PreviewProgress", "RenderError",
    "MissingSceneRoot", "UnsupportedObjectType", "ExpectedObject", "ParseError", "EvalError", "CudaError",
    "SceneIoError", "MissingImport", "ImportCycle", "AmbiguousImport", "LibraryItem", "library_from_dir",
    "parse_and_eval", "load_and_eval_scene", "extract_scene_render_settings", "render_depth",
    "render_depth_png_with_accel", "render_preview_progressive_with_accel", "write_png", "read_png",
]


class AccelMode(enum.IntEnum):
    Naive = 0
    Bvh = 1
    Bricks = 2


@dataclasses.dataclass
class RenderOptions:
    """``RenderOptions`` with the reference defaults (R:43-55)."""

    width: int = 800
    height: int = 800
    max_steps: int = 128
    max_dist: float = 40.0
    epsilon: float = 0.001
    step_scale: float = 0.7
    camera_z: float = 6.0
    fov_y_degrees: float = 45.0

    def to_c(self) -> _native.RenderOptionsC:
        return _native.RenderOptionsC(int(self.width), int(self.height), int(self.max_steps), float(self.max_dist),
                                      float(self.epsilon), float(self.step_scale), float(self.camera_z),
                                      float(self.fov_y_degrees))


# ---------------------------------------------------------------- errors
class RenderError(RuntimeError):
    """Base of the renderer's errors (``enum RenderError``, R:159-168)."""

    status = -1


class MissingSceneRoot(RenderError):
    status = _native.FT_ERR_MISSING_SCENE_ROOT


class UnsupportedObjectType(RenderError):
    status = _native.FT_ERR_UNSUPPORTED_OBJECT


class ExpectedObject(RenderError):
    status = _native.FT_ERR_EXPECTED_OBJECT


class ParseError(RenderError):
    status = _native.FT_ERR_PARSE


class EvalError(RenderError):
    status = _native.FT_ERR_EVAL


class JitError(RenderError):
    status = _native.FT_ERR_JIT


class CudaError(RenderError):
    status = _native.FT_ERR_CUDA


class SceneIoError(RenderError):
    """A scene file could not be read (``CoreError::Io``, lib.rs:251-256)."""

    status = _native.FT_ERR_IO


class MissingImport(RenderError):
    """A relative import names no file (``CoreError::MissingImport``)."""

    status = _native.FT_ERR_MISSING_IMPORT


class ImportCycle(RenderError):
    """A file imports itself through a chain of imports (``CoreError::ImportCycle``)."""

    status = _native.FT_ERR_IMPORT_CYCLE


class AmbiguousImport(RenderError):
    """A library name matches several items (``CoreError::AmbiguousBuiltinImport``)."""

    status = _native.FT_ERR_AMBIGUOUS_IMPORT


_ERRORS = {cls.status: cls for cls in (MissingSceneRoot, UnsupportedObjectType, ExpectedObject, ParseError,
                                       EvalError, CudaError, JitError, SceneIoError, MissingImport, ImportCycle,
                                       AmbiguousImport)}


def _check(status: int) -> None:
    if status != _native.FT_OK:
        cls = _ERRORS.get(status, RenderError)
        err = cls(_native.last_error() or f"native call failed with status {status}")
        err.status = status
        raise err


# ---------------------------------------------------------------- scenes
@dataclasses.dataclass
class SceneRenderSettings:
    """``SceneRenderSettings`` (R:66-81), render-option part."""

    width: Optional[int] = None
    height: Optional[int] = None
    max_steps: Optional[int] = None
    max_dist: Optional[float] = None
    epsilon: Optional[float] = None
    step_scale: Optional[float] = None
    camera_z: Optional[float] = None
    fov_y_degrees: Optional[float] = None
    accel: Optional[AccelMode] = None


class SceneState:
    """An evaluated and lowered `.ft` scene (the role of ``EvalState``).

    Holds the flat scene description produced by the native front-end.  The
    GPU copy is created on first use and cached.
    """

    def __init__(self, source: Optional[str] = None, path=None, library=None):
        lib = _native.lib()
        ptr = ctypes.POINTER(_native.SceneDescC)()
        self._desc = ptr
        self._gpu: Optional[GpuScene] = None
        if path is not None and library is not None:
            items = list(library)
            arr = (_native.LibraryItemC * max(1, len(items)))()
            keep = []
            for i, it in enumerate(items):
                fields = [x.encode("utf-8") for x in (it.name, it.path, it.source)]
                keep.append(fields)
                arr[i] = _native.LibraryItemC(*fields)
            _check(lib.ft_scene_desc_from_file_with_library(os.fsencode(path), arr, len(items), ctypes.byref(ptr)))
        elif path is not None:
            _check(lib.ft_scene_desc_from_file(os.fsencode(path), ctypes.byref(ptr)))
        else:
            _check(lib.ft_scene_desc_from_source(source.encode("utf-8"), ctypes.byref(ptr)))
        self._desc = ptr
        self.source = source
        self.path = path

    @property
    def desc_ptr(self):
        return self._desc

    @property
    def desc(self) -> _native.SceneDescC:
        """A view of the native description; it keeps this state (which owns
        the memory) alive, so ``parse_and_eval(src).desc`` stays valid."""
        d = self._desc.contents
        d._owner = self
        return d

    def gpu(self) -> "GpuScene":
        if self._gpu is None:
            self._gpu = GpuScene(self)
        return self._gpu

    def close(self) -> None:
        if self._gpu is not None:
            self._gpu.close()
            self._gpu = None
        if self._desc:
            _native.lib().ft_scene_desc_free(self._desc)
            self._desc = ctypes.POINTER(_native.SceneDescC)()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def parse_and_eval(source: str) -> SceneState:
    return SceneState(source)


@dataclasses.dataclass(frozen=True)
class LibraryItem:
    """An asset library item (``BuiltinLibraryItem``, lib.rs:54-61)."""

    name: str
    path: str
    source: str


def library_from_dir(root) -> list:
    """Library items for every ``.ft`` file under ``root``: ``path`` is the
    file's path below ``root`` with ``/`` separators, ``name`` its stem in
    CamelCase (``materials/checker_floor.ft`` -> ``CheckerFloor``), the
    naming of the reference's library directory."""
    root = Path(root)
    items = []
    for f in sorted(root.rglob("*.ft")):
        name = "".join(part[:1].upper() + part[1:] for part in f.stem.split("_") if part)
        items.append(LibraryItem(name, f.relative_to(root).as_posix(), f.read_text()))
    return items


def load_and_eval_scene(path, library=None) -> SceneState:
    """A scene file with its imports resolved (``load_and_eval_scene``,
    lib.rs:280-284).  ``library`` gives the items that non-relative imports
    select: a sequence of :class:`LibraryItem`, or a directory read with
    :func:`library_from_dir`.  Without it, ``FT_LIBRARY_DIR`` names the
    directory if set; otherwise such an import raises ``RenderError``."""
    if library is None and os.environ.get("FT_LIBRARY_DIR"):
        library = os.environ["FT_LIBRARY_DIR"]
    if isinstance(library, (str, os.PathLike)):
        library = library_from_dir(library)
    return SceneState(path=path, library=library)


def extract_scene_render_settings(state: SceneState) -> SceneRenderSettings:
    d = state.desc
    s = d.settings
    m = d.settings_mask
    out = SceneRenderSettings()
    names = ["width", "height", "max_steps", "max_dist", "epsilon", "step_scale", "camera_z", "fov_y_degrees"]
    for bit, name in enumerate(names):
        if m & (1 << bit):
            setattr(out, name, getattr(s, name))
    if d.settings_accel >= 0:
        out.accel = AccelMode(d.settings_accel)
    return out


class GpuScene:
    """A scene resident on the current CUDA device (``ft_scene``)."""

    def __init__(self, state: SceneState):
        lib = _native.lib()
        h = ctypes.c_void_p()
        _check(lib.ft_scene_create(state.desc_ptr, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def jit(self) -> dict:
        """Compile the scene's hook programs with the march and trace kernels
        at run time (NVRTC, ``ft_scene_jit``); later renders of this scene use
        the compiled kernels."""
        info = _native.JitInfoC()
        _check(_native.lib().ft_scene_jit(self._h, ctypes.byref(info)))
        return {"programs": info.programs, "cached": bool(info.cached), "source_bytes": info.source_bytes,
                "cubin_bytes": info.cubin_bytes, "compile_ms": info.compile_ms, "load_ms": info.load_ms}

    def build_bricks(self, voxel_size: float = 0.02, band: float = 0.0, safety: float = 0.0,
                     max_lattice_points: int = 0, far_steps_per_pass: int = 0,
                     free_far_steps: bool = False) -> "BrickInfo":
        """Build the FP16 brick distance cache (``ft_scene_build_bricks``)."""
        o = _native.BrickOptionsC(voxel_size, band, safety, max_lattice_points, far_steps_per_pass,
                                  _native.FT_BRICK_FREE_FAR_STEPS if free_far_steps else 0)
        info = _native.BrickInfoC()
        _check(_native.lib().ft_scene_build_bricks(self._h, ctypes.byref(o), ctypes.byref(info)))
        return BrickInfo(tuple(info.region_min), tuple(info.region_max), tuple(info.bricks), info.near_bricks,
                         info.exact_leaves, info.max_lipschitz, info.band, info.device_bytes, info.build_ms)

    def brick_bounds(self, points: np.ndarray) -> tuple:
        """(far-field bound, exact distance) at ``points`` (N, 3)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        n = pts.shape[0]
        bound = np.empty(n, np.float32)
        exact = np.empty(n, np.float32)
        _check(_native.lib().ft_scene_brick_bounds(self._h, _ptr(pts), n, _ptr(bound), _ptr(exact)))
        return bound, exact

    def close(self) -> None:
        if self._h:
            _native.lib().ft_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class BrickInfo:
    """``ft_brick_info``: the FP16 brick cache of a scene."""

    region_min: tuple
    region_max: tuple
    bricks: tuple
    near_bricks: int
    exact_leaves: int
    max_lipschitz: float
    band: float
    device_bytes: int
    build_ms: float


@dataclasses.dataclass
class DepthImage:
    width: int
    height: int
    aa: int
    t: Optional[np.ndarray]         # (H, W, aa) float32 refined hit distance, 0 on miss
    mask: Optional[np.ndarray]      # (H, W, aa) uint8
    material: Optional[np.ndarray]  # (H, W, aa) uint32
    normal: Optional[np.ndarray]    # (H, W, aa, 3) float32
    rgb8: Optional[np.ndarray]      # (H, W, 3) uint8 depth preview


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def render_depth(state: SceneState, options: RenderOptions, accel: AccelMode = AccelMode.Bvh, aa_samples: int = 1,
                 *, want_t: bool = True, want_mask: bool = True, want_material: bool = False,
                 want_normal: bool = False, want_rgb8: bool = True, fp16_bricks: bool = False,
                 jitter_seed: int | None = None) -> DepthImage:
    """Depth preview of ``state`` on the GPU (host output buffers).  With
    ``fp16_bricks`` the march uses the scene's FP16 brick cache
    (``state.gpu().build_bricks()`` must have run)."""
    aa = max(int(aa_samples), 1)
    h, w = int(options.height), int(options.width)
    t = np.empty((h, w, aa), np.float32) if want_t else None
    mask = np.empty((h, w, aa), np.uint8) if want_mask else None
    mat = np.empty((h, w, aa), np.uint32) if want_material else None
    nrm = np.empty((h, w, aa, 3), np.float32) if want_normal else None
    rgb = np.empty((h, w, 3), np.uint8) if want_rgb8 else None
    opts = options.to_c()
    _check(_native.lib().ft_render_depth(state.gpu().handle, ctypes.byref(opts), int(accel), aa, _ptr(t), _ptr(mask),
                                         _ptr(mat), _ptr(nrm), _ptr(rgb),
                                         (_native.FT_FLAG_FP16_BRICKS if fp16_bricks else 0)
                                         | jitter_flags(jitter_seed), None))
    return DepthImage(w, h, aa, t, mask, mat, nrm, rgb)


@dataclasses.dataclass
class RaySettings:
    """``RaySettings`` (R:124-141)."""

    max_depth: int = 8
    tile_size: int = 64
    aa_samples: int = 1


def jitter_flags(jitter_seed: int | None) -> int:
    """Render flags of jittered AA with ``jitter_seed`` (None: the grid)."""
    if jitter_seed is None:
        return 0
    return _native.FT_FLAG_JITTERED_AA | ((int(jitter_seed) & 0xFFFF) << _native.FT_JITTER_SEED_SHIFT)


def render_trace(state: SceneState, options: RenderOptions, accel: AccelMode = AccelMode.Bvh, aa_samples: int = 1,
                 max_depth: int = 8, *, want_linear: bool = True, jitter_seed: int | None = None,
                 fp16_bricks: bool = False) -> tuple:
    """Whitted trace of ``state`` on the GPU: (linear rgb (H, W, 3) float32 or
    None, rgb8 (H, W, 3) uint8).  ``jitter_seed`` selects jittered AA offsets
    (XorShift64 per pixel sample, the seed xor-ed in) instead of the grid.
    With ``fp16_bricks`` the primary hits come from the FP16 brick depth march
    (``SceneState.gpu().build_bricks()`` first)."""
    h, w = int(options.height), int(options.width)
    lin = np.empty((h, w, 3), np.float32) if want_linear else None
    rgb8 = np.empty((h, w, 3), np.uint8)
    opts = options.to_c()
    _check(_native.lib().ft_render_trace(state.gpu().handle, ctypes.byref(opts), int(accel), max(int(aa_samples), 1),
                                         int(max_depth), _ptr(lin), _ptr(rgb8),
                                         jitter_flags(jitter_seed) | (_native.FT_FLAG_FP16_BRICKS if fp16_bricks else 0),
                                         None))
    return lin, rgb8


@dataclasses.dataclass
class PathtraceSettings:
    """``PathtraceSettings`` (R:107-125)."""

    spp: int = 16
    max_bounces: int = 4
    preview_every: int = 5
    min_spp: int = 8
    noise_threshold: float = 0.03


def render_pathtrace(state: SceneState, options: RenderOptions, accel: AccelMode = AccelMode.Bvh,
                     settings: PathtraceSettings | None = None) -> tuple:
    """The MIS path tracer on the GPU (render_pathtrace_with_accel_progressive,
    R:3974-4045): (linear rgb (H, W, 3) float32, rgb8 (H, W, 3) uint8,
    samples per pixel (H, W) uint32)."""
    ps = settings or PathtraceSettings()
    h, w = int(options.height), int(options.width)
    lin = np.empty((h, w, 3), np.float32)
    rgb8 = np.empty((h, w, 3), np.uint8)
    count = np.empty((h, w), np.uint32)
    c = _native.PathtraceSettingsC(int(ps.spp), int(ps.max_bounces), int(ps.min_spp), float(ps.noise_threshold))
    opts = options.to_c()
    _check(_native.lib().ft_render_pathtrace(state.gpu().handle, ctypes.byref(opts), int(accel), ctypes.byref(c),
                                             _ptr(lin), _ptr(rgb8), _ptr(count), 0, None))
    return lin, rgb8, count


def render_ray_progressive_with_accel(state: SceneState, options: RenderOptions, accel: AccelMode,
                                      settings: RaySettings, on_tile) -> np.ndarray:
    """Whitted render with the reference's per-tile progress callback (R:1201-1236)."""
    import time

    start = time.monotonic()
    _, img = render_trace(state, options, accel, settings.aa_samples, settings.max_depth, want_linear=False)
    out = np.zeros_like(img)
    jobs = list(_tile_jobs(options.width, options.height, max(int(settings.tile_size), 1)))
    for done, (tx, ty, tw, th) in enumerate(jobs, 1):
        out[ty:ty + th, tx:tx + tw] = img[ty:ty + th, tx:tx + tw]
        on_tile(PreviewProgress(done, len(jobs), int((time.monotonic() - start) * 1000)), out.copy())
    return out


@dataclasses.dataclass
class PreviewProgress:
    """``PreviewProgress`` (R:96-101)."""

    tiles_done: int
    tiles_total: int
    elapsed_ms: int


def _tile_jobs(width: int, height: int, tile: int):
    # tile_jobs (R:3849-3862)
    for ty in range(0, height, tile):
        for tx in range(0, width, tile):
            yield tx, ty, min(tile, width - tx), min(tile, height - ty)


def render_preview_progressive_with_accel(state: SceneState, options: RenderOptions, accel: AccelMode,
                                          tile_size: int, aa_samples: int,
                                          on_tile: Callable[[PreviewProgress, np.ndarray], None]) -> np.ndarray:
    """Depth preview with the reference's per-tile progress callback.

    The GPU renders the frame in one launch; ``on_tile`` then sees the image
    with tiles revealed in the reference's tile order.  An exception raised by
    the callback aborts the call, as a callback ``Err`` does (R:3815-3830).
    """
    import time

    start = time.monotonic()
    img = render_depth(state, options, accel, aa_samples, want_t=False, want_mask=False).rgb8
    out = np.zeros_like(img)
    jobs = list(_tile_jobs(options.width, options.height, max(int(tile_size), 1)))
    for done, (tx, ty, tw, th) in enumerate(jobs, 1):
        out[ty:ty + th, tx:tx + tw] = img[ty:ty + th, tx:tx + tw]
        on_tile(PreviewProgress(done, len(jobs), int((time.monotonic() - start) * 1000)), out.copy())
    return out


def render_depth_png_with_accel(state: SceneState, output_path, options: RenderOptions,
                                accel: AccelMode = AccelMode.Naive) -> None:
    img = render_depth(state, options, accel, 1, want_t=False, want_mask=False).rgb8
    write_png(output_path, img)


# ---------------------------------------------------------------- PNG I/O
def write_png(path, rgb: np.ndarray) -> None:
    """Write an 8-bit RGB image (H, W, 3) as PNG."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, c = rgb.shape
    if c != 3:
        raise ValueError("write_png expects an RGB image")
    raw = b"".join(b"\x00" + rgb[y].tobytes() for y in range(h))

    def chunk(tag: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    Path(path).write_bytes(png)


def read_png(path) -> np.ndarray:
    """Read an 8-bit non-interlaced gray/RGB/RGBA PNG as (H, W, 3) uint8."""
    data = Path(path).read_bytes()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace != 0 or ctype not in (0, 2, 6):
        raise ValueError("unsupported PNG format")
    ch = {0: 1, 2: 3, 6: 4}[ctype]
    raw = zlib.decompress(idat)
    stride = w * ch
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - ch] if x >= ch else 0
            b = prev[x]
            c = prev[x - ch] if x >= ch else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    img = out.reshape(h, w, ch).astype(np.uint8)
    if ch == 1:
        img = np.repeat(img, 3, axis=2)
    return img[:, :, :3]


class Batch:
    """Many renders in one CUDA-graph launch (``ft_batch``).

    ``items`` are ``(SceneState, RenderOptions, aa_samples, max_depth)``
    tuples; ``max_depth`` 0 renders the depth preview, 1..10 a Whitted trace.
    The scenes must stay alive while the batch exists.
    """

    def __init__(self, items, fp16_bricks: bool = False):
        lib = _native.lib()
        arr = (_native.BatchItemC * len(items))()
        self._states = []
        self._items = []
        for k, (state, options, aa, max_depth) in enumerate(items):
            arr[k].scene = state.gpu().handle.value
            arr[k].options = options.to_c()
            arr[k].aa_samples = max(int(aa), 1)
            arr[k].max_depth = int(max_depth)
            self._states.append(state)
            self._items.append((int(options.width), int(options.height), max(int(aa), 1), int(max_depth)))
        h = ctypes.c_void_p()
        _check(lib.ft_batch_create(arr, len(items), _native.FT_BATCH_FP16_BRICKS if fp16_bricks else 0,
                                   ctypes.byref(h)))
        self._h = h

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def samples(self) -> int:
        n = ctypes.c_uint64()
        _check(_native.lib().ft_batch_samples(self._h, ctypes.byref(n)))
        return int(n.value)

    def set_tuning(self, tile_w: int, tile_h: int, refill: int) -> None:
        t = _native.BatchTuningC(tile_w, tile_h, refill, 0.0)
        _check(_native.lib().ft_batch_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self) -> dict:
        t = _native.BatchTuningC()
        _check(_native.lib().ft_batch_autotune(self._h, ctypes.byref(t)))
        return {"tile_w": t.tile_w, "tile_h": t.tile_h, "refill": t.refill, "ms": t.ms}

    def launch(self, stream=None) -> None:
        _check(_native.lib().ft_batch_launch(self._h, stream))

    def read(self, item: int) -> dict:
        """Outputs of one item (synchronises): depth items give t, mask, rgb
        (preview value), rgb8; traces give rgb (linear radiance) and rgb8."""
        if not 0 <= item < len(self._items):
            raise RenderError(f"batch item {item} out of range")
        w, h, aa, depth = self._items[item]
        t = np.empty((h, w, aa), np.float32) if depth == 0 else None
        mask = np.empty((h, w, aa), np.uint8) if depth == 0 else None
        rgb = np.empty((h, w, 3), np.float32)
        rgb8 = np.empty((h, w, 3), np.uint8)
        _check(_native.lib().ft_batch_read(self._h, item, _ptr(t), _ptr(mask), _ptr(rgb), _ptr(rgb8)))
        return {"t": t, "mask": mask, "rgb": rgb, "rgb8": rgb8}

    def close(self) -> None:
        if self._h:
            _native.lib().ft_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ differentiation

def views_c(views) -> ctypes.Array:
    """``ft_view`` array from (origin, target, fov_y_degrees) triples."""
    arr = (_native.ViewC * len(views))()
    for k, v in enumerate(views):
        if isinstance(v, _native.ViewC):
            arr[k] = v
        else:
            o, t, f = v
            arr[k] = _native.ViewC((ctypes.c_float * 3)(*o), (ctypes.c_float * 3)(*t), float(f))
    return arr


def ring_views(n: int, radius: float = 5.0, height: float = 1.5, fov: float = 45.0, target=(0.0, 0.0, 0.0)):
    """n cameras evenly spaced on a horizontal ring, looking at ``target``."""
    out = []
    for k in range(n):
        a = 2.0 * np.pi * k / n
        out.append(((radius * np.sin(a), height, -radius * np.cos(a)), tuple(target), fov))
    return out


class ParamScene:
    """A scene whose union_round tree(s) carry differentiable parameters:
    per sphere / box primitive (cx, cy, cz, rot_y, s0, s1, s2) and each
    tree's blend radius (``ft_scene_param_layout``)."""

    def __init__(self, source: str):
        self.state = SceneState(source)
        lib = _native.lib()
        n = ctypes.c_uint32()
        _check(lib.ft_scene_param_layout(self.state.desc_ptr, 0, None, ctypes.byref(n)))
        self.layout = (_native.ParamC * n.value)()
        _check(lib.ft_scene_param_layout(self.state.desc_ptr, n.value, self.layout, ctypes.byref(n)))

    @property
    def n_params(self) -> int:
        return len(self.layout)

    def names(self) -> list:
        return [f"node{p.node}.{_native.FT_PARAM_FIELDS[p.field]}" for p in self.layout]

    def get_params(self) -> np.ndarray:
        v = np.empty(self.n_params, np.float32)
        _check(_native.lib().ft_scene_desc_get_params(self.state.desc_ptr, self.layout, self.n_params, _ptr(v)))
        return v

    def set_params(self, values) -> None:
        v = np.ascontiguousarray(values, np.float32).reshape(-1)
        if v.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters")
        _check(_native.lib().ft_scene_desc_set_params(self.state.desc_ptr, self.layout, self.n_params, _ptr(v)))
        if self.state._gpu is not None:  # the GPU copy is rebuilt on next use
            self.state._gpu.close()
            self.state._gpu = None

    def render(self, views, options: RenderOptions, tau: float = 0.05):
        """(t, mask, sil), each (n_views, H, W): ``ft_render_views``."""
        varr = views_c(views)
        n, h, w = len(views), int(options.height), int(options.width)
        t = np.empty((n, h, w), np.float32)
        mask = np.empty((n, h, w), np.uint8)
        sil = np.empty((n, h, w), np.float32)
        opts = options.to_c()
        _check(_native.lib().ft_render_views(self.state.gpu().handle, varr, n, ctypes.byref(opts), float(tau),
                                             _ptr(t), _ptr(mask), _ptr(sil), 0, None))
        return t, mask, sil

    def backward(self, views, options: RenderOptions, dl_dt=None, dl_dsil=None, tau: float = 0.05) -> np.ndarray:
        """dL/dparams (float64) for upstream gradients of the depth and
        silhouette images: ``ft_render_backward``."""
        varr = views_c(views)
        a = None if dl_dt is None else np.ascontiguousarray(dl_dt, np.float32)
        b = None if dl_dsil is None else np.ascontiguousarray(dl_dsil, np.float32)
        g = np.zeros(self.n_params, np.float64)
        opts = options.to_c()
        _check(_native.lib().ft_render_backward(self.state.gpu().handle, varr, len(views), ctypes.byref(opts),
                                                float(tau), self.layout, self.n_params, _ptr(a), _ptr(b), _ptr(g), 0,
                                                None))
        return g


def render_function():
    """A ``torch.autograd.Function`` over ParamScene: forward renders depth and
    silhouette for a parameter tensor, backward is the adjoint march
    (``render_backward``).  Built lazily so importing the package does not
    import torch."""
    import torch

    class RenderViews(torch.autograd.Function):
        @staticmethod
        def forward(ctx, params, scene: ParamScene, views, options: RenderOptions, tau: float):
            scene.set_params(params.detach().cpu().numpy())
            t, mask, sil = scene.render(views, options, tau)
            ctx.scene, ctx.views, ctx.options, ctx.tau = scene, views, options, tau
            ctx.device, ctx.dtype = params.device, params.dtype
            out_t = torch.from_numpy(t).to(params.device)
            out_mask = torch.from_numpy(mask).to(params.device)
            out_sil = torch.from_numpy(sil).to(params.device)
            ctx.mark_non_differentiable(out_mask)
            return out_t, out_mask, out_sil

        @staticmethod
        def backward(ctx, grad_t, grad_mask, grad_sil):
            gt = None if grad_t is None else grad_t.detach().float().cpu().numpy()
            gs = None if grad_sil is None else grad_sil.detach().float().cpu().numpy()
            g = ctx.scene.backward(ctx.views, ctx.options, gt, gs, ctx.tau)
            return torch.from_numpy(g).to(ctx.device, ctx.dtype), None, None, None, None

    return RenderViews
