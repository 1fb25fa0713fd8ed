"""ctypes binding of the C ABI in ``include/forgedthoughts_gb300.h``.

The library is built in-tree (``forgedthoughts_gb300/_build``); importing this
module never falls back to another implementation: a missing library raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libforgedthoughts_gb300.so"

FT_OK = 0
FT_ERR_INVALID_ARGUMENT = 1
FT_ERR_MISSING_SCENE_ROOT = 2
FT_ERR_UNSUPPORTED_OBJECT = 3
FT_ERR_EXPECTED_OBJECT = 4
FT_ERR_PARSE = 5
FT_ERR_EVAL = 6
FT_ERR_CUDA = 7
FT_ERR_TIMEOUT = 8
FT_ERR_OUT_OF_MEMORY = 9
FT_ERR_UNSUPPORTED = 10
FT_ERR_NO_DEVICE = 11
FT_ERR_JIT = 12
FT_ERR_INTERNAL = 13
FT_ERR_IO = 14
FT_ERR_MISSING_IMPORT = 15
FT_ERR_IMPORT_CYCLE = 16
FT_ERR_AMBIGUOUS_IMPORT = 17

# ft_light_kind
FT_LIGHT_POINT = 0
FT_LIGHT_ENV = 1
FT_LIGHT_SPHERE = 2

# ft_node_kind: the primitives
FT_NODE_SPHERE = 0
FT_NODE_BOX = 1
FT_NODE_CYLINDER = 2
FT_NODE_TORUS = 3
FT_NODE_EXTRUDE_POLYGON = 4
FT_NODE_UNION = 8
FT_NODE_UNION_ROUND = 11
FT_NODE_CUSTOM = 30

FT_FLAG_DEVICE_POINTERS = 1
FT_FLAG_FP16_BRICKS = 2
FT_FLAG_JITTERED_AA = 4
FT_JITTER_SEED_SHIFT = 16
FT_BRICK_FREE_FAR_STEPS = 1
FT_MAT_STANDARD, FT_MAT_LAMBERT, FT_MAT_METAL, FT_MAT_DIELECTRIC = 0, 1, 2, 3  # ft_material_kind
# ft_material_hook: slots of ft_material.hook_program
(FT_HOOK_EMISSION_COLOR, FT_HOOK_EMISSION_STRENGTH, FT_HOOK_METALLIC, FT_HOOK_SPECULAR, FT_HOOK_SPECULAR_WEIGHT,
 FT_HOOK_TRANSMISSION, FT_HOOK_COAT_COLOR, FT_HOOK_COAT_ROUGHNESS, FT_HOOK_COAT_IOR, FT_HOOK_COAT_WEIGHT,
 FT_HOOK_COAT_MASK, FT_HOOK_BUMP, FT_HOOK_NORMAL, FT_HOOK_EVAL, FT_HOOK_PDF, FT_HOOK_SAMPLE_WI, FT_HOOK_SAMPLE_F,
 FT_HOOK_SAMPLE_PDF, FT_HOOK_SAMPLE_DELTA, FT_HOOK_SAMPLE_APPLY_COS, FT_HOOK_SAMPLE_TRANSMISSION,
 FT_HOOK_SAMPLE_THIN_WALLED, FT_HOOK_SAMPLE_NEXT_IOR, FT_HOOK_MEDIUM_IOR, FT_HOOK_MEDIUM_ABSORPTION,
 FT_HOOK_MEDIUM_DENSITY) = range(26)
FT_MATERIAL_HOOKS, FT_MATERIAL_HOOK_SLOTS = 26, 32
FT_MATERIAL_HOOK_PARAMS, FT_BSDF_HOOK_PARAMS = 7, 13
FT_MATERIAL_HOOK_PARAMS = 7
FT_ABI_VERSION = 4
FT_MAX_PROGRAM_REGS = 64


class RenderOptionsC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("max_steps", ctypes.c_uint32),
                ("max_dist", ctypes.c_float), ("epsilon", ctypes.c_float), ("step_scale", ctypes.c_float),
                ("camera_z", ctypes.c_float), ("fov_y_degrees", ctypes.c_float)]


class NodeC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_int32), ("b", ctypes.c_int32),
                ("program", ctypes.c_int32), ("object_id", ctypes.c_uint32), ("material_id", ctypes.c_uint32),
                ("ival", ctypes.c_int32), ("reserved", ctypes.c_int32), ("center", ctypes.c_float * 3),
                ("rot_deg", ctypes.c_float * 3), ("f", ctypes.c_float * 6), ("bounds_min", ctypes.c_float * 3),
                ("bounds_max", ctypes.c_float * 3)]


class InstrC(ctypes.Structure):
    _fields_ = [("op", ctypes.c_uint8), ("flags", ctypes.c_uint8), ("dst", ctypes.c_uint8), ("a", ctypes.c_uint8),
                ("b", ctypes.c_uint8), ("c", ctypes.c_uint8), ("pad", ctypes.c_uint8 * 2),
                ("imm", ctypes.c_float * 3)]


class ProgramC(ctypes.Structure):
    _fields_ = [("first_instr", ctypes.c_uint32), ("n_instr", ctypes.c_uint32), ("n_regs", ctypes.c_uint32),
                ("n_params", ctypes.c_uint32), ("param_is_vec3", ctypes.c_uint32),
                ("result_is_vec3", ctypes.c_uint32)]


class LightC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("samples", ctypes.c_uint32), ("position", ctypes.c_float * 3),
                ("radius", ctypes.c_float), ("intensity", ctypes.c_float * 3)]


class MaterialC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("has_medium", ctypes.c_int32), ("thin_walled", ctypes.c_int32),
                ("color_program", ctypes.c_int32), ("color", ctypes.c_float * 3), ("roughness", ctypes.c_float),
                ("metallic", ctypes.c_float), ("ior", ctypes.c_float), ("transmission", ctypes.c_float),
                ("emission_strength", ctypes.c_float), ("emission_color", ctypes.c_float * 3),
                ("medium_ior", ctypes.c_float), ("medium_absorption", ctypes.c_float * 3),
                ("medium_density", ctypes.c_float), ("specular", ctypes.c_float),
                ("specular_weight", ctypes.c_float), ("specular_color", ctypes.c_float * 3),
                ("clearcoat", ctypes.c_float), ("clearcoat_roughness", ctypes.c_float),
                ("roughness_program", ctypes.c_int32), ("ior_program", ctypes.c_int32),
                ("thin_walled_program", ctypes.c_int32), ("hook_program", ctypes.c_int32 * 32)]


class CameraC(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("target", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_y_degrees", ctypes.c_float)]


class SceneDescC(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_uint32), ("root", ctypes.c_int32), ("nodes", ctypes.POINTER(NodeC)),
                ("n_nodes", ctypes.c_uint32), ("n_instrs", ctypes.c_uint32), ("instrs", ctypes.POINTER(InstrC)),
                ("programs", ctypes.POINTER(ProgramC)), ("n_programs", ctypes.c_uint32),
                ("n_lights", ctypes.c_uint32), ("lights", ctypes.POINTER(LightC)),
                ("materials", ctypes.POINTER(MaterialC)), ("n_materials", ctypes.c_uint32),
                ("environment_program", ctypes.c_int32), ("camera", CameraC), ("has_camera", ctypes.c_int32),
                ("scene_center", ctypes.c_float * 3), ("settings_mask", ctypes.c_uint32),
                ("settings", RenderOptionsC), ("settings_accel", ctypes.c_int32)]


class LibraryItemC(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("path", ctypes.c_char_p), ("source", ctypes.c_char_p)]


class BuildInfoC(ctypes.Structure):
    _fields_ = [("leaves", ctypes.c_uint32), ("primitive_leaves", ctypes.c_uint32),
                ("generic_leaves", ctypes.c_uint32), ("union_round_leaves", ctypes.c_uint32),
                ("bvh_nodes", ctypes.c_uint32), ("grid_cells", ctypes.c_uint64), ("grid_entries", ctypes.c_uint64),
                ("grid_max_list", ctypes.c_uint32), ("generic_ops", ctypes.c_uint32), ("build_ms", ctypes.c_double),
                ("outer_grid_cells", ctypes.c_uint64), ("outer_grid_entries", ctypes.c_uint64)]


class RenderStatsC(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("distance_evals", ctypes.c_uint64), ("primitive_evals", ctypes.c_uint64),
                ("box_tests", ctypes.c_uint64), ("hook_instrs", ctypes.c_uint64), ("march_steps", ctypes.c_uint64),
                ("far_steps", ctypes.c_uint64), ("brick_fetches", ctypes.c_uint64), ("blend_ops", ctypes.c_uint64),
                ("candidate_entries", ctypes.c_uint64)]


FT_KERNEL_PRIMARY, FT_KERNEL_MARCH, FT_KERNEL_SHADE, FT_KERNEL_SHADOW, FT_KERNEL_PIXELS, FT_KERNEL_DEPTH_MARCH = range(6)
FT_KERNEL_KINDS = 6
KERNEL_KIND_NAMES = ["wf_primary_kernel", "wf_march_persistent", "wf_shade_kernel", "wf_shadow_persistent",
                     "pixels", "march_depth_persistent"]


class PathtraceSettingsC(ctypes.Structure):
    _fields_ = [("spp", ctypes.c_uint32), ("max_bounces", ctypes.c_uint32), ("min_spp", ctypes.c_uint32),
                ("noise_threshold", ctypes.c_float)]


class KernelTimesC(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * FT_KERNEL_KINDS), ("launches", ctypes.c_uint64 * FT_KERNEL_KINDS)]


class BrickOptionsC(ctypes.Structure):
    _fields_ = [("voxel_size", ctypes.c_float), ("band", ctypes.c_float), ("safety", ctypes.c_float),
                ("max_lattice_points", ctypes.c_uint32), ("far_steps_per_pass", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class BrickInfoC(ctypes.Structure):
    _fields_ = [("region_min", ctypes.c_float * 3), ("region_max", ctypes.c_float * 3),
                ("bricks", ctypes.c_uint32 * 3), ("near_bricks", ctypes.c_uint32), ("exact_leaves", ctypes.c_uint32),
                ("max_lipschitz", ctypes.c_float), ("band", ctypes.c_float), ("device_bytes", ctypes.c_uint64),
                ("build_ms", ctypes.c_double)]


class BatchItemC(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("options", RenderOptionsC), ("aa_samples", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32)]


class BatchTuningC(ctypes.Structure):
    _fields_ = [("tile_w", ctypes.c_uint32), ("tile_h", ctypes.c_uint32), ("refill", ctypes.c_uint32),
                ("ms", ctypes.c_float)]


FT_BATCH_FP16_BRICKS = 1


class JitInfoC(ctypes.Structure):
    _fields_ = [("programs", ctypes.c_uint32), ("cached", ctypes.c_uint32), ("source_bytes", ctypes.c_uint64),
                ("cubin_bytes", ctypes.c_uint64), ("compile_ms", ctypes.c_double), ("load_ms", ctypes.c_double)]


class ViewC(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("target", ctypes.c_float * 3), ("fov_y_degrees", ctypes.c_float)]


class ParamC(ctypes.Structure):
    _fields_ = [("node", ctypes.c_int32), ("field", ctypes.c_int32)]


FT_PARAM_FIELDS = ("cx", "cy", "cz", "rot_y", "s0", "s1", "s2", "radius")

# Every symbol include/forgedthoughts_gb300.h declares, with its signature.
SIGNATURES = {
    "ft_abi_version": (ctypes.c_uint32, []),
    "ft_last_error": (ctypes.c_char_p, []),
    "ft_scene_desc_from_source": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(SceneDescC))]),
    "ft_scene_desc_from_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(SceneDescC))]),
    "ft_scene_desc_from_file_with_library": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(LibraryItemC),
                                                             ctypes.c_uint32,
                                                             ctypes.POINTER(ctypes.POINTER(SceneDescC))]),
    "ft_scene_desc_free": (None, [ctypes.POINTER(SceneDescC)]),
    "ft_scene_create": (ctypes.c_int, [ctypes.POINTER(SceneDescC), ctypes.POINTER(ctypes.c_void_p)]),
    "ft_scene_destroy": (None, [ctypes.c_void_p]),
    "ft_scene_device_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "ft_scene_last_launches": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "ft_scene_build_info": (ctypes.c_int, [ctypes.POINTER(SceneDescC), ctypes.POINTER(BuildInfoC)]),
    "ft_render_depth": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                       ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]),
    "ft_render_trace": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                       ctypes.c_void_p]),
    "ft_render_depth_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(RenderStatsC)]),
    "ft_scene_build_bricks": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BrickOptionsC),
                                             ctypes.POINTER(BrickInfoC)]),
    "ft_scene_brick_bounds": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                             ctypes.c_void_p]),
    "ft_measure_fp32_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double)]),
    "ft_render_trace_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                             ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(RenderStatsC)]),
    "ft_render_trace_kernel_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(RenderStatsC),
                                                    ctypes.POINTER(RenderStatsC), ctypes.POINTER(RenderStatsC)]),
    "ft_scene_profile": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
    "ft_render_pathtrace": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                           ctypes.POINTER(PathtraceSettingsC), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]),
    "ft_scene_kernel_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(KernelTimesC)]),
    "ft_batch_create": (ctypes.c_int, [ctypes.POINTER(BatchItemC), ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "ft_batch_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchTuningC)]),
    "ft_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchTuningC)]),
    "ft_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "ft_batch_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    "ft_batch_samples": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "ft_batch_destroy": (None, [ctypes.c_void_p]),
    "ft_scene_param_layout": (ctypes.c_int, [ctypes.POINTER(SceneDescC), ctypes.c_uint32, ctypes.POINTER(ParamC),
                                             ctypes.POINTER(ctypes.c_uint32)]),
    "ft_scene_desc_get_params": (ctypes.c_int, [ctypes.POINTER(SceneDescC), ctypes.POINTER(ParamC), ctypes.c_uint32,
                                                ctypes.c_void_p]),
    "ft_scene_desc_set_params": (ctypes.c_int, [ctypes.POINTER(SceneDescC), ctypes.POINTER(ParamC), ctypes.c_uint32,
                                                ctypes.c_void_p]),
    "ft_render_views": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ViewC), ctypes.c_uint32,
                                       ctypes.POINTER(RenderOptionsC), ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p]),
    "ft_render_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ViewC), ctypes.c_uint32,
                                          ctypes.POINTER(RenderOptionsC), ctypes.c_float, ctypes.POINTER(ParamC),
                                          ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_uint32, ctypes.c_void_p]),
    "ft_scene_jit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(JitInfoC)]),
    "ft_render_depth_preview_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(RenderOptionsC), ctypes.c_int,
                                                       ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p]),
}

FT_NOALLOC_MAX_SAMPLES = 1 << 21

_lib = None


def lib() -> ctypes.CDLL:
    """Load the native library (built by ``forgedthoughts_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("FT_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise RuntimeError(
            f"native library {path} is missing; build it with `python -m forgedthoughts_gb300.build` "
            "(there is no non-native fallback)")
    handle = ctypes.CDLL(str(path), mode=ctypes.RTLD_GLOBAL)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    if handle.ft_abi_version() != FT_ABI_VERSION:
        raise RuntimeError("native library ABI version mismatch")
    _lib = handle
    return _lib


def last_error() -> str:
    msg = lib().ft_last_error()
    return msg.decode("utf-8", "replace") if msg else ""
