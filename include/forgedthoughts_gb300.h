/*
 * forgedthoughts_gb300 — C ABI of the GB300 (sm_103a) sphere-tracing library.
 *
 * This header is the drop-in boundary between a ForgedThoughts host (the Rust
 * `forgedthoughts` crate, or the C++/Python hosts shipped here) and the GPU
 * renderer.  Every entry point takes plain pointers and sizes; no C++ or torch
 * types cross it.  Each declaration names the reference function it replaces
 * (paths relative to the reference project root).
 *
 * Reference abbreviations used below:
 *   R = crates/forgedthoughts/src/renderer.rs
 *   E = crates/forgedthoughts/src/eval.rs
 *   M = crates/ftc/src/main.rs
 *
 * Threading: calls on distinct scene handles may run concurrently from
 * different host threads.  A single handle must not be used by two threads at
 * once.  ft_last_error() is thread-local.
 */
#ifndef FORGEDTHOUGHTS_GB300_H
#define FORGEDTHOUGHTS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FT_ABI_VERSION 4u

/* Status codes.  FT_ERR_MISSING_SCENE_ROOT / UNSUPPORTED_OBJECT /
 * EXPECTED_OBJECT mirror `enum RenderError` (R:159-168); PARSE / EVAL mirror
 * `CoreError::{Parse,Eval}` (crates/forgedthoughts/src/lib.rs:248-269). */
typedef enum ft_status {
  FT_OK = 0,
  FT_ERR_INVALID_ARGUMENT = 1,
  FT_ERR_MISSING_SCENE_ROOT = 2,
  FT_ERR_UNSUPPORTED_OBJECT = 3,
  FT_ERR_EXPECTED_OBJECT = 4,
  FT_ERR_PARSE = 5,
  FT_ERR_EVAL = 6,
  FT_ERR_CUDA = 7,
  FT_ERR_TIMEOUT = 8,
  FT_ERR_OUT_OF_MEMORY = 9,
  FT_ERR_UNSUPPORTED = 10,
  FT_ERR_NO_DEVICE = 11,
  FT_ERR_JIT = 12,          /* run-time compilation (NVRTC) or module load failed */
  FT_ERR_INTERNAL = 13,     /* an unexpected host-side failure; no C++ exception crosses this ABI */
  /* Scene-file loading, `CoreError::{Io,MissingImport,ImportCycle}`
   * (crates/forgedthoughts/src/lib.rs:251-262). */
  FT_ERR_IO = 14,             /* a scene file could not be read */
  FT_ERR_MISSING_IMPORT = 15, /* a relative import names no file */
  FT_ERR_IMPORT_CYCLE = 16,   /* a file imports itself through a chain of imports */
  FT_ERR_AMBIGUOUS_IMPORT = 17 /* a library name matches several items (`AmbiguousBuiltinImport`) */
} ft_status;

/* `enum AccelMode` (R:58-63). */
typedef enum ft_accel_mode {
  FT_ACCEL_NAIVE = 0,
  FT_ACCEL_BVH = 1,
  FT_ACCEL_BRICKS = 2
} ft_accel_mode;

/* `struct RenderOptions` (R:32-56); defaults 800x800, 128 steps, max_dist 40,
 * epsilon 1e-3, step_scale 0.7, camera_z 6, fov 45. */
typedef struct ft_render_options {
  uint32_t width;
  uint32_t height;
  uint32_t max_steps;
  float max_dist;
  float epsilon;
  float step_scale;
  float camera_z;
  float fov_y_degrees;
} ft_render_options;

/* ---------------------------------------------------------------------------
 * Flat scene IR.  A lowered `SdfNode` tree (R:171-355) as an array of nodes
 * addressed by index, plus the hook programs that replace the Cranelift JIT
 * (crates/forgedthoughts/src/jit.rs:501-747) and the render setup (camera,
 * lights, materials, environment) built by `build_render_setup` (R:6242).
 * ------------------------------------------------------------------------- */

typedef enum ft_node_kind {
  FT_NODE_SPHERE = 0,          /* f0 radius, f1 shell */
  FT_NODE_BOX = 1,             /* f0..f2 half size, f3 round, f4 shell */
  FT_NODE_CYLINDER = 2,        /* f0 radius, f1 half height, f2 round, f3 shell */
  FT_NODE_TORUS = 3,           /* f0 major radius, f1 minor radius */
  FT_NODE_EXTRUDE_POLYGON = 4, /* ival sides, f0 radius, f1 half height, f2 round, f3 shell */
  FT_NODE_DOMAIN = 5,          /* a base, program domain(p)->vec3, transform, bounds */
  FT_NODE_DISTANCE_POST = 6,   /* a base, program distance_post(d,p)->f32, transform, bounds */
  FT_NODE_NOISE = 7,           /* a base, ival octaves, f0 scale, f1 lacunarity, transform, bounds */
  FT_NODE_UNION = 8,           /* hard `+` */
  FT_NODE_INTERSECT = 9,       /* `&` */
  FT_NODE_SUBTRACT = 10,       /* `-` */
  FT_NODE_UNION_ROUND = 11,    /* f0 r */
  FT_NODE_UNION_CHAMFER = 12,  /* f0 r */
  FT_NODE_UNION_COLUMNS = 13,  /* f0 r, f1 n */
  FT_NODE_UNION_STAIRS = 14,   /* f0 r, f1 n */
  FT_NODE_UNION_SOFT = 15,     /* f0 r */
  FT_NODE_INTERSECT_ROUND = 16,
  FT_NODE_INTERSECT_CHAMFER = 17,
  FT_NODE_INTERSECT_COLUMNS = 18,
  FT_NODE_INTERSECT_STAIRS = 19,
  FT_NODE_DIFF_ROUND = 20,
  FT_NODE_DIFF_CHAMFER = 21,
  FT_NODE_DIFF_COLUMNS = 22,
  FT_NODE_DIFF_STAIRS = 23,
  FT_NODE_PIPE = 24,           /* f0 r */
  FT_NODE_ENGRAVE = 25,        /* f0 r */
  FT_NODE_GROOVE = 26,         /* f0 ra, f1 rb */
  FT_NODE_TONGUE = 27,         /* f0 ra, f1 rb */
  FT_NODE_SLICE = 28,          /* a base, ival axis, f0 min, f1 max */
  FT_NODE_SMOOTH = 29,         /* a base, f0 k */
  FT_NODE_CUSTOM = 30,         /* user `sdf` definition (SdfNode::Custom, R:213-220): program = distance(p),
                                  ival = domain(p) program or -1, reserved = distance_post(d, p) program or
                                  -1, f0..f2 bounds() half extents, transform, bounds = world box; no children */
  FT_NODE_KIND_COUNT = 31
} ft_node_kind;

typedef struct ft_node {
  int32_t kind;          /* ft_node_kind */
  int32_t a;             /* lhs / base child index, -1 if none */
  int32_t b;             /* rhs child index, -1 if none */
  int32_t program;       /* hook program index for DOMAIN / DISTANCE_POST, else -1 */
  uint32_t object_id;    /* primitives only */
  uint32_t material_id;  /* primitives only */
  int32_t ival;          /* sides / axis / octaves */
  int32_t reserved;
  float center[3];       /* PrimitiveTransform::center (R:368-372) */
  float rot_deg[3];      /* PrimitiveTransform::rot_deg, degrees */
  float f[6];            /* kind-specific parameters, see ft_node_kind */
  float bounds_min[3];   /* stored AABB of DOMAIN / DISTANCE_POST / NOISE */
  float bounds_max[3];
} ft_node;

/* Hook programs: typed register code lowered from `.ft` function bodies.
 * Registers hold a vec3; scalar registers use lane x.  Operand flag bits
 * FT_INSTR_A_SCALAR etc. mark scalar operands broadcast to vec3. */
typedef enum ft_opcode {
  FT_OP_CONST = 0,   /* dst = imm (vec3; scalar uses imm[0]) */
  FT_OP_MOV = 1,
  FT_OP_ADD = 2,
  FT_OP_SUB = 3,
  FT_OP_MUL = 4,
  FT_OP_DIV = 5,
  FT_OP_NEG = 6,
  FT_OP_GETX = 7,
  FT_OP_GETY = 8,
  FT_OP_GETZ = 9,
  FT_OP_VEC3 = 10,   /* dst = (a.x, b.x, c.x) */
  FT_OP_ABS = 11,
  FT_OP_FLOOR = 12,
  FT_OP_CEIL = 13,
  FT_OP_FRACT = 14,
  FT_OP_SQRT = 15,
  FT_OP_SIN = 16,
  FT_OP_COS = 17,
  FT_OP_SATURATE = 18,
  FT_OP_MIN = 19,
  FT_OP_MAX = 20,
  FT_OP_POW = 21,
  FT_OP_CLAMP = 22,
  FT_OP_MIX = 23,
  FT_OP_STEP = 24,        /* scalar: x < edge ? 0 : 1, a = edge, b = x */
  FT_OP_SMOOTHSTEP = 25,  /* scalar: a = edge0, b = edge1, c = x */
  FT_OP_DOT = 26,
  FT_OP_LENGTH = 27,
  FT_OP_NORMALIZE = 28,
  FT_OP_ROTX = 29,        /* a = vec3, b = degrees */
  FT_OP_ROTY = 30,
  FT_OP_ROTZ = 31,
  FT_OP_RET = 32,
  FT_OP_COUNT = 33
} ft_opcode;

#define FT_INSTR_VEC3 1u      /* result is a vec3 (else scalar) */
#define FT_INSTR_A_SCALAR 2u  /* operand a is scalar: broadcast */
#define FT_INSTR_B_SCALAR 4u
#define FT_INSTR_C_SCALAR 8u

typedef struct ft_instr {
  uint8_t op;     /* ft_opcode */
  uint8_t flags;  /* FT_INSTR_* */
  uint8_t dst;
  uint8_t a;
  uint8_t b;
  uint8_t c;
  uint8_t pad[2];
  float imm[3];
} ft_instr;

#define FT_MAX_PROGRAM_REGS 64

typedef struct ft_program {
  uint32_t first_instr;  /* index into ft_scene_desc::instrs */
  uint32_t n_instr;
  uint32_t n_regs;       /* <= FT_MAX_PROGRAM_REGS; params occupy r0.. */
  uint32_t n_params;
  uint32_t param_is_vec3; /* bit i set: parameter i is a vec3 */
  uint32_t result_is_vec3;
} ft_program;

typedef enum ft_light_kind {
  FT_LIGHT_POINT = 0,   /* render_api.rs:172-188 */
  FT_LIGHT_ENV = 1,     /* render_api.rs:190-205 */
  FT_LIGHT_SPHERE = 2   /* render_api.rs:207-259 */
} ft_light_kind;

typedef struct ft_light {
  int32_t kind;
  uint32_t samples;      /* SphereLight shadow samples */
  float position[3];
  float radius;
  float intensity[3];    /* radiance for FT_LIGHT_ENV */
} ft_light;

typedef enum ft_material_kind {
  FT_MAT_STANDARD = 0,
  FT_MAT_LAMBERT = 1,
  FT_MAT_METAL = 2,
  FT_MAT_DIELECTRIC = 3
} ft_material_kind;

/* Slots of ft_material.hook_program (FT_MATERIAL_HOOKS used, the rest -1). */
#define FT_MATERIAL_HOOK_SLOTS 32

/* Subset of `MaterialParams` (crates/forgedthoughts/src/materials/mod.rs:66-86)
 * read by the Whitted integrator. */
typedef struct ft_material {
  int32_t kind;            /* ft_material_kind */
  int32_t has_medium;
  int32_t thin_walled;
  int32_t color_program;   /* per-hit `fn color(ctx)` hook (vec3 or number), -1 if none */
  float color[3];
  float roughness;
  float metallic;
  float ior;
  float transmission;
  float emission_strength;
  float emission_color[3];
  float medium_ior;
  float medium_absorption[3];
  float medium_density;
  float specular;
  float specular_weight;
  float specular_color[3];
  float clearcoat;
  float clearcoat_roughness;
  int32_t roughness_program;  /* per-hit `fn roughness(ctx)` hook (number), -1 if none */
  int32_t ior_program;        /* per-hit `fn ior(ctx)` hook (number), -1 if none */
  int32_t thin_walled_program; /* per-hit `fn thin_walled(ctx)` hook (number, >= 0.5 thin), -1 if none */
  int32_t hook_program[FT_MATERIAL_HOOK_SLOTS]; /* the further hooks by ft_material_hook; -1 if none */
} ft_material;

/* The further hooks of a material definition (crates/forgedthoughts/src/
 * renderer.rs, "R:" below), by slot of ft_material.hook_program.  The
 * property hooks take the shading context (FT_MATERIAL_HOOK_PARAMS) and are
 * applied where a leaf's material is resolved (resolve_leaf_material,
 * R:7164-7530), with the reference's clamps:
 *   every definition    emission_color (vec3 or number), emission_strength
 *                       (>= 0);
 *   Standard / Layered  metallic, specular, specular_weight, transmission
 *                       ([0, 1]) and the coat: coat_color, coat_roughness
 *                       ([0, 1]), coat_ior ([1, 3]), coat_weight and
 *                       coat_mask ([0, 1]), which replace the specular
 *                       colour, IOR, clearcoat (weight x mask) and clearcoat
 *                       roughness at every hit (R:7397-7468);
 *   every definition    `fn medium(ctx)` (a Medium record; its ior, absorption_color
 *                       and density fields one program each, defaulted and clamped
 *                       as medium_from_value, R:6834-6845), replacing the
 *                       material's medium (R:7217-7226).
 * The shading-normal hooks (build_bsdf_context, R:4397-4449) belong to the
 * hit's own material: `fn bump(ctx)` (number, a height field differentiated
 * along a tangent frame, R:7776-7818), then `fn normal(ctx)` (vec3,
 * R:7749-7774), each seeing the normal so far as ctx.normal.
 * The BSDF hooks (R:4905-4950) belong to the dominant parameters of the
 * shaded material (a blend of two parameter sets keeps none) and take the
 * BSDF context (FT_BSDF_HOOK_PARAMS): `fn eval(ctx)` replaces Material::eval
 * in the Whitted light loop and the path tracer, `fn pdf(ctx)`
 * Material::pdf, and `fn sample(ctx)` Material::sample in the path tracer;
 * the sample's record fields are one program each (wi and f are required,
 * the others default as bsdf_sample_from_value, R:5032-5060, reads them). */
typedef enum ft_material_hook {
  FT_HOOK_EMISSION_COLOR = 0,
  FT_HOOK_EMISSION_STRENGTH = 1,
  FT_HOOK_METALLIC = 2,
  FT_HOOK_SPECULAR = 3,
  FT_HOOK_SPECULAR_WEIGHT = 4,
  FT_HOOK_TRANSMISSION = 5,
  FT_HOOK_COAT_COLOR = 6,
  FT_HOOK_COAT_ROUGHNESS = 7,
  FT_HOOK_COAT_IOR = 8,
  FT_HOOK_COAT_WEIGHT = 9,
  FT_HOOK_COAT_MASK = 10,
  FT_HOOK_BUMP = 11,
  FT_HOOK_NORMAL = 12,
  FT_HOOK_EVAL = 13,
  FT_HOOK_PDF = 14,
  FT_HOOK_SAMPLE_WI = 15,
  FT_HOOK_SAMPLE_F = 16,
  FT_HOOK_SAMPLE_PDF = 17,
  FT_HOOK_SAMPLE_DELTA = 18,
  FT_HOOK_SAMPLE_APPLY_COS = 19,
  FT_HOOK_SAMPLE_TRANSMISSION = 20,
  FT_HOOK_SAMPLE_THIN_WALLED = 21,
  FT_HOOK_SAMPLE_NEXT_IOR = 22,
  FT_HOOK_MEDIUM_IOR = 23,
  FT_HOOK_MEDIUM_ABSORPTION = 24,
  FT_HOOK_MEDIUM_DENSITY = 25,
  FT_MATERIAL_HOOKS = 26
} ft_material_hook;

/* Material hook programs take the shading context of a hit
 * (make_shading_context, R:7875-7911) as seven parameters: position,
 * local_position (the hit in the leaf primitive's frame), normal (facing the
 * ray), view_dir (-ray direction) as vec3s, then front_face (1 or 0),
 * object_id and material_id as numbers. */
#define FT_MATERIAL_HOOK_PARAMS 7
/* BSDF hook programs (bsdf_context_value, R:5006-5030) take those seven with
 * normal = the shading normal, then wo, wi (vec3s), current_ior and, for
 * `fn sample`, the random numbers u1, u2, u3 (numbers): thirteen parameters,
 * of which eval and pdf read the first ten. */
#define FT_BSDF_HOOK_PARAMS 13

typedef struct ft_camera {
  float origin[3];
  float target[3];
  float up[3];
  float fov_y_degrees;
} ft_camera;

typedef struct ft_scene_desc {
  uint32_t abi_version;         /* FT_ABI_VERSION */
  int32_t root;                 /* index of the scene root node */
  const ft_node* nodes;
  uint32_t n_nodes;
  uint32_t n_instrs;
  const ft_instr* instrs;
  const ft_program* programs;
  uint32_t n_programs;
  uint32_t n_lights;
  const ft_light* lights;       /* in shading order */
  const ft_material* materials; /* material_id indexes this; 0 = default */
  uint32_t n_materials;
  int32_t environment_program;  /* `environment X { fn color(dir) }`, -1 if none */
  ft_camera camera;
  int32_t has_camera;           /* 0: camera derived from scene centre (R:6263-6286) */
  float scene_center[3];        /* sdf_center of the root (R:4048-4089) */
  /* RenderSettings found in the scene (R:1316-1354); has_* flags mark presence */
  uint32_t settings_mask;       /* bit i: field i of ft_render_options present */
  ft_render_options settings;
  int32_t settings_accel;       /* -1 none, else ft_accel_mode */
} ft_scene_desc;

typedef struct ft_scene ft_scene;

/* Render-call flags. */
#define FT_FLAG_DEVICE_POINTERS 1u  /* output pointers are device memory */
/* Jittered AA (ft_render_depth / ft_render_trace): sample s of pixel (x, y)
 * is offset by two draws of XorShift64 seeded with
 * seed_pixel_sample(x, y, width, s) ^ seed (R:4735-4774, the progressive
 * renderer's sampling), seed = flags >> FT_JITTER_SEED_SHIFT, instead of the
 * sqrt(aa) x sqrt(aa) grid of pixel_sample_offsets (R:4838-4854). */
#define FT_FLAG_JITTERED_AA 4u
#define FT_JITTER_SEED_SHIFT 16
#define FT_FLAG_JITTER_SEED(seed) (((uint32_t)(seed) & 0xffffu) << FT_JITTER_SEED_SHIFT)
#define FT_FLAG_FP16_BRICKS 2u      /* depth march through the FP16 brick cache
                                       (ft_scene_build_bricks must have run);
                                       for ft_render_trace, the primary hits
                                       come from that march and every later
                                       bounce is the plain march */

/* ---------------------------------------------------------------------------
 * Entry points.
 * ------------------------------------------------------------------------- */

/* Library ABI version (FT_ABI_VERSION). */
uint32_t ft_abi_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* ft_last_error(void);

/* `.ft` front-end: parse + evaluate + lower a scene source.  Replaces
 * `parse_program` (crates/forgedthoughts/src/parser.rs:25), `eval_program`
 * (E:138-162) and `compile_scene` (R:1384-1401) for hosts without the Rust
 * crate.  The returned description is owned by the library; release it with
 * ft_scene_desc_free. */
ft_status ft_scene_desc_from_source(const char* source, ft_scene_desc** out);

/* The same for a scene file, with its imports resolved: replaces
 * `load_and_eval_scene` / `load_program_with_imports`
 * (crates/forgedthoughts/src/lib.rs:280-383).  `import "./x.ft";` and
 * `import "../x.ft" as name;` load from the importing file's directory; an
 * aliased import's top-level names become `name.binding`; a file with an
 * `export { ... };` list contributes only those names and their
 * dependencies; each (file, alias) pair is loaded once.  Imports that name
 * the reference's built-in library (paths without ./ or ../) return
 * FT_ERR_UNSUPPORTED: that library is not shipped.  A source passed to
 * ft_scene_desc_from_source has no directory, so an import there returns
 * FT_ERR_UNSUPPORTED as well. */
ft_status ft_scene_desc_from_file(const char* path, ft_scene_desc** out);

/* One item of an asset library, the role of `BuiltinLibraryItem`
 * (crates/forgedthoughts/src/lib.rs:54-61): `import "materials/gold.ft";`
 * selects an item by `path`, `import "Gold";` by `name` (a name that several
 * items share is FT_ERR_AMBIGUOUS_IMPORT). */
typedef struct ft_library_item {
  const char* name;
  const char* path;
  const char* source; /* the item's `.ft` text */
} ft_library_item;

/* ft_scene_desc_from_file with an asset library for imports that are not
 * relative paths (`resolve_import`, lib.rs:385-416): the reference passes its
 * built-in library table here.  With a library, an import that matches no
 * item is FT_ERR_MISSING_IMPORT; imports inside an item resolve relative
 * paths from the working directory, as the reference's do.  The strings are
 * read during the call only. */
ft_status ft_scene_desc_from_file_with_library(const char* path, const ft_library_item* items, uint32_t n_items,
                                               ft_scene_desc** out);
void ft_scene_desc_free(ft_scene_desc* desc);

/* Upload a scene to the current CUDA device and build its culling structures
 * (leaf list + BVH, `Accelerator::from_scene`, R:609-623, R:1024-1129).  The
 * description is copied; the caller keeps ownership of `desc`. */
ft_status ft_scene_create(const ft_scene_desc* desc, ft_scene** out);
void ft_scene_destroy(ft_scene* scene);

/* Host-only summary of the culling structures ft_scene_create would build for
 * `desc` (no device needed): hard-union leaves by evaluation kind, the
 * union_round trees and their candidate grids. */
typedef struct ft_build_info {
  uint32_t leaves;
  uint32_t primitive_leaves;
  uint32_t generic_leaves;
  uint32_t union_round_leaves;
  uint32_t bvh_nodes;
  uint64_t grid_cells;
  uint64_t grid_entries;      /* sum of candidate-list lengths */
  uint32_t grid_max_list;
  uint32_t generic_ops;
  double build_ms;            /* host time to build the structures */
  uint64_t outer_grid_cells;  /* the coarser grids around the union_round trees' grids */
  uint64_t outer_grid_entries;
} ft_build_info;

ft_status ft_scene_build_info(const ft_scene_desc* desc, ft_build_info* info);

/* Bytes of scene data the last ft_scene_create copied host -> device. */
ft_status ft_scene_device_bytes(const ft_scene* scene, uint64_t* bytes);

/* Kernels launched by the scene's last ft_render_depth or ft_render_trace
 * call (the Whitted trace launches a data-dependent number: three per bounce
 * level that still holds rays).  No counterpart in the reference
 * (measurement). */
ft_status ft_scene_last_launches(const ft_scene* scene, uint32_t* launches);

/* Depth preview: `render_depth_png_with_accel` (R:1139-1156) /
 * `render_preview_progressive_with_accel` (R:1238-1277) without the PNG step.
 * One primary ray per (pixel, AA offset) with the reference's deterministic
 * sqrt(aa) x sqrt(aa) offset grid (R:4838-4854).  Outputs (each nullable):
 *   t_out        width*height*aa floats, refined hit distance, 0 on miss
 *   mask_out     width*height*aa bytes, 1 = hit
 *   material_out width*height*aa uint32 material ids (0 on miss)
 *   normal_out   width*height*aa*3 floats, estimate_normal at the hit
 *                (R:4202-4215), 0 on miss
 *   rgb8_out     width*height*3 bytes, the reference's gray depth preview
 * Sample index within a pixel is the offset index.  With
 * FT_FLAG_DEVICE_POINTERS the outputs are device pointers and no host copy is
 * made.  `stream` is a cudaStream_t (NULL = legacy default stream); the call
 * returns after the work on `stream` has completed. */
ft_status ft_render_depth(ft_scene* scene, const ft_render_options* options,
                          ft_accel_mode accel, uint32_t aa_samples,
                          float* t_out, uint8_t* mask_out,
                          uint32_t* material_out, float* normal_out,
                          uint8_t* rgb8_out, uint32_t flags, void* stream);

/* Whitted trace: `render_ray_progressive_with_accel` (R:1201-1236) /
 * `trace_ray_recursive` (crates/forgedthoughts/src/renderer/ray.rs:3-222)
 * without the tile callback.  max_depth is RaySettings::max_depth (1..10).
 * Outputs (each nullable):
 *   rgb_out   width*height*3 floats, linear radiance averaged over AA samples
 *   rgb8_out  width*height*3 bytes, Reinhard + gamma 2.2 (R:5229-5239)
 * Other arguments as ft_render_depth. */
ft_status ft_render_trace(ft_scene* scene, const ft_render_options* options,
                          ft_accel_mode accel, uint32_t aa_samples, uint32_t max_depth,
                          float* rgb_out, uint8_t* rgb8_out, uint32_t flags, void* stream);

/* Kernel statistics of the last render on this scene: number of distance
 * evaluations, primitive evaluations and culling-box tests, summed over all
 * rays (used for the FP32 roofline). */
typedef struct ft_render_stats {
  uint64_t rays;
  uint64_t distance_evals;
  uint64_t primitive_evals;
  uint64_t box_tests;
  uint64_t hook_instrs;
  uint64_t march_steps;     /* exact (FP32) march steps */
  uint64_t far_steps;       /* far-field steps on the FP16 brick bound */
  uint64_t brick_fetches;   /* trilinear FP16 texture fetches */
  uint64_t blend_ops;       /* union_round combines of the restricted folds */
  uint64_t candidate_entries; /* candidate-grid list entries tested */
} ft_render_stats;

/* Depth preview for callers that cannot allocate device memory.
 *
 * No counterpart in the reference: it exists for hosts that must not call
 * cudaMalloc while rendering, such as an engine whose allocator owns all
 * device memory, a real-time loop that cannot afford the implicit device
 * synchronisation of cudaMalloc/cudaFree, or a plugin running inside another
 * framework's memory budget.  Output is the same gray preview as
 * ft_render_depth's rgb8_out, written to `rgb8_out`, a DEVICE pointer of
 * width*height*3 bytes owned by the caller.
 *
 * The per-sample depth and hit mask live in one fixed scratch array inside the
 * library (FT_NOALLOC_MAX_SAMPLES samples, 5 bytes each, about 10 MiB), which
 * every GPU that loads the library holds until the process exits.  Calls with
 * width*height*max(aa,1) above FT_NOALLOC_MAX_SAMPLES fail with
 * FT_ERR_INVALID_ARGUMENT and launch nothing.  The first call on a device
 * looks up that array's device address (a one-time set-up); make that first
 * call before any stream capture.  The address is kept for the life of the
 * process, so do not use this entry point on a device after cudaDeviceReset
 * (or any other teardown of its primary context), which moves the array.
 * The call allocates nothing, enqueues its
 * two kernels on `stream` and returns without waiting: the image is ready
 * when the stream's work completes.  All calls share the scratch array and it
 * keeps the last call's contents, so calls whose work can overlap on the GPU
 * (other streams, other threads) race with each other; serialise them. */
#define FT_NOALLOC_MAX_SAMPLES (1u << 21)
ft_status ft_render_depth_preview_noalloc(ft_scene* scene, const ft_render_options* options,
                                          ft_accel_mode accel, uint32_t aa_samples,
                                          uint8_t* rgb8_out, void* stream);

/* Counters of one depth march with `flags` (FT_FLAG_FP16_BRICKS selects the
 * precision form); the outputs are discarded. */
ft_status ft_render_depth_stats(ft_scene* scene, const ft_render_options* options,
                                ft_accel_mode accel, uint32_t aa_samples, uint32_t flags,
                                ft_render_stats* stats);

/* The same counters for a Whitted trace (ft_render_trace); output discarded.
 * They come from counting variants of the wavefront's own kernels (march,
 * shade, shadow), summed over every bounce level. */
ft_status ft_render_trace_stats(ft_scene* scene, const ft_render_options* options,
                                ft_accel_mode accel, uint32_t aa_samples, uint32_t max_depth,
                                ft_render_stats* stats);

/* `PathtraceSettings` (R:107-125): samples per pixel, bounces, and the
 * adaptive stop (a pixel stops after min_spp samples once the relative
 * standard error of its luminance is at most noise_threshold; 0 disables). */
typedef struct ft_pathtrace_settings {
  uint32_t spp;             /* default 16 */
  uint32_t max_bounces;     /* default 4 */
  uint32_t min_spp;         /* default 8 */
  float noise_threshold;    /* default 0.03 */
} ft_pathtrace_settings;

/* The reference's MIS path tracer (render_pathtrace_with_accel_progressive,
 * R:3974-4045; trace_path renderer/path.rs:3-112; estimate_direct_mis
 * R:4572-4704).  Dead code in the reference (no CLI entry); here a render
 * entry point.  Every pixel sample draws from its own XorShift64 seeded by
 * seed_pixel_sample (R:4735-4774), so the image is deterministic.  Outputs
 * (each nullable): the average linear radiance (width*height*3 floats), its
 * spectrum_to_rgb8 (R:5221-5227) and the samples each pixel took.  The
 * reference's preview callback (preview_every) is left to the caller: the
 * call returns the final image. */
ft_status ft_render_pathtrace(ft_scene* scene, const ft_render_options* options, ft_accel_mode accel,
                              const ft_pathtrace_settings* settings, float* rgb_out, uint8_t* rgb8_out,
                              uint32_t* samples_out, uint32_t flags, void* stream);

/* The trace's counters per wavefront kernel kind: the ray march
 * (wf_march_persistent), the shading of the hits (wf_shade_kernel) and the
 * soft-shadow march (wf_shadow_persistent).  No counterpart in the reference
 * (measurement). */
ft_status ft_render_trace_kernel_stats(ft_scene* scene, const ft_render_options* options,
                                       ft_accel_mode accel, uint32_t aa_samples, uint32_t max_depth,
                                       ft_render_stats* march, ft_render_stats* shade,
                                       ft_render_stats* shadow);

/* Per-kernel device time of a scene's renders, measured with a CUDA event
 * pair around every launch on the launch's own stream.  No counterpart in the
 * reference (measurement). */
#define FT_KERNEL_PRIMARY 0     /* wf_primary_kernel: camera rays of a trace */
#define FT_KERNEL_MARCH 1       /* wf_march_persistent: the trace's ray march */
#define FT_KERNEL_SHADE 2       /* wf_shade_kernel */
#define FT_KERNEL_SHADOW 3      /* wf_shadow_persistent */
#define FT_KERNEL_PIXELS 4      /* AA average / preview pixels */
#define FT_KERNEL_DEPTH_MARCH 5 /* march_depth_persistent */
#define FT_KERNEL_KINDS 6

typedef struct ft_kernel_times {
  double ms[FT_KERNEL_KINDS];          /* summed launch durations */
  uint64_t launches[FT_KERNEL_KINDS];  /* launches timed */
} ft_kernel_times;

/* enable != 0 starts timing every kernel that ft_render_depth / ft_render_trace
 * launch on this scene (the sums restart at zero); 0 stops it. */
ft_status ft_scene_profile(ft_scene* scene, uint32_t enable);
/* The sums since the last ft_scene_profile call. */
ft_status ft_scene_kernel_times(ft_scene* scene, ft_kernel_times* out);

/* FP16 brick distance cache: the precision form of the depth march.
 *
 * No counterpart in the reference, whose `Bricks` accelerator is a grid of
 * leaf lists (R:824-1022).  The scene's distance field without its few very
 * large leaves (a ground box) is sampled on a lattice of `voxel_size` over the
 * region around the other leaves, cut into bricks of 8^3 voxels.  Each brick
 * gets an interpolation error bound (its Lipschitz estimate x voxel diagonal
 * x `safety`); every lattice point is stored as one FP16 texel of a 3D
 * texture holding the sample minus the largest bound of the bricks sharing
 * it, rounded down, so a hardware trilinear fetch is a lower bound of the
 * distance.  Bricks whose Lipschitz estimate exceeds 4 (the field jumps there,
 * e.g. where the reference's leaf culling switches), and bricks a hooked or
 * modified leaf can reach (hooks move surfaces off their boxes; a domain +
 * distance_post pair applies its transform twice), store no bound: the march
 * is exact inside them.
 *
 * ft_render_depth with FT_FLAG_FP16_BRICKS (default, counted form) takes the
 * plain method's samples, so it ends on the same rays as the plain march,
 * including those the plain march gives up on at its step limit.  When the
 * only large leaf is an axis-aligned box (a ground), the nearest leaf at a
 * sample is that box, the ray descends onto its top face, and the cached
 * leaves are farther than the face along the ray (one fetch; outside the
 * brick region the distance to the region's box less the largest blend
 * radius, for scenes without hooked or modified leaves), the rest of the
 * approach is the plain march towards a plane: its step count is computed in
 * closed form, and the march jumps to the eps-shell crossing.
 * With FT_BRICK_FREE_FAR_STEPS it instead marches on the bound while it is at
 * least `band`, stepping by the bound minus band/2, then continues with the
 * exact FP32 march of the plain method (same step rule), returning to the far
 * field when the exact distance exceeds band_exit.  In both forms secant
 * steps on the exact distance between the last two exact points find the
 * eps-shell crossing at a hit (each verified by an exact evaluation), and the
 * normal is the plain method's six-tap estimate.  Build once per scene;
 * rebuilding replaces the cache.  Synchronous on the legacy default stream. */
typedef struct ft_brick_options {
  float voxel_size;             /* lattice spacing; 0 = 0.02 */
  float band;                   /* far-field threshold; 0 = 10 voxels */
  float safety;                 /* factor on the error bound; 0 = 1.25 */
  uint32_t max_lattice_points;  /* refuse larger lattices; 0 = 2^29 */
  uint32_t far_steps_per_pass;  /* far-field steps a lane takes per pass of its warp; 0 = 4 */
  uint32_t flags;               /* FT_BRICK_* */
} ft_brick_options;

/* March the far field with free steps (bound minus band/2, each counted as one
 * step of the plain method) instead of the default counted form below; on
 * rays the plain march gives up on (its step limit) the two can disagree. */
#define FT_BRICK_FREE_FAR_STEPS 1u

typedef struct ft_brick_info {
  float region_min[3];
  float region_max[3];
  uint32_t bricks[3];         /* bricks per axis */
  uint32_t near_bricks;       /* bricks with a surface within band + half a brick */
  uint32_t exact_leaves;      /* large leaves evaluated exactly */
  float max_lipschitz;        /* largest per-brick Lipschitz estimate */
  float band;                 /* effective far-field threshold */
  uint64_t device_bytes;      /* FP16 texture */
  double build_ms;
} ft_brick_info;

ft_status ft_scene_build_bricks(ft_scene* scene, const ft_brick_options* options, ft_brick_info* info);

/* Far-field bound and exact scene distance at `n` points (host arrays of
 * n*3 / n floats): bound_out[i] is the brick cache's lower bound (NaN outside
 * the brick region), exact_out[i] the exact FP32 distance of the plain march.
 * For validating the cache. */
ft_status ft_scene_brick_bounds(ft_scene* scene, const float* points, uint32_t n, float* bound_out,
                                float* exact_out);

/* ---------------------------------------------------------------------------
 * Batched form: many independent renders (scenes, views, resolutions, depth
 * previews and Whitted traces mixed) in one CUDA-graph launch.  No
 * counterpart in the reference, which renders one scene per call.
 *
 * The depth items run in one persistent march kernel whose warps take rays of
 * any item from a global counter (a lane keeps its item's scene, parameters
 * and brick cache).  The trace items run as one wavefront over all of them:
 * per bounce level (up to the largest max_depth) a march, a shade and a
 * shadow kernel over shared queues whose counts stay on the device; a level
 * may hold at most 16 rays per primary sample (ft_batch_read and
 * ft_batch_autotune report an overflow).  One pixel kernel writes every
 * item's image; everything is captured once into a CUDA graph.  Work items
 * are tiles of tile_w x tile_h pixels (x AA samples); a warp of the depth
 * march refills its idle lanes when at least `refill` of them are idle.
 * ft_batch_autotune times the candidate tiles (8x8, 16x8, 32x8) and refill
 * thresholds (4, 8, 16) on this batch, one launch each after one warm-up, and
 * keeps the fastest.
 * ------------------------------------------------------------------------- */
typedef struct ft_batch ft_batch;

typedef struct ft_batch_item {
  ft_scene* scene;             /* must outlive the batch */
  ft_render_options options;   /* resolution and march parameters */
  uint32_t aa_samples;
  uint32_t max_depth;          /* 0: depth preview; 1..10: Whitted trace depth */
} ft_batch_item;

typedef struct ft_batch_tuning {
  uint32_t tile_w, tile_h;     /* pixels per work tile (1..64 each) */
  uint32_t refill;             /* 1..32 */
  float ms;                    /* batch time measured by ft_batch_autotune */
} ft_batch_tuning;

#define FT_BATCH_FP16_BRICKS 1u  /* depth items march through their scenes' brick caches */

ft_status ft_batch_create(const ft_batch_item* items, uint32_t n_items, uint32_t flags, ft_batch** out);
ft_status ft_batch_set_tuning(ft_batch* batch, const ft_batch_tuning* tuning);
ft_status ft_batch_autotune(ft_batch* batch, ft_batch_tuning* best);
/* Enqueue the whole batch (one graph launch) on `stream`; returns without
 * waiting.  A launch waits on the GPU for the batch's previous launch (on
 * whatever stream that was), and ft_batch_set_tuning, ft_batch_autotune,
 * ft_batch_read and ft_batch_destroy wait on the host for the last launch
 * before they touch the batch's tables, counters and queues. */
ft_status ft_batch_launch(ft_batch* batch, void* stream);
/* Host copies of one item's outputs after the launch has completed (the call
 * synchronises the device): t_out / mask_out (w*h*aa, depth items only),
 * rgb_out (w*h*3 floats: preview value or averaged radiance), rgb8_out
 * (w*h*3: the gray preview or the Reinhard image).  Each nullable. */
ft_status ft_batch_read(ft_batch* batch, uint32_t item, float* t_out, uint8_t* mask_out, float* rgb_out,
                        uint8_t* rgb8_out);
ft_status ft_batch_samples(const ft_batch* batch, uint64_t* primary_samples);
void ft_batch_destroy(ft_batch* batch);

/* ---------------------------------------------------------------------------
 * Differentiation form: multi-view depth + soft silhouette of a scene whose
 * union_round tree carries the parameters, and the adjoint of that render.
 * No counterpart in the reference (it has no gradients).
 *
 * Forward, per ray of each view (the reference camera, R:6263-6286, one
 * sample per pixel at the pixel centre):
 *   - the plain march (step rule, eps hit, ten bisections, R:4091-4200);
 *   - on a hit, depth t* = the zero of f(o + t d) found by three secant
 *     steps from the bisection bracket (the eps-shell crossing moved onto the
 *     surface, so depth is a smooth function of the parameters), mask 1,
 *     silhouette 1;
 *   - on a miss, m* = the local minimum of f(o + t d) next to the smallest
 *     march sample (bracket continued past either end of the samples while
 *     f falls, then 40 golden-section steps); silhouette =
 *     exp(-max(m*, 0) / tau), depth 0, mask 0.
 * Backward (ft_render_backward) re-marches every ray (no per-step state is
 * stored) and, by implicit differentiation,
 *   d depth / d theta = -(df / d theta) / (grad_p f . d)   at the hit point,
 *   d sil / d theta = -(sil / tau) df / d theta           at the miss minimum,
 * with df / d theta from the primitives' and union_round blends' analytic
 * derivatives; dL / d theta = sum over rays of dL_dt d depth / d theta +
 * dL_dsil d sil / d theta, reduced across pixels in FP64.
 * ------------------------------------------------------------------------- */
typedef struct ft_view {
  float origin[3];
  float target[3];
  float fov_y_degrees;
} ft_view;

typedef enum ft_param_field {
  FT_PARAM_CX = 0,     /* primitive centre */
  FT_PARAM_CY = 1,
  FT_PARAM_CZ = 2,
  FT_PARAM_ROT_Y = 3,  /* rotation about y, degrees */
  FT_PARAM_S0 = 4,     /* sphere radius, box half size x */
  FT_PARAM_S1 = 5,     /* box half size y (inert for spheres) */
  FT_PARAM_S2 = 6,     /* box half size z (inert for spheres) */
  FT_PARAM_RADIUS = 7  /* union_round blend radius of a whole tree (node = any of its union_round nodes) */
} ft_param_field;

typedef struct ft_param {
  int32_t node;   /* ft_node index */
  int32_t field;  /* ft_param_field */
} ft_param;

/* The differentiable parameters of `desc`: for each sphere / box primitive
 * under a union_round tree (in node order) its seven fields, then each tree's
 * radius.  Such primitives must have no x / z rotation, rounding or shell.
 * Writes min(capacity, count) entries and the count. */
ft_status ft_scene_param_layout(const ft_scene_desc* desc, uint32_t capacity, ft_param* params, uint32_t* count);
/* Read / write parameter values in a description (radius writes every
 * union_round node of the tree); rebuild the GPU scene after writing. */
ft_status ft_scene_desc_get_params(const ft_scene_desc* desc, const ft_param* params, uint32_t n, float* values);
ft_status ft_scene_desc_set_params(ft_scene_desc* desc, const ft_param* params, uint32_t n, const float* values);

/* Forward: per view `width*height` samples (options give resolution and
 * march parameters); outputs (each nullable, view-major): t_out floats,
 * mask_out bytes, sil_out floats.  Host pointers unless
 * FT_FLAG_DEVICE_POINTERS. */
ft_status ft_render_views(ft_scene* scene, const ft_view* views, uint32_t n_views,
                          const ft_render_options* options, float tau, float* t_out, uint8_t* mask_out,
                          float* sil_out, uint32_t flags, void* stream);
/* Adjoint: dL_dt and dL_dsil (n_views*width*height floats each, nullable =
 * zero) to dL_dparams (n_params doubles, overwritten). */
ft_status ft_render_backward(ft_scene* scene, const ft_view* views, uint32_t n_views,
                             const ft_render_options* options, float tau, const ft_param* params,
                             uint32_t n_params, const float* dL_dt, const float* dL_dsil, double* dL_dparams,
                             uint32_t flags, void* stream);

/* ---------------------------------------------------------------------------
 * Scene JIT: the role of the reference's Cranelift JIT (J:607-747,
 * J:2931-3016).  The scene's hook programs (domain, distance_post, the
 * environment colour) are lowered to CUDA C++, one straight-line function per
 * program with its registers as locals, and compiled together with the march
 * and trace kernels for sm_103a by NVRTC; the module is loaded with the CUDA
 * runtime's library API.  Afterwards ft_render_depth (plain and FP16-brick)
 * and ft_render_trace of this scene launch the compiled kernels instead of
 * the precompiled ones with the hook interpreter; statistics, batch,
 * no-allocation and adjoint entry points keep the precompiled kernels.
 * Results equal the interpreter's up to FMA contraction differences.
 * Modules are cached per process by source, so scenes with the same hook
 * programs compile once.  Synchronous. */
typedef struct ft_jit_info {
  uint32_t programs;      /* hook programs lowered */
  uint32_t cached;        /* 1 when the module came from the process cache */
  uint64_t source_bytes;  /* generated CUDA source */
  uint64_t cubin_bytes;
  double compile_ms;      /* NVRTC compile (0 when cached) */
  double load_ms;         /* module load and kernel lookup */
} ft_jit_info;

ft_status ft_scene_jit(ft_scene* scene, ft_jit_info* info);

/* Measured FP32 FMA throughput of the current device in TFLOP/s (a short
 * dependent-FMA kernel), used as the roofline denominator of the march. */
ft_status ft_measure_fp32_peak(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* FORGEDTHOUGHTS_GB300_H */
