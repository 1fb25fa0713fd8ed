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

#define FT_ABI_VERSION 1u

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
  FT_ERR_NO_DEVICE = 11
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
  FT_NODE_KIND_COUNT = 30
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

/* Subset of `MaterialParams` (crates/forgedthoughts/src/materials/mod.rs:66-86)
 * read by the Whitted integrator. */
typedef struct ft_material {
  int32_t kind;            /* ft_material_kind */
  int32_t has_medium;
  int32_t thin_walled;
  int32_t color_program;   /* dynamic `fn color(ctx)` hook, -1 if none */
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
} ft_material;

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
} ft_build_info;

ft_status ft_scene_build_info(const ft_scene_desc* desc, ft_build_info* info);

/* Bytes of scene data the last ft_scene_create copied host -> device. */
ft_status ft_scene_device_bytes(const ft_scene* scene, uint64_t* bytes);

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
  uint64_t march_steps;
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
 * call before any stream capture.  The call allocates nothing, enqueues its
 * two kernels on `stream` and returns without waiting: the image is ready
 * when the stream's work completes.  All calls share the scratch array and it
 * keeps the last call's contents, so calls whose work can overlap on the GPU
 * (other streams, other threads) race with each other; serialise them. */
#define FT_NOALLOC_MAX_SAMPLES (1u << 21)
ft_status ft_render_depth_preview_noalloc(ft_scene* scene, const ft_render_options* options,
                                          ft_accel_mode accel, uint32_t aa_samples,
                                          uint8_t* rgb8_out, void* stream);

ft_status ft_render_depth_stats(ft_scene* scene, const ft_render_options* options,
                                ft_accel_mode accel, uint32_t aa_samples,
                                ft_render_stats* stats);

/* The same counters for a Whitted trace (ft_render_trace); output discarded. */
ft_status ft_render_trace_stats(ft_scene* scene, const ft_render_options* options,
                                ft_accel_mode accel, uint32_t aa_samples, uint32_t max_depth,
                                ft_render_stats* stats);

/* Measured FP32 FMA throughput of the current device in TFLOP/s (a short
 * dependent-FMA kernel), used as the roofline denominator of the march. */
ft_status ft_measure_fp32_peak(double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* FORGEDTHOUGHTS_GB300_H */
