// sm_103a sphere-tracing kernels and the C ABI around them.
//
// One thread marches one primary sample (pixel x AA offset).  Threads of a
// warp cover a compact 8x4-pixel tile so their rays stay coherent.  The scene
// distance is the minimum over hard-union leaves found by walking the leaf
// BVH in the reference's order (R:743-786, R = crates/forgedthoughts/src/
// renderer.rs); each leaf is evaluated with a cutoff, the running best, below
// which its value must be exact.  The march itself (raymarch_hit R:4091-4139,
// refine_hit_distance R:4180-4200, estimate_normal R:4202-4215) and the depth
// preview (R:3931-3971, R:5215-5227) follow the reference step for step.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.h"
#include "ft_device.cuh"
#include "jit.h"
#include "scene_build.h"

#include "ft_kernels.cuh"

static_assert(sizeof(DevLeaf) == sizeof(ftgpu::HostLeaf), "leaf layout");
static_assert(sizeof(DevBvhNode) == sizeof(ftgpu::HostBvhNode), "bvh layout");
static_assert(sizeof(DevUrTree) == sizeof(ftgpu::HostUrTree), "urtree layout");
static_assert(sizeof(DevUrBvh) == sizeof(ftgpu::HostUrBvh), "urbvh layout");
static_assert(sizeof(DevUrInner) == sizeof(ftgpu::HostUrInner), "urinner layout");

namespace {

std::string cuda_msg(cudaError_t e, const char* what) {
  return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

#define FT_CUDA_TRY(expr, what)                                                    \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) return ftcommon::fail(FT_ERR_CUDA, cuda_msg(_e, what)); \
  } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Per-scene counter block: kNumCounters statistics words, then the
// persistent depth march's work counter and its self-check flags.
constexpr int kStatWords = 16;
constexpr int kStatWork = 12;
static_assert(kNumCounters <= kStatWork, "statistics overlap the work counter");

}  // namespace

// Scratch of ft_render_depth_preview_noalloc: FT_NOALLOC_MAX_SAMPLES refined
// distances (f32) followed by as many hit-mask bytes.  A file-scope device
// array, so the entry point needs no allocation; every device that loads the
// library holds it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[FT_NOALLOC_MAX_SAMPLES * (sizeof(float) + 1)];

namespace {

constexpr int kMaxNoallocDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_address[kMaxNoallocDevices] = {};

// In host code `g_noalloc_scratch` names a host-side stand-in, not device
// memory: the device address is looked up once per device, with that device
// current, and then passed to the kernels.
ft_status noalloc_scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxNoallocDevices)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "device ordinal out of range for the no-allocation path");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_address[device]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) return ftcommon::fail(FT_ERR_CUDA, cuda_msg(e, "cudaGetSymbolAddress(scratch)"));
    g_noalloc_address[device] = static_cast<unsigned char*>(ptr);
  }
  *out = g_noalloc_address[device];
  return FT_OK;
}

}  // namespace

struct ft_scene {
  int device = 0;
  ftgpu::SceneImage img;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  DevScene dev{};
  // Per-render buffers, grown on demand and reused across calls.
  float* d_t = nullptr;
  uint8_t* d_mask = nullptr;
  uint32_t* d_mat = nullptr;
  float* d_normal = nullptr;  // also the per-sample radiance of traces
  float* d_rgbf = nullptr;
  uint8_t* d_rgb = nullptr;
  size_t cap_items = 0, cap_pixels = 0;
  unsigned long long* d_stats = nullptr;
  int persistent_blocks = 1;
  // FP16 brick cache (ft_scene_build_bricks)
  bool has_bricks = false;
  DevBricks bricks{};
  cudaArray_t brick_array = nullptr;
  uint64_t brick_bytes = 0;
  int persistent_blocks_bricks = 1;
  // Scene JIT (ft_scene_jit): the run-time compiled module and its kernels
  cudaLibrary_t jit_lib = nullptr;
  cudaKernel_t jit_depth[2] = {nullptr, nullptr};  // plain, FP16 bricks
  cudaKernel_t jit_wf[3] = {nullptr, nullptr, nullptr};  // march, shade, shadow
  int jit_blocks[2] = {1, 1};
  // Wavefront trace queues (grown on demand, reused across calls)
  WJob* wf_jobs[2] = {nullptr, nullptr};
  uint64_t wf_jobs_cap[2] = {0, 0};
  WHit* wf_hits = nullptr;
  uint64_t wf_hits_cap = 0;
  WShadow* wf_shadows = nullptr;
  uint64_t wf_shadows_cap = 0;
  float* wf_primary_normal = nullptr;  // per-sample normals of a depth-marched primary level
  uint64_t wf_primary_normal_cap = 0;
  // job counts (2), shadow count, overflow flag, march and shadow work
  // counters, self-check flags (kWfCounters)
  unsigned long long* wf_counters = nullptr;
  uint32_t last_launches = 0;  // kernels launched by the last ft_render_depth / ft_render_trace
  // Per-kernel CUDA-event timing (ft_scene_profile): an event pair around each
  // launch since the last collection, and the sums per kernel kind.
  bool profiling = false;
  std::vector<cudaEvent_t> prof_pool;             // created on demand, reused
  std::vector<std::pair<int, int>> prof_pending;  // (kind, first event of the pair)
  double prof_ms[FT_KERNEL_KINDS] = {};
  uint64_t prof_launches[FT_KERNEL_KINDS] = {};
  std::mutex mu;
};

namespace {

// Record the start event of a launch of `kind` on `st` when the scene is
// profiling; returns the pair's index for prof_end (-1: not profiling).
int prof_begin(ft_scene* sc, cudaStream_t st, int kind) {
  if (!sc->profiling) return -1;
  const size_t first = 2 * sc->prof_pending.size();
  while (sc->prof_pool.size() < first + 2) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return -1;
    }
    sc->prof_pool.push_back(e);
  }
  if (cudaEventRecord(sc->prof_pool[first], st) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  sc->prof_pending.emplace_back(kind, static_cast<int>(first));
  return static_cast<int>(first);
}

void prof_end(ft_scene* sc, cudaStream_t st, int first) {
  if (first >= 0) cudaEventRecord(sc->prof_pool[first + 1], st);
}

// After the stream has completed: add the pending launches' times.
void prof_collect(ft_scene* sc) {
  for (const auto& pk : sc->prof_pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, sc->prof_pool[pk.second], sc->prof_pool[pk.second + 1]) == cudaSuccess) {
      sc->prof_ms[pk.first] += ms;
      sc->prof_launches[pk.first] += 1;
    } else {
      cudaGetLastError();
    }
  }
  sc->prof_pending.clear();
}

ft_status upload_scene(ft_scene* sc) {
  const ftgpu::SceneImage& im = sc->img;
  struct Part {
    const void* src;
    size_t bytes;
    size_t off;
  };
  std::vector<Part> parts = {
      {im.nodes.data(), im.nodes.size() * sizeof(DevNode), 0},
      {im.leaves.data(), im.leaves.size() * sizeof(DevLeaf), 0},
      {im.bvh.data(), im.bvh.size() * sizeof(DevBvhNode), 0},
      {im.gops.data(), im.gops.size() * sizeof(uint32_t), 0},
      {im.urtrees.data(), im.urtrees.size() * sizeof(DevUrTree), 0},
      {im.ur_bvh.data(), im.ur_bvh.size() * sizeof(DevUrBvh), 0},
      {im.ur_bvh_prims.data(), im.ur_bvh_prims.size() * sizeof(int32_t), 0},
      {im.ur_prims.data(), im.ur_prims.size() * sizeof(int32_t), 0},
      {im.ur_inner.data(), im.ur_inner.size() * sizeof(DevUrInner), 0},
      {im.programs.data(), im.programs.size() * sizeof(ft_program), 0},
      {im.instrs.data(), im.instrs.size() * sizeof(ft_instr), 0},
      {im.ur_cell_offsets.data(), im.ur_cell_offsets.size() * sizeof(uint32_t), 0},
      {im.ur_cell_prims.data(), im.ur_cell_prims.size() * sizeof(int32_t), 0},
      {im.materials.data(), im.materials.size() * sizeof(ft_material), 0},
      {im.lights.data(), im.lights.size() * sizeof(ft_light), 0},
      {im.node_op_begin.data(), im.node_op_begin.size() * sizeof(int32_t), 0},
      {im.node_op_end.data(), im.node_op_end.size() * sizeof(int32_t), 0},
      {im.ur_inner_blend.data(), im.ur_inner_blend.size() * sizeof(int32_t), 0},
      {im.ur_cell_gaps.data(), im.ur_cell_gaps.size() * sizeof(float), 0},
      {im.ur_inner_up.data(), im.ur_inner_up.size() * sizeof(int32_t), 0},
      {im.ur_prim_up.data(), im.ur_prim_up.size() * sizeof(int32_t), 0},
      {im.obj_node.data(), im.obj_node.size() * sizeof(int32_t), 0},
      {im.ur_cell_nodes.data(), im.ur_cell_nodes.size() * sizeof(int32_t), 0},
  };
  size_t total = 0;
  for (Part& p : parts) {
    p.off = total;
    total = align_up(total + std::max<size_t>(p.bytes, 16), 256);
  }
  std::vector<unsigned char> staging(total, 0);
  for (const Part& p : parts)
    if (p.bytes) std::memcpy(staging.data() + p.off, p.src, p.bytes);
  FT_CUDA_TRY(cudaMalloc(&sc->arena, total), "cudaMalloc(scene)");
  sc->arena_bytes = total;
  FT_CUDA_TRY(cudaMemcpy(sc->arena, staging.data(), total, cudaMemcpyHostToDevice), "cudaMemcpy(scene)");
  unsigned char* base = static_cast<unsigned char*>(sc->arena);
  DevScene& d = sc->dev;
  d.nodes = reinterpret_cast<const DevNode*>(base + parts[0].off);
  d.leaves = reinterpret_cast<const DevLeaf*>(base + parts[1].off);
  d.bvh = reinterpret_cast<const DevBvhNode*>(base + parts[2].off);
  d.gops = reinterpret_cast<const uint32_t*>(base + parts[3].off);
  d.urtrees = reinterpret_cast<const DevUrTree*>(base + parts[4].off);
  d.ur_bvh = reinterpret_cast<const DevUrBvh*>(base + parts[5].off);
  d.ur_bvh_prims = reinterpret_cast<const int32_t*>(base + parts[6].off);
  d.ur_prims = reinterpret_cast<const int32_t*>(base + parts[7].off);
  d.ur_inner = reinterpret_cast<const DevUrInner*>(base + parts[8].off);
  d.programs = reinterpret_cast<const ft_program*>(base + parts[9].off);
  d.instrs = reinterpret_cast<const ft_instr*>(base + parts[10].off);
  d.ur_cell_offsets = reinterpret_cast<const uint32_t*>(base + parts[11].off);
  d.ur_cell_prims = reinterpret_cast<const int32_t*>(base + parts[12].off);
  d.materials = reinterpret_cast<const ft_material*>(base + parts[13].off);
  d.lights = reinterpret_cast<const ft_light*>(base + parts[14].off);
  d.node_op_begin = reinterpret_cast<const int32_t*>(base + parts[15].off);
  d.node_op_end = reinterpret_cast<const int32_t*>(base + parts[16].off);
  d.ur_inner_blend = reinterpret_cast<const int32_t*>(base + parts[17].off);
  d.ur_cell_gaps = reinterpret_cast<const float*>(base + parts[18].off);
  d.ur_inner_up = reinterpret_cast<const int32_t*>(base + parts[19].off);
  d.ur_prim_up = reinterpret_cast<const int32_t*>(base + parts[20].off);
  d.obj_node = reinterpret_cast<const int32_t*>(base + parts[21].off);
  d.n_obj_node = static_cast<int32_t>(im.obj_node.size());
  d.ur_cell_nodes = reinterpret_cast<const int32_t*>(base + parts[22].off);
  d.n_materials = static_cast<int32_t>(im.materials.size());
  d.n_lights = static_cast<int32_t>(im.lights.size());
  d.env_program = im.environment_program;
  d.bvh_root = im.bvh_root;
  std::memcpy(d.smin, im.scene_min, sizeof(d.smin));
  std::memcpy(d.smax, im.scene_max, sizeof(d.smax));
  // [0, 8): statistics counters; [8]: work-item counter of the persistent march
  FT_CUDA_TRY(cudaMalloc(&sc->d_stats, kStatWords * sizeof(unsigned long long)), "cudaMalloc(stats)");
  int sms = 0, per_sm = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device), "sm count");
  FT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_depth_persistent<false, false, false>, 128, 0),
              "occupancy");
  sc->persistent_blocks = std::max(1, sms * std::max(per_sm, 1));
  FT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_depth_persistent<false, true, false>, 128, 0),
              "occupancy");
  sc->persistent_blocks_bricks = std::max(1, sms * std::max(per_sm, 1));
  return FT_OK;
}

ft_status ensure_buffers(ft_scene* sc, size_t items, size_t pixels) {
  if (items > sc->cap_items) {
    cudaFree(sc->d_t);
    cudaFree(sc->d_mask);
    cudaFree(sc->d_mat);
    cudaFree(sc->d_normal);
    sc->d_t = nullptr;
    sc->d_mask = nullptr;
    sc->d_mat = nullptr;
    sc->d_normal = nullptr;
    sc->cap_items = 0;
    FT_CUDA_TRY(cudaMalloc(&sc->d_t, items * sizeof(float)), "cudaMalloc(depth)");
    FT_CUDA_TRY(cudaMalloc(&sc->d_mask, items), "cudaMalloc(mask)");
    FT_CUDA_TRY(cudaMalloc(&sc->d_mat, items * sizeof(uint32_t)), "cudaMalloc(material)");
    FT_CUDA_TRY(cudaMalloc(&sc->d_normal, items * 3 * sizeof(float)), "cudaMalloc(normal)");
    sc->cap_items = items;
  }
  if (pixels > sc->cap_pixels) {
    cudaFree(sc->d_rgb);
    cudaFree(sc->d_rgbf);
    sc->d_rgb = nullptr;
    sc->d_rgbf = nullptr;
    sc->cap_pixels = 0;
    FT_CUDA_TRY(cudaMalloc(&sc->d_rgb, pixels * 3), "cudaMalloc(rgb)");
    FT_CUDA_TRY(cudaMalloc(&sc->d_rgbf, pixels * 3 * sizeof(float)), "cudaMalloc(rgb linear)");
    sc->cap_pixels = pixels;
  }
  return FT_OK;
}

ft_status check_options(const ft_render_options* o, uint32_t aa) {
  if (!o) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "options must be non-null");
  if (o->width == 0 || o->height == 0) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "width and height must be >= 1");
  if (o->width > 32768 || o->height > 32768)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "width and height must be <= 32768");
  if (aa > 256) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "aa_samples must be <= 256");
  if (!(o->epsilon > 0.0f) || !std::isfinite(o->max_dist))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "epsilon must be > 0 and max_dist finite");
  return FT_OK;
}

void set_tiles(RayParams* P, uint32_t tw, uint32_t th) {
  P->tile_w = tw;
  P->tile_h = th;
  P->tiles_x = (P->width + tw - 1) / tw;
  uint64_t tiles_y = (P->height + th - 1) / th;
  P->n_items = static_cast<uint64_t>(P->tiles_x) * tiles_y * tw * th * P->aa;
}

RayParams make_params(const ft_scene* sc, const ft_render_options& o, uint32_t aa) {
  RayParams P{};
  ftgpu::CameraBasis cb = ftgpu::resolve_camera(sc->img, o);
  std::memcpy(P.origin, cb.origin, sizeof(P.origin));
  std::memcpy(P.fwd, cb.forward, sizeof(P.fwd));
  std::memcpy(P.right, cb.right, sizeof(P.right));
  std::memcpy(P.up, cb.up, sizeof(P.up));
  P.tan_fov = cb.tan_fov;
  P.aspect = static_cast<float>(o.width) / static_cast<float>(o.height);
  P.width = o.width;
  P.height = o.height;
  P.aa = aa;
  P.grid = static_cast<uint32_t>(std::ceil(std::sqrt(static_cast<float>(aa))));
  P.max_steps = o.max_steps;
  P.max_dist = o.max_dist;
  P.eps = o.epsilon;
  P.step_scale = o.step_scale;
  set_tiles(&P, 8, 4);
  P.refill = 8;
  P.jitter = 0;
  P.jitter_seed = 0;
  return P;
}

// FT_FLAG_JITTERED_AA: jittered sub-pixel offsets with the seed in the flags'
// upper half.
void apply_jitter(RayParams* P, uint32_t flags) {
  if (flags & FT_FLAG_JITTERED_AA) {
    P->jitter = 1;
    P->jitter_seed = flags >> FT_JITTER_SEED_SHIFT;
  }
}

ft_status launch_depth(ft_scene* sc, const RayParams& P, cudaStream_t st, bool stats, bool bricks, float* t,
                       uint8_t* mask, uint32_t* mat, float* normal) {
  if (bricks && !sc->has_bricks)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "FT_FLAG_FP16_BRICKS needs ft_scene_build_bricks first");
  uint64_t blocks = (P.n_items + 127) / 128;
  if (blocks > 0x7fffffffull) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "image too large");
  int resident = bricks ? sc->persistent_blocks_bricks : sc->persistent_blocks;
  unsigned grid = static_cast<unsigned>(std::min<uint64_t>(blocks, static_cast<uint64_t>(resident)));
  unsigned long long* counter = sc->d_stats + kStatWork;
  unsigned long long* st_ptr = stats ? sc->d_stats : nullptr;
  if (stats)
    FT_CUDA_TRY(cudaMemsetAsync(sc->d_stats, 0, kStatWords * sizeof(unsigned long long), st), "cudaMemsetAsync(stats)");
  else
    FT_CUDA_TRY(cudaMemsetAsync(counter, 0, 2 * sizeof(unsigned long long), st), "cudaMemsetAsync(counter)");
  const DevBricks& B = sc->bricks;
  if (!stats && sc->jit_depth[bricks ? 1 : 0]) {
    // run-time compiled kernel: same signature as march_depth_persistent
    unsigned jgrid = static_cast<unsigned>(std::min<uint64_t>(blocks, static_cast<uint64_t>(sc->jit_blocks[bricks ? 1 : 0])));
    DevScene S = sc->dev;
    RayParams PP = P;
    DevBricks BB = B;
    BatchView V{};
    unsigned long long* none = nullptr;
    void* args[] = {&S, &PP, &BB, &V, &t, &mask, &mat, &normal, &none, &counter};
    int ev = prof_begin(sc, st, FT_KERNEL_DEPTH_MARCH);
    FT_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(sc->jit_depth[bricks ? 1 : 0]), dim3(jgrid), dim3(128),
                                 args, 0, st),
                "launch of the compiled march kernel");
    prof_end(sc, st, ev);
    return FT_OK;
  }
  int ev = prof_begin(sc, st, FT_KERNEL_DEPTH_MARCH);
  if (stats && bricks)
    march_depth_persistent<true, true, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else if (stats)
    march_depth_persistent<true, false, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else if (bricks)
    march_depth_persistent<false, true, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else
    march_depth_persistent<false, false, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  prof_end(sc, st, ev);
  FT_CUDA_TRY(cudaGetLastError(), "march_depth_persistent launch");
  return FT_OK;
}

void free_bricks(ft_scene* sc) {
  if (sc->bricks.atlas) cudaDestroyTextureObject(sc->bricks.atlas);
  if (sc->brick_array) cudaFreeArray(sc->brick_array);
  sc->bricks = DevBricks{};
  sc->brick_array = nullptr;
  sc->brick_bytes = 0;
  sc->has_bricks = false;
}

// Device buffers freed when the build returns, whatever the outcome.
struct DeviceTemps {
  std::vector<void*> ptrs;
  ~DeviceTemps() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
};

float aabb_volume(const float* mn, const float* mx) {
  float v = 1.0f;
  for (int a = 0; a < 3; ++a) v *= std::max(mx[a] - mn[a], 1.0e-6f);
  return v;
}

// Leaves evaluated exactly at every far-field step instead of being cached:
// the few whose box dwarfs the box of all remaining leaves (a ground slab).
std::vector<int> choose_exact_leaves(const ftgpu::SceneImage& im) {
  const int n = static_cast<int>(im.leaves.size());
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return aabb_volume(im.leaves[a].bmin, im.leaves[a].bmax) > aabb_volume(im.leaves[b].bmin, im.leaves[b].bmax);
  });
  std::vector<int> exact;
  std::vector<char> is_exact(n, 0);
  for (int k = 0; k < n - 1 && static_cast<int>(exact.size()) < kMaxExactLeaves; ++k) {
    int i = order[k];
    float mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
    for (int j = 0; j < n; ++j) {
      if (j == i || is_exact[j]) continue;
      for (int a = 0; a < 3; ++a) {
        mn[a] = std::min(mn[a], im.leaves[j].bmin[a]);
        mx[a] = std::max(mx[a], im.leaves[j].bmax[a]);
      }
    }
    if (aabb_volume(im.leaves[i].bmin, im.leaves[i].bmax) <= 8.0f * aabb_volume(mn, mx)) break;
    exact.push_back(i);
    is_exact[i] = 1;
  }
  return exact;
}


// Device tables of one kernel's share of a batch (depth or trace items).
struct BatchPart {
  std::vector<uint32_t> items;  // indices into ft_batch::items
  DevScene* d_scenes = nullptr;
  RayParams* d_params = nullptr;
  DevBricks* d_bricks = nullptr;
  uint64_t* d_ray_first = nullptr;
  uint64_t* d_out_first = nullptr;
  uint32_t* d_max_depth = nullptr;
  uint64_t n_rays = 0;
  uint64_t n_samples = 0;
  std::vector<uint64_t> out_first;
  int blocks = 1;
  BatchView view() const {
    BatchView v{};
    v.scenes = d_scenes;
    v.params = d_params;
    v.bricks = d_bricks;
    v.ray_first = d_ray_first;
    v.out_first = d_out_first;
    v.n_items = static_cast<uint32_t>(items.size());
    v.n_rays = n_rays;
    return v;
  }
};

}  // namespace

struct ft_batch {
  int device = 0;
  bool bricks = false;
  std::vector<ft_batch_item> items;
  BatchPart part[2];  // 0: depth previews, 1: traces
  std::vector<BatchPixItem> pix;
  BatchPixItem* d_pix = nullptr;
  uint64_t n_pixels = 0;
  float* d_t = nullptr;
  uint8_t* d_mask = nullptr;
  float* d_srgb = nullptr;
  float* d_rgbf = nullptr;
  uint8_t* d_rgb8 = nullptr;
  unsigned long long* d_counters = nullptr;
  cudaStream_t stream = nullptr;
  // Recorded after every ft_batch_launch on the caller's stream: the calls
  // that rewrite the tables, counters and queues of a launch wait on it, so
  // they never touch them under a launch still running on another stream.
  cudaEvent_t done = nullptr;
  cudaGraphExec_t exec = nullptr;
  ft_batch_tuning tuning{8, 8, 8, 0.0f};
  std::mutex mu;
  // Wavefront queues of the trace items (sized per tuning: tiles pad the
  // work items), their counters (job counts x2, shadow count, overflow
  // flag), the bounce levels captured and the most light samples of a scene.
  WJob* wf_jobs[2] = {nullptr, nullptr};
  uint64_t wf_jobs_cap[2] = {0, 0};
  WHit* wf_hits = nullptr;
  uint64_t wf_hits_cap = 0;
  WShadow* wf_shadows = nullptr;
  uint64_t wf_shadows_cap = 0;
  unsigned long long* wf_counters = nullptr;
  uint32_t wf_levels = 0;
  uint32_t wf_light_samples = 1;
  uint64_t wf_max_push = 4;  // most rays a hit of any trace item pushes
  int sms = 1;
};

namespace {

void free_part(BatchPart& p) {
  cudaFree(p.d_scenes);
  cudaFree(p.d_params);
  cudaFree(p.d_bricks);
  cudaFree(p.d_ray_first);
  cudaFree(p.d_out_first);
  cudaFree(p.d_max_depth);
  p = BatchPart{};
}

template <class T>
ft_status grow(T** buf, uint64_t* cap, uint64_t want, const char* what) {
  if (want <= *cap) return FT_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  uint64_t n = want + want / 4 + 1024;
  FT_CUDA_TRY(cudaMalloc(buf, n * sizeof(T)), what);
  *cap = n;
  return FT_OK;
}

// Most secondary rays one hit can push: two materials (a smooth boolean's
// split) x (reflection + refraction), or x (3 + 4) lobe rays when a
// transmissive material may be rough (roughness above 0.06, or set per hit by
// a hook; blends mix the roughness of any two materials).
uint64_t max_rays_per_hit(const ftgpu::SceneImage& im) {
  bool transmissive = false, rough = false;
  for (const ft_material& m : im.materials) {
    transmissive |= m.kind == FT_MAT_DIELECTRIC || (m.kind == FT_MAT_STANDARD && m.transmission > 1.0e-4f);
    rough |= m.roughness > 0.06f || m.roughness_program >= 0;
  }
  return transmissive && rough ? 2 * (3 + 4) : 2 * 2;
}

// Queue capacity of bounce level k of a batch wavefront over n work items: a
// job pushes at most `push` rays (max_rays_per_hit), so n * push^k is exact;
// it is capped at 16 n (Whitted queues shrink fast: diffuse hits push
// nothing) and an overflow is reported when the results are read.
uint64_t level_capacity(uint64_t n, uint32_t k, uint64_t push) {
  uint64_t f = 1;
  for (uint32_t i = 0; i < k && f < 16; ++i) f *= push;
  return n * std::min<uint64_t>(f, 16);
}

// Per-item parameters and work prefix sums for the current tuning; uploads
// them and (re)captures the batch graph.
ft_status batch_apply_tuning(ft_batch* b) {
  for (int k = 0; k < 2; ++k) {
    BatchPart& part = b->part[k];
    if (part.items.empty()) continue;
    std::vector<RayParams> params;
    std::vector<uint64_t> ray_first(1, 0);
    for (uint32_t it : part.items) {
      const ft_batch_item& bi = b->items[it];
      RayParams P = make_params(bi.scene, bi.options, std::max(bi.aa_samples, 1u));
      set_tiles(&P, b->tuning.tile_w, b->tuning.tile_h);
      P.refill = b->tuning.refill;
      params.push_back(P);
      ray_first.push_back(ray_first.back() + P.n_items);
    }
    part.n_rays = ray_first.back();
    FT_CUDA_TRY(cudaMemcpy(part.d_params, params.data(), params.size() * sizeof(RayParams), cudaMemcpyHostToDevice),
                "upload batch parameters");
    FT_CUDA_TRY(cudaMemcpy(part.d_ray_first, ray_first.data(), ray_first.size() * sizeof(uint64_t),
                           cudaMemcpyHostToDevice),
                "upload batch work offsets");
  }
  if (!b->part[1].items.empty()) {
    const uint64_t n = b->part[1].n_rays;
    uint64_t want[2] = {0, 0}, hits = 0;
    for (uint32_t k = 0; k < b->wf_levels; ++k) {
      uint64_t c = level_capacity(n, k, b->wf_max_push);
      want[k & 1] = std::max(want[k & 1], c);
      hits = std::max(hits, c);
    }
    for (int q = 0; q < 2; ++q)
      if (ft_status s = grow(&b->wf_jobs[q], &b->wf_jobs_cap[q], std::max<uint64_t>(want[q], 1), "cudaMalloc(batch ray jobs)"))
        return s;
    if (ft_status s = grow(&b->wf_hits, &b->wf_hits_cap, hits, "cudaMalloc(batch hits)")) return s;
    if (ft_status s = grow(&b->wf_shadows, &b->wf_shadows_cap, 2 * hits * b->wf_light_samples,
                           "cudaMalloc(batch shadow jobs)"))
      return s;
  }
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  FT_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin batch capture");
  cudaMemsetAsync(b->d_counters, 0, 2 * sizeof(unsigned long long), b->stream);
  const BatchPart& D = b->part[0];
  const BatchPart& T = b->part[1];
  if (!D.items.empty()) {
    if (b->bricks)
      march_depth_persistent<false, true, true><<<D.blocks, 128, 0, b->stream>>>(
          DevScene{}, RayParams{}, DevBricks{}, D.view(), b->d_t, b->d_mask, nullptr, nullptr, nullptr, b->d_counters);
    else
      march_depth_persistent<false, false, true><<<D.blocks, 128, 0, b->stream>>>(
          DevScene{}, RayParams{}, DevBricks{}, D.view(), b->d_t, b->d_mask, nullptr, nullptr, nullptr, b->d_counters);
  }
  if (!T.items.empty()) {
    // the Whitted items as a wavefront: one march, shade and shadow kernel
    // per bounce level over every item's queue (counts stay on the device)
    unsigned long long* c = b->wf_counters;
    const BatchView V = T.view();
    cudaMemsetAsync(b->d_srgb, 0, T.n_samples * 3 * sizeof(float), b->stream);
    cudaMemsetAsync(c, 0, kWfCounters * sizeof(unsigned long long), b->stream);
    const unsigned grid = static_cast<unsigned>(T.blocks);
    const unsigned mgrid = static_cast<unsigned>(b->sms * 6), sgrid = static_cast<unsigned>(b->sms * 8);
    wf_primary_batch_kernel<<<grid, 128, 0, b->stream>>>(V, b->wf_jobs[0], c);
    for (uint32_t level = 0; level < b->wf_levels; ++level) {
      const int cur = static_cast<int>(level & 1), nxt = 1 - cur;
      cudaMemsetAsync(c + nxt, 0, sizeof(unsigned long long), b->stream);
      cudaMemsetAsync(c + 2, 0, sizeof(unsigned long long), b->stream);
      cudaMemsetAsync(c + 4, 0, 2 * sizeof(unsigned long long), b->stream);
      wf_march_persistent<true, false><<<mgrid, 128, 0, b->stream>>>(DevScene{}, RayParams{}, V, b->wf_jobs[cur],
                                                                     c + cur, b->wf_jobs_cap[cur], b->wf_hits,
                                                                     b->d_srgb, c + 4, c + 6, nullptr);
      WQueues Q{b->d_srgb, b->wf_jobs[nxt], c + nxt, b->wf_jobs_cap[nxt], b->wf_shadows, c + 2,
                b->wf_shadows_cap, reinterpret_cast<unsigned int*>(c + 3), 0};
      wf_shade_batch_kernel<<<grid, 128, 0, b->stream>>>(V, T.d_max_depth, b->wf_jobs[cur], c + cur,
                                                         b->wf_jobs_cap[cur], b->wf_hits, Q);
      wf_shadow_persistent<true, false><<<sgrid, 128, 0, b->stream>>>(DevScene{}, RayParams{}, V, b->wf_shadows,
                                                                      c + 2, b->wf_shadows_cap, b->d_srgb, c + 5,
                                                                      c + 6, nullptr);
    }
  }
  {
    uint64_t want = (b->n_pixels + 255) / 256;
    unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(want, 152ull * 64)));
    batch_pixels_kernel<<<grid, 256, 0, b->stream>>>(b->d_pix, static_cast<uint32_t>(b->pix.size()), b->n_pixels,
                                                    b->d_t, b->d_mask, b->d_srgb, b->d_rgbf, b->d_rgb8);
  }
  cudaError_t le = cudaGetLastError();
  cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
  FT_CUDA_TRY(le, "batch kernel launch");
  FT_CUDA_TRY(ce, "end batch capture");
  cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  FT_CUDA_TRY(ie, "instantiate batch graph");
  return FT_OK;
}

// The persistent march's self-check slot (next to its work counter): bits of
// the phases in which a ray exceeded its iteration limit, bit 8 when a warp
// exceeded its time limit.
ft_status march_check(unsigned long long flags) {
  if (!flags) return FT_OK;
  return ftcommon::fail(FT_ERR_TIMEOUT, "march gave up (self-check flags 0x" + [&] {
    char buf[32];
    std::snprintf(buf, sizeof(buf), "%llx", flags);
    return std::string(buf);
  }() + "): a ray exceeded max_steps + 64 iterations or a warp ran for over 20 s");
}

// After the batch's work has completed: fail if a Whitted queue overflowed or
// the depth march gave up.
ft_status batch_overflow(ft_batch* b) {
  unsigned long long march = 0;
  FT_CUDA_TRY(cudaMemcpy(&march, b->d_counters + 1, sizeof(march), cudaMemcpyDeviceToHost), "batch march flags");
  if (ft_status s = march_check(march)) return s;
  if (!b->wf_counters) return FT_OK;
  unsigned long long flag = 0, wf_march = 0;
  FT_CUDA_TRY(cudaMemcpy(&wf_march, b->wf_counters + 6, sizeof(wf_march), cudaMemcpyDeviceToHost), "batch queue flags");
  if (ft_status s = march_check(wf_march)) return s;
  FT_CUDA_TRY(cudaMemcpy(&flag, b->wf_counters + 3, sizeof(flag), cudaMemcpyDeviceToHost), "batch queue flags");
  if (flag) return ftcommon::fail(FT_ERR_CUDA, "batch Whitted queue overflow (more than 16 rays per primary sample "
                                               "at one bounce level)");
  return FT_OK;
}

ft_status check_tuning(const ft_batch_tuning& t) {
  if (t.tile_w < 1 || t.tile_w > 64 || t.tile_h < 1 || t.tile_h > 64 || t.refill < 1 || t.refill > 32)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "tile sides must be 1..64 and refill 1..32");
  return FT_OK;
}



// Whitted trace of one frame as a wavefront: per bounce level one march, one
// shade and one shadow kernel over queues (ft_wavefront.cuh).  Radiance per
// sample lands in sc->d_normal.  Queue sizes are read back once per level to
// size the next one; the capacities are exact upper bounds (a job pushes at
// most max_rays_per_hit rays, and two materials x the light samples).
// With primary_bricks the level-0 hits come from the FP16 brick depth march of
// the primary samples (launch_depth, then wf_hits_from_depth_kernel) instead
// of the wavefront march; every later level is unchanged.
ft_status trace_wavefront(ft_scene* sc, const RayParams& P, uint32_t max_depth, cudaStream_t st,
                          uint32_t* launches, unsigned long long* const* kind_stats = nullptr,
                          bool primary_bricks = false) {
  const ftgpu::SceneImage& im = sc->img;
  uint64_t light_samples = 0;
  const uint64_t max_push = max_rays_per_hit(im);
  for (const ft_light& L : im.lights) light_samples += L.kind == FT_LIGHT_SPHERE ? std::max(L.samples, 1u) : 1u;
  uint64_t n = P.n_items;  // work items, tile padding included
  if (!sc->wf_counters)
    FT_CUDA_TRY(cudaMalloc(&sc->wf_counters, kWfCounters * sizeof(unsigned long long)), "cudaMalloc(queues)");
  if (ft_status s = grow(&sc->wf_jobs[0], &sc->wf_jobs_cap[0], n, "cudaMalloc(ray jobs)")) return s;
  unsigned long long* c = sc->wf_counters;
  float* radiance = sc->d_normal;
  const size_t samples = static_cast<size_t>(P.width) * P.height * P.aa;
  FT_CUDA_TRY(cudaMemsetAsync(radiance, 0, samples * 3 * sizeof(float), st), "cudaMemsetAsync(radiance)");
  FT_CUDA_TRY(cudaMemsetAsync(c, 0, kWfCounters * sizeof(unsigned long long), st), "cudaMemsetAsync(queues)");
  unsigned long long first = n;
  FT_CUDA_TRY(cudaMemcpyAsync(c, &first, sizeof(first), cudaMemcpyHostToDevice, st), "queue count");
  int ev = prof_begin(sc, st, FT_KERNEL_PRIMARY);
  wf_primary_kernel<<<static_cast<unsigned>((n + 127) / 128), 128, 0, st>>>(P, sc->wf_jobs[0]);
  prof_end(sc, st, ev);
  FT_CUDA_TRY(cudaGetLastError(), "wf_primary_kernel launch");
  *launches = 1;
  int sms = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device), "sm count");
  // statistics runs take the precompiled counting variants; the run-time
  // compiled kernels, when present, serve every other trace
  const bool stats = kind_stats != nullptr;
  const void* k_march = stats ? reinterpret_cast<const void*>(wf_march_persistent<false, true>)
                        : sc->jit_wf[0] ? reinterpret_cast<const void*>(sc->jit_wf[0])
                                        : reinterpret_cast<const void*>(wf_march_persistent<false, false>);
  const void* k_shade = stats ? reinterpret_cast<const void*>(wf_shade_kernel<true>)
                        : sc->jit_wf[1] ? reinterpret_cast<const void*>(sc->jit_wf[1])
                                        : reinterpret_cast<const void*>(wf_shade_kernel<false>);
  const void* k_shadow = stats ? reinterpret_cast<const void*>(wf_shadow_persistent<false, true>)
                         : sc->jit_wf[2] ? reinterpret_cast<const void*>(sc->jit_wf[2])
                                         : reinterpret_cast<const void*>(wf_shadow_persistent<false, false>);
  unsigned long long* st_march = stats ? kind_stats[0] : nullptr;
  unsigned long long* st_shade = stats ? kind_stats[1] : nullptr;
  unsigned long long* st_shadow = stats ? kind_stats[2] : nullptr;
  DevScene S = sc->dev;
  RayParams PP = P;
  BatchView none{};
  unsigned long long* march_next = c + 4;
  unsigned long long* shadow_next = c + 5;
  unsigned long long* flags = c + 6;
  int cur = 0;
  for (uint32_t level = 0; level < max_depth && n > 0; ++level) {
    const int nxt = 1 - cur;
    if (ft_status s = grow(&sc->wf_hits, &sc->wf_hits_cap, n, "cudaMalloc(hits)")) return s;
    if (ft_status s = grow(&sc->wf_jobs[nxt], &sc->wf_jobs_cap[nxt], max_push * n, "cudaMalloc(ray jobs)")) return s;
    if (ft_status s = grow(&sc->wf_shadows, &sc->wf_shadows_cap, std::max<uint64_t>(2 * n * light_samples, 1),
                           "cudaMalloc(shadow jobs)"))
      return s;
    FT_CUDA_TRY(cudaMemsetAsync(c + nxt, 0, sizeof(unsigned long long), st), "cudaMemsetAsync(queues)");
    FT_CUDA_TRY(cudaMemsetAsync(c + 2, 0, sizeof(unsigned long long), st), "cudaMemsetAsync(queues)");
    unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + 127) / 128,
                                                                                  static_cast<uint64_t>(sms) * 16)));
    const WJob* jobs = sc->wf_jobs[cur];
    const unsigned long long* count = c + cur;
    WHit* hits = sc->wf_hits;
    unsigned long long jcap = sc->wf_jobs_cap[cur];
    FT_CUDA_TRY(cudaMemsetAsync(march_next, 0, sizeof(unsigned long long), st), "cudaMemsetAsync(queues)");
    unsigned mgrid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((n + 127) / 128,
                                                                                   static_cast<uint64_t>(sms) * 5)));
    if (level == 0 && primary_bricks) {
      const uint64_t samples3 = 3 * static_cast<uint64_t>(samples);
      if (ft_status s = grow(&sc->wf_primary_normal, &sc->wf_primary_normal_cap, samples3, "cudaMalloc(normals)"))
        return s;
      if (ft_status s = launch_depth(sc, P, st, false, true, sc->d_t, sc->d_mask, nullptr, sc->wf_primary_normal))
        return s;
      ev = prof_begin(sc, st, FT_KERNEL_MARCH);
      wf_hits_from_depth_kernel<<<grid, 128, 0, st>>>(S, PP, jobs, n, sc->d_t, sc->d_mask, sc->wf_primary_normal,
                                                       hits, radiance);
      prof_end(sc, st, ev);
      FT_CUDA_TRY(cudaGetLastError(), "wf_hits_from_depth_kernel launch");
      *launches += 1;
    } else {
      void* margs[] = {&S, &PP, &none, &jobs, &count, &jcap, &hits, &radiance, &march_next, &flags, &st_march};
      ev = prof_begin(sc, st, FT_KERNEL_MARCH);
      FT_CUDA_TRY(cudaLaunchKernel(k_march, dim3(mgrid), dim3(128), margs, 0, st), "wavefront march launch");
      prof_end(sc, st, ev);
    }
    WQueues Q{radiance, sc->wf_jobs[nxt], c + nxt, sc->wf_jobs_cap[nxt], sc->wf_shadows, c + 2,
              sc->wf_shadows_cap, reinterpret_cast<unsigned int*>(c + 3), max_depth};
    const WHit* chits = hits;
    void* sargs[] = {&S, &PP, &jobs, &count, &jcap, &chits, &Q, &st_shade};
    ev = prof_begin(sc, st, FT_KERNEL_SHADE);
    FT_CUDA_TRY(cudaLaunchKernel(k_shade, dim3(grid), dim3(128), sargs, 0, st), "wavefront shade launch");
    prof_end(sc, st, ev);
    *launches += 2;
    unsigned long long h[2] = {0, 0};
    FT_CUDA_TRY(cudaMemcpyAsync(&h[0], c + nxt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "queue count");
    FT_CUDA_TRY(cudaMemcpyAsync(&h[1], c + 2, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "queue count");
    FT_CUDA_TRY(cudaStreamSynchronize(st), "wavefront level");
    if (h[1] > 0) {
      unsigned sgrid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>((h[1] + 127) / 128,
                                                                                     static_cast<uint64_t>(sms) * 8)));
      const WShadow* shadows = sc->wf_shadows;
      const unsigned long long* scount = c + 2;
      unsigned long long scap = sc->wf_shadows_cap;
      FT_CUDA_TRY(cudaMemsetAsync(shadow_next, 0, sizeof(unsigned long long), st), "cudaMemsetAsync(queues)");
      void* hargs[] = {&S, &PP, &none, &shadows, &scount, &scap, &radiance, &shadow_next, &flags, &st_shadow};
      ev = prof_begin(sc, st, FT_KERNEL_SHADOW);
      FT_CUDA_TRY(cudaLaunchKernel(k_shadow, dim3(sgrid), dim3(128), hargs, 0, st), "wavefront shadow launch");
      prof_end(sc, st, ev);
      *launches += 1;
    }
    n = std::min<uint64_t>(h[0], sc->wf_jobs_cap[nxt]);  // an overflowed queue holds its capacity
    cur = nxt;
  }
  unsigned long long tail[4] = {0, 0, 0, 0};  // overflow flag, work counters, self-check flags
  FT_CUDA_TRY(cudaMemcpyAsync(tail, c + 3, sizeof(tail), cudaMemcpyDeviceToHost, st), "queue flags");
  FT_CUDA_TRY(cudaStreamSynchronize(st), "wavefront");
  if (tail[0]) return ftcommon::fail(FT_ERR_CUDA, "wavefront queue overflow");
  if (ft_status s = march_check(tail[3])) return s;
  if (primary_bricks) {
    unsigned long long depth_flags = 0;
    FT_CUDA_TRY(cudaMemcpyAsync(&depth_flags, sc->d_stats + kStatWork + 1, sizeof(depth_flags), cudaMemcpyDeviceToHost,
                                st),
                "march flags");
    FT_CUDA_TRY(cudaStreamSynchronize(st), "march flags");
    if (ft_status s = march_check(depth_flags)) return s;
  }
  return FT_OK;
}

}  // namespace

extern "C" {

ft_status ft_scene_create(const ft_scene_desc* desc, ft_scene** out) {
  FT_API_BEGIN
  if (!desc || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "desc and out must be non-null");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return ftcommon::fail(FT_ERR_NO_DEVICE, e != cudaSuccess ? cuda_msg(e, "cudaGetDeviceCount") : "no CUDA device");
  auto* sc = new (std::nothrow) ft_scene();
  if (!sc) return ftcommon::fail(FT_ERR_OUT_OF_MEMORY, "out of host memory");
  std::string err;
  bool built = false;
  try {
    built = ftgpu::build_scene_image(*desc, &sc->img, &err);
  } catch (...) {
    delete sc;
    throw;
  }
  if (!built) {
    delete sc;
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, err);
  }
  e = cudaGetDevice(&sc->device);
  if (e != cudaSuccess) {
    delete sc;
    return ftcommon::fail(FT_ERR_CUDA, cuda_msg(e, "cudaGetDevice"));
  }
  ft_status s = FT_OK;
  try {
    s = upload_scene(sc);
  } catch (...) {
    ft_scene_destroy(sc);
    throw;
  }
  if (s != FT_OK) {
    ft_scene_destroy(sc);
    return s;
  }
  *out = sc;
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_build_info(const ft_scene_desc* desc, ft_build_info* info) {
  FT_API_BEGIN
  if (!desc || !info) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "desc and info must be non-null");
  ftgpu::SceneImage img;
  std::string err;
  auto t0 = std::chrono::steady_clock::now();
  if (!ftgpu::build_scene_image(*desc, &img, &err)) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, err);
  auto t1 = std::chrono::steady_clock::now();
  std::memset(info, 0, sizeof(*info));
  info->leaves = static_cast<uint32_t>(img.leaves.size());
  for (const auto& l : img.leaves) {
    info->primitive_leaves += l.kind == ftgpu::kLeafPrim;
    info->generic_leaves += l.kind == ftgpu::kLeafGeneric;
    info->union_round_leaves += l.kind == ftgpu::kLeafUrTree;
  }
  info->bvh_nodes = static_cast<uint32_t>(img.bvh.size());
  if (!img.ur_cell_offsets.empty()) {
    for (const auto& t : img.urtrees) {
      if (t.dims[0] <= 0) continue;
      uint64_t cells = static_cast<uint64_t>(t.dims[0]) * t.dims[1] * t.dims[2];
      info->grid_cells += cells;
      for (uint64_t c = 0; c < cells; ++c) {
        uint32_t len = img.ur_cell_offsets[t.cell_first + c + 1] - img.ur_cell_offsets[t.cell_first + c];
        info->grid_entries += len;
        info->grid_max_list = std::max(info->grid_max_list, len);
      }
      if (t.odims[0] <= 0) continue;
      uint64_t ocells = static_cast<uint64_t>(t.odims[0]) * t.odims[1] * t.odims[2];
      info->outer_grid_cells += ocells;
      info->outer_grid_entries += img.ur_cell_offsets[t.ocell_first + ocells] - img.ur_cell_offsets[t.ocell_first];
    }
  }
  info->generic_ops = static_cast<uint32_t>(img.gops.size());
  info->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_last_launches(const ft_scene* sc, uint32_t* launches) {
  if (!sc || !launches) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and launches must be non-null");
  *launches = sc->last_launches;
  return FT_OK;
}

ft_status ft_scene_device_bytes(const ft_scene* sc, uint64_t* bytes) {
  if (!sc || !bytes) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and bytes must be non-null");
  *bytes = sc->arena_bytes + sc->brick_bytes;
  return FT_OK;
}

void ft_scene_destroy(ft_scene* sc) {
  if (!sc) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(sc->device);
  cudaFree(sc->arena);
  cudaFree(sc->d_t);
  cudaFree(sc->d_mask);
  cudaFree(sc->d_mat);
  cudaFree(sc->d_normal);
  cudaFree(sc->d_rgbf);
  cudaFree(sc->d_rgb);
  cudaFree(sc->d_stats);
  free_bricks(sc);
  if (sc->jit_lib) cudaLibraryUnload(sc->jit_lib);
  cudaFree(sc->wf_jobs[0]);
  cudaFree(sc->wf_jobs[1]);
  cudaFree(sc->wf_hits);
  cudaFree(sc->wf_shadows);
  cudaFree(sc->wf_primary_normal);
  cudaFree(sc->wf_counters);
  for (cudaEvent_t e : sc->prof_pool) cudaEventDestroy(e);
  cudaSetDevice(prev);
  delete sc;
}

ft_status ft_render_depth(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel, uint32_t aa_samples,
                          float* t_out, uint8_t* mask_out, uint32_t* material_out, float* normal_out,
                          uint8_t* rgb8_out, uint32_t flags, void* stream) {
  FT_API_BEGIN
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  size_t pixels = static_cast<size_t>(options->width) * options->height;
  size_t items = pixels * aa;
  if (ft_status s = ensure_buffers(sc, items, pixels)) return s;
  RayParams P = make_params(sc, *options, aa);
  apply_jitter(&P, flags);
  float* t = dev_ptrs && t_out ? t_out : sc->d_t;
  uint8_t* mask = dev_ptrs && mask_out ? mask_out : sc->d_mask;
  uint32_t* mat = material_out ? (dev_ptrs ? material_out : sc->d_mat) : nullptr;
  float* nrm = normal_out ? (dev_ptrs ? normal_out : sc->d_normal) : nullptr;
  const bool bricks = (flags & FT_FLAG_FP16_BRICKS) != 0;
  if (ft_status s = launch_depth(sc, P, st, false, bricks, t, mask, mat, nrm)) return s;
  sc->last_launches = rgb8_out ? 2 : 1;
  if (rgb8_out) {
    uint8_t* rgb = dev_ptrs ? rgb8_out : sc->d_rgb;
    uint32_t np = static_cast<uint32_t>(pixels);
    int ev = prof_begin(sc, st, FT_KERNEL_PIXELS);
    depth_rgb8_kernel<<<(np + 255) / 256, 256, 0, st>>>(t, mask, np, aa, options->max_dist, rgb);
    prof_end(sc, st, ev);
    FT_CUDA_TRY(cudaGetLastError(), "depth_rgb8_kernel launch");
    if (!dev_ptrs)
      FT_CUDA_TRY(cudaMemcpyAsync(rgb8_out, rgb, pixels * 3, cudaMemcpyDeviceToHost, st), "copy rgb8");
  }
  if (!dev_ptrs) {
    if (t_out) FT_CUDA_TRY(cudaMemcpyAsync(t_out, t, items * sizeof(float), cudaMemcpyDeviceToHost, st), "copy depth");
    if (mask_out) FT_CUDA_TRY(cudaMemcpyAsync(mask_out, mask, items, cudaMemcpyDeviceToHost, st), "copy mask");
    if (material_out)
      FT_CUDA_TRY(cudaMemcpyAsync(material_out, mat, items * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                  "copy material");
    if (normal_out)
      FT_CUDA_TRY(cudaMemcpyAsync(normal_out, nrm, items * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                  "copy normal");
  }
  unsigned long long march_flags = 0;
  FT_CUDA_TRY(cudaMemcpyAsync(&march_flags, sc->d_stats + kStatWork + 1, sizeof(march_flags), cudaMemcpyDeviceToHost, st),
              "march flags");
  FT_CUDA_TRY(cudaStreamSynchronize(st), "render");
  prof_collect(sc);
  if (ft_status s = march_check(march_flags)) return s;
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_render_depth_preview_noalloc(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                          uint32_t aa_samples, uint8_t* rgb8_out, void* stream) {
  FT_API_BEGIN
  if (!sc || !rgb8_out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and rgb8_out must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  uint64_t pixels = static_cast<uint64_t>(options->width) * options->height;
  uint64_t items = pixels * aa;
  if (items > FT_NOALLOC_MAX_SAMPLES)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT,
                          "width*height*aa = " + std::to_string(items) + " samples exceeds the no-allocation scratch "
                          "limit of " + std::to_string(FT_NOALLOC_MAX_SAMPLES) + " samples");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  unsigned char* scratch = nullptr;
  if (ft_status s = noalloc_scratch_address(sc->device, &scratch)) return s;
  float* t = reinterpret_cast<float*>(scratch);
  uint8_t* mask = scratch + sizeof(float) * FT_NOALLOC_MAX_SAMPLES;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  RayParams P = make_params(sc, *options, aa);
  uint64_t blocks = (P.n_items + 127) / 128;
  march_depth_kernel<false><<<static_cast<unsigned>(blocks), 128, 0, st>>>(sc->dev, P, t, mask, nullptr, nullptr,
                                                                           nullptr);
  FT_CUDA_TRY(cudaGetLastError(), "march_depth_kernel launch");
  uint32_t np = static_cast<uint32_t>(pixels);
  depth_rgb8_kernel<<<(np + 255) / 256, 256, 0, st>>>(t, mask, np, aa, options->max_dist, rgb8_out);
  FT_CUDA_TRY(cudaGetLastError(), "depth_rgb8_kernel launch");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_render_pathtrace(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                              const ft_pathtrace_settings* settings, float* rgb_out, uint8_t* rgb8_out,
                              uint32_t* samples_out, uint32_t flags, void* stream) {
  FT_API_BEGIN
  if (!sc || !settings) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and settings must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  if (ft_status s = check_options(options, 1)) return s;
  if (settings->spp > 65536 || settings->max_bounces > 64 || !(settings->noise_threshold >= 0.0f))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "spp must be <= 65536, max_bounces <= 64, noise_threshold >= 0");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  const size_t pixels = static_cast<size_t>(options->width) * options->height;
  if (ft_status s = ensure_buffers(sc, pixels, pixels)) return s;
  RayParams P = make_params(sc, *options, 1);
  PathSettingsD ps;
  // PathtraceSettings' clamps (R:3986-3990)
  ps.spp = std::max(settings->spp, 1u);
  ps.max_bounces = std::max(settings->max_bounces, 1u);
  ps.min_spp = std::min(std::max(settings->min_spp, 1u), ps.spp);
  ps.noise_threshold = std::max(settings->noise_threshold, 0.0f);
  float* rgbf = rgb_out ? (dev_ptrs ? rgb_out : sc->d_rgbf) : nullptr;
  uint8_t* rgb8 = rgb8_out ? (dev_ptrs ? rgb8_out : sc->d_rgb) : nullptr;
  uint32_t* cnt = samples_out ? (dev_ptrs ? samples_out : sc->d_mat) : nullptr;
  const unsigned blocks = static_cast<unsigned>((pixels + 127) / 128);
  path_pixel_kernel<false><<<blocks, 128, 0, st>>>(sc->dev, P, ps, rgbf, rgb8, cnt, nullptr);
  FT_CUDA_TRY(cudaGetLastError(), "path_pixel_kernel launch");
  sc->last_launches = 1;
  if (!dev_ptrs) {
    if (rgb_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb_out, rgbf, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                             "copy rgb");
    if (rgb8_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb8_out, rgb8, pixels * 3, cudaMemcpyDeviceToHost, st), "copy rgb8");
    if (samples_out)
      FT_CUDA_TRY(cudaMemcpyAsync(samples_out, cnt, pixels * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                  "copy samples");
  }
  FT_CUDA_TRY(cudaStreamSynchronize(st), "path trace");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_render_trace(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel, uint32_t aa_samples,
                          uint32_t max_depth, float* rgb_out, uint8_t* rgb8_out, uint32_t flags, void* stream) {
  FT_API_BEGIN
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  uint32_t depth = std::max(max_depth, 1u);  // RaySettings::max_depth.max(1)
  if (depth > 10) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "max_depth must be <= 10");
  std::lock_guard<std::mutex> lock(sc->mu);
  const bool primary_bricks = (flags & FT_FLAG_FP16_BRICKS) != 0;
  if (primary_bricks && !sc->has_bricks)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "FT_FLAG_FP16_BRICKS needs ft_scene_build_bricks first");
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  size_t pixels = static_cast<size_t>(options->width) * options->height;
  size_t items = pixels * aa;
  if (ft_status s = ensure_buffers(sc, items, pixels)) return s;
  RayParams P = make_params(sc, *options, aa);
  apply_jitter(&P, flags);
  uint64_t blocks = (P.n_items + 127) / 128;
  if (blocks > 0x7fffffffull) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "image too large");
  uint32_t launches = 0;
  if (ft_status s = trace_wavefront(sc, P, depth, st, &launches, nullptr, primary_bricks))
    return s;
  float* rgbf = rgb_out ? (dev_ptrs ? rgb_out : sc->d_rgbf) : nullptr;
  uint8_t* rgb8 = rgb8_out ? (dev_ptrs ? rgb8_out : sc->d_rgb) : nullptr;
  uint32_t np = static_cast<uint32_t>(pixels);
  int ev = prof_begin(sc, st, FT_KERNEL_PIXELS);
  trace_pixels_kernel<<<(np + 255) / 256, 256, 0, st>>>(sc->d_normal, np, aa, rgbf, rgb8);
  prof_end(sc, st, ev);
  FT_CUDA_TRY(cudaGetLastError(), "trace_pixels_kernel launch");
  sc->last_launches = launches + 1;
  if (!dev_ptrs) {
    if (rgb_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb_out, rgbf, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                             "copy rgb");
    if (rgb8_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb8_out, rgb8, pixels * 3, cudaMemcpyDeviceToHost, st), "copy rgb8");
  }
  FT_CUDA_TRY(cudaStreamSynchronize(st), "trace");
  prof_collect(sc);
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

// Statistics of one Whitted trace, summed per kernel kind of the wavefront
// (march, shade, shadow) from the counting variants of the same kernels.
static ft_status trace_kind_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel, uint32_t aa_samples,
                           uint32_t max_depth, ft_render_stats out[3]) {
  if (!sc || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and stats must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  uint32_t depth = std::max(max_depth, 1u);
  if (depth > 10) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "max_depth must be <= 10");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  size_t pixels = static_cast<size_t>(options->width) * options->height;
  if (ft_status s = ensure_buffers(sc, pixels * aa, pixels)) return s;
  RayParams P = make_params(sc, *options, aa);
  unsigned long long* d = nullptr;
  FT_CUDA_TRY(cudaMalloc(&d, 3 * kStatWords * sizeof(unsigned long long)), "cudaMalloc(stats)");
  std::unique_ptr<unsigned long long, cudaError_t (*)(void*)> guard(d, cudaFree);
  FT_CUDA_TRY(cudaMemset(d, 0, 3 * kStatWords * sizeof(unsigned long long)), "cudaMemset(stats)");
  unsigned long long* kinds[3] = {d, d + kStatWords, d + 2 * kStatWords};
  const bool was = sc->profiling;
  sc->profiling = false;
  uint32_t launches = 0;
  ft_status st = trace_wavefront(sc, P, depth, nullptr, &launches, kinds);
  sc->profiling = was;
  if (st) return st;
  unsigned long long h[3 * kStatWords];
  FT_CUDA_TRY(cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost), "copy stats");
  for (int k = 0; k < 3; ++k) {
    const unsigned long long* v = h + k * kStatWords;
    ft_render_stats& o = out[k];
    std::memset(&o, 0, sizeof(o));
    o.rays = pixels * aa;
    o.distance_evals = v[0];
    o.primitive_evals = v[1];
    o.box_tests = v[2];
    o.hook_instrs = v[3];
    o.march_steps = v[4];
    o.far_steps = v[5];
    o.brick_fetches = v[6];
    o.blend_ops = v[7];
    o.candidate_entries = v[8];
  }
  return FT_OK;
}

ft_status ft_render_trace_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                uint32_t aa_samples, uint32_t max_depth, ft_render_stats* stats) {
  FT_API_BEGIN
  if (!stats) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "stats must be non-null");
  ft_render_stats k[3];
  if (ft_status s = trace_kind_stats(sc, options, accel, aa_samples, max_depth, k)) return s;
  std::memset(stats, 0, sizeof(*stats));
  stats->rays = k[0].rays;
  for (const ft_render_stats& v : k) {
    stats->distance_evals += v.distance_evals;
    stats->primitive_evals += v.primitive_evals;
    stats->box_tests += v.box_tests;
    stats->hook_instrs += v.hook_instrs;
    stats->march_steps += v.march_steps;
    stats->far_steps += v.far_steps;
    stats->brick_fetches += v.brick_fetches;
    stats->blend_ops += v.blend_ops;
    stats->candidate_entries += v.candidate_entries;
  }
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_render_trace_kernel_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                       uint32_t aa_samples, uint32_t max_depth, ft_render_stats* march,
                                       ft_render_stats* shade, ft_render_stats* shadow) {
  FT_API_BEGIN
  if (!march || !shade || !shadow) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "stats must be non-null");
  ft_render_stats k[3];
  if (ft_status s = trace_kind_stats(sc, options, accel, aa_samples, max_depth, k)) return s;
  *march = k[0];
  *shade = k[1];
  *shadow = k[2];
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_profile(ft_scene* sc, uint32_t enable) {
  FT_API_BEGIN
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  std::lock_guard<std::mutex> lock(sc->mu);
  sc->profiling = enable != 0;
  sc->prof_pending.clear();
  for (int k = 0; k < FT_KERNEL_KINDS; ++k) {
    sc->prof_ms[k] = 0.0;
    sc->prof_launches[k] = 0;
  }
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_kernel_times(ft_scene* sc, ft_kernel_times* out) {
  FT_API_BEGIN
  if (!sc || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and out must be non-null");
  std::lock_guard<std::mutex> lock(sc->mu);
  for (int k = 0; k < FT_KERNEL_KINDS; ++k) {
    out->ms[k] = sc->prof_ms[k];
    out->launches[k] = sc->prof_launches[k];
  }
  return FT_OK;
  FT_API_END
}

ft_status ft_render_depth_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                uint32_t aa_samples, uint32_t flags, ft_render_stats* stats) {
  FT_API_BEGIN
  if (!sc || !stats) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and stats must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  size_t pixels = static_cast<size_t>(options->width) * options->height;
  if (ft_status s = ensure_buffers(sc, pixels * aa, pixels)) return s;
  RayParams P = make_params(sc, *options, aa);
  const bool bricks = (flags & FT_FLAG_FP16_BRICKS) != 0;
  const bool was = sc->profiling;
  sc->profiling = false;  // a statistics pass is not one of the timed launches
  ft_status ls = launch_depth(sc, P, nullptr, true, bricks, sc->d_t, sc->d_mask, nullptr, sc->d_normal);
  sc->profiling = was;
  if (ls) return ls;
  unsigned long long h[kStatWords] = {0};
  FT_CUDA_TRY(cudaMemcpy(h, sc->d_stats, sizeof(h), cudaMemcpyDeviceToHost), "copy stats");
  std::memset(stats, 0, sizeof(*stats));
  if (ft_status st = march_check(h[kStatWork + 1])) return st;
  stats->rays = pixels * aa;
  stats->blend_ops = h[7];
  stats->candidate_entries = h[8];
  stats->far_steps = h[5];
  stats->brick_fetches = h[6];
  stats->distance_evals = h[0];
  stats->primitive_evals = h[1];
  stats->box_tests = h[2];
  stats->hook_instrs = h[3];
  stats->march_steps = h[4];
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_build_bricks(ft_scene* sc, const ft_brick_options* options, ft_brick_info* info) {
  FT_API_BEGIN
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  ft_brick_options o{};
  if (options) o = *options;
  const float h = o.voxel_size > 0.0f ? o.voxel_size : 0.02f;
  const float band = o.band > 0.0f ? o.band : 10.0f * h;
  const float safety = o.safety > 0.0f ? o.safety : 1.25f;
  const uint64_t max_points = o.max_lattice_points ? o.max_lattice_points : (1ull << 29);
  if (!std::isfinite(h) || h < 1.0e-4f || !std::isfinite(band) || !std::isfinite(safety) || safety < 1.0f)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "voxel_size must be >= 1e-4, band finite, safety >= 1");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  auto t0 = std::chrono::steady_clock::now();
  free_bricks(sc);
  const ftgpu::SceneImage& im = sc->img;

  DevBricks B{};
  std::vector<int> exact = choose_exact_leaves(im);
  B.n_exact = static_cast<int32_t>(exact.size());
  for (size_t i = 0; i < exact.size(); ++i) B.exact_leaf[i] = exact[i];
  // Region: the cached leaves' boxes, padded, clipped to the scene box.
  float mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
  for (size_t j = 0; j < im.leaves.size(); ++j) {
    if (std::find(exact.begin(), exact.end(), static_cast<int>(j)) != exact.end()) continue;
    for (int a = 0; a < 3; ++a) {
      mn[a] = std::min(mn[a], im.leaves[j].bmin[a]);
      mx[a] = std::max(mx[a], im.leaves[j].bmax[a]);
    }
  }
  const float bs = h * static_cast<float>(kBrickVox);
  float ext = 0.0f;
  for (int a = 0; a < 3; ++a) ext = std::max(ext, mx[a] - mn[a]);
  if (!(ext > 0.0f) || !std::isfinite(ext))
    return ftcommon::fail(FT_ERR_UNSUPPORTED, "scene has no bounded leaves to cache");
  const float pad = std::max(4.0f * bs, 0.1f * ext);
  BrickBuild G{};
  uint64_t n_points = 1;
  for (int a = 0; a < 3; ++a) {
    float lo = std::max(mn[a] - pad, im.scene_min[a]);
    float hi = std::min(mx[a] + pad, im.scene_max[a]);
    if (!(hi > lo)) hi = lo + bs;
    int cells = static_cast<int>(std::ceil((hi - lo) / bs));
    if (cells < 1 || cells > 65536) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "brick region too large for voxel_size");
    G.rmin[a] = lo;
    G.dims[a] = cells;
    n_points *= static_cast<uint64_t>(cells) * kBrickVox + 1;
  }
  if (n_points > max_points)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "brick lattice of " + std::to_string(n_points) +
                                                       " points exceeds max_lattice_points; raise voxel_size");
  G.h = h;
  G.nx = static_cast<uint32_t>(G.dims[0]) * kBrickVox + 1;
  G.ny = static_cast<uint32_t>(G.dims[1]) * kBrickVox + 1;
  G.nz = static_cast<uint32_t>(G.dims[2]) * kBrickVox + 1;
  const uint64_t n_cells = static_cast<uint64_t>(G.dims[0]) * G.dims[1] * G.dims[2];
  int mw = 0, mh = 0, md = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&mw, cudaDevAttrMaxTexture3DWidth, sc->device), "texture limits");
  FT_CUDA_TRY(cudaDeviceGetAttribute(&mh, cudaDevAttrMaxTexture3DHeight, sc->device), "texture limits");
  FT_CUDA_TRY(cudaDeviceGetAttribute(&md, cudaDevAttrMaxTexture3DDepth, sc->device), "texture limits");
  if (G.nx > static_cast<uint32_t>(mw) || G.ny > static_cast<uint32_t>(mh) || G.nz > static_cast<uint32_t>(md))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "brick lattice exceeds the 3D texture limits; raise voxel_size");
  std::memcpy(B.rmin, G.rmin, sizeof(B.rmin));
  B.inv_h = 1.0f / h;
  B.last[0] = static_cast<float>(G.nx - 1);
  B.last[1] = static_cast<float>(G.ny - 1);
  B.last[2] = static_cast<float>(G.nz - 1);
  B.band = band;
  B.far_batch = static_cast<int32_t>(std::min(o.far_steps_per_pass ? o.far_steps_per_pass : 4u, 64u));
  // back to the far field once the exact distance clearly exceeds where the
  // bound of a 1-Lipschitz brick would hand over again
  B.band_exit = 2.0f * (band + safety * h * 1.7320508f);
  for (int a = 0; a < 3; ++a) B.rmax[a] = G.rmin[a] + bs * static_cast<float>(G.dims[a]);
  B.free_far = (o.flags & FT_BRICK_FREE_FAR_STEPS) ? 1 : 0;
  // Outside the region the cached leaves are at least the distance to its
  // box away when each lies in its own box: primitives and union_round trees
  // (a round blend can bulge out of its operands' boxes by 0.3 r, hence the
  // margin), not hooked or modified leaves.
  B.outside_ok = 1;
  float r_max = 0.0f;
  for (const ftgpu::HostUrTree& t : im.urtrees) r_max = std::max(r_max, t.r);
  for (size_t j = 0; j < im.leaves.size(); ++j) {
    if (std::find(exact.begin(), exact.end(), static_cast<int>(j)) != exact.end()) continue;
    int kind = im.leaves[j].kind;
    if (kind != ftgpu::kLeafPrim && kind != ftgpu::kLeafUrTree) B.outside_ok = 0;
  }
  B.outside_margin = std::max(band, r_max);
  // A single exact leaf that is an axis-aligned box with sharp edges and no
  // shell: its distance above the top face is the height over that face.
  B.plane_leaf = -1;
  if (exact.size() == 1 && im.leaves[exact[0]].kind == ftgpu::kLeafPrim) {
    const ftgpu::HostNode& n = im.nodes[im.leaves[exact[0]].node];
    if (n.kind == FT_NODE_BOX && !n.has_rot && n.f[3] == 0.0f && n.f[4] == 0.0f && n.program < 0) {
      B.plane_leaf = exact[0];
      B.plane_obj = n.object_id;
      B.plane_top = n.c[1] + n.f[1];
      B.plane_lo[0] = n.c[0] - n.f[0];
      B.plane_hi[0] = n.c[0] + n.f[0];
      B.plane_lo[1] = n.c[2] - n.f[2];
      B.plane_hi[1] = n.c[2] + n.f[2];
    }
  }

  DeviceTemps tmp;
  float* lattice = nullptr;
  float* delta = nullptr;
  unsigned int* counters = nullptr;
  FT_CUDA_TRY(tmp.alloc(&lattice, n_points), "cudaMalloc(brick lattice)");
  FT_CUDA_TRY(tmp.alloc(&delta, n_cells), "cudaMalloc(brick bounds)");
  FT_CUDA_TRY(tmp.alloc(&counters, 2), "cudaMalloc(brick counters)");
  FT_CUDA_TRY(cudaMemset(counters, 0, 2 * sizeof(unsigned int)), "cudaMemset(brick counters)");
  int sms = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device), "sm count");
  const unsigned grid = static_cast<unsigned>(std::max(sms, 1) * 16);
  brick_lattice_kernel<<<grid, 128>>>(sc->dev, B, G, lattice);
  FT_CUDA_TRY(cudaGetLastError(), "brick_lattice_kernel launch");
  // Box no cached bound may be trusted in: every generic (hooked or
  // modified) leaf's box, grown by the largest translation in the scene (a
  // domain + distance_post pair applies its transform twice) and the band.
  float untrusted[6] = {kInf, kInf, kInf, -kInf, -kInf, -kInf};
  {
    float shift = 0.0f;
    for (const ftgpu::HostNode& n : im.nodes)
      shift = std::max(shift, std::sqrt(n.c[0] * n.c[0] + n.c[1] * n.c[1] + n.c[2] * n.c[2]));
    for (size_t j = 0; j < im.leaves.size(); ++j) {
      const ftgpu::HostLeaf& lf = im.leaves[j];
      if (lf.kind != ftgpu::kLeafGeneric) continue;
      if (std::find(exact.begin(), exact.end(), static_cast<int>(j)) != exact.end()) continue;
      for (int a = 0; a < 3; ++a) {
        untrusted[a] = std::min(untrusted[a], lf.bmin[a] - shift - band);
        untrusted[3 + a] = std::max(untrusted[3 + a], lf.bmax[a] + shift + band);
      }
    }
  }
  float* d_untrusted = nullptr;
  FT_CUDA_TRY(tmp.alloc(&d_untrusted, 6), "cudaMalloc(untrusted box)");
  FT_CUDA_TRY(cudaMemcpy(d_untrusted, untrusted, sizeof(untrusted), cudaMemcpyHostToDevice), "upload");
  brick_bound_kernel<<<grid, 128>>>(G, lattice, safety, band + 0.5f * bs, d_untrusted, delta, counters, counters + 1);
  FT_CUDA_TRY(cudaGetLastError(), "brick_bound_kernel launch");
  cudaChannelFormatDesc fmt = cudaCreateChannelDescHalf();
  cudaExtent extent = make_cudaExtent(G.nx, G.ny, G.nz);
  FT_CUDA_TRY(cudaMalloc3DArray(&sc->brick_array, &fmt, extent, cudaArraySurfaceLoadStore), "cudaMalloc3DArray(bricks)");
  cudaResourceDesc res{};
  res.resType = cudaResourceTypeArray;
  res.res.array.array = sc->brick_array;
  cudaSurfaceObject_t surf = 0;
  FT_CUDA_TRY(cudaCreateSurfaceObject(&surf, &res), "cudaCreateSurfaceObject(bricks)");
  brick_texel_kernel<<<grid, 256>>>(G, lattice, delta, surf);
  cudaError_t fe = cudaGetLastError();
  if (fe == cudaSuccess) fe = cudaDeviceSynchronize();
  cudaDestroySurfaceObject(surf);
  FT_CUDA_TRY(fe, "brick_texel_kernel");
  unsigned int hc[2] = {0, 0};
  FT_CUDA_TRY(cudaMemcpy(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost), "brick build");
  const uint32_t n_near = hc[0];
  float max_lip = 0.0f;
  std::memcpy(&max_lip, &hc[1], sizeof(max_lip));
  cudaTextureDesc td{};
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
  td.filterMode = cudaFilterModeLinear;
  td.readMode = cudaReadModeElementType;
  td.normalizedCoords = 0;
  FT_CUDA_TRY(cudaCreateTextureObject(&B.atlas, &res, &td, nullptr), "cudaCreateTextureObject(bricks)");
  sc->bricks = B;
  sc->has_bricks = true;
  sc->brick_bytes = n_points * sizeof(uint16_t);
  auto t1 = std::chrono::steady_clock::now();
  if (info) {
    std::memset(info, 0, sizeof(*info));
    for (int a = 0; a < 3; ++a) {
      info->region_min[a] = G.rmin[a];
      info->region_max[a] = G.rmin[a] + bs * static_cast<float>(G.dims[a]);
      info->bricks[a] = static_cast<uint32_t>(G.dims[a]);
    }
    info->near_bricks = n_near;
    info->exact_leaves = static_cast<uint32_t>(exact.size());
    info->max_lipschitz = max_lip;
    info->band = band;
    info->device_bytes = sc->brick_bytes;
    info->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_brick_bounds(ft_scene* sc, const float* points, uint32_t n, float* bound_out, float* exact_out) {
  FT_API_BEGIN
  if (!sc || (n && (!points || !bound_out || !exact_out)))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene, points and outputs must be non-null");
  std::lock_guard<std::mutex> lock(sc->mu);
  if (!sc->has_bricks) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "no brick cache: call ft_scene_build_bricks first");
  if (n == 0) return FT_OK;
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  DeviceTemps tmp;
  float *dp = nullptr, *db = nullptr, *de = nullptr;
  FT_CUDA_TRY(tmp.alloc(&dp, static_cast<size_t>(n) * 3), "cudaMalloc(points)");
  FT_CUDA_TRY(tmp.alloc(&db, n), "cudaMalloc(bounds)");
  FT_CUDA_TRY(tmp.alloc(&de, n), "cudaMalloc(exact)");
  FT_CUDA_TRY(cudaMemcpy(dp, points, static_cast<size_t>(n) * 3 * sizeof(float), cudaMemcpyHostToDevice), "copy points");
  brick_query_kernel<<<(n + 127) / 128, 128>>>(sc->dev, sc->bricks, dp, n, db, de);
  FT_CUDA_TRY(cudaGetLastError(), "brick_query_kernel launch");
  FT_CUDA_TRY(cudaMemcpy(bound_out, db, static_cast<size_t>(n) * sizeof(float), cudaMemcpyDeviceToHost), "copy bounds");
  FT_CUDA_TRY(cudaMemcpy(exact_out, de, static_cast<size_t>(n) * sizeof(float), cudaMemcpyDeviceToHost), "copy exact");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_create(const ft_batch_item* items, uint32_t n, uint32_t flags, ft_batch** out) {
  FT_API_BEGIN
  if (!out || (n && !items)) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "items and out must be non-null");
  *out = nullptr;
  if (n == 0) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "a batch needs at least one item");
  int device = 0;
  FT_CUDA_TRY(cudaGetDevice(&device), "cudaGetDevice");
  const bool bricks = (flags & FT_BATCH_FP16_BRICKS) != 0;
  for (uint32_t i = 0; i < n; ++i) {
    const ft_batch_item& it = items[i];
    if (!it.scene) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch item " + std::to_string(i) + " has no scene");
    if (it.scene->device != device)
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch items must live on the current device");
    if (ft_status st = check_options(&it.options, std::max(it.aa_samples, 1u))) return st;
    if (it.max_depth > 10) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "max_depth must be <= 10");
    if (bricks && it.max_depth == 0 && !it.scene->has_bricks)
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT,
                            "FT_BATCH_FP16_BRICKS needs ft_scene_build_bricks on every depth item's scene");
  }
  auto* b = new (std::nothrow) ft_batch();
  if (!b) return ftcommon::fail(FT_ERR_OUT_OF_MEMORY, "out of host memory");
  std::unique_ptr<ft_batch, void (*)(ft_batch*)> guard(b, ft_batch_destroy);
  b->device = device;
  b->bricks = bricks;
  b->items.assign(items, items + n);
  FT_CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  FT_CUDA_TRY(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "cudaEventCreate");
  uint64_t pix_total = 0, samples[2] = {0, 0};
  for (uint32_t i = 0; i < n; ++i) {
    const ft_batch_item& it = items[i];
    int k = it.max_depth == 0 ? 0 : 1;
    uint32_t aa = std::max(it.aa_samples, 1u);
    uint64_t px = static_cast<uint64_t>(it.options.width) * it.options.height;
    b->part[k].items.push_back(i);
    b->part[k].out_first.push_back(samples[k]);
    BatchPixItem pi{};
    pi.pix_first = pix_total;
    pi.out_first = samples[k];
    pi.aa = aa;
    pi.kind = static_cast<uint32_t>(k);
    pi.max_dist = it.options.max_dist;
    b->pix.push_back(pi);
    pix_total += px;
    samples[k] += px * aa;
  }
  b->n_pixels = pix_total;
  int sms = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "sm count");
  for (int k = 0; k < 2; ++k) {
    BatchPart& part = b->part[k];
    part.n_samples = samples[k];
    size_t m = part.items.size();
    if (m == 0) continue;
    std::vector<DevScene> scenes;
    std::vector<DevBricks> bricks_v;
    std::vector<uint32_t> depth;
    for (uint32_t it : part.items) {
      scenes.push_back(b->items[it].scene->dev);
      bricks_v.push_back(b->items[it].scene->bricks);
      depth.push_back(std::max(b->items[it].max_depth, 1u));
    }
    FT_CUDA_TRY(cudaMalloc(&part.d_scenes, m * sizeof(DevScene)), "cudaMalloc(batch scenes)");
    FT_CUDA_TRY(cudaMalloc(&part.d_params, m * sizeof(RayParams)), "cudaMalloc(batch params)");
    FT_CUDA_TRY(cudaMalloc(&part.d_bricks, m * sizeof(DevBricks)), "cudaMalloc(batch bricks)");
    FT_CUDA_TRY(cudaMalloc(&part.d_ray_first, (m + 1) * sizeof(uint64_t)), "cudaMalloc(batch offsets)");
    FT_CUDA_TRY(cudaMalloc(&part.d_out_first, m * sizeof(uint64_t)), "cudaMalloc(batch offsets)");
    FT_CUDA_TRY(cudaMalloc(&part.d_max_depth, m * sizeof(uint32_t)), "cudaMalloc(batch depths)");
    FT_CUDA_TRY(cudaMemcpy(part.d_scenes, scenes.data(), m * sizeof(DevScene), cudaMemcpyHostToDevice), "upload");
    FT_CUDA_TRY(cudaMemcpy(part.d_bricks, bricks_v.data(), m * sizeof(DevBricks), cudaMemcpyHostToDevice), "upload");
    FT_CUDA_TRY(cudaMemcpy(part.d_out_first, part.out_first.data(), m * sizeof(uint64_t), cudaMemcpyHostToDevice),
                "upload");
    FT_CUDA_TRY(cudaMemcpy(part.d_max_depth, depth.data(), m * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload");
    int per_sm = 1;
    if (k == 0) {
      if (bricks)
        FT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_depth_persistent<false, true, true>,
                                                                  128, 0), "occupancy");
      else
        FT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_depth_persistent<false, false, true>,
                                                                  128, 0), "occupancy");
    } else {
      per_sm = 16;  // grid-stride wavefront kernels
      for (uint32_t it : part.items) {
        b->wf_levels = std::max(b->wf_levels, std::max(b->items[it].max_depth, 1u));
        uint32_t ls = 0;
        for (const ft_light& L : b->items[it].scene->img.lights)
          ls += L.kind == FT_LIGHT_SPHERE ? std::max(L.samples, 1u) : 1u;
        b->wf_light_samples = std::max(b->wf_light_samples, ls);
        b->wf_max_push = std::max(b->wf_max_push, max_rays_per_hit(b->items[it].scene->img));
      }
    }
    part.blocks = std::max(1, sms * std::max(per_sm, 1));
  }
  FT_CUDA_TRY(cudaMalloc(&b->d_pix, b->pix.size() * sizeof(BatchPixItem)), "cudaMalloc(batch pixels)");
  FT_CUDA_TRY(cudaMemcpy(b->d_pix, b->pix.data(), b->pix.size() * sizeof(BatchPixItem), cudaMemcpyHostToDevice),
              "upload");
  FT_CUDA_TRY(cudaMalloc(&b->d_t, std::max<uint64_t>(samples[0], 1) * sizeof(float)), "cudaMalloc(batch depth)");
  FT_CUDA_TRY(cudaMalloc(&b->d_mask, std::max<uint64_t>(samples[0], 1)), "cudaMalloc(batch mask)");
  FT_CUDA_TRY(cudaMalloc(&b->d_srgb, std::max<uint64_t>(samples[1], 1) * 3 * sizeof(float)),
              "cudaMalloc(batch radiance)");
  FT_CUDA_TRY(cudaMalloc(&b->d_rgbf, pix_total * 3 * sizeof(float)), "cudaMalloc(batch rgb)");
  FT_CUDA_TRY(cudaMalloc(&b->d_rgb8, pix_total * 3), "cudaMalloc(batch rgb8)");
  FT_CUDA_TRY(cudaMalloc(&b->d_counters, 2 * sizeof(unsigned long long)), "cudaMalloc(batch counters)");
  FT_CUDA_TRY(cudaMalloc(&b->wf_counters, kWfCounters * sizeof(unsigned long long)),
              "cudaMalloc(batch queue counters)");
  FT_CUDA_TRY(cudaMemset(b->wf_counters, 0, kWfCounters * sizeof(unsigned long long)),
              "cudaMemset(batch queue counters)");
  b->sms = sms;
  if (samples[1] >= kNoSample) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "too many Whitted samples in one batch");
  if (ft_status st = batch_apply_tuning(b)) return st;
  *out = guard.release();
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_set_tuning(ft_batch* b, const ft_batch_tuning* t) {
  FT_API_BEGIN
  if (!b || !t) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch and tuning must be non-null");
  if (ft_status st = check_tuning(*t)) return st;
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaEventSynchronize(b->done), "wait for the last batch launch");
  FT_CUDA_TRY(cudaStreamSynchronize(b->stream), "batch");
  b->tuning = *t;
  if (ft_status st = batch_apply_tuning(b)) return st;
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_autotune(ft_batch* b, ft_batch_tuning* best) {
  FT_API_BEGIN
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaEventSynchronize(b->done), "wait for the last batch launch");
  const uint32_t tiles[3][2] = {{8, 8}, {16, 8}, {32, 8}};
  const uint32_t refills[3] = {4, 8, 16};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FT_CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
  FT_CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
  ft_batch_tuning top{8, 8, 8, 1e30f};
  ft_status status = FT_OK;
  bool warm = false;
  for (const auto& tl : tiles) {
    for (uint32_t rf : refills) {
      b->tuning = ft_batch_tuning{tl[0], tl[1], rf, 0.0f};
      if ((status = batch_apply_tuning(b)) != FT_OK) break;
      if (!warm) cudaGraphLaunch(b->exec, b->stream);  // one warm-up (first touch of the queues)
      warm = true;
      cudaEventRecord(e0, b->stream);
      cudaGraphLaunch(b->exec, b->stream);
      cudaEventRecord(e1, b->stream);
      cudaError_t e = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        status = ftcommon::fail(FT_ERR_CUDA, cuda_msg(e, "batch autotune"));
        break;
      }
      if ((status = batch_overflow(b)) != FT_OK) break;
      if (ms < top.ms) top = ft_batch_tuning{tl[0], tl[1], rf, ms};
    }
    if (status != FT_OK) break;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status != FT_OK) return status;
  b->tuning = top;
  if (ft_status st = batch_apply_tuning(b)) return st;
  if (best) *best = top;
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_launch(ft_batch* b, void* stream) {
  FT_API_BEGIN
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  // Two launches of one batch share its counters and queues: the graph waits
  // for the previous launch, wherever that was enqueued.
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  FT_CUDA_TRY(cudaStreamWaitEvent(st, b->done, 0), "order after the last batch launch");
  FT_CUDA_TRY(cudaGraphLaunch(b->exec, st), "cudaGraphLaunch(batch)");
  FT_CUDA_TRY(cudaEventRecord(b->done, st), "record batch completion");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_read(ft_batch* b, uint32_t item, float* t_out, uint8_t* mask_out, float* rgb_out,
                        uint8_t* rgb8_out) {
  FT_API_BEGIN
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  if (item >= b->items.size()) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch item out of range");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaDeviceSynchronize(), "batch");
  if (ft_status s = batch_overflow(b)) return s;
  const ft_batch_item& it = b->items[item];
  const BatchPixItem& pi = b->pix[item];
  uint64_t px = static_cast<uint64_t>(it.options.width) * it.options.height;
  uint64_t ns = px * pi.aa;
  if ((t_out || mask_out) && pi.kind != 0)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "t_out and mask_out exist for depth items only");
  if (t_out)
    FT_CUDA_TRY(cudaMemcpy(t_out, b->d_t + pi.out_first, ns * sizeof(float), cudaMemcpyDeviceToHost), "copy depth");
  if (mask_out) FT_CUDA_TRY(cudaMemcpy(mask_out, b->d_mask + pi.out_first, ns, cudaMemcpyDeviceToHost), "copy mask");
  if (rgb_out)
    FT_CUDA_TRY(cudaMemcpy(rgb_out, b->d_rgbf + 3 * pi.pix_first, px * 3 * sizeof(float), cudaMemcpyDeviceToHost),
                "copy rgb");
  if (rgb8_out)
    FT_CUDA_TRY(cudaMemcpy(rgb8_out, b->d_rgb8 + 3 * pi.pix_first, px * 3, cudaMemcpyDeviceToHost), "copy rgb8");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_batch_samples(const ft_batch* b, uint64_t* primary_samples) {
  if (!b || !primary_samples) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch and output must be non-null");
  *primary_samples = b->part[0].n_samples + b->part[1].n_samples;
  return FT_OK;
}

void ft_batch_destroy(ft_batch* b) {
  if (!b) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  if (b->done) cudaEventSynchronize(b->done);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto& p : b->part) free_part(p);
  cudaFree(b->d_pix);
  cudaFree(b->d_t);
  cudaFree(b->d_mask);
  cudaFree(b->d_srgb);
  cudaFree(b->d_rgbf);
  cudaFree(b->d_rgb8);
  cudaFree(b->d_counters);
  cudaFree(b->wf_jobs[0]);
  cudaFree(b->wf_jobs[1]);
  cudaFree(b->wf_hits);
  cudaFree(b->wf_shadows);
  cudaFree(b->wf_counters);
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->done) cudaEventDestroy(b->done);
  cudaSetDevice(prev);
  delete b;
}

// Per-view ray parameters: the view's camera, one sample per pixel.
std::vector<RayParams> view_params(const ft_scene* sc, const ft_view* views, uint32_t n, const ft_render_options& o) {
  std::vector<RayParams> out;
  for (uint32_t v = 0; v < n; ++v) {
    RayParams P = make_params(sc, o, 1);
    ftgpu::CameraBasis cb = ftgpu::camera_basis(views[v].origin, views[v].target, views[v].fov_y_degrees);
    std::memcpy(P.origin, cb.origin, sizeof(P.origin));
    std::memcpy(P.fwd, cb.forward, sizeof(P.fwd));
    std::memcpy(P.right, cb.right, sizeof(P.right));
    std::memcpy(P.up, cb.up, sizeof(P.up));
    P.tan_fov = cb.tan_fov;
    out.push_back(P);
  }
  return out;
}

ft_status check_views(const ft_scene* sc, const ft_view* views, uint32_t n, const ft_render_options* o, float tau) {
  if (!sc || !views || n == 0) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and views must be non-null");
  if (ft_status s = check_options(o, 1)) return s;
  if (!(tau > 0.0f) || !std::isfinite(tau)) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "tau must be > 0");
  return FT_OK;
}

ft_status ft_render_views(ft_scene* sc, const ft_view* views, uint32_t n_views, const ft_render_options* options,
                          float tau, float* t_out, uint8_t* mask_out, float* sil_out, uint32_t flags, void* stream) {
  FT_API_BEGIN
  if (ft_status s = check_views(sc, views, n_views, options, tau)) return s;
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  std::vector<RayParams> vp = view_params(sc, views, n_views, *options);
  const uint64_t per_view_px = static_cast<uint64_t>(options->width) * options->height;
  const uint64_t items = vp[0].n_items;
  DeviceTemps tmp;
  RayParams* d_views = nullptr;
  FT_CUDA_TRY(tmp.alloc(&d_views, n_views), "cudaMalloc(views)");
  FT_CUDA_TRY(cudaMemcpyAsync(d_views, vp.data(), n_views * sizeof(RayParams), cudaMemcpyHostToDevice, st), "upload");
  float* t = t_out;
  uint8_t* m = mask_out;
  float* sil = sil_out;
  const uint64_t total_px = per_view_px * n_views;
  if (!dev_ptrs) {
    if (t_out) FT_CUDA_TRY(tmp.alloc(&t, total_px), "cudaMalloc(depth)");
    if (mask_out) FT_CUDA_TRY(tmp.alloc(&m, total_px), "cudaMalloc(mask)");
    if (sil_out) FT_CUDA_TRY(tmp.alloc(&sil, total_px), "cudaMalloc(silhouette)");
  }
  uint64_t threads = items * n_views;
  views_forward_kernel<<<static_cast<unsigned>((threads + 127) / 128), 128, 0, st>>>(sc->dev, d_views, n_views, items,
                                                                                     tau, t, m, sil);
  FT_CUDA_TRY(cudaGetLastError(), "views_forward_kernel launch");
  if (!dev_ptrs) {
    if (t_out) FT_CUDA_TRY(cudaMemcpyAsync(t_out, t, total_px * sizeof(float), cudaMemcpyDeviceToHost, st), "copy");
    if (mask_out) FT_CUDA_TRY(cudaMemcpyAsync(mask_out, m, total_px, cudaMemcpyDeviceToHost, st), "copy");
    if (sil_out) FT_CUDA_TRY(cudaMemcpyAsync(sil_out, sil, total_px * sizeof(float), cudaMemcpyDeviceToHost, st), "copy");
  }
  FT_CUDA_TRY(cudaStreamSynchronize(st), "views");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_render_backward(ft_scene* sc, const ft_view* views, uint32_t n_views, const ft_render_options* options,
                             float tau, const ft_param* params, uint32_t n_params, const float* dL_dt,
                             const float* dL_dsil, double* dL_dparams, uint32_t flags, void* stream) {
  FT_API_BEGIN
  if (ft_status s = check_views(sc, views, n_views, options, tau)) return s;
  if (!dL_dparams || (n_params && !params))
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "params and dL_dparams must be non-null");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  const ftgpu::SceneImage& im = sc->img;
  // parameter slots per (node, field) and per union_round tree
  std::vector<int32_t> slot(im.nodes.size() * 8, -1);
  for (uint32_t k = 0; k < n_params; ++k) {
    const ft_param& p = params[k];
    if (p.node < 0 || static_cast<size_t>(p.node) >= im.nodes.size() || p.field < 0 || p.field > FT_PARAM_RADIUS)
      return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "parameter " + std::to_string(k) + " is out of range");
    slot[static_cast<size_t>(p.node) * 8 + p.field] = static_cast<int32_t>(k);
  }
  std::vector<int32_t> tree_radius(std::max<size_t>(im.urtrees.size(), 1), -1);
  for (const ftgpu::HostLeaf& lf : im.leaves) {
    if (lf.kind != ftgpu::kLeafUrTree) continue;
    // any union_round node of the tree may name its radius
    std::vector<int> stack{lf.node};
    while (!stack.empty()) {
      int k = stack.back();
      stack.pop_back();
      if (k < 0 || static_cast<size_t>(k) >= im.nodes.size() || im.nodes[k].kind != FT_NODE_UNION_ROUND) continue;
      int32_t s = slot[static_cast<size_t>(k) * 8 + FT_PARAM_RADIUS];
      if (s >= 0) tree_radius[lf.first] = s;
      stack.push_back(im.nodes[k].a);
      stack.push_back(im.nodes[k].b);
    }
  }
  std::vector<RayParams> vp = view_params(sc, views, n_views, *options);
  const uint64_t per_view_px = static_cast<uint64_t>(options->width) * options->height;
  const uint64_t total_px = per_view_px * n_views;
  const uint64_t items = vp[0].n_items;
  DeviceTemps tmp;
  RayParams* d_views = nullptr;
  int32_t *d_slot = nullptr, *d_tree = nullptr;
  int* d_bad = nullptr;
  double* d_grad = nullptr;
  FT_CUDA_TRY(tmp.alloc(&d_views, n_views), "cudaMalloc(views)");
  FT_CUDA_TRY(tmp.alloc(&d_slot, slot.size()), "cudaMalloc(slots)");
  FT_CUDA_TRY(tmp.alloc(&d_tree, tree_radius.size()), "cudaMalloc(slots)");
  FT_CUDA_TRY(tmp.alloc(&d_bad, 1), "cudaMalloc(flag)");
  FT_CUDA_TRY(tmp.alloc(&d_grad, std::max<uint32_t>(n_params, 1)), "cudaMalloc(gradient)");
  FT_CUDA_TRY(cudaMemcpyAsync(d_views, vp.data(), n_views * sizeof(RayParams), cudaMemcpyHostToDevice, st), "upload");
  FT_CUDA_TRY(cudaMemcpyAsync(d_slot, slot.data(), slot.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st), "upload");
  FT_CUDA_TRY(cudaMemcpyAsync(d_tree, tree_radius.data(), tree_radius.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                              st),
              "upload");
  FT_CUDA_TRY(cudaMemsetAsync(d_bad, 0, sizeof(int), st), "memset");
  FT_CUDA_TRY(cudaMemsetAsync(d_grad, 0, std::max<uint32_t>(n_params, 1) * sizeof(double), st), "memset");
  const float* a = dL_dt;
  const float* b = dL_dsil;
  if (!dev_ptrs) {
    float *da = nullptr, *db = nullptr;
    if (dL_dt) {
      FT_CUDA_TRY(tmp.alloc(&da, total_px), "cudaMalloc(dL_dt)");
      FT_CUDA_TRY(cudaMemcpyAsync(da, dL_dt, total_px * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
    }
    if (dL_dsil) {
      FT_CUDA_TRY(tmp.alloc(&db, total_px), "cudaMalloc(dL_dsil)");
      FT_CUDA_TRY(cudaMemcpyAsync(db, dL_dsil, total_px * sizeof(float), cudaMemcpyHostToDevice, st), "upload");
    }
    a = da;
    b = db;
  }
  DiffTables T{d_slot, d_tree, n_params};
  const size_t smem = static_cast<size_t>(n_params) * sizeof(double);
  const int shared_acc = (n_params > 0 && smem <= 48 * 1024) ? 1 : 0;
  int sms = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device), "sm count");
  uint64_t want = (items * n_views + 127) / 128;
  unsigned grid = static_cast<unsigned>(std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(sms) * 8)));
  views_backward_kernel<<<grid, 128, shared_acc ? smem : 0, st>>>(sc->dev, d_views, n_views, items, tau, T, a, b,
                                                                  d_grad, shared_acc, d_bad);
  FT_CUDA_TRY(cudaGetLastError(), "views_backward_kernel launch");
  int bad = 0;
  FT_CUDA_TRY(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st), "copy");
  if (dev_ptrs)
    FT_CUDA_TRY(cudaMemcpyAsync(dL_dparams, d_grad, n_params * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
  else
    FT_CUDA_TRY(cudaMemcpyAsync(dL_dparams, d_grad, n_params * sizeof(double), cudaMemcpyDeviceToHost, st), "copy");
  FT_CUDA_TRY(cudaStreamSynchronize(st), "backward");
  if (bad) return ftcommon::fail(FT_ERR_UNSUPPORTED, "the hit leaf is not a union_round tree of spheres / boxes "
                                                     "(or has more than 512 primitives): no adjoint");
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_scene_jit(ft_scene* sc, ft_jit_info* info) {
  FT_API_BEGIN
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  const ftgpu::SceneImage& im = sc->img;
  ft_jit_info out{};
  out.programs = static_cast<uint32_t>(im.programs.size());
  std::string src = "// scene module compiled at run time\n#include \"ft_kernels.cuh\"\nnamespace {\n" +
                    ftgpu::jit_hook_source(im.programs.data(), static_cast<uint32_t>(im.programs.size()),
                                           im.instrs.data()) +
                    "}  // namespace\n";
  out.source_bytes = src.size();
  constexpr int kJitKernels = 5;
  static const char* const kExprs[kJitKernels] = {"march_depth_persistent<false, false, false>",
                                                  "march_depth_persistent<false, true, false>",
                                                  "wf_march_persistent<false, false>", "wf_shade_kernel<false>",
                                                  "wf_shadow_persistent<false, false>"};
  struct Module {
    std::vector<char> cubin;
    std::string lowered[kJitKernels];
  };
  static std::mutex cache_mu;
  static std::map<std::string, Module> cache;
  Module mod;
  bool cached = false;
  {
    std::lock_guard<std::mutex> cl(cache_mu);
    auto it = cache.find(src);
    if (it != cache.end()) {
      mod = it->second;
      cached = true;
    }
  }
  auto t0 = std::chrono::steady_clock::now();
  if (!cached) {
    const int nh = ftgpu::jit_header_count();
    std::vector<const char*> texts(nh), names(nh);
    for (int i = 0; i < nh; ++i) {
      texts[i] = ftgpu::jit_header_text(i);
      names[i] = ftgpu::jit_header_name(i);
    }
    nvrtcProgram prog = nullptr;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "ft_scene_jit.cu", nh, texts.data(), names.data());
    if (r != NVRTC_SUCCESS) return ftcommon::fail(FT_ERR_JIT, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    std::unique_ptr<nvrtcProgram, void (*)(nvrtcProgram*)> guard(&prog, [](nvrtcProgram* p) { nvrtcDestroyProgram(p); });
    for (const char* e : kExprs) nvrtcAddNameExpression(prog, e);
    int major = 0, minor = 0;
    FT_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, sc->device), "device arch");
    FT_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, sc->device), "device arch");
    // arch-specific target (sm_103a on GB300), as the precompiled kernels
    std::string arch = "--gpu-architecture=sm_" + std::to_string(major * 10 + minor) + "a";
    const char* opts[] = {arch.c_str(), "-std=c++17", "-DFT_JIT=1", "--device-as-default-execution-space"};
    r = nvrtcCompileProgram(prog, 4, opts);
    if (r != NVRTC_SUCCESS) {
      size_t n = 0;
      nvrtcGetProgramLogSize(prog, &n);
      std::string log(n, '\0');
      if (n) nvrtcGetProgramLog(prog, &log[0]);
      if (log.size() > 2000) log.resize(2000);
      return ftcommon::fail(FT_ERR_JIT, std::string("nvrtcCompileProgram: ") + nvrtcGetErrorString(r) + "\n" + log);
    }
    size_t cubin_size = 0;
    r = nvrtcGetCUBINSize(prog, &cubin_size);
    if (r != NVRTC_SUCCESS || cubin_size == 0) return ftcommon::fail(FT_ERR_JIT, "nvrtcGetCUBINSize failed");
    mod.cubin.resize(cubin_size);
    r = nvrtcGetCUBIN(prog, mod.cubin.data());
    if (r != NVRTC_SUCCESS) return ftcommon::fail(FT_ERR_JIT, "nvrtcGetCUBIN failed");
    for (int k = 0; k < kJitKernels; ++k) {
      const char* lowered = nullptr;
      r = nvrtcGetLoweredName(prog, kExprs[k], &lowered);
      if (r != NVRTC_SUCCESS || !lowered) return ftcommon::fail(FT_ERR_JIT, std::string("no kernel ") + kExprs[k]);
      mod.lowered[k] = lowered;
    }
    std::lock_guard<std::mutex> cl(cache_mu);
    cache.emplace(src, mod);
  }
  auto t1 = std::chrono::steady_clock::now();
  cudaLibrary_t lib = nullptr;
  FT_CUDA_TRY(cudaLibraryLoadData(&lib, mod.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
              "cudaLibraryLoadData(scene module)");
  cudaKernel_t k[kJitKernels] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int i = 0; i < kJitKernels; ++i) {
    cudaError_t e = cudaLibraryGetKernel(&k[i], lib, mod.lowered[i].c_str());
    if (e != cudaSuccess) {
      cudaLibraryUnload(lib);
      return ftcommon::fail(FT_ERR_JIT, cuda_msg(e, "cudaLibraryGetKernel"));
    }
  }
  int sms = 0;
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device), "sm count");
  int blocks[2] = {sc->persistent_blocks, sc->persistent_blocks_bricks};
  for (int i = 0; i < 2; ++i) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void*>(k[i]), 128, 0) ==
            cudaSuccess &&
        per_sm > 0)
      blocks[i] = sms * per_sm;
    else
      cudaGetLastError();
  }
  if (sc->jit_lib) cudaLibraryUnload(sc->jit_lib);
  sc->jit_lib = lib;
  sc->jit_depth[0] = k[0];
  sc->jit_depth[1] = k[1];
  sc->jit_wf[0] = k[2];
  sc->jit_wf[1] = k[3];
  sc->jit_wf[2] = k[4];
  sc->jit_blocks[0] = blocks[0];
  sc->jit_blocks[1] = blocks[1];
  auto t2 = std::chrono::steady_clock::now();
  out.cached = cached ? 1u : 0u;
  out.cubin_bytes = mod.cubin.size();
  out.compile_ms = cached ? 0.0 : std::chrono::duration<double, std::milli>(t1 - t0).count();
  out.load_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  if (info) *info = out;
  ftcommon::clear_last_error();
  return FT_OK;
  FT_API_END
}

ft_status ft_measure_fp32_peak(double* tflops) {
  FT_API_BEGIN
  if (!tflops) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "tflops must be non-null");
  int dev = 0, sms = 0;
  FT_CUDA_TRY(cudaGetDevice(&dev), "cudaGetDevice");
  FT_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "sm count");
  float* out = nullptr;
  FT_CUDA_TRY(cudaMalloc(&out, sizeof(float)), "cudaMalloc");
  const int iters = 1 << 16, threads = 256, blocks = sms * 8;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  fma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 0.001f);
  cudaEventRecord(a);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) fma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 0.001f);
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess) return ftcommon::fail(FT_ERR_CUDA, cuda_msg(e, "fma_peak_kernel"));
  double flops = 2.0 * 8.0 * iters * double(threads) * blocks * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return FT_OK;
  FT_API_END
}

}  // extern "C"
