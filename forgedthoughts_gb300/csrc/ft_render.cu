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

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.h"
#include "ft_device.cuh"
#include "scene_build.h"

using ftd::DevNode;
using ftd::F3;
using ftd::f3;
using ftd::Info;

namespace {

constexpr float kInf = __builtin_huge_valf();

struct DevLeaf {
  float bmin[3], bmax[3];
  int32_t kind, node, first, count;
};
struct DevBvhNode {
  float bmin[3], bmax[3];
  int32_t lhs, rhs, leaf, pad;
};
struct DevUrTree {
  float r;
  int32_t n_prims, prim_first, bvh_root, inner_root, depth, fallback_first, fallback_count;
  float gmin[3];
  float cell, inv_cell;
  int32_t dims[3];
  int32_t cell_first, pad;
};
struct DevUrBvh {
  float bmin[3], bmax[3];
  int32_t left, right, prim_begin, prim_count;
};
struct DevUrInner {
  int32_t child[2];
  int32_t lo, hi;
};
static_assert(sizeof(DevLeaf) == sizeof(ftgpu::HostLeaf), "leaf layout");
static_assert(sizeof(DevBvhNode) == sizeof(ftgpu::HostBvhNode), "bvh layout");
static_assert(sizeof(DevUrTree) == sizeof(ftgpu::HostUrTree), "urtree layout");
static_assert(sizeof(DevUrBvh) == sizeof(ftgpu::HostUrBvh), "urbvh layout");
static_assert(sizeof(DevUrInner) == sizeof(ftgpu::HostUrInner), "urinner layout");

struct DevScene {
  const DevNode* __restrict__ nodes;
  const DevLeaf* __restrict__ leaves;
  const DevBvhNode* __restrict__ bvh;
  const uint32_t* __restrict__ gops;
  const DevUrTree* __restrict__ urtrees;
  const DevUrBvh* __restrict__ ur_bvh;
  const int32_t* __restrict__ ur_bvh_prims;
  const int32_t* __restrict__ ur_prims;
  const DevUrInner* __restrict__ ur_inner;
  const uint32_t* __restrict__ ur_cell_offsets;
  const int32_t* __restrict__ ur_cell_prims;
  const ft_program* __restrict__ programs;
  const ft_instr* __restrict__ instrs;
  const ft_material* __restrict__ materials;
  const ft_light* __restrict__ lights;
  const int32_t* __restrict__ node_op_begin;
  const int32_t* __restrict__ node_op_end;
  const int32_t* __restrict__ ur_inner_blend;
  int32_t n_materials, n_lights, env_program;
  int32_t bvh_root;
  float smin[3], smax[3];
};

struct RayParams {
  float origin[3], fwd[3], right[3], up[3];
  float tan_fov, aspect;
  uint32_t width, height, aa, grid, max_steps;
  float max_dist, eps, step_scale;
  uint32_t tiles_x;
  uint32_t tile_w, tile_h;  // pixels per work tile (rays of a tile are consecutive work items)
  uint32_t refill;          // idle lanes that make a warp of the persistent march refill
  uint64_t n_items;
};


// Per-thread work counters (only compiled into the statistics variant).
struct Counters {
  unsigned long long evals, prims, boxes, hook_instrs, steps, far_steps, fetches;
};
constexpr int kNumCounters = 7;

template <bool kStats>
struct Ctx {
  Counters c;
  __device__ void eval() {
    if (kStats) ++c.evals;
  }
  __device__ void prim() {
    if (kStats) ++c.prims;
  }
  __device__ void box() {
    if (kStats) ++c.boxes;
  }
  __device__ void step() {
    if (kStats) ++c.steps;
  }
  __device__ void far_step() {
    if (kStats) ++c.far_steps;
  }
  __device__ void fetch() {
    if (kStats) ++c.fetches;
  }
  __device__ unsigned long long* hooks() { return kStats ? &c.hook_instrs : nullptr; }
};

__device__ __forceinline__ float node_lb(F3 p, const float* mn, const float* mx) { return ftd::aabb_lb(p, mn, mx); }

// Generic leaf: postfix program over the leaf's node tree (exact).
template <bool kStats>
__device__ __noinline__ Info eval_generic(const DevScene& S, int first, int count, F3 p, Ctx<kStats>& cx) {
  Info vs[ftgpu::kMaxGenericValueStack];
  F3 ps[ftgpu::kMaxGenericPointStack];
  int vsp = 0, psp = 0;
  ps[0] = p;
  for (int k = 0; k < count; ++k) {
    uint32_t w = S.gops[first + k];
    uint32_t op = w >> ftgpu::kGOpShift;
    const DevNode& n = S.nodes[w & ftgpu::kGNodeMask];
    switch (op) {
      case ftgpu::kGPrim:
        cx.prim();
        vs[vsp++] = Info{ftd::prim_distance(n, ps[psp]), n.object_id, n.material_id};
        break;
      case ftgpu::kGDomainPush: {
        F3 q = ftd::to_local(ps[psp], n);
        ps[psp + 1] = ftd::run_program(S.programs[n.program], S.instrs, &q, cx.hooks());
        ++psp;
        break;
      }
      case ftgpu::kGLocalPush:
        ps[psp + 1] = ftd::to_local(ps[psp], n);
        ++psp;
        break;
      case ftgpu::kGPostPop: {
        float d = vs[vsp - 1].d;
        F3 args[2] = {f3(d, d, d), ps[psp]};
        vs[vsp - 1].d = ftd::run_program(S.programs[n.program], S.instrs, args, cx.hooks()).x;
        --psp;
        break;
      }
      case ftgpu::kGNoisePop:
        vs[vsp - 1].d = ftd::apply_noise(ps[psp], vs[vsp - 1].d, n.ival, n.f[0], n.f[1]);
        --psp;
        break;
      case ftgpu::kGPop: --psp; break;
      case ftgpu::kGBinary: {
        Info r = vs[--vsp];
        Info l = vs[--vsp];
        vs[vsp++] = ftd::combine(n.kind, n.f[0], n.f[1], l, r);
        break;
      }
      case ftgpu::kGSlice: {
        F3 q = ps[psp];
        float coord = n.ival == 0 ? q.x : (n.ival == 1 ? q.y : q.z);
        float slab = ftd::rmax(n.f[0] - coord, coord - n.f[1]);
        vs[vsp - 1].d = ftd::rmax(vs[vsp - 1].d, slab);
        break;
      }
      case ftgpu::kGSmooth: vs[vsp - 1].d -= n.f[0] * 0.1f; break;
    }
  }
  return vs[0];
}

// union_round tree of primitives with a single radius r.
//
// For every primitive with exact distance >= r each union_round it feeds is
// in its min(a, b) regime (op_union_round, R:6024-6029), so the tree value
// only depends on the set N of primitives closer than r:
//   * N empty: the value is the minimum primitive distance, exactly;
//   * otherwise: evaluate the tree restricted to subtrees containing an
//     N-primitive, treating every other subtree as +inf, which reproduces
//     op_union_round(a, b, r) bit for bit for any b >= r.
// N is gathered through a BVH over the tree's primitives with pruning bound
// max(r, min(best so far, cutoff)); primitive AABBs bound their distances from
// below, so no primitive that can change the result is skipped.
__device__ __noinline__ Info ur_fold(const DevScene& S, const DevUrTree& t, const int* near_pos,
                                     const Info* near_info, int nn);

template <bool kStats>
__device__ __forceinline__ Info eval_urtree(const DevScene& S, const DevUrTree& t, F3 p, float cutoff,
                                            Ctx<kStats>& cx) {
  const float r = t.r;
  int near_pos[ftgpu::kUrNear];
  Info near_info[ftgpu::kUrNear];
  int nn = 0;
  bool overflow = false;
  Info best{kInf, 0u, 0u};
  // Test one primitive against the running bound; evaluate it if it can
  // matter and record it in the near set when closer than r.
  auto consider = [&](int pos) {
    const DevNode& pn = S.nodes[S.ur_prims[t.prim_first + pos]];
    cx.box();
    float lim = ftd::rmax(r, fminf(best.d, cutoff));
    if (node_lb(p, pn.bmin, pn.bmax) >= lim) return;
    cx.prim();
    float d = ftd::prim_distance(pn, p);
    if (d < best.d) best = Info{d, pn.object_id, pn.material_id};
    if (d < r) {
      if (nn < ftgpu::kUrNear) {
        near_pos[nn] = pos;
        near_info[nn] = Info{d, pn.object_id, pn.material_id};
        ++nn;
      } else {
        overflow = true;
      }
    }
  };
  int stack[48];
  int sp = 0;
  // Inside the candidate grid one cell list replaces the BVH walk.
  float gx = (p.x - t.gmin[0]) * t.inv_cell, gy = (p.y - t.gmin[1]) * t.inv_cell, gz = (p.z - t.gmin[2]) * t.inv_cell;
  if (t.dims[0] > 0 && gx >= 0.0f && gy >= 0.0f && gz >= 0.0f && gx < (float)t.dims[0] && gy < (float)t.dims[1] &&
      gz < (float)t.dims[2]) {
    int ix = min((int)gx, t.dims[0] - 1), iy = min((int)gy, t.dims[1] - 1), iz = min((int)gz, t.dims[2] - 1);
    int cell = t.cell_first + ix + t.dims[0] * (iy + t.dims[1] * iz);
    uint32_t beg = S.ur_cell_offsets[cell], end = S.ur_cell_offsets[cell + 1];
    for (uint32_t k = beg; k < end; ++k) consider(S.ur_cell_prims[k]);
  } else {
    stack[sp++] = t.bvh_root;
  }
  while (sp > 0) {
    const DevUrBvh& bn = S.ur_bvh[stack[--sp]];
    cx.box();
    float bound = ftd::rmax(r, fminf(best.d, cutoff));
    if (node_lb(p, bn.bmin, bn.bmax) >= bound) continue;
    if (bn.prim_count > 0) {
      for (int k = 0; k < bn.prim_count; ++k) consider(S.ur_bvh_prims[bn.prim_begin + k]);
      continue;
    }
    const DevUrBvh& L = S.ur_bvh[bn.left];
    const DevUrBvh& R = S.ur_bvh[bn.right];
    float ll = node_lb(p, L.bmin, L.bmax), rl = node_lb(p, R.bmin, R.bmax);
    if (sp + 2 > 48) {
      overflow = true;
      break;
    }
    if (ll <= rl) {
      stack[sp++] = bn.right;
      stack[sp++] = bn.left;
    } else {
      stack[sp++] = bn.left;
      stack[sp++] = bn.right;
    }
  }
  if (overflow) return eval_generic(S, t.fallback_first, t.fallback_count, p, cx);
  if (nn == 0) return best;
  return ur_fold(S, t, near_pos, near_info, nn);
}

// Restricted union_round fold over the subtrees holding near primitives
// (out of line: only points within r of a primitive take it).
__device__ __noinline__ Info ur_fold(const DevScene& S, const DevUrTree& t, const int* near_pos,
                                     const Info* near_info, int nn) {
  const float r = t.r;
  // Frames hold partially combined inner nodes.
  struct Frame {
    int inner, stage;
    Info slot[2];
  };
  Frame fr[ftgpu::kMaxUrDepth + 1];
  int fp = 0;
  fr[0].inner = t.inner_root;
  fr[0].stage = 0;
  for (;;) {
    Frame& F = fr[fp];
    if (F.stage < 2) {
      const DevUrInner& in = S.ur_inner[F.inner];
      int c = in.child[F.stage];
      if (c < 0) {
        int pos = -c - 1;
        Info v{kInf, 0u, 0u};
        for (int k = 0; k < nn; ++k)
          if (near_pos[k] == pos) v = near_info[k];
        F.slot[F.stage++] = v;
        continue;
      }
      const DevUrInner& ci = S.ur_inner[c];
      bool has = false;
      for (int k = 0; k < nn; ++k) has |= (near_pos[k] >= ci.lo && near_pos[k] < ci.hi);
      if (!has) {
        F.slot[F.stage++] = Info{kInf, 0u, 0u};
        continue;
      }
      ++F.stage;
      ++fp;
      fr[fp].inner = c;
      fr[fp].stage = 0;
      continue;
    }
    Info res = ftd::combine(FT_NODE_UNION_ROUND, r, 0.0f, F.slot[0], F.slot[1]);
    if (fp == 0) return res;
    --fp;
    fr[fp].slot[fr[fp].stage - 1] = res;
  }
}

template <bool kStats>
__device__ __forceinline__ Info eval_leaf(const DevScene& S, const DevLeaf& lf, F3 p, float cutoff, Ctx<kStats>& cx) {
  if (lf.kind == ftgpu::kLeafPrim) {
    const DevNode& n = S.nodes[lf.node];
    cx.prim();
    return Info{ftd::prim_distance(n, p), n.object_id, n.material_id};
  }
  if (lf.kind == ftgpu::kLeafUrTree) return eval_urtree(S, S.urtrees[lf.first], p, cutoff, cx);
  return eval_generic(S, lf.first, lf.count, p, cx);
}

// Accelerator::distance_info over the leaf BVH (bvh_distance_info,
// R:743-786): nearest-first, a node is skipped when its box bound exceeds the
// best distance so far, a later leaf replaces the result only when strictly
// closer.
template <bool kStats>
__device__ __noinline__ Info scene_distance_bvh(const DevScene& S, F3 p, Ctx<kStats>& cx) {
  float best = kInf;
  Info cur{kInf, 0u, 0u};
  int stack[64];
  float stack_lb[64];
  int sp = 0;
  stack[sp] = S.bvh_root;
  stack_lb[sp] = node_lb(p, S.bvh[S.bvh_root].bmin, S.bvh[S.bvh_root].bmax);
  ++sp;
  cx.box();
  while (sp > 0) {
    --sp;
    int ni = stack[sp];
    if (stack_lb[sp] > best) continue;
    const DevBvhNode& n = S.bvh[ni];
    if (n.leaf >= 0) {
      Info in = eval_leaf(S, S.leaves[n.leaf], p, best, cx);
      if (in.d < best) {
        best = in.d;
        cur = in;
      }
      continue;
    }
    const DevBvhNode& L = S.bvh[n.lhs];
    const DevBvhNode& R = S.bvh[n.rhs];
    float ll = node_lb(p, L.bmin, L.bmax), rl = node_lb(p, R.bmin, R.bmax);
    cx.box();
    cx.box();
    if (sp + 2 > 64) break;  // depth is bounded by the median-split build
    if (ll <= rl) {
      stack[sp] = n.rhs; stack_lb[sp] = rl; ++sp;
      stack[sp] = n.lhs; stack_lb[sp] = ll; ++sp;
    } else {
      stack[sp] = n.lhs; stack_lb[sp] = ll; ++sp;
      stack[sp] = n.rhs; stack_lb[sp] = rl; ++sp;
    }
  }
  return cur;
}

// Same traversal, with the one- and two-leaf BVHs (a single object, or a
// ground plus one composite object) walked without a stack.
template <bool kStats>
__device__ __forceinline__ Info scene_distance_inl(const DevScene& S, F3 p, Ctx<kStats>& cx) {
  cx.eval();
  const DevBvhNode& root = S.bvh[S.bvh_root];
  if (root.leaf >= 0) return eval_leaf(S, S.leaves[root.leaf], p, kInf, cx);
  const DevBvhNode& L = S.bvh[root.lhs];
  const DevBvhNode& R = S.bvh[root.rhs];
  if (L.leaf < 0 || R.leaf < 0) return scene_distance_bvh(S, p, cx);
  cx.box();
  cx.box();
  float ll = node_lb(p, L.bmin, L.bmax), rl = node_lb(p, R.bmin, R.bmax);
  const bool lfirst = ll <= rl;
  const DevLeaf& first = S.leaves[lfirst ? L.leaf : R.leaf];
  const DevLeaf& second = S.leaves[lfirst ? R.leaf : L.leaf];
  Info cur = eval_leaf(S, first, p, kInf, cx);
  if ((lfirst ? rl : ll) <= cur.d) {
    Info in = eval_leaf(S, second, p, cur.d, cx);
    if (in.d < cur.d) cur = in;
  }
  return cur;
}

template <bool kStats>
__device__ __noinline__ Info scene_distance(const DevScene& S, F3 p, Ctx<kStats>& cx) {
  return scene_distance_inl(S, p, cx);
}

template <bool kStats>
__device__ __forceinline__ float scene_d(const DevScene& S, F3 p, Ctx<kStats>& cx) {
  return scene_distance(S, p, cx).d;
}

// The same leaf-BVH walk reporting the winning hard-union leaf: the leaf whose
// subtree the reference's Union walks descend into when resolving a hit's
// normal and material (R:4471-4478, R:6995-7002).
template <bool kStats>
__device__ __noinline__ Info scene_distance_leaf(const DevScene& S, F3 p, int* leaf, Ctx<kStats>& cx) {
  cx.eval();
  float best = kInf;
  Info cur{kInf, 0u, 0u};
  *leaf = 0;
  int stack[64];
  float stack_lb[64];
  int sp = 0;
  stack[sp] = S.bvh_root;
  stack_lb[sp] = node_lb(p, S.bvh[S.bvh_root].bmin, S.bvh[S.bvh_root].bmax);
  ++sp;
  while (sp > 0) {
    --sp;
    int ni = stack[sp];
    if (stack_lb[sp] > best) continue;
    const DevBvhNode& n = S.bvh[ni];
    if (n.leaf >= 0) {
      Info in = eval_leaf(S, S.leaves[n.leaf], p, best, cx);
      if (in.d < best) {
        best = in.d;
        cur = in;
        *leaf = n.leaf;
      }
      continue;
    }
    float ll = node_lb(p, S.bvh[n.lhs].bmin, S.bvh[n.lhs].bmax), rl = node_lb(p, S.bvh[n.rhs].bmin, S.bvh[n.rhs].bmax);
    if (sp + 2 > 64) break;
    if (ll <= rl) {
      stack[sp] = n.rhs; stack_lb[sp] = rl; ++sp;
      stack[sp] = n.lhs; stack_lb[sp] = ll; ++sp;
    } else {
      stack[sp] = n.lhs; stack_lb[sp] = ll; ++sp;
      stack[sp] = n.rhs; stack_lb[sp] = rl; ++sp;
    }
  }
  return cur;
}

// ray_aabb_intersection (R:4141-4173)
__device__ bool ray_aabb(F3 o, F3 d, const float* mn, const float* mx, float* t0o, float* t1o) {
  float tmin = -kInf, tmax = kInf;
  float os[3] = {o.x, o.y, o.z}, ds[3] = {d.x, d.y, d.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (fabsf(ds[k]) <= 1.0e-8f) {
      if (os[k] < mn[k] || os[k] > mx[k]) return false;
      continue;
    }
    float inv = 1.0f / ds[k];
    float t0 = (mn[k] - os[k]) * inv, t1 = (mx[k] - os[k]) * inv;
    if (t0 > t1) {
      float tt = t0;
      t0 = t1;
      t1 = tt;
    }
    tmin = fmaxf(tmin, t0);
    tmax = fminf(tmax, t1);
    if (tmax < tmin) return false;
  }
  *t0o = tmin;
  *t1o = tmax;
  return true;
}

struct HitOut {
  float t;
  uint32_t mat;
  bool hit;
  F3 normal;
};

template <bool kStats>
__device__ HitOut march(const DevScene& S, const RayParams& P, F3 o, F3 d, bool want_normal, Ctx<kStats>& cx) {
  HitOut h{0.0f, 0u, false, f3(0.0f, 0.0f, 0.0f)};
  float t0, t1;
  if (!ray_aabb(o, d, S.smin, S.smax, &t0, &t1)) return h;
  float max_t = fminf(P.max_dist, t1);
  float traveled = fmaxf(0.0f, fmaxf(t0, 0.0f));
  float prev = traveled;
  const float eps = P.eps;
  const float scale = ftd::rclamp(P.step_scale, 0.05f, 1.0f);
  const float min_step = fmaxf(eps * 0.5f, 1.0e-5f);
  for (uint32_t s = 0; s < P.max_steps; ++s) {
    if (traveled > max_t) return h;
    cx.step();
    Info info = scene_distance(S, o + d * traveled, cx);
    if (fabsf(info.d) < eps) {
      float lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        float mid = 0.5f * (lo + hi);
        float dm = fabsf(scene_d(S, o + d * mid, cx));
        if (dm < eps) hi = mid;
        else lo = mid;
      }
      F3 pos = o + d * hi;
      if (want_normal) {
        // estimate_normal (R:4202-4215)
        float e = fmaxf(eps * 4.0f, 1.0e-5f);
        float dx = scene_d(S, f3(pos.x + e, pos.y, pos.z), cx) - scene_d(S, f3(pos.x - e, pos.y, pos.z), cx);
        float dy = scene_d(S, f3(pos.x, pos.y + e, pos.z), cx) - scene_d(S, f3(pos.x, pos.y - e, pos.z), cx);
        float dz = scene_d(S, f3(pos.x, pos.y, pos.z + e), cx) - scene_d(S, f3(pos.x, pos.y, pos.z - e), cx);
        F3 nn = f3(dx, dy, dz);
        h.normal = ftd::len3(nn) > 1.0e-8f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      }
      Info fin = scene_distance(S, pos, cx);
      h.t = hi;
      h.mat = fin.mat;
      h.hit = true;
      return h;
    }
    prev = traveled;
    traveled += fmaxf(fabsf(info.d) * scale, min_step);
  }
  return h;
}

__device__ __forceinline__ void item_coords(const RayParams& P, uint64_t i, uint32_t* px, uint32_t* py, uint32_t* s) {
  uint32_t per_tile = P.tile_w * P.tile_h * P.aa;
  uint64_t tile = i / per_tile;
  uint32_t k = static_cast<uint32_t>(i - tile * per_tile);
  *s = k % P.aa;
  uint32_t j = k / P.aa;
  *px = static_cast<uint32_t>(tile % P.tiles_x) * P.tile_w + j % P.tile_w;
  *py = static_cast<uint32_t>(tile / P.tiles_x) * P.tile_h + j / P.tile_w;
}

#include "ft_bricks.cuh"

// Many renders in one launch: per-item scene, parameters and brick cache, and
// the prefix sums that map a global work item to (item, local work item) and
// an item's outputs into the concatenated output arrays.
struct BatchView {
  const DevScene* scenes;
  const RayParams* params;
  const DevBricks* bricks;
  const uint64_t* ray_first;  // n_items + 1 entries
  const uint64_t* out_first;  // first output sample of each item
  uint32_t n_items;
  uint64_t n_rays;
};

// Item holding global work item `g` (ray_first is sorted; ray_first[0] = 0).
__device__ __forceinline__ uint32_t batch_item(const BatchView& V, uint64_t g) {
  uint32_t lo = 0, hi = V.n_items;  // ray_first[lo] <= g < ray_first[hi]
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&V.ray_first[mid]) <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <bool kStats>
__global__ void __launch_bounds__(128) march_depth_kernel(DevScene S, RayParams P, float* __restrict__ t_out,
                                                          uint8_t* __restrict__ mask_out,
                                                          uint32_t* __restrict__ mat_out,
                                                          float* __restrict__ normal_out,
                                                          unsigned long long* __restrict__ stats) {
  uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  Ctx<kStats> cx;
  cx.c = Counters{};
  bool active = i < P.n_items;
  uint32_t px = 0, py = 0, s = 0;
  if (active) {
    item_coords(P, i, &px, &py, &s);
    active = px < P.width && py < P.height;
  }
  if (active) {
    // pixel_sample_offsets (R:4838-4854) and the NDC map of render_depth_tile.
    float sx = (static_cast<float>(s % P.grid) + 0.5f) / static_cast<float>(P.grid);
    float sy = (static_cast<float>(s / P.grid) + 0.5f) / static_cast<float>(P.grid);
    float ndc_x = ((static_cast<float>(px) + sx) / static_cast<float>(P.width)) * 2.0f - 1.0f;
    float ndc_y = 1.0f - ((static_cast<float>(py) + sy) / static_cast<float>(P.height)) * 2.0f;
    ndc_x *= P.aspect;
    F3 fwd = f3(P.fwd[0], P.fwd[1], P.fwd[2]), rt = f3(P.right[0], P.right[1], P.right[2]);
    F3 up = f3(P.up[0], P.up[1], P.up[2]);
    F3 dir = ftd::normalize3(fwd + rt * (ndc_x * P.tan_fov) + up * (ndc_y * P.tan_fov));
    dir = ftd::normalize3(dir);
    F3 o = f3(P.origin[0], P.origin[1], P.origin[2]);
    HitOut h = march(S, P, o, dir, normal_out != nullptr, cx);
    size_t idx = (static_cast<size_t>(py) * P.width + px) * P.aa + s;
    t_out[idx] = h.hit ? h.t : 0.0f;
    mask_out[idx] = h.hit ? 1 : 0;
    if (mat_out) mat_out[idx] = h.hit ? h.mat : 0u;
    if (normal_out) {
      normal_out[3 * idx] = h.normal.x;
      normal_out[3 * idx + 1] = h.normal.y;
      normal_out[3 * idx + 2] = h.normal.z;
    }
  }
  if (kStats) {
    unsigned long long v[5] = {cx.c.evals, cx.c.prims, cx.c.boxes, cx.c.hook_instrs, cx.c.steps};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      unsigned long long x = v[k];
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      if ((threadIdx.x & 31) == 0 && x) atomicAdd(&stats[k], x);
    }
  }
}

// Primary ray of work item i (pixel_sample_offsets R:4838-4854, NDC map of
// render_depth_tile R:3951-3955, generate_ray render_api.rs:132-144 and the
// second normalisation of the tile loop).
__device__ __forceinline__ bool item_ray(const RayParams& P, uint64_t i, F3* dir, size_t* out_idx) {
  uint32_t px, py, s;
  item_coords(P, i, &px, &py, &s);
  if (px >= P.width || py >= P.height) return false;
  float sx = (static_cast<float>(s % P.grid) + 0.5f) / static_cast<float>(P.grid);
  float sy = (static_cast<float>(s / P.grid) + 0.5f) / static_cast<float>(P.grid);
  float ndc_x = ((static_cast<float>(px) + sx) / static_cast<float>(P.width)) * 2.0f - 1.0f;
  float ndc_y = 1.0f - ((static_cast<float>(py) + sy) / static_cast<float>(P.height)) * 2.0f;
  ndc_x *= P.aspect;
  F3 fwd = f3(P.fwd[0], P.fwd[1], P.fwd[2]), rt = f3(P.right[0], P.right[1], P.right[2]);
  F3 up = f3(P.up[0], P.up[1], P.up[2]);
  F3 d = ftd::normalize3(fwd + rt * (ndc_x * P.tan_fov) + up * (ndc_y * P.tan_fov));
  *dir = ftd::normalize3(d);
  *out_idx = (static_cast<size_t>(py) * P.width + px) * P.aa + s;
  return true;
}

// Persistent march with per-lane state machines.
//
// Every loop iteration performs exactly one scene distance evaluation per
// live lane, whatever the lane is doing: a march step (R:4100-4137), one of
// the ten bisection steps (refine_hit_distance, R:4180-4200), one of the six
// estimate_normal taps (R:4202-4215) or the final material lookup.  Lanes
// whose ray finished pick up the next work item from a global counter once a
// quarter of the warp is idle, so divergent march lengths do not leave lanes
// idle for the rest of the warp's life.  The sequence of evaluation points of
// each ray is exactly the reference's.
//
// With kBricks (the FP16 precision form) a ray starts in the far-field phase:
// up to far_batch steps per iteration on the brick lower bound b (one texture
// fetch each), stepping by b - band/2 so the exact distance stays above band/2,
// until b < band or the ray leaves the brick region (each far-field step counts
// as one step against max_steps).  It then continues from that point with the
// plain method's exact FP32 march (same step rule), and goes back to the far
// field whenever an exact step finds
// |d| > band_exit.  At the hit the eps-shell crossing between the last two
// exact points is found by secant steps on the exact distance (each verified
// by an exact evaluation) instead of ten bisections, and the material comes
// from the accepted point's evaluation; the normal is the plain method's.
enum Phase : int { kMarch = 0, kRefine = 1, kNormal = 2, kFinal = 3, kFar = 4, kSecant = 5 };

//
// With kBatch the launch serves many renders: each lane carries the index of
// the item its ray belongs to and reads that item's scene, parameters and
// brick cache from the batch tables (otherwise they are the kernel's own
// parameters); outputs are the concatenated arrays of all items.
template <bool kStats, bool kBricks, bool kBatch>
__global__ void __launch_bounds__(128) march_depth_persistent(DevScene S0, RayParams P0, DevBricks B0, BatchView V,
                                                              float* __restrict__ t_out,
                                                              uint8_t* __restrict__ mask_out,
                                                              uint32_t* __restrict__ mat_out,
                                                              float* __restrict__ normal_out,
                                                              unsigned long long* __restrict__ stats,
                                                              unsigned long long* __restrict__ next_item) {
  const unsigned lane = threadIdx.x & 31u;
  const bool want_normal = normal_out != nullptr;
  const uint64_t n_work = kBatch ? V.n_rays : P0.n_items;
  const unsigned refill = kBatch ? V.params[0].refill : P0.refill;
  Ctx<kStats> cx;
  cx.c = Counters{};

  bool live = false;
  bool queue_done = false;
  size_t idx = 0;
  uint32_t item_of_lane = 0;
  // per-ray constants (per item with kBatch)
  F3 o = f3(P0.origin[0], P0.origin[1], P0.origin[2]);
  float eps = P0.eps;
  float scale = ftd::rclamp(P0.step_scale, 0.05f, 1.0f);
  float min_step = fmaxf(eps * 0.5f, 1.0e-5f);
  float ne = fmaxf(eps * 4.0f, 1.0e-5f);
  F3 d = f3(0.0f, 0.0f, 0.0f), pos = f3(0.0f, 0.0f, 0.0f);
  float traveled = 0.0f, prev = 0.0f, max_t = 0.0f, lo = 0.0f, hi = 0.0f;
  float nx = 0.0f, ny = 0.0f, nz = 0.0f;  // estimate_normal differences
  uint32_t steps = 0;
  int phase = kMarch, k = 0;
  // precision form: exact distance at `prev` (< 0: unknown), secant bracket
  // values, material of the accepted hit point
  float dprev = -1.0f, dlo = 0.0f, dhi = 0.0f;
  uint32_t hit_mat = 0u;
  bool mat_known = false;
  auto write_miss = [&]() {
    live = false;
    t_out[idx] = 0.0f;
    mask_out[idx] = 0;
    if (mat_out) mat_out[idx] = 0u;
    if (normal_out) {
      normal_out[3 * idx] = 0.0f;
      normal_out[3 * idx + 1] = 0.0f;
      normal_out[3 * idx + 2] = 0.0f;
    }
  };
  auto write_hit = [&](uint32_t mat) {
    live = false;
    t_out[idx] = hi;
    mask_out[idx] = 1;
    if (mat_out) mat_out[idx] = mat;
    if (normal_out) {
      F3 nn = f3(nx, ny, nz);
      F3 nr = ftd::len3(nn) > 1.0e-8f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      normal_out[3 * idx] = nr.x;
      normal_out[3 * idx + 1] = nr.y;
      normal_out[3 * idx + 2] = nr.z;
    }
  };

  for (;;) {
    // Refill idle lanes when enough of the warp is idle (or all of it).
    unsigned idle = __ballot_sync(0xffffffffu, !live);
    if (!queue_done && (__popc(idle) >= refill || idle == 0xffffffffu)) {
      unsigned n = __popc(idle);
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(next_item, static_cast<unsigned long long>(n));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= n_work) queue_done = true;
      if (!live) {
        unsigned rank = __popc(idle & ((1u << lane) - 1u));
        uint64_t item = base + rank;
        bool got = false;
        if (item < n_work) {
          if (kBatch) {
            item_of_lane = batch_item(V, item);
            const RayParams& Pi = V.params[item_of_lane];
            got = item_ray(Pi, item - V.ray_first[item_of_lane], &d, &idx);
            idx += V.out_first[item_of_lane];
            o = f3(Pi.origin[0], Pi.origin[1], Pi.origin[2]);
            eps = Pi.eps;
            scale = ftd::rclamp(Pi.step_scale, 0.05f, 1.0f);
            min_step = fmaxf(eps * 0.5f, 1.0e-5f);
            ne = fmaxf(eps * 4.0f, 1.0e-5f);
          } else {
            got = item_ray(P0, item, &d, &idx);
          }
        }
        const DevScene& S = kBatch ? V.scenes[item_of_lane] : S0;
        const RayParams& P = kBatch ? V.params[item_of_lane] : P0;
        if (got) {
          float t0, t1;
          bool inside = ray_aabb(o, d, S.smin, S.smax, &t0, &t1);
          traveled = fmaxf(0.0f, fmaxf(t0, 0.0f));
          max_t = fminf(P.max_dist, t1);
          if (inside && P.max_steps > 0 && !(traveled > max_t)) {
            live = true;
            prev = traveled;
            steps = 0;
            phase = kBricks ? kFar : kMarch;
            dprev = -1.0f;
            mat_known = false;
          } else {
            write_miss();
          }
        }
      }
    }
    if (__ballot_sync(0xffffffffu, live) == 0u) {
      if (queue_done) break;
      continue;
    }
    if (!live) continue;
    const DevScene& S = kBatch ? V.scenes[item_of_lane] : S0;
    const RayParams& P = kBatch ? V.params[item_of_lane] : P0;
    const DevBricks& B = kBatch ? V.bricks[item_of_lane] : B0;

    if (kBricks && phase == kFar) {
      bool exact = false, missed = false;
      for (int f = 0; f < B.far_batch; ++f) {
        float b;
        if (!far_bound(S, B, o + d * traveled, &b, cx) || b < B.band) {
          exact = true;
          break;
        }
        traveled += b - 0.5f * B.band;
        cx.far_step();
        ++steps;  // a far-field step is one step of the march
        if (steps >= P.max_steps || traveled > max_t) {
          missed = true;
          break;
        }
      }
      if (missed) {
        write_miss();
        continue;
      }
      if (!exact) continue;
      phase = kMarch;  // exact evaluation at `traveled` in this iteration
      prev = traveled;
      dprev = -1.0f;
    }

    // The point this lane evaluates in this iteration.
    F3 q;
    float mid = 0.0f;
    if (phase == kMarch) {
      q = o + d * traveled;
      cx.step();
    } else if (phase == kRefine) {
      mid = 0.5f * (lo + hi);
      q = o + d * mid;
    } else if (kBricks && phase == kSecant) {
      // crossing of d = eps on the line through (lo, dlo) and (hi, dhi)
      mid = lo + (dlo - eps) / (dlo - dhi) * (hi - lo);
      mid = fminf(fmaxf(mid, lo), hi);
      q = o + d * mid;
    } else if (phase == kNormal) {
      float sgn = (k & 1) ? -ne : ne;
      q = pos;
      if (k < 2) q.x += sgn;
      else if (k < 4) q.y += sgn;
      else q.z += sgn;
    } else {
      q = pos;
    }
    Info info = scene_distance_inl(S, q, cx);

    if (phase == kMarch) {
      if (fabsf(info.d) < eps) {
        lo = prev;
        hi = traveled;
        k = 0;
        if (kBricks && dprev >= eps) {
          phase = kSecant;
          dlo = dprev;
          dhi = info.d;
          hit_mat = info.mat;
        } else {
          phase = kRefine;
        }
      } else {
        prev = traveled;
        if (kBricks) dprev = info.d;
        traveled += fmaxf(fabsf(info.d) * scale, min_step);
        ++steps;
        if (kBricks && fabsf(info.d) > B.band_exit) phase = kFar;
        if (steps >= P.max_steps || traveled > max_t) write_miss();
      }
    } else if (kBricks && phase == kSecant) {
      bool accept = true;
      if (fabsf(info.d) < eps) {
        hi = mid;
        hit_mat = info.mat;
      } else if (info.d > 0.0f && ++k < 3) {
        lo = mid;
        dlo = info.d;
        accept = false;
      }
      if (accept) {
        pos = o + d * hi;
        mat_known = true;
        k = 0;
        if (want_normal) phase = kNormal;
        else write_hit(hit_mat);
      }
    } else if (phase == kRefine) {
      if (fabsf(info.d) < eps) hi = mid;
      else lo = mid;
      if (++k == 10) {
        pos = o + d * hi;
        phase = want_normal ? kNormal : kFinal;
        k = 0;
      }
    } else if (phase == kNormal) {
      // dx = d(p + e x) - d(p - e x), one subtraction as in the reference
      if (k == 0) nx = info.d;
      else if (k == 1) nx = nx - info.d;
      else if (k == 2) ny = info.d;
      else if (k == 3) ny = ny - info.d;
      else if (k == 4) nz = info.d;
      else nz = nz - info.d;
      if (++k == 6) {
        if (kBricks && mat_known) write_hit(hit_mat);
        else phase = kFinal;
      }
    } else {
      write_hit(info.mat);
    }
  }
  if (kStats) {
    unsigned long long v[kNumCounters] = {cx.c.evals, cx.c.prims,     cx.c.boxes,  cx.c.hook_instrs,
                                          cx.c.steps, cx.c.far_steps, cx.c.fetches};
#pragma unroll
    for (int j = 0; j < kNumCounters; ++j) {
      unsigned long long x = v[j];
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      if (lane == 0 && x) atomicAdd(&stats[j], x);
    }
  }
}

// Depth preview pixels (render_depth_tile R:3931-3971, depth_preview_value
// R:5215-5219, spectrum_to_rgb8 R:5221-5227).
__device__ __forceinline__ float depth_pixel_value(const float* __restrict__ t, const uint8_t* __restrict__ mask,
                                                   size_t first, uint32_t aa, float max_dist) {
  float sum = 0.0f;
  float md = fmaxf(max_dist, 1.0e-6f);
  for (uint32_t s = 0; s < aa; ++s) {
    size_t k = first + s;
    float depth = 0.0f;
    if (mask[k]) {
      float d = ftd::rclamp(t[k] / md, 0.0f, 1.0f);
      float shaped = 1.0f - d;
      depth = shaped * shaped;
    }
    sum += depth;
  }
  return sum * (1.0f / static_cast<float>(aa));
}

// spectrum_to_rgb8 (R:5221-5227): gamma 2.2, clamped, truncated
__device__ __forceinline__ uint8_t gamma_u8(float v) {
  float mapped = fminf(powf(fmaxf(v, 0.0f), 1.0f / 2.2f), 1.0f);
  return static_cast<uint8_t>(mapped * 255.0f);
}

// spectrum_to_rgb8_reinhard (R:5229-5239)
__device__ __forceinline__ uint8_t reinhard_u8(float v) {
  float x = fmaxf(v, 0.0f);
  float t = x / (1.0f + x);
  float mapped = fminf(powf(t, 1.0f / 2.2f), 1.0f);
  return static_cast<uint8_t>(mapped * 255.0f);
}

__global__ void depth_rgb8_kernel(const float* __restrict__ t, const uint8_t* __restrict__ mask, uint32_t n_pixels,
                                  uint32_t aa, float max_dist, uint8_t* __restrict__ rgb) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pixels) return;
  uint8_t g = gamma_u8(depth_pixel_value(t, mask, static_cast<size_t>(i) * aa, aa, max_dist));
  rgb[3 * static_cast<size_t>(i)] = g;
  rgb[3 * static_cast<size_t>(i) + 1] = g;
  rgb[3 * static_cast<size_t>(i) + 2] = g;
}

#include "ft_trace.cuh"

struct TraceHit {
  float t;
  F3 pos, normal;
  uint32_t mat;
  int leaf;
};

// raymarch_hit (R:4091-4139) from min_t, with the six-tap normal and the
// winning leaf of the final evaluation.
template <bool kStats>
__device__ bool march_hit(const DevScene& S, const RayParams& P, F3 o, F3 d, float min_t, TraceHit* h,
                          Ctx<kStats>& cx) {
  float t0, t1;
  if (!ray_aabb(o, d, S.smin, S.smax, &t0, &t1)) return false;
  float max_t = fminf(P.max_dist, t1);
  float traveled = fmaxf(min_t, fmaxf(t0, 0.0f));
  float prev = traveled;
  const float eps = P.eps;
  const float scale = ftd::rclamp(P.step_scale, 0.05f, 1.0f);
  const float min_step = fmaxf(eps * 0.5f, 1.0e-5f);
  for (uint32_t s = 0; s < P.max_steps; ++s) {
    if (traveled > max_t) return false;
    cx.step();
    Info info = scene_distance(S, o + d * traveled, cx);
    if (fabsf(info.d) < eps) {
      float lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        float mid = 0.5f * (lo + hi);
        if (fabsf(scene_d(S, o + d * mid, cx)) < eps) hi = mid;
        else lo = mid;
      }
      F3 pos = o + d * hi;
      float e = fmaxf(eps * 4.0f, 1.0e-5f);
      float dx = scene_d(S, f3(pos.x + e, pos.y, pos.z), cx) - scene_d(S, f3(pos.x - e, pos.y, pos.z), cx);
      float dy = scene_d(S, f3(pos.x, pos.y + e, pos.z), cx) - scene_d(S, f3(pos.x, pos.y - e, pos.z), cx);
      float dz = scene_d(S, f3(pos.x, pos.y, pos.z + e), cx) - scene_d(S, f3(pos.x, pos.y, pos.z - e), cx);
      F3 nn = f3(dx, dy, dz);
      h->normal = ftd::len3(nn) > 1.0e-8f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      Info fin = scene_distance_leaf(S, pos, &h->leaf, cx);
      h->t = hi;
      h->pos = pos;
      h->mat = fin.mat;
      return true;
    }
    prev = traveled;
    traveled += fmaxf(fabsf(info.d) * scale, min_step);
  }
  return false;
}

// environment_color (R:4328-4333), falling back to the sum of EnvLight
// radiances (env_radiance, R:4318-4326).
__device__ F3 environment(const DevScene& S, F3 dir) {
  if (S.env_program >= 0) return ftd::run_program(S.programs[S.env_program], S.instrs, &dir, nullptr);
  F3 s = f3(0.0f, 0.0f, 0.0f);
  for (int i = 0; i < S.n_lights; ++i)
    if (S.lights[i].kind == FT_LIGHT_ENV) s = s + f3(S.lights[i].intensity[0], S.lights[i].intensity[1], S.lights[i].intensity[2]);
  return s;
}

// The full Whitted tree of one primary sample (trace_ray_recursive,
// ray.rs:3-222), as a stack of ray jobs carrying their throughput weights.
template <bool kStats>
__device__ __forceinline__ F3 trace_sample(const DevScene& S, const RayParams& P, uint32_t max_depth, F3 dir,
                                           Ctx<kStats>& cx) {
  F3 acc = f3(0.0f, 0.0f, 0.0f);
  {
    const float eps = P.eps;
    RayJob stack[kTraceStack];
    int sp = 0;
    stack[sp++] = RayJob{f3(P.origin[0], P.origin[1], P.origin[2]), dir, f3(1.0f, 1.0f, 1.0f), air(), 0};
    while (sp > 0) {
      RayJob J = stack[--sp];
      if (static_cast<uint32_t>(J.depth) >= max_depth) continue;
      float min_t = J.depth == 0 ? 0.0f : eps * 2.0f;  // secondary_min_t (R:4175-4178)
      TraceHit h;
      if (!march_hit(S, P, J.o, J.d, min_t, &h, cx)) {
        acc = acc + mul3(J.w, mul3(environment(S, J.d), transmittance(J.med, P.max_dist)));
        continue;
      }
      Resolved rs;
      resolve_hit(S, h.leaf, h.pos, &rs, cx);
      bool front = ftd::dot3(h.normal, J.d) < 0.0f;
      F3 normal = front ? ftd::normalize3(h.normal) : ftd::normalize3(h.normal * -1.0f);
      F3 shading_n = normal;
      if (rs.ok) shading_n = ftd::normalize3(front ? rs.normal : rs.normal * -1.0f);
      DMat mats[2];
      float ws[2];
      int nm = 0;
      if (rs.ok && rs.split) {
        float tt = clamp01(rs.t);  // lerp_spectrum(a, b, t): a (1 - t) + b t
        if (tt != 1.0f) { mats[nm] = rs.m; ws[nm++] = 1.0f - tt; }
        if (tt != 0.0f) { mats[nm] = rs.mb; ws[nm++] = tt; }
      } else {
        mats[0] = rs.ok ? rs.m : mat_of_id(S, h.mat);
        ws[0] = 1.0f;
        nm = 1;
      }
      F3 att = transmittance(J.med, h.t);
      F3 wo = ftd::normalize3(J.d * -1.0f);
      for (int mi = 0; mi < nm; ++mi) {
        const DMat& mat = mats[mi];
        F3 W = mul3(J.w * ws[mi], att);
        // trace_hit_with_material (ray.rs:41-222)
        const DParams& Pm = dom_params(mat);
        float rough = clamp01(Pm.roughness);
        int model = dom_model(mat);
        float transmission, ior, metallic, clearcoat, specular_strength;
        bool thin;
        F3 spec_color, base_color;
        if (model == FT_MAT_STANDARD) {
          transmission = clamp01(Pm.transmission); ior = ftd::rclamp(Pm.ior, 1.0f, 3.0f); thin = Pm.thin != 0;
          spec_color = Pm.spec_color; base_color = Pm.color; metallic = clamp01(Pm.metallic);
          clearcoat = clamp01(Pm.clearcoat); specular_strength = clamp01(Pm.specular * Pm.specular_weight);
        } else if (model == FT_MAT_LAMBERT) {
          transmission = 0.0f; ior = 1.0f; thin = false; spec_color = f3(0.0f, 0.0f, 0.0f); base_color = Pm.color;
          metallic = 0.0f; clearcoat = 0.0f; specular_strength = 0.0f;
        } else if (model == FT_MAT_METAL) {
          transmission = 0.0f; ior = 1.0f; thin = false; spec_color = Pm.color; base_color = Pm.color;
          metallic = 1.0f; clearcoat = 0.0f; specular_strength = 1.0f;
        } else {
          transmission = 1.0f; ior = ftd::rclamp(Pm.ior, 1.0f, 3.0f); thin = Pm.thin != 0;
          spec_color = f3(1.0f, 1.0f, 1.0f); base_color = Pm.color; metallic = 0.0f; clearcoat = 0.0f;
          specular_strength = 1.0f;
        }
        float eta_i, eta_t, next_ior;
        if (thin) { eta_i = 1.0f; eta_t = 1.0f; next_ior = J.med.ior; }
        else if (front) { eta_i = J.med.ior; eta_t = ior; next_ior = ior; }
        else { eta_i = J.med.ior; eta_t = 1.0f; next_ior = 1.0f; }
        float cosv = fabsf(ftd::dot3(normal, wo));
        float fresnel;
        if (transmission > 1.0e-4f) {
          fresnel = fresnel_dielectric(cosv, eta_i, eta_t);
        } else {
          float f0 = clamp01(f0_from_ior(ior));
          float x = 1.0f - clamp01(cosv);
          float m5 = x * x * x * x * x;
          fresnel = clamp01(f0 + (1.0f - f0) * m5);
        }
        float reflect_w;
        if (transmission > 1.0e-4f) {
          reflect_w = clamp01(fresnel);
        } else {
          float base = metallic > 0.5f ? 1.0f : clamp01(specular_strength);
          reflect_w = clamp01(base * fresnel + metallic * 0.8f + clearcoat * 0.2f);
        }
        float local_w = clamp01((1.0f - transmission) * (1.0f - reflect_w));
        F3 local = shade_color(S, mat, h.pos, normal, shading_n, wo, eps, P.max_dist, cx) * local_w;
        acc = acc + mul3(W, local + mat_emission(mat));
        if (reflect_w > 1.0e-4f && sp < kTraceStack) {
          F3 rd = ftd::normalize3(J.d - normal * (2.0f * ftd::dot3(J.d, normal)));
          F3 ro = offset_origin(h.pos, normal, rd, eps * (1.0f + rough * 6.0f));
          F3 tint = lerp_sp(spec_color, base_color, clamp01(metallic));
          stack[sp++] = RayJob{ro, rd, mul3(W, tint * reflect_w), J.med, J.depth + 1};
        }
        if (transmission > 1.0e-4f && sp < kTraceStack) {
          MediumD next = thin ? J.med : transition(mat, front, J.med);
          next.ior = ftd::rclamp(next_ior, 1.0f, 3.0f);
          F3 td;
          if (refract_dir(J.d, normal, eta_i / eta_t, &td)) {
            F3 to = offset_origin(h.pos, normal, td, eps * (8.0f + rough * 12.0f));
            float tt = clamp01(transmission);
            F3 tint = f3(1.0f - (1.0f - clamp01(base_color.x)) * tt, 1.0f - (1.0f - clamp01(base_color.y)) * tt,
                         1.0f - (1.0f - clamp01(base_color.z)) * tt);
            stack[sp++] = RayJob{to, ftd::normalize3(td), mul3(W, tint * (transmission * (1.0f - fresnel))), next,
                                 J.depth + 1};
          }
        }
      }
    }
  }
  return acc;
}

template <bool kStats>
__device__ __forceinline__ void flush_counters(const Ctx<kStats>& cx, unsigned long long* stats) {
  if (kStats) {
    unsigned long long v[5] = {cx.c.evals, cx.c.prims, cx.c.boxes, cx.c.hook_instrs, cx.c.steps};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      unsigned long long x = v[k];
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      if ((threadIdx.x & 31) == 0 && x) atomicAdd(&stats[k], x);
    }
  }
}

// One thread per (pixel, AA sample).
template <bool kStats>
__global__ void __launch_bounds__(128) trace_kernel(DevScene S, RayParams P, uint32_t max_depth,
                                                    float* __restrict__ sample_rgb,
                                                    unsigned long long* __restrict__ stats) {
  uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  Ctx<kStats> cx;
  cx.c = Counters{};
  F3 dir;
  size_t idx = 0;
  if (i < P.n_items && item_ray(P, i, &dir, &idx)) {
    F3 acc = trace_sample(S, P, max_depth, dir, cx);
    sample_rgb[3 * idx] = acc.x;
    sample_rgb[3 * idx + 1] = acc.y;
    sample_rgb[3 * idx + 2] = acc.z;
  }
  flush_counters(cx, stats);
}

// Batched traces: a persistent grid whose warps take 32 work items at a time
// from a global counter; each item's scene and parameters come from the batch
// tables and its samples land in the concatenated sample array.
__global__ void __launch_bounds__(128) trace_batch_kernel(BatchView V, const uint32_t* __restrict__ max_depth,
                                                          float* __restrict__ sample_rgb,
                                                          unsigned long long* __restrict__ next_item) {
  const unsigned lane = threadIdx.x & 31u;
  Ctx<false> cx;
  cx.c = Counters{};
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(next_item, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= V.n_rays) break;
    uint64_t g = base + lane;
    if (g >= V.n_rays) continue;
    uint32_t it = batch_item(V, g);
    const RayParams& P = V.params[it];
    F3 dir;
    size_t idx = 0;
    if (!item_ray(P, g - V.ray_first[it], &dir, &idx)) continue;
    F3 acc = trace_sample(V.scenes[it], P, max_depth[it], dir, cx);
    idx += V.out_first[it];
    sample_rgb[3 * idx] = acc.x;
    sample_rgb[3 * idx + 1] = acc.y;
    sample_rgb[3 * idx + 2] = acc.z;
  }
}

// AA average per pixel and spectrum_to_rgb8_reinhard (R:3908-3921, R:5229-5239).
__global__ void trace_pixels_kernel(const float* __restrict__ sample_rgb, uint32_t n_pixels, uint32_t aa,
                                    float* __restrict__ rgb_out, uint8_t* __restrict__ rgb8_out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pixels) return;
  float s[3] = {0.0f, 0.0f, 0.0f};
  for (uint32_t k = 0; k < aa; ++k)
    for (int c = 0; c < 3; ++c) s[c] += sample_rgb[(static_cast<size_t>(i) * aa + k) * 3 + c];
  float inv = 1.0f / static_cast<float>(aa);
  for (int c = 0; c < 3; ++c) {
    float v = s[c] * inv;
    if (rgb_out) rgb_out[3 * static_cast<size_t>(i) + c] = v;
    if (rgb8_out) rgb8_out[3 * static_cast<size_t>(i) + c] = reinhard_u8(v);
  }
}

// Pixels of a batch: each item's depth preview or AA-averaged trace in the
// concatenated image arrays (rgb holds the linear value: the preview value of
// depth items, the averaged radiance of traces).
struct BatchPixItem {
  uint64_t pix_first;  // first pixel of the item in the image arrays
  uint64_t out_first;  // first sample in the depth (t, mask) or trace sample arrays
  uint32_t aa, kind;   // kind 0: depth preview, 1: trace
  float max_dist;
  uint32_t pad;
};

__global__ void batch_pixels_kernel(const BatchPixItem* __restrict__ items, uint32_t n_items, uint64_t n_pixels,
                                    const float* __restrict__ t, const uint8_t* __restrict__ mask,
                                    const float* __restrict__ sample_rgb, float* __restrict__ rgb_out,
                                    uint8_t* __restrict__ rgb8_out) {
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n_pixels;
       g += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = n_items;
    while (hi - lo > 1) {
      uint32_t mid = (lo + hi) >> 1;
      if (items[mid].pix_first <= g) lo = mid;
      else hi = mid;
    }
    const BatchPixItem& it = items[lo];
    uint64_t local = g - it.pix_first;
    size_t first = it.out_first + local * it.aa;
    if (it.kind == 0) {
      float v = depth_pixel_value(t, mask, first, it.aa, it.max_dist);
      uint8_t c8 = gamma_u8(v);
      for (int c = 0; c < 3; ++c) {
        rgb_out[3 * g + c] = v;
        rgb8_out[3 * g + c] = c8;
      }
    } else {
      float s[3] = {0.0f, 0.0f, 0.0f};
      for (uint32_t k = 0; k < it.aa; ++k)
        for (int c = 0; c < 3; ++c) s[c] += sample_rgb[(first + k) * 3 + c];
      float inv = 1.0f / static_cast<float>(it.aa);
      for (int c = 0; c < 3; ++c) {
        float v = s[c] * inv;
        rgb_out[3 * g + c] = v;
        rgb8_out[3 * g + c] = reinhard_u8(v);
      }
    }
  }
}

#include "ft_diff.cuh"

// Dependent-FMA chains, 8 per thread, for the FP32 roofline denominator.
__global__ void fma_peak_kernel(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
        x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
    x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
  }
  float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678f) out[0] = s;
}

std::string cuda_msg(cudaError_t e, const char* what) {
  return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

#define FT_CUDA_TRY(expr, what)                                                    \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) return ftcommon::fail(FT_ERR_CUDA, cuda_msg(_e, what)); \
  } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

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
  std::mutex mu;
};

namespace {

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
  d.n_materials = static_cast<int32_t>(im.materials.size());
  d.n_lights = static_cast<int32_t>(im.lights.size());
  d.env_program = im.environment_program;
  d.bvh_root = im.bvh_root;
  std::memcpy(d.smin, im.scene_min, sizeof(d.smin));
  std::memcpy(d.smax, im.scene_max, sizeof(d.smax));
  // [0, 8): statistics counters; [8]: work-item counter of the persistent march
  FT_CUDA_TRY(cudaMalloc(&sc->d_stats, 16 * sizeof(unsigned long long)), "cudaMalloc(stats)");
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
  return P;
}

ft_status launch_depth(ft_scene* sc, const RayParams& P, cudaStream_t st, bool stats, bool bricks, float* t,
                       uint8_t* mask, uint32_t* mat, float* normal) {
  if (bricks && !sc->has_bricks)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "FT_FLAG_FP16_BRICKS needs ft_scene_build_bricks first");
  uint64_t blocks = (P.n_items + 127) / 128;
  if (blocks > 0x7fffffffull) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "image too large");
  int resident = bricks ? sc->persistent_blocks_bricks : sc->persistent_blocks;
  unsigned grid = static_cast<unsigned>(std::min<uint64_t>(blocks, static_cast<uint64_t>(resident)));
  unsigned long long* counter = sc->d_stats + 8;
  unsigned long long* st_ptr = stats ? sc->d_stats : nullptr;
  if (stats)
    FT_CUDA_TRY(cudaMemsetAsync(sc->d_stats, 0, 16 * sizeof(unsigned long long), st), "cudaMemsetAsync(stats)");
  else
    FT_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st), "cudaMemsetAsync(counter)");
  const DevBricks& B = sc->bricks;
  if (stats && bricks)
    march_depth_persistent<true, true, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else if (stats)
    march_depth_persistent<true, false, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else if (bricks)
    march_depth_persistent<false, true, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
  else
    march_depth_persistent<false, false, false><<<grid, 128, 0, st>>>(sc->dev, P, B, BatchView{}, t, mask, mat, normal, st_ptr, counter);
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
  cudaGraphExec_t exec = nullptr;
  ft_batch_tuning tuning{8, 8, 8, 0.0f};
  std::mutex mu;
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
  if (!T.items.empty())
    trace_batch_kernel<<<T.blocks, 128, 0, b->stream>>>(T.view(), T.d_max_depth, b->d_srgb, b->d_counters + 1);
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

ft_status check_tuning(const ft_batch_tuning& t) {
  if (t.tile_w < 1 || t.tile_w > 64 || t.tile_h < 1 || t.tile_h > 64 || t.refill < 1 || t.refill > 32)
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "tile sides must be 1..64 and refill 1..32");
  return FT_OK;
}

}  // namespace

extern "C" {

ft_status ft_scene_create(const ft_scene_desc* desc, ft_scene** out) {
  if (!desc || !out) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "desc and out must be non-null");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return ftcommon::fail(FT_ERR_NO_DEVICE, e != cudaSuccess ? cuda_msg(e, "cudaGetDeviceCount") : "no CUDA device");
  auto* sc = new (std::nothrow) ft_scene();
  if (!sc) return ftcommon::fail(FT_ERR_OUT_OF_MEMORY, "out of host memory");
  std::string err;
  if (!ftgpu::build_scene_image(*desc, &sc->img, &err)) {
    delete sc;
    return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, err);
  }
  FT_CUDA_TRY(cudaGetDevice(&sc->device), "cudaGetDevice");
  ft_status s = upload_scene(sc);
  if (s != FT_OK) {
    ft_scene_destroy(sc);
    return s;
  }
  *out = sc;
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_scene_build_info(const ft_scene_desc* desc, ft_build_info* info) {
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
    }
  }
  info->generic_ops = static_cast<uint32_t>(img.gops.size());
  info->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
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
  cudaSetDevice(prev);
  delete sc;
}

ft_status ft_render_depth(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel, uint32_t aa_samples,
                          float* t_out, uint8_t* mask_out, uint32_t* material_out, float* normal_out,
                          uint8_t* rgb8_out, uint32_t flags, void* stream) {
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
  float* t = dev_ptrs && t_out ? t_out : sc->d_t;
  uint8_t* mask = dev_ptrs && mask_out ? mask_out : sc->d_mask;
  uint32_t* mat = material_out ? (dev_ptrs ? material_out : sc->d_mat) : nullptr;
  float* nrm = normal_out ? (dev_ptrs ? normal_out : sc->d_normal) : nullptr;
  const bool bricks = (flags & FT_FLAG_FP16_BRICKS) != 0;
  if (ft_status s = launch_depth(sc, P, st, false, bricks, t, mask, mat, nrm)) return s;
  if (rgb8_out) {
    uint8_t* rgb = dev_ptrs ? rgb8_out : sc->d_rgb;
    uint32_t np = static_cast<uint32_t>(pixels);
    depth_rgb8_kernel<<<(np + 255) / 256, 256, 0, st>>>(t, mask, np, aa, options->max_dist, rgb);
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
  FT_CUDA_TRY(cudaStreamSynchronize(st), "render");
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_render_depth_preview_noalloc(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                          uint32_t aa_samples, uint8_t* rgb8_out, void* stream) {
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
}

ft_status ft_render_trace(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel, uint32_t aa_samples,
                          uint32_t max_depth, float* rgb_out, uint8_t* rgb8_out, uint32_t flags, void* stream) {
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  if (accel < FT_ACCEL_NAIVE || accel > FT_ACCEL_BRICKS) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "unknown accel mode");
  uint32_t aa = std::max(aa_samples, 1u);
  if (ft_status s = check_options(options, aa)) return s;
  uint32_t depth = std::max(max_depth, 1u);  // RaySettings::max_depth.max(1)
  if (depth > 10) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "max_depth must be <= 10");
  std::lock_guard<std::mutex> lock(sc->mu);
  FT_CUDA_TRY(cudaSetDevice(sc->device), "cudaSetDevice");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool dev_ptrs = (flags & FT_FLAG_DEVICE_POINTERS) != 0;
  size_t pixels = static_cast<size_t>(options->width) * options->height;
  size_t items = pixels * aa;
  if (ft_status s = ensure_buffers(sc, items, pixels)) return s;
  RayParams P = make_params(sc, *options, aa);
  uint64_t blocks = (P.n_items + 127) / 128;
  if (blocks > 0x7fffffffull) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "image too large");
  trace_kernel<false><<<static_cast<unsigned>(blocks), 128, 0, st>>>(sc->dev, P, depth, sc->d_normal, nullptr);
  FT_CUDA_TRY(cudaGetLastError(), "trace_kernel launch");
  float* rgbf = rgb_out ? (dev_ptrs ? rgb_out : sc->d_rgbf) : nullptr;
  uint8_t* rgb8 = rgb8_out ? (dev_ptrs ? rgb8_out : sc->d_rgb) : nullptr;
  uint32_t np = static_cast<uint32_t>(pixels);
  trace_pixels_kernel<<<(np + 255) / 256, 256, 0, st>>>(sc->d_normal, np, aa, rgbf, rgb8);
  FT_CUDA_TRY(cudaGetLastError(), "trace_pixels_kernel launch");
  if (!dev_ptrs) {
    if (rgb_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb_out, rgbf, pixels * 3 * sizeof(float), cudaMemcpyDeviceToHost, st),
                             "copy rgb");
    if (rgb8_out) FT_CUDA_TRY(cudaMemcpyAsync(rgb8_out, rgb8, pixels * 3, cudaMemcpyDeviceToHost, st), "copy rgb8");
  }
  FT_CUDA_TRY(cudaStreamSynchronize(st), "trace");
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_render_trace_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                uint32_t aa_samples, uint32_t max_depth, ft_render_stats* stats) {
  if (!sc || !stats) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene and stats must be non-null");
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
  uint64_t blocks = (P.n_items + 127) / 128;
  FT_CUDA_TRY(cudaMemset(sc->d_stats, 0, 16 * sizeof(unsigned long long)), "cudaMemset(stats)");
  trace_kernel<true><<<static_cast<unsigned>(blocks), 128>>>(sc->dev, P, depth, sc->d_normal, sc->d_stats);
  FT_CUDA_TRY(cudaGetLastError(), "trace_kernel launch");
  unsigned long long h[8] = {0};
  FT_CUDA_TRY(cudaMemcpy(h, sc->d_stats, sizeof(h), cudaMemcpyDeviceToHost), "copy stats");
  std::memset(stats, 0, sizeof(*stats));
  stats->rays = pixels * aa;
  stats->distance_evals = h[0];
  stats->primitive_evals = h[1];
  stats->box_tests = h[2];
  stats->hook_instrs = h[3];
  stats->march_steps = h[4];
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_render_depth_stats(ft_scene* sc, const ft_render_options* options, ft_accel_mode accel,
                                uint32_t aa_samples, uint32_t flags, ft_render_stats* stats) {
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
  if (ft_status s = launch_depth(sc, P, nullptr, true, bricks, sc->d_t, sc->d_mask, nullptr, sc->d_normal)) return s;
  unsigned long long h[8] = {0};
  FT_CUDA_TRY(cudaMemcpy(h, sc->d_stats, sizeof(h), cudaMemcpyDeviceToHost), "copy stats");
  std::memset(stats, 0, sizeof(*stats));
  stats->rays = pixels * aa;
  stats->far_steps = h[5];
  stats->brick_fetches = h[6];
  stats->distance_evals = h[0];
  stats->primitive_evals = h[1];
  stats->box_tests = h[2];
  stats->hook_instrs = h[3];
  stats->march_steps = h[4];
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_scene_build_bricks(ft_scene* sc, const ft_brick_options* options, ft_brick_info* info) {
  if (!sc) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "scene must be non-null");
  ft_brick_options o{};
  if (options) o = *options;
  const float h = o.voxel_size > 0.0f ? o.voxel_size : 0.02f;
  const float band = o.band > 0.0f ? o.band : h;
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
  brick_bound_kernel<<<grid, 128>>>(G, lattice, safety, band + 0.5f * bs, delta, counters, counters + 1);
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
}

ft_status ft_scene_brick_bounds(ft_scene* sc, const float* points, uint32_t n, float* bound_out, float* exact_out) {
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
}

ft_status ft_batch_create(const ft_batch_item* items, uint32_t n, uint32_t flags, ft_batch** out) {
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
      FT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_batch_kernel, 128, 0), "occupancy");
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
  if (ft_status st = batch_apply_tuning(b)) return st;
  *out = guard.release();
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_batch_set_tuning(ft_batch* b, const ft_batch_tuning* t) {
  if (!b || !t) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch and tuning must be non-null");
  if (ft_status st = check_tuning(*t)) return st;
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaStreamSynchronize(b->stream), "batch");
  b->tuning = *t;
  if (ft_status st = batch_apply_tuning(b)) return st;
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_batch_autotune(ft_batch* b, ft_batch_tuning* best) {
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  const uint32_t tiles[3][2] = {{8, 8}, {16, 8}, {32, 8}};
  const uint32_t refills[3] = {4, 8, 16};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FT_CUDA_TRY(cudaEventCreate(&e0), "cudaEventCreate");
  FT_CUDA_TRY(cudaEventCreate(&e1), "cudaEventCreate");
  ft_batch_tuning top{8, 8, 8, 1e30f};
  ft_status status = FT_OK;
  for (const auto& tl : tiles) {
    for (uint32_t rf : refills) {
      b->tuning = ft_batch_tuning{tl[0], tl[1], rf, 0.0f};
      if ((status = batch_apply_tuning(b)) != FT_OK) break;
      cudaGraphLaunch(b->exec, b->stream);  // warm-up
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
}

ft_status ft_batch_launch(ft_batch* b, void* stream) {
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaGraphLaunch(b->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch(batch)");
  ftcommon::clear_last_error();
  return FT_OK;
}

ft_status ft_batch_read(ft_batch* b, uint32_t item, float* t_out, uint8_t* mask_out, float* rgb_out,
                        uint8_t* rgb8_out) {
  if (!b) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch must be non-null");
  if (item >= b->items.size()) return ftcommon::fail(FT_ERR_INVALID_ARGUMENT, "batch item out of range");
  std::lock_guard<std::mutex> lock(b->mu);
  FT_CUDA_TRY(cudaSetDevice(b->device), "cudaSetDevice");
  FT_CUDA_TRY(cudaDeviceSynchronize(), "batch");
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
  if (b->stream) cudaStreamDestroy(b->stream);
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
}

ft_status ft_render_backward(ft_scene* sc, const ft_view* views, uint32_t n_views, const ft_render_options* options,
                             float tau, const ft_param* params, uint32_t n_params, const float* dL_dt,
                             const float* dL_dsil, double* dL_dparams, uint32_t flags, void* stream) {
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
}

ft_status ft_measure_fp32_peak(double* tflops) {
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
}

}  // extern "C"
