// FP16 brick distance cache: the precision form of the depth march.
//
// There is no counterpart in the reference (its `Bricks` accelerator,
// R:824-1022, is a grid of leaf lists).  The distance field of the scene
// without its few very large leaves is sampled on a lattice of spacing h over
// a region around the other leaves.  The region is cut into bricks of 8^3
// voxels; each brick gets an interpolation error bound
//
//     delta_b = safety * max(L_b, 1) * h * sqrt(3),
//
// where L_b is the largest finite difference |dF| / h between neighbouring
// lattice points of the brick.  Every lattice point is stored as one FP16
// texel of a 3D texture holding
//
//     round_down_fp16( F(point) - max delta_b over the bricks sharing it ).
//
// For a field that is L_b-Lipschitz inside the brick, every corner of the
// voxel holding p then stores a value <= F(p), and so does any convex
// combination of them: the hardware trilinear fetch (its 8-bit fixed-point
// weights still sum to one) is a lower bound of F(p), one fetch per step with
// no table indirection.  All bricks are stored (2 bytes per lattice point):
// far from surfaces the bound is F - delta too, so far-field steps stay at
// least as long as the plain march's 0.7 |F| once |F| exceeds about 3 delta.
//
// Included by ft_render.cu after the exact evaluators, inside its anonymous
// namespace.
#pragma once

constexpr int kBrickVox = 8;   // voxels per brick edge
constexpr int kMaxExactLeaves = 4;
constexpr float kTrustLipschitz = 4.0f;  // larger per-brick estimates: exact marching only

struct DevBricks {
  float rmin[3];             // lattice point (0, 0, 0)
  float rmax[3];             // last lattice point
  float inv_h;               // 1 / voxel size
  float last[3];             // lattice points per axis - 1
  cudaTextureObject_t atlas; // FP16 texels, linear filtering, unnormalised coordinates
  float band, band_exit;
  int32_t far_batch;         // far-field steps per pass of the warp
  int32_t n_exact;
  int32_t exact_leaf[kMaxExactLeaves];
  int32_t free_far;          // FT_BRICK_FREE_FAR_STEPS: free far-field steps instead of the counted form
  int32_t outside_ok;        // the cached leaves lie in the region box (no hooked or modified leaves)
  float outside_margin;      // subtracted from the region-box distance (blend bulges)
  int32_t plane_leaf;        // the only exact leaf when it is an axis-aligned box, else -1
  uint32_t plane_obj;        // its object id
  float plane_top;           // its top face: y = plane_top over [plane_lo, plane_hi] in x and z
  float plane_lo[2], plane_hi[2];
};

// Leaf-BVH walk of the scene minus the exact leaves (bvh_distance_info,
// R:743-786, with those leaves left out): the field the cache samples.
template <bool kStats>
__device__ Info scene_distance_skip(const DevScene& S, F3 p, const DevBricks& B, Ctx<kStats>& cx) {
  float best = kInf;
  Info cur{kInf, 0u, 0u};
  int stack[64];
  float stack_lb[64];
  int sp = 0;
  stack[sp] = S.bvh_root;
  stack_lb[sp] = node_lb(p, S.bvh[S.bvh_root].bmin, S.bvh[S.bvh_root].bmax);
  ++sp;
  for (int walk = 0; sp > 0 && walk < ftgpu::kMaxWalk; ++walk) {  // a tree walk pops each node once
    --sp;
    int ni = stack[sp];
    if (stack_lb[sp] > best) continue;
    const DevBvhNode& n = S.bvh[ni];
    if (n.leaf >= 0) {
      bool skip = false;
      for (int i = 0; i < B.n_exact; ++i) skip |= (B.exact_leaf[i] == n.leaf);
      if (skip) continue;
      Info in = eval_leaf(S, S.leaves[n.leaf], p, best, cx);
      if (in.d < best) {
        best = in.d;
        cur = in;
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

// Far-field lower bound of the scene distance at p: the cached field (one
// texture fetch) and the exact leaves.  Returns false outside the brick
// region, where the march is exact (a distance-to-region bound would give
// tiny steps to rays passing close to the region's box, and the exact field
// outside it is cheap: the cached leaves are culled by their boxes).
template <bool kStats>
__device__ __forceinline__ bool far_bound(const DevScene& S, const DevBricks& B, F3 p, float* out, Ctx<kStats>& cx) {
  float gx = (p.x - B.rmin[0]) * B.inv_h, gy = (p.y - B.rmin[1]) * B.inv_h, gz = (p.z - B.rmin[2]) * B.inv_h;
  if (!(gx >= 0.0f && gy >= 0.0f && gz >= 0.0f && gx <= B.last[0] && gy <= B.last[1] && gz <= B.last[2]))
    return false;
  cx.fetch();
  // texel centres sit at integer + 0.5 in unnormalised coordinates
  float v = tex3D<float>(B.atlas, gx + 0.5f, gy + 0.5f, gz + 0.5f);
  for (int i = 0; i < B.n_exact; ++i) v = fminf(v, eval_leaf(S, S.leaves[B.exact_leaf[i]], p, kInf, cx).d);
  *out = v;
  return true;
}

// Lower bound of the distance to the cached leaves (the scene without its
// exact leaves) at p: the fetched bound inside the brick region; outside it
// the distance to the region box less the margin where every cached leaf
// lies inside that box, else -inf.
template <bool kStats>
__device__ __forceinline__ float cached_lb(const DevBricks& B, F3 p, Ctx<kStats>& cx) {
  float gx = (p.x - B.rmin[0]) * B.inv_h, gy = (p.y - B.rmin[1]) * B.inv_h, gz = (p.z - B.rmin[2]) * B.inv_h;
  if (gx >= 0.0f && gy >= 0.0f && gz >= 0.0f && gx <= B.last[0] && gy <= B.last[1] && gz <= B.last[2]) {
    cx.fetch();
    return tex3D<float>(B.atlas, gx + 0.5f, gy + 0.5f, gz + 0.5f);
  }
  if (!B.outside_ok) return -kInf;
  return ftd::aabb_lb(p, B.rmin, B.rmax) - B.outside_margin;
}

// Whether the rest of a plain march from q (scene distance g, the plane
// leaf's) is a descent onto the plane leaf's top face: the ray goes
// down, q and the crossing lie over the face, and the cached leaves are
// farther than the crossing along the ray (their distance shrinks by at most
// the distance travelled, the plane's by sin(angle) times it, so the plane
// stays the minimum at every sample).  Requires the minimum step to stay
// below scale * eps, so every step above the shell is scale * height.
__device__ __forceinline__ bool plane_jump(const DevBricks& B, F3 q, F3 d, float g, float cached, float eps,
                                           float scale, float min_step) {
  const float sdn = -d.y;
  if (!(sdn > 0.0f) || !(g >= eps) || !(min_step < scale * eps) || !(scale * sdn < 1.0f)) return false;
  if (!(q.y > B.plane_top)) return false;
  const float along = g / sdn;
  if (!(cached > along)) return false;
  const float ex = q.x + d.x * along, ez = q.z + d.z * along;
  return q.x > B.plane_lo[0] && q.x < B.plane_hi[0] && q.z > B.plane_lo[1] && q.z < B.plane_hi[1] &&
         ex > B.plane_lo[0] && ex < B.plane_hi[0] && ez > B.plane_lo[1] && ez < B.plane_hi[1];
}

// Steps of the plain march's descent onto the plane from height g >= eps on
// a ray of downward slope sdn, step = scale x distance: the heights are
// g (1 - c)^k with c = scale sdn, so the first sample inside the eps shell is
// n = floor(ln(eps / g) / ln(1 - c)) + 1 steps on.  All in FP32: the closed
// form's n is checked against the heights at n - 1 and n (one powf each) and
// moved by one where rounding of the logarithms put it on the wrong side.
// *along = distance travelled in those n steps, g (1 - (1 - c)^n) / sdn.
// Returns -1 when the count does not fit (grazing rays: n > 2^24).
__device__ __forceinline__ int plane_descent_steps(float g, float sdn, float scale, float eps, float* along) {
  const float c = scale * sdn;
  const float q = 1.0f - c;
  const float x = logf(eps / g) / log1pf(-c);
  if (!(x < 16777216.0f)) return -1;
  int n = static_cast<int>(floorf(x)) + 1;
  if (n > 1 && g * powf(q, static_cast<float>(n - 1)) < eps) --n;
  else if (g * powf(q, static_cast<float>(n)) >= eps) ++n;
  *along = (g - g * powf(q, static_cast<float>(n))) / sdn;
  return n;
}

#ifndef FT_JIT  // build and query kernels: precompiled only
// ------------------------------------------------------------------ build

struct BrickBuild {
  float rmin[3];
  float h;
  int32_t dims[3];
  uint32_t nx, ny, nz;  // lattice points per axis (dims * 8 + 1)
};

// Sample the cached field at every lattice point.
__global__ void __launch_bounds__(128) brick_lattice_kernel(DevScene S, DevBricks B, BrickBuild G,
                                                            float* __restrict__ lattice) {
  Ctx<false> cx;
  cx.c = Counters{};
  const uint64_t n = (uint64_t)G.nx * G.ny * G.nz;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x = (uint32_t)(i % G.nx);
    uint64_t r = i / G.nx;
    uint32_t y = (uint32_t)(r % G.ny);
    uint32_t z = (uint32_t)(r / G.ny);
    F3 p = f3(G.rmin[0] + G.h * (float)x, G.rmin[1] + G.h * (float)y, G.rmin[2] + G.h * (float)z);
    lattice[i] = scene_distance_skip(S, p, B, cx).d;
  }
}

__device__ __forceinline__ size_t lattice_index(const BrickBuild& G, uint32_t x, uint32_t y, uint32_t z) {
  return (size_t)x + (size_t)G.nx * ((size_t)y + (size_t)G.ny * z);
}

// One warp per brick: its Lipschitz estimate and error bound, and whether a
// surface passes within `near` of it (for the build summary).
__global__ void __launch_bounds__(128) brick_bound_kernel(BrickBuild G, const float* __restrict__ lattice,
                                                          float safety, float near, const float* __restrict__ untrusted,
                                                          float* __restrict__ delta,
                                                          unsigned int* __restrict__ near_count,
                                                          unsigned int* __restrict__ max_lip_bits) {
  constexpr uint32_t kPts = kBrickVox + 1;
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t n_cells = (uint64_t)G.dims[0] * G.dims[1] * G.dims[2];
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
  for (uint64_t cell = (uint64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; cell < n_cells; cell += warps) {
    uint32_t cx = (uint32_t)(cell % G.dims[0]);
    uint64_t r = cell / G.dims[0];
    uint32_t cy = (uint32_t)(r % G.dims[1]);
    uint32_t cz = (uint32_t)(r / G.dims[1]);
    float vmin = kInf, dmax = 0.0f;
    for (uint32_t k = lane; k < kPts * kPts * kPts; k += 32) {
      uint32_t lx = k % kPts, ly = (k / kPts) % kPts, lz = k / (kPts * kPts);
      uint32_t x = cx * kBrickVox + lx, y = cy * kBrickVox + ly, z = cz * kBrickVox + lz;
      float v = lattice[lattice_index(G, x, y, z)];
      vmin = fminf(vmin, v);
      // Pairs with both samples inside a solid are left out: the far field is
      // only used at points with a positive bound, and the reference's leaf
      // culling makes the field jump inside overlapping solids.
      float w;
      if (lx + 1 < kPts) {
        w = lattice[lattice_index(G, x + 1, y, z)];
        if (v >= 0.0f || w >= 0.0f) dmax = fmaxf(dmax, fabsf(w - v));
      }
      if (ly + 1 < kPts) {
        w = lattice[lattice_index(G, x, y + 1, z)];
        if (v >= 0.0f || w >= 0.0f) dmax = fmaxf(dmax, fabsf(w - v));
      }
      if (lz + 1 < kPts) {
        w = lattice[lattice_index(G, x, y, z + 1)];
        if (v >= 0.0f || w >= 0.0f) dmax = fmaxf(dmax, fabsf(w - v));
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, off));
      dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, off));
    }
    if (lane == 0) {
      float lip = fmaxf(dmax / G.h, 1.0f);
      // A brick whose samples jump (the field is not Lipschitz there, e.g.
      // where leaf culling switches), or that a hooked leaf can reach (hooks
      // move surfaces off their boxes), gets no usable bound: the march is
      // exact inside it.  (A large finite bound keeps trilinear mixes finite.)
      const float bs = G.h * kBrickVox;
      float lo[3] = {G.rmin[0] + bs * cx, G.rmin[1] + bs * cy, G.rmin[2] + bs * cz};
      bool hooked = untrusted[0] <= untrusted[3];
      for (int a = 0; a < 3; ++a) hooked &= lo[a] <= untrusted[3 + a] && lo[a] + bs >= untrusted[a];
      float del = (lip > kTrustLipschitz || hooked) ? 1.0e4f : safety * lip * G.h * 1.7320508f;
      delta[cell] = del;
      if (vmin - del < near) atomicAdd(near_count, 1u);
      atomicMax(max_lip_bits, __float_as_uint(lip));  // positive floats order like their bits
    }
  }
}

// One texel per lattice point: the sample lowered by the largest bound of the
// (up to eight) bricks sharing the point, rounded down to FP16.
__global__ void __launch_bounds__(256) brick_texel_kernel(BrickBuild G, const float* __restrict__ lattice,
                                                          const float* __restrict__ delta, cudaSurfaceObject_t atlas) {
  const uint64_t n = (uint64_t)G.nx * G.ny * G.nz;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t x = (uint32_t)(i % G.nx);
    uint64_t r = i / G.nx;
    uint32_t y = (uint32_t)(r % G.ny);
    uint32_t z = (uint32_t)(r / G.ny);
    // bricks along each axis that contain this lattice coordinate
    int bx1 = min((int)(x / kBrickVox), G.dims[0] - 1), bx0 = (x % kBrickVox == 0 && x > 0) ? bx1 - 1 : bx1;
    int by1 = min((int)(y / kBrickVox), G.dims[1] - 1), by0 = (y % kBrickVox == 0 && y > 0) ? by1 - 1 : by1;
    int bz1 = min((int)(z / kBrickVox), G.dims[2] - 1), bz0 = (z % kBrickVox == 0 && z > 0) ? bz1 - 1 : bz1;
    if (x == G.nx - 1) bx0 = bx1;
    if (y == G.ny - 1) by0 = by1;
    if (z == G.nz - 1) bz0 = bz1;
    float del = 0.0f;
    for (int bz = bz0; bz <= bz1; ++bz)
      for (int by = by0; by <= by1; ++by)
        for (int bx = bx0; bx <= bx1; ++bx)
          del = fmaxf(del, delta[(size_t)bx + (size_t)G.dims[0] * ((size_t)by + (size_t)G.dims[1] * bz)]);
    __half hv = __float2half_rd(lattice[i] - del);
    surf3Dwrite(__half_as_ushort(hv), atlas, (int)(x * sizeof(unsigned short)), (int)y, (int)z);
  }
}

// Validation: the far-field bound and the exact distance at given points.
__global__ void brick_query_kernel(DevScene S, DevBricks B, const float* __restrict__ pts, uint32_t n,
                                   float* __restrict__ bound, float* __restrict__ exact) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Ctx<false> cx;
  cx.c = Counters{};
  F3 p = f3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
  float b;
  bound[i] = far_bound(S, B, p, &b, cx) ? b : __int_as_float(0x7fc00000);  // NaN: no bound here
  exact[i] = scene_distance(S, p, cx).d;
}
#endif  // FT_JIT
