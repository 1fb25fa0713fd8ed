// Differentiation form: multi-view depth + soft silhouette and the adjoint
// march (ft_render_views / ft_render_backward).  No counterpart in the
// reference.  Definitions, shared with the FP64 CPU restatement:
//
//   forward, per ray: the plain march (step rule, eps hit, ten bisections);
//   on a hit the depth is the zero of f(o + t d), three secant steps from the
//   bisection bracket; on a miss m = the local minimum of f along the ray
//   next to the smallest march sample (its bracket continued past either end
//   of the samples while f falls, then a 40-step golden-section search), and
//   silhouette = exp(-max(m, 0) / tau) (1 on a hit).
//
//   backward: the march is recomputed (nothing per step is stored); at the
//   hit point  d depth / d theta = -(df/dtheta) / (grad_p f . d), at the
//   miss minimum  d sil / d theta = -(sil / tau) df/dtheta  (its position
//   is stationary along the ray, and is polished by secant steps on
//   grad_p f . d = 0 before the derivative is taken); df/dtheta comes from a full fold of the
//   winning union_round tree with reverse-mode derivatives of op_union_round
//   and of the sphere / box distances.  Per-parameter sums across pixels are
//   FP64: shared-memory accumulators per block, one global atomic per block
//   and parameter.
//
// Included by ft_render.cu inside its anonymous namespace.
#pragma once

constexpr int kMaxDiffPrims = 512;  // union_round trees the adjoint folds (primitives)
constexpr int kGoldenSteps = 40;
constexpr int kSecantSteps = 3;
constexpr int kMinPolishSteps = 4;  // secant steps on df/dt at the silhouette minimum (backward)

struct DiffTables {
  const int32_t* slot;         // node * 8 + field -> parameter index, -1 if none
  const int32_t* tree_radius;  // per union_round tree: radius parameter index, -1 if none
  uint32_t n_params;
};

struct ViewRayOut {
  bool hit;
  float t, sil, tm, m;
};

// Plain march with the smallest sample tracked, then the forward definitions.
template <bool kStats>
__device__ ViewRayOut view_ray(const DevScene& S, const RayParams& P, F3 o, F3 d, float tau, Ctx<kStats>& cx) {
  ViewRayOut out{false, 0.0f, 0.0f, 0.0f, 0.0f};
  float t0, t1;
  if (!ray_aabb(o, d, S.smin, S.smax, &t0, &t1)) return out;
  const float eps = P.eps;
  const float scale = ftd::rclamp(P.step_scale, 0.05f, 1.0f);
  const float min_step = fmaxf(eps * 0.5f, 1.0e-5f);
  float max_t = fminf(P.max_dist, t1);
  float traveled = fmaxf(t0, 0.0f), prev = traveled;
  float best = kInf, tb_prev = traveled, tb = traveled, tb_next = traveled;
  bool need_next = false;
  for (uint32_t s = 0; s < P.max_steps; ++s) {
    if (traveled > max_t) break;
    float dv = scene_d(S, o + d * traveled, cx);
    if (need_next) {
      tb_next = traveled;
      need_next = false;
    }
    if (dv < best) {
      best = dv;
      tb_prev = prev;
      tb = traveled;
      tb_next = traveled;
      need_next = true;
    }
    if (fabsf(dv) < eps) {
      float lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        float mid = 0.5f * (lo + hi);
        if (fabsf(scene_d(S, o + d * mid, cx)) < eps) hi = mid;
        else lo = mid;
      }
      float fa = scene_d(S, o + d * lo, cx), fb = scene_d(S, o + d * hi, cx);
      for (int k = 0; k < kSecantSteps; ++k) {
        if (fb == fa) break;
        float tn = hi - fb * (hi - lo) / (fb - fa);
        lo = hi;
        fa = fb;
        hi = tn;
        fb = scene_d(S, o + d * hi, cx);
      }
      out.hit = true;
      out.t = hi;
      out.sil = 1.0f;
      return out;
    }
    prev = traveled;
    traveled += fmaxf(fabsf(dv) * scale, min_step);
  }
  if (!(best < kInf)) return out;
  // Bracket a local minimum around the smallest sample, continuing the
  // descent past either end of the samples while f keeps falling, then a
  // golden-section search on the triple (a, x, b) with f(x) <= f(a), f(b).
  auto step_of = [&](float fv) { return fmaxf(fabsf(fv) * scale, min_step); };
  float a = tb_prev, x = tb, fx = best;
  float b = need_next ? x + step_of(fx) : tb_next;
  float fb = scene_d(S, o + d * b, cx);
  for (int k = 0; k < 64 && fb < fx && b < P.max_dist; ++k) {
    a = x;
    x = b;
    fx = fb;
    b = x + step_of(fx);
    fb = scene_d(S, o + d * b, cx);
  }
  if (!(a < x)) a = fmaxf(x - step_of(fx), 0.0f);
  float fa = scene_d(S, o + d * a, cx);
  for (int k = 0; k < 64 && fa < fx && a > 0.0f; ++k) {
    b = x;
    x = a;
    fx = fa;
    a = fmaxf(x - step_of(fx), 0.0f);
    fa = scene_d(S, o + d * a, cx);
  }
  for (int k = 0; k < kGoldenSteps; ++k) {
    float u = (b - x > x - a) ? x + 0.3819660112501051f * (b - x) : x - 0.3819660112501051f * (x - a);
    float fu = scene_d(S, o + d * u, cx);
    if (fu < fx) {
      if (u > x) a = x;
      else b = x;
      x = u;
      fx = fu;
    } else {
      if (u > x) b = u;
      else a = u;
    }
  }
  out.tm = x;
  out.m = fx;
  out.sil = expf(-fmaxf(out.m, 0.0f) / tau);
  return out;
}

// Gradient sink: parameter partials scaled by `scale` into FP64 accumulators
// (shared memory when the block holds one per parameter), and grad_p f.
struct GradSink {
  double* acc;      // shared or global
  const DiffTables* T;
  float scale;      // multiplies every parameter partial (0: gradient in p only)
  F3 gp;
  __device__ void add(int node, int field, float v) {
    if (scale == 0.0f) return;
    int k = __ldg(&T->slot[node * 8 + field]);
    if (k >= 0) atomicAdd(&acc[k], static_cast<double>(scale * v));
  }
};

// Reverse-mode derivative of one sphere / box primitive (no x / z rotation,
// rounding or shell: the parameter layout guarantees it).
__device__ void prim_backprop(const DevNode& n, int node, F3 p, float adj, GradSink& g) {
  F3 dpc = f3(p.x - n.c[0], p.y - n.c[1], p.z - n.c[2]);
  // DevNode keeps sin / cos of -rot.y
  const float c = n.has_rot ? n.cy : 1.0f, s = n.has_rot ? n.sy : 0.0f;
  F3 q = f3(c * dpc.x + s * dpc.z, dpc.y, -s * dpc.x + c * dpc.z);
  F3 dq;
  if (n.kind == FT_NODE_SPHERE) {
    float l = ftd::len3(q);
    dq = l > 0.0f ? q * (1.0f / l) : f3(0.0f, 0.0f, 0.0f);
    g.add(node, FT_PARAM_S0, -adj);
  } else {
    float qv[3] = {q.x, q.y, q.z}, qa[3], o[3];
    for (int i = 0; i < 3; ++i) {
      qa[i] = fabsf(qv[i]) - n.f[i];
      o[i] = fmaxf(qa[i], 0.0f);
    }
    float outside = sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
    float dqa[3] = {0.0f, 0.0f, 0.0f};
    if (outside > 0.0f) {
      for (int i = 0; i < 3; ++i) dqa[i] = o[i] / outside;
    } else {
      int m = 0;
      for (int i = 1; i < 3; ++i)
        if (qa[i] > qa[m]) m = i;
      dqa[m] = 1.0f;
    }
    dq = f3(qv[0] < 0.0f ? -dqa[0] : dqa[0], qv[1] < 0.0f ? -dqa[1] : dqa[1], qv[2] < 0.0f ? -dqa[2] : dqa[2]);
    g.add(node, FT_PARAM_S0, -adj * dqa[0]);
    g.add(node, FT_PARAM_S1, -adj * dqa[1]);
    g.add(node, FT_PARAM_S2, -adj * dqa[2]);
  }
  F3 dp = f3(c * dq.x - s * dq.z, dq.y, s * dq.x + c * dq.z);
  g.gp = g.gp + dp * adj;
  g.add(node, FT_PARAM_CX, -adj * dp.x);
  g.add(node, FT_PARAM_CY, -adj * dp.y);
  g.add(node, FT_PARAM_CZ, -adj * dp.z);
  g.add(node, FT_PARAM_ROT_Y, adj * (dq.x * q.z - dq.z * q.x) * (-3.14159265358979323846f / 180.0f));
}

// op_union_round partials (value = max(r, min(a, b)) - |max(r - (a, b), 0)|).
__device__ __forceinline__ void union_round_partials(float a, float b, float r, float* pa, float* pb, float* pr) {
  float ux = fmaxf(r - a, 0.0f), uy = fmaxf(r - b, 0.0f);
  float l = sqrtf(ux * ux + uy * uy);
  if (l > 0.0f) {
    *pa = ux / l;
    *pb = uy / l;
    *pr = 1.0f - (ux + uy) / l;
  } else {
    *pa = a < b ? 1.0f : 0.0f;
    *pb = a < b ? 0.0f : 1.0f;
    *pr = 0.0f;
  }
}

// Full fold of union_round tree `ti` at p with reverse-mode derivatives.
// `vals` holds the two child values of every inner node (2 * (n - 1)).
// Returns false for trees the adjoint does not handle.
__device__ bool urtree_backprop(const DevScene& S, int ti, F3 p, float* vals, float* adjs, const DiffTables& T,
                                GradSink& g) {
  const DevUrTree& t = S.urtrees[ti];
  const int n_inner = t.n_prims - 1;
  if (t.n_prims > kMaxDiffPrims || n_inner < 1) return false;
  const int base = t.inner_root;
  const float r0 = t.r;
  const float r = fmaxf(fabsf(r0), 1.0e-6f);
  auto prim_value = [&](int pos) {
    const DevNode& pn = S.nodes[S.ur_prims[t.prim_first + pos]];
    return ftd::prim_distance(pn, p);
  };
  // Pre-order numbering: children of inner i have larger indices, so a
  // reverse sweep evaluates every inner node after its children.
  for (int i = n_inner - 1; i >= 0; --i) {
    const DevUrInner& in = S.ur_inner[base + i];
    for (int c = 0; c < 2; ++c) {
      int ch = in.child[c];
      float v;
      if (ch < 0) {
        v = prim_value(-ch - 1);
      } else {
        const float a = vals[2 * (ch - base)], b = vals[2 * (ch - base) + 1];
        v = ftd::op_union_round(a, b, r0);
      }
      vals[2 * i + c] = v;
    }
  }
  for (int i = 0; i < n_inner; ++i) adjs[i] = 0.0f;
  adjs[0] = 1.0f;
  float dr = 0.0f;
  for (int i = 0; i < n_inner; ++i) {
    float ai = adjs[i];
    if (ai == 0.0f) continue;
    float pa, pb, pr;
    union_round_partials(vals[2 * i], vals[2 * i + 1], r, &pa, &pb, &pr);
    dr += ai * pr;
    const DevUrInner& in = S.ur_inner[base + i];
    float pc[2] = {pa, pb};
    for (int c = 0; c < 2; ++c) {
      if (pc[c] == 0.0f) continue;
      int ch = in.child[c];
      if (ch < 0) {
        int node = S.ur_prims[t.prim_first + (-ch - 1)];
        prim_backprop(S.nodes[node], node, p, ai * pc[c], g);
      } else {
        adjs[ch - base] += ai * pc[c];
      }
    }
  }
  int kr = __ldg(&T.tree_radius[ti]);
  if (kr >= 0 && g.scale != 0.0f && fabsf(r0) > 1.0e-6f)
    atomicAdd(&g.acc[kr], static_cast<double>(g.scale * dr * (r0 < 0.0f ? -1.0f : 1.0f)));
  return true;
}

// df/dtheta and grad_p f at p through the winning leaf of the scene.
template <bool kStats>
__device__ bool scene_backprop(const DevScene& S, F3 p, float* vals, float* adjs, const DiffTables& T, GradSink& g,
                               Ctx<kStats>& cx) {
  int leaf = 0;
  scene_distance_leaf(S, p, &leaf, cx);
  const DevLeaf& lf = S.leaves[leaf];
  if (lf.kind == ftgpu::kLeafUrTree) return urtree_backprop(S, lf.first, p, vals, adjs, T, g);
  if (lf.kind == ftgpu::kLeafPrim) {
    const DevNode& n = S.nodes[lf.node];
    if (n.kind != FT_NODE_SPHERE && n.kind != FT_NODE_BOX) return false;
    prim_backprop(n, lf.node, p, 1.0f, g);
    return true;
  }
  return false;
}

// One thread per (view, work item).
__global__ void __launch_bounds__(128) views_forward_kernel(DevScene S, const RayParams* __restrict__ views,
                                                            uint32_t n_views, uint64_t items_per_view, float tau,
                                                            float* __restrict__ t_out, uint8_t* __restrict__ mask_out,
                                                            float* __restrict__ sil_out) {
  uint64_t g = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= items_per_view * n_views) return;
  uint32_t v = static_cast<uint32_t>(g / items_per_view);
  const RayParams& P = views[v];
  F3 d;
  size_t idx = 0;
  if (!item_ray(P, g - static_cast<uint64_t>(v) * items_per_view, &d, &idx)) return;
  idx += static_cast<size_t>(v) * P.width * P.height;
  Ctx<false> cx;
  cx.c = Counters{};
  ViewRayOut r = view_ray(S, P, f3(P.origin[0], P.origin[1], P.origin[2]), d, tau, cx);
  if (t_out) t_out[idx] = r.hit ? r.t : 0.0f;
  if (mask_out) mask_out[idx] = r.hit ? 1 : 0;
  if (sil_out) sil_out[idx] = r.sil;
}

// Adjoint: recompute each ray, then accumulate its parameter gradient.
// Dynamic shared memory: n_params doubles when `shared_acc`.
__global__ void __launch_bounds__(128) views_backward_kernel(DevScene S, const RayParams* __restrict__ views,
                                                             uint32_t n_views, uint64_t items_per_view, float tau,
                                                             DiffTables T, const float* __restrict__ dl_dt,
                                                             const float* __restrict__ dl_dsil, double* __restrict__ grad,
                                                             int shared_acc, int* __restrict__ unsupported) {
  extern __shared__ double sacc[];
  if (shared_acc) {
    for (uint32_t k = threadIdx.x; k < T.n_params; k += blockDim.x) sacc[k] = 0.0;
    __syncthreads();
  }
  double* acc = shared_acc ? sacc : grad;
  const uint64_t total = items_per_view * n_views;
  for (uint64_t g = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
       g += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    uint32_t v = static_cast<uint32_t>(g / items_per_view);
    const RayParams& P = views[v];
    F3 d;
    size_t idx = 0;
    if (!item_ray(P, g - static_cast<uint64_t>(v) * items_per_view, &d, &idx)) continue;
    idx += static_cast<size_t>(v) * P.width * P.height;
    float wt = dl_dt ? dl_dt[idx] : 0.0f, ws = dl_dsil ? dl_dsil[idx] : 0.0f;
    if (wt == 0.0f && ws == 0.0f) continue;
    Ctx<false> cx;
    cx.c = Counters{};
    const F3 o = f3(P.origin[0], P.origin[1], P.origin[2]);
    ViewRayOut r = view_ray(S, P, o, d, tau, cx);
    float vals[2 * (kMaxDiffPrims - 1)];
    float adjs[kMaxDiffPrims - 1];
    if (r.hit && wt != 0.0f) {
      F3 p = o + d * r.t;
      GradSink probe{acc, &T, 0.0f, f3(0.0f, 0.0f, 0.0f)};
      if (!scene_backprop(S, p, vals, adjs, T, probe, cx)) {
        atomicOr(unsupported, 1);
        continue;
      }
      float den = ftd::dot3(probe.gp, d);
      if (fabsf(den) <= 1.0e-8f) continue;
      GradSink sink{acc, &T, -wt / den, f3(0.0f, 0.0f, 0.0f)};
      scene_backprop(S, p, vals, adjs, T, sink, cx);
    } else if (!r.hit && ws != 0.0f && r.m > 0.0f && r.sil > 0.0f) {
      // The minimum is flat along the ray, so its FP32 position is only known
      // to ~1e-3: polish it with secant steps on df/dt = grad_p f . d = 0.
      float tm = r.tm;
      bool ok = true;
      auto slope = [&](float tt) {
        GradSink probe{acc, &T, 0.0f, f3(0.0f, 0.0f, 0.0f)};
        ok &= scene_backprop(S, o + d * tt, vals, adjs, T, probe, cx);
        return ftd::dot3(probe.gp, d);
      };
      const float dt0 = 1.0e-3f * fmaxf(1.0f, tm);
      const float g0 = slope(tm);
      float ta = tm - dt0, tb = tm + dt0;
      float ga = slope(ta), gb = slope(tb);
      for (int k = 0; k < kMinPolishSteps && ok && gb != ga; ++k) {
        float tn = tb - gb * (tb - ta) / (gb - ga);
        tn = fminf(fmaxf(tn, tm - 4.0f * dt0), tm + 4.0f * dt0);
        ta = tb;
        ga = gb;
        tb = tn;
        gb = slope(tb);
      }
      if (ok && fabsf(gb) < fabsf(g0)) tm = tb;
      GradSink sink{acc, &T, -ws * r.sil / tau, f3(0.0f, 0.0f, 0.0f)};
      if (!ok || !scene_backprop(S, o + d * tm, vals, adjs, T, sink, cx)) atomicOr(unsupported, 1);
    }
  }
  if (shared_acc) {
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < T.n_params; k += blockDim.x)
      if (sacc[k] != 0.0) atomicAdd(&grad[k], sacc[k]);
  }
}
