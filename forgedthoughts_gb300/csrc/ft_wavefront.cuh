// Wavefront form of the Whitted trace: the same integrator as trace_sample
// (shade_hit with its sinks) with every bounce level processed by three
// kernels over queues instead of one thread walking one sample's ray tree:
//
//   wf_march_kernel   marches the level's ray jobs (misses add the
//                     environment, hits are recorded),
//   wf_shade_kernel   shades the hits (shade_hit): emission and unshadowed
//                     terms are added at once, light samples become shadow
//                     jobs, reflected / refracted rays become next-level jobs,
//   wf_shadow_kernel  marches the shadow jobs (shadow_visibility) and adds
//                     contribution x visibility.
//
// Kernels of one kind run the same code on every lane, so the divergence of
// the per-sample tree (different bounce paths, shadow marches inside shading)
// is gone.  Radiance is accumulated per sample with float atomics; the order
// of those additions, hence the last bits, varies from run to run.
//
// Included by ft_kernels.cuh after the trace integrator.
#pragma once

constexpr uint32_t kNoSample = 0xffffffffu;
// Queue counters of a wavefront: job counts of the two levels in flight, the
// shadow count, the overflow flag, the march and shadow kernels' work
// counters and the self-check flags.
constexpr int kWfCounters = 8;

struct WJob {
  float o[3], d[3], w[3];
  float ior, absorption[3], density;
  int32_t depth;
  uint32_t sample;
};

struct WHit {
  float t, pos[3], normal[3];
  uint32_t mat, obj;
  int32_t leaf;  // -1: missed (environment added), -2: no job
};

struct WShadow {
  float o[3], d[3], max_t, contrib[3];
  uint32_t sample;
};

struct WQueues {
  float* radiance;  // per sample rgb
  WJob* next;
  unsigned long long* next_count;
  unsigned long long next_cap;
  WShadow* shadows;
  unsigned long long* shadow_count;
  unsigned long long shadow_cap;
  unsigned int* overflow;
  uint32_t max_depth;
};

__device__ __forceinline__ void add_radiance(float* radiance, uint32_t sample, F3 v) {
  if (v.x != 0.0f) atomicAdd(&radiance[3 * static_cast<size_t>(sample)], v.x);
  if (v.y != 0.0f) atomicAdd(&radiance[3 * static_cast<size_t>(sample) + 1], v.y);
  if (v.z != 0.0f) atomicAdd(&radiance[3 * static_cast<size_t>(sample) + 2], v.z);
}

__device__ __forceinline__ RayJob job_of(const WJob& j) {
  return RayJob{f3(j.o[0], j.o[1], j.o[2]), f3(j.d[0], j.d[1], j.d[2]), f3(j.w[0], j.w[1], j.w[2]),
                MediumD{j.ior, f3(j.absorption[0], j.absorption[1], j.absorption[2]), j.density}, j.depth};
}

// Sink of the wavefront integrator: everything goes to queues.
struct QueueSink {
  const WQueues& Q;
  uint32_t sample;
  __device__ void emit(F3 v) { add_radiance(Q.radiance, sample, v); }
  __device__ void light(F3 contrib, F3 o, F3 d, float max_t) {
    if (contrib.x == 0.0f && contrib.y == 0.0f && contrib.z == 0.0f) return;
    unsigned long long k = atomicAdd(Q.shadow_count, 1ull);
    if (k >= Q.shadow_cap) {
      atomicOr(Q.overflow, 1u);
      return;
    }
    WShadow& s = Q.shadows[k];
    s.o[0] = o.x; s.o[1] = o.y; s.o[2] = o.z;
    s.d[0] = d.x; s.d[1] = d.y; s.d[2] = d.z;
    s.max_t = max_t;
    s.contrib[0] = contrib.x; s.contrib[1] = contrib.y; s.contrib[2] = contrib.z;
    s.sample = sample;
  }
  __device__ void push(const RayJob& j) {
    if (static_cast<uint32_t>(j.depth) >= Q.max_depth) return;  // popped and skipped by the stack form
    unsigned long long k = atomicAdd(Q.next_count, 1ull);
    if (k >= Q.next_cap) {
      atomicOr(Q.overflow, 1u);
      return;
    }
    WJob& n = Q.next[k];
    n.o[0] = j.o.x; n.o[1] = j.o.y; n.o[2] = j.o.z;
    n.d[0] = j.d.x; n.d[1] = j.d.y; n.d[2] = j.d.z;
    n.w[0] = j.w.x; n.w[1] = j.w.y; n.w[2] = j.w.z;
    n.ior = j.med.ior;
    n.absorption[0] = j.med.absorption.x; n.absorption[1] = j.med.absorption.y;
    n.absorption[2] = j.med.absorption.z;
    n.density = j.med.density;
    n.depth = j.depth;
    n.sample = sample;
  }
};

// Primary jobs: one per camera work item (tile padding gets kNoSample).
__global__ void __launch_bounds__(128) wf_primary_kernel(RayParams P, WJob* __restrict__ jobs) {
  uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P.n_items) return;
  F3 d;
  size_t idx = 0;
  WJob j{};
  if (item_ray(P, i, &d, &idx)) {
    j.o[0] = P.origin[0]; j.o[1] = P.origin[1]; j.o[2] = P.origin[2];
    j.d[0] = d.x; j.d[1] = d.y; j.d[2] = d.z;
    j.w[0] = j.w[1] = j.w[2] = 1.0f;
    MediumD a = air();
    j.ior = a.ior;
    j.absorption[0] = a.absorption.x; j.absorption[1] = a.absorption.y; j.absorption[2] = a.absorption.z;
    j.density = a.density;
    j.depth = 0;
    j.sample = static_cast<uint32_t>(idx);
  } else {
    j.sample = kNoSample;
  }
  jobs[i] = j;
}

// One recorded hit: shade it into the queues.
template <bool kStats>
__device__ __forceinline__ void wf_shade_job(const DevScene& S, const RayParams& P, const WJob& wj, const WHit& wh,
                                             const WQueues& Q, Ctx<kStats>& cx) {
  TraceHit h;
  h.t = wh.t;
  h.pos = f3(wh.pos[0], wh.pos[1], wh.pos[2]);
  h.normal = f3(wh.normal[0], wh.normal[1], wh.normal[2]);
  h.mat = wh.mat;
  h.obj = wh.obj;
  h.leaf = wh.leaf;
  RayJob J = job_of(wj);
  QueueSink sink{Q, wj.sample};
  shade_hit(S, P, J, h, sink, cx);
}

#define FT_GRID_STRIDE(i, n)                                                                             \
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; \
       i < (n); i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)

// With kStats the kernel sums its work counters into stats[0 .. kNumCounters).
template <bool kStats>
__global__ void __launch_bounds__(128) wf_shade_kernel(DevScene S, RayParams P, const WJob* __restrict__ jobs,
                                                       const unsigned long long* __restrict__ count,
                                                       unsigned long long cap, const WHit* __restrict__ hits,
                                                       WQueues Q, unsigned long long* __restrict__ stats) {
  Ctx<kStats> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) {
    if (hits[i].leaf < 0) continue;
    wf_shade_job(S, P, jobs[i], hits[i], Q, cx);
  }
  if (kStats) flush_stats(cx.c, stats);
}


// Render of a queued job in a batch: the last whose first sample is not
// above the job's sample.
__device__ __forceinline__ uint32_t sample_item(const BatchView& V, uint64_t sample) {
  uint32_t lo = 0, hi = V.n_items;  // out_first[lo] <= sample < out_first[hi]
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (V.out_first[mid] <= sample) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Queue kernels with warp refill.  A grid-stride loop gives each lane one
// job to the end, so a warp waits for its longest march (the shadow kernel
// kept 8 of 32 lanes busy).  Here every lane runs one distance evaluation per
// iteration of a small state machine and takes the next job of the queue
// (one atomic per warp) once at least kWfRefill lanes are idle.  With kBatch
// each job's render (scene, parameters) is looked up from its sample index.
// Self-checks as in march_depth_persistent: a job may take at most
// max_steps + 64 iterations, a warp at most kMarchWallNs; a lane past either
// limit sets a bit in *flags and gives up.
constexpr unsigned kWfRefill = 8;

#define FT_WF_REFILL_TOP(live, queue_done, n_jobs, next_job, base_out, took)                       \
  if ((++loop_iters & 1023u) == 0u) {                                                            \
    unsigned long long now_ = lane == 0 ? ftd::global_ns() : 0ull;                               \
    now_ = __shfl_sync(0xffffffffu, now_, 0);                                                    \
    if (now_ - t_start > kMarchWallNs) {                                                         \
      if (lane == 0) atomicOr(flags, 1ull << 8);                                                 \
      break;                                                                                     \
    }                                                                                            \
  }                                                                                              \
  bool took = false;                                                                             \
  unsigned long long base_out = 0;                                                               \
  {                                                                                              \
    unsigned idle_ = __ballot_sync(0xffffffffu, !(live));                                        \
    if (!(queue_done) && (__popc(idle_) >= kWfRefill || idle_ == 0xffffffffu)) {                 \
      unsigned want_ = __popc(idle_);                                                            \
      unsigned long long b_ = 0;                                                                 \
      if (lane == 0) b_ = atomicAdd(next_job, static_cast<unsigned long long>(want_));           \
      b_ = __shfl_sync(0xffffffffu, b_, 0);                                                      \
      if (b_ >= (n_jobs)) queue_done = true;                                                     \
      if (!(live)) {                                                                             \
        base_out = b_ + __popc(idle_ & ((1u << lane) - 1u));                                     \
        took = base_out < (n_jobs);                                                              \
      }                                                                                          \
    }                                                                                            \
  }

enum WfPhase : int { kWfMarch = 0, kWfRefine = 1, kWfNormal = 2, kWfFinal = 3 };

// A missed ray adds the environment seen through its medium.  Out of line:
// the environment program's interpreter would otherwise be inlined at every
// miss site of the march loop, whose body has to stay within the
// instruction cache; a ray misses once, after all its steps.
__device__ __noinline__ void wf_add_miss(const DevScene& S, const RayParams& P, const WJob& wj,
                                         float* __restrict__ radiance) {
  RayJob J = job_of(wj);
  add_radiance(radiance, wj.sample, mul3(J.w, mul3(environment(S, J.d), transmittance(J.med, P.max_dist))));
}

// raymarch_hit (R:4091-4139) of every queued ray: march from the ray's
// secondary_min_t (R:4175-4178), ten bisections, the six-tap normal and the
// hit leaf's lookup (march_hit, one evaluation per iteration); a miss adds
// the environment seen through the ray's medium.  Five resident blocks per SM
// (the launch is five per SM): on the 512-primitive field's depth-6 trace,
// 181 ms of march per frame against 185 with six and 195 with four.
template <bool kBatch, bool kStats>
__global__ void __launch_bounds__(128, 5) wf_march_persistent(DevScene S0, RayParams P0, BatchView V,
                                                              const WJob* __restrict__ jobs,
                                                              const unsigned long long* __restrict__ count,
                                                              unsigned long long cap, WHit* __restrict__ hits,
                                                              float* __restrict__ radiance,
                                                              unsigned long long* __restrict__ next_job,
                                                              unsigned long long* __restrict__ flags,
                                                              unsigned long long* __restrict__ stats) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long n_jobs = min(*count, cap);
  Ctx<kStats> cx;
  cx.c = Counters{};
  const unsigned long long t_start = __shfl_sync(0xffffffffu, lane == 0 ? ftd::global_ns() : 0ull, 0);
  uint32_t loop_iters = 0;
  bool live = false, queue_done = false;
  unsigned long long job = 0;
  uint32_t item = 0, steps = 0, ray_iters = 0;
  int phase = kWfMarch, k = 0;
  F3 o = f3(0.0f, 0.0f, 0.0f), d = o, pos = o;
  float traveled = 0.0f, prev = 0.0f, max_t = 0.0f, lo = 0.0f, hi = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f;
  auto miss = [&](const DevScene& S, const RayParams& P) {
    wf_add_miss(S, P, jobs[job], radiance);
    hits[job].leaf = -1;
    live = false;
  };
  for (;;) {
    FT_WF_REFILL_TOP(live, queue_done, n_jobs, next_job, mine, took)
    if (took) {
      job = mine;
      const WJob& wj = jobs[job];
      if (wj.sample == kNoSample) {
        hits[job].leaf = -2;
      } else {
        item = kBatch ? sample_item(V, wj.sample) : 0u;
        const DevScene& S = kBatch ? V.scenes[item] : S0;
        const RayParams& P = kBatch ? V.params[item] : P0;
        o = f3(wj.o[0], wj.o[1], wj.o[2]);
        d = f3(wj.d[0], wj.d[1], wj.d[2]);
        float t0, t1;
        if (!ray_aabb(o, d, S.smin, S.smax, &t0, &t1)) {
          miss(S, P);
        } else {
          const float min_t = wj.depth == 0 ? 0.0f : P.eps * 2.0f;  // secondary_min_t (R:4175-4178)
          max_t = fminf(P.max_dist, t1);
          traveled = fmaxf(min_t, fmaxf(t0, 0.0f));
          prev = traveled;
          steps = 0;
          ray_iters = 0;
          phase = kWfMarch;
          live = true;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, live) == 0u) {
      if (queue_done) break;
      continue;
    }
    if (!live) continue;
    const DevScene& S = kBatch ? V.scenes[item] : S0;
    const RayParams& P = kBatch ? V.params[item] : P0;
    const float eps = P.eps;
    if (++ray_iters > P.max_steps + 64u) {
      atomicOr(flags, 1ull << (phase & 7));
      miss(S, P);
      continue;
    }
    if (phase == kWfMarch && (steps >= P.max_steps || traveled > max_t)) {
      miss(S, P);
      continue;
    }
    const float ne = fmaxf(eps * 4.0f, 1.0e-5f);
    F3 q;
    float mid = 0.0f;
    if (phase == kWfMarch) {
      q = o + d * traveled;
      cx.step();
    } else if (phase == kWfRefine) {
      mid = 0.5f * (lo + hi);
      q = o + d * mid;
    } else if (phase == kWfNormal) {
      float sgn = (k & 1) ? -ne : ne;
      q = pos;
      if (k < 2) q.x += sgn;
      else if (k < 4) q.y += sgn;
      else q.z += sgn;
    } else {
      q = pos;
    }
    if (phase == kWfFinal) {
      WHit h{};
      Info fin = scene_distance_leaf(S, pos, &h.leaf, cx);
      F3 nn = f3(nx, ny, nz);
      F3 nr = ftd::len3(nn) > 1.0e-8f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      h.t = hi;
      h.pos[0] = pos.x; h.pos[1] = pos.y; h.pos[2] = pos.z;
      h.normal[0] = nr.x; h.normal[1] = nr.y; h.normal[2] = nr.z;
      h.mat = fin.mat;
      h.obj = fin.obj;
      hits[job] = h;
      live = false;
      continue;
    }
    const float dq = scene_distance_inl(S, q, cx).d;
    if (phase == kWfMarch) {
      if (fabsf(dq) < eps) {
        lo = prev;
        hi = traveled;
        k = 0;
        phase = kWfRefine;
      } else {
        prev = traveled;
        traveled += fmaxf(fabsf(dq) * ftd::rclamp(P.step_scale, 0.05f, 1.0f), fmaxf(eps * 0.5f, 1.0e-5f));
        ++steps;
      }
    } else if (phase == kWfRefine) {
      if (fabsf(dq) < eps) hi = mid;
      else lo = mid;
      if (++k == 10) {
        pos = o + d * hi;
        k = 0;
        phase = kWfNormal;
      }
    } else {
      // dx = d(p + e x) - d(p - e x), one subtraction as march_hit
      if (k == 0) nx = dq;
      else if (k == 1) nx = nx - dq;
      else if (k == 2) ny = dq;
      else if (k == 3) ny = ny - dq;
      else if (k == 4) nz = dq;
      else nz = nz - dq;
      if (++k == 6) phase = kWfFinal;
    }
  }
  if (kStats) flush_stats(cx.c, stats);
}

// A step of shadow_visibility (R:4706-4733): the leaf-box lower bound when it
// exceeds max(8 eps, 0.02), else the exact distance.  With one or two leaves
// the lower bound's box bounds are the ones the exact evaluation orders its
// leaves by, so they are computed once; the values are those of
// scene_lower_bound and scene_distance_inl.
template <bool kStats>
__device__ __forceinline__ float shadow_step_h(const DevScene& S, F3 p, float eps, Ctx<kStats>& cx) {
  const DevBvhNode& root = S.bvh[S.bvh_root];
  int leaf = root.leaf, second = -1;
  float second_lb = kInf, lower;
  bool small = true;
  if (leaf >= 0) {
    cx.box();
    lower = node_lb(p, root.bmin, root.bmax);
  } else {
    const DevBvhNode& L = S.bvh[root.lhs];
    const DevBvhNode& R = S.bvh[root.rhs];
    if (L.leaf >= 0 && R.leaf >= 0) {
      cx.box(3);
      const float ll = node_lb(p, L.bmin, L.bmax), rl = node_lb(p, R.bmin, R.bmax);
      lower = fminf(ll, rl);
      const bool lfirst = ll <= rl;
      leaf = lfirst ? L.leaf : R.leaf;
      second = lfirst ? R.leaf : L.leaf;
      second_lb = lfirst ? rl : ll;
    } else {
      small = false;
      lower = scene_lower_bound(S, p, cx);
    }
  }
  lower = fabsf(lower);
  if (lower > fmaxf(eps * 8.0f, 0.02f)) return lower;
  cx.eval();
  return fabsf(small ? scene_distance_leaves<kStats, false>(S, p, leaf, second, second_lb, cx).d
                     : scene_distance_bvh(S, p, cx).d);
}

// shadow_visibility (R:4706-4733) of every queued shadow job, one step per
// iteration; the radiance gets contribution x visibility.
template <bool kBatch, bool kStats>
__global__ void __launch_bounds__(128, 8) wf_shadow_persistent(DevScene S0, RayParams P0, BatchView V,
                                                               const WShadow* __restrict__ shadows,
                                                               const unsigned long long* __restrict__ count,
                                                               unsigned long long cap, float* __restrict__ radiance,
                                                               unsigned long long* __restrict__ next_job,
                                                               unsigned long long* __restrict__ flags,
                                                               unsigned long long* __restrict__ stats) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long n_jobs = min(*count, cap);
  Ctx<kStats> cx;
  cx.c = Counters{};
  const unsigned long long t_start = __shfl_sync(0xffffffffu, lane == 0 ? ftd::global_ns() : 0ull, 0);
  uint32_t loop_iters = 0;
  bool live = false, queue_done = false;
  unsigned long long job = 0;
  uint32_t item = 0;
  int it = 0;
  F3 o = f3(0.0f, 0.0f, 0.0f), d = o;
  float t = 0.0f, max_t = 0.0f, vis = 1.0f;
  auto finish = [&](float v) {
    if (v > 0.0f) {
      const WShadow& sj = shadows[job];
      add_radiance(radiance, sj.sample, f3(sj.contrib[0], sj.contrib[1], sj.contrib[2]) * v);
    }
    live = false;
  };
  for (;;) {
    FT_WF_REFILL_TOP(live, queue_done, n_jobs, next_job, mine, took)
    if (took) {
      job = mine;
      const WShadow& sj = shadows[job];
      item = kBatch ? sample_item(V, sj.sample) : 0u;
      const RayParams& P = kBatch ? V.params[item] : P0;
      o = f3(sj.o[0], sj.o[1], sj.o[2]);
      d = f3(sj.d[0], sj.d[1], sj.d[2]);
      max_t = sj.max_t;
      t = P.eps * 2.0f;
      vis = 1.0f;
      it = 0;
      live = true;
    }
    if (__ballot_sync(0xffffffffu, live) == 0u) {
      if (queue_done) break;
      continue;
    }
    if (!live) continue;
    const DevScene& S = kBatch ? V.scenes[item] : S0;
    const RayParams& P = kBatch ? V.params[item] : P0;
    const float eps = P.eps;
    if (it >= 80 || t >= max_t) {
      finish(clamp01(vis));
      continue;
    }
    F3 p = o + d * t;
    const float h = shadow_step_h(S, p, eps, cx);
    if (h < eps * 4.0f) {
      finish(0.0f);
      continue;
    }
    vis = fminf(vis, clamp01(10.0f * h / t));
    t += fmaxf(h, eps * 2.0f);
    ++it;
  }
  if (kStats) flush_stats(cx.c, stats);
}

#undef FT_WF_REFILL_TOP

#ifndef FT_JIT
// Level-0 hits from a depth march of the same primary samples (the FP16 brick
// form of a trace): the depth march gives t, the hit mask and the six-tap
// normal per sample; the hit record takes the point o + d t and the leaf
// lookup there, as the wavefront march's final phase does, and a miss adds
// the environment.
__global__ void __launch_bounds__(128) wf_hits_from_depth_kernel(DevScene S, RayParams P,
                                                                 const WJob* __restrict__ jobs, unsigned long long n,
                                                                 const float* __restrict__ t_in,
                                                                 const uint8_t* __restrict__ mask_in,
                                                                 const float* __restrict__ normal_in,
                                                                 WHit* __restrict__ hits, float* __restrict__ radiance) {
  Ctx<false> cx;
  FT_GRID_STRIDE(i, n) {
    const WJob& wj = jobs[i];
    if (wj.sample == kNoSample) {
      hits[i].leaf = -2;
      continue;
    }
    const uint32_t s = wj.sample;
    const F3 o = f3(wj.o[0], wj.o[1], wj.o[2]);
    const F3 d = f3(wj.d[0], wj.d[1], wj.d[2]);
    if (!mask_in[s]) {
      RayJob J = job_of(wj);
      add_radiance(radiance, s, mul3(J.w, mul3(environment(S, J.d), transmittance(J.med, P.max_dist))));
      hits[i].leaf = -1;
      continue;
    }
    WHit h{};
    const float t = t_in[s];
    const F3 pos = o + d * t;
    Info fin = scene_distance_leaf(S, pos, &h.leaf, cx);
    h.t = t;
    h.pos[0] = pos.x; h.pos[1] = pos.y; h.pos[2] = pos.z;
    h.normal[0] = normal_in[3 * s]; h.normal[1] = normal_in[3 * s + 1]; h.normal[2] = normal_in[3 * s + 2];
    h.mat = fin.mat;
    h.obj = fin.obj;
    hits[i] = h;
  }
}

// ---------------------------------------------------------------- batches
// The same kernels over the queues of many renders at once (ft_batch): every
// job carries its global sample index, and the render it belongs to is the
// last whose first sample is not above it.  The counts stay on the device, so
// a batch captures its levels into one CUDA graph.


// Primary jobs of every render; the level-0 count is the work-item total.
__global__ void __launch_bounds__(128) wf_primary_batch_kernel(BatchView V, WJob* __restrict__ jobs,
                                                               unsigned long long* __restrict__ count) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = V.n_rays;
  FT_GRID_STRIDE(g, V.n_rays) {
    const uint32_t it = batch_item(V, g);
    const RayParams& P = V.params[it];
    F3 d;
    size_t idx = 0;
    WJob j{};
    if (item_ray(P, g - V.ray_first[it], &d, &idx)) {
      j.o[0] = P.origin[0]; j.o[1] = P.origin[1]; j.o[2] = P.origin[2];
      j.d[0] = d.x; j.d[1] = d.y; j.d[2] = d.z;
      j.w[0] = j.w[1] = j.w[2] = 1.0f;
      MediumD a = air();
      j.ior = a.ior;
      j.absorption[0] = a.absorption.x; j.absorption[1] = a.absorption.y; j.absorption[2] = a.absorption.z;
      j.density = a.density;
      j.depth = 0;
      j.sample = static_cast<uint32_t>(idx + V.out_first[it]);
    } else {
      j.sample = kNoSample;
    }
    jobs[g] = j;
  }
}

__global__ void __launch_bounds__(128) wf_shade_batch_kernel(BatchView V, const uint32_t* __restrict__ max_depth,
                                                             const WJob* __restrict__ jobs,
                                                             const unsigned long long* __restrict__ count,
                                                             unsigned long long cap, const WHit* __restrict__ hits,
                                                             WQueues Q) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) {
    if (hits[i].leaf < 0) continue;
    const uint32_t it = sample_item(V, jobs[i].sample);
    WQueues Qi = Q;
    Qi.max_depth = max_depth[it];
    wf_shade_job(V.scenes[it], V.params[it], jobs[i], hits[i], Qi, cx);
  }
}

#endif  // FT_JIT

#undef FT_GRID_STRIDE
