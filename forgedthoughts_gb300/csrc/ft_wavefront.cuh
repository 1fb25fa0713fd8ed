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

struct WJob {
  float o[3], d[3], w[3];
  float ior, absorption[3], density;
  int32_t depth;
  uint32_t sample;
};

struct WHit {
  float t, pos[3], normal[3];
  uint32_t mat;
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

// One queued ray: march it; a miss adds the environment, a hit is recorded.
__device__ __forceinline__ void wf_march_job(const DevScene& S, const RayParams& P, const WJob& wj, WHit* out,
                                             float* radiance, Ctx<false>& cx) {
  WHit h_out{};
  RayJob J = job_of(wj);
  float min_t = J.depth == 0 ? 0.0f : P.eps * 2.0f;  // secondary_min_t (R:4175-4178)
  TraceHit h;
  if (!march_hit(S, P, J.o, J.d, min_t, &h, cx)) {
    add_radiance(radiance, wj.sample, mul3(J.w, mul3(environment(S, J.d), transmittance(J.med, P.max_dist))));
    h_out.leaf = -1;
  } else {
    h_out.t = h.t;
    h_out.pos[0] = h.pos.x; h_out.pos[1] = h.pos.y; h_out.pos[2] = h.pos.z;
    h_out.normal[0] = h.normal.x; h_out.normal[1] = h.normal.y; h_out.normal[2] = h.normal.z;
    h_out.mat = h.mat;
    h_out.leaf = h.leaf;
  }
  *out = h_out;
}

// One recorded hit: shade it into the queues.
__device__ __forceinline__ void wf_shade_job(const DevScene& S, const RayParams& P, const WJob& wj, const WHit& wh,
                                             const WQueues& Q, Ctx<false>& cx) {
  TraceHit h;
  h.t = wh.t;
  h.pos = f3(wh.pos[0], wh.pos[1], wh.pos[2]);
  h.normal = f3(wh.normal[0], wh.normal[1], wh.normal[2]);
  h.mat = wh.mat;
  h.leaf = wh.leaf;
  RayJob J = job_of(wj);
  QueueSink sink{Q, wj.sample};
  shade_hit(S, P, J, h, sink, cx);
}

// One shadow job: its visibility times its contribution.
__device__ __forceinline__ void wf_shadow_job(const DevScene& S, const RayParams& P, const WShadow& sj,
                                              float* radiance, Ctx<false>& cx) {
  float vis = shadow_visibility(S, f3(sj.o[0], sj.o[1], sj.o[2]), f3(sj.d[0], sj.d[1], sj.d[2]), sj.max_t, P.eps, cx);
  if (vis > 0.0f) add_radiance(radiance, sj.sample, f3(sj.contrib[0], sj.contrib[1], sj.contrib[2]) * vis);
}

#define FT_GRID_STRIDE(i, n)                                                                             \
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; \
       i < (n); i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)

__global__ void __launch_bounds__(128) wf_march_kernel(DevScene S, RayParams P, const WJob* __restrict__ jobs,
                                                       const unsigned long long* __restrict__ count,
                                                       unsigned long long cap, WHit* __restrict__ hits,
                                                       float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);  // a queue that overflowed holds cap jobs
  FT_GRID_STRIDE(i, n) {
    if (jobs[i].sample == kNoSample) {
      hits[i].leaf = -2;
      continue;
    }
    wf_march_job(S, P, jobs[i], &hits[i], radiance, cx);
  }
}

__global__ void __launch_bounds__(128) wf_shade_kernel(DevScene S, RayParams P, const WJob* __restrict__ jobs,
                                                       const unsigned long long* __restrict__ count,
                                                       unsigned long long cap, const WHit* __restrict__ hits,
                                                       WQueues Q) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) {
    if (hits[i].leaf < 0) continue;
    wf_shade_job(S, P, jobs[i], hits[i], Q, cx);
  }
}

__global__ void __launch_bounds__(128) wf_shadow_kernel(DevScene S, RayParams P, const WShadow* __restrict__ shadows,
                                                        const unsigned long long* __restrict__ count,
                                                        unsigned long long cap, float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) wf_shadow_job(S, P, shadows[i], radiance, cx);
}

#ifndef FT_JIT
// ---------------------------------------------------------------- batches
// The same kernels over the queues of many renders at once (ft_batch): every
// job carries its global sample index, and the render it belongs to is the
// last whose first sample is not above it.  The counts stay on the device, so
// a batch captures its levels into one CUDA graph.

__device__ __forceinline__ uint32_t sample_item(const BatchView& V, uint64_t sample) {
  uint32_t lo = 0, hi = V.n_items;  // out_first[lo] <= sample < out_first[hi]
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (V.out_first[mid] <= sample) lo = mid;
    else hi = mid;
  }
  return lo;
}

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

__global__ void __launch_bounds__(128) wf_march_batch_kernel(BatchView V, const WJob* __restrict__ jobs,
                                                             const unsigned long long* __restrict__ count,
                                                             unsigned long long cap, WHit* __restrict__ hits,
                                                             float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) {
    if (jobs[i].sample == kNoSample) {
      hits[i].leaf = -2;
      continue;
    }
    const uint32_t it = sample_item(V, jobs[i].sample);
    wf_march_job(V.scenes[it], V.params[it], jobs[i], &hits[i], radiance, cx);
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

__global__ void __launch_bounds__(128) wf_shadow_batch_kernel(BatchView V, const WShadow* __restrict__ shadows,
                                                              const unsigned long long* __restrict__ count,
                                                              unsigned long long cap, float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = min(*count, cap);
  FT_GRID_STRIDE(i, n) {
    const uint32_t it = sample_item(V, shadows[i].sample);
    wf_shadow_job(V.scenes[it], V.params[it], shadows[i], radiance, cx);
  }
}
#endif  // FT_JIT

#undef FT_GRID_STRIDE
