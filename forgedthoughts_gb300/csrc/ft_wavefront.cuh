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

__global__ void __launch_bounds__(128) wf_march_kernel(DevScene S, RayParams P, const WJob* __restrict__ jobs,
                                                       const unsigned long long* __restrict__ count,
                                                       WHit* __restrict__ hits, float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = *count;
  const float eps = P.eps;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const WJob& wj = jobs[i];
    WHit out{};
    if (wj.sample == kNoSample) {
      out.leaf = -2;
      hits[i] = out;
      continue;
    }
    RayJob J = job_of(wj);
    float min_t = J.depth == 0 ? 0.0f : eps * 2.0f;  // secondary_min_t (R:4175-4178)
    TraceHit h;
    if (!march_hit(S, P, J.o, J.d, min_t, &h, cx)) {
      add_radiance(radiance, wj.sample, mul3(J.w, mul3(environment(S, J.d), transmittance(J.med, P.max_dist))));
      out.leaf = -1;
    } else {
      out.t = h.t;
      out.pos[0] = h.pos.x; out.pos[1] = h.pos.y; out.pos[2] = h.pos.z;
      out.normal[0] = h.normal.x; out.normal[1] = h.normal.y; out.normal[2] = h.normal.z;
      out.mat = h.mat;
      out.leaf = h.leaf;
    }
    hits[i] = out;
  }
}

__global__ void __launch_bounds__(128) wf_shade_kernel(DevScene S, RayParams P, const WJob* __restrict__ jobs,
                                                       const unsigned long long* __restrict__ count,
                                                       const WHit* __restrict__ hits, WQueues Q) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = *count;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const WHit& wh = hits[i];
    if (wh.leaf < 0) continue;
    TraceHit h;
    h.t = wh.t;
    h.pos = f3(wh.pos[0], wh.pos[1], wh.pos[2]);
    h.normal = f3(wh.normal[0], wh.normal[1], wh.normal[2]);
    h.mat = wh.mat;
    h.leaf = wh.leaf;
    RayJob J = job_of(jobs[i]);
    QueueSink sink{Q, jobs[i].sample};
    shade_hit(S, P, J, h, sink, cx);
  }
}

__global__ void __launch_bounds__(128) wf_shadow_kernel(DevScene S, RayParams P, const WShadow* __restrict__ shadows,
                                                        const unsigned long long* __restrict__ count,
                                                        float* __restrict__ radiance) {
  Ctx<false> cx;
  cx.c = Counters{};
  const unsigned long long n = *count;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const WShadow& s = shadows[i];
    float vis = shadow_visibility(S, f3(s.o[0], s.o[1], s.o[2]), f3(s.d[0], s.d[1], s.d[2]), s.max_t, P.eps, cx);
    if (vis > 0.0f) add_radiance(radiance, s.sample, f3(s.contrib[0], s.contrib[1], s.contrib[2]) * vis);
  }
}
