// The reference's MIS path tracer on the GPU: trace_path (renderer/path.rs:
// 3-112) with estimate_direct_mis / sample_one_light (R:4572-4704), the BSDF
// sampling and pdfs of materials/*.rs, and the progressive driver's per-pixel
// adaptive sampling (render_pathtrace_with_accel_progressive R:3974-4045,
// PixelAccumulator R:4778-4817).
//
// One thread renders one pixel: its samples 0, 1, ... each draw from an
// XorShift64 seeded by seed_pixel_sample (jitter, then the path's own
// draws), until spp or until the pixel's relative error falls to the noise
// threshold after min_spp samples.  A pixel's result depends on its own
// samples only, so this gives the reference's image, pass structure aside.
//
// Included by ft_kernels.cuh after the wavefront (precompiled only).
#pragma once

struct PathSettingsD {
  uint32_t spp, max_bounces, min_spp;
  float noise_threshold;
};

// raymarch_hit (R:4091-4139) from min_t: march, ten bisections, the six-tap
// normal and the hit leaf's lookup.
template <bool kStats>
__device__ bool march_hit(const DevScene& S, const RayParams& P, F3 o, F3 d, float min_t, TraceHit* h,
                          Ctx<kStats>& cx) {
  float t0, t1;
  if (!ray_aabb(o, d, S.smin, S.smax, &t0, &t1)) return false;
  const float max_t = fminf(P.max_dist, t1);
  float traveled = fmaxf(min_t, fmaxf(t0, 0.0f));
  float prev = traveled;
  const float eps = P.eps;
  const float scale = ftd::rclamp(P.step_scale, 0.05f, 1.0f);
  const float min_step = fmaxf(eps * 0.5f, 1.0e-5f);
  for (uint32_t s = 0; s < P.max_steps; ++s) {
    if (traveled > max_t) return false;
    cx.step();
    const float dq = scene_distance(S, o + d * traveled, cx).d;
    if (fabsf(dq) < eps) {
      float lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        const float mid = 0.5f * (lo + hi);
        if (fabsf(scene_d(S, o + d * mid, cx)) < eps) hi = mid;
        else lo = mid;
      }
      const F3 pos = o + d * hi;
      const float e = fmaxf(eps * 4.0f, 1.0e-5f);
      const float dx = scene_d(S, f3(pos.x + e, pos.y, pos.z), cx) - scene_d(S, f3(pos.x - e, pos.y, pos.z), cx);
      const float dy = scene_d(S, f3(pos.x, pos.y + e, pos.z), cx) - scene_d(S, f3(pos.x, pos.y - e, pos.z), cx);
      const float dz = scene_d(S, f3(pos.x, pos.y, pos.z + e), cx) - scene_d(S, f3(pos.x, pos.y, pos.z - e), cx);
      const F3 nn = f3(dx, dy, dz);
      h->normal = ftd::len3(nn) > 1.0e-8f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      const Info fin = scene_distance_leaf(S, pos, &h->leaf, cx);
      h->t = hi;
      h->pos = pos;
      h->mat = fin.mat;
      h->obj = fin.obj;
      return true;
    }
    prev = traveled;
    traveled += fmaxf(fabsf(dq) * scale, min_step);
  }
  return false;
}

// shadow_visibility (R:4706-4733)
template <bool kStats>
__device__ float shadow_visibility(const DevScene& S, F3 o, F3 d, float max_t, float eps, Ctx<kStats>& cx) {
  float t = eps * 2.0f;
  float vis = 1.0f;
  for (int i = 0; i < 80; ++i) {
    if (t >= max_t) return clamp01(vis);
    const F3 p = o + d * t;
    const float lower = fabsf(scene_lower_bound(S, p, cx));
    const float h = lower > fmaxf(eps * 8.0f, 0.02f) ? lower : fabsf(scene_distance(S, p, cx).d);
    if (h < eps * 4.0f) return 0.0f;
    vis = fminf(vis, clamp01(10.0f * h / t));
    t += fmaxf(h, eps * 2.0f);
  }
  return clamp01(vis);
}

// ---------------------------------------------------------------- BSDF sampling
struct BsdfSampleD {  // BsdfSample (materials/mod.rs:232-241)
  F3 wi, f;
  float pdf;
  bool delta, apply_cos, transmission, thin_walled;
  float next_ior;
};
struct SampleInD {  // SampleInput (materials/mod.rs:243-250)
  bool front_face;
  float current_ior, u1, u2, u3;
};

// to_world (lambert.rs:52-61, metal.rs:65-74)
__device__ F3 to_world(F3 normal, float x, float y, float z) {
  const F3 n = ftd::normalize3(normal);
  const F3 helper = fabsf(n.y) < 0.99f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
  const F3 t = ftd::normalize3(ftd::cross3(helper, n));
  const F3 b = ftd::normalize3(ftd::cross3(n, t));
  return ftd::normalize3((t * x + b * y) + n * z);
}
__device__ __forceinline__ F3 reflect_about(F3 v, F3 n) { return v - n * (2.0f * ftd::dot3(v, n)); }
__device__ __forceinline__ float lambert_pdf(F3 n, F3 wi) { return fmaxf(ftd::dot3(n, wi), 0.0f) / kPi; }

// lambert.rs:15-50
__device__ BsdfSampleD lambert_sample(const DParams& m, F3 n, const SampleInD& in) {
  const float uu1 = ftd::rclamp(in.u1, 1.0e-6f, 1.0f - 1.0e-6f), uu2 = ftd::rclamp(in.u2, 1.0e-6f, 1.0f - 1.0e-6f);
  const float r = sqrtf(uu1), phi = 2.0f * kPi * uu2;
  const F3 wi = to_world(n, r * cosf(phi), r * sinf(phi), sqrtf(1.0f - uu1));
  const F3 f = ftd::dot3(n, wi) <= 0.0f ? f3(0.0f, 0.0f, 0.0f) : m.color * (1.0f / kPi);
  return BsdfSampleD{wi, f, fmaxf(lambert_pdf(n, wi), 1.0e-6f), false, true, false, false, in.current_ior};
}

// metal.rs:22-63
__device__ float metal_pdf(float roughness, F3 n, F3 wi, F3 wo) {
  if (ftd::dot3(n, wi) <= 0.0f || ftd::dot3(n, wo) <= 0.0f) return 0.0f;
  const F3 h = ftd::normalize3(wi + wo);
  const float ndoth = fmaxf(ftd::dot3(n, h), 0.0f), vdoth = fmaxf(fabsf(ftd::dot3(wo, h)), 1.0e-6f);
  const float rr = ftd::rclamp(roughness, 0.02f, 1.0f);
  return fmaxf(ggx_d(ndoth, rr * rr) * ndoth / (4.0f * vdoth), 0.0f);
}
__device__ BsdfSampleD metal_sample(F3 color, float roughness, F3 n, F3 wo, const SampleInD& in) {
  const float rr = ftd::rclamp(roughness, 0.02f, 1.0f);
  const float alpha = rr * rr;
  const float uu1 = ftd::rclamp(in.u1, 1.0e-6f, 1.0f - 1.0e-6f), uu2 = ftd::rclamp(in.u2, 1.0e-6f, 1.0f - 1.0e-6f);
  const float phi = 2.0f * kPi * uu2;
  const float cos_t = sqrtf((1.0f - uu1) / (1.0f + (alpha * alpha - 1.0f) * uu1));
  const float sin_t = sqrtf(fmaxf(1.0f - cos_t * cos_t, 0.0f));
  const F3 h = to_world(n, sin_t * cosf(phi), sin_t * sinf(phi), cos_t);
  const F3 wi = ftd::normalize3(reflect_about(wo * -1.0f, h));
  return BsdfSampleD{wi, metal_eval(color, roughness, n, wi, wo), fmaxf(metal_pdf(roughness, n, wi, wo), 1.0e-6f),
                     false, true, false, false, in.current_ior};
}

// dielectric.rs:13-79
__device__ BsdfSampleD dielectric_sample(F3 color, float ior_in, bool thin, F3 normal, F3 wo, const SampleInD& in) {
  const float ior = ftd::rclamp(ior_in, 1.0f, 3.0f);
  float eta_i, eta_t, next_ior;
  if (thin) { eta_i = 1.0f; eta_t = 1.0f; next_ior = in.current_ior; }
  else if (in.front_face) { eta_i = in.current_ior; eta_t = ior; next_ior = ior; }
  else { eta_i = in.current_ior; eta_t = 1.0f; next_ior = 1.0f; }
  const F3 n = ftd::normalize3(normal), incident = wo * -1.0f;
  const float fresnel = clamp01(fresnel_dielectric(fabsf(ftd::dot3(n, wo)), eta_i, eta_t));
  if (in.u1 < fresnel)
    return BsdfSampleD{ftd::normalize3(reflect_about(incident, n)), f3(1.0f, 1.0f, 1.0f), fmaxf(fresnel, 1.0e-6f),
                       true, false, false, thin, in.current_ior};
  F3 wt;
  if (refract_dir(incident, n, eta_i / eta_t, &wt))
    return BsdfSampleD{ftd::normalize3(wt), color, fmaxf(1.0f - fresnel, 1.0e-6f), true, false, true, thin, next_ior};
  return BsdfSampleD{ftd::normalize3(reflect_about(incident, n)), f3(1.0f, 1.0f, 1.0f), 1.0f, true, false, false, thin,
                     in.current_ior};
}

// standard.rs:45-160: lobe weights, pdf and sample
__device__ void standard_weights(const DParams& m, F3 n, F3 wo, float* dw, float* sw, float* cw) {
  const float metallic = clamp01(m.metallic), transmission = clamp01(m.transmission), clearcoat = clamp01(m.clearcoat);
  const float cx = clamp01(1.0f - clamp01(fmaxf(ftd::dot3(n, wo), 0.0f)));
  const float x2 = cx * cx;
  const float coat = ftd::rclamp(clearcoat * (0.2f + 0.8f * (x2 * x2 * cx)) * 0.65f, 0.0f, 0.95f);
  *dw = fmaxf((1.0f - metallic) * (1.0f - transmission), 0.0f) * (1.0f - coat);
  *sw = clamp01((m.specular * m.specular_weight) * (1.0f - transmission)) * (1.0f - coat * 0.85f);
  *cw = clearcoat * 0.18f;
}
__device__ float standard_pdf(const DParams& m, F3 n, F3 wi, F3 wo) {
  float dw, sw, cw;
  standard_weights(m, n, wo, &dw, &sw, &cw);
  const float sum = dw + sw + cw;
  if (sum <= 1.0e-6f) return lambert_pdf(n, wi);
  return (dw / sum) * lambert_pdf(n, wi) + (sw / sum) * metal_pdf(m.roughness, n, wi, wo) +
         (cw / sum) * metal_pdf(ftd::rclamp(m.clearcoat_roughness, 0.02f, 1.0f), n, wi, wo);
}
__device__ BsdfSampleD standard_sample(const DParams& m, F3 n, F3 wo, const SampleInD& in) {
  float dw, sw, cw;
  standard_weights(m, n, wo, &dw, &sw, &cw);
  const float tw = clamp01(m.transmission);
  const float sum = dw + sw + cw + tw;
  if (sum <= 1.0e-6f) return lambert_sample(m, n, in);
  const float pick = clamp01(in.u3) * sum;
  BsdfSampleD s;
  if (pick < dw) {
    s = lambert_sample(m, n, in);
  } else if (pick < dw + sw) {
    // blended_f0 (standard.rs:168-175), standard.rs's unclamped lerp
    const float f0d = clamp01(f0_from_ior(m.ior));
    const F3 base = mul3(f3(f0d, f0d, f0d) * (clamp01(m.specular) * clamp01(m.specular_weight)), m.spec_color);
    const float met = clamp01(m.metallic);
    s = metal_sample(base * (1.0f - met) + m.color * met, m.roughness, n, wo, in);
  } else if (pick < dw + sw + cw) {
    s = metal_sample(f3(1.0f, 1.0f, 1.0f), ftd::rclamp(m.clearcoat_roughness, 0.02f, 1.0f), n, wo, in);
  } else {
    s = dielectric_sample(m.color, m.ior, m.thin != 0, n, wo, in);
    s.f = s.transmission ? m.color : standard_eval(m, n, s.wi, wo);
    s.pdf = s.delta ? fmaxf(s.pdf, 1.0e-6f) : fmaxf(standard_pdf(m, n, s.wi, wo), 1.0e-6f);
    return s;
  }
  s.f = standard_eval(m, n, s.wi, wo);
  s.pdf = fmaxf(standard_pdf(m, n, s.wi, wo), 1.0e-6f);
  return s;
}

__device__ float model_pdf(int model, const DParams& p, F3 n, F3 wi, F3 wo) {
  switch (model) {
    case FT_MAT_STANDARD: return standard_pdf(p, n, wi, wo);
    case FT_MAT_LAMBERT: return lambert_pdf(n, wi);
    case FT_MAT_METAL: return metal_pdf(p.roughness, n, wi, wo);
    default: return 0.0f;  // dielectric.rs:9-11
  }
}
__device__ BsdfSampleD model_sample(int model, const DParams& p, F3 n, F3 wo, const SampleInD& in) {
  switch (model) {
    case FT_MAT_STANDARD: return standard_sample(p, n, wo, in);
    case FT_MAT_LAMBERT: return lambert_sample(p, n, in);
    case FT_MAT_METAL: return metal_sample(p.color, p.roughness, n, wo, in);
    default: return dielectric_sample(p.color, p.ior, p.thin != 0, n, wo, in);
  }
}
// Material::pdf / Material::sample incl. sample_blend (materials/mod.rs:312-340, 399-432)
__device__ float mat_pdf(const DMat& m, F3 n, F3 wi, F3 wo) {
  if (m.kind != kBlendKind) return model_pdf(m.kind, m.a, n, wi, wo);
  const float t = clamp01(m.t);
  return model_pdf(m.a_model, m.a, n, wi, wo) * (1.0f - t) + model_pdf(m.b_model, m.b, n, wi, wo) * t;
}
__device__ BsdfSampleD mat_sample(const DMat& m, F3 n, F3 wo, const SampleInD& in) {
  if (m.kind != kBlendKind) return model_sample(m.kind, m.a, n, wo, in);
  const float t = clamp01(m.t);
  const BsdfSampleD c = in.u3 < t ? model_sample(m.b_model, m.b, n, wo, in) : model_sample(m.a_model, m.a, n, wo, in);
  BsdfSampleD out = c;
  out.f = lerp_sp(model_eval(m.a_model, m.a, n, c.wi, wo), model_eval(m.b_model, m.b, n, c.wi, wo), t);
  out.pdf = fmaxf(model_pdf(m.a_model, m.a, n, c.wi, wo) * (1.0f - t) + model_pdf(m.b_model, m.b, n, c.wi, wo) * t,
                  1.0e-6f);
  out.delta = c.delta && m.a_model == FT_MAT_DIELECTRIC && m.b_model == FT_MAT_DIELECTRIC;
  return out;
}

__device__ __forceinline__ float luminance(F3 s) { return 0.2126f * s.x + 0.7152f * s.y + 0.0722f * s.z; }
__device__ __forceinline__ F3 clamp_luma(F3 s, float max_luma) {  // clamp_spectrum (R:5168-5175)
  const float l = luminance(s);
  return (l <= max_luma || l <= 1.0e-6f) ? s : s * (max_luma / l);
}
__device__ __forceinline__ float power_heuristic(float pa, float pb) {  // R:5098-5102
  const float a2 = pa * pa, b2 = pb * pb;
  return a2 / fmaxf(a2 + b2, 1.0e-6f);
}

// BsdfContextBase (R:4397-4449): the BSDF context with its shading normal
// and wo, and the geometric normal of the hit facing the ray
struct PathCtxD {
  F3 normal, wo, hit_normal;
  bool front;
  float current_ior;
  BsdfCtx b;
};

// pdf_bsdf (R:4922-4933): the material definition's `fn pdf(ctx)` (at least
// 0), else Material::pdf.
__device__ float bsdf_pdf(const DevScene& S, const DMat& m, const PathCtxD& c, F3 wi) {
  const int prog = bsdf_hook(S, m, FT_HOOK_PDF);
  if (prog < 0) return mat_pdf(m, c.normal, wi, c.wo);
  F3 a[FT_BSDF_HOOK_PARAMS];
  bsdf_args(c.b, wi, 0.0f, 0.0f, 0.0f, a);
  return fmaxf(scene_program(S, prog, a, nullptr).x, 0.0f);
}

// sample_bsdf_lobe (R:4869-4903): the material definition's `fn sample(ctx)`
// (sample_bsdf_ft R:4934-4950, its context's wi the normal), read as
// bsdf_sample_from_value (R:5032-5060) does, else Material::sample.
__device__ BsdfSampleD bsdf_sample(const DevScene& S, const DMat& m, const PathCtxD& c, const SampleInD& in) {
  const int dyn = dom_params(m).dyn;
  const int32_t* hp = dyn >= 0 ? S.materials[dyn].hook_program : nullptr;
  if (!hp || hp[FT_HOOK_SAMPLE_WI] < 0 || hp[FT_HOOK_SAMPLE_F] < 0) return mat_sample(m, c.normal, c.wo, in);
  F3 a[FT_BSDF_HOOK_PARAMS];
  bsdf_args(c.b, c.b.normal, in.u1, in.u2, in.u3, a);
  auto num = [&](int slot, float dflt) { return hp[slot] >= 0 ? scene_program(S, hp[slot], a, nullptr).x : dflt; };
  BsdfSampleD r;
  r.wi = scene_program(S, hp[FT_HOOK_SAMPLE_WI], a, nullptr);
  r.f = hook_colour(S, hp[FT_HOOK_SAMPLE_F], a);
  r.pdf = fmaxf(num(FT_HOOK_SAMPLE_PDF, 0.0f), 0.0f);
  r.delta = num(FT_HOOK_SAMPLE_DELTA, 0.0f) >= 0.5f;
  r.apply_cos = num(FT_HOOK_SAMPLE_APPLY_COS, 1.0f) >= 0.5f;
  r.transmission = num(FT_HOOK_SAMPLE_TRANSMISSION, 0.0f) >= 0.5f;
  r.thin_walled = num(FT_HOOK_SAMPLE_THIN_WALLED, 0.0f) >= 0.5f;
  r.next_ior = ftd::rclamp(num(FT_HOOK_SAMPLE_NEXT_IOR, 1.0f), 1.0f, 3.0f);
  return r;
}

// env_light_pdf_for_dir (R:4336-4355)
__device__ float env_light_pdf(const DevScene& S, const DMat& m, const PathCtxD& c, F3 wi) {
  if (S.n_lights == 0) return 0.0f;
  float env = 0.0f;
  for (int i = 0; i < S.n_lights; ++i) env += S.lights[i].kind == FT_LIGHT_ENV ? 1.0f : 0.0f;
  if (env <= 0.0f) return 0.0f;
  return (env / static_cast<float>(S.n_lights)) * fmaxf(bsdf_pdf(S, m, c, wi), 1.0e-6f);
}

// estimate_direct_mis with sample_one_light (R:4572-4675): one light chosen
// uniformly; point and sphere lights as points, the environment light by
// cosine sampling around the normal (cosine_sample_hemisphere R:4676-4695).
template <bool kStats>
__device__ F3 estimate_direct_mis(const DevScene& S, const RayParams& P, const DMat& m, F3 p, const PathCtxD& c,
                                  XorShift64& rng, Ctx<kStats>& cx) {
  if (S.n_lights == 0) return f3(0.0f, 0.0f, 0.0f);
  const float count = static_cast<float>(S.n_lights);
  const int idx = min(static_cast<int>(floorf(rng.next_f32() * count)), S.n_lights - 1);
  const ft_light& L = S.lights[idx];
  const float select_pdf = 1.0f / count;
  F3 wi, rad;
  float pdf, max_t;
  bool delta;
  if (L.kind == FT_LIGHT_ENV) {
    const float u1 = ftd::rclamp(rng.next_f32(), 1.0e-6f, 1.0f - 1.0e-6f);
    const float u2 = ftd::rclamp(rng.next_f32(), 1.0e-6f, 1.0f - 1.0e-6f);
    const float r = sqrtf(u1), phi = 2.0f * kPi * u2;
    wi = to_world(c.normal, r * cosf(phi), r * sinf(phi), sqrtf(1.0f - u1));
    const float env_pdf = fmaxf(fmaxf(ftd::dot3(c.normal, wi), 0.0f) / kPi, 1.0e-6f);
    rad = f3(L.intensity[0], L.intensity[1], L.intensity[2]);
    pdf = select_pdf * fmaxf(env_pdf, 1.0e-6f);
    max_t = kInf;
    delta = false;
  } else {
    const F3 to_light = f3(L.position[0], L.position[1], L.position[2]) - p;
    const float dist = fmaxf(ftd::len3(to_light), 1.0e-4f);
    wi = to_light * (1.0f / dist);
    rad = f3(L.intensity[0], L.intensity[1], L.intensity[2]) * (1.0f / (dist * dist));
    pdf = select_pdf;
    max_t = dist - 1.0e-4f;
    delta = true;
  }
  if (pdf <= 1.0e-6f) return f3(0.0f, 0.0f, 0.0f);
  const float cos_t = fmaxf(ftd::dot3(c.normal, wi), 0.0f);
  if (cos_t <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
  const F3 so = offset_origin(p, c.hit_normal, wi, P.eps);
  const float vis = shadow_visibility(S, so, wi, max_t, P.eps, cx);
  if (vis <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
  const F3 f = bsdf_eval(S, m, c.b, wi);
  const float bpdf = fmaxf(bsdf_pdf(S, m, c, wi), 1.0e-6f);
  const float w = delta ? 1.0f : power_heuristic(pdf, bpdf);
  return mul3(f, rad) * ((cos_t * vis * w) / fmaxf(pdf, 1.0e-6f));
}

// trace_path (renderer/path.rs:3-112)
template <bool kStats>
__device__ F3 trace_path(const DevScene& S, const RayParams& P, F3 origin, F3 dir, uint32_t max_bounces,
                         XorShift64& rng, Ctx<kStats>& cx) {
  F3 throughput = f3(1.0f, 1.0f, 1.0f), radiance = f3(0.0f, 0.0f, 0.0f);
  bool have_prev = false;
  float prev_pdf = 0.0f;
  PathCtxD prev_ctx{};
  DMat prev_mat;
  MediumD medium = air();
  const float eps = P.eps;
  for (uint32_t bounce = 0; bounce < max_bounces; ++bounce) {
    const float min_t = bounce == 0 ? 0.0f : eps * 2.0f;  // secondary_min_t (R:4175-4178)
    TraceHit h;
    if (!march_hit(S, P, origin, dir, min_t, &h, cx)) {
      const F3 env = mul3(environment(S, dir), transmittance(medium, P.max_dist));
      float weight = 1.0f;
      if (have_prev)
        weight = power_heuristic(fmaxf(prev_pdf, 1.0e-6f), fmaxf(env_light_pdf(S, prev_mat, prev_ctx, dir), 1.0e-6f));
      radiance = radiance + mul3(throughput, env) * weight;
      break;
    }
    throughput = mul3(throughput, transmittance(medium, h.t));
    const bool front = ftd::dot3(h.normal, dir) < 0.0f;
    PathCtxD c;
    c.front = front;
    c.hit_normal = front ? ftd::normalize3(h.normal) : ftd::normalize3(h.normal * -1.0f);
    c.wo = ftd::normalize3(dir * -1.0f);
    c.current_ior = medium.ior;
    const HookCtx hc{h.pos, c.hit_normal, c.wo, front ? 1.0f : 0.0f};
    Resolved rs;
    resolve_hit(S, h.leaf, h.pos, hc, &rs, cx, false);
    c.normal = rs.ok ? ftd::normalize3(front ? rs.normal : rs.normal * -1.0f) : c.hit_normal;
    c.b.pos = h.pos;
    c.b.local = object_local(S, h.obj, h.pos);
    c.b.normal = c.normal;
    c.b.wo = c.wo;
    c.b.front = front ? 1.0f : 0.0f;
    c.b.obj = static_cast<float>(h.obj);
    c.b.mat = static_cast<float>(h.mat);
    c.b.current_ior = c.current_ior;
    c.normal = hooked_shading_normal(S, c.b, dir * -1.0f, h.mat);
    c.b.normal = c.normal;
    const DMat m = rs.ok ? rs.m : mat_of_id(S, h.mat);
    const F3 em = mat_emission(m);
    if (em.x > 0.0f || em.y > 0.0f || em.z > 0.0f) radiance = radiance + mul3(throughput, em);
    const F3 direct = estimate_direct_mis(S, P, m, h.pos, c, rng, cx);
    radiance = radiance + clamp_luma(mul3(throughput, direct), 12.0f);
    // sample_bsdf_lobe (R:4870-4903): three draws
    SampleInD in;
    in.front_face = front;
    in.current_ior = c.current_ior;
    in.u1 = rng.next_f32();
    in.u2 = rng.next_f32();
    in.u3 = rng.next_f32();
    const BsdfSampleD smp = bsdf_sample(S, m, c, in);
    if (smp.pdf <= 1.0e-6f) break;
    if (smp.apply_cos) {
      const float ct = fmaxf(ftd::dot3(c.normal, smp.wi), 0.0f);
      if (ct <= 0.0f) break;
      throughput = mul3(throughput, smp.f * (ct / fmaxf(smp.pdf, 1.0e-6f)));
    } else {
      throughput = mul3(throughput, smp.f * (1.0f / fmaxf(smp.pdf, 1.0e-6f)));
    }
    throughput = clamp_luma(throughput, 8.0f);
    if (smp.delta) {
      have_prev = false;
    } else {
      have_prev = true;
      prev_pdf = fmaxf(smp.pdf, 1.0e-6f);
      prev_ctx = c;
      prev_mat = m;
    }
    if (bounce >= 2) {  // Russian roulette
      const float pr = ftd::rclamp(luminance(throughput), 0.05f, 0.98f);
      if (rng.next_f32() > pr) break;
      throughput = throughput * (1.0f / pr);
    }
    dir = ftd::normalize3(smp.wi);
    if (smp.transmission && !smp.thin_walled) {
      medium = transition(m, front, medium);
      medium.ior = ftd::rclamp(smp.next_ior, 1.0f, 3.0f);
      origin = offset_origin(h.pos, c.hit_normal, dir, eps * 8.0f);
    } else {
      origin = offset_origin(h.pos, c.hit_normal, dir, eps);
    }
  }
  return radiance;
}

// One pixel per thread: the progressive renderer's samples with adaptive
// stopping.  Outputs the average (linear), its spectrum_to_rgb8 (R:5221-5227)
// and the samples taken.
template <bool kStats>
__global__ void __launch_bounds__(128) path_pixel_kernel(DevScene S, RayParams P, PathSettingsD ps,
                                                         float* __restrict__ rgb_out, uint8_t* __restrict__ rgb8_out,
                                                         uint32_t* __restrict__ count_out,
                                                         unsigned long long* __restrict__ stats) {
  const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t n_pixels = static_cast<uint64_t>(P.width) * P.height;
  Ctx<kStats> cx;
  cx.c = Counters{};
  if (i < n_pixels) {
    const uint32_t x = static_cast<uint32_t>(i % P.width), y = static_cast<uint32_t>(i / P.width);
    const F3 o = f3(P.origin[0], P.origin[1], P.origin[2]);
    const F3 fwd = f3(P.fwd[0], P.fwd[1], P.fwd[2]), rt = f3(P.right[0], P.right[1], P.right[2]);
    const F3 up = f3(P.up[0], P.up[1], P.up[2]);
    F3 sum = f3(0.0f, 0.0f, 0.0f);
    uint32_t count = 0;
    float mean = 0.0f, m2 = 0.0f;
    for (uint32_t s = 0; s < ps.spp; ++s) {
      XorShift64 rng(seed_pixel_sample(x, y, P.width, s));
      const float jx = rng.next_f32() - 0.5f;
      const float jy = rng.next_f32() - 0.5f;
      const float px = (((static_cast<float>(x) + 0.5f + jx) / static_cast<float>(P.width)) * 2.0f - 1.0f) * P.aspect;
      const float py = 1.0f - ((static_cast<float>(y) + 0.5f + jy) / static_cast<float>(P.height)) * 2.0f;
      const F3 d = ftd::normalize3(ftd::normalize3(fwd + rt * (px * P.tan_fov) + up * (py * P.tan_fov)));
      const F3 c = trace_path(S, P, o, d, ps.max_bounces, rng, cx);
      // PixelAccumulator::add_sample
      sum = sum + c;
      count += 1;
      const float xl = luminance(c);
      const float delta = xl - mean;
      mean += delta / static_cast<float>(count);
      m2 += delta * (xl - mean);
      if (ps.noise_threshold > 0.0f && count >= ps.min_spp && count >= 2) {
        const float n = static_cast<float>(count);
        const float var = fmaxf(m2 / (n - 1.0f), 0.0f);
        if (sqrtf(var / n) / fmaxf(fabsf(mean), 1.0e-4f) <= ps.noise_threshold) break;
      }
    }
    const F3 avg = count ? sum * (1.0f / static_cast<float>(count)) : f3(0.0f, 0.0f, 0.0f);
    if (rgb_out) {
      rgb_out[3 * i] = avg.x;
      rgb_out[3 * i + 1] = avg.y;
      rgb_out[3 * i + 2] = avg.z;
    }
    if (rgb8_out) {
      rgb8_out[3 * i] = gamma_u8(avg.x);
      rgb8_out[3 * i + 1] = gamma_u8(avg.y);
      rgb8_out[3 * i + 2] = gamma_u8(avg.z);
    }
    if (count_out) count_out[i] = count;
  }
  if (kStats) flush_stats(cx.c, stats);
}
