// Whitted ray tracing on sm_103a (included by ft_render.cu, inside its
// anonymous namespace, after the distance evaluators).
//
// Restates trace_ray_recursive / trace_hit_with_material
// (crates/forgedthoughts/src/renderer/ray.rs:3-222) as a stack-based bounce
// loop: each stacked ray carries the product of the weights and medium
// attenuations of its ancestors, so the recursion's nested sums become one
// accumulation per sample.  Shading at a hit follows build_bsdf_context
// (R:4397-4449): the geometric normal is the tree-resolved, smoothstep-blended
// normal (R:4462-4570), the material is the blended material of the tree
// (R:6926-7162, R:7602-7683) and a smooth boolean at the root splits the hit
// into two material traces mixed by its blend weight (ray.rs:31-35).
//
// Blend weights that are exactly 0 or 1 contribute exactly nothing, which lets
// the union_round path resolve normals and materials from the primitives near
// the hit only.  Whether a subtree's material becomes a Blend depends only on
// whether its primitives mix material models, a static per-node flag.

constexpr int kGather = 32;
constexpr float kNormalEps = 1.0e-4f;  // resolve_surface_normal_at_hit epsilon (R:4411)

struct DParams {  // MaterialParams (materials/mod.rs:66-86)
  F3 color;
  float roughness, metallic, specular, specular_weight;
  F3 spec_color;
  float ior, clearcoat, clearcoat_roughness, transmission;
  int thin;
  F3 emission_color;
  float emission_strength;
  // explicit medium (medium_from_value R:6826-6845), entered by transmissive
  // materials in transition()
  int has_medium;
  float medium_ior, medium_density;
  F3 medium_absorption;
  // dynamic_material_id (R:6669): the ft_material whose BSDF hooks apply to
  // these parameters, -1 for none (a blend of two parameter sets keeps none)
  int dyn;
};

struct DMat {  // Material incl. Blend (materials/mod.rs:214-230)
  int kind;  // ft_material_kind, or kBlendKind
  int a_model, b_model;
  float t;
  DParams a, b;
};
constexpr int kBlendKind = 4;

__device__ __forceinline__ F3 mul3(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float clamp01(float x) { return ftd::rclamp(x, 0.0f, 1.0f); }
// lerp_spectrum (R:5205-5213)
__device__ __forceinline__ F3 lerp_sp(F3 a, F3 b, float t) {
  float tt = clamp01(t);
  return f3(a.x * (1.0f - tt) + b.x * tt, a.y * (1.0f - tt) + b.y * tt, a.z * (1.0f - tt) + b.z * tt);
}

__device__ DParams params_of(const ft_material& m) {
  DParams p;
  p.color = f3(m.color[0], m.color[1], m.color[2]);
  p.roughness = m.roughness;
  p.metallic = m.metallic;
  p.specular = m.specular;
  p.specular_weight = m.specular_weight;
  p.spec_color = f3(m.specular_color[0], m.specular_color[1], m.specular_color[2]);
  p.ior = m.ior;
  p.clearcoat = m.clearcoat;
  p.clearcoat_roughness = m.clearcoat_roughness;
  p.transmission = m.transmission;
  p.thin = m.thin_walled;
  p.emission_color = f3(m.emission_color[0], m.emission_color[1], m.emission_color[2]);
  p.emission_strength = m.emission_strength;
  p.has_medium = m.has_medium != 0;
  p.medium_ior = m.medium_ior;
  p.medium_density = m.medium_density;
  p.medium_absorption = f3(m.medium_absorption[0], m.medium_absorption[1], m.medium_absorption[2]);
  p.dyn = -1;
  return p;
}

// material_for_id (R:6895-6900)
__device__ DMat mat_of_id(const DevScene& S, uint32_t id) {
  const uint32_t k = id < static_cast<uint32_t>(S.n_materials) ? id : 0u;
  const ft_material& fm = S.materials[k];
  DMat m;
  m.kind = fm.kind;
  m.a_model = m.b_model = fm.kind;
  m.t = 0.0f;
  m.a = params_of(fm);
  m.a.dyn = static_cast<int>(k);
  m.b = m.a;
  return m;
}

// The shading context of a hit for material hooks (make_shading_context,
// R:7875-7911): position, the normal facing the ray, view_dir = -ray
// direction, front_face.
struct HookCtx {
  F3 pos, normal, view_dir;
  float front_face;
};

// resolve_leaf_material (R:7164-7600) for a leaf primitive: its material,
// with the colour, roughness, IOR and thin_walled hooks evaluated on the hit
// in the primitive's frame.  Roughness is clamped to [0, 1] and the IOR to
// [1, 3]; a Metal takes neither IOR nor thin_walled.  A numeric colour is
// grey (spectrum_from_value, R:7924-7935).
//
// The further property hooks (ft_material_hook): the emission of every
// definition, and for Standard / Layered definitions metallic, specular,
// specular_weight, transmission and the coat, whose colour, roughness and IOR
// replace the specular colour, clearcoat roughness and IOR, and whose weight
// times mask the clearcoat (R:7258-7470).  The lowering compiles the latter
// only for those two models.
__device__ __forceinline__ bool has_leaf_hooks(const ft_material& fm) {
  if (fm.color_program >= 0 || fm.roughness_program >= 0 || fm.ior_program >= 0 || fm.thin_walled_program >= 0)
    return true;
  for (int k = FT_HOOK_EMISSION_COLOR; k <= FT_HOOK_COAT_MASK; ++k)
    if (fm.hook_program[k] >= 0) return true;
  for (int k = FT_HOOK_MEDIUM_IOR; k <= FT_HOOK_MEDIUM_DENSITY; ++k)
    if (fm.hook_program[k] >= 0) return true;
  return false;
}
__device__ __forceinline__ F3 hook_colour(const DevScene& S, int prog, const F3* args) {
  const F3 c = scene_program(S, prog, args, nullptr);
  return S.programs[prog].result_is_vec3 ? c : f3(c.x, c.x, c.x);
}
__device__ DMat mat_of_leaf(const DevScene& S, const DevNode& pn, const HookCtx& hc) {
  DMat m = mat_of_id(S, pn.material_id);
  const ft_material& fm = S.materials[pn.material_id < static_cast<uint32_t>(S.n_materials) ? pn.material_id : 0u];
  if (!has_leaf_hooks(fm)) return m;
  const float obj = static_cast<float>(pn.object_id), mat = static_cast<float>(pn.material_id);
  F3 args[FT_MATERIAL_HOOK_PARAMS] = {hc.pos, ftd::to_local(hc.pos, pn), hc.normal, hc.view_dir,
                                      f3(hc.front_face, hc.front_face, hc.front_face), f3(obj, obj, obj),
                                      f3(mat, mat, mat)};
  if (fm.color_program >= 0) m.a.color = hook_colour(S, fm.color_program, args);
  if (fm.roughness_program >= 0) m.a.roughness = clamp01(scene_program(S, fm.roughness_program, args, nullptr).x);
  if (fm.kind != FT_MAT_METAL) {
    if (fm.ior_program >= 0) m.a.ior = ftd::rclamp(scene_program(S, fm.ior_program, args, nullptr).x, 1.0f, 3.0f);
    if (fm.thin_walled_program >= 0) m.a.thin = scene_program(S, fm.thin_walled_program, args, nullptr).x >= 0.5f;
  }
  const int32_t* hp = fm.hook_program;
  auto num = [&](int slot) { return scene_program(S, hp[slot], args, nullptr).x; };
  if (hp[FT_HOOK_EMISSION_COLOR] >= 0) m.a.emission_color = hook_colour(S, hp[FT_HOOK_EMISSION_COLOR], args);
  if (hp[FT_HOOK_EMISSION_STRENGTH] >= 0) m.a.emission_strength = fmaxf(num(FT_HOOK_EMISSION_STRENGTH), 0.0f);
  if (hp[FT_HOOK_METALLIC] >= 0) m.a.metallic = clamp01(num(FT_HOOK_METALLIC));
  if (hp[FT_HOOK_SPECULAR] >= 0) m.a.specular = clamp01(num(FT_HOOK_SPECULAR));
  if (hp[FT_HOOK_SPECULAR_WEIGHT] >= 0) m.a.specular_weight = clamp01(num(FT_HOOK_SPECULAR_WEIGHT));
  if (hp[FT_HOOK_TRANSMISSION] >= 0) m.a.transmission = clamp01(num(FT_HOOK_TRANSMISSION));
  if (hp[FT_HOOK_COAT_COLOR] >= 0) m.a.spec_color = hook_colour(S, hp[FT_HOOK_COAT_COLOR], args);
  if (hp[FT_HOOK_COAT_ROUGHNESS] >= 0) m.a.clearcoat_roughness = clamp01(num(FT_HOOK_COAT_ROUGHNESS));
  if (hp[FT_HOOK_COAT_IOR] >= 0) m.a.ior = ftd::rclamp(num(FT_HOOK_COAT_IOR), 1.0f, 3.0f);
  if (hp[FT_HOOK_COAT_WEIGHT] >= 0 || hp[FT_HOOK_COAT_MASK] >= 0) {
    // the static clearcoat is the clamped static coat_weight
    const float w = hp[FT_HOOK_COAT_WEIGHT] >= 0 ? clamp01(num(FT_HOOK_COAT_WEIGHT)) : m.a.clearcoat;
    const float k = hp[FT_HOOK_COAT_MASK] >= 0 ? clamp01(num(FT_HOOK_COAT_MASK)) : 1.0f;
    m.a.clearcoat = clamp01(w * k);
  }
  if (hp[FT_HOOK_MEDIUM_IOR] >= 0 || hp[FT_HOOK_MEDIUM_ABSORPTION] >= 0 || hp[FT_HOOK_MEDIUM_DENSITY] >= 0) {
    // `fn medium(ctx)` replaces the material's medium (medium_from_value, R:6834-6845)
    m.a.has_medium = 1;
    m.a.medium_ior = hp[FT_HOOK_MEDIUM_IOR] >= 0 ? ftd::rclamp(num(FT_HOOK_MEDIUM_IOR), 1.0f, 3.0f) : 1.0f;
    m.a.medium_absorption =
        hp[FT_HOOK_MEDIUM_ABSORPTION] >= 0 ? hook_colour(S, hp[FT_HOOK_MEDIUM_ABSORPTION], args) : f3(1.0f, 1.0f, 1.0f);
    m.a.medium_density = hp[FT_HOOK_MEDIUM_DENSITY] >= 0 ? fmaxf(num(FT_HOOK_MEDIUM_DENSITY), 0.0f) : 0.0f;
  }
  m.b = m.a;
  return m;
}

__device__ __forceinline__ int dom_model(const DMat& m) {
  if (m.kind != kBlendKind) return m.kind;
  return m.t < 0.5f ? m.a_model : m.b_model;
}
__device__ __forceinline__ const DParams& dom_params(const DMat& m) {
  if (m.kind != kBlendKind) return m.a;
  return m.t < 0.5f ? m.a : m.b;
}

// blend_params (R:7602-7627)
__device__ DParams blend_params(DParams a, const DParams& b, float t) {
  a.color = lerp_sp(a.color, b.color, t);
  a.roughness = a.roughness + (b.roughness - a.roughness) * t;
  a.metallic = a.metallic + (b.metallic - a.metallic) * t;
  a.specular = a.specular + (b.specular - a.specular) * t;
  a.specular_weight = a.specular_weight + (b.specular_weight - a.specular_weight) * t;
  a.spec_color = lerp_sp(a.spec_color, b.spec_color, t);
  a.ior = a.ior + (b.ior - a.ior) * t;
  a.clearcoat = a.clearcoat + (b.clearcoat - a.clearcoat) * t;
  a.clearcoat_roughness = a.clearcoat_roughness + (b.clearcoat_roughness - a.clearcoat_roughness) * t;
  a.transmission = a.transmission + (b.transmission - a.transmission) * t;
  a.thin = t < 0.5f ? a.thin : b.thin;
  a.emission_color = lerp_sp(a.emission_color, b.emission_color, t);
  a.emission_strength = a.emission_strength + (b.emission_strength - a.emission_strength) * t;
  // blend_medium (R:7543-7565): two media blend (the colour through
  // lerp_spectrum's clamped t); a single one stays on its side of t = 0.5
  if (a.has_medium && b.has_medium) {
    a.medium_ior = a.medium_ior + (b.medium_ior - a.medium_ior) * t;
    a.medium_absorption = lerp_sp(a.medium_absorption, b.medium_absorption, t);
    a.medium_density = a.medium_density + (b.medium_density - a.medium_density) * t;
  } else if (a.has_medium) {
    a.has_medium = t < 0.5f;
  } else if (b.has_medium && t >= 0.5f) {
    a.has_medium = 1;
    a.medium_ior = b.medium_ior;
    a.medium_absorption = b.medium_absorption;
    a.medium_density = b.medium_density;
  }
  a.dyn = -1;  // dynamic_material_id = None (R:7624)
  return a;
}

// blend_materials (R:7629-7651)
__device__ DMat blend_materials(const DMat& a, const DMat& b, float t) {
  DMat m;
  if (a.kind != kBlendKind && a.kind == b.kind) {
    m.kind = a.kind;
    m.a_model = m.b_model = a.kind;
    m.t = 0.0f;
    m.a = blend_params(a.a, b.a, t);
    m.b = m.a;
    return m;
  }
  m.kind = kBlendKind;
  m.a_model = dom_model(a);
  m.a = dom_params(a);
  m.b_model = dom_model(b);
  m.b = dom_params(b);
  m.t = clamp01(t);
  return m;
}

// The material of a node whose other child has blend weight exactly 0 (near
// child taken with t = 0 when it is the lhs, t = 1 when it is the rhs): equal
// to blend_materials with any finite far material in every later use.
__device__ DMat blend_with_far(const DMat& near_m, bool near_is_lhs, bool node_mixes_models) {
  if (!node_mixes_models) return near_m;
  DMat m;
  m.kind = kBlendKind;
  m.a_model = m.b_model = dom_model(near_m);
  m.a = dom_params(near_m);
  m.b = m.a;
  m.t = near_is_lhs ? 0.0f : 1.0f;
  return m;
}

__device__ __forceinline__ F3 emission_of(const DParams& p) { return p.emission_color * fmaxf(p.emission_strength, 0.0f); }
// Material::emission (materials/mod.rs:284-296)
__device__ F3 mat_emission(const DMat& m) {
  if (m.kind != kBlendKind) return emission_of(m.a);
  return lerp_sp(emission_of(m.a), emission_of(m.b), m.t);
}

constexpr float kPi = 3.14159265358979323846f;

// metal.rs:7-20, 84-102
__device__ float ggx_d(float ndoth, float alpha) {
  float a2 = alpha * alpha, n2 = ndoth * ndoth;
  float denom = fmaxf(n2 * (a2 - 1.0f) + 1.0f, 1.0e-5f);
  return a2 / (kPi * denom * denom);
}
__device__ float smith_g1(float ndotx, float alpha) {
  float k = (alpha * alpha) * 0.5f;
  return ndotx / fmaxf(ndotx * (1.0f - k) + k, 1.0e-5f);
}
__device__ F3 metal_eval(F3 color, float roughness, F3 n, F3 wi, F3 wo) {
  float ndotl = fmaxf(ftd::dot3(n, wi), 0.0f), ndotv = fmaxf(ftd::dot3(n, wo), 0.0f);
  if (ndotl <= 0.0f || ndotv <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
  F3 h = ftd::normalize3(wi + wo);
  float ndoth = fmaxf(ftd::dot3(n, h), 0.0f), vdoth = fmaxf(ftd::dot3(wo, h), 0.0f);
  float rr = ftd::rclamp(roughness, 0.02f, 1.0f);
  float alpha = rr * rr;
  float d = ggx_d(ndoth, alpha);
  float g = smith_g1(ndotl, alpha) * smith_g1(ndotv, alpha);
  float x = 1.0f - clamp01(vdoth);
  float m5 = x * x * x * x * x;
  F3 fres = color + f3(m5, m5, m5) + color * (-m5);
  return fres * ((d * g) / fmaxf(4.0f * ndotl * ndotv, 1.0e-5f));
}
__device__ float f0_from_ior(float ior) {
  float i = fmaxf(ior, 1.0e-3f);
  float r = (i - 1.0f) / (i + 1.0f);
  return r * r;
}
// standard.rs:6-43, 170-183
__device__ F3 standard_eval(const DParams& m, F3 n, F3 wi, F3 wo) {
  float ndotl = fmaxf(ftd::dot3(n, wi), 0.0f), ndotv = fmaxf(ftd::dot3(n, wo), 0.0f);
  if (ndotl <= 0.0f || ndotv <= 0.0f) return f3(0.0f, 0.0f, 0.0f);
  float metallic = clamp01(m.metallic), transmission = clamp01(m.transmission), clearcoat = clamp01(m.clearcoat);
  float cx = clamp01(1.0f - clamp01(ndotv));
  float x2 = cx * cx;
  float sw = x2 * x2 * cx;
  float coat = ftd::rclamp(clearcoat * (0.2f + 0.8f * sw) * 0.65f, 0.0f, 0.95f);
  float base_kd = clamp01((1.0f - metallic) * (1.0f - transmission)) * (1.0f - coat);
  F3 diffuse = m.color * (base_kd / kPi);
  float f0d = clamp01(f0_from_ior(m.ior));
  F3 base_f0 = mul3(f3(f0d, f0d, f0d) * (clamp01(m.specular) * clamp01(m.specular_weight)), m.spec_color);
  F3 spec_f0 = base_f0 * (1.0f - metallic) + m.color * metallic;
  F3 specular = metal_eval(spec_f0, m.roughness, n, wi, wo) * (1.0f - coat * 0.85f);
  F3 cc = f3(0.0f, 0.0f, 0.0f);
  if (clearcoat > 1.0e-5f)
    cc = metal_eval(f3(1.0f, 1.0f, 1.0f), ftd::rclamp(m.clearcoat_roughness, 0.02f, 1.0f), n, wi, wo) *
         (clearcoat * 0.18f);
  return diffuse + specular + cc;
}
__device__ F3 model_eval(int model, const DParams& p, F3 n, F3 wi, F3 wo) {
  switch (model) {
    case FT_MAT_STANDARD: return standard_eval(p, n, wi, wo);
    case FT_MAT_LAMBERT:
      return ftd::dot3(n, wi) <= 0.0f ? f3(0.0f, 0.0f, 0.0f) : p.color * (1.0f / kPi);  // lambert.rs:7-13
    case FT_MAT_METAL: return metal_eval(p.color, p.roughness, n, wi, wo);
    default: return f3(0.0f, 0.0f, 0.0f);  // dielectric.rs:5-7
  }
}
// Material::eval (materials/mod.rs:298-310)
__device__ F3 mat_eval(const DMat& m, F3 n, F3 wi, F3 wo) {
  if (m.kind != kBlendKind) return model_eval(m.kind, m.a, n, wi, wo);
  return lerp_sp(model_eval(m.a_model, m.a, n, wi, wo), model_eval(m.b_model, m.b, n, wi, wo), m.t);
}

// The BSDF context of a hit (BsdfContextBase, build_bsdf_context
// R:4397-4449): position, local position in the hit object's frame, the
// shading normal (after the bump and normal hooks), wo, front face, the hit's
// object and material ids and the current medium's IOR.
struct BsdfCtx {
  F3 pos, local, normal, wo;
  float front, obj, mat, current_ior;
};

// Arguments of a BSDF hook program (bsdf_context_value, R:5006-5030).
__device__ __forceinline__ void bsdf_args(const BsdfCtx& c, F3 wi, float u1, float u2, float u3, F3* a) {
  a[0] = c.pos;
  a[1] = c.local;
  a[2] = c.normal;
  a[3] = c.wo;  // view_dir of the context is wo
  a[4] = f3(c.front, c.front, c.front);
  a[5] = f3(c.obj, c.obj, c.obj);
  a[6] = f3(c.mat, c.mat, c.mat);
  a[7] = c.wo;
  a[8] = wi;
  a[9] = f3(c.current_ior, c.current_ior, c.current_ior);
  a[10] = f3(u1, u1, u1);
  a[11] = f3(u2, u2, u2);
  a[12] = f3(u3, u3, u3);
}

// The BSDF hook `slot` of the shaded material's dominant parameters, -1 if
// none (dynamic_material_name, R:4996-5002).
__device__ __forceinline__ int bsdf_hook(const DevScene& S, const DMat& m, int slot) {
  const int dyn = dom_params(m).dyn;
  return dyn >= 0 ? S.materials[dyn].hook_program[slot] : -1;
}

// eval_bsdf (R:4905-4920): the material definition's `fn eval(ctx)`, else
// Material::eval with the context's normal and wo.
__device__ F3 bsdf_eval(const DevScene& S, const DMat& m, const BsdfCtx& c, F3 wi) {
  const int prog = bsdf_hook(S, m, FT_HOOK_EVAL);
  if (prog < 0) return mat_eval(m, c.normal, wi, c.wo);
  F3 a[FT_BSDF_HOOK_PARAMS];
  bsdf_args(c, wi, 0.0f, 0.0f, 0.0f, a);
  return hook_colour(S, prog, a);
}

// orthonormal_tangent (R:7820-7827)
__device__ __forceinline__ F3 orthonormal_tangent(F3 n) {
  const F3 up = fabsf(n.y) < 0.999f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
  return ftd::normalize3(ftd::cross3(n, up));
}

// The shading normal of build_bsdf_context (R:4418-4439): the geometric
// normal through the hit material's `fn bump(ctx)` (resolve_dynamic_bump,
// R:7776-7818: a height field differentiated by forward differences of 0.01
// along a tangent frame) and then its `fn normal(ctx)` (resolve_dynamic_normal,
// R:7749-7774), each normalised, turned to the side of its input and dropped
// when degenerate.  c.normal holds the geometric normal on entry; the hook
// context is the hit's shading context with that normal and view_dir.
__device__ F3 hooked_shading_normal(const DevScene& S, const BsdfCtx& c, F3 view_dir, uint32_t hit_mat) {
  const ft_material& fm = S.materials[hit_mat < static_cast<uint32_t>(S.n_materials) ? hit_mat : 0u];
  F3 n = c.normal;
  const int bump = fm.hook_program[FT_HOOK_BUMP], nrm = fm.hook_program[FT_HOOK_NORMAL];
  if (bump < 0 && nrm < 0) return n;
  F3 a[FT_MATERIAL_HOOK_PARAMS] = {c.pos, c.local, n, view_dir, f3(c.front, c.front, c.front),
                                   f3(c.obj, c.obj, c.obj), f3(c.mat, c.mat, c.mat)};
  if (bump >= 0) {
    const float eps = 0.01f;
    const float center = scene_program(S, bump, a, nullptr).x;
    const F3 tangent = orthonormal_tangent(n);
    const F3 bitangent = ftd::normalize3(ftd::cross3(n, tangent));
    a[1] = c.local + tangent * eps;
    const float dx = scene_program(S, bump, a, nullptr).x - center;
    a[1] = c.local + bitangent * eps;
    const float dy = scene_program(S, bump, a, nullptr).x - center;
    a[1] = c.local;
    F3 b = ftd::normalize3((n - tangent * (dx / eps)) - bitangent * (dy / eps));
    if (ftd::len3(b) > 1.0e-6f) {
      if (ftd::dot3(b, n) < 0.0f) b = b * -1.0f;
      n = b;
    }
    a[2] = n;
  }
  if (nrm >= 0) {
    F3 b = ftd::normalize3(scene_program(S, nrm, a, nullptr));
    if (ftd::len3(b) > 1.0e-6f) {
      if (ftd::dot3(b, n) < 0.0f) b = b * -1.0f;
      n = b;
    }
  }
  return n;
}

// The hit's position in its object's frame (object_transforms, identity for
// an object without one).
__device__ __forceinline__ F3 object_local(const DevScene& S, uint32_t obj, F3 p) {
  const int ni = obj < static_cast<uint32_t>(S.n_obj_node) ? S.obj_node[obj] : -1;
  return ni >= 0 ? ftd::to_local(p, S.nodes[ni]) : p;
}

// smoothstepf (R:7538-7541) of the blend weight (R:4540-4545, R:7105-7110)
__device__ __forceinline__ float blend_weight(float l, float r, float radius, bool diff) {
  float k = fmaxf(fabsf(radius), 1.0e-6f);
  float x = diff ? 0.5f + 0.5f * (((-r) - l) / k) : 0.5f + 0.5f * ((l - r) / k);
  float t = clamp01(x / fmaxf(1.0f, 1.0e-6f));
  return t * t * (3.0f - 2.0f * t);
}

__device__ bool blend_kind(int kind, bool* diff) {
  switch (kind) {
    case FT_NODE_UNION_ROUND: case FT_NODE_UNION_CHAMFER: case FT_NODE_UNION_SOFT: case FT_NODE_INTERSECT_ROUND:
    case FT_NODE_INTERSECT_CHAMFER: case FT_NODE_UNION_COLUMNS: case FT_NODE_UNION_STAIRS:
    case FT_NODE_INTERSECT_COLUMNS: case FT_NODE_INTERSECT_STAIRS:
      *diff = false;
      return true;
    case FT_NODE_DIFF_ROUND: case FT_NODE_DIFF_CHAMFER: case FT_NODE_DIFF_COLUMNS: case FT_NODE_DIFF_STAIRS:
    case FT_NODE_PIPE: case FT_NODE_ENGRAVE: case FT_NODE_GROOVE: case FT_NODE_TONGUE:
      *diff = true;
      return true;
    default: return false;
  }
}
__device__ __forceinline__ float blend_radius(const DevNode& n) {
  return (n.kind == FT_NODE_GROOVE || n.kind == FT_NODE_TONGUE) ? fmaxf(n.f[0], n.f[1]) : n.f[0];
}

// blend_surface_normals' combination (R:4529-4552)
__device__ F3 blend_normals(F3 left, F3 right, float t, bool diff) {
  if (diff) right = right * -1.0f;
  F3 m = left * (1.0f - t) + right * t;
  if (ftd::len3(m) > 1.0e-6f) return ftd::normalize3(m);
  return t < 0.5f ? left : right;
}

// estimate_node_normal (R:4554-4570) of one primitive.
__device__ F3 prim_normal(const DevNode& n, F3 p) {
  const float e = kNormalEps;
  F3 k1 = f3(1.0f, -1.0f, -1.0f), k2 = f3(-1.0f, -1.0f, 1.0f), k3 = f3(-1.0f, 1.0f, -1.0f), k4 = f3(1.0f, 1.0f, 1.0f);
  F3 nn = k1 * ftd::prim_distance(n, p + k1 * e) + k2 * ftd::prim_distance(n, p + k2 * e) +
          k3 * ftd::prim_distance(n, p + k3 * e) + k4 * ftd::prim_distance(n, p + k4 * e);
  return ftd::len3(nn) > 1.0e-6f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
}

// estimate_node_normal (R:4554-4570) of a Custom node.
__device__ F3 custom_normal(const DevScene& S, const DevNode& n, F3 p) {
  const float e = kNormalEps;
  Ctx<false> cx;
  cx.c = Counters{};
  F3 k1 = f3(1.0f, -1.0f, -1.0f), k2 = f3(-1.0f, -1.0f, 1.0f), k3 = f3(-1.0f, 1.0f, -1.0f), k4 = f3(1.0f, 1.0f, 1.0f);
  F3 nn = k1 * custom_distance(S, n, p + k1 * e, cx) + k2 * custom_distance(S, n, p + k2 * e, cx) +
          k3 * custom_distance(S, n, p + k3 * e, cx) + k4 * custom_distance(S, n, p + k4 * e, cx);
  return ftd::len3(nn) > 1.0e-6f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
}

// Result of resolving a hit against the tree: geometric normal (not yet
// oriented to the front face), material, and the optional root split.
struct Resolved {
  F3 normal;
  DMat m;       // material (or the split's left material)
  DMat mb;      // split's right material, unless mb_same
  float t;      // split weight
  bool split;
  bool mb_same;  // the split's right material is m (a root with one weighted child)
  bool ok;
};

// ---------------------------------------------------------------- generic leaves
struct GEntry {
  float d;
  F3 n;
  DMat m;
};

// Post-order over a generic leaf's node tree: each node's value at p, its
// resolved normal and material (R:4462-4552, R:6945-7113).  Subtree values of
// modifiers come from their postfix op range.
template <bool kStats>
__device__ __noinline__ void resolve_generic(const DevScene& S, int root, F3 p, const HookCtx& hc, Resolved* out,
                                             Ctx<kStats>& cx, bool split_root) {
  GEntry st[8];
  int sp = 0;
  int node_stack[24];
  unsigned char stage[24];
  int top = 0;
  node_stack[0] = root;
  stage[0] = 0;
  out->ok = false;
  out->split = false;
  for (int walk = 0; top >= 0 && walk < ftgpu::kMaxWalk; ++walk) {  // each node is visited once
    int ni = node_stack[top];
    const DevNode& n = S.nodes[ni];
    bool is_prim = n.kind <= FT_NODE_EXTRUDE_POLYGON || n.kind == FT_NODE_CUSTOM;
    bool unary = n.kind == FT_NODE_DOMAIN || n.kind == FT_NODE_DISTANCE_POST || n.kind == FT_NODE_NOISE ||
                 n.kind == FT_NODE_SLICE || n.kind == FT_NODE_SMOOTH;
    int nchild = is_prim ? 0 : (unary ? 1 : 2);
    if (stage[top] < nchild) {
      int c = stage[top] == 0 ? n.a : n.b;
      ++stage[top];
      if (top + 1 >= 24 || sp + 2 > 8) return;  // deeper than supported: leave out->ok false
      ++top;
      node_stack[top] = c;
      stage[top] = 0;
      continue;
    }
    GEntry e;
    if (is_prim) {
      if (n.kind == FT_NODE_CUSTOM) {
        e.d = custom_distance(S, n, p, cx);
        e.n = custom_normal(S, n, p);
      } else {
        e.d = ftd::prim_distance(n, p);
        e.n = prim_normal(n, p);
      }
      e.m = mat_of_leaf(S, n, hc);
    } else if (n.kind == FT_NODE_DOMAIN || n.kind == FT_NODE_DISTANCE_POST || n.kind == FT_NODE_NOISE) {
      GEntry base = st[--sp];
      int b = S.node_op_begin[ni], c = S.node_op_end[ni] - S.node_op_begin[ni];
      const float ee = kNormalEps;
      F3 k1 = f3(1.0f, -1.0f, -1.0f), k2 = f3(-1.0f, -1.0f, 1.0f), k3 = f3(-1.0f, 1.0f, -1.0f),
         k4 = f3(1.0f, 1.0f, 1.0f);
      e.d = eval_generic(S, b, c, p, cx).d;
      F3 nn = k1 * eval_generic(S, b, c, p + k1 * ee, cx).d + k2 * eval_generic(S, b, c, p + k2 * ee, cx).d +
              k3 * eval_generic(S, b, c, p + k3 * ee, cx).d + k4 * eval_generic(S, b, c, p + k4 * ee, cx).d;
      e.n = ftd::len3(nn) > 1.0e-6f ? ftd::normalize3(nn) : f3(0.0f, 1.0f, 0.0f);
      e.m = base.m;  // modifiers resolve the base's material (R:6990-6993)
    } else if (n.kind == FT_NODE_SLICE || n.kind == FT_NODE_SMOOTH) {
      e = st[--sp];
      if (n.kind == FT_NODE_SMOOTH) {
        e.d -= n.f[0] * 0.1f;
      } else {
        float coord = n.ival == 0 ? p.x : (n.ival == 1 ? p.y : p.z);
        e.d = ftd::rmax(e.d, ftd::rmax(n.f[0] - coord, coord - n.f[1]));
      }
    } else {
      GEntry r = st[--sp];
      GEntry l = st[--sp];
      Info li{l.d, 0u, 0u}, ri{r.d, 0u, 0u};
      float d = ftd::combine(n.kind, n.f[0], n.f[1], li, ri).d;
      bool diff;
      if (n.kind == FT_NODE_UNION) {
        e = l.d <= r.d ? l : r;
      } else if (n.kind == FT_NODE_INTERSECT) {
        e = l.d >= r.d ? l : r;
      } else if (n.kind == FT_NODE_SUBTRACT) {
        if (l.d >= -r.d) {
          e = l;
        } else {
          e = r;
          e.n = r.n * -1.0f;
        }
      } else if (blend_kind(n.kind, &diff)) {
        float t = blend_weight(l.d, r.d, blend_radius(n), diff);
        e.n = blend_normals(l.n, r.n, t, diff);
        if (top == 0 && split_root) {  // smooth boolean at the leaf root: material split
          out->m = l.m;
          out->mb = r.m;
          out->mb_same = false;
          out->t = t;
          out->split = true;
        }
        e.m = blend_materials(l.m, r.m, t);
      } else {
        e = l;
      }
      e.d = d;
    }
    st[sp++] = e;
    --top;
  }
  out->normal = st[0].n;
  if (!out->split) out->m = st[0].m;
  out->ok = true;
}

// ---------------------------------------------------------------- union_round trees
// Gather the primitives within `reach` of p (exact distances) through the
// tree's BVH.  Returns false when more than kGather qualify.
__device__ bool ur_gather(const DevScene& S, const DevUrTree& t, F3 p, float reach, int* pos, float* dist, int* n) {
  int stack[48];
  int sp = 0;
  *n = 0;
  stack[sp++] = t.bvh_root;
  for (int walk = 0; sp > 0 && walk < ftgpu::kMaxWalk; ++walk) {  // a tree walk pops each node once
    const DevUrBvh& bn = S.ur_bvh[stack[--sp]];
    if (node_lb(p, bn.bmin, bn.bmax) >= reach) continue;
    if (bn.prim_count > 0) {
      for (int k = 0; k < bn.prim_count; ++k) {
        int ps = S.ur_bvh_prims[bn.prim_begin + k];
        const DevNode& pn = S.nodes[S.ur_prims[t.prim_first + ps]];
        if (node_lb(p, pn.bmin, pn.bmax) >= reach) continue;
        float d = ftd::prim_distance(pn, p);
        if (d < reach) {
          if (*n >= kGather) return false;
          pos[*n] = ps;
          dist[*n] = d;
          ++*n;
        }
      }
      continue;
    }
    if (sp + 2 > 48) return false;
    stack[sp++] = bn.left;
    stack[sp++] = bn.right;
  }
  return true;
}

// Exact value of the union_round subtree `c` (inner index, or -(pos + 1) for
// a primitive) at p from the gathered primitives; kInf when it holds none
// (its true value is then >= reach).  Primitives outside the gather are >= the
// reach, which keeps every union_round on the fold's path exact.
__device__ float ur_subtree_value(const DevScene& S, const DevUrTree& t, int c, const int* gpos, const float* gdist,
                                  int ng) {
  auto prim_value = [&](int ps) {
    for (int k = 0; k < ng; ++k)
      if (gpos[k] == ps) return gdist[k];
    return kInf;
  };
  if (c < 0) return prim_value(-c - 1);
  auto has = [&](int in) {
    const DevUrInner& u = S.ur_inner[in];
    for (int k = 0; k < ng; ++k)
      if (gpos[k] >= u.lo && gpos[k] < u.hi) return true;
    return false;
  };
  if (!has(c)) return kInf;
  struct VF {
    int inner, stage;
    float v[2];
  };
  VF fr[24];
  int fp = 0;
  fr[0].inner = c;
  fr[0].stage = 0;
  for (int walk = 0; walk < ftgpu::kMaxWalk; ++walk) {  // each inner node is opened once
    VF& F = fr[fp];
    if (F.stage < 2) {
      int ch = S.ur_inner[F.inner].child[F.stage];
      if (ch < 0) {
        F.v[F.stage++] = prim_value(-ch - 1);
        continue;
      }
      if (!has(ch)) {
        F.v[F.stage++] = kInf;
        continue;
      }
      if (fp + 1 >= 24) return kInf;  // deeper than supported; the caller widens and falls back
      ++F.stage;
      ++fp;
      fr[fp].inner = ch;
      fr[fp].stage = 0;
      continue;
    }
    float v = (F.v[0] == kInf && F.v[1] == kInf)
                  ? kInf
                  : ftd::combine(FT_NODE_UNION_ROUND, t.r, 0.0f, Info{F.v[0], 0u, 0u}, Info{F.v[1], 0u, 0u}).d;
    if (fp == 0) return v;
    --fp;
    fr[fp].v[fr[fp].stage - 1] = v;
  }
  return kInf;  // only a corrupted tree gets here
}

struct NEntry {
  F3 n;
  DMat m;
};

// Top-down resolution over the nodes with nonzero blend weight.  Each visited
// node gets both child values from exact restricted folds, hence its exact
// weight t; a child with weight exactly 0 is skipped.  A child without
// gathered primitives is provably weightless when reach >= (other value) + r;
// otherwise *need receives the reach required.
//
// The result of the child completed last travels up in `carry` (registers).
// Only a node that uses both children keeps its left child's result while the
// right subtree resolves, on the `pend` stack; the chain of single-child
// nodes between the root and the hit's primitives (most of the walk) touches
// no per-thread memory beyond the frames' few scalars.
__device__ __noinline__ bool resolve_urtree_reach(const DevScene& S, const DevUrTree& t, F3 p, const HookCtx& hc,
                                                  float reach, Resolved* out, float* need, bool split_root) {
  int gpos[kGather];
  float gdist[kGather];
  int ng = 0;
  if (!ur_gather(S, t, p, reach, gpos, gdist, &ng)) {
    *need = -1.0f;
    return false;
  }
  struct Frame {
    int inner, stage;
    float tw;
    bool useL, useR;
  };
  Frame fr[20];
  NEntry pend[20];  // left results of two-child nodes whose right subtree is open
  int np = 0;
  NEntry carry;
  int fp = 0;
  const float r = t.r;
  // Set up a frame: child values, exact weight, which children carry weight.
  auto open = [&](int fi, int inner) -> bool {
    Frame& F = fr[fi];
    F.inner = inner;
    F.stage = 0;
    const DevUrInner& u = S.ur_inner[inner];
    float vL = ur_subtree_value(S, t, u.child[0], gpos, gdist, ng);
    float vR = ur_subtree_value(S, t, u.child[1], gpos, gdist, ng);
    if (vL == kInf && vR == kInf) {
      *need = -1.0f;
      return false;
    }
    if (vL == kInf || vR == kInf) {
      float vn = vL == kInf ? vR : vL;
      if (reach < vn + r) {
        *need = vn + r;
        return false;
      }
    }
    F.tw = blend_weight(vL, vR, r, false);
    F.useL = F.tw != 1.0f;
    F.useR = F.tw != 0.0f;
    return true;
  };
  if (!open(0, t.inner_root)) return false;
  for (int walk = 0; walk < ftgpu::kMaxWalk; ++walk) {  // each inner node is opened once
    Frame& F = fr[fp];
    bool child_done = false;  // carry holds the result of fr[fp]'s child (stage - 1)
    if (F.stage < 2) {
      bool use = F.stage == 0 ? F.useL : F.useR;
      int c = S.ur_inner[F.inner].child[F.stage];
      if (!use) {
        ++F.stage;
        continue;
      }
      if (c < 0) {
        const DevNode& pn = S.nodes[S.ur_prims[t.prim_first + (-c - 1)]];
        carry.n = prim_normal(pn, p);
        carry.m = mat_of_leaf(S, pn, hc);
        ++F.stage;
        child_done = true;
      } else {
        if (fp + 1 >= 20) {
          *need = -1.0f;
          return false;
        }
        ++F.stage;
        ++fp;
        if (!open(fp, c)) return false;
        continue;
      }
    } else {
      // both children done: a two-child node's left result is on pend, the
      // right one (or a single child's) in carry
      const bool both = F.useL && F.useR;
      if (fp == 0 && split_root) {
        if (both) {
          const NEntry& L = pend[--np];
          out->normal = blend_normals(L.n, carry.n, F.tw, false);
          out->m = L.m;
          out->mb = carry.m;
          out->mb_same = false;
        } else {
          out->normal = blend_normals(carry.n, carry.n, F.tw, false);
          out->m = carry.m;  // the one material, not written twice
          out->mb_same = true;
        }
        out->t = F.tw;
        out->split = true;
        out->ok = true;
        return true;
      }
      if (both) {
        const NEntry& L = pend[--np];
        carry.n = blend_normals(L.n, carry.n, F.tw, false);
        carry.m = blend_materials(L.m, carry.m, F.tw);
      } else {
        carry.n = blend_normals(carry.n, carry.n, F.tw, false);
        carry.m = blend_with_far(carry.m, F.useL, S.ur_inner_blend[F.inner] != 0);
      }
      if (fp == 0) {  // the root's blended material (resolve_material_at_hit)
        out->normal = carry.n;
        out->m = carry.m;
        out->split = false;
        out->ok = true;
        return true;
      }
      --fp;
      child_done = true;
    }
    // A left child completed under a node that also uses its right child:
    // keep its result until the right subtree is done.
    if (child_done && fr[fp].stage == 1 && fr[fp].useR) pend[np++] = carry;
  }
  *need = -1.0f;  // only a corrupted tree gets here
  return false;
}

__device__ void resolve_urtree(const DevScene& S, const DevUrTree& t, F3 p, const HookCtx& hc, Resolved* out,
                               bool split_root) {
  float reach = 3.0f * t.r;
  out->ok = false;
  for (int attempt = 0; attempt < 6; ++attempt) {
    float need = 0.0f;
    if (resolve_urtree_reach(S, t, p, hc, reach, out, &need, split_root)) return;
    if (need < 0.0f) return;  // capacity exceeded
    reach = fmaxf(1.5f * reach, need * 1.0001f + 1.0e-6f);
  }
}

// Normal and material at a hit on leaf `li`.  With split_root a smooth
// boolean at the root gives its two materials and weight (the Whitted
// tracer's split, ray.rs:31-35); without it, the root's blended material
// (resolve_material_at_hit, as the path tracer shades).
template <bool kStats>
__device__ void resolve_hit(const DevScene& S, int li, F3 p, const HookCtx& hc, Resolved* out, Ctx<kStats>& cx,
                            bool split_root = true) {
  const DevLeaf& lf = S.leaves[li];
  out->split = false;
  out->ok = false;
  if (lf.kind == ftgpu::kLeafPrim) {
    const DevNode& n = S.nodes[lf.node];
    out->normal = prim_normal(n, p);
    out->m = mat_of_leaf(S, n, hc);
    out->ok = true;
    return;
  }
  if (lf.kind == ftgpu::kLeafUrTree) {
    resolve_urtree(S, S.urtrees[lf.first], p, hc, out, split_root);
    if (out->ok) return;
  }
  resolve_generic(S, lf.node, p, hc, out, cx, split_root);
}

// ---------------------------------------------------------------- lights and shadows
// Accelerator::lower_bound over the leaf BVH (bvh_lower_bound, R:788-822):
// the nearest leaf box.
template <bool kStats>
__device__ float scene_lower_bound(const DevScene& S, F3 p, Ctx<kStats>& cx) {
  // One- and two-leaf BVHs (a single object, or a ground plus one composite
  // object) without a stack: the walk below returns the root leaf's box
  // bound, or the smaller of two leaf children's.
  const DevBvhNode& root = S.bvh[S.bvh_root];
  if (root.leaf >= 0) {
    cx.box();
    return node_lb(p, root.bmin, root.bmax);
  }
  {
    const DevBvhNode& L = S.bvh[root.lhs];
    const DevBvhNode& R = S.bvh[root.rhs];
    if (L.leaf >= 0 && R.leaf >= 0) {
      cx.box(3);
      return fminf(node_lb(p, L.bmin, L.bmax), node_lb(p, R.bmin, R.bmax));
    }
  }
  float best = kInf;
  cx.box();
  int stack[64];
  float slb[64];
  int sp = 0;
  stack[0] = S.bvh_root;
  slb[0] = node_lb(p, S.bvh[S.bvh_root].bmin, S.bvh[S.bvh_root].bmax);
  sp = 1;
  for (int walk = 0; sp > 0 && walk < ftgpu::kMaxWalk; ++walk) {  // a tree walk pops each node once
    --sp;
    if (slb[sp] > best) continue;
    const DevBvhNode& n = S.bvh[stack[sp]];
    if (n.leaf >= 0) {
      best = fminf(best, slb[sp]);
      continue;
    }
    if (sp + 2 > 64) break;
    float ll = node_lb(p, S.bvh[n.lhs].bmin, S.bvh[n.lhs].bmax), rl = node_lb(p, S.bvh[n.rhs].bmin, S.bvh[n.rhs].bmax);
    cx.box(2);
    if (ll <= rl) {
      stack[sp] = n.rhs; slb[sp] = rl; ++sp;
      stack[sp] = n.lhs; slb[sp] = ll; ++sp;
    } else {
      stack[sp] = n.lhs; slb[sp] = ll; ++sp;
      stack[sp] = n.rhs; slb[sp] = rl; ++sp;
    }
  }
  return best;
}

// Light::sample_li_indexed (render_api.rs:172-259)
__device__ void sample_light(const ft_light& L, F3 p, uint32_t idx, uint32_t count, F3* wi, F3* rad, float* dist) {
  F3 inten = f3(L.intensity[0], L.intensity[1], L.intensity[2]);
  if (L.kind == FT_LIGHT_ENV) {
    *wi = f3(0.0f, 1.0f, 0.0f);
    *rad = inten;
    *dist = kInf;
    return;
  }
  F3 lp = f3(L.position[0], L.position[1], L.position[2]);
  F3 target = lp;
  if (L.kind == FT_LIGHT_SPHERE && L.radius > 1.0e-5f) {
    F3 nrm = ftd::normalize3(p - lp);
    F3 up = fabsf(nrm.y) < 0.99f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
    auto cross3 = [](F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); };
    F3 tangent = ftd::normalize3(cross3(nrm, up));
    F3 bit = ftd::normalize3(cross3(tangent, nrm));
    uint32_t nsm = count > 0 ? count : 1u;
    float u = (static_cast<float>(idx) + 0.5f) / static_cast<float>(nsm);  // hammersley_2d (render_api.rs:262-272)
    uint32_t bits = (idx >> 16) | (idx << 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    float v = static_cast<float>(bits) * 2.3283064e-10f;
    float sx = 2.0f * u - 1.0f, sy = 2.0f * v - 1.0f;  // concentric_disk_sample (render_api.rs:274-289)
    float dx = 0.0f, dy = 0.0f;
    if (!(fabsf(sx) <= 1.1920929e-7f && fabsf(sy) <= 1.1920929e-7f)) {
      float rr, th;
      if (fabsf(sx) > fabsf(sy)) {
        rr = sx;
        th = 0.78539816339744830962f * (sy / sx);
      } else {
        rr = sy;
        th = 1.57079632679489661923f - 0.78539816339744830962f * (sx / sy);
      }
      dx = rr * cosf(th);
      dy = rr * sinf(th);
    }
    target = lp + tangent * (dx * L.radius) + bit * (dy * L.radius);
  }
  F3 to = target - p;
  float dd = fmaxf(ftd::len3(to), 1.0e-4f);
  *wi = to * (1.0f / dd);
  *rad = inten * (1.0f / (dd * dd));
  *dist = dd;
}

// offset_ray_origin (R:5067-5078)
__device__ F3 offset_origin(F3 pos, F3 gn, F3 dir, float eps) {
  F3 n = ftd::len3(gn) > 1.0e-8f ? ftd::normalize3(gn) : ftd::normalize3(dir);
  float sign = ftd::dot3(dir, n) >= 0.0f ? 1.0f : -1.0f;
  F3 no = n * (sign * fmaxf(eps * 16.0f, 2.0e-4f));
  float step = fmaxf(eps * 8.0f, 1.0e-4f);
  return pos + no + ftd::normalize3(dir) * step;
}

// fresnel_dielectric_scalar (R:5188-5204)
__device__ float fresnel_dielectric(float ci, float eta_i, float eta_t) {
  float ei = fmaxf(eta_i, 1.0e-4f), et = fmaxf(eta_t, 1.0e-4f);
  if (fabsf(ei - et) < 1.0e-6f) return 0.0f;
  ci = clamp01(ci);
  float eta = ei / et;
  float sin2 = eta * eta * (1.0f - ci * ci);
  if (sin2 >= 1.0f) return 1.0f;
  float ct = sqrtf(1.0f - sin2);
  float rs = ((ei * ci) - (et * ct)) / fmaxf((ei * ci) + (et * ct), 1.0e-6f);
  float rp = ((et * ci) - (ei * ct)) / fmaxf((et * ci) + (ei * ct), 1.0e-6f);
  return 0.5f * (rs * rs + rp * rp);
}

// refract (R:5080-5095)
__device__ bool refract_dir(F3 inc, F3 nrm, float eta, F3* out) {
  F3 i = ftd::normalize3(inc);
  F3 n = ftd::normalize3(nrm);
  float cosi = ftd::rclamp(ftd::dot3(i, n), -1.0f, 1.0f);
  if (cosi > 0.0f) n = n * -1.0f;
  else cosi = -cosi;
  float sin2 = eta * eta * (1.0f - cosi * cosi);
  if (sin2 > 1.0f) return false;
  float cost = sqrtf(1.0f - sin2);
  *out = ftd::normalize3(i * eta + n * (eta * cosi - cost));
  return true;
}

// rough_lobe_directions (ray.rs:376-411): the ideal direction, then up to six
// directions offset by the roughness spread along a tangent frame.
constexpr int kMaxLobes = 4;  // rough_dielectric_refraction_samples' largest count
__device__ int rough_lobe_directions(F3 ideal_dir, float roughness, int count, F3* dirs) {
  const F3 ideal = ftd::normalize3(ideal_dir);
  const F3 seed = fabsf(ideal.y) < 0.99f ? f3(0.0f, 1.0f, 0.0f) : f3(1.0f, 0.0f, 0.0f);
  const F3 tangent = ftd::normalize3(ftd::cross3(ideal, seed));
  const F3 bitangent = ftd::normalize3(ftd::cross3(tangent, ideal));
  const float spread = ftd::rclamp(roughness, 0.0f, 0.5f) * 0.35f;
  dirs[0] = ideal;
  if (count <= 1 || spread <= 1.0e-4f) return 1;
  const float ox[kMaxLobes - 1] = {1.0f, -1.0f, 0.0f};
  const float oy[kMaxLobes - 1] = {0.0f, 0.0f, 1.0f};
  const int n = count < kMaxLobes ? count : kMaxLobes;
  for (int k = 1; k < n; ++k)
    dirs[k] = ftd::normalize3((ideal + tangent * (ox[k - 1] * spread)) + bitangent * (oy[k - 1] * spread));
  return n;
}
// rough_dielectric_reflection_samples / _refraction_samples (ray.rs:413-435)
__device__ __forceinline__ int rough_reflection_samples(float r) { return r < 0.12f ? 1 : (r < 0.28f ? 2 : 3); }
__device__ __forceinline__ int rough_refraction_samples(float r) { return r < 0.1f ? 2 : (r < 0.24f ? 3 : 4); }

struct MediumD {
  float ior;
  F3 absorption;
  float density;
};
__device__ __forceinline__ MediumD air() { return MediumD{1.0f, f3(1.0f, 1.0f, 1.0f), 0.0f}; }

// medium_transmittance (R:5109-5119)
__device__ F3 transmittance(const MediumD& m, float dist) {
  if (m.density <= 0.0f || dist <= 0.0f) return f3(1.0f, 1.0f, 1.0f);
  float e = m.density * fmaxf(dist, 0.0f);
  return f3(powf(clamp01(m.absorption.x), e), powf(clamp01(m.absorption.y), e), powf(clamp01(m.absorption.z), e));
}

// transition_medium with medium_state_from_material (R:5125-5175): entering a
// transmissive material takes its explicit medium (IOR clamped to [1, 3],
// density at least 0), else a medium of its IOR without absorption; leaving
// it returns to air; other materials keep the current medium.
__device__ MediumD transition(const DMat& m, bool front, MediumD cur) {
  int model = dom_model(m);
  const DParams& p = dom_params(m);
  bool transmissive = model == FT_MAT_DIELECTRIC || (model == FT_MAT_STANDARD && p.transmission > 0.01f);
  if (!transmissive) return cur;
  if (!front) return air();
  if (p.has_medium)
    return MediumD{ftd::rclamp(p.medium_ior, 1.0f, 3.0f), p.medium_absorption, fmaxf(p.medium_density, 0.0f)};
  return MediumD{ftd::rclamp(p.ior, 1.0f, 3.0f), f3(1.0f, 1.0f, 1.0f), 0.0f};
}

struct RayJob {
  F3 o, d, w;  // origin, direction, throughput
  MediumD med;
  int depth;
};

struct TraceParams {
  RayParams P;
  uint32_t max_depth;
};
