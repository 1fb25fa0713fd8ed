// Lowering of an evaluated `.ft` scene to the flat scene IR.
//
// compile_sdf / compile_scene: R:1384-1742 (primitives, booleans, hg_sdf
// operators, mirror/repeat expansion R:1640-1680 + R:1973-2326, slice, noise,
// smooth), modifier hooks R:1750-1948 (including the double transform of an
// object carrying both `domain` and `distance_post`), material interning
// R:558-570, camera R:6263-6286, lights R:6288-6388 (ordered by binding
// name), render settings R:1316-1354, scene root R:1375-1382,
// sdf_center R:4047-4089, sdf_bounds R:5242-5386.
//
// Hook bodies (`domain(p)`, `distance_post(d, p)`, `environment color(dir)`)
// are partially evaluated into register programs: captured values and scene
// bindings fold to constants, parameters become registers, user functions are
// inlined.  This takes the role of the Cranelift JIT
// (crates/forgedthoughts/src/jit.rs:501-747, 2931-3016).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <map>

#include "frontend.h"

namespace ftfe {

void OwnedSceneDesc::finalize() {
  desc.abi_version = FT_ABI_VERSION;
  desc.nodes = nodes.data();
  desc.n_nodes = static_cast<uint32_t>(nodes.size());
  desc.instrs = instrs.data();
  desc.n_instrs = static_cast<uint32_t>(instrs.size());
  desc.programs = programs.data();
  desc.n_programs = static_cast<uint32_t>(programs.size());
  desc.lights = lights.data();
  desc.n_lights = static_cast<uint32_t>(lights.size());
  desc.materials = materials.data();
  desc.n_materials = static_cast<uint32_t>(materials.size());
}

namespace {

[[noreturn]] void lower_fail(ft_status s, const std::string& m) { throw FrontendError(s, m); }

struct V3 {
  float x = 0, y = 0, z = 0;
};
V3 v3(float x, float y, float z) { return V3{x, y, z}; }
V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
float length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
V3 vmin(V3 a, V3 b) { return v3(std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)); }
V3 vmax(V3 a, V3 b) { return v3(std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)); }

struct Aabb {
  V3 mn, mx;
};
Aabb aabb_union(Aabb a, Aabb b) { return Aabb{vmin(a.mn, b.mn), vmax(a.mx, b.mx)}; }
Aabb aabb_expand(Aabb a, float d) { return Aabb{sub(a.mn, v3(d, d, d)), add(a.mx, v3(d, d, d))}; }

struct Xf {
  V3 c, r;
};

float deg_to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }
V3 rot_x(V3 v, float deg) {
  float r = deg_to_rad(deg), s = std::sin(r), c = std::cos(r);
  return v3(v.x, c * v.y - s * v.z, s * v.y + c * v.z);
}
V3 rot_y(V3 v, float deg) {
  float r = deg_to_rad(deg), s = std::sin(r), c = std::cos(r);
  return v3(c * v.x + s * v.z, v.y, -s * v.x + c * v.z);
}
V3 rot_z(V3 v, float deg) {
  float r = deg_to_rad(deg), s = std::sin(r), c = std::cos(r);
  return v3(c * v.x - s * v.y, s * v.x + c * v.y, v.z);
}
// transform_offset (R:2432-2437)
V3 transform_offset(const Xf& t, V3 o) { return rot_z(rot_y(rot_x(o, t.r.x), t.r.y), t.r.z); }

Xf node_xf(const ft_node& n) { return Xf{v3(n.center[0], n.center[1], n.center[2]), v3(n.rot_deg[0], n.rot_deg[1], n.rot_deg[2])}; }
void set_xf(ft_node& n, const Xf& t) {
  n.center[0] = t.c.x; n.center[1] = t.c.y; n.center[2] = t.c.z;
  n.rot_deg[0] = t.r.x; n.rot_deg[1] = t.r.y; n.rot_deg[2] = t.r.z;
}
void set_bounds(ft_node& n, const Aabb& b) {
  n.bounds_min[0] = b.mn.x; n.bounds_min[1] = b.mn.y; n.bounds_min[2] = b.mn.z;
  n.bounds_max[0] = b.mx.x; n.bounds_max[1] = b.mx.y; n.bounds_max[2] = b.mx.z;
}

bool is_primitive(int k) { return k <= FT_NODE_EXTRUDE_POLYGON || k == FT_NODE_CUSTOM; }
bool is_modifier(int k) { return k == FT_NODE_DOMAIN || k == FT_NODE_DISTANCE_POST || k == FT_NODE_NOISE; }
bool is_binary(int k) { return k >= FT_NODE_UNION && k <= FT_NODE_TONGUE; }

bool read_number(const ObjectData& o, std::initializer_list<const char*> names, float* out) {
  for (const char* n : names) {
    const Value* v = o.get(n);
    if (v && v->kind == Value::Number) {
      *out = v->num;
      return true;
    }
  }
  return false;
}
float number_or(const ObjectData& o, std::initializer_list<const char*> names, float def) {
  float v;
  return read_number(o, names, &v) ? v : def;
}
bool read_number_path(const ObjectData& o, const char* parent, const char* leaf, float* out) {
  const Value* p = o.get(parent);
  if (!p || p->kind != Value::Object) return false;
  return read_number(*p->obj, {leaf}, out);
}
// read_vec3_field (R:3599-3608)
bool read_vec3_field(const ObjectData& o, const char* name, V3* out) {
  const Value* v = o.get(name);
  if (!v || v->kind != Value::Object) return false;
  float x, y, z;
  if (!read_number(*v->obj, {"x"}, &x) || !read_number(*v->obj, {"y"}, &y) || !read_number(*v->obj, {"z"}, &z))
    return false;
  *out = v3(x, y, z);
  return true;
}
// read_spectrum_field (R:6772-6784)
bool read_spectrum(const ObjectData& o, const char* name, V3* out) {
  const Value* v = o.get(name);
  if (!v) return false;
  if (v->kind == Value::Number) {
    *out = v3(v->num, v->num, v->num);
    return true;
  }
  if (v->kind != Value::Object) return false;
  float r, g, b;
  if (!read_number(*v->obj, {"r", "x"}, &r) || !read_number(*v->obj, {"g", "y"}, &g) ||
      !read_number(*v->obj, {"b", "z"}, &b))
    return false;
  *out = v3(r, g, b);
  return true;
}
// read_center / read_transform (R:3570-3597)
Xf read_transform(const ObjectData& o) {
  Xf t;
  float v;
  t.c.x = read_number_path(o, "pos", "x", &v) ? v : number_or(o, {"x"}, 0.0f);
  t.c.y = read_number_path(o, "pos", "y", &v) ? v : number_or(o, {"y"}, 0.0f);
  t.c.z = read_number_path(o, "pos", "z", &v) ? v : number_or(o, {"z"}, 0.0f);
  t.r.x = read_number_path(o, "rot", "x", &v) ? v : number_or(o, {"rot_x"}, 0.0f);
  t.r.y = read_number_path(o, "rot", "y", &v) ? v : number_or(o, {"rot_y"}, 0.0f);
  t.r.z = read_number_path(o, "rot", "z", &v) ? v : number_or(o, {"rot_z"}, 0.0f);
  return t;
}
V3 read_center(const ObjectData& o) { return read_transform(o).c; }

float clampf(float x, float lo, float hi) { return std::min(std::max(x, lo), hi); }

ft_material material_defaults(int kind) {
  ft_material m;
  std::memset(&m, 0, sizeof(m));
  m.kind = kind;
  m.color_program = m.roughness_program = m.ior_program = m.thin_walled_program = -1;
  for (int32_t& h : m.hook_program) h = -1;
  m.color[0] = m.color[1] = m.color[2] = 0.8f;
  m.roughness = 0.5f;
  m.ior = 1.5f;
  // MaterialParams constructors (crates/forgedthoughts/src/materials/mod.rs:90-212)
  m.specular = 0.5f;
  m.specular_weight = 1.0f;
  m.specular_color[0] = m.specular_color[1] = m.specular_color[2] = 1.0f;
  m.clearcoat = 0.0f;
  m.clearcoat_roughness = 0.1f;
  return m;
}

// default_material (R:7937-7953)
ft_material default_material() { return material_defaults(FT_MAT_STANDARD); }

bool material_equal(const ft_material& a, const ft_material& b) { return std::memcmp(&a, &b, sizeof(a)) == 0; }

// ------------------------------------------------------------ hook compiler
struct SVal {
  bool is_const = true;
  Value cv;
  int reg = -1;
  bool vec3 = false;
  // a record of run-time fields (the shading context of material hooks)
  std::shared_ptr<std::map<std::string, SVal>> rec;
};

class HookCompiler {
 public:
  HookCompiler(const EvalState& st, std::vector<ft_instr>& code) : st_(st), code_(code) {}

  // Compile `params -> body` with `locals` as captured constants.  Returns a
  // program whose result is the requested type, or throws.
  ft_program compile(const std::vector<std::string>& params, const std::vector<bool>& param_vec3,
                     const std::vector<FnStmt>& body, const std::map<std::string, Value>& captures,
                     const BlockDef* block, bool want_vec3, const char* what) {
    first_ = static_cast<uint32_t>(code_.size());
    nregs_ = 0;
    what_ = what;
    block_ = block;
    std::map<std::string, SVal> locals;
    for (const auto& kv : captures) {
      SVal c;
      c.cv = kv.second;
      locals[kv.first] = c;
    }
    if (block) {
      // Block-level `let` bindings (environment/material scope, E:3768-3790).
      for (const BlockStmt& s : block->statements) {
        if (s.kind != BlockStmt::Binding) continue;
        locals[s.name] = eval(*s.expr, locals, 0);
        block_locals_[s.name] = locals[s.name];
      }
    }
    ft_program prog{};
    prog.first_instr = first_;
    prog.n_params = static_cast<uint32_t>(params.size());
    for (size_t i = 0; i < params.size(); ++i) {
      SVal p;
      p.is_const = false;
      p.reg = nregs_++;
      p.vec3 = param_vec3[i];
      if (p.vec3) prog.param_is_vec3 |= 1u << i;
      locals[params[i]] = p;
    }
    SVal result = run_body(body, locals, 0);
    int r = materialize(result);
    bool rv = reg_vec3(result);
    if (rv != want_vec3) lower_fail(FT_ERR_UNSUPPORTED, std::string(what) + " hook returns the wrong type");
    ft_instr ret{};
    ret.op = FT_OP_RET;
    ret.a = static_cast<uint8_t>(r);
    ret.flags = rv ? FT_INSTR_VEC3 : 0;
    code_.push_back(ret);
    prog.n_instr = static_cast<uint32_t>(code_.size()) - first_;
    prog.n_regs = static_cast<uint32_t>(nregs_);
    prog.result_is_vec3 = want_vec3 ? 1u : 0u;
    if (nregs_ > FT_MAX_PROGRAM_REGS) lower_fail(FT_ERR_UNSUPPORTED, std::string(what) + " hook needs too many registers");
    return prog;
  }

 // A function of a block definition (an `sdf` definition's distance, domain
  // or distance_post, eval_sdf_function_with_overrides, E:2960-3050): its
  // parameters are registers (vec3 where param_vec3 says so), the
  // definition's bindings (an instance field of the same name replacing one)
  // constants, its helper functions callable.  want: 0 a number, 1 a vec3.
  // Returns false, emitting nothing, when it does not fold to such a program.
  bool compile_block_fn(const BlockStmt& fn, const BlockDef& def, const ObjectData& overrides,
                        const std::vector<bool>& param_vec3, int want, ft_program* out) {
    const size_t mark = code_.size();
    first_ = static_cast<uint32_t>(mark);
    nregs_ = 0;
    what_ = "sdf";
    block_ = &def;
    try {
      std::map<std::string, SVal> locals = block_scope(def, overrides);
      ft_program prog{};
      prog.first_instr = first_;
      prog.n_params = static_cast<uint32_t>(fn.params.size());
      for (size_t i = 0; i < fn.params.size(); ++i) {
        locals[fn.params[i]] = reg(nregs_++, param_vec3[i]);
        if (param_vec3[i]) prog.param_is_vec3 |= 1u << i;
      }
      SVal result = run_body(fn.body, locals, 0);
      if (result.rec) fail("returns a record");
      int r = materialize(result);
      bool rv = reg_vec3(result);
      if (rv != (want == 1) || nregs_ > FT_MAX_PROGRAM_REGS) {
        code_.resize(mark);
        return false;
      }
      ft_instr ret{};
      ret.op = FT_OP_RET;
      ret.a = static_cast<uint8_t>(r);
      ret.flags = rv ? FT_INSTR_VEC3 : 0;
      code_.push_back(ret);
      prog.n_instr = static_cast<uint32_t>(code_.size()) - first_;
      prog.n_regs = static_cast<uint32_t>(nregs_);
      prog.result_is_vec3 = rv ? 1u : 0u;
      *out = prog;
      return true;
    } catch (const FrontendError&) {
      code_.resize(mark);
      return false;
    }
  }

  // A zero-argument function of a block definition folded to a constant
  // (eval_sdf_zero_arg_function_with_overrides); false if it does not fold.
  bool const_block_fn(const BlockStmt& fn, const BlockDef& def, const ObjectData& overrides, Value* out) {
    what_ = "sdf";
    block_ = &def;
    try {
      std::map<std::string, SVal> locals = block_scope(def, overrides);
      SVal v = run_body(fn.body, locals, 0);
      if (!v.is_const || v.rec) return false;
      *out = v.cv;
      return true;
    } catch (const FrontendError&) {
      return false;
    }
  }

  // A material hook `fn name(ctx)` (eval_material_function_with_overrides,
  // E:2860-2940): the definition's bindings (an instance field of the same
  // name replacing one) are constants, `ctx` is the shading context record of
  // seven parameters (FT_MATERIAL_HOOK_PARAMS).  want: 0 a number, 1 a vec3,
  // 2 either.  Returns false, emitting nothing, when the body does not fold to
  // a program of the wanted type.
  //
  // With bsdf set the context is the BSDF context of bsdf_context_value
  // (R:5006-5030), FT_BSDF_HOOK_PARAMS parameters: the seven (normal = the
  // shading normal, view_dir = wo), then wo, wi, current_ior and, when
  // sample_randoms, u1, u2, u3 (the registers exist either way; eval and pdf
  // see no u fields).  With field set the body returns a record (a
  // BsdfSample) and the program computes that field of it; a record without
  // the field emits nothing and returns false.
  bool compile_ctx(const BlockStmt& fn, const BlockDef& def, const ObjectData& overrides, int want,
                   ft_program* out, bool bsdf = false, bool sample_randoms = false, const char* field = nullptr) {
    const size_t mark = code_.size();
    first_ = static_cast<uint32_t>(mark);
    nregs_ = 0;
    what_ = "material";
    block_ = &def;
    try {
      std::map<std::string, SVal> locals = block_scope(def, overrides);
      static const char* const kFields[FT_BSDF_HOOK_PARAMS] = {
          "position", "local_position", "normal", "view_dir", "front_face", "object_id", "material_id",
          "wo", "wi", "current_ior", "u1", "u2", "u3"};
      const int n_params = bsdf ? FT_BSDF_HOOK_PARAMS : FT_MATERIAL_HOOK_PARAMS;
      SVal ctx;
      ctx.is_const = false;
      ctx.rec = std::make_shared<std::map<std::string, SVal>>();
      for (int k = 0; k < n_params; ++k) {
        SVal r = reg(nregs_++, k < 4 || k == 7 || k == 8);
        if (k < 10 || sample_randoms) (*ctx.rec)[kFields[k]] = r;
      }
      locals[fn.params[0]] = ctx;
      SVal result = run_body(fn.body, locals, 0);
      if (field) {
        SVal picked;
        if (result.rec) {
          auto it = result.rec->find(field);
          if (it == result.rec->end()) {
            code_.resize(mark);
            return false;
          }
          picked = it->second;
        } else if (result.is_const && result.cv.kind == Value::Object) {
          const Value* v = result.cv.obj->get(field);
          if (!v) {
            code_.resize(mark);
            return false;
          }
          picked = cst(*v);
        } else {
          fail("sample does not return a record");
        }
        result = picked;
      }
      if (result.rec) fail("returns the context");
      int r = materialize(result);
      bool rv = reg_vec3(result);
      if ((want == 0 && rv) || (want == 1 && !rv)) {
        code_.resize(mark);
        return false;
      }
      ft_instr ret{};
      ret.op = FT_OP_RET;
      ret.a = static_cast<uint8_t>(r);
      ret.flags = rv ? FT_INSTR_VEC3 : 0;
      code_.push_back(ret);
      ft_program prog{};
      prog.first_instr = first_;
      prog.n_instr = static_cast<uint32_t>(code_.size()) - first_;
      prog.n_params = static_cast<uint32_t>(n_params);
      prog.param_is_vec3 = bsdf ? 0x18fu : 0xfu;
      prog.n_regs = static_cast<uint32_t>(nregs_);
      prog.result_is_vec3 = rv ? 1u : 0u;
      if (nregs_ > FT_MAX_PROGRAM_REGS) {
        code_.resize(mark);
        return false;
      }
      *out = prog;
      return true;
    } catch (const FrontendError&) {
      code_.resize(mark);
      return false;
    }
  }

  // eval_material_properties_with_overrides (E:2804-2858): the definition's
  // bindings and property assignments in order, an instance field of the same
  // name replacing either; property values must fold to constants.  Returns
  // false when the evaluation fails (the reference then applies none).
  bool eval_properties(const BlockDef& def, const ObjectData& overrides, std::map<std::string, Value>* props) {
    what_ = "material property";
    try {
      std::map<std::string, SVal> locals;
      for (const auto& kv : overrides.fields) locals[kv.first] = cst(kv.second);
      for (const BlockStmt& s : def.statements) {
        if (s.kind == BlockStmt::Function || !s.expr) continue;
        const Value* ov = overrides.get(s.name);
        SVal v = ov ? cst(*ov) : eval(*s.expr, locals, 0);
        if (s.kind == BlockStmt::Binding) {
          locals[s.name] = v;
        } else {
          if (!v.is_const) return false;
          (*props)[s.name] = v.cv;
        }
      }
      return true;
    } catch (const FrontendError&) {
      return false;
    }
  }

 private:
  // The scope of a block definition's functions: instance fields, then the
  // bindings in order (an instance field of the same name replacing one);
  // helper functions see the same bindings.
  std::map<std::string, SVal> block_scope(const BlockDef& def, const ObjectData& overrides) {
    std::map<std::string, SVal> locals;
    for (const auto& kv : overrides.fields) locals[kv.first] = cst(kv.second);
    block_locals_.clear();
    for (const BlockStmt& s : def.statements) {
      if (s.kind != BlockStmt::Binding || !s.expr) continue;
      const Value* ov = overrides.get(s.name);
      locals[s.name] = ov ? cst(*ov) : eval(*s.expr, locals, 0);
      block_locals_[s.name] = locals[s.name];
    }
    return locals;
  }

  const EvalState& st_;
  std::vector<ft_instr>& code_;
  uint32_t first_ = 0;
  int nregs_ = 0;
  const char* what_ = "";
  const BlockDef* block_ = nullptr;
  std::map<std::string, SVal> block_locals_;

  [[noreturn]] void fail(const std::string& m) { lower_fail(FT_ERR_UNSUPPORTED, std::string(what_) + " hook: " + m); }

  bool reg_vec3(const SVal& v) {
    if (!v.is_const) return v.vec3;
    if (v.cv.kind == Value::Number) return false;
    float t[3];
    if (as_vec3(v.cv, t)) return true;
    fail("value is neither a number nor a vec3");
  }

  int emit(uint8_t op, uint8_t flags, int a = 0, int b = 0, int c = 0) {
    ft_instr in{};
    in.op = op;
    in.flags = flags;
    in.dst = static_cast<uint8_t>(nregs_);
    in.a = static_cast<uint8_t>(a);
    in.b = static_cast<uint8_t>(b);
    in.c = static_cast<uint8_t>(c);
    code_.push_back(in);
    if (nregs_ >= 255) fail("too many registers");
    return nregs_++;
  }

  int materialize(const SVal& v) {
    if (!v.is_const) return v.reg;
    ft_instr in{};
    in.op = FT_OP_CONST;
    in.dst = static_cast<uint8_t>(nregs_);
    if (v.cv.kind == Value::Number) {
      in.imm[0] = in.imm[1] = in.imm[2] = v.cv.num;
    } else {
      float t[3];
      if (!as_vec3(v.cv, t)) fail("value is neither a number nor a vec3");
      in.flags = FT_INSTR_VEC3;
      in.imm[0] = t[0]; in.imm[1] = t[1]; in.imm[2] = t[2];
    }
    code_.push_back(in);
    return nregs_++;
  }

  SVal reg(int r, bool vec) {
    SVal s;
    s.is_const = false;
    s.reg = r;
    s.vec3 = vec;
    return s;
  }
  SVal cst(const Value& v) {
    SVal s;
    s.cv = v;
    return s;
  }

  SVal run_body(const std::vector<FnStmt>& body, std::map<std::string, SVal>& locals, int depth) {
    for (const FnStmt& s : body) {
      if (s.is_return) return eval(*s.expr, locals, depth);
      locals[s.name] = eval(*s.expr, locals, depth);
    }
    fail("function missing return");
  }

  SVal call_user(const std::vector<std::string>& params, const std::vector<FnStmt>& body,
                 const std::vector<SVal>& args, std::map<std::string, SVal> locals, int depth) {
    if (depth >= 32) fail("call depth exceeded");
    if (params.size() != args.size()) fail("call on unsupported callee");
    for (size_t i = 0; i < params.size(); ++i) locals[params[i]] = args[i];
    return run_body(body, locals, depth + 1);
  }

  SVal eval(const Expr& e, std::map<std::string, SVal>& locals, int depth) {
    switch (e.kind) {
      case Expr::Number: return cst(Value::number(static_cast<float>(e.number)));
      case Expr::String: {
        Value v;
        v.kind = Value::String;
        v.str = e.text;
        return cst(v);
      }
      case Expr::Ident: {
        auto it = locals.find(e.text);
        if (it != locals.end()) return it->second;
        auto b = st_.bindings.find(e.text);
        if (b == st_.bindings.end()) fail("undefined identifier '" + e.text + "'");
        return cst(b->second.value);
      }
      case Expr::ObjectLiteral: {
        // A literal whose fields all fold is a constant object; one with
        // run-time fields is a record (a BsdfSample returned by a sample
        // hook), whose fields are read by member access.
        std::map<std::string, SVal> vals;
        bool all_const = true;
        for (const auto& kv : e.fields) {
          SVal v = eval(*kv.second, locals, depth);
          if (!v.is_const) {
            if (e.text == "vec3") return vec3_literal(e, locals, depth);
            all_const = false;
          }
          vals[kv.first] = v;
        }
        if (all_const) {
          std::map<std::string, Value> f;
          for (auto& kv : vals) f[kv.first] = kv.second.cv;
          return cst(make_object(e.text, std::move(f)));
        }
        SVal r;
        r.is_const = false;
        r.rec = std::make_shared<std::map<std::string, SVal>>(std::move(vals));
        return r;
      }
      case Expr::Member: {
        // A dotted name bound at top level (`alias.name` of an aliased
        // import) is read before member access (E:494-499).
        std::string flat;
        if (flatten_member(e, &flat)) {
          auto b = st_.bindings.find(flat);
          if (b != st_.bindings.end()) return cst(b->second.value);
        }
        SVal base = eval(*e.lhs, locals, depth);
        if (base.rec) {
          auto it = base.rec->find(e.text);
          if (it == base.rec->end()) fail("undefined identifier '" + e.text + "'");
          return it->second;
        }
        if (base.is_const) {
          if (base.cv.kind != Value::Object) fail("member access requires object value");
          const Value* v = base.cv.obj->get(e.text);
          if (!v) fail("undefined identifier '" + e.text + "'");
          return cst(*v);
        }
        if (!base.vec3) fail("member access on a number");
        uint8_t op = e.text == "x" ? FT_OP_GETX : e.text == "y" ? FT_OP_GETY : e.text == "z" ? FT_OP_GETZ : 0;
        if (!op) fail("undefined identifier '" + e.text + "'");
        return reg(emit(op, 0, base.reg), false);
      }
      case Expr::Unary: {
        SVal v = eval(*e.lhs, locals, depth);
        if (v.is_const) {
          if (v.cv.kind == Value::Number) return cst(Value::number(-v.cv.num));
          float t[3];
          if (!as_vec3(v.cv, t)) fail("unary operation requires numeric or vec3 operand");
          return cst(make_vec3(-t[0], -t[1], -t[2]));
        }
        return reg(emit(FT_OP_NEG, v.vec3 ? FT_INSTR_VEC3 : 0, v.reg), v.vec3);
      }
      case Expr::Binary: {
        SVal l = eval(*e.lhs, locals, depth);
        SVal r = eval(*e.rhs, locals, depth);
        if (e.op == '&') fail("binary operation requires numeric operands");
        uint8_t op = e.op == '+' ? FT_OP_ADD : e.op == '-' ? FT_OP_SUB : e.op == '*' ? FT_OP_MUL : FT_OP_DIV;
        if (l.is_const && r.is_const) return cst(fold_binary(l.cv, e.op, r.cv));
        return arith({l, r}, op);
      }
      case Expr::Call: return call(e, locals, depth);
      case Expr::FunctionLiteral: {
        // A closure literal inside a hook: keep as a constant function value.
        Value v;
        v.kind = Value::Function;
        v.fn = std::make_shared<FunctionData>();
        v.fn->params = e.params;
        v.fn->body = e.body;
        for (const auto& kv : locals)
          if (kv.second.is_const) v.fn->captures[kv.first] = kv.second.cv;
        return cst(v);
      }
      case Expr::Array: fail("arrays are not supported in hooks");
    }
    fail("unsupported expression");
  }

  SVal vec3_literal(const Expr& e, std::map<std::string, SVal>& locals, int depth) {
    SVal comp[3];
    const char* names[3] = {"x", "y", "z"};
    for (int k = 0; k < 3; ++k) {
      const ExprP* found = nullptr;
      for (const auto& kv : e.fields)
        if (kv.first == names[k]) found = &kv.second;
      if (!found) fail("vec3 literal without field " + std::string(names[k]));
      comp[k] = eval(**found, locals, depth);
      if (reg_vec3(comp[k])) fail("vec3 literal field is not a number");
    }
    int a = materialize(comp[0]), b = materialize(comp[1]), c = materialize(comp[2]);
    return reg(emit(FT_OP_VEC3, FT_INSTR_VEC3, a, b, c), true);
  }

  Value fold_binary(const Value& l, char op, const Value& r) {
    if (l.kind == Value::Number && r.kind == Value::Number) {
      switch (op) {
        case '+': return Value::number(l.num + r.num);
        case '-': return Value::number(l.num - r.num);
        case '*': return Value::number(l.num * r.num);
        default: return Value::number(l.num / r.num);
      }
    }
    float a[3], b[3];
    if (!as_broadcast_vec3(l, a) || !as_broadcast_vec3(r, b)) fail("binary operation requires numeric operands");
    switch (op) {
      case '+': return make_vec3(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
      case '-': return make_vec3(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
      case '*': return make_vec3(a[0] * b[0], a[1] * b[1], a[2] * b[2]);
      default: return make_vec3(a[0] / b[0], a[1] / b[1], a[2] / b[2]);
    }
  }

  // Component-wise op over scalar/vec3 operands with broadcasting.
  SVal arith(const std::vector<SVal>& ops, uint8_t op) {
    bool any_vec = false;
    for (const SVal& s : ops) any_vec |= reg_vec3(s);
    int r[3] = {0, 0, 0};
    uint8_t flags = any_vec ? FT_INSTR_VEC3 : 0;
    for (size_t i = 0; i < ops.size(); ++i) {
      r[i] = materialize(ops[i]);
      if (any_vec && !reg_vec3(ops[i])) flags |= static_cast<uint8_t>(FT_INSTR_A_SCALAR << i);
    }
    return reg(emit(op, flags, r[0], r[1], r[2]), any_vec);
  }

  SVal call(const Expr& e, std::map<std::string, SVal>& locals, int depth) {
    const Expr& callee = *e.lhs;
    std::vector<SVal> args;
    for (const ExprP& a : e.items) args.push_back(eval(*a, locals, depth));
    bool all_const = true;
    for (const SVal& a : args) all_const &= a.is_const;
    if (callee.kind == Expr::Ident) {
      const std::string& name = callee.text;
      if (all_const) {
        std::vector<Value> cv;
        for (const SVal& a : args) cv.push_back(a.cv);
        bool found = false;
        Value r = eval_builtin(name, cv, &found);
        if (found) return cst(r);
      } else if (SVal out; builtin_symbolic(name, args, &out)) {
        return out;
      }
      auto li = locals.find(name);
      if (li != locals.end() && li->second.is_const && li->second.cv.kind == Value::Function) {
        const FunctionData& fn = *li->second.cv.fn;
        std::map<std::string, SVal> inner;
        for (const auto& kv : fn.captures) inner[kv.first] = cst(kv.second);
        return call_user(fn.params, fn.body, args, inner, depth);
      }
      if (block_) {
        for (const BlockStmt& s : block_->statements) {
          if (s.kind == BlockStmt::Function && s.name == name)
            return call_user(s.params, s.body, args, block_locals_, depth);
        }
      }
      auto fi = st_.function_defs.find(name);
      if (fi != st_.function_defs.end()) return call_user(fi->second->params, fi->second->body, args, {}, depth);
      auto bi = st_.bindings.find(name);
      if (bi != st_.bindings.end() && bi->second.value.kind == Value::Function) {
        const FunctionData& fn = *bi->second.value.fn;
        std::map<std::string, SVal> inner;
        for (const auto& kv : fn.captures) inner[kv.first] = cst(kv.second);
        return call_user(fn.params, fn.body, args, inner, depth);
      }
      fail("call to unknown function '" + name + "'");
    }
    // `alias.fn(...)`: a function of an aliased import (E:1855-1866).
    std::string flat;
    if (flatten_member(callee, &flat)) {
      auto fi = st_.function_defs.find(flat);
      if (fi != st_.function_defs.end()) return call_user(fi->second->params, fi->second->body, args, {}, depth);
    }
    fail("call on unsupported callee");
  }

  bool builtin_symbolic(const std::string& name, const std::vector<SVal>& a, SVal* out) {
    auto need = [&](size_t n) {
      if (a.size() != n) fail("builtin " + name + " expects " + std::to_string(n) + " args");
    };
    struct U { const char* n; uint8_t op; };
    static const U unary[] = {{"abs", FT_OP_ABS}, {"floor", FT_OP_FLOOR}, {"ceil", FT_OP_CEIL},
                              {"fract", FT_OP_FRACT}, {"sqrt", FT_OP_SQRT}, {"sin", FT_OP_SIN},
                              {"cos", FT_OP_COS}, {"saturate", FT_OP_SATURATE}};
    for (const U& u : unary) {
      if (name == u.n) {
        need(1);
        *out = arith(a, u.op);
        return true;
      }
    }
    if (name == "min" || name == "max" || name == "pow") {
      need(2);
      *out = arith(a, name == "min" ? FT_OP_MIN : name == "max" ? FT_OP_MAX : FT_OP_POW);
      return true;
    }
    if (name == "clamp" || name == "mix") {
      need(3);
      *out = arith(a, name == "clamp" ? FT_OP_CLAMP : FT_OP_MIX);
      return true;
    }
    if (name == "step" || name == "smoothstep") {
      need(name == "step" ? 2 : 3);
      for (const SVal& s : a)
        if (reg_vec3(s)) fail("builtin " + name + " expects numeric args");
      *out = arith(a, name == "step" ? FT_OP_STEP : FT_OP_SMOOTHSTEP);
      return true;
    }
    if (name == "vec3") {
      if (a.size() == 1) {
        if (reg_vec3(a[0])) fail("builtin vec3 expects numeric args");
        int r = materialize(a[0]);
        *out = reg(emit(FT_OP_VEC3, FT_INSTR_VEC3, r, r, r), true);
        return true;
      }
      need(3);
      int r[3];
      for (int k = 0; k < 3; ++k) {
        if (reg_vec3(a[k])) fail("builtin vec3 expects numeric args");
        r[k] = materialize(a[k]);
      }
      *out = reg(emit(FT_OP_VEC3, FT_INSTR_VEC3, r[0], r[1], r[2]), true);
      return true;
    }
    if (name == "dot") {
      need(2);
      if (!reg_vec3(a[0]) || !reg_vec3(a[1])) fail("builtin dot expects vec3 args");
      int x = materialize(a[0]), y = materialize(a[1]);
      *out = reg(emit(FT_OP_DOT, 0, x, y), false);
      return true;
    }
    if (name == "length" || name == "normalize") {
      need(1);
      if (!reg_vec3(a[0])) fail("builtin " + name + " expects vec3 args");
      int x = materialize(a[0]);
      bool n = name == "normalize";
      *out = reg(emit(n ? FT_OP_NORMALIZE : FT_OP_LENGTH, n ? FT_INSTR_VEC3 : 0, x), n);
      return true;
    }
    if (name == "rotate_x" || name == "rotate_y" || name == "rotate_z") {
      need(2);
      if (!reg_vec3(a[0])) fail("builtin " + name + " expects vec3 args");
      if (reg_vec3(a[1])) fail("builtin " + name + " expects numeric args");
      int x = materialize(a[0]), d = materialize(a[1]);
      uint8_t op = name == "rotate_x" ? FT_OP_ROTX : name == "rotate_y" ? FT_OP_ROTY : FT_OP_ROTZ;
      *out = reg(emit(op, FT_INSTR_VEC3, x, d), true);
      return true;
    }
    return false;
  }
};

// ------------------------------------------------------------ scene lowering
class Lowerer {
 public:
  Lowerer(const EvalState& st, OwnedSceneDesc& out) : st_(st), out_(out) {}

  void run() {
    const Value* root = find_scene_root();
    if (!root) lower_fail(FT_ERR_MISSING_SCENE_ROOT, "no suitable scene root found (expected binding like scene/result/b/s)");
    default_material_ = parse_material(*root);
    out_.materials.push_back(default_material_);  // CompileContext::new (R:466-475)
    int r = compile_sdf(*root);
    out_.desc.root = r;
    V3 c = sdf_center(r);
    out_.desc.scene_center[0] = c.x;
    out_.desc.scene_center[1] = c.y;
    out_.desc.scene_center[2] = c.z;
    parse_camera();
    parse_lights();
    parse_settings();
    parse_environment();
  }

 private:
  const EvalState& st_;
  OwnedSceneDesc& out_;
  uint32_t next_object_id_ = 1;
  ft_material default_material_{};
  std::vector<std::pair<const FunctionData*, int>> hook_cache_;
  std::map<std::array<float, 7>, int32_t> pattern_programs_;  // (colour a, colour b, scale) -> program

  const Value* find_scene_root() {
    for (const char* k : {"scene", "result", "b", "s"}) {
      auto it = st_.bindings.find(k);
      if (it != st_.bindings.end()) return &it->second.value;
    }
    return nullptr;
  }

  int push(const ft_node& n) {
    out_.nodes.push_back(n);
    return static_cast<int>(out_.nodes.size()) - 1;
  }
  static ft_node blank(int kind) {
    ft_node n;
    std::memset(&n, 0, sizeof(n));
    n.kind = kind;
    n.a = n.b = n.program = -1;
    return n;
  }

  uint32_t alloc_object_id() { return next_object_id_++; }

  uint32_t intern_material(const ft_material& m) {
    for (size_t i = 0; i < out_.materials.size(); ++i)
      if (material_equal(out_.materials[i], m)) return static_cast<uint32_t>(i);
    out_.materials.push_back(m);
    return static_cast<uint32_t>(out_.materials.size()) - 1;
  }

  // medium_from_value (R:6834-6845): an object value of any type gives an
  // explicit medium, IOR clamped to [1, 3], absorption colour white and
  // density 0 (at least 0) unless given; any other value leaves none.
  static void read_medium(const Value* v, ft_material* m) {
    if (!v || v->kind != Value::Object) return;
    const ObjectData& mo = *v->obj;
    V3 a;
    if (!read_spectrum(mo, "absorption_color", &a)) a = v3(1.0f, 1.0f, 1.0f);
    m->has_medium = 1;
    m->medium_ior = clampf(number_or(mo, {"ior"}, 1.0f), 1.0f, 3.0f);
    m->medium_absorption[0] = a.x;
    m->medium_absorption[1] = a.y;
    m->medium_absorption[2] = a.z;
    m->medium_density = std::max(number_or(mo, {"density"}, 0.0f), 0.0f);
  }

  // material_from_object (R:6439-6570), without the dynamic-hook machinery.
  // Every model reads the `medium` and `pattern` fields (R:6458-6460,
  // R:6517-6519, R:6535-6537, R:6564-6566).
  ft_material material_from_object(const ObjectData& o) {
    if (st_.material_defs.count(o.type_name)) return material_from_dynamic_def(*st_.material_defs.at(o.type_name), o);
    ft_material m = material_from_builtin(o);
    read_medium(o.get("medium"), &m);
    m.color_program = pattern_program(o.get("pattern"));
    return m;
  }

  // read_pattern_field (R:6802-6825) with resolve_pattern_color (R:7233-7250):
  // a Checker3d (or Checker) pattern gives a hit colour_a or colour_b by the
  // parity of floor(local position * scale) summed over the axes.  It is
  // lowered as the material's colour hook, through the hook compiler, so it
  // runs wherever hooks run and replaces the colour where the reference's
  // pattern does (resolve_leaf_material, R:7164-7530).  Sums of the floors
  // in f32 equal the reference's i32 sums while |local * scale| < 2^24.
  // One program per distinct (colours, scale); -1 for no or another pattern.
  int32_t pattern_program(const Value* v) {
    if (!v || v->kind != Value::Object) return -1;
    const ObjectData& po = *v->obj;
    std::string kind = po.type_name;
    for (char& ch : kind) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    if (kind != "checker3d" && kind != "checker") return -1;
    V3 a, b;
    if (!read_spectrum(po, "color_a", &a) && !read_spectrum(po, "color1", &a) && !read_spectrum(po, "a", &a))
      a = v3(0.15f, 0.15f, 0.15f);
    if (!read_spectrum(po, "color_b", &b) && !read_spectrum(po, "color2", &b) && !read_spectrum(po, "b", &b))
      b = v3(0.85f, 0.85f, 0.85f);
    const float scale = std::max(number_or(po, {"scale", "frequency", "freq"}, 4.0f), 1.0e-4f);
    const std::array<float, 7> key = {a.x, a.y, a.z, b.x, b.y, b.z, scale};
    auto hit = pattern_programs_.find(key);
    if (hit != pattern_programs_.end()) return hit->second;
    // The pattern's constants enter as instance overrides of the definition's
    // bindings, so no number is printed into source text.
    static const std::shared_ptr<BlockDef> def = parse_program(
        "material Checker3dPattern {\n"
        "  model: Lambert;\n"
        "  let color_a = vec3(0.0);\n"
        "  let color_b = vec3(0.0);\n"
        "  let scale = 1.0;\n"
        "  fn color(ctx) {\n"
        "    let s = floor(ctx.local_position * scale);\n"
        "    let n = s.x + s.y + s.z;\n"
        "    return mix(color_a, color_b, n - 2.0 * floor(n * 0.5));\n"
        "  }\n"
        "};\n")[0].block;
    ObjectData overrides;
    overrides.fields["color_a"] = make_vec3(a.x, a.y, a.z);
    overrides.fields["color_b"] = make_vec3(b.x, b.y, b.z);
    overrides.fields["scale"] = Value::number(scale);
    int32_t idx = -1;
    for (const BlockStmt& st : def->statements) {
      if (st.kind != BlockStmt::Function || st.name != "color") continue;
      HookCompiler hook(st_, out_.instrs);
      ft_program prog;
      if (hook.compile_ctx(st, *def, overrides, 1, &prog)) {
        out_.programs.push_back(prog);
        idx = static_cast<int32_t>(out_.programs.size()) - 1;
      }
    }
    pattern_programs_[key] = idx;
    return idx;
  }

  ft_material material_from_builtin(const ObjectData& o) {
    const std::string& t = o.type_name;
    auto lower = [](std::string s) {
      for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
      return s;
    };
    std::string lt = lower(t);
    V3 col;
    ft_material m;
    auto emission = [&](ft_material& mm) {
      V3 ec;
      if (read_spectrum(o, "emission_color", &ec)) {
        mm.emission_color[0] = ec.x; mm.emission_color[1] = ec.y; mm.emission_color[2] = ec.z;
      }
      mm.emission_strength = std::max(number_or(o, {"emission_strength"}, 0.0f), 0.0f);
    };
    auto set_color = [&](ft_material& mm, V3 def) {
      if (!read_spectrum(o, "color", &col) && !read_spectrum(o, "base_color", &col)) col = def;
      mm.color[0] = col.x; mm.color[1] = col.y; mm.color[2] = col.z;
    };
    if (lt == "lambert") {
      m = material_defaults(FT_MAT_LAMBERT);
      set_color(m, v3(0.8f, 0.8f, 0.8f));
      m.roughness = 1.0f;
      emission(m);
      return m;
    }
    if (lt == "metal") {
      m = material_defaults(FT_MAT_METAL);
      set_color(m, v3(0.9f, 0.9f, 0.9f));
      m.roughness = clampf(number_or(o, {"roughness"}, 0.1f), 0.0f, 1.0f);
      m.metallic = 1.0f;
      m.specular = 1.0f;
      emission(m);
      return m;
    }
    if (lt == "dielectric") {
      m = material_defaults(FT_MAT_DIELECTRIC);
      set_color(m, v3(1.0f, 1.0f, 1.0f));
      m.ior = clampf(number_or(o, {"ior"}, 1.5f), 1.0f, 3.0f);
      m.roughness = clampf(number_or(o, {"roughness"}, 0.0f), 0.0f, 1.0f);
      m.thin_walled = number_or(o, {"thin_walled"}, 0.0f) >= 0.5f;
      m.transmission = 1.0f;
      emission(m);
      return m;
    }
    m = material_defaults(FT_MAT_STANDARD);
    if (!read_spectrum(o, "color", &col) && !read_spectrum(o, "base_color", &col) && !read_spectrum(o, "albedo", &col))
      col = v3(0.8f, 0.8f, 0.8f);
    m.color[0] = col.x; m.color[1] = col.y; m.color[2] = col.z;
    m.roughness = clampf(number_or(o, {"roughness"}, 0.5f), 0.0f, 1.0f);
    m.metallic = clampf(number_or(o, {"metallic", "metalness"}, 0.0f), 0.0f, 1.0f);
    m.ior = clampf(number_or(o, {"ior", "specular_ior"}, 1.5f), 1.0f, 3.0f);
    m.transmission = clampf(number_or(o, {"transmission", "transmission_weight"}, 0.0f), 0.0f, 1.0f);
    m.thin_walled = number_or(o, {"thin_walled"}, 0.0f) >= 0.5f;
    m.specular = clampf(number_or(o, {"specular"}, 0.5f), 0.0f, 1.0f);
    m.specular_weight = clampf(number_or(o, {"specular_weight"}, 1.0f), 0.0f, 1.0f);
    V3 sc;
    if (read_spectrum(o, "specular_color", &sc)) {
      m.specular_color[0] = sc.x; m.specular_color[1] = sc.y; m.specular_color[2] = sc.z;
    }
    m.clearcoat = clampf(number_or(o, {"clearcoat"}, 0.0f), 0.0f, 1.0f);
    m.clearcoat_roughness = clampf(number_or(o, {"clearcoat_roughness"}, 0.1f), 0.0f, 1.0f);
    emission(m);
    return m;
  }

  // material_from_dynamic_def (R:6633-6690) with apply_dynamic_material_
  // properties (R:6692-6770): the model's parameters, then the definition's
  // property assignments.  Metal and Dielectric definitions keep their kind;
  // every other model (Lambert included) is a Standard material, with the
  // Lambert parameters unless the model is Standard or Layered.  The
  // definition's functions (`fn color(ctx)` and the other per-hit hooks) are
  // not evaluated.
  ft_material material_from_dynamic_def(const BlockDef& def, const ObjectData& overrides) {
    ft_material m;
    const std::string& model = def.model;
    if (model == "Metal") {
      m = material_defaults(FT_MAT_METAL);  // MaterialParams::metal (materials/mod.rs:154-181)
      m.color[0] = m.color[1] = m.color[2] = 0.9f;
      m.roughness = 0.1f;
      m.metallic = 1.0f;
      m.specular = 1.0f;
    } else if (model == "Dielectric") {
      m = material_defaults(FT_MAT_DIELECTRIC);  // MaterialParams::dielectric (materials/mod.rs:183-212)
      m.color[0] = m.color[1] = m.color[2] = 1.0f;
      m.ior = 1.5f;
      m.roughness = 0.0f;
      m.transmission = 1.0f;
    } else {
      m = material_defaults(FT_MAT_STANDARD);
      if (model != "Standard" && model != "Layered") m.roughness = 1.0f;  // MaterialParams::lambert
    }
    std::vector<ft_instr> scratch;
    HookCompiler hc(st_, scratch);
    std::map<std::string, Value> props;
    if (!hc.eval_properties(def, overrides, &props)) return m;
    auto num = [&](const char* k, float* out) {
      auto it = props.find(k);
      if (it == props.end() || it->second.kind != Value::Number) return false;
      *out = it->second.num;
      return true;
    };
    auto spec = [&](const char* k, float* out3) {
      auto it = props.find(k);
      if (it == props.end()) return false;
      ObjectData holder;
      holder.fields[k] = it->second;
      V3 c;
      if (!read_spectrum(holder, k, &c)) return false;
      out3[0] = c.x; out3[1] = c.y; out3[2] = c.z;
      return true;
    };
    float v;
    spec("color", m.color);
    if (num("roughness", &v)) m.roughness = clampf(v, 0.0f, 1.0f);
    if (num("ior", &v)) m.ior = clampf(v, 1.0f, 3.0f);
    if (num("metallic", &v)) m.metallic = clampf(v, 0.0f, 1.0f);
    if (num("specular", &v)) m.specular = clampf(v, 0.0f, 1.0f);
    if (num("specular_weight", &v)) m.specular_weight = clampf(v, 0.0f, 1.0f);
    spec("specular_color", m.specular_color);
    if (num("clearcoat", &v)) m.clearcoat = clampf(v, 0.0f, 1.0f);
    if (num("clearcoat_roughness", &v)) m.clearcoat_roughness = clampf(v, 0.0f, 1.0f);
    if (num("transmission", &v)) m.transmission = clampf(v, 0.0f, 1.0f);
    if (num("thin_walled", &v)) m.thin_walled = v >= 0.5f;
    spec("emission_color", m.emission_color);
    if (num("emission_strength", &v)) m.emission_strength = std::max(v, 0.0f);
    auto medium = props.find("medium");
    if (medium != props.end()) read_medium(&medium->second, &m);
    // Per-hit hooks (resolve_leaf_material, R:7164-7530; build_bsdf_context
    // R:4397-4449; the BSDF functions R:4905-4950).  A Standard or Layered
    // definition's specular colour, IOR, clearcoat and clearcoat roughness are
    // the coat's at every hit whatever their own hooks return, so those hooks
    // are left out; metallic, specular, specular_weight, transmission and the
    // coat hooks are read for those two models only.  `fn medium(ctx)`'s record
    // is one program per field; a record with none of the three fields is not
    // lowered (the reference would take a medium of the defaults).
    // `fn subsurface(ctx)` is not lowered: no renderer path reads subsurface
    // parameters.
    const bool coated = model == "Standard" || model == "Layered";
    struct Slot {
      const char* name;
      int slot;
      int want;  // 0 number, 1 vec3, 2 either
      bool coated_only;
    };
    static const Slot kSlots[] = {
        {"emission_color", FT_HOOK_EMISSION_COLOR, 2, false},
        {"emission_strength", FT_HOOK_EMISSION_STRENGTH, 0, false},
        {"metallic", FT_HOOK_METALLIC, 0, true},
        {"specular", FT_HOOK_SPECULAR, 0, true},
        {"specular_weight", FT_HOOK_SPECULAR_WEIGHT, 0, true},
        {"transmission", FT_HOOK_TRANSMISSION, 0, true},
        {"coat_color", FT_HOOK_COAT_COLOR, 2, true},
        {"coat_roughness", FT_HOOK_COAT_ROUGHNESS, 0, true},
        {"coat_ior", FT_HOOK_COAT_IOR, 0, true},
        {"coat_weight", FT_HOOK_COAT_WEIGHT, 0, true},
        {"coat_mask", FT_HOOK_COAT_MASK, 0, true},
        {"bump", FT_HOOK_BUMP, 0, false},
        {"normal", FT_HOOK_NORMAL, 1, false},
    };
    // bsdf_sample_from_value (R:5032-5060): wi and f are required
    static const Slot kSample[] = {
        {"wi", FT_HOOK_SAMPLE_WI, 1, false},
        {"f", FT_HOOK_SAMPLE_F, 2, false},
        {"pdf", FT_HOOK_SAMPLE_PDF, 0, false},
        {"delta", FT_HOOK_SAMPLE_DELTA, 0, false},
        {"apply_cos", FT_HOOK_SAMPLE_APPLY_COS, 0, false},
        {"transmission", FT_HOOK_SAMPLE_TRANSMISSION, 0, false},
        {"thin_walled", FT_HOOK_SAMPLE_THIN_WALLED, 0, false},
        {"next_ior", FT_HOOK_SAMPLE_NEXT_IOR, 0, false},
    };
    auto add = [&](const BlockStmt& st, int want, bool bsdf, bool randoms, const char* field) -> int32_t {
      HookCompiler hook(st_, out_.instrs);
      ft_program prog;
      if (!hook.compile_ctx(st, def, overrides, want, &prog, bsdf, randoms, field)) return -1;
      out_.programs.push_back(prog);
      return static_cast<int32_t>(out_.programs.size()) - 1;
    };
    for (const BlockStmt& st : def.statements) {
      if (st.kind != BlockStmt::Function || st.params.size() != 1) continue;
      if (st.name == "color") {
        m.color_program = add(st, 2, false, false, nullptr);
      } else if (st.name == "roughness") {
        m.roughness_program = add(st, 0, false, false, nullptr);
      } else if (st.name == "ior") {
        if (!coated) m.ior_program = add(st, 0, false, false, nullptr);
      } else if (st.name == "thin_walled") {
        m.thin_walled_program = add(st, 0, false, false, nullptr);
      } else if (st.name == "eval") {
        m.hook_program[FT_HOOK_EVAL] = add(st, 2, true, false, nullptr);
      } else if (st.name == "pdf") {
        m.hook_program[FT_HOOK_PDF] = add(st, 0, true, false, nullptr);
      } else if (st.name == "medium") {
        // medium_from_value (R:6834-6845): ior, absorption_color and density,
        // each defaulted when the record lacks it
        const int32_t ior = add(st, 0, false, false, "ior");
        const int32_t absorption = add(st, 2, false, false, "absorption_color");
        const int32_t density = add(st, 0, false, false, "density");
        m.hook_program[FT_HOOK_MEDIUM_IOR] = ior;
        m.hook_program[FT_HOOK_MEDIUM_ABSORPTION] = absorption;
        m.hook_program[FT_HOOK_MEDIUM_DENSITY] = density;
      } else if (st.name == "sample") {
        int32_t progs[8];
        bool ok = true;
        for (int k = 0; k < 8; ++k) {
          progs[k] = add(st, kSample[k].want, true, true, kSample[k].name);
          if (k == 1 && progs[k] < 0) progs[k] = add(st, kSample[k].want, true, true, "color");
          if (k < 2 && progs[k] < 0) ok = false;
        }
        if (ok)
          for (int k = 0; k < 8; ++k) m.hook_program[kSample[k].slot] = progs[k];
      } else {
        for (const Slot& sl : kSlots)
          if (st.name == sl.name && (coated || !sl.coated_only))
            m.hook_program[sl.slot] = add(st, sl.want, false, false, nullptr);
      }
    }
    if (model == "Standard" || model == "Layered") {
      // resolve_leaf_material (R:7258-7470) then sets the coat at every hit:
      // specular colour, IOR, clearcoat and its roughness come from the
      // coat_* properties (defaults 1, 1.33, 0 and 0.08; coat_mask, a
      // per-hit hook only, is 1 without one).
      float cc[3] = {1.0f, 1.0f, 1.0f};
      spec("coat_color", cc);
      std::memcpy(m.specular_color, cc, sizeof(cc));
      m.ior = clampf(num("coat_ior", &v) ? v : 1.33f, 1.0f, 3.0f);
      m.clearcoat = clampf(num("coat_weight", &v) ? v : 0.0f, 0.0f, 1.0f);
      m.clearcoat_roughness = clampf(num("coat_roughness", &v) ? v : 0.08f, 0.0f, 1.0f);
    }
    return m;
  }

  // extract_material_kind (R:6404-6437); object fields are visited in name
  // order (the reference iterates a HashMap).
  bool extract_material_kind(const Value& v, ft_material* out) {
    if (v.kind != Value::Object) return false;
    const ObjectData& o = *v.obj;
    const Value* mv = o.get("material");
    if (mv && mv->kind == Value::Object) {
      *out = material_from_object(*mv->obj);
      return true;
    }
    for (const auto& kv : o.fields)
      if (extract_material_kind(kv.second, out)) return true;
    std::string lt = o.type_name;
    for (char& ch : lt) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    if (lt == "material" || lt == "standard" || lt == "openpbr" || lt == "lambert" || lt == "metal" ||
        lt == "dielectric" || st_.material_defs.count(o.type_name)) {
      *out = material_from_object(o);
      return true;
    }
    return false;
  }

  // parse_material (R:6390-6402)
  ft_material parse_material(const Value& root) {
    ft_material m;
    auto it = st_.bindings.find("material");
    if (it != st_.bindings.end() && extract_material_kind(it->second.value, &m)) return m;
    if (extract_material_kind(root, &m)) return m;
    return default_material();
  }

  uint32_t primitive_material_id(const ObjectData& o) {
    const Value* mv = o.get("material");
    if (mv && mv->kind == Value::Object) return intern_material(material_from_object(*mv->obj));
    return intern_material(default_material_);
  }

  // sdf_bounds (R:5242-5386)
  Aabb bounds(int idx) {
    const ft_node& n = out_.nodes[idx];
    V3 c = v3(n.center[0], n.center[1], n.center[2]);
    auto cube = [&](float r) { return Aabb{sub(c, v3(r, r, r)), add(c, v3(r, r, r))}; };
    switch (n.kind) {
      case FT_NODE_SPHERE: return cube(n.f[0]);
      case FT_NODE_BOX: return cube(length(v3(n.f[0], n.f[1], n.f[2])));
      case FT_NODE_CYLINDER:
      case FT_NODE_EXTRUDE_POLYGON: return cube(std::sqrt(n.f[0] * n.f[0] + n.f[1] * n.f[1]));
      case FT_NODE_TORUS: return cube(n.f[0] + n.f[1]);
      case FT_NODE_DOMAIN:
      case FT_NODE_DISTANCE_POST:
      case FT_NODE_NOISE:
      case FT_NODE_CUSTOM:
        return Aabb{v3(n.bounds_min[0], n.bounds_min[1], n.bounds_min[2]),
                    v3(n.bounds_max[0], n.bounds_max[1], n.bounds_max[2])};
      case FT_NODE_SUBTRACT: return bounds(n.a);
      case FT_NODE_SLICE: {
        Aabb b = bounds(n.a);
        float* mn = n.ival == 0 ? &b.mn.x : n.ival == 1 ? &b.mn.y : &b.mn.z;
        float* mx = n.ival == 0 ? &b.mx.x : n.ival == 1 ? &b.mx.y : &b.mx.z;
        *mn = std::max(*mn, n.f[0]);
        *mx = std::min(*mx, n.f[1]);
        if (*mx < *mn) *mx = *mn;
        return b;
      }
      case FT_NODE_SMOOTH: return aabb_expand(bounds(n.a), n.f[0] * 0.1f);
      default: return aabb_union(bounds(n.a), bounds(n.b));
    }
  }

  // sdf_center (R:4047-4089)
  V3 sdf_center(int idx) {
    const ft_node& n = out_.nodes[idx];
    if (is_primitive(n.kind) || is_modifier(n.kind)) return v3(n.center[0], n.center[1], n.center[2]);
    switch (n.kind) {
      case FT_NODE_UNION:
      case FT_NODE_INTERSECT:
      case FT_NODE_UNION_ROUND:
      case FT_NODE_UNION_CHAMFER:
      case FT_NODE_UNION_COLUMNS:
      case FT_NODE_UNION_STAIRS:
      case FT_NODE_UNION_SOFT:
      case FT_NODE_INTERSECT_ROUND:
      case FT_NODE_INTERSECT_CHAMFER:
      case FT_NODE_INTERSECT_COLUMNS:
      case FT_NODE_INTERSECT_STAIRS: {
        V3 l = sdf_center(n.a), r = sdf_center(n.b);
        return v3((l.x + r.x) * 0.5f, (l.y + r.y) * 0.5f, (l.z + r.z) * 0.5f);
      }
      default: return sdf_center(n.a);
    }
  }

  // transformed_modifier_bounds (R:2381-2394)
  Aabb transformed_modifier_bounds(int base, const Xf& t) {
    Aabb lb = bounds(base);
    V3 lc = mul(add(lb.mn, lb.mx), 0.5f);
    float lr = length(mul(sub(lb.mx, lb.mn), 0.5f));
    V3 c = add(t.c, transform_offset(t, lc));
    return aabb_expand(Aabb{sub(c, v3(lr, lr, lr)), add(c, v3(lr, lr, lr))}, 0.1f);
  }

  // split_modifier_base (R:1810-1948): strip the transform of a primitive or
  // noise node; returns (base, transform, bounds).
  int split_modifier_base(int idx, Xf* xf, Aabb* bb) {
    *bb = bounds(idx);
    ft_node n = out_.nodes[idx];
    if ((is_primitive(n.kind) && n.kind != FT_NODE_CUSTOM) || n.kind == FT_NODE_NOISE) {
      *xf = node_xf(n);
      set_xf(n, Xf{});
      if (n.kind == FT_NODE_NOISE) set_bounds(n, *bb);
      return push(n);
    }
    *xf = Xf{};
    return idx;
  }

  int compile_hook(const Value& fnv, bool domain) {
    const FunctionData* key = fnv.fn.get();
    for (const auto& kv : hook_cache_) {
      if (kv.first == key) return kv.second;
    }
    HookCompiler hc(st_, out_.instrs);
    ft_program p;
    if (domain) {
      if (fnv.fn->params.size() != 1) lower_fail(FT_ERR_UNSUPPORTED, "domain hook must take one parameter");
      p = hc.compile(fnv.fn->params, {true}, fnv.fn->body, fnv.fn->captures, nullptr, true, "domain");
    } else {
      if (fnv.fn->params.size() != 2) lower_fail(FT_ERR_UNSUPPORTED, "distance_post hook must take two parameters");
      p = hc.compile(fnv.fn->params, {false, true}, fnv.fn->body, fnv.fn->captures, nullptr, false, "distance_post");
    }
    out_.programs.push_back(p);
    int id = static_cast<int>(out_.programs.size()) - 1;
    hook_cache_.emplace_back(key, id);
    return id;
  }

  // apply_object_modifier_hooks (R:1750-1808)
  int apply_hooks(const ObjectData& o, int node) {
    const Value* dom = o.get("domain");
    const Value* post = o.get("distance_post");
    if (!dom && !post) return node;
    bool dom_fn = dom && dom->kind == Value::Function;
    bool post_fn = post && post->kind == Value::Function;
    Xf xf;
    Aabb bb;
    node = split_modifier_base(node, &xf, &bb);
    if (dom_fn) {
      ft_node m = blank(FT_NODE_DOMAIN);
      m.a = node;
      m.program = compile_hook(*dom, true);
      set_xf(m, xf);
      set_bounds(m, bb);
      node = push(m);
    }
    if (post_fn) {
      ft_node m = blank(FT_NODE_DISTANCE_POST);
      m.a = node;
      m.program = compile_hook(*post, false);
      set_xf(m, xf);
      set_bounds(m, bb);
      node = push(m);
    }
    return node;
  }

  // remap_sdf_node (R:2029-2326)
  int remap(int idx, const std::function<Xf(const Xf&)>& map) {
    ft_node n = out_.nodes[idx];
    if (is_primitive(n.kind)) {
      set_xf(n, map(node_xf(n)));
      if (n.kind == FT_NODE_CUSTOM) set_custom_box(n);
      n.object_id = alloc_object_id();
      return push(n);
    }
    if (is_modifier(n.kind)) {
      Xf t = map(node_xf(n));
      set_xf(n, t);
      set_bounds(n, transformed_modifier_bounds(n.a, t));
      return push(n);
    }
    if (is_binary(n.kind)) {
      int a = remap(n.a, map);
      int b = remap(n.b, map);
      n.a = a;
      n.b = b;
      return push(n);
    }
    // slice / smooth
    n.a = remap(n.a, map);
    return push(n);
  }

  const Value& required(const ObjectData& o, const char* name) {
    const Value* v = o.get(name);
    if (!v) lower_fail(FT_ERR_UNSUPPORTED_OBJECT, "unsupported object type '" + o.type_name + "' for rendering");
    return *v;
  }
  float required_number(const ObjectData& o, const char* name, float def) {
    const Value& v = required(o, name);
    return v.kind == Value::Number ? v.num : def;
  }

  int primitive(const ObjectData& o, int kind) {
    ft_node n = blank(kind);
    Xf t = read_transform(o);
    set_xf(n, t);
    switch (kind) {
      case FT_NODE_SPHERE: {
        float r = number_or(o, {"radius", "r"}, 1.0f);
        n.f[0] = r;
        n.f[1] = std::min(std::max(number_or(o, {"shell"}, 0.0f), 0.0f), r);
        break;
      }
      case FT_NODE_BOX: {
        V3 size;
        if (!read_vec3_field(o, "size", &size)) size = v3(1, 1, 1);
        V3 h = mul(size, 0.5f);
        float mh = std::min(h.x, std::min(h.y, h.z));
        n.f[0] = h.x; n.f[1] = h.y; n.f[2] = h.z;
        n.f[3] = std::min(std::max(number_or(o, {"round", "rounding"}, 0.0f), 0.0f), mh);
        n.f[4] = std::min(std::max(number_or(o, {"shell"}, 0.0f), 0.0f), mh);
        break;
      }
      case FT_NODE_CYLINDER:
      case FT_NODE_EXTRUDE_POLYGON: {
        if (kind == FT_NODE_EXTRUDE_POLYGON) {
          float s = number_or(o, {"sides", "n"}, 6.0f);
          n.ival = std::max(3, static_cast<int>(std::round(s)));
        }
        float r = number_or(o, {"radius", "r"}, 1.0f);
        float hh = number_or(o, {"height", "h"}, 1.0f) * 0.5f;
        float m = std::min(r, hh);
        n.f[0] = r;
        n.f[1] = hh;
        n.f[2] = std::min(std::max(number_or(o, {"round", "rounding"}, 0.0f), 0.0f), m);
        n.f[3] = std::min(std::max(number_or(o, {"shell"}, 0.0f), 0.0f), m);
        break;
      }
      case FT_NODE_TORUS:
        n.f[0] = number_or(o, {"major_radius", "R"}, 1.0f);
        n.f[1] = number_or(o, {"minor_radius", "r"}, 0.25f);
        break;
    }
    n.object_id = alloc_object_id();
    n.material_id = primitive_material_id(o);
    return push(n);
  }

  // World box of a Custom node: its half-extent box's corners through the
  // transform (sdf_bounds, R:5304-5326).
  static void set_custom_box(ft_node& n) {
    const float inf = std::numeric_limits<float>::infinity();
    Xf xf = node_xf(n);
    Aabb box{v3(inf, inf, inf), v3(-inf, -inf, -inf)};
    for (int c = 0; c < 8; ++c) {
      V3 corner = v3((c & 4) ? n.f[0] : -n.f[0], (c & 2) ? n.f[1] : -n.f[1], (c & 1) ? n.f[2] : -n.f[2]);
      V3 w = add(xf.c, transform_offset(xf, corner));
      box.mn = v3(std::min(box.mn.x, w.x), std::min(box.mn.y, w.y), std::min(box.mn.z, w.z));
      box.mx = v3(std::max(box.mx.x, w.x), std::max(box.mx.y, w.y), std::max(box.mx.z, w.z));
    }
    set_bounds(n, box);
  }

  // A user `sdf` definition as a Custom leaf (compile_sdf, R:1528-1550): its
  // distance / domain / distance_post functions lowered to hook programs, the
  // half extents of `bounds()` (eval_custom_sdf_bounds_half_extents,
  // R:6182-6204: a vec3 or a radius, each at least 1e-3, else 10,000), the
  // object's transform and material.  The world box is the transformed
  // corners of the half-extent box (sdf_bounds, R:5304-5326).
  int custom_sdf(const ObjectData& o, const BlockDef& def) {
    ft_node n = blank(FT_NODE_CUSTOM);
    Xf xf = read_transform(o);
    set_xf(n, xf);
    n.ival = n.reserved = -1;
    auto find_fn = [&](const char* name, size_t nparams) -> const BlockStmt* {
      for (const BlockStmt& st : def.statements)
        if (st.kind == BlockStmt::Function && st.name == name && st.params.size() == nparams) return &st;
      return nullptr;
    };
    auto lower_fn = [&](const BlockStmt* fn, const std::vector<bool>& vec, int want) -> int {
      if (!fn) return -1;
      HookCompiler hc(st_, out_.instrs);
      ft_program prog;
      if (!hc.compile_block_fn(*fn, def, o, vec, want, &prog)) return -2;
      out_.programs.push_back(prog);
      return static_cast<int>(out_.programs.size()) - 1;
    };
    n.program = lower_fn(find_fn("distance", 1), {true}, 0);
    if (n.program < 0)
      lower_fail(FT_ERR_UNSUPPORTED, "sdf '" + def.name + "': distance(p) must fold to a number program");
    n.ival = lower_fn(find_fn("domain", 1), {true}, 1);
    n.reserved = lower_fn(find_fn("distance_post", 2), {false, true}, 0);
    if (n.ival == -2 || n.reserved == -2)
      lower_fail(FT_ERR_UNSUPPORTED, "sdf '" + def.name + "': domain / distance_post hook cannot be lowered");
    V3 half = v3(10000.0f, 10000.0f, 10000.0f);
    if (const BlockStmt* bf = find_fn("bounds", 0)) {
      HookCompiler hc(st_, out_.instrs);
      Value bv;
      if (hc.const_block_fn(*bf, def, o, &bv)) {
        float t[3];
        if (bv.kind == Value::Number) {
          float r = std::max(std::fabs(bv.num), 1.0e-3f);
          half = v3(r, r, r);
        } else if (bv.kind == Value::Object) {
          float x = 0.0f, y = 0.0f, z = 0.0f;
          read_number(*bv.obj, {"x"}, &x);
          read_number(*bv.obj, {"y"}, &y);
          read_number(*bv.obj, {"z"}, &z);
          half = v3(std::max(std::fabs(x), 1.0e-3f), std::max(std::fabs(y), 1.0e-3f), std::max(std::fabs(z), 1.0e-3f));
          (void)t;
        }
      }
    }
    n.f[0] = half.x; n.f[1] = half.y; n.f[2] = half.z;
    set_custom_box(n);
    n.object_id = alloc_object_id();
    n.material_id = primitive_material_id(o);
    return push(n);
  }

  int compile_sdf(const Value& v) {
    if (v.kind != Value::Object) lower_fail(FT_ERR_EXPECTED_OBJECT, "expected object value for rendering");
    const ObjectData& o = *v.obj;
    const std::string t = o.has_type ? o.type_name : "anonymous";
    int node;
    struct Op { const char* name; int kind; int nargs; };
    static const Op binops[] = {
        {"add", FT_NODE_UNION, 0}, {"intersect", FT_NODE_INTERSECT, 0}, {"sub", FT_NODE_SUBTRACT, 0},
        {"union_round", FT_NODE_UNION_ROUND, 1}, {"union_chamfer", FT_NODE_UNION_CHAMFER, 1},
        {"union_soft", FT_NODE_UNION_SOFT, 1}, {"intersect_round", FT_NODE_INTERSECT_ROUND, 1},
        {"intersect_chamfer", FT_NODE_INTERSECT_CHAMFER, 1}, {"diff_round", FT_NODE_DIFF_ROUND, 1},
        {"diff_chamfer", FT_NODE_DIFF_CHAMFER, 1}, {"pipe", FT_NODE_PIPE, 1}, {"engrave", FT_NODE_ENGRAVE, 1},
        {"union_columns", FT_NODE_UNION_COLUMNS, 2}, {"union_stairs", FT_NODE_UNION_STAIRS, 2},
        {"intersect_columns", FT_NODE_INTERSECT_COLUMNS, 2}, {"intersect_stairs", FT_NODE_INTERSECT_STAIRS, 2},
        {"diff_columns", FT_NODE_DIFF_COLUMNS, 2}, {"diff_stairs", FT_NODE_DIFF_STAIRS, 2},
        {"groove", FT_NODE_GROOVE, 3}, {"tongue", FT_NODE_TONGUE, 3}};
    if (t == "Sphere") node = primitive(o, FT_NODE_SPHERE);
    else if (t == "Box") node = primitive(o, FT_NODE_BOX);
    else if (t == "Cylinder") node = primitive(o, FT_NODE_CYLINDER);
    else if (t == "Torus") node = primitive(o, FT_NODE_TORUS);
    else if (t == "ExtrudePolygon") node = primitive(o, FT_NODE_EXTRUDE_POLYGON);
    else {
      const Op* op = nullptr;
      for (const Op& b : binops)
        if (t == b.name) op = &b;
      if (op) {
        int l = compile_sdf(required(o, "lhs"));
        int r = compile_sdf(required(o, "rhs"));
        ft_node n = blank(op->kind);
        n.a = l;
        n.b = r;
        if (op->nargs == 1) {
          n.f[0] = required_number(o, "r", 0.0f);
        } else if (op->nargs == 2) {
          n.f[0] = required_number(o, "r", 0.0f);
          n.f[1] = required_number(o, "n", 4.0f);
        } else if (op->nargs == 3) {
          n.f[0] = required_number(o, "ra", 0.0f);
          n.f[1] = required_number(o, "rb", 0.0f);
        }
        node = push(n);
      } else if (t == "mirror_x" || t == "mirror_y" || t == "mirror_z") {
        const Value& base = required(o, "base");
        int lhs = compile_sdf(base);
        int axis = t == "mirror_x" ? 0 : t == "mirror_y" ? 1 : 2;
        int rhs0 = compile_sdf(base);
        int rhs = remap(rhs0, [axis](const Xf& x) {
          Xf m = x;
          if (axis == 0) { m.c.x = -m.c.x; m.r.y = -m.r.y; m.r.z = -m.r.z; }
          else if (axis == 1) { m.c.y = -m.c.y; m.r.x = -m.r.x; m.r.z = -m.r.z; }
          else { m.c.z = -m.c.z; m.r.x = -m.r.x; m.r.y = -m.r.y; }
          return m;
        });
        ft_node n = blank(FT_NODE_UNION);
        n.a = lhs;
        n.b = rhs;
        node = push(n);
      } else if (t == "repeat_x" || t == "repeat_y" || t == "repeat_z") {
        const Value& base = required(o, "base");
        float spacing = required_number(o, "spacing", 0.0f);
        const Value& cv = required(o, "count");
        size_t count = cv.kind == Value::Number ? static_cast<size_t>(std::max(std::round(cv.num), 1.0f)) : 1;
        int axis = t == "repeat_x" ? 0 : t == "repeat_y" ? 1 : 2;
        float start = -0.5f * static_cast<float>(count - 1) * spacing;
        auto offset_copy = [&](float delta) {
          int b = compile_sdf(base);
          return remap(b, [axis, delta](const Xf& x) {
            Xf m = x;
            if (axis == 0) m.c.x += delta;
            else if (axis == 1) m.c.y += delta;
            else m.c.z += delta;
            return m;
          });
        };
        node = offset_copy(start);
        for (size_t i = 1; i < count; ++i) {
          int part = offset_copy(start + static_cast<float>(i) * spacing);
          ft_node n = blank(FT_NODE_UNION);
          n.a = node;
          n.b = part;
          node = push(n);
        }
      } else if (t == "slice_x" || t == "slice_y" || t == "slice_z") {
        int b = compile_sdf(required(o, "base"));
        ft_node n = blank(FT_NODE_SLICE);
        n.a = b;
        n.ival = t == "slice_x" ? 0 : t == "slice_y" ? 1 : 2;
        n.f[0] = required_number(o, "min", -std::numeric_limits<float>::infinity());
        n.f[1] = required_number(o, "max", std::numeric_limits<float>::infinity());
        node = push(n);
      } else if (t == "noise") {
        int b = compile_sdf(required(o, "base"));
        const Value& oct = required(o, "octaves");
        const Value& sc = required(o, "scale");
        const Value& la = required(o, "lacunarity");
        Xf xf;
        Aabb bb;
        b = split_modifier_base(b, &xf, &bb);
        ft_node n = blank(FT_NODE_NOISE);
        n.a = b;
        n.ival = oct.kind == Value::Number ? static_cast<int>(clampf(std::round(oct.num), 1.0f, 16.0f)) : 7;
        n.f[0] = sc.kind == Value::Number ? std::max(sc.num, 1.0e-4f) : 1.0f;
        n.f[1] = la.kind == Value::Number ? std::max(la.num, 1.0e-4f) : 1.0f;
        set_xf(n, xf);
        set_bounds(n, bb);
        node = push(n);
      } else if (t == "smooth") {
        int b = compile_sdf(required(o, "base"));
        ft_node n = blank(FT_NODE_SMOOTH);
        n.a = b;
        n.f[0] = required_number(o, "k", 0.0f);
        node = push(n);
      } else if (st_.sdf_defs.count(t)) {
        node = custom_sdf(o, *st_.sdf_defs.at(t));
      } else {
        lower_fail(FT_ERR_UNSUPPORTED_OBJECT, "unsupported object type '" + t + "' for rendering");
      }
    }
    return apply_hooks(o, node);
  }

  // parse_camera (R:6263-6286).  Absent fields are stored as NaN so the
  // renderer can fall back to the scene centre / RenderOptions at render time.
  void parse_camera() {
    ft_camera& c = out_.desc.camera;
    const float nan = std::numeric_limits<float>::quiet_NaN();
    for (int i = 0; i < 3; ++i) c.origin[i] = c.target[i] = nan;
    c.up[0] = 0; c.up[1] = 1; c.up[2] = 0;
    c.fov_y_degrees = nan;
    out_.desc.has_camera = 0;
    auto it = st_.bindings.find("camera");
    if (it == st_.bindings.end() || it->second.value.kind != Value::Object) return;
    const ObjectData& o = *it->second.value.obj;
    out_.desc.has_camera = 1;
    V3 v;
    if (read_vec3_field(o, "origin", &v) || read_vec3_field(o, "position", &v)) {
      c.origin[0] = v.x; c.origin[1] = v.y; c.origin[2] = v.z;
    }
    if (read_vec3_field(o, "target", &v)) {
      c.target[0] = v.x; c.target[1] = v.y; c.target[2] = v.z;
    }
    float f;
    if (read_number(o, {"fov_y", "fov"}, &f)) c.fov_y_degrees = f;
  }

  // read_light_spectrum (R:6786-6800)
  bool light_spectrum(const ObjectData& o, std::initializer_list<const char*> legacy, V3* out) {
    V3 c;
    if (read_spectrum(o, "color", &c)) {
      float s = std::max(number_or(o, {"intensity"}, 1.0f), 0.0f);
      *out = mul(c, s);
      return true;
    }
    for (const char* f : legacy)
      if (read_spectrum(o, f, out)) return true;
    return false;
  }

  // parse_lights (R:6288-6388); bindings visited in name order.
  void parse_lights() {
    for (const auto& kv : st_.bindings) {
      const Value& v = kv.second.value;
      if (v.kind != Value::Object || !v.obj->has_type) continue;
      const ObjectData& o = *v.obj;
      ft_light l;
      std::memset(&l, 0, sizeof(l));
      V3 p, s;
      if (o.type_name == "PointLight" || o.type_name == "SphereLight") {
        if (!read_vec3_field(o, "position", &p)) p = read_center(o);
        if (!light_spectrum(o, {"intensity"}, &s)) s = v3(8, 8, 8);
        l.kind = o.type_name == "PointLight" ? FT_LIGHT_POINT : FT_LIGHT_SPHERE;
        l.position[0] = p.x; l.position[1] = p.y; l.position[2] = p.z;
        l.intensity[0] = s.x; l.intensity[1] = s.y; l.intensity[2] = s.z;
        if (l.kind == FT_LIGHT_SPHERE) {
          l.radius = std::max(number_or(o, {"radius", "r"}, 0.35f), 0.0f);
          float smp;
          l.samples = read_number(o, {"samples"}, &smp) ? static_cast<uint32_t>(std::max(smp, 1.0f)) : 8u;
        } else {
          l.samples = 1;
        }
        out_.lights.push_back(l);
      } else if (o.type_name == "EnvLight") {
        if (!light_spectrum(o, {"radiance", "color"}, &s)) s = v3(0.15f, 0.15f, 0.15f);
        l.kind = FT_LIGHT_ENV;
        l.samples = 1;
        l.intensity[0] = s.x; l.intensity[1] = s.y; l.intensity[2] = s.z;
        out_.lights.push_back(l);
      }
    }
    if (out_.lights.empty()) {
      ft_light p;
      std::memset(&p, 0, sizeof(p));
      p.kind = FT_LIGHT_POINT;
      p.samples = 1;
      p.position[0] = 3; p.position[1] = 3; p.position[2] = 6;
      p.intensity[0] = p.intensity[1] = p.intensity[2] = 6;
      out_.lights.push_back(p);
      ft_light e;
      std::memset(&e, 0, sizeof(e));
      e.kind = FT_LIGHT_ENV;
      e.samples = 1;
      e.intensity[0] = e.intensity[1] = e.intensity[2] = 0.1f;
      out_.lights.push_back(e);
    }
  }

  static bool float_to_u32(float v, uint32_t* out) {
    if (std::isfinite(v) && v >= 1.0f) {
      float r = std::round(v);
      if (std::fabs(r - v) < 1.0e-5f) {
        *out = static_cast<uint32_t>(r);
        return true;
      }
    }
    return false;
  }

  // extract_scene_render_settings (R:1316-1354)
  void parse_settings() {
    out_.desc.settings_mask = 0;
    out_.desc.settings_accel = -1;
    const ObjectData* o = nullptr;
    for (const char* k : {"render", "render_settings", "settings"}) {
      auto it = st_.bindings.find(k);
      if (it != st_.bindings.end() && it->second.value.kind == Value::Object) {
        o = it->second.value.obj.get();
        break;
      }
    }
    if (!o) return;
    ft_render_options& s = out_.desc.settings;
    float v;
    uint32_t u;
    if (read_number(*o, {"width"}, &v) && float_to_u32(v, &u)) { s.width = u; out_.desc.settings_mask |= 1u; }
    if (read_number(*o, {"height"}, &v) && float_to_u32(v, &u)) { s.height = u; out_.desc.settings_mask |= 2u; }
    if (read_number(*o, {"max_steps"}, &v) && float_to_u32(v, &u)) { s.max_steps = u; out_.desc.settings_mask |= 4u; }
    if (read_number(*o, {"max_dist"}, &v)) { s.max_dist = v; out_.desc.settings_mask |= 8u; }
    if (read_number(*o, {"epsilon"}, &v)) { s.epsilon = v; out_.desc.settings_mask |= 16u; }
    if (read_number(*o, {"step_scale"}, &v)) { s.step_scale = v; out_.desc.settings_mask |= 32u; }
    if (read_number(*o, {"camera_z"}, &v)) { s.camera_z = v; out_.desc.settings_mask |= 64u; }
    if (read_number(*o, {"fov_y", "fov"}, &v)) { s.fov_y_degrees = v; out_.desc.settings_mask |= 128u; }
    const Value* acc = o->get("accel");
    if (acc) {
      if (acc->kind == Value::Object) {
        const std::string& n = acc->obj->type_name;
        if (n == "Naive" || n == "naive") out_.desc.settings_accel = FT_ACCEL_NAIVE;
        else if (n == "Bvh" || n == "bvh") out_.desc.settings_accel = FT_ACCEL_BVH;
        else if (n == "Bricks" || n == "bricks") out_.desc.settings_accel = FT_ACCEL_BRICKS;
      } else if (acc->kind == Value::Number) {
        int k = static_cast<int>(acc->num);
        if (k >= 0 && k <= 2) out_.desc.settings_accel = k;
      }
    }
  }

  // find_environment_name (R:6908-6924) + its `fn color(dir)`.
  void parse_environment() {
    out_.desc.environment_program = -1;
    const BlockDef* def = nullptr;
    for (const char* k : {"environment", "env", "sky"}) {
      auto it = st_.bindings.find(k);
      if (it != st_.bindings.end() && it->second.value.kind == Value::Object) {
        auto d = st_.environment_defs.find(it->second.value.obj->type_name);
        if (d != st_.environment_defs.end()) {
          def = d->second.get();
          break;
        }
      }
    }
    if (!def && st_.environment_defs.size() == 1) def = st_.environment_defs.begin()->second.get();
    if (!def) return;
    for (const BlockStmt& s : def->statements) {
      if (s.kind == BlockStmt::Function && s.name == "color" && s.params.size() == 1) {
        HookCompiler hc(st_, out_.instrs);
        ft_program p = hc.compile(s.params, {true}, s.body, {}, def, true, "environment color");
        out_.programs.push_back(p);
        out_.desc.environment_program = static_cast<int32_t>(out_.programs.size()) - 1;
        return;
      }
    }
  }
};

}  // namespace

std::unique_ptr<OwnedSceneDesc> lower_scene(const EvalState& state) {
  auto out = std::make_unique<OwnedSceneDesc>();
  Lowerer l(state, *out);
  l.run();
  out->finalize();
  return out;
}

}  // namespace ftfe
