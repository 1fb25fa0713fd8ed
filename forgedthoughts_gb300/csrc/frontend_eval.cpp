// `.ft` evaluator: statements, expressions, builtins and closures.
//
// Follows crates/forgedthoughts/src/eval.rs: eval_program (E:138-162),
// eval_statement (E:191-332), assign_path (E:334-383), expression evaluation
// (E:419-535), eval_binary (E:1228-1293), SDF member operators
// (E:1295-1536, E:1713-1745), eval_unary (E:1747-1757), eval_call
// (E:1759-1869), eval_function_value (E:2011-2146, tree-walking form),
// builtins (E:2223-2690), top-level functions (E:4187-4228) and
// rotate_vec3 (E:4733-4741).  Numbers are f32 (`Value::Number(f32)`), number
// literals are parsed as f64 and rounded to f32 (E:431).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>

#include "frontend.h"

namespace ftfe {

namespace {
[[noreturn]] void eval_fail(const std::string& msg) { throw FrontendError(FT_ERR_EVAL, msg); }
std::atomic<uint64_t> g_function_identity{1};
}  // namespace

Value make_object(const std::string& type_name, std::map<std::string, Value> fields) {
  Value v;
  v.kind = Value::Object;
  v.obj = std::make_shared<ObjectData>();
  v.obj->has_type = true;
  v.obj->type_name = type_name;
  v.obj->fields = std::move(fields);
  return v;
}

Value make_vec3(float x, float y, float z) {
  std::map<std::string, Value> f;
  f["x"] = Value::number(x);
  f["y"] = Value::number(y);
  f["z"] = Value::number(z);
  return make_object("vec3", std::move(f));
}

// `as_vec3` (E:5041-5058): any object with numeric x, y, z.
bool as_vec3(const Value& v, float out[3]) {
  if (v.kind != Value::Object) return false;
  const char* names[3] = {"x", "y", "z"};
  for (int i = 0; i < 3; ++i) {
    const Value* c = v.obj->get(names[i]);
    if (!c || c->kind != Value::Number) return false;
    out[i] = c->num;
  }
  return true;
}

// `as_broadcastable_vec3` (E:4346-4351).
bool as_broadcast_vec3(const Value& v, float out[3]) {
  if (v.kind == Value::Number) {
    out[0] = out[1] = out[2] = v.num;
    return true;
  }
  return as_vec3(v, out);
}

bool values_equal(const Value& a, const Value& b) {
  if (a.kind != b.kind) return false;
  switch (a.kind) {
    case Value::Number: return a.num == b.num;
    case Value::String: return a.str == b.str;
    case Value::Array: {
      if (a.arr == b.arr) return true;
      if (a.arr->size() != b.arr->size()) return false;
      for (size_t i = 0; i < a.arr->size(); ++i)
        if (!values_equal((*a.arr)[i], (*b.arr)[i])) return false;
      return true;
    }
    case Value::Object: {
      if (a.obj == b.obj) return true;
      if (a.obj->has_type != b.obj->has_type || a.obj->type_name != b.obj->type_name) return false;
      if (a.obj->fields.size() != b.obj->fields.size()) return false;
      auto ia = a.obj->fields.begin();
      auto ib = b.obj->fields.begin();
      for (; ia != a.obj->fields.end(); ++ia, ++ib) {
        if (ia->first != ib->first || !values_equal(ia->second, ib->second)) return false;
      }
      return true;
    }
    case Value::Function: {
      if (a.fn == b.fn) return true;
      if (a.fn->params != b.fn->params || a.fn->body.size() != b.fn->body.size()) return false;
      for (size_t i = 0; i < a.fn->body.size(); ++i)
        if (a.fn->body[i].expr != b.fn->body[i].expr) return false;
      if (a.fn->captures.size() != b.fn->captures.size()) return false;
      auto ia = a.fn->captures.begin();
      auto ib = b.fn->captures.begin();
      for (; ia != a.fn->captures.end(); ++ia, ++ib)
        if (ia->first != ib->first || !values_equal(ia->second, ib->second)) return false;
      return true;
    }
  }
  return false;
}

namespace {

float rust_clamp(float x, float lo, float hi) {
  // f32::clamp: max then min (NaN passes through).
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}
float rust_min(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a < b ? a : b;
}
float rust_max(float a, float b) {
  if (std::isnan(a)) return b;
  if (std::isnan(b)) return a;
  return a > b ? a : b;
}
float deg_to_rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

// rotate_vec3 (E:4733-4741).
void rotate_vec3(const float v[3], float deg, char axis, float out[3]) {
  float r = deg_to_rad(deg);
  float s = std::sin(r), c = std::cos(r);
  if (axis == 'x') {
    out[0] = v[0]; out[1] = c * v[1] - s * v[2]; out[2] = s * v[1] + c * v[2];
  } else if (axis == 'y') {
    out[0] = c * v[0] + s * v[2]; out[1] = v[1]; out[2] = -s * v[0] + c * v[2];
  } else {
    out[0] = c * v[0] - s * v[1]; out[1] = s * v[0] + c * v[1]; out[2] = v[2];
  }
}

template <class F>
Value map1(const char* name, const Value& a, F f) {
  if (a.kind == Value::Number) return Value::number(f(a.num));
  float v[3];
  if (!as_vec3(a, v)) eval_fail(std::string("builtin ") + name + " expects number or vec3 args");
  return make_vec3(f(v[0]), f(v[1]), f(v[2]));
}
template <class F>
Value map2(const char* name, const Value& a, const Value& b, F f) {
  if (a.kind == Value::Number && b.kind == Value::Number) return Value::number(f(a.num, b.num));
  float va[3], vb[3];
  if (!as_broadcast_vec3(a, va) || !as_broadcast_vec3(b, vb))
    eval_fail(std::string("builtin ") + name + " expects number or vec3 args");
  return make_vec3(f(va[0], vb[0]), f(va[1], vb[1]), f(va[2], vb[2]));
}
template <class F>
Value map3(const char* name, const Value& a, const Value& b, const Value& c, F f) {
  if (a.kind == Value::Number && b.kind == Value::Number && c.kind == Value::Number)
    return Value::number(f(a.num, b.num, c.num));
  float va[3], vb[3], vc[3];
  if (!as_broadcast_vec3(a, va) || !as_broadcast_vec3(b, vb) || !as_broadcast_vec3(c, vc))
    eval_fail(std::string("builtin ") + name + " expects number or vec3 args");
  return make_vec3(f(va[0], vb[0], vc[0]), f(va[1], vb[1], vc[1]), f(va[2], vb[2], vc[2]));
}

void arity(const char* name, const std::vector<Value>& args, size_t n) {
  if (args.size() != n)
    eval_fail(std::string("builtin ") + name + " expects exactly " + std::to_string(n) +
              " numeric args, got " + std::to_string(args.size()));
}

}  // namespace

// flatten_member_expr (E:537-545).
bool flatten_member(const Expr& e, std::string* out) {
  if (e.kind == Expr::Ident) { *out = e.text; return true; }
  if (e.kind == Expr::Member) {
    std::string t;
    if (!flatten_member(*e.lhs, &t)) return false;
    *out = t + "." + e.text;
    return true;
  }
  return false;
}

// eval_ident_call (E:2223-2690), render-relevant builtins.
Value eval_builtin(const std::string& name, const std::vector<Value>& args, bool* found) {
  *found = true;
  if (name == "vec3") {
    if (args.size() != 1 && args.size() != 3) eval_fail("builtin vec3 expects exactly 1 or 3 numeric args");
    for (const Value& a : args)
      if (a.kind != Value::Number) eval_fail("builtin vec3 expects exactly 1 or 3 numeric args");
    if (args.size() == 1) return make_vec3(args[0].num, args[0].num, args[0].num);
    return make_vec3(args[0].num, args[1].num, args[2].num);
  }
  if (name == "clamp") {
    arity("clamp", args, 3);
    return map3("clamp", args[0], args[1], args[2], [](float x, float a, float b) {
      float lo = a <= b ? a : b, hi = a <= b ? b : a;
      return rust_clamp(x, lo, hi);
    });
  }
  if (name == "mix") {
    arity("mix", args, 3);
    return map3("mix", args[0], args[1], args[2], [](float x, float y, float a) { return x * (1.0f - a) + y * a; });
  }
  if (name == "step") {
    arity("step", args, 2);
    if (args[0].kind != Value::Number || args[1].kind != Value::Number) eval_fail("builtin step expects numeric args");
    return Value::number(args[1].num < args[0].num ? 0.0f : 1.0f);
  }
  if (name == "smoothstep") {
    arity("smoothstep", args, 3);
    for (const Value& a : args)
      if (a.kind != Value::Number) eval_fail("builtin smoothstep expects numeric args");
    float e0 = args[0].num, e1 = args[1].num, x = args[2].num;
    float span = e1 - e0;
    float t = std::fabs(span) < std::numeric_limits<float>::epsilon() ? (x < e0 ? 0.0f : 1.0f)
                                                                     : rust_clamp((x - e0) / span, 0.0f, 1.0f);
    return Value::number(t * t * (3.0f - 2.0f * t));
  }
  if (name == "saturate") { arity("saturate", args, 1); return map1("saturate", args[0], [](float x) { return rust_clamp(x, 0.0f, 1.0f); }); }
  if (name == "abs") { arity("abs", args, 1); return map1("abs", args[0], [](float x) { return std::fabs(x); }); }
  if (name == "floor") { arity("floor", args, 1); return map1("floor", args[0], [](float x) { return std::floor(x); }); }
  if (name == "ceil") { arity("ceil", args, 1); return map1("ceil", args[0], [](float x) { return std::ceil(x); }); }
  if (name == "fract") { arity("fract", args, 1); return map1("fract", args[0], [](float x) { return x - std::floor(x); }); }
  if (name == "sqrt") { arity("sqrt", args, 1); return map1("sqrt", args[0], [](float x) { return std::sqrt(x); }); }
  if (name == "sin") { arity("sin", args, 1); return map1("sin", args[0], [](float x) { return std::sin(x); }); }
  if (name == "cos") { arity("cos", args, 1); return map1("cos", args[0], [](float x) { return std::cos(x); }); }
  if (name == "min") { arity("min", args, 2); return map2("min", args[0], args[1], rust_min); }
  if (name == "max") { arity("max", args, 2); return map2("max", args[0], args[1], rust_max); }
  if (name == "pow") { arity("pow", args, 2); return map2("pow", args[0], args[1], [](float a, float b) { return std::pow(a, b); }); }
  if (name == "dot") {
    arity("dot", args, 2);
    float a[3], b[3];
    if (!as_vec3(args[0], a) || !as_vec3(args[1], b)) eval_fail("builtin dot expects vec3 args");
    return Value::number(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
  }
  if (name == "length") {
    arity("length", args, 1);
    float v[3];
    if (!as_vec3(args[0], v)) eval_fail("builtin length expects vec3 args");
    return Value::number(std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
  }
  if (name == "normalize") {
    arity("normalize", args, 1);
    float v[3];
    if (!as_vec3(args[0], v)) eval_fail("builtin normalize expects vec3 args");
    float len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (len <= std::numeric_limits<float>::epsilon()) return make_vec3(0, 0, 0);
    return make_vec3(v[0] / len, v[1] / len, v[2] / len);
  }
  if (name == "rotate_x" || name == "rotate_y" || name == "rotate_z") {
    arity(name.c_str(), args, 2);
    float v[3], o[3];
    if (!as_vec3(args[0], v)) eval_fail("builtin " + name + " expects vec3 args");
    if (args[1].kind != Value::Number) eval_fail("builtin " + name + " expects numeric args");
    rotate_vec3(v, args[1].num, name.back(), o);
    return make_vec3(o[0], o[1], o[2]);
  }
  *found = false;
  return Value();
}

namespace {

struct Scope {
  const std::map<std::string, Value>* locals;
  const BlockDef* material_def;     // material runtime (E:125-130)
  const BlockDef* environment_def;  // environment scope (E:3811-3874)
  int depth;
};

Value eval_expr(const Expr& e, const EvalState& st, const Scope& sc);
Value call_user_body(const EvalState& st, const std::vector<std::string>& params, const std::vector<FnStmt>& body,
                     const std::vector<Value>& args, std::map<std::string, Value> locals, const Scope& sc);

Value eval_binary(const Value& l, char op, const Value& r) {
  if (l.kind == Value::Number && r.kind == Value::Number) {
    switch (op) {
      case '+': return Value::number(l.num + r.num);
      case '-': return Value::number(l.num - r.num);
      case '*': return Value::number(l.num * r.num);
      case '/': return Value::number(l.num / r.num);
      default: eval_fail("binary operation requires numeric operands");
    }
  }
  if (op != '&') {
    float a[3], b[3];
    if (as_broadcast_vec3(l, a) && as_broadcast_vec3(r, b)) {
      switch (op) {
        case '+': return make_vec3(a[0] + b[0], a[1] + b[1], a[2] + b[2]);
        case '-': return make_vec3(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
        case '*': return make_vec3(a[0] * b[0], a[1] * b[1], a[2] * b[2]);
        case '/': return make_vec3(a[0] / b[0], a[1] / b[1], a[2] / b[2]);
      }
    }
  }
  if (Value anchored; anchor_arithmetic(l, op, r, &anchored)) return anchored;
  if (op == '+' || op == '-' || op == '&') {
    std::map<std::string, Value> f;
    f["lhs"] = l;
    f["rhs"] = r;
    return make_object(op == '+' ? "add" : op == '-' ? "sub" : "intersect", std::move(f));
  }
  eval_fail("binary operation requires numeric operands");
}

Value eval_unary(const Value& v) {
  if (v.kind == Value::Number) return Value::number(-v.num);
  float a[3];
  if (!as_vec3(v, a)) eval_fail("unary operation requires numeric or vec3 operand");
  return make_vec3(-a[0], -a[1], -a[2]);
}

bool is_sdf_member_operator(const std::string& f) {
  static const char* ops[] = {"smooth", "union_round", "union_chamfer", "union_columns", "union_stairs",
                              "union_soft", "intersect_round", "intersect_chamfer", "intersect_columns",
                              "intersect_stairs", "diff_round", "diff_chamfer", "diff_columns", "diff_stairs",
                              "pipe", "engrave", "groove", "tongue", "mirror_x", "mirror_y", "mirror_z",
                              "repeat_x", "repeat_y", "repeat_z", "slice_x", "slice_y", "slice_z", "noise"};
  for (const char* o : ops)
    if (f == o) return true;
  return false;
}

// build_sdf_member_value (E:1295-1536).
Value build_sdf_member(const std::string& field, const Value& base, const std::vector<Value>& args) {
  auto num = [&](size_t i) -> float {
    if (args[i].kind != Value::Number) eval_fail("call on unsupported callee");
    return args[i].num;
  };
  auto need = [&](size_t n) {
    if (args.size() != n) eval_fail("call on unsupported callee");
  };
  std::map<std::string, Value> f;
  if (field == "smooth") {
    need(1);
    f["base"] = base;
    f["k"] = Value::number(num(0));
  } else if (field == "union_round" || field == "union_chamfer" || field == "union_soft" ||
             field == "intersect_round" || field == "intersect_chamfer" || field == "diff_round" ||
             field == "diff_chamfer" || field == "pipe" || field == "engrave") {
    need(2);
    f["lhs"] = base;
    f["rhs"] = args[0];
    f["r"] = Value::number(num(1));
  } else if (field == "union_columns" || field == "union_stairs" || field == "intersect_columns" ||
             field == "intersect_stairs" || field == "diff_columns" || field == "diff_stairs") {
    need(3);
    f["lhs"] = base;
    f["rhs"] = args[0];
    f["r"] = Value::number(num(1));
    f["n"] = Value::number(num(2));
  } else if (field == "groove" || field == "tongue") {
    need(3);
    f["lhs"] = base;
    f["rhs"] = args[0];
    f["ra"] = Value::number(num(1));
    f["rb"] = Value::number(num(2));
  } else if (field == "mirror_x" || field == "mirror_y" || field == "mirror_z") {
    need(0);
    f["base"] = base;
  } else if (field == "repeat_x" || field == "repeat_y" || field == "repeat_z") {
    need(2);
    f["base"] = base;
    f["spacing"] = Value::number(num(0));
    f["count"] = Value::number(num(1));
  } else if (field == "slice_x" || field == "slice_y" || field == "slice_z") {
    need(2);
    f["base"] = base;
    f["min"] = Value::number(num(0));
    f["max"] = Value::number(num(1));
  } else if (field == "noise") {
    if (args.empty() || args.size() > 3) eval_fail("call on unsupported callee");
    f["base"] = base;
    f["octaves"] = Value::number(num(0));
    f["scale"] = Value::number(args.size() > 1 ? num(1) : 1.0f);
    f["lacunarity"] = Value::number(args.size() > 2 ? num(2) : 1.0f);
  } else {
    eval_fail("call on unsupported callee");
  }
  return make_object(field, std::move(f));
}

std::vector<Value> eval_args(const std::vector<ExprP>& args, const EvalState& st, const Scope& sc) {
  std::vector<Value> out;
  out.reserve(args.size());
  for (const ExprP& a : args) out.push_back(eval_expr(*a, st, sc));
  return out;
}

Value eval_function_value_impl(const EvalState& st, const FunctionData& fn, const std::vector<Value>& args) {
  if (args.size() != fn.params.size()) eval_fail("call on unsupported callee");
  Scope sc{nullptr, nullptr, nullptr, 0};
  return call_user_body(st, fn.params, fn.body, args, fn.captures, sc);
}

const BlockStmt* find_block_fn(const BlockDef* def, const std::string& name) {
  if (!def) return nullptr;
  for (const BlockStmt& s : def->statements)
    if (s.kind == BlockStmt::Function && s.name == name) return &s;
  return nullptr;
}

Value call_top_level(const EvalState& st, const FunctionDef& def, const std::vector<Value>& args, int depth) {
  if (args.size() != def.params.size()) eval_fail("call on unsupported callee");
  if (depth >= 32) eval_fail("material call depth exceeded");
  Scope sc{nullptr, nullptr, nullptr, depth};
  return call_user_body(st, def.params, def.body, args, {}, sc);
}

Value eval_call(const Expr& e, const EvalState& st, const Scope& sc) {
  const Expr& callee = *e.lhs;
  if (callee.kind != Expr::Ident && callee.kind != Expr::Member) {
    Value cv = eval_expr(callee, st, sc);
    std::vector<Value> args = eval_args(e.items, st, sc);
    if (cv.kind == Value::Function) return eval_function_value_impl(st, *cv.fn, args);
    eval_fail("call on unsupported callee");
  }
  if (callee.kind == Expr::Ident) {
    std::vector<Value> args = eval_args(e.items, st, sc);
    bool found = false;
    Value v = eval_builtin(callee.text, args, &found);
    if (found) return v;
    // A local function value (closure bound by `let f = fn ...`).
    if (sc.locals) {
      auto it = sc.locals->find(callee.text);
      if (it != sc.locals->end() && it->second.kind == Value::Function)
        return eval_function_value_impl(st, *it->second.fn, args);
    }
    const BlockDef* blk = sc.material_def ? sc.material_def : sc.environment_def;
    if (const BlockStmt* f = find_block_fn(blk, callee.text)) {
      if (sc.depth >= 32) eval_fail("material call depth exceeded");
      if (args.size() != f->params.size()) eval_fail("call on unsupported callee");
      Scope inner{nullptr, sc.material_def, sc.environment_def, sc.depth + 1};
      std::map<std::string, Value> locals;
      // Block-level `let` bindings are visible inside block functions.
      for (const BlockStmt& s : blk->statements) {
        if (s.kind != BlockStmt::Binding) continue;
        Scope bs{&locals, sc.material_def, sc.environment_def, sc.depth + 1};
        locals[s.name] = eval_expr(*s.expr, st, bs);
      }
      return call_user_body(st, f->params, f->body, args, std::move(locals), inner);
    }
    auto fit = st.function_defs.find(callee.text);
    if (fit != st.function_defs.end()) return call_top_level(st, *fit->second, args, sc.depth + 1);
    auto bit = st.bindings.find(callee.text);
    if (bit != st.bindings.end() && bit->second.value.kind == Value::Function)
      return eval_function_value_impl(st, *bit->second.value.fn, args);
    eval_fail("call on unsupported callee");
  }
  // Member callee.
  const std::string& field = callee.text;
  if (is_sdf_member_operator(field)) {
    Value base = eval_expr(*callee.lhs, st, sc);
    std::vector<Value> args = eval_args(e.items, st, sc);
    return build_sdf_member(field, base, args);
  }
  if (is_layout_member_operator(field)) {
    Value base = eval_expr(*callee.lhs, st, sc);
    std::vector<Value> args = eval_args(e.items, st, sc);
    return build_layout_member(field, std::move(base), args);
  }
  std::string flat;
  if (flatten_member(callee, &flat)) {
    std::vector<Value> args = eval_args(e.items, st, sc);
    auto fit = st.function_defs.find(flat);
    if (fit != st.function_defs.end()) return call_top_level(st, *fit->second, args, sc.depth + 1);
  }
  eval_fail("call on unsupported callee");
}

// augment_object_literal_fields (E:547-575) for an instance of an `sdf`
// definition: its layout bounds `__bounds` (the definition's `bounds()`) and
// its `anchors` binding, each evaluated with the instance's fields replacing
// the definition's bindings, and each left out when its evaluation fails.
void augment_sdf_instance(const EvalState& st, const BlockDef& def, std::map<std::string, Value>& fields,
                          int depth) {
  if (depth >= 32) return;
  std::map<std::string, Value> locals = fields;  // sdf_override_locals (E:3338-3342)
  bool have_anchors = false, locals_ok = false;
  Value anchors;
  try {
    Scope bs{&locals, &def, nullptr, depth + 1};
    for (const BlockStmt& s : def.statements) {
      if (s.kind != BlockStmt::Binding) continue;
      auto it = fields.find(s.name);
      locals[s.name] = it != fields.end() ? it->second : eval_expr(*s.expr, st, bs);
      if (s.name == "anchors" && !have_anchors) {
        anchors = locals[s.name];
        have_anchors = true;
      }
    }
    locals_ok = true;
  } catch (const FrontendError&) {
  }
  if (!fields.count("__bounds") && locals_ok) {
    const BlockStmt* fn = find_block_fn(&def, "bounds");
    if (fn && fn->params.empty()) {
      try {
        Scope inner{nullptr, &def, nullptr, depth + 1};
        fields["__bounds"] = call_user_body(st, {}, fn->body, {}, locals, inner);
      } catch (const FrontendError&) {
      }
    }
  }
  if (!fields.count("anchors") && have_anchors) fields["anchors"] = anchors;
}

Value eval_expr(const Expr& e, const EvalState& st, const Scope& sc) {
  switch (e.kind) {
    case Expr::Number: return Value::number(static_cast<float>(e.number));
    case Expr::String: {
      Value v;
      v.kind = Value::String;
      v.str = e.text;
      return v;
    }
    case Expr::Array: {
      Value v;
      v.kind = Value::Array;
      v.arr = std::make_shared<std::vector<Value>>(eval_args(e.items, st, sc));
      return v;
    }
    case Expr::FunctionLiteral: {
      Value v;
      v.kind = Value::Function;
      v.fn = std::make_shared<FunctionData>();
      v.fn->params = e.params;
      v.fn->body = e.body;
      if (sc.locals) v.fn->captures = *sc.locals;
      v.fn->identity = g_function_identity.fetch_add(1);
      return v;
    }
    case Expr::Ident: {
      if (sc.locals) {
        auto it = sc.locals->find(e.text);
        if (it != sc.locals->end()) return it->second;
      }
      // Anchor symbols come before bindings (E:454-466).
      if (is_anchor_symbol(e.text)) return anchor_symbol(e.text, 0.0f);
      auto it = st.bindings.find(e.text);
      if (it == st.bindings.end()) eval_fail("undefined identifier '" + e.text + "'");
      return it->second.value;
    }
    case Expr::ObjectLiteral: {
      std::map<std::string, Value> f;
      for (const auto& kv : e.fields) f[kv.first] = eval_expr(*kv.second, st, sc);
      auto def = st.sdf_defs.find(e.text);
      if (def != st.sdf_defs.end()) augment_sdf_instance(st, *def->second, f, sc.depth);
      return make_object(e.text, std::move(f));
    }
    case Expr::Binary: {
      Value l = eval_expr(*e.lhs, st, sc);
      Value r = eval_expr(*e.rhs, st, sc);
      return eval_binary(l, e.op, r);
    }
    case Expr::Member: {
      std::string flat;
      if (flatten_member(e, &flat)) {
        auto it = st.bindings.find(flat);
        if (it != st.bindings.end()) return it->second.value;
      }
      Value base = eval_expr(*e.lhs, st, sc);
      if (base.kind != Value::Object) eval_fail("member access requires object value");
      const Value* v = base.obj->get(e.text);
      if (!v) eval_fail("undefined identifier '" + e.text + "'");
      return *v;
    }
    case Expr::Call: return eval_call(e, st, sc);
    case Expr::Unary: return eval_unary(eval_expr(*e.lhs, st, sc));
  }
  eval_fail("unsupported expression");
}

Value call_user_body(const EvalState& st, const std::vector<std::string>& params, const std::vector<FnStmt>& body,
                     const std::vector<Value>& args, std::map<std::string, Value> locals, const Scope& sc) {
  for (size_t i = 0; i < params.size(); ++i) locals[params[i]] = args[i];
  Scope inner{&locals, sc.material_def, sc.environment_def, sc.depth};
  for (const FnStmt& s : body) {
    if (s.is_return) return eval_expr(*s.expr, st, inner);
    Value v = eval_expr(*s.expr, st, inner);
    locals[s.name] = v;
  }
  eval_fail("function missing return");
}

// Copy-on-write descent for `a.b.c = v` (E:358-383).
void assign_in_object(Value& target, const std::vector<std::string>& path, size_t at, const Value& v) {
  if (target.kind != Value::Object) eval_fail("member access requires object value");
  if (target.obj.use_count() > 1) target.obj = std::make_shared<ObjectData>(*target.obj);
  if (at + 1 == path.size()) {
    target.obj->fields[path[at]] = v;
    return;
  }
  auto it = target.obj->fields.find(path[at]);
  if (it == target.obj->fields.end()) {
    Value empty;
    empty.kind = Value::Object;
    empty.obj = std::make_shared<ObjectData>();
    it = target.obj->fields.emplace(path[at], empty).first;
  }
  assign_in_object(it->second, path, at + 1, v);
}

void assign_path(EvalState& st, const std::vector<std::string>& path, const Value& v) {
  // resolve_binding_path (E:1215-1226): longest dotted prefix naming a binding.
  std::string name = path[0];
  size_t consumed = 1;
  for (size_t len = path.size(); len >= 1; --len) {
    std::string cand;
    for (size_t k = 0; k < len; ++k) cand += (k ? "." : "") + path[k];
    if (st.bindings.count(cand)) {
      name = cand;
      consumed = len;
      break;
    }
  }
  auto it = st.bindings.find(name);
  if (it == st.bindings.end()) eval_fail("undefined identifier '" + name + "'");
  if (!it->second.mutable_) eval_fail("cannot assign to immutable binding '" + name + "'");
  if (consumed == path.size()) {
    it->second.value = v;
    return;
  }
  std::vector<std::string> rest(path.begin() + consumed, path.end());
  assign_in_object(it->second.value, rest, 0, v);
}

}  // namespace

EvalState eval_program(const std::vector<Stmt>& program) {
  EvalState st;
  Scope top{nullptr, nullptr, nullptr, 0};
  for (const Stmt& s : program) {
    switch (s.kind) {
      case Stmt::Import:
        // A source string has no directory to resolve an import from; the
        // file loader splices imports before evaluation.
        throw FrontendError(FT_ERR_UNSUPPORTED, "import \"" + s.name +
                                                    "\" needs a scene file: load it with ft_scene_desc_from_file");
      case Stmt::Export:
      case Stmt::Skeleton:
        break;
      case Stmt::Binding: {
        Value v = eval_expr(*s.expr, st, top);
        st.bindings[s.name] = Binding{s.mutable_, v};
        break;
      }
      case Stmt::Assign: {
        Value v = eval_expr(*s.expr, st, top);
        assign_path(st, s.path, v);
        break;
      }
      case Stmt::Function: st.function_defs[s.fn->name] = s.fn; break;
      case Stmt::Material: st.material_defs[s.block->name] = s.block; break;
      case Stmt::Sdf: st.sdf_defs[s.block->name] = s.block; break;
      case Stmt::Environment: st.environment_defs[s.block->name] = s.block; break;
    }
  }
  return st;
}

}  // namespace ftfe
