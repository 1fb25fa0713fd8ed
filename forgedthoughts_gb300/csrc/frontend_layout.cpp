// Layout member operators of the `.ft` language: `a.attach(floor, Top)`,
// `.align_x/y/z(other, anchor)`, `.right_of / left_of / on_top_of / below /
// in_front_of / behind(other, gap)`, `.rotate_x/y/z(deg)`, `.offset_x/y/z(d)`
// and `.face_to(other[, anchor])`, with the anchor symbols (`Top`,
// `Center + 0.3`, ...) they take.  They move or turn an object value before
// it is lowered, from the layout bounds of the objects involved.
//
// Follows crates/forgedthoughts/src/eval.rs (E:):
//   build_layout_member_value / is_layout_member_operator  E:1538-1660
//   builtin_symbol_value / anchor_spec / anchor_value       E:4404-4451
//   builtin_anchor_modes / object_anchor_point              E:4467-4586
//   object_position / object_rotation / rotate/offset/face  E:4610-4713
//   rotate_xyz / transformed_bounds / object_bounds          E:4715-4932
//   attach_object / align_object_axis / place_object_rel.    E:4934-5039
//   anchor arithmetic in eval_binary                         E:1258-1273
// Skeleton binding (`.bind(bone)`) needs skeleton assets, which this
// front-end does not evaluate: it fails with FT_ERR_UNSUPPORTED.
#include <algorithm>
#include <cmath>
#include <limits>

#include "frontend.h"

namespace ftfe {
namespace {

[[noreturn]] void layout_fail(const std::string& m) { throw FrontendError(FT_ERR_EVAL, m); }
[[noreturn]] void unsupported_call() { layout_fail("call on unsupported callee"); }
[[noreturn]] void unbounded() { layout_fail("layout operation requires bounded object values"); }

struct Bounds3 {
  float min[3], max[3];
  void center(float c[3]) const {
    for (int a = 0; a < 3; ++a) c[a] = (min[a] + max[a]) * 0.5f;
  }
  Bounds3 merged(const Bounds3& o) const {
    Bounds3 r;
    for (int a = 0; a < 3; ++a) {
      r.min[a] = std::min(min[a], o.min[a]);
      r.max[a] = std::max(max[a], o.max[a]);
    }
    return r;
  }
};

Bounds3 box_around(const float p[3], const float half[3]) {
  Bounds3 b;
  for (int a = 0; a < 3; ++a) {
    b.min[a] = p[a] - half[a];
    b.max[a] = p[a] + half[a];
  }
  return b;
}

const char* const kAnchorNames[] = {
    "Top", "Bottom", "Left", "Right", "Front", "Back", "Center", "FrontLeftCorner", "FrontRightCorner",
    "BackLeftCorner", "BackRightCorner", "BottomFrontLeft", "BottomFrontRight", "BottomBackLeft",
    "BottomBackRight", "TopFrontLeft", "TopFrontRight", "TopBackLeft", "TopBackRight", "Start", "End"};

struct AnchorSpec {
  std::string name;
  float offset = 0.0f;
};

bool anchor_spec(const Value& v, AnchorSpec* out) {
  if (v.kind == Value::String) {
    out->name = v.str;
    out->offset = 0.0f;
    return true;
  }
  if (v.kind != Value::Object || !v.obj->has_type || v.obj->type_name != "symbol") return false;
  const Value* name = v.obj->get("name");
  if (!name || name->kind != Value::Object || !name->obj->has_type) return false;
  out->name = name->obj->type_name;
  const Value* off = v.obj->get("offset");
  out->offset = off && off->kind == Value::Number ? off->num : 0.0f;
  return true;
}

enum Mode { kMin, kMax, kMid };

// builtin_anchor_modes (E:4467-4548): per axis, which face of the bounds.
bool anchor_modes(const std::string& n, Mode m[3]) {
  struct Row { const char* name; Mode x, y, z; };
  static const Row rows[] = {
      {"Center", kMid, kMid, kMid},           {"Top", kMid, kMax, kMid},
      {"Bottom", kMid, kMin, kMid},           {"Left", kMin, kMid, kMid},
      {"Right", kMax, kMid, kMid},            {"Front", kMid, kMid, kMax},
      {"Back", kMid, kMid, kMin},             {"FrontLeftCorner", kMin, kMin, kMax},
      {"BottomFrontLeft", kMin, kMin, kMax},  {"FrontRightCorner", kMax, kMin, kMax},
      {"BottomFrontRight", kMax, kMin, kMax}, {"BackLeftCorner", kMin, kMin, kMin},
      {"BottomBackLeft", kMin, kMin, kMin},   {"BackRightCorner", kMax, kMin, kMin},
      {"BottomBackRight", kMax, kMin, kMin},  {"TopFrontLeft", kMin, kMax, kMax},
      {"TopFrontRight", kMax, kMax, kMax},    {"TopBackLeft", kMin, kMax, kMin},
      {"TopBackRight", kMax, kMax, kMin}};
  for (const Row& r : rows) {
    if (n == r.name) {
      m[0] = r.x;
      m[1] = r.y;
      m[2] = r.z;
      return true;
    }
  }
  return false;
}

// object_position / object_rotation (E:4610-4652): a nested vec3 field, else
// the flat fields, else 0.
void object_vec(const Value& v, const char* nested, const char* const flat[3], float out[3]) {
  out[0] = out[1] = out[2] = 0.0f;
  if (v.kind != Value::Object) return;
  const Value* n = v.obj->get(nested);
  const char* comp[3] = {"x", "y", "z"};
  for (int a = 0; a < 3; ++a) {
    if (n && n->kind == Value::Object) {
      const Value* c = n->obj->get(comp[a]);
      if (c && c->kind == Value::Number) {
        out[a] = c->num;
        continue;
      }
    }
    const Value* f = v.obj->get(flat[a]);
    if (f && f->kind == Value::Number) out[a] = f->num;
  }
}

void object_position(const Value& v, float out[3]) {
  static const char* const flat[3] = {"x", "y", "z"};
  object_vec(v, "pos", flat, out);
}

void object_rotation(const Value& v, float out[3]) {
  static const char* const flat[3] = {"rot_x", "rot_y", "rot_z"};
  object_vec(v, "rot", flat, out);
}

ObjectData& writable(Value& v) {
  if (v.kind != Value::Object) layout_fail("member access requires object value");
  if (v.obj.use_count() > 1) v.obj = std::make_shared<ObjectData>(*v.obj);
  return *v.obj;
}

void set_position(Value& v, const float p[3]) { writable(v).fields["pos"] = make_vec3(p[0], p[1], p[2]); }

float deg_to_rad(float d) { return d * (static_cast<float>(M_PI) / 180.0f); }
float rad_to_deg(float r) { return r * (180.0f / static_cast<float>(M_PI)); }

// rotate_xyz (E:4715-4731): about x, then y, then z, in degrees.
void rotate_xyz(const float p[3], const float rot[3], float out[3]) {
  const float sx = std::sin(deg_to_rad(rot[0])), cx = std::cos(deg_to_rad(rot[0]));
  const float sy = std::sin(deg_to_rad(rot[1])), cy = std::cos(deg_to_rad(rot[1]));
  const float sz = std::sin(deg_to_rad(rot[2])), cz = std::cos(deg_to_rad(rot[2]));
  const float py = p[1] * cx - p[2] * sx;
  const float pz = p[1] * sx + p[2] * cx;
  const float px2 = p[0] * cy + pz * sy;
  const float pz2 = -p[0] * sy + pz * cy;
  out[0] = px2 * cz - py * sz;
  out[1] = px2 * sz + py * cz;
  out[2] = pz2;
}

// The eight corners of a centred box, rotated and moved (E:4743-4755).
Bounds3 turned_box(const float pos[3], const float rot[3], const float half[3]) {
  Bounds3 b;
  for (int a = 0; a < 3; ++a) {
    b.min[a] = std::numeric_limits<float>::infinity();
    b.max[a] = -std::numeric_limits<float>::infinity();
  }
  for (int i = 0; i < 8; ++i) {
    const float c[3] = {(i & 4) ? half[0] : -half[0], (i & 2) ? half[1] : -half[1], (i & 1) ? half[2] : -half[2]};
    float p[3];
    rotate_xyz(c, rot, p);
    for (int a = 0; a < 3; ++a) {
      b.min[a] = std::min(b.min[a], pos[a] + p[a]);
      b.max[a] = std::max(b.max[a], pos[a] + p[a]);
    }
  }
  return b;
}

bool number_field(const ObjectData& o, std::initializer_list<const char*> names, float* out) {
  for (const char* n : names) {
    const Value* v = o.get(n);
    if (v && v->kind == Value::Number) {
      *out = v->num;
      return true;
    }
  }
  return false;
}

bool is_one_of(const std::string& s, std::initializer_list<const char*> names) {
  for (const char* n : names)
    if (s == n) return true;
  return false;
}

// object_bounds (E:4784-4916): the layout bounds of an object value.
bool object_bounds(const Value& v, Bounds3* out) {
  if (v.kind != Value::Object || !v.obj) return false;
  const ObjectData& o = *v.obj;
  float pos[3];
  object_position(v, pos);
  if (const Value* b = o.get("__bounds")) {
    float half[3];
    if (b->kind == Value::Number) {
      const float r = std::fabs(b->num);
      half[0] = half[1] = half[2] = r;
    } else if (!as_vec3(*b, half)) {
      return false;
    }
    *out = box_around(pos, half);
    return true;
  }
  if (!o.has_type) return false;
  const std::string& t = o.type_name;
  auto sub = [&](const char* field, Bounds3* b) {
    const Value* f = o.get(field);
    return f && object_bounds(*f, b);
  };
  float r, h;
  if (t == "Sphere") {
    if (!number_field(o, {"radius", "r"}, &r)) return false;
    const float half[3] = {r, r, r};
    *out = box_around(pos, half);
    return true;
  }
  if (t == "Box" || t == "Room") {
    float half[3], rot[3];
    if (t == "Box") {
      const Value* s = o.get("size");
      if (!s || !as_broadcast_vec3(*s, half)) return false;
    } else {
      half[0] = 8.0f, half[1] = 4.0f, half[2] = 8.0f;
      number_field(o, {"width"}, &half[0]);
      number_field(o, {"height"}, &half[1]);
      number_field(o, {"depth"}, &half[2]);
    }
    for (float& x : half) x *= 0.5f;
    object_rotation(v, rot);
    *out = turned_box(pos, rot, half);
    return true;
  }
  if (t == "Cylinder" || t == "ExtrudePolygon") {
    if (!number_field(o, {"radius", "r"}, &r) || !number_field(o, {"height", "h"}, &h)) return false;
    const float half[3] = {r, h * 0.5f, r};
    *out = box_around(pos, half);
    return true;
  }
  if (t == "Torus") {
    float major, minor;
    if (!number_field(o, {"major_radius", "R"}, &major) || !number_field(o, {"minor_radius", "r"}, &minor))
      return false;
    const float half[3] = {major + minor, minor, major + minor};
    *out = box_around(pos, half);
    return true;
  }
  if (is_one_of(t, {"add", "intersect", "union_round", "union_chamfer", "union_columns", "union_stairs",
                    "union_soft", "intersect_round", "intersect_chamfer", "intersect_columns", "intersect_stairs",
                    "diff_round", "diff_chamfer", "diff_columns", "diff_stairs", "pipe", "engrave", "groove",
                    "tongue"})) {
    Bounds3 a, b;
    if (!sub("lhs", &a) || !sub("rhs", &b)) return false;
    *out = a.merged(b);
    return true;
  }
  if (t == "sub") return sub("lhs", out);
  if (t == "noise") return sub("base", out);
  const int axis = t.empty() ? 0 : t.back() == 'x' ? 0 : t.back() == 'y' ? 1 : 2;
  if (t == "mirror_x" || t == "mirror_y" || t == "mirror_z") {
    Bounds3 base;
    if (!sub("base", &base)) return false;
    Bounds3 m = base;
    m.min[axis] = -base.max[axis];
    m.max[axis] = -base.min[axis];
    *out = base.merged(m);
    return true;
  }
  if (t == "repeat_x" || t == "repeat_y" || t == "repeat_z") {
    Bounds3 base;
    if (!sub("base", &base)) return false;
    float spacing = 0.0f, count_f = 1.0f;
    number_field(o, {"spacing"}, &spacing);
    number_field(o, {"count"}, &count_f);
    const size_t count = static_cast<size_t>(std::max(std::round(count_f), 1.0f));
    const float start = -0.5f * static_cast<float>(count - 1) * spacing;
    auto shifted = [&](float d) {
      Bounds3 s = base;
      s.min[axis] += d;
      s.max[axis] += d;
      return s;
    };
    Bounds3 acc = shifted(start);
    for (size_t i = 1; i < count; ++i) acc = acc.merged(shifted(start + static_cast<float>(i) * spacing));
    *out = acc;
    return true;
  }
  if (t == "slice_x" || t == "slice_y" || t == "slice_z") {
    Bounds3 base;
    if (!sub("base", &base)) return false;
    float lo = -std::numeric_limits<float>::infinity(), hi = std::numeric_limits<float>::infinity();
    number_field(o, {"min"}, &lo);
    number_field(o, {"max"}, &hi);
    base.min[axis] = std::max(base.min[axis], lo);
    base.max[axis] = std::min(base.max[axis], hi);
    if (base.max[axis] < base.min[axis]) base.max[axis] = base.min[axis];
    *out = base;
    return true;
  }
  if (t == "smooth") {
    Bounds3 base;
    if (!sub("base", &base)) return false;
    float k = 0.0f;
    number_field(o, {"k"}, &k);
    for (int a = 0; a < 3; ++a) {
      base.min[a] -= k * 0.1f;
      base.max[a] += k * 0.1f;
    }
    *out = base;
    return true;
  }
  return false;
}

// object_anchor_point (E:4567-4586): a named face or corner of the bounds,
// else the object's own `anchors` entry moved by its position.
bool anchor_point(const Value& v, const std::string& name, float out[3]) {
  Bounds3 b;
  if (!object_bounds(v, &b)) return false;
  Mode m[3];
  if (anchor_modes(name, m)) {
    float c[3];
    b.center(c);
    for (int a = 0; a < 3; ++a) out[a] = m[a] == kMin ? b.min[a] : m[a] == kMax ? b.max[a] : c[a];
    return true;
  }
  const Value* anchors = v.obj->get("anchors");
  if (!anchors || anchors->kind != Value::Object) return false;
  const Value* p = anchors->obj->get(name);
  float local[3], pos[3];
  if (!p || !as_vec3(*p, local)) return false;
  object_position(v, pos);
  for (int a = 0; a < 3; ++a) out[a] = local[a] + pos[a];
  return true;
}

float number_arg(const Value& v) {
  if (v.kind != Value::Number) unsupported_call();
  return v.num;
}

Value shift_by_anchors(Value v, const Value& other, const std::string& other_name, const std::string& self_name) {
  float to[3], from[3], pos[3];
  if (!anchor_point(other, other_name, to) || !anchor_point(v, self_name, from)) unsupported_call();
  object_position(v, pos);
  for (int a = 0; a < 3; ++a) pos[a] += to[a] - from[a];
  set_position(v, pos);
  return v;
}

// attach_object (E:4934-4986).
Value attach(Value v, const Value& other, const Value& face, const Value* self_face, float gap) {
  Bounds3 sb, ob;
  if (!object_bounds(v, &sb) || !object_bounds(other, &ob)) unbounded();
  AnchorSpec anchor;
  if (!anchor_spec(face, &anchor)) unsupported_call();
  if (self_face) {
    AnchorSpec self_anchor;
    if (!anchor_spec(*self_face, &self_anchor)) unsupported_call();
    return shift_by_anchors(std::move(v), other, anchor.name, self_anchor.name);
  }
  if (!is_one_of(anchor.name, {"Top", "Bottom", "Left", "Right", "Front", "Back"}))
    return shift_by_anchors(std::move(v), other, anchor.name, anchor.name);
  float pos[3];
  object_position(v, pos);
  const float o = anchor.offset;
  if (anchor.name == "Top") pos[1] += ob.max[1] + gap + o - sb.min[1];
  else if (anchor.name == "Bottom") pos[1] += ob.min[1] - gap - o - sb.max[1];
  else if (anchor.name == "Left") pos[0] += ob.min[0] - gap - o - sb.max[0];
  else if (anchor.name == "Right") pos[0] += ob.max[0] + gap + o - sb.min[0];
  else if (anchor.name == "Front") pos[2] += ob.max[2] + gap + o - sb.min[2];
  else pos[2] += ob.min[2] - gap - o - sb.max[2];
  set_position(v, pos);
  return v;
}

// align_object_axis (E:4988-5019).
Value align(Value v, const Value& other, int axis, const Value& anchor_v) {
  AnchorSpec anchor;
  if (!anchor_spec(anchor_v, &anchor)) unsupported_call();
  Bounds3 sb, ob;
  if (!object_bounds(v, &sb) || !object_bounds(other, &ob)) unbounded();
  float pos[3], to[3], delta;
  object_position(v, pos);
  if (anchor_point(other, anchor.name, to)) {
    float from[3];
    if (!anchor_point(v, anchor.name, from)) unsupported_call();
    delta = to[axis] - from[axis] + anchor.offset;
  } else {
    // Reached only for names without built-in modes, which "Center" and the
    // faces all have; kept as the reference states it.
    float sc[3], oc[3];
    sb.center(sc);
    ob.center(oc);
    const std::string& n = anchor.name;
    if (n == "Center") delta = oc[axis] - sc[axis];
    else if (n == "Left" && axis == 0) delta = ob.min[0] - sb.min[0];
    else if (n == "Right" && axis == 0) delta = ob.max[0] - sb.max[0];
    else if (n == "Bottom" && axis == 1) delta = ob.min[1] - sb.min[1];
    else if (n == "Top" && axis == 1) delta = ob.max[1] - sb.max[1];
    else if (n == "Back" && axis == 2) delta = ob.min[2] - sb.min[2];
    else if (n == "Front" && axis == 2) delta = ob.max[2] - sb.max[2];
    else unsupported_call();
    delta += anchor.offset;
  }
  pos[axis] += delta;
  set_position(v, pos);
  return v;
}

// place_object_relative (E:5021-5039).
Value place(Value v, const Value& other, int axis, float sign, float gap) {
  Bounds3 sb, ob;
  if (!object_bounds(v, &sb) || !object_bounds(other, &ob)) unbounded();
  float pos[3];
  object_position(v, pos);
  pos[axis] += sign > 0.0f ? ob.max[axis] + gap - sb.min[axis] : ob.min[axis] - gap - sb.max[axis];
  set_position(v, pos);
  return v;
}

void read_rot(const Value& v, float rot[3]) {
  rot[0] = rot[1] = rot[2] = 0.0f;
  const Value* r = v.kind == Value::Object ? v.obj->get("rot") : nullptr;
  float t[3];
  if (r && as_vec3(*r, t)) std::copy(t, t + 3, rot);
}

// face_object_to (E:4679-4713): pitch and yaw towards the other object.
Value face_to(Value v, const Value& other, const Value* target_anchor) {
  Bounds3 sb;
  if (!object_bounds(v, &sb)) unbounded();
  float target[3];
  if (target_anchor) {
    AnchorSpec a;
    if (!anchor_spec(*target_anchor, &a) || !anchor_point(other, a.name, target)) unsupported_call();
  } else {
    Bounds3 ob;
    if (!object_bounds(other, &ob)) unbounded();
    ob.center(target);
  }
  float origin[3];
  sb.center(origin);
  const float dx = target[0] - origin[0], dy = target[1] - origin[1], dz = target[2] - origin[2];
  const float horizontal = std::sqrt(dx * dx + dz * dz);
  float rot[3];
  read_rot(v, rot);
  rot[0] = rad_to_deg(std::atan2(-dy, std::max(horizontal, 1.0e-9f)));
  rot[1] = rad_to_deg(std::atan2(dx, dz));
  writable(v).fields["rot"] = make_vec3(rot[0], rot[1], rot[2]);
  return v;
}

}  // namespace

bool is_anchor_symbol(const std::string& name) {
  for (const char* n : kAnchorNames)
    if (name == n) return true;
  return false;
}

Value anchor_symbol(const std::string& name, float offset) {
  std::map<std::string, Value> f;
  f["name"] = make_object(name, {});
  f["offset"] = Value::number(offset);
  return make_object("symbol", std::move(f));
}

bool anchor_arithmetic(const Value& l, char op, const Value& r, Value* out) {
  if (op != '+' && op != '-') return false;
  const float sign = op == '+' ? 1.0f : -1.0f;
  AnchorSpec a;
  if (anchor_spec(l, &a) && r.kind == Value::Number) {
    *out = anchor_symbol(a.name, a.offset + sign * r.num);
    return true;
  }
  if (anchor_spec(r, &a) && l.kind == Value::Number) {
    *out = anchor_symbol(a.name, sign * l.num + a.offset);
    return true;
  }
  return false;
}

bool is_layout_member_operator(const std::string& f) {
  return is_one_of(f, {"bind", "attach", "align_x", "align_y", "align_z", "right_of", "left_of", "on_top_of",
                       "below", "in_front_of", "behind", "rotate_x", "rotate_y", "rotate_z", "offset_x", "offset_y",
                       "offset_z", "face_to"});
}

Value build_layout_member(const std::string& field, Value base, const std::vector<Value>& args) {
  auto need = [&](size_t lo, size_t hi) {
    if (args.size() < lo || args.size() > hi) unsupported_call();
  };
  if (field == "bind")
    throw FrontendError(FT_ERR_UNSUPPORTED, "bind: skeleton assets are not evaluated by this front-end");
  if (field == "attach") {
    need(2, 3);
    const Value* self_face = nullptr;
    float gap = 0.0f;
    if (args.size() == 3) {
      if (args[2].kind == Value::Number) gap = args[2].num;
      else self_face = &args[2];
    }
    return attach(std::move(base), args[0], args[1], self_face, gap);
  }
  if (field == "align_x" || field == "align_y" || field == "align_z") {
    need(2, 2);
    return align(std::move(base), args[0], field.back() - 'x', args[1]);
  }
  struct Rel { const char* name; int axis; float sign; };
  static const Rel rels[] = {{"right_of", 0, 1.0f}, {"left_of", 0, -1.0f},    {"on_top_of", 1, 1.0f},
                             {"below", 1, -1.0f},   {"in_front_of", 2, 1.0f}, {"behind", 2, -1.0f}};
  for (const Rel& r : rels) {
    if (field == r.name) {
      need(2, 2);
      return place(std::move(base), args[0], r.axis, r.sign, number_arg(args[1]));
    }
  }
  if (field == "rotate_x" || field == "rotate_y" || field == "rotate_z") {
    need(1, 1);
    const float angle = number_arg(args[0]);
    float rot[3];
    if (base.kind != Value::Object) layout_fail("member access requires object value");
    read_rot(base, rot);
    rot[field.back() - 'x'] = angle;
    writable(base).fields["rot"] = make_vec3(rot[0], rot[1], rot[2]);
    return base;
  }
  if (field == "offset_x" || field == "offset_y" || field == "offset_z") {
    need(1, 1);
    const float d = number_arg(args[0]);
    float pos[3];
    object_position(base, pos);
    pos[field.back() - 'x'] += d;
    set_position(base, pos);
    return base;
  }
  if (field == "face_to") {
    need(1, 2);
    return face_to(std::move(base), args[0], args.size() == 2 ? &args[1] : nullptr);
  }
  unsupported_call();
}

}  // namespace ftfe
