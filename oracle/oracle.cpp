// CPU oracle for the sphere-tracing hot path — TEST INFRASTRUCTURE ONLY.
//
// A restatement of the reference renderer's depth path, templated on the
// arithmetic type R (float reproduces the reference's f32 arithmetic; double
// is the FP64 oracle).  Every function cites the reference code it follows
// (R = crates/forgedthoughts/src/renderer.rs, A = render_api.rs, E = eval.rs).
// The product library never links or calls this file.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_error;

template <class R>
struct V {
  R x, y, z;
};
template <class R> V<R> mk(R x, R y, R z) { return V<R>{x, y, z}; }
template <class R> V<R> operator+(V<R> a, V<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> V<R> operator-(V<R> a, V<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> V<R> operator*(V<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R> R dot(V<R> a, V<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> R len(V<R> a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
template <class R> V<R> cross(V<R> a, V<R> b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// Vec3::normalize (R:414-420, A:24-31)
template <class R> V<R> normalize(V<R> a) {
  R l = len(a);
  if (l <= std::numeric_limits<float>::epsilon()) return a;
  return a * (R(1) / l);
}
template <class R> V<R> vabs(V<R> a) { return mk(std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)); }

// Rust f32::max / f32::min / f32::clamp semantics.
template <class R> R rmax(R a, R b) { return std::fmax(a, b); }
template <class R> R rmin(R a, R b) { return std::fmin(a, b); }
template <class R> R rclamp(R x, R lo, R hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}
template <class R> R rem_euclid(R a, R b) {
  R r = std::fmod(a, b);
  return r < R(0) ? r + std::fabs(b) : r;
}

template <class R> R pi() { return R(3.14159265358979323846); }
template <class R> R to_radians(R d) { return d * (pi<R>() / R(180)); }

template <class R>
struct Aabb {
  V<R> mn, mx;
  V<R> centroid() const { return (mn + mx) * R(0.5); }
  V<R> extent() const { return mx - mn; }
};
template <class R> Aabb<R> aunion(Aabb<R> a, Aabb<R> b) {
  return Aabb<R>{mk(std::min(a.mn.x, b.mn.x), std::min(a.mn.y, b.mn.y), std::min(a.mn.z, b.mn.z)),
                 mk(std::max(a.mx.x, b.mx.x), std::max(a.mx.y, b.mx.y), std::max(a.mx.z, b.mx.z))};
}
template <class R> Aabb<R> expand(Aabb<R> a, R d) { return Aabb<R>{a.mn - mk(d, d, d), a.mx + mk(d, d, d)}; }

// point_aabb_lower_bound (R:5388-5411)
template <class R> R point_aabb_lb(V<R> p, const Aabb<R>& b) {
  R dx = p.x < b.mn.x ? b.mn.x - p.x : (p.x > b.mx.x ? p.x - b.mx.x : R(0));
  R dy = p.y < b.mn.y ? b.mn.y - p.y : (p.y > b.mx.y ? p.y - b.mx.y : R(0));
  R dz = p.z < b.mn.z ? b.mn.z - p.z : (p.z > b.mx.z ? p.z - b.mx.z : R(0));
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// rotate_x / rotate_y / rotate_z (R:6224-6240)
template <class R> V<R> rotate_x(V<R> v, R deg) {
  R r = to_radians(deg), s = std::sin(r), c = std::cos(r);
  return mk(v.x, c * v.y - s * v.z, s * v.y + c * v.z);
}
template <class R> V<R> rotate_y(V<R> v, R deg) {
  R r = to_radians(deg), s = std::sin(r), c = std::cos(r);
  return mk(c * v.x + s * v.z, v.y, -s * v.x + c * v.z);
}
template <class R> V<R> rotate_z(V<R> v, R deg) {
  R r = to_radians(deg), s = std::sin(r), c = std::cos(r);
  return mk(c * v.x - s * v.y, s * v.x + c * v.y, v.z);
}

template <class R>
struct Info {  // DistanceInfo (R:454-459)
  R d;
  uint32_t obj, mat;
};

// hg_sdf operators (R:6019-6137)
template <class R> R op_union_round(R a, R b, R r) {
  r = rmax(std::fabs(r), R(1.0e-6));
  R ux = rmax(r - a, R(0)), uy = rmax(r - b, R(0));
  return rmax(r, rmin(a, b)) - std::sqrt(ux * ux + uy * uy);
}
template <class R> R op_intersect_round(R a, R b, R r) {
  r = rmax(std::fabs(r), R(1.0e-6));
  R ux = rmax(r + a, R(0)), uy = rmax(r + b, R(0));
  return rmin(-r, rmax(a, b)) + std::sqrt(ux * ux + uy * uy);
}
template <class R> R op_diff_round(R a, R b, R r) { return op_intersect_round(a, -b, r); }
template <class R> R frac_1_sqrt_2() { return R(0.70710678118654752440); }
template <class R> R op_union_chamfer(R a, R b, R r) { return rmin(rmin(a, b), (a - r + b) * frac_1_sqrt_2<R>()); }
template <class R> R op_intersect_chamfer(R a, R b, R r) { return rmax(rmax(a, b), (a + r + b) * frac_1_sqrt_2<R>()); }
template <class R> R op_diff_chamfer(R a, R b, R r) { return op_intersect_chamfer(a, -b, r); }
template <class R> R repeat_centered(R p, R size) {
  size = rmax(size, R(1.0e-6));
  return rem_euclid(p + size * R(0.5), size) - size * R(0.5);
}
template <class R> R op_union_columns(R a, R b, R r, R n) {
  if (a < r && b < r) {
    n = rmax(std::round(n), R(2));
    R sq2 = std::sqrt(R(2));
    R col = r * sq2 / ((n - R(1)) * R(2) + sq2);
    R x = a + col, y = b + col;
    bool odd = (static_cast<int>(n) % 2) == 1;
    if (odd) x += col;
    R rx = (x + y) * frac_1_sqrt_2<R>(), ry = (y - x) * frac_1_sqrt_2<R>();
    x = rx;
    y = ry;
    x -= sq2 * R(0.5) * r;
    x += -col * sq2;
    if (odd) y += col;
    y = repeat_centered(y, col * R(2));
    return std::sqrt(x * x + y * y) - col;
  }
  return rmin(a, b);
}
template <class R> R op_intersect_columns(R a, R b, R r, R n) { return -op_union_columns(-a, -b, r, n); }
template <class R> R op_diff_columns(R a, R b, R r, R n) { return -op_union_columns(-a, b, r, n); }
template <class R> R op_union_stairs(R a, R b, R r, R n) {
  n = rmax(std::round(n), R(1));
  R s = r / n;
  R u = b - r;
  return rmin(rmin(a, b), R(0.5) * (u + a + std::fabs(rem_euclid(u - a + s, R(2) * s) - s)));
}
template <class R> R op_intersect_stairs(R a, R b, R r, R n) { return -op_union_stairs(-a, -b, r, n); }
template <class R> R op_diff_stairs(R a, R b, R r, R n) { return -op_union_stairs(-a, b, r, n); }
template <class R> R op_union_soft(R a, R b, R r) {
  r = rmax(std::fabs(r), R(1.0e-6));
  R e = rmax(r - std::fabs(a - b), R(0));
  return rmin(a, b) - e * e * R(0.25) / r;
}
template <class R> R op_pipe(R a, R b, R r) { return std::sqrt(a * a + b * b) - std::fabs(r); }
template <class R> R op_engrave(R a, R b, R r) { return rmax(a, (a + std::fabs(r) - std::fabs(b)) * frac_1_sqrt_2<R>()); }
template <class R> R op_groove(R a, R b, R ra, R rb) { return rmax(a, rmin(a + std::fabs(ra), std::fabs(rb) - std::fabs(b))); }
template <class R> R op_tongue(R a, R b, R ra, R rb) { return rmin(a, rmax(a - std::fabs(ra), std::fabs(b) - std::fabs(rb))); }
template <class R> R op_smax(R a, R b, R k) {
  R h = rmax(k - std::fabs(a - b), R(0));
  return rmax(a, b) + h * h * R(0.25) / rmax(k, R(1.0e-6));
}
template <class R> R op_smin(R a, R b, R k) {
  R h = rmax(k - std::fabs(a - b), R(0));
  return rmin(a, b) - h * h * R(0.25) / rmax(k, R(1.0e-6));
}

// Noise modifier (R:5957-6017)
template <class R> R fractr(R x) { return x - std::floor(x); }
template <class R> R hash_noise(V<R> p) {
  R f1pi = R(0.31830988618379067154);
  V<R> q = mk(fractr(p.x * f1pi + R(0.11)), fractr(p.y * f1pi + R(0.17)), fractr(p.z * f1pi + R(0.13))) * R(17);
  return fractr(q.x * q.y * q.z * (q.x + q.y + q.z));
}
template <class R> R sd_base_noise(V<R> p) {
  p = p + mk(R(0.5), R(0.5), R(0.5));
  V<R> i = mk(std::floor(p.x), std::floor(p.y), std::floor(p.z));
  V<R> f = mk(fractr(p.x), fractr(p.y), fractr(p.z));
  R d = std::numeric_limits<R>::infinity();
  for (int ix = 0; ix <= 1; ++ix)
    for (int iy = 0; iy <= 1; ++iy)
      for (int iz = 0; iz <= 1; ++iz) {
        V<R> c = mk(R(ix), R(iy), R(iz));
        R r = hash_noise(i + c);
        r = r * r * R(0.7);
        d = rmin(d, len(f - c) - r);
      }
  return d;
}
template <class R> R apply_noise(V<R> p, R d, int octaves, R scale, R lac) {
  const R m[3][3] = {{R(0.00), R(1.60), R(1.20)}, {R(-1.60), R(0.72), R(-0.96)}, {R(-1.20), R(-0.96), R(1.28)}};
  V<R> q = p * rmax(scale, R(1.0e-4));
  R os = rmax(lac, R(1.0e-4));
  R s = 1, t = 0;
  for (int o = 0; o < std::max(octaves, 1); ++o) {
    R n = s * sd_base_noise(q);
    n = op_smax(n, d - R(0.1) * s, R(0.3) * s);
    d = op_smin(n, d, R(0.3) * s);
    t += d;
    q = mk(m[0][0] * q.x + m[0][1] * q.y + m[0][2] * q.z, m[1][0] * q.x + m[1][1] * q.y + m[1][2] * q.z,
           m[2][0] * q.x + m[2][1] * q.y + m[2][2] * q.z) * os;
    s *= R(0.415);
    q.z += R(-4.33) * t * s;
  }
  return d;
}

// sd_regular_ngon (R:6206-6214)
template <class R> R sd_regular_ngon(V<R> p, int sides, R radius) {
  R n = R(std::max(sides, 3));
  R an = pi<R>() / n;
  R apothem = radius * std::cos(an);
  R angle = std::atan2(p.z, p.x);
  R sector = R(2) * an;
  R wrapped = rem_euclid(angle + an, sector) - an;
  return std::hypot(p.x, p.z) * std::cos(wrapped) - apothem;
}

template <class R>
class Scene {
 public:
  explicit Scene(const ft_scene_desc& d) : d_(d) {
    // object id -> the primitive or Custom node carrying its transform
    // (object_transforms, R:485-555)
    for (uint32_t i = 0; i < d_.n_nodes; ++i) {
      const ft_node& n = d_.nodes[i];
      if (!(n.kind <= FT_NODE_EXTRUDE_POLYGON || n.kind == FT_NODE_CUSTOM) || n.object_id >= (1u << 20)) continue;
      if (obj_node_.size() <= n.object_id) obj_node_.resize(n.object_id + 1, -1);
      if (obj_node_[n.object_id] < 0) obj_node_[n.object_id] = static_cast<int>(i);
    }
  }

  const ft_scene_desc& desc() const { return d_; }
  const ft_node& node(int i) const { return d_.nodes[i]; }
  int object_node(uint32_t obj) const { return obj < obj_node_.size() ? obj_node_[obj] : -1; }
  // The hard-union leaf (collect_accel_leaves, R:659-671) holding object
  // `obj`, -1 if none.
  int object_leaf(uint32_t obj) const {
    if (!leaves_done_) {
      std::vector<int> stack{d_.root};
      while (!stack.empty()) {
        int i = stack.back();
        stack.pop_back();
        if (d_.nodes[i].kind == FT_NODE_UNION) {
          stack.push_back(d_.nodes[i].a);
          stack.push_back(d_.nodes[i].b);
          continue;
        }
        std::vector<int> sub{i};
        while (!sub.empty()) {
          int k = sub.back();
          sub.pop_back();
          const ft_node& n = d_.nodes[k];
          if (n.kind <= FT_NODE_EXTRUDE_POLYGON || n.kind == FT_NODE_CUSTOM) {
            if (n.object_id < (1u << 20)) {
              if (obj_leaf_.size() <= n.object_id) obj_leaf_.resize(n.object_id + 1, -1);
              if (obj_leaf_[n.object_id] < 0) obj_leaf_[n.object_id] = i;
            }
            continue;
          }
          if (n.a >= 0) sub.push_back(n.a);
          if (n.b >= 0 && n.kind >= FT_NODE_UNION && n.kind <= FT_NODE_TONGUE) sub.push_back(n.b);
        }
      }
      leaves_done_ = true;
    }
    return obj < obj_leaf_.size() ? obj_leaf_[obj] : -1;
  }

  V<R> center(const ft_node& n) const { return mk(R(n.center[0]), R(n.center[1]), R(n.center[2])); }

  // to_local (R:6216-6222)
  V<R> to_local(V<R> p, const ft_node& n) const {
    V<R> q = p - center(n);
    q = rotate_z(q, -R(n.rot_deg[2]));
    q = rotate_y(q, -R(n.rot_deg[1]));
    q = rotate_x(q, -R(n.rot_deg[0]));
    return q;
  }

  // sdf_bounds (R:5242-5386)
  Aabb<R> bounds(int idx) const {
    const ft_node& n = node(idx);
    V<R> c = center(n);
    auto cube = [&](R r) { return Aabb<R>{c - mk(r, r, r), c + mk(r, r, r)}; };
    switch (n.kind) {
      case FT_NODE_SPHERE: return cube(R(n.f[0]));
      case FT_NODE_BOX: return cube(len(mk(R(n.f[0]), R(n.f[1]), R(n.f[2]))));
      case FT_NODE_CYLINDER:
      case FT_NODE_EXTRUDE_POLYGON: return cube(std::sqrt(R(n.f[0]) * R(n.f[0]) + R(n.f[1]) * R(n.f[1])));
      case FT_NODE_TORUS: return cube(R(n.f[0]) + R(n.f[1]));
      case FT_NODE_DOMAIN:
      case FT_NODE_DISTANCE_POST:
      case FT_NODE_NOISE:
      case FT_NODE_CUSTOM:  // the lowering stores the transformed half-extent box (R:5304-5326)
        return Aabb<R>{mk(R(n.bounds_min[0]), R(n.bounds_min[1]), R(n.bounds_min[2])),
                       mk(R(n.bounds_max[0]), R(n.bounds_max[1]), R(n.bounds_max[2]))};
      case FT_NODE_SUBTRACT: return bounds(n.a);
      case FT_NODE_SLICE: {
        Aabb<R> b = bounds(n.a);
        R* mn = n.ival == 0 ? &b.mn.x : n.ival == 1 ? &b.mn.y : &b.mn.z;
        R* mx = n.ival == 0 ? &b.mx.x : n.ival == 1 ? &b.mx.y : &b.mx.z;
        *mn = std::max(*mn, R(n.f[0]));
        *mx = std::min(*mx, R(n.f[1]));
        if (*mx < *mn) *mx = *mn;
        return b;
      }
      case FT_NODE_SMOOTH: return expand(bounds(n.a), R(n.f[0]) * R(0.1));
      default: return aunion(bounds(n.a), bounds(n.b));
    }
  }

  R shell(R d, R sh) const { return sh > R(0) ? rmax(d, -(d + sh)) : d; }

  R prim_distance(const ft_node& n, V<R> p) const {
    V<R> q = to_local(p, n);
    switch (n.kind) {
      case FT_NODE_SPHERE: return shell(len(q) - R(n.f[0]), R(n.f[1]));
      case FT_NODE_BOX: {
        R rd = R(n.f[3]);
        V<R> inner = mk(rmax(R(n.f[0]) - rd, R(0)), rmax(R(n.f[1]) - rd, R(0)), rmax(R(n.f[2]) - rd, R(0)));
        V<R> qq = vabs(q) - inner;
        R outside = len(mk(rmax(qq.x, R(0)), rmax(qq.y, R(0)), rmax(qq.z, R(0))));
        R inside = rmin(rmax(rmax(qq.x, qq.y), qq.z), R(0));
        return shell(outside + inside - rd, R(n.f[4]));
      }
      case FT_NODE_CYLINDER: {
        R rd = R(n.f[2]);
        R radial = std::sqrt(q.x * q.x + q.z * q.z);
        R dx = radial - rmax(R(n.f[0]) - rd, R(0));
        R dy = std::fabs(q.y) - rmax(R(n.f[1]) - rd, R(0));
        R ox = rmax(dx, R(0)), oy = rmax(dy, R(0));
        R outside = std::sqrt(ox * ox + oy * oy);
        R inside = rmin(rmax(dx, dy), R(0));
        return shell(outside + inside - rd, R(n.f[3]));
      }
      case FT_NODE_TORUS: {
        R qx = std::sqrt(q.x * q.x + q.z * q.z) - R(n.f[0]);
        return std::sqrt(qx * qx + q.y * q.y) - R(n.f[1]);
      }
      case FT_NODE_EXTRUDE_POLYGON: {
        R rd = R(n.f[2]);
        R radial = sd_regular_ngon(mk(q.x, R(0), q.z), n.ival, rmax(R(n.f[0]) - rd, R(0)));
        R dy = std::fabs(q.y) - rmax(R(n.f[1]) - rd, R(0));
        R ox = rmax(radial, R(0)), oy = rmax(dy, R(0));
        R outside = std::sqrt(ox * ox + oy * oy);
        R inside = rmin(rmax(radial, dy), R(0));
        return shell(outside + inside - rd, R(n.f[3]));
      }
    }
    return R(0);
  }

  // sdf_lower_bound (R:5413-5543)
  R lower_bound(int idx, V<R> p) const {
    const ft_node& n = node(idx);
    if (n.kind <= FT_NODE_EXTRUDE_POLYGON) return prim_distance(n, p);
    if (n.kind == FT_NODE_CUSTOM) {  // the half-extent box in the node's frame (R:5506-5515)
      V<R> h = mk(R(n.f[0]), R(n.f[1]), R(n.f[2]));
      return point_aabb_lb(to_local(p, n), Aabb<R>{h * R(-1), h});
    }
    switch (n.kind) {
      case FT_NODE_UNION: return rmin(lower_bound(n.a, p), lower_bound(n.b, p));
      case FT_NODE_INTERSECT: return rmax(lower_bound(n.a, p), lower_bound(n.b, p));
      case FT_NODE_SUBTRACT: return lower_bound(n.a, p);
      case FT_NODE_SMOOTH: return lower_bound(n.a, p) - R(n.f[0]) * R(0.1);
      default: return point_aabb_lb(p, bounds(idx));
    }
  }

  // Hook program interpreter (role of the JIT'd hook, E:2011-2146).
  void run_program(int prog, const V<R>* args, V<R>* out) const {
    const ft_program& pg = d_.programs[prog];
    V<R> regs[FT_MAX_PROGRAM_REGS + 256];
    for (uint32_t i = 0; i < pg.n_params; ++i) regs[i] = args[i];
    const R eps = R(std::numeric_limits<float>::epsilon());
    for (uint32_t k = 0; k < pg.n_instr; ++k) {
      const ft_instr& in = d_.instrs[pg.first_instr + k];
      auto opnd = [&](int which) {
        int r = which == 0 ? in.a : which == 1 ? in.b : in.c;
        V<R> v = regs[r];
        if (in.flags & (FT_INSTR_A_SCALAR << which)) v = mk(v.x, v.x, v.x);
        return v;
      };
      V<R> a = opnd(0), b = opnd(1), c = opnd(2);
      V<R> o = mk(R(0), R(0), R(0));
      auto lanes1 = [&](auto f) { o = mk(f(a.x), f(a.y), f(a.z)); };
      auto lanes2 = [&](auto f) { o = mk(f(a.x, b.x), f(a.y, b.y), f(a.z, b.z)); };
      auto lanes3 = [&](auto f) { o = mk(f(a.x, b.x, c.x), f(a.y, b.y, c.y), f(a.z, b.z, c.z)); };
      switch (in.op) {
        case FT_OP_CONST: o = mk(R(in.imm[0]), R(in.imm[1]), R(in.imm[2])); break;
        case FT_OP_MOV: o = a; break;
        case FT_OP_ADD: lanes2([](R x, R y) { return x + y; }); break;
        case FT_OP_SUB: lanes2([](R x, R y) { return x - y; }); break;
        case FT_OP_MUL: lanes2([](R x, R y) { return x * y; }); break;
        case FT_OP_DIV: lanes2([](R x, R y) { return x / y; }); break;
        case FT_OP_NEG: lanes1([](R x) { return -x; }); break;
        case FT_OP_GETX: o = mk(a.x, a.x, a.x); break;
        case FT_OP_GETY: o = mk(a.y, a.y, a.y); break;
        case FT_OP_GETZ: o = mk(a.z, a.z, a.z); break;
        case FT_OP_VEC3: o = mk(a.x, b.x, c.x); break;
        case FT_OP_ABS: lanes1([](R x) { return std::fabs(x); }); break;
        case FT_OP_FLOOR: lanes1([](R x) { return std::floor(x); }); break;
        case FT_OP_CEIL: lanes1([](R x) { return std::ceil(x); }); break;
        case FT_OP_FRACT: lanes1([](R x) { return x - std::floor(x); }); break;
        case FT_OP_SQRT: lanes1([](R x) { return std::sqrt(x); }); break;
        case FT_OP_SIN: lanes1([](R x) { return std::sin(x); }); break;
        case FT_OP_COS: lanes1([](R x) { return std::cos(x); }); break;
        case FT_OP_SATURATE: lanes1([](R x) { return rclamp(x, R(0), R(1)); }); break;
        case FT_OP_MIN: lanes2([](R x, R y) { return rmin(x, y); }); break;
        case FT_OP_MAX: lanes2([](R x, R y) { return rmax(x, y); }); break;
        case FT_OP_POW: lanes2([](R x, R y) { return std::pow(x, y); }); break;
        case FT_OP_CLAMP:
          lanes3([](R x, R lo, R hi) { return lo <= hi ? rclamp(x, lo, hi) : rclamp(x, hi, lo); });
          break;
        case FT_OP_MIX: lanes3([](R x, R y, R t) { return x * (R(1) - t) + y * t; }); break;
        case FT_OP_STEP: o.x = b.x < a.x ? R(0) : R(1); o.y = o.z = o.x; break;
        case FT_OP_SMOOTHSTEP: {
          R span = b.x - a.x;
          R t = std::fabs(span) < eps ? (c.x < a.x ? R(0) : R(1)) : rclamp((c.x - a.x) / span, R(0), R(1));
          o.x = o.y = o.z = t * t * (R(3) - R(2) * t);
          break;
        }
        case FT_OP_DOT: o.x = o.y = o.z = a.x * b.x + a.y * b.y + a.z * b.z; break;
        case FT_OP_LENGTH: o.x = o.y = o.z = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); break;
        case FT_OP_NORMALIZE: {
          R l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
          o = l <= eps ? mk(R(0), R(0), R(0)) : mk(a.x / l, a.y / l, a.z / l);
          break;
        }
        case FT_OP_ROTX: o = rotate_x(a, b.x); break;
        case FT_OP_ROTY: o = rotate_y(a, b.x); break;
        case FT_OP_ROTZ: o = rotate_z(a, b.x); break;
        case FT_OP_RET: *out = a; return;
      }
      regs[in.dst] = o;
    }
    *out = mk(R(0), R(0), R(0));
  }

  // sdf_distance_info (R:5545-5955)
  Info<R> info(int idx, V<R> p) const {
    const ft_node& n = node(idx);
    if (n.kind <= FT_NODE_EXTRUDE_POLYGON) return Info<R>{prim_distance(n, p), n.object_id, n.material_id};
    if (n.kind == FT_NODE_CUSTOM) {
      // eval_custom_sdf_distance (R:6139-6180): domain, distance, distance_post
      V<R> q = to_local(p, n), t;
      if (n.ival >= 0) {
        run_program(n.ival, &q, &t);
        q = t;
      }
      V<R> o;
      run_program(n.program, &q, &o);
      R d = o.x;
      if (n.reserved >= 0) {
        V<R> args[2] = {mk(d, d, d), q};
        run_program(n.reserved, args, &o);
        d = o.x;
      }
      return Info<R>{d, n.object_id, n.material_id};
    }
    switch (n.kind) {
      case FT_NODE_DOMAIN: {
        V<R> q = to_local(p, n), out;
        run_program(n.program, &q, &out);
        return info(n.a, out);
      }
      case FT_NODE_DISTANCE_POST: {
        V<R> q = to_local(p, n);
        Info<R> i = info(n.a, q);
        V<R> args[2] = {mk(i.d, i.d, i.d), q}, out;
        run_program(n.program, args, &out);
        i.d = out.x;
        return i;
      }
      case FT_NODE_NOISE: {
        V<R> q = to_local(p, n);
        Info<R> i = info(n.a, q);
        i.d = apply_noise(q, i.d, n.ival, R(n.f[0]), R(n.f[1]));
        return i;
      }
      case FT_NODE_UNION: {
        R llb = lower_bound(n.a, p), rlb = lower_bound(n.b, p);
        if (llb <= rlb) {
          Info<R> l = info(n.a, p);
          if (l.d <= rlb) return l;
          Info<R> r = info(n.b, p);
          return l.d <= r.d ? l : r;
        }
        Info<R> r = info(n.b, p);
        if (r.d <= llb) return r;
        Info<R> l = info(n.a, p);
        return l.d <= r.d ? l : r;
      }
      case FT_NODE_INTERSECT: {
        Info<R> l = info(n.a, p), r = info(n.b, p);
        return l.d >= r.d ? l : r;
      }
      case FT_NODE_SUBTRACT: {
        Info<R> l = info(n.a, p), r = info(n.b, p);
        R rd = -r.d;
        if (l.d >= rd) return l;
        return Info<R>{rd, r.obj, r.mat};
      }
      case FT_NODE_SLICE: {
        Info<R> i = info(n.a, p);
        R coord = n.ival == 0 ? p.x : n.ival == 1 ? p.y : p.z;
        R slab = rmax(R(n.f[0]) - coord, coord - R(n.f[1]));
        i.d = rmax(i.d, slab);
        return i;
      }
      case FT_NODE_SMOOTH: {
        Info<R> i = info(n.a, p);
        i.d -= R(n.f[0]) * R(0.1);
        return i;
      }
      default: break;
    }
    Info<R> l = info(n.a, p), r = info(n.b, p);
    R ra = R(n.f[0]), rb = R(n.f[1]);
    R d;
    switch (n.kind) {
      case FT_NODE_UNION_ROUND: d = op_union_round(l.d, r.d, ra); break;
      case FT_NODE_UNION_CHAMFER: d = op_union_chamfer(l.d, r.d, ra); break;
      case FT_NODE_UNION_COLUMNS: d = op_union_columns(l.d, r.d, ra, rb); break;
      case FT_NODE_UNION_STAIRS: d = op_union_stairs(l.d, r.d, ra, rb); break;
      case FT_NODE_UNION_SOFT: d = op_union_soft(l.d, r.d, ra); break;
      case FT_NODE_INTERSECT_ROUND: d = op_intersect_round(l.d, r.d, ra); break;
      case FT_NODE_INTERSECT_CHAMFER: d = op_intersect_chamfer(l.d, r.d, ra); break;
      case FT_NODE_INTERSECT_COLUMNS: d = op_intersect_columns(l.d, r.d, ra, rb); break;
      case FT_NODE_INTERSECT_STAIRS: d = op_intersect_stairs(l.d, r.d, ra, rb); break;
      case FT_NODE_DIFF_ROUND: d = op_diff_round(l.d, r.d, ra); break;
      case FT_NODE_DIFF_CHAMFER: d = op_diff_chamfer(l.d, r.d, ra); break;
      case FT_NODE_DIFF_COLUMNS: d = op_diff_columns(l.d, r.d, ra, rb); break;
      case FT_NODE_DIFF_STAIRS: d = op_diff_stairs(l.d, r.d, ra, rb); break;
      case FT_NODE_PIPE: return Info<R>{op_pipe(l.d, r.d, ra), l.obj, l.mat};
      case FT_NODE_ENGRAVE: return Info<R>{op_engrave(l.d, r.d, ra), l.obj, l.mat};
      case FT_NODE_GROOVE: return Info<R>{op_groove(l.d, r.d, ra, rb), l.obj, l.mat};
      case FT_NODE_TONGUE: return Info<R>{op_tongue(l.d, r.d, ra, rb), l.obj, l.mat};
      default: return l;
    }
    bool union_like = n.kind >= FT_NODE_UNION_ROUND && n.kind <= FT_NODE_UNION_SOFT;
    bool inter_like = n.kind >= FT_NODE_INTERSECT_ROUND && n.kind <= FT_NODE_INTERSECT_STAIRS;
    if (union_like) return l.d <= r.d ? Info<R>{d, l.obj, l.mat} : Info<R>{d, r.obj, r.mat};
    if (inter_like) return l.d >= r.d ? Info<R>{d, l.obj, l.mat} : Info<R>{d, r.obj, r.mat};
    // diff_*: keep lhs ids when lhs dominates -rhs
    return l.d >= -r.d ? Info<R>{d, l.obj, l.mat} : Info<R>{d, r.obj, r.mat};
  }

 private:
  const ft_scene_desc& d_;
  std::vector<int> obj_node_;
  mutable std::vector<int> obj_leaf_;
  mutable bool leaves_done_ = false;
};

// ------------------------------------------------------------ accelerators
template <class R>
struct Leaf {  // AccelLeaf (R:625-629)
  Aabb<R> bounds;
  int node;
};

template <class R>
struct Accel {
  const Scene<R>& scene;
  int mode;
  Aabb<R> scene_bounds;
  std::vector<Leaf<R>> leaves;
  // BVH (R:673-732): flat nodes, child indices or leaf index
  struct BNode {
    Aabb<R> b;
    int lhs = -1, rhs = -1, leaf = -1;
  };
  std::vector<BNode> bvh;
  int bvh_root = -1;
  // Brick grid (R:824-1022)
  size_t dims = 0;
  std::vector<std::vector<size_t>> cells;
  bool has_grid = false;

  Accel(const Scene<R>& s, int m) : scene(s), mode(m) {
    int root = s.desc().root;
    scene_bounds = s.bounds(root);
    if (mode == FT_ACCEL_NAIVE) return;
    collect(root);
    if (mode == FT_ACCEL_BVH) {
      std::vector<size_t> idx(leaves.size());
      for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
      bvh_root = build(idx);
    } else {
      build_grid();
    }
  }

  // collect_accel_leaves (R:659-670)
  void collect(int idx) {
    const ft_node& n = scene.node(idx);
    if (n.kind == FT_NODE_UNION) {
      collect(n.a);
      collect(n.b);
      return;
    }
    leaves.push_back(Leaf<R>{scene.bounds(idx), idx});
  }

  static R centroid_axis(const Aabb<R>& b, int axis) {
    V<R> c = b.centroid();
    return axis == 0 ? c.x : axis == 1 ? c.y : c.z;
  }

  // build_bvh (R:693-732)
  int build(const std::vector<size_t>& indices) {
    if (indices.empty()) return -1;
    if (indices.size() == 1) {
      BNode n;
      n.b = leaves[indices[0]].bounds;
      n.leaf = static_cast<int>(indices[0]);
      bvh.push_back(n);
      return static_cast<int>(bvh.size()) - 1;
    }
    Aabb<R> b = leaves[indices[0]].bounds;
    for (size_t k = 1; k < indices.size(); ++k) b = aunion(b, leaves[indices[k]].bounds);
    V<R> e = b.extent();
    int axis = (e.x >= e.y && e.x >= e.z) ? 0 : (e.y >= e.z ? 1 : 2);
    std::vector<size_t> sorted = indices;
    std::stable_sort(sorted.begin(), sorted.end(), [&](size_t x, size_t y) {
      return centroid_axis(leaves[x].bounds, axis) < centroid_axis(leaves[y].bounds, axis);
    });
    size_t mid = sorted.size() / 2;
    int l = build(std::vector<size_t>(sorted.begin(), sorted.begin() + mid));
    int r = build(std::vector<size_t>(sorted.begin() + mid, sorted.end()));
    BNode n;
    n.b = b;
    n.lhs = l;
    n.rhs = r;
    bvh.push_back(n);
    return static_cast<int>(bvh.size()) - 1;
  }

  // accel_leaf_distance_info (R:635-657): a Custom leaf farther from its box
  // than a tenth of the box diagonal (clamped to [0.05, 0.5]) is that bound.
  Info<R> leaf_info(const Leaf<R>& l, V<R> p) const {
    const ft_node& n = scene.node(l.node);
    if (n.kind == FT_NODE_CUSTOM) {
      R lb = point_aabb_lb(p, l.bounds);
      R far = rclamp(len(l.bounds.mx - l.bounds.mn) * R(0.1), R(0.05), R(0.5));
      if (lb > far) return Info<R>{lb, n.object_id, n.material_id};
    }
    return scene.info(l.node, p);
  }

  // bvh_distance_info (R:743-786)
  bool bvh_info(int ni, V<R> p, R& best, Info<R>& out) const {
    const BNode& n = bvh[ni];
    if (point_aabb_lb(p, n.b) > best) return false;
    if (n.leaf >= 0) {
      Info<R> i = leaf_info(leaves[n.leaf], p);
      if (i.d < best) best = i.d;
      out = i;
      return true;
    }
    R llb = point_aabb_lb(p, bvh[n.lhs].b), rlb = point_aabb_lb(p, bvh[n.rhs].b);
    int first = n.lhs, second = n.rhs;
    R flb = llb, slb = rlb;
    if (!(llb <= rlb)) {
      first = n.rhs; second = n.lhs; flb = rlb; slb = llb;
    }
    bool have = false;
    Info<R> cur{};
    if (flb <= best) have = bvh_info(first, p, best, cur);
    Info<R> other;
    if (slb <= best && bvh_info(second, p, best, other)) {
      if (!(have && cur.d <= other.d)) cur = other;
      have = true;
    }
    if (have) out = cur;
    return have;
  }

  // bvh_lower_bound (R:788-822)
  bool bvh_lb(int ni, V<R> p, R& best, R& out) const {
    const BNode& n = bvh[ni];
    if (point_aabb_lb(p, n.b) > best) return false;
    if (n.leaf >= 0) {
      R lb = point_aabb_lb(p, n.b);
      if (lb < best) best = lb;
      out = lb;
      return true;
    }
    R llb = point_aabb_lb(p, bvh[n.lhs].b), rlb = point_aabb_lb(p, bvh[n.rhs].b);
    int first = llb <= rlb ? n.lhs : n.rhs, second = llb <= rlb ? n.rhs : n.lhs;
    bool have = false;
    R cur = 0;
    if (point_aabb_lb(p, bvh[first].b) <= best) have = bvh_lb(first, p, best, cur);
    R other;
    if (point_aabb_lb(p, bvh[second].b) <= best && bvh_lb(second, p, best, other)) {
      cur = have ? std::min(cur, other) : other;
      have = true;
    }
    if (have) out = cur;
    return have;
  }

  size_t cell_index(const size_t c[3]) const { return c[0] + dims * (c[1] + dims * c[2]); }

  // brick_cell_coords (R:980-993)
  void cell_coords(V<R> p, size_t out[3]) const {
    V<R> e = scene_bounds.extent();
    R pv[3] = {p.x, p.y, p.z}, mn[3] = {scene_bounds.mn.x, scene_bounds.mn.y, scene_bounds.mn.z};
    R ex[3] = {e.x, e.y, e.z};
    for (int k = 0; k < 3; ++k) {
      if (ex[k] <= R(1.0e-6)) {
        out[k] = 0;
        continue;
      }
      R v = rclamp((pv[k] - mn[k]) / ex[k], R(0), R(0.999999)) * R(dims);
      out[k] = static_cast<size_t>(v);
    }
  }

  // brick_cell_aabb (R:995-1012)
  Aabb<R> cell_aabb(const size_t c[3]) const {
    V<R> e = scene_bounds.extent();
    R dm = R(std::max<size_t>(dims, 1));
    V<R> size = mk(e.x / dm, e.y / dm, e.z / dm);
    V<R> mn = mk(scene_bounds.mn.x + size.x * R(c[0]), scene_bounds.mn.y + size.y * R(c[1]),
                 scene_bounds.mn.z + size.z * R(c[2]));
    return Aabb<R>{mn, mn + size};
  }

  // brick_shell_lower_bound (R:1014-1044)
  R shell_lb(const size_t o[3], size_t shell, V<R> p) const {
    if (shell == 0) return R(0);
    size_t mnc[3], mxc[3];
    for (int k = 0; k < 3; ++k) {
      mnc[k] = o[k] >= shell ? o[k] - shell : 0;
      mxc[k] = std::min(o[k] + shell, dims - 1);
    }
    Aabb<R> a = cell_aabb(mnc), b = cell_aabb(mxc);
    return point_aabb_lb(p, Aabb<R>{a.mn, b.mx});
  }

  // BrickGrid::from_leaves (R:831-864)
  void build_grid() {
    if (leaves.empty()) return;
    float cnt = static_cast<float>(std::max<size_t>(leaves.size(), 1));
    dims = static_cast<size_t>(std::max(std::ceil(std::cbrt(cnt)), 1.0f));
    cells.assign(dims * dims * dims, {});
    for (size_t li = 0; li < leaves.size(); ++li) {
      size_t a[3], b[3];
      cell_coords(leaves[li].bounds.mn, a);
      cell_coords(leaves[li].bounds.mx, b);
      for (size_t z = a[2]; z <= b[2]; ++z)
        for (size_t y = a[1]; y <= b[1]; ++y)
          for (size_t x = a[0]; x <= b[0]; ++x) {
            size_t c[3] = {x, y, z};
            cells[cell_index(c)].push_back(li);
          }
    }
    for (auto& c : cells) {
      std::sort(c.begin(), c.end());
      c.erase(std::unique(c.begin(), c.end()), c.end());
    }
    has_grid = true;
  }

  template <class Visit>
  void grid_walk(V<R> p, R& best, Visit visit) const {
    size_t o[3];
    cell_coords(p, o);
    size_t max_shell = dims;
    std::vector<char> visited(leaves.size(), 0);
    for (size_t shell = 0; shell < max_shell; ++shell) {
      if (shell_lb(o, shell, p) > best) break;
      size_t lo[3], hi[3];
      for (int k = 0; k < 3; ++k) {
        lo[k] = o[k] >= shell ? o[k] - shell : 0;
        hi[k] = std::min(o[k] + shell, dims - 1);
      }
      for (size_t z = lo[2]; z <= hi[2]; ++z)
        for (size_t y = lo[1]; y <= hi[1]; ++y)
          for (size_t x = lo[0]; x <= hi[0]; ++x) {
            if (shell > 0 && x > lo[0] && x < hi[0] && y > lo[1] && y < hi[1] && z > lo[2] && z < hi[2]) continue;
            size_t c[3] = {x, y, z};
            for (size_t li : cells[cell_index(c)]) {
              if (visited[li]) continue;
              visited[li] = 1;
              visit(li);
            }
          }
    }
  }

  // Accelerator::distance_info for the three modes (R:1024-1129, R:866-922)
  Info<R> distance_info(V<R> p) const {
    int root = scene.desc().root;
    if (mode == FT_ACCEL_NAIVE) return scene.info(root, p);
    if (mode == FT_ACCEL_BVH) {
      R best = std::numeric_limits<R>::infinity();
      Info<R> out;
      if (bvh_root >= 0 && bvh_info(bvh_root, p, best, out)) return out;
      return scene.info(root, p);
    }
    if (!has_grid) return scene.info(root, p);
    R best = std::numeric_limits<R>::infinity();
    bool have = false;
    Info<R> bi{};
    grid_walk(p, best, [&](size_t li) {
      R lb = point_aabb_lb(p, leaves[li].bounds);
      if (lb > best) return;
      Info<R> i = leaf_info(leaves[li], p);
      if (i.d < best) {
        best = i.d;
        bi = i;
        have = true;
      }
    });
    return have ? bi : scene.info(leaves[0].node, p);
  }

  R distance(V<R> p) const { return distance_info(p).d; }

  // Accelerator::lower_bound (R:1040-1042, R:1078-1084, R:1118-1124, R:924-963)
  R lower_bound(V<R> p) const {
    int root = scene.desc().root;
    if (mode == FT_ACCEL_NAIVE) return scene.lower_bound(root, p);
    if (mode == FT_ACCEL_BVH) {
      R best = std::numeric_limits<R>::infinity();
      R out;
      if (bvh_root >= 0 && bvh_lb(bvh_root, p, best, out)) return out;
      return scene.lower_bound(root, p);
    }
    if (!has_grid) return scene.lower_bound(root, p);
    R best = std::numeric_limits<R>::infinity();
    grid_walk(p, best, [&](size_t li) {
      R lb = point_aabb_lb(p, leaves[li].bounds);
      if (lb < best) best = lb;
    });
    return best;
  }
};

// ------------------------------------------------------------ march
template <class R>
struct Hit {
  R t;
  V<R> pos, normal;
  uint32_t obj, mat;
};

struct Opts {
  uint32_t width, height, max_steps;
  float max_dist, epsilon, step_scale, camera_z, fov;
};

// ray_aabb_intersection (R:4141-4173)
template <class R> bool ray_aabb(V<R> o, V<R> d, const Aabb<R>& b, R* t0o, R* t1o) {
  R tmin = -std::numeric_limits<R>::infinity(), tmax = std::numeric_limits<R>::infinity();
  R os[3] = {o.x, o.y, o.z}, ds[3] = {d.x, d.y, d.z};
  R mn[3] = {b.mn.x, b.mn.y, b.mn.z}, mx[3] = {b.mx.x, b.mx.y, b.mx.z};
  for (int k = 0; k < 3; ++k) {
    if (std::fabs(ds[k]) <= R(1.0e-8)) {
      if (os[k] < mn[k] || os[k] > mx[k]) return false;
      continue;
    }
    R inv = R(1) / ds[k];
    R t0 = (mn[k] - os[k]) * inv, t1 = (mx[k] - os[k]) * inv;
    if (t0 > t1) std::swap(t0, t1);
    tmin = rmax(tmin, t0);
    tmax = rmin(tmax, t1);
    if (tmax < tmin) return false;
  }
  *t0o = tmin;
  *t1o = tmax;
  return true;
}

// raymarch_hit (R:4091-4139), refine_hit_distance (R:4180-4200),
// estimate_normal (R:4202-4215)
template <class R>
bool raymarch(const Accel<R>& acc, V<R> o, V<R> d, const Opts& op, R min_t, R max_t, Hit<R>* hit, uint64_t* evals) {
  R t0, t1;
  if (!ray_aabb(o, d, acc.scene_bounds, &t0, &t1)) return false;
  max_t = rmin(max_t, t1);
  R traveled = rmax(min_t, rmax(t0, R(0)));
  R prev = traveled;
  R eps = R(op.epsilon);
  for (uint32_t s = 0; s < op.max_steps; ++s) {
    if (traveled > max_t) return false;
    V<R> p = o + d * traveled;
    Info<R> info = acc.distance_info(p);
    ++*evals;
    if (std::fabs(info.d) < eps) {
      R lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        R mid = R(0.5) * (lo + hi);
        R dm = std::fabs(acc.distance(o + d * mid));
        ++*evals;
        if (dm < eps) hi = mid;
        else lo = mid;
      }
      V<R> pos = o + d * hi;
      R e = rmax(eps * R(4), R(1.0e-5));
      R dx = acc.distance(mk(pos.x + e, pos.y, pos.z)) - acc.distance(mk(pos.x - e, pos.y, pos.z));
      R dy = acc.distance(mk(pos.x, pos.y + e, pos.z)) - acc.distance(mk(pos.x, pos.y - e, pos.z));
      R dz = acc.distance(mk(pos.x, pos.y, pos.z + e)) - acc.distance(mk(pos.x, pos.y, pos.z - e));
      *evals += 6;
      V<R> nn = mk(dx, dy, dz);
      V<R> normal = len(nn) > R(1.0e-8) ? normalize(nn) : mk(R(0), R(1), R(0));
      Info<R> fin = acc.distance_info(pos);
      ++*evals;
      hit->t = hi;
      hit->pos = pos;
      hit->normal = normal;
      hit->obj = fin.obj;
      hit->mat = fin.mat;
      return true;
    }
    prev = traveled;
    R step = rmax(std::fabs(info.d) * rclamp(R(op.step_scale), R(0.05), R(1)), rmax(eps * R(0.5), R(1.0e-5)));
    traveled += step;
  }
  return false;
}

// Camera resolution (R:6263-6286) and PinholeCamera::generate_ray (A:132-144).
template <class R>
struct Camera {
  V<R> origin, forward, right, up;
  R tan_fov;
  Camera(const ft_scene_desc& d, const Opts& op) {
    V<R> c = mk(R(d.scene_center[0]), R(d.scene_center[1]), R(d.scene_center[2]));
    V<R> org = c + mk(R(0), R(0), R(op.camera_z));
    V<R> tgt = c;
    R fov = R(op.fov);
    if (d.has_camera) {
      if (!std::isnan(d.camera.origin[0])) org = mk(R(d.camera.origin[0]), R(d.camera.origin[1]), R(d.camera.origin[2]));
      if (!std::isnan(d.camera.target[0])) tgt = mk(R(d.camera.target[0]), R(d.camera.target[1]), R(d.camera.target[2]));
      if (!std::isnan(d.camera.fov_y_degrees)) fov = R(d.camera.fov_y_degrees);
    }
    origin = org;
    V<R> upv = mk(R(0), R(1), R(0));
    forward = normalize(tgt - org);
    right = normalize(cross(forward, upv));
    up = normalize(cross(right, forward));
    tan_fov = std::tan(R(0.5) * to_radians(fov));
  }
  V<R> dir(R ndc_x, R ndc_y) const {
    V<R> d = normalize(forward + right * (ndc_x * tan_fov) + up * (ndc_y * tan_fov));
    return normalize(d);  // render_*_tile normalizes the API ray again (R:3904, R:3956)
  }
};

// pixel_sample_offsets (R:4838-4854)
std::vector<std::pair<float, float>> sample_offsets(uint32_t samples) {
  samples = std::max(samples, 1u);
  uint32_t grid = static_cast<uint32_t>(std::ceil(std::sqrt(static_cast<float>(samples))));
  std::vector<std::pair<float, float>> out;
  for (uint32_t iy = 0; iy < grid; ++iy)
    for (uint32_t ix = 0; ix < grid; ++ix) {
      if (out.size() >= samples) break;
      out.emplace_back((static_cast<float>(ix) + 0.5f) / static_cast<float>(grid),
                       (static_cast<float>(iy) + 0.5f) / static_cast<float>(grid));
    }
  return out;
}

// XorShift64 (R:4735-4761) and seed_pixel_sample (R:4763-4774): the jittered
// sub-pixel offsets of the progressive renderer (R:4008-4013).
struct XorShift64 {
  uint64_t state;
  explicit XorShift64(uint64_t seed) : state(seed == 0 ? 0x9E3779B97F4A7C15ull : seed) {}
  uint64_t next_u64() {
    uint64_t x = state;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    state = x;
    return x;
  }
  float next_f32() { return static_cast<float>(static_cast<uint32_t>(next_u64() >> 40)) / static_cast<float>(1u << 24); }
};

uint64_t seed_pixel_sample(uint32_t x, uint32_t y, uint32_t width, uint32_t sample) {
  uint64_t base = (static_cast<uint64_t>(y) * width + x) * 0x9E3779B97F4A7C15ull + 0xBF58476D1CE4E5B9ull;
  return base ^ (static_cast<uint64_t>(sample) * 0x94D049BB133111EBull) ^ 0xD6E8FEB86659FD93ull;
}

// NDC (before the aspect scale) of sample s of pixel (x, y): the AA grid, or
// with jitter_seed >= 0 the jittered offsets seeded with
// seed_pixel_sample ^ jitter_seed.
inline void sample_ndc(uint32_t x, uint32_t y, uint32_t s, uint32_t width, uint32_t height,
                       const std::vector<std::pair<float, float>>& offs, int64_t jitter_seed, float* px, float* py) {
  if (jitter_seed >= 0) {
    XorShift64 rng(seed_pixel_sample(x, y, width, s) ^ static_cast<uint64_t>(jitter_seed));
    const float jx = rng.next_f32() - 0.5f;
    const float jy = rng.next_f32() - 0.5f;
    *px = ((static_cast<float>(x) + 0.5f + jx) / static_cast<float>(width)) * 2.0f - 1.0f;
    *py = 1.0f - ((static_cast<float>(y) + 0.5f + jy) / static_cast<float>(height)) * 2.0f;
    return;
  }
  *px = ((static_cast<float>(x) + offs[s].first) / static_cast<float>(width)) * 2.0f - 1.0f;
  *py = 1.0f - ((static_cast<float>(y) + offs[s].second) / static_cast<float>(height)) * 2.0f;
}

// depth_preview_value + spectrum_to_rgb8 (R:5215-5227)
uint8_t depth_to_u8(float v) {
  float mapped = std::min(std::pow(std::fmax(v, 0.0f), 1.0f / 2.2f), 1.0f);
  return static_cast<uint8_t>(mapped * 255.0f);
}

Opts resolve(const ft_render_options* o) {
  return Opts{o->width, o->height, o->max_steps, o->max_dist, o->epsilon, o->step_scale, o->camera_z, o->fov_y_degrees};
}

// Pixels per work item of the host thread pool (a row segment, so that a
// sample of a few rows still spreads over every core).
constexpr uint32_t kSegment = 32;

// Columns of a (possibly strided) pixel sample of each row.
inline std::vector<uint32_t> sample_columns(uint32_t width, uint32_t col_begin, uint32_t col_step) {
  std::vector<uint32_t> cols;
  col_step = std::max(col_step, 1u);
  for (uint32_t x = col_begin; x < width; x += col_step) cols.push_back(x);
  return cols;
}

template <class R>
int render_depth(const ft_scene_desc* desc, const ft_render_options* options, int accel, uint32_t aa, int threads,
                 uint32_t row_begin, uint32_t row_end, uint32_t row_step, float* t_out, uint8_t* mask_out,
                 uint32_t* mat_out, float* normal_out, uint8_t* rgb_out, uint64_t* evals_out,
                 uint32_t col_begin = 0, uint32_t col_step = 1, int64_t jitter_seed = -1) {
  Opts op = resolve(options);
  Scene<R> scene(*desc);
  Accel<R> acc(scene, accel);
  Camera<R> cam(*desc, op);
  aa = std::max(aa, 1u);
  auto offs = sample_offsets(aa);
  // render_*_tile (R:3931-3971): aspect and NDC in f32.
  float aspect = static_cast<float>(op.width) / static_cast<float>(op.height);
  if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  row_step = std::max(row_step, 1u);
  row_end = std::min(row_end, op.height);
  std::vector<uint32_t> rows;
  for (uint32_t y = row_begin; y < row_end; y += row_step) rows.push_back(y);
  std::vector<uint32_t> cols = sample_columns(op.width, col_begin, col_step);
  const size_t segs = (cols.size() + kSegment - 1) / kSegment;  // work item: one row segment
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> total{0};
  auto worker = [&]() {
    uint64_t evals = 0;
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= rows.size() * segs) break;
      uint32_t y = rows[k / segs];
      size_t c0 = (k % segs) * kSegment, c1 = std::min(c0 + kSegment, cols.size());
      for (size_t ci = c0; ci < c1; ++ci) {
        const uint32_t x = cols[ci];
        float sum = 0.0f;
        for (uint32_t s = 0; s < aa; ++s) {
          float px, py;
          sample_ndc(x, y, s, op.width, op.height, offs, jitter_seed, &px, &py);
          V<R> d = cam.dir(R(px * aspect), R(py));
          Hit<R> h;
          bool hit = raymarch(acc, cam.origin, d, op, R(0), R(op.max_dist), &h, &evals);
          size_t idx = (static_cast<size_t>(y) * op.width + x) * aa + s;
          float depth = 0.0f;
          if (hit) {
            // depth_preview_value is computed in f32 from the f32 hit distance.
            float t = static_cast<float>(h.t);
            float dd = rclamp(t / std::max(op.max_dist, 1.0e-6f), 0.0f, 1.0f);
            float shaped = 1.0f - dd;
            depth = shaped * shaped;
          }
          sum += depth;
          if (t_out) t_out[idx] = hit ? static_cast<float>(h.t) : 0.0f;
          if (mask_out) mask_out[idx] = hit ? 1 : 0;
          if (mat_out) mat_out[idx] = hit ? h.mat : 0;
          if (normal_out) {
            normal_out[3 * idx] = hit ? static_cast<float>(h.normal.x) : 0.0f;
            normal_out[3 * idx + 1] = hit ? static_cast<float>(h.normal.y) : 0.0f;
            normal_out[3 * idx + 2] = hit ? static_cast<float>(h.normal.z) : 0.0f;
          }
        }
        if (rgb_out) {
          uint8_t g = depth_to_u8(sum * (1.0f / static_cast<float>(aa)));
          size_t pi = (static_cast<size_t>(y) * op.width + x) * 3;
          rgb_out[pi] = rgb_out[pi + 1] = rgb_out[pi + 2] = g;
        }
      }
    }
    total.fetch_add(evals);
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (evals_out) *evals_out = total.load();
  return 0;
}

// ============================================================ Whitted trace
// Restates crates/forgedthoughts/src/renderer/ray.rs:3-222 (trace_ray_recursive,
// trace_hit_with_material) with the shading helpers of renderer.rs, the
// materials of materials/{mod,lambert,metal,dielectric,standard}.rs and the
// lights of render_api.rs.  Dynamic material hooks and rough-dielectric lobes
// (roughness > 0.06 on transmissive materials) are not restated.

template <class R>
struct Sp {
  R r, g, b;
};
template <class R> Sp<R> sp(R r, R g, R b) { return Sp<R>{r, g, b}; }
template <class R> Sp<R> operator+(Sp<R> a, Sp<R> b) { return sp(a.r + b.r, a.g + b.g, a.b + b.b); }
template <class R> Sp<R> operator*(Sp<R> a, Sp<R> b) { return sp(a.r * b.r, a.g * b.g, a.b * b.b); }
template <class R> Sp<R> scale(Sp<R> a, R s) { return sp(a.r * s, a.g * s, a.b * s); }
template <class R> Sp<R> black() { return sp(R(0), R(0), R(0)); }
// lerp_spectrum (R:5205-5213): clamped t, a*(1-t) + b*t
template <class R> Sp<R> lerp_sp(Sp<R> a, Sp<R> b, R t) {
  R tt = rclamp(t, R(0), R(1));
  return sp(a.r * (R(1) - tt) + b.r * tt, a.g * (R(1) - tt) + b.g * tt, a.b * (R(1) - tt) + b.b * tt);
}

enum Model { kStandard = 0, kLambert = 1, kMetal = 2, kDielectric = 3, kBlend = 4 };

template <class R>
struct Params {  // MaterialParams (materials/mod.rs:66-86), render-relevant fields
  Sp<R> color;
  R roughness, metallic, specular, specular_weight;
  Sp<R> specular_color;
  R ior, clearcoat, clearcoat_roughness, transmission;
  bool thin_walled;
  Sp<R> emission_color;
  R emission_strength;
  // MediumParams (materials/mod.rs), present when the material has one
  bool has_medium = false;
  R medium_ior = R(1);
  Sp<R> medium_absorption = Sp<R>{R(1), R(1), R(1)};
  R medium_density = R(0);
  // dynamic_material_id (R:6669): the material whose BSDF hooks apply, -1 none
  int dyn = -1;
};

template <class R>
struct Mat {  // Material enum incl. Blend (materials/mod.rs:214-230)
  int kind = kStandard;  // Model
  Params<R> p;           // Standard/Lambert/Metal/Dielectric params, or blend's a
  int b_model = 0, a_model = 0;
  Params<R> pb;
  R t = 0;
};

template <class R> Params<R> params_from(const ft_material& m) {
  Params<R> p;
  p.color = sp(R(m.color[0]), R(m.color[1]), R(m.color[2]));
  p.roughness = R(m.roughness);
  p.metallic = R(m.metallic);
  p.specular = R(m.specular);
  p.specular_weight = R(m.specular_weight);
  p.specular_color = sp(R(m.specular_color[0]), R(m.specular_color[1]), R(m.specular_color[2]));
  p.ior = R(m.ior);
  p.clearcoat = R(m.clearcoat);
  p.clearcoat_roughness = R(m.clearcoat_roughness);
  p.transmission = R(m.transmission);
  p.thin_walled = m.thin_walled != 0;
  p.emission_color = sp(R(m.emission_color[0]), R(m.emission_color[1]), R(m.emission_color[2]));
  p.emission_strength = R(m.emission_strength);
  p.has_medium = m.has_medium != 0;
  p.medium_ior = R(m.medium_ior);
  p.medium_absorption = sp(R(m.medium_absorption[0]), R(m.medium_absorption[1]), R(m.medium_absorption[2]));
  p.medium_density = R(m.medium_density);
  return p;
}

// material_for_id (R:6895-6900)
template <class R> Mat<R> material_for_id(const ft_scene_desc& d, uint32_t id) {
  Mat<R> m;
  if (d.n_materials == 0) {
    m.kind = kStandard;
    ft_material dm;
    std::memset(&dm, 0, sizeof(dm));
    dm.color[0] = dm.color[1] = dm.color[2] = 0.8f;
    dm.roughness = 0.5f; dm.ior = 1.5f; dm.specular = 0.5f; dm.specular_weight = 1.0f;
    dm.specular_color[0] = dm.specular_color[1] = dm.specular_color[2] = 1.0f; dm.clearcoat_roughness = 0.1f;
    m.p = params_from<R>(dm);
    return m;
  }
  const ft_material& fm = d.materials[id < d.n_materials ? id : 0];
  m.kind = fm.kind;
  m.p = params_from<R>(fm);
  m.p.dyn = static_cast<int>(id < d.n_materials ? id : 0);
  return m;
}

template <class R> int dominant_model(const Mat<R>& m) {
  if (m.kind != kBlend) return m.kind;
  return m.t < R(0.5) ? m.a_model : m.b_model;
}
template <class R> Params<R> dominant_params(const Mat<R>& m) {
  if (m.kind != kBlend) return m.p;
  return m.t < R(0.5) ? m.p : m.pb;
}

// blend_params / blend_materials (R:7602-7651)
template <class R> Params<R> blend_params(Params<R> a, const Params<R>& b, R t) {
  a.color = lerp_sp(a.color, b.color, t);
  a.roughness = a.roughness + (b.roughness - a.roughness) * t;
  a.metallic = a.metallic + (b.metallic - a.metallic) * t;
  a.specular = a.specular + (b.specular - a.specular) * t;
  a.specular_weight = a.specular_weight + (b.specular_weight - a.specular_weight) * t;
  a.specular_color = lerp_sp(a.specular_color, b.specular_color, t);
  a.ior = a.ior + (b.ior - a.ior) * t;
  a.clearcoat = a.clearcoat + (b.clearcoat - a.clearcoat) * t;
  a.clearcoat_roughness = a.clearcoat_roughness + (b.clearcoat_roughness - a.clearcoat_roughness) * t;
  a.transmission = a.transmission + (b.transmission - a.transmission) * t;
  a.thin_walled = t < R(0.5) ? a.thin_walled : b.thin_walled;
  a.emission_color = lerp_sp(a.emission_color, b.emission_color, t);
  a.emission_strength = a.emission_strength + (b.emission_strength - a.emission_strength) * t;
  // blend_medium (R:7543-7565): both present blend (the colour through
  // lerp_spectrum's clamped t); one present is kept on its side of t = 0.5
  if (a.has_medium && b.has_medium) {
    a.medium_ior = a.medium_ior + (b.medium_ior - a.medium_ior) * t;
    a.medium_absorption = lerp_sp(a.medium_absorption, b.medium_absorption, t);
    a.medium_density = a.medium_density + (b.medium_density - a.medium_density) * t;
  } else if (a.has_medium) {
    a.has_medium = t < R(0.5);
  } else if (b.has_medium && t >= R(0.5)) {
    a.has_medium = true;
    a.medium_ior = b.medium_ior;
    a.medium_absorption = b.medium_absorption;
    a.medium_density = b.medium_density;
  }
  a.dyn = -1;  // dynamic_material_id = None (R:7624)
  return a;
}
template <class R> Mat<R> blend_materials(const Mat<R>& a, const Mat<R>& b, R t) {
  if (a.kind != kBlend && a.kind == b.kind) {
    Mat<R> m;
    m.kind = a.kind;
    m.p = blend_params(a.p, b.p, t);
    return m;
  }
  Mat<R> m;
  m.kind = kBlend;
  m.a_model = dominant_model(a);
  m.p = dominant_params(a);
  m.b_model = dominant_model(b);
  m.pb = dominant_params(b);
  m.t = rclamp(t, R(0), R(1));
  return m;
}

// Material::emission (materials/mod.rs:284-296)
template <class R> Sp<R> emission(const Mat<R>& m) {
  auto e = [](const Params<R>& p) { return scale(p.emission_color, rmax(p.emission_strength, R(0))); };
  if (m.kind != kBlend) return e(m.p);
  return lerp_sp(e(m.p), e(m.pb), m.t);
}

template <class R> R pi_() { return R(3.14159265358979323846); }

// metal.rs:7-20, 84-102
template <class R> R ggx_d(R ndoth, R alpha) {
  R a2 = alpha * alpha, n2 = ndoth * ndoth;
  R denom = rmax(n2 * (a2 - R(1)) + R(1), R(1.0e-5));
  return a2 / (pi_<R>() * denom * denom);
}
template <class R> R smith_g1(R ndotx, R alpha) {
  R k = (alpha * alpha) * R(0.5);
  return ndotx / rmax(ndotx * (R(1) - k) + k, R(1.0e-5));
}
template <class R> Sp<R> fresnel_schlick_sp(Sp<R> f0, R c) {
  R x = R(1) - rclamp(c, R(0), R(1));
  R m = x * x * x * x * x;
  return f0 + scale(sp(R(1), R(1), R(1)), m) + scale(f0, -m);
}
template <class R> Sp<R> metal_eval(const Params<R>& m, V<R> n, V<R> wi, V<R> wo) {
  R ndotl = rmax(dot(n, wi), R(0)), ndotv = rmax(dot(n, wo), R(0));
  if (ndotl <= R(0) || ndotv <= R(0)) return black<R>();
  V<R> h = normalize(wi + wo);
  R ndoth = rmax(dot(n, h), R(0)), vdoth = rmax(dot(wo, h), R(0));
  R rr = rclamp(m.roughness, R(0.02), R(1));
  R alpha = rr * rr;
  R d = ggx_d(ndoth, alpha);
  R g = smith_g1(ndotl, alpha) * smith_g1(ndotv, alpha);
  Sp<R> f = fresnel_schlick_sp(m.color, vdoth);
  return scale(f, (d * g) / rmax(R(4) * ndotl * ndotv, R(1.0e-5)));
}
// lambert.rs:7-13
template <class R> Sp<R> lambert_eval(const Params<R>& m, V<R> n, V<R> wi) {
  if (dot(n, wi) <= R(0)) return black<R>();
  return scale(m.color, R(1) / pi_<R>());
}
template <class R> R f0_from_ior(R ior) {
  R i = rmax(ior, R(1.0e-3));
  R r = (i - R(1)) / (i + R(1));
  return r * r;
}
// standard.rs:6-43, 170-183
template <class R> Sp<R> standard_eval(const Params<R>& m, V<R> n, V<R> wi, V<R> wo) {
  R ndotl = rmax(dot(n, wi), R(0)), ndotv = rmax(dot(n, wo), R(0));
  if (ndotl <= R(0) || ndotv <= R(0)) return black<R>();
  R metallic = rclamp(m.metallic, R(0), R(1));
  R transmission = rclamp(m.transmission, R(0), R(1));
  R clearcoat = rclamp(m.clearcoat, R(0), R(1));
  R cx = rclamp(R(1) - rclamp(ndotv, R(0), R(1)), R(0), R(1));
  R x2 = cx * cx;
  R schlick_w = x2 * x2 * cx;
  R coat_cover = rclamp(clearcoat * (R(0.2) + R(0.8) * schlick_w) * R(0.65), R(0), R(0.95));
  R base_kd = rclamp((R(1) - metallic) * (R(1) - transmission), R(0), R(1)) * (R(1) - coat_cover);
  Sp<R> diffuse = scale(m.color, base_kd / pi_<R>());
  R f0d = rclamp(f0_from_ior(m.ior), R(0), R(1));
  Sp<R> base_f0 = scale(sp(f0d, f0d, f0d), rclamp(m.specular, R(0), R(1)) * rclamp(m.specular_weight, R(0), R(1))) *
                  m.specular_color;
  // standard.rs lerp_spectrum: a.scale(1 - t) + b.scale(t), unclamped
  Sp<R> spec_f0 = scale(base_f0, R(1) - metallic) + scale(m.color, metallic);
  Params<R> sparams = m;
  sparams.color = spec_f0;
  Sp<R> specular = scale(metal_eval(sparams, n, wi, wo), R(1) - coat_cover * R(0.85));
  Sp<R> cc = black<R>();
  if (clearcoat > R(1.0e-5)) {
    Params<R> cp = m;
    cp.color = sp(R(1), R(1), R(1));
    cp.roughness = rclamp(m.clearcoat_roughness, R(0.02), R(1));
    cc = scale(metal_eval(cp, n, wi, wo), clearcoat * R(0.18));
  }
  return diffuse + specular + cc;
}
template <class R> Sp<R> model_eval(int model, const Params<R>& p, V<R> n, V<R> wi, V<R> wo) {
  switch (model) {
    case kStandard: return standard_eval(p, n, wi, wo);
    case kLambert: return lambert_eval(p, n, wi);
    case kMetal: return metal_eval(p, n, wi, wo);
    default: return black<R>();  // dielectric.rs:5-7
  }
}
// Material::eval (materials/mod.rs:298-310)
template <class R> Sp<R> mat_eval(const Mat<R>& m, V<R> n, V<R> wi, V<R> wo) {
  if (m.kind != kBlend) return model_eval(m.kind, m.p, n, wi, wo);
  return lerp_sp(model_eval(m.a_model, m.p, n, wi, wo), model_eval(m.b_model, m.pb, n, wi, wo), m.t);
}

// ---------------------------------------------------------------- BSDF sampling
// Material::sample / Material::pdf for the MIS path tracer (materials/mod.rs:
// 312-340, 399-432; lambert.rs, metal.rs, dielectric.rs, standard.rs).
template <class R> struct BsdfSampleT {
  V<R> wi;
  Sp<R> f;
  R pdf;
  bool delta, apply_cos, transmission, thin_walled;
  R next_ior;
};
template <class R> struct SampleInputT {
  bool front_face;
  R current_ior, u1, u2, u3;
};
// to_world (lambert.rs:52-61, metal.rs:65-74)
template <class R> V<R> to_world(V<R> normal, R x, R y, R z) {
  V<R> n = normalize(normal);
  V<R> helper = std::fabs(n.y) < R(0.99) ? mk(R(0), R(1), R(0)) : mk(R(1), R(0), R(0));
  V<R> t = normalize(cross(helper, n));
  V<R> b = normalize(cross(n, t));
  return normalize((t * x + b * y) + n * z);
}
template <class R> R lambert_pdf(V<R> n, V<R> wi) { return rmax(dot(n, wi), R(0)) / pi_<R>(); }
template <class R> BsdfSampleT<R> lambert_sample(const Params<R>& m, V<R> n, const SampleInputT<R>& in) {
  R uu1 = rclamp(in.u1, R(1.0e-6), R(1) - R(1.0e-6)), uu2 = rclamp(in.u2, R(1.0e-6), R(1) - R(1.0e-6));
  R r = std::sqrt(uu1), phi = R(2) * pi_<R>() * uu2;
  V<R> wi = to_world(n, r * std::cos(phi), r * std::sin(phi), std::sqrt(R(1) - uu1));
  return BsdfSampleT<R>{wi, lambert_eval(m, n, wi), rmax(lambert_pdf(n, wi), R(1.0e-6)), false, true, false, false,
                        in.current_ior};
}
template <class R> R metal_pdf_of(R roughness, V<R> n, V<R> wi, V<R> wo) {
  if (dot(n, wi) <= R(0) || dot(n, wo) <= R(0)) return R(0);
  V<R> h = normalize(wi + wo);
  R ndoth = rmax(dot(n, h), R(0)), vdoth = rmax(std::fabs(dot(wo, h)), R(1.0e-6));
  R rr = rclamp(roughness, R(0.02), R(1));
  R d = ggx_d(ndoth, rr * rr);
  return rmax(d * ndoth / (R(4) * vdoth), R(0));
}
template <class R> V<R> reflect_about(V<R> v, V<R> n) { return v - n * (R(2) * dot(v, n)); }
template <class R> BsdfSampleT<R> metal_sample(const Params<R>& m, V<R> n, V<R> wo, const SampleInputT<R>& in) {
  R rr = rclamp(m.roughness, R(0.02), R(1));
  R alpha = rr * rr;
  R uu1 = rclamp(in.u1, R(1.0e-6), R(1) - R(1.0e-6)), uu2 = rclamp(in.u2, R(1.0e-6), R(1) - R(1.0e-6));
  R phi = R(2) * pi_<R>() * uu2;
  R cos_t = std::sqrt((R(1) - uu1) / (R(1) + (alpha * alpha - R(1)) * uu1));
  R sin_t = std::sqrt(rmax(R(1) - cos_t * cos_t, R(0)));
  V<R> h = to_world(n, sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t);
  V<R> wi = normalize(reflect_about(wo * R(-1), h));
  return BsdfSampleT<R>{wi, metal_eval(m, n, wi, wo), rmax(metal_pdf_of(m.roughness, n, wi, wo), R(1.0e-6)), false,
                        true, false, false, in.current_ior};
}
template <class R> R fresnel_dielectric_of(R ci, R eta_i, R eta_t) {  // R:5188-5204
  R ei = rmax(eta_i, R(1.0e-4)), et = rmax(eta_t, R(1.0e-4));
  if (std::fabs(ei - et) < R(1.0e-6)) return R(0);
  ci = rclamp(ci, R(0), R(1));
  R eta = ei / et;
  R sin2 = eta * eta * (R(1) - ci * ci);
  if (sin2 >= R(1)) return R(1);
  R ct = std::sqrt(R(1) - sin2);
  R rs = ((ei * ci) - (et * ct)) / rmax((ei * ci) + (et * ct), R(1.0e-6));
  R rp = ((et * ci) - (ei * ct)) / rmax((et * ci) + (ei * ct), R(1.0e-6));
  return R(0.5) * (rs * rs + rp * rp);
}
// dielectric.rs refract (lines 81-94)
template <class R> bool refract_of(V<R> incident, V<R> normal, R eta, V<R>* out) {
  V<R> i = normalize(incident), n = normalize(normal);
  R cosi = rclamp(dot(i, n), R(-1), R(1));
  if (cosi > R(0)) n = n * R(-1);
  else cosi = -cosi;
  R sin2 = eta * eta * (R(1) - cosi * cosi);
  if (sin2 > R(1)) return false;
  R cost = std::sqrt(R(1) - sin2);
  *out = normalize(i * eta + n * (eta * cosi - cost));
  return true;
}
template <class R> BsdfSampleT<R> dielectric_sample(Sp<R> color, R ior_in, bool thin, V<R> normal, V<R> wo,
                                                   const SampleInputT<R>& in) {
  R ior = rclamp(ior_in, R(1), R(3));
  R eta_i, eta_t, next_ior;
  if (thin) { eta_i = R(1); eta_t = R(1); next_ior = in.current_ior; }
  else if (in.front_face) { eta_i = in.current_ior; eta_t = ior; next_ior = ior; }
  else { eta_i = in.current_ior; eta_t = R(1); next_ior = R(1); }
  V<R> n = normalize(normal), incident = wo * R(-1);
  R fresnel = rclamp(fresnel_dielectric_of(std::fabs(dot(n, wo)), eta_i, eta_t), R(0), R(1));
  if (in.u1 < fresnel)
    return BsdfSampleT<R>{normalize(reflect_about(incident, n)), sp(R(1), R(1), R(1)), rmax(fresnel, R(1.0e-6)), true,
                          false, false, thin, in.current_ior};
  V<R> wt;
  if (refract_of(incident, n, eta_i / eta_t, &wt))
    return BsdfSampleT<R>{normalize(wt), color, rmax(R(1) - fresnel, R(1.0e-6)), true, false, true, thin, next_ior};
  return BsdfSampleT<R>{normalize(reflect_about(incident, n)), sp(R(1), R(1), R(1)), R(1), true, false, false, thin,
                        in.current_ior};
}
// standard.rs:45-160
template <class R> void standard_weights(const Params<R>& m, V<R> n, V<R> wo, R* dw, R* sw, R* cw) {
  R metallic = rclamp(m.metallic, R(0), R(1)), transmission = rclamp(m.transmission, R(0), R(1));
  R clearcoat = rclamp(m.clearcoat, R(0), R(1));
  R ndotv = rmax(dot(n, wo), R(0));
  R cx = rclamp(R(1) - rclamp(ndotv, R(0), R(1)), R(0), R(1));
  R x2 = cx * cx;
  R coat_cover = rclamp(clearcoat * (R(0.2) + R(0.8) * (x2 * x2 * cx)) * R(0.65), R(0), R(0.95));
  *dw = rmax((R(1) - metallic) * (R(1) - transmission), R(0)) * (R(1) - coat_cover);
  *sw = rclamp((m.specular * m.specular_weight) * (R(1) - transmission), R(0), R(1)) * (R(1) - coat_cover * R(0.85));
  *cw = clearcoat * R(0.18);
}
template <class R> R standard_pdf(const Params<R>& m, V<R> n, V<R> wi, V<R> wo) {
  R dw, sw, cw;
  standard_weights(m, n, wo, &dw, &sw, &cw);
  R sum = dw + sw + cw;
  if (sum <= R(1.0e-6)) return lambert_pdf(n, wi);
  return (dw / sum) * lambert_pdf(n, wi) + (sw / sum) * metal_pdf_of(m.roughness, n, wi, wo) +
         (cw / sum) * metal_pdf_of(rclamp(m.clearcoat_roughness, R(0.02), R(1)), n, wi, wo);
}
template <class R> BsdfSampleT<R> standard_sample(const Params<R>& m, V<R> n, V<R> wo, const SampleInputT<R>& in) {
  R dw, sw, cw;
  standard_weights(m, n, wo, &dw, &sw, &cw);
  R tw = rclamp(m.transmission, R(0), R(1));
  R sum = dw + sw + cw + tw;
  if (sum <= R(1.0e-6)) return lambert_sample(m, n, in);
  R pick = rclamp(in.u3, R(0), R(1)) * sum;
  if (pick < dw) {
    BsdfSampleT<R> s = lambert_sample(m, n, in);
    s.f = standard_eval(m, n, s.wi, wo);
    s.pdf = rmax(standard_pdf(m, n, s.wi, wo), R(1.0e-6));
    return s;
  }
  if (pick < dw + sw || pick < dw + sw + cw) {
    Params<R> mp = m;
    if (pick < dw + sw) {
      // blended_f0 (standard.rs:168-175), lerp unclamped as standard.rs
      R f0d = rclamp(f0_from_ior(m.ior), R(0), R(1));
      Sp<R> base = scale(sp(f0d, f0d, f0d), rclamp(m.specular, R(0), R(1)) * rclamp(m.specular_weight, R(0), R(1))) *
                   m.specular_color;
      R met = rclamp(m.metallic, R(0), R(1));
      mp.color = scale(base, R(1) - met) + scale(m.color, met);
    } else {
      mp.color = sp(R(1), R(1), R(1));
      mp.roughness = rclamp(m.clearcoat_roughness, R(0.02), R(1));
    }
    BsdfSampleT<R> s = metal_sample(mp, n, wo, in);
    s.f = standard_eval(m, n, s.wi, wo);
    s.pdf = rmax(standard_pdf(m, n, s.wi, wo), R(1.0e-6));
    return s;
  }
  BsdfSampleT<R> s = dielectric_sample(m.color, m.ior, m.thin_walled, n, wo, in);
  s.f = s.transmission ? m.color : standard_eval(m, n, s.wi, wo);
  s.pdf = s.delta ? rmax(s.pdf, R(1.0e-6)) : rmax(standard_pdf(m, n, s.wi, wo), R(1.0e-6));
  return s;
}
template <class R> R model_pdf(int model, const Params<R>& p, V<R> n, V<R> wi, V<R> wo) {
  switch (model) {
    case kStandard: return standard_pdf(p, n, wi, wo);
    case kLambert: return lambert_pdf(n, wi);
    case kMetal: return metal_pdf_of(p.roughness, n, wi, wo);
    default: return R(0);  // dielectric.rs:9-11
  }
}
template <class R> BsdfSampleT<R> model_sample(int model, const Params<R>& p, V<R> n, V<R> wo,
                                              const SampleInputT<R>& in) {
  switch (model) {
    case kStandard: return standard_sample(p, n, wo, in);
    case kLambert: return lambert_sample(p, n, in);
    case kMetal: return metal_sample(p, n, wo, in);
    default: return dielectric_sample(p.color, p.ior, p.thin_walled, n, wo, in);
  }
}
template <class R> R mat_pdf(const Mat<R>& m, V<R> n, V<R> wi, V<R> wo) {
  if (m.kind != kBlend) return model_pdf(m.kind, m.p, n, wi, wo);
  R t = rclamp(m.t, R(0), R(1));
  return model_pdf(m.a_model, m.p, n, wi, wo) * (R(1) - t) + model_pdf(m.b_model, m.pb, n, wi, wo) * t;
}
// Material::sample incl. sample_blend (materials/mod.rs:399-432)
template <class R> BsdfSampleT<R> mat_sample(const Mat<R>& m, V<R> n, V<R> wo, const SampleInputT<R>& in) {
  if (m.kind != kBlend) return model_sample(m.kind, m.p, n, wo, in);
  R t = rclamp(m.t, R(0), R(1));
  BsdfSampleT<R> c = in.u3 < t ? model_sample(m.b_model, m.pb, n, wo, in) : model_sample(m.a_model, m.p, n, wo, in);
  Sp<R> f = lerp_sp(model_eval(m.a_model, m.p, n, c.wi, wo), model_eval(m.b_model, m.pb, n, c.wi, wo), t);
  R pdf = rmax(model_pdf(m.a_model, m.p, n, c.wi, wo) * (R(1) - t) + model_pdf(m.b_model, m.pb, n, c.wi, wo) * t,
               R(1.0e-6));
  bool all_delta = m.a_model == kDielectric && m.b_model == kDielectric;
  return BsdfSampleT<R>{c.wi, f, pdf, c.delta && all_delta, c.apply_cos, c.transmission, c.thin_walled, c.next_ior};
}
template <class R> R luminance(const Sp<R>& s) { return R(0.2126) * s.r + R(0.7152) * s.g + R(0.0722) * s.b; }
template <class R> Sp<R> clamp_luma(const Sp<R>& s, R max_luma) {  // clamp_spectrum (R:5168-5175)
  R l = luminance(s);
  if (l <= max_luma || l <= R(1.0e-6)) return s;
  return scale(s, max_luma / l);
}
template <class R> R power_heuristic(R pa, R pb) {  // R:5098-5102
  R a2 = pa * pa, b2 = pb * pb;
  return a2 / rmax(a2 + b2, R(1.0e-6));
}

template <class R> R smoothstepf(R e0, R e1, R x) {  // R:7538-7541
  R t = rclamp((x - e0) / rmax(e1 - e0, R(1.0e-6)), R(0), R(1));
  return t * t * (R(3) - R(2) * t);
}

template <class R>
struct Medium {  // MediumState (R:4372-4387)
  R ior;
  Sp<R> absorption;
  R density;
  static Medium air() { return Medium{R(1), sp(R(1), R(1), R(1)), R(0)}; }
};

// medium_transmittance (R:5109-5119): per channel, the clamped absorption
// colour to the power density * distance; white without density or distance.
template <class R> Sp<R> medium_transmittance(const Medium<R>& m, R dist) {
  if (m.density <= R(0) || dist <= R(0)) return sp(R(1), R(1), R(1));
  R e = m.density * rmax(dist, R(0));
  return sp(std::pow(rclamp(m.absorption.r, R(0), R(1)), e), std::pow(rclamp(m.absorption.g, R(0), R(1)), e),
            std::pow(rclamp(m.absorption.b, R(0), R(1)), e));
}

// transition_medium with medium_state_from_material (R:5125-5166): crossing
// into a transmissive material enters its explicit medium (IOR clamped to
// [1, 3], density at least 0), else one of its IOR with no absorption;
// leaving it returns to air; other materials keep the current medium.
template <class R> Medium<R> transition_medium(const Mat<R>& m, bool front, Medium<R> cur) {
  int model = dominant_model(m);
  Params<R> p = dominant_params(m);
  bool transmissive = model == kDielectric || (model == kStandard && p.transmission > R(0.01));
  if (!transmissive) return cur;
  if (!front) return Medium<R>::air();
  if (p.has_medium)
    return Medium<R>{rclamp(p.medium_ior, R(1), R(3)), p.medium_absorption, rmax(p.medium_density, R(0))};
  return Medium<R>{rclamp(p.ior, R(1), R(3)), sp(R(1), R(1), R(1)), R(0)};
}

// Where a hit's normal and material are resolved from: 0 = the scene root,
// walking its unions with sdf_distance_info as the reference does
// (resolve_surface_normal_at_hit / resolve_material_at_hit); 1 = the
// hard-union leaf holding the hit's object, the leaf the accelerator's
// distance evaluation found (the GPU's resolution).  The two differ only
// where a union's culling in sdf_distance_info skips the hit's leaf: a leaf
// whose surface lies outside its box (an object with both hooks, whose
// transform applies twice).  Test-only switch (oracle_set_resolve_mode).
int g_resolve_mode = 0;

template <class R>
class Tracer {
 public:
  // BsdfContextBase (build_bsdf_context, R:4397-4449): position, local
  // position in the hit object's frame (object_transforms), shading normal,
  // wo, front face, object and material ids, current IOR.
  struct BsdfCtx {
    V<R> pos, local, normal, wo;
    R front, obj, mat, current_ior;
  };
  Tracer(const Scene<R>& s, const Accel<R>& a, const Opts& op, uint32_t max_depth)
      : S(s), A(a), op_(op), max_depth_(std::max(max_depth, 1u)) {}

  // rough_lobe_directions (ray.rs:376-411)
  static int lobe_directions(V<R> ideal_dir, R roughness, int count, V<R>* dirs) {
    V<R> ideal = normalize(ideal_dir);
    V<R> seed = std::fabs(ideal.y) < R(0.99) ? mk(R(0), R(1), R(0)) : mk(R(1), R(0), R(0));
    V<R> tangent = normalize(cross(ideal, seed));
    V<R> bitangent = normalize(cross(tangent, ideal));
    R spread = rclamp(roughness, R(0), R(0.5)) * R(0.35);
    dirs[0] = ideal;
    if (count <= 1 || spread <= R(1.0e-4)) return 1;
    const R ox[6] = {R(1), R(-1), R(0), R(0), R(0.707), R(-0.707)};
    const R oy[6] = {R(0), R(0), R(1), R(-1), R(0.707), R(0.707)};
    int n = 1;
    for (int k = 0; k < 6 && k < count - 1; ++k)
      dirs[n++] = normalize((ideal + tangent * (ox[k] * spread)) + bitangent * (oy[k] * spread));
    return n;
  }
  // rough_dielectric_reflection_samples / _refraction_samples (ray.rs:413-435)
  static int rough_reflection_samples(R r) { return r < R(0.12) ? 1 : (r < R(0.28) ? 2 : 3); }
  static int rough_refraction_samples(R r) { return r < R(0.1) ? 2 : (r < R(0.24) ? 3 : 4); }
  // trace_lobe_average (ray.rs:354-374)
  Sp<R> lobe_average(V<R> hit_point, V<R> gn, V<R> ideal, Medium<R> med, uint32_t depth, R rough, int count,
                     uint64_t* evals) const {
    V<R> dirs[7];
    int n = lobe_directions(ideal, rough, count, dirs);
    R inv = R(1) / R(n);
    Sp<R> sum = black<R>();
    for (int k = 0; k < n; ++k) {
      V<R> o = offset_origin(hit_point, gn, dirs[k], R(op_.epsilon) * (R(8) + rough * R(12)));
      sum = sum + scale(trace(o, dirs[k], med, depth + 1, evals), inv);
    }
    return sum;
  }

  // ---------------------------------------------------------------- MIS path tracer
  // trace_path (renderer/path.rs:3-112) with estimate_direct_mis and
  // sample_one_light (R:4572-4704).  The path lights are the scene's lights
  // with sphere lights as points (parse_lights R:6288-6388), in binding-name
  // order.
  struct PathCtx {  // BsdfContextBase (R:4397-4449) and the hit's geometric normal
    V<R> normal, wo, hit_normal;
    bool front;
    R current_ior;
    BsdfCtx b;
  };
  R env_light_pdf_for_dir(const Mat<R>& m, const PathCtx& c, V<R> wi) const {  // R:4336-4355
    const ft_scene_desc& d = S.desc();
    if (d.n_lights == 0) return R(0);
    R env = 0;
    for (uint32_t i = 0; i < d.n_lights; ++i) env += d.lights[i].kind == FT_LIGHT_ENV ? R(1) : R(0);
    if (env <= R(0)) return R(0);
    return (env / R(d.n_lights)) * rmax(bsdf_pdf(m, c.b, wi), R(1.0e-6));
  }
  // cosine_sample_hemisphere (R:4676-4695): two draws of the path's generator
  static V<R> cosine_hemisphere(V<R> normal, XorShift64& rng) {
    R u1 = rclamp(R(rng.next_f32()), R(1.0e-6), R(1) - R(1.0e-6));
    R u2 = rclamp(R(rng.next_f32()), R(1.0e-6), R(1) - R(1.0e-6));
    R r = std::sqrt(u1), phi = R(2) * pi_<R>() * u2;
    return to_world(normal, r * std::cos(phi), r * std::sin(phi), std::sqrt(R(1) - u1));
  }
  Sp<R> estimate_direct_mis(const Mat<R>& m, V<R> p, const PathCtx& c, XorShift64& rng, uint64_t* evals) const {
    const ft_scene_desc& d = S.desc();
    if (d.n_lights == 0) return black<R>();
    // sample_one_light
    const R count = R(d.n_lights);
    size_t idx = std::min(static_cast<size_t>(std::floor(R(rng.next_f32()) * count)), size_t(d.n_lights - 1));
    const ft_light& L = d.lights[idx];
    const R select_pdf = R(1) / count;
    V<R> wi;
    Sp<R> rad;
    R pdf, max_t;
    bool delta;
    if (L.kind == FT_LIGHT_ENV) {
      wi = cosine_hemisphere(c.normal, rng);
      R env_pdf = rmax(rmax(dot(c.normal, wi), R(0)) / pi_<R>(), R(1.0e-6));
      rad = sp(R(L.intensity[0]), R(L.intensity[1]), R(L.intensity[2]));
      pdf = select_pdf * rmax(env_pdf, R(1.0e-6));
      max_t = std::numeric_limits<R>::infinity();
      delta = false;
    } else {
      V<R> to_light = mk(R(L.position[0]), R(L.position[1]), R(L.position[2])) - p;
      R dist = rmax(std::sqrt(dot(to_light, to_light)), R(1.0e-4));
      wi = to_light * (R(1) / dist);
      rad = scale(sp(R(L.intensity[0]), R(L.intensity[1]), R(L.intensity[2])), R(1) / (dist * dist));
      pdf = select_pdf;
      max_t = dist - R(1.0e-4);
      delta = true;
    }
    if (pdf <= R(1.0e-6)) return black<R>();
    R cos_t = rmax(dot(c.normal, wi), R(0));
    if (cos_t <= R(0)) return black<R>();
    V<R> so = offset_origin(p, c.hit_normal, wi, R(op_.epsilon));
    R vis = shadow(so, wi, max_t, evals);
    if (vis <= R(0)) return black<R>();
    Sp<R> f = bsdf_eval(m, c.b, wi);
    R bpdf = rmax(bsdf_pdf(m, c.b, wi), R(1.0e-6));
    R w = delta ? R(1) : power_heuristic(pdf, bpdf);
    return scale(f * rad, (cos_t * vis * w) / rmax(pdf, R(1.0e-6)));
  }
  Sp<R> trace_path(V<R> origin, V<R> dir, uint32_t max_bounces, XorShift64& rng, uint64_t* evals) const {
    Sp<R> throughput = sp(R(1), R(1), R(1)), radiance = black<R>();
    bool have_prev = false;
    R prev_pdf = 0;
    PathCtx prev_ctx{};
    Mat<R> prev_mat;
    Medium<R> medium = Medium<R>::air();
    const R eps = R(op_.epsilon);
    for (uint32_t bounce = 0; bounce < max_bounces; ++bounce) {
      R min_t = bounce == 0 ? R(0) : eps * R(2);
      Hit<R> h;
      if (!raymarch(A, origin, dir, op_, min_t, R(op_.max_dist), &h, evals)) {
        Sp<R> env = attenuate(environment(dir), medium, R(op_.max_dist));
        R weight = R(1);
        if (have_prev)
          weight = power_heuristic(rmax(prev_pdf, R(1.0e-6)),
                                   rmax(env_light_pdf_for_dir(prev_mat, prev_ctx, dir), R(1.0e-6)));
        radiance = radiance + scale(throughput * env, weight);
        break;
      }
      throughput = throughput * medium_transmittance(medium, h.t);
      const bool front = dot(h.normal, dir) < R(0);
      V<R> wo = normalize(dir * R(-1));
      const HookCtx hc{h.pos, front ? normalize(h.normal) : normalize(h.normal * R(-1)), wo, front ? R(1) : R(0)};
      Mat<R> m;
      if (!material_from_node(resolve_root(h), h.pos, hc, &m)) m = material_for_id<R>(S.desc(), h.mat);
      PathCtx c;
      c.front = front;
      c.hit_normal = front ? normalize(h.normal) : normalize(h.normal * R(-1));
      c.normal = c.hit_normal;
      V<R> gnode;
      if (surface_normal(resolve_root(h), h.pos, R(1.0e-4), &gnode)) c.normal = normalize(front ? gnode : gnode * R(-1));
      c.wo = wo;
      c.current_ior = medium.ior;
      c.b = bsdf_context(h, front, c.normal, dir * R(-1), medium.ior);
      c.normal = c.b.normal;
      Sp<R> em = emission(m);
      if (em.r > R(0) || em.g > R(0) || em.b > R(0)) radiance = radiance + throughput * em;
      Sp<R> direct = estimate_direct_mis(m, h.pos, c, rng, evals);
      radiance = radiance + clamp_luma(throughput * direct, R(12));
      // sample_bsdf_lobe (R:4870-4903)
      SampleInputT<R> in{front, c.current_ior, R(rng.next_f32()), R(rng.next_f32()), R(rng.next_f32())};
      BsdfSampleT<R> smp = bsdf_sample(m, c.b, in);
      if (smp.pdf <= R(1.0e-6)) break;
      if (smp.apply_cos) {
        R ct = rmax(dot(c.normal, smp.wi), R(0));
        if (ct <= R(0)) break;
        throughput = throughput * scale(smp.f, ct / rmax(smp.pdf, R(1.0e-6)));
      } else {
        throughput = throughput * scale(smp.f, R(1) / rmax(smp.pdf, R(1.0e-6)));
      }
      throughput = clamp_luma(throughput, R(8));
      if (smp.delta) {
        have_prev = false;
      } else {
        have_prev = true;
        prev_pdf = rmax(smp.pdf, R(1.0e-6));
        prev_ctx = c;
        prev_mat = m;
      }
      if (bounce >= 2) {
        R pr = rclamp(luminance(throughput), R(0.05), R(0.98));
        if (R(rng.next_f32()) > pr) break;
        throughput = scale(throughput, R(1) / pr);
      }
      dir = normalize(smp.wi);
      if (smp.transmission && !smp.thin_walled) {
        medium = transition(m, front, medium);
        medium.ior = rclamp(smp.next_ior, R(1), R(3));
        origin = offset_origin(h.pos, c.hit_normal, dir, eps * R(8));
      } else {
        origin = offset_origin(h.pos, c.hit_normal, dir, eps);
      }
    }
    return radiance;
  }

  // trace_ray_recursive (ray.rs:3-39)
  Sp<R> trace(V<R> o, V<R> d, Medium<R> med, uint32_t depth, uint64_t* evals) const {
    if (depth >= max_depth_) return black<R>();
    R min_t = depth == 0 ? R(0) : R(op_.epsilon) * R(2);
    Hit<R> h;
    if (!raymarch(A, o, d, op_, min_t, R(op_.max_dist), &h, evals)) {
      return attenuate(environment(d), med, R(op_.max_dist));
    }
    V<R> view = normalize(d * R(-1));
    // make_shading_context (R:7875-7911); front_face as raymarch_hit (R:4122)
    const bool front = dot(h.normal, d) < R(0);
    const HookCtx hc{h.pos, front ? normalize(h.normal) : normalize(h.normal * R(-1)), view, front ? R(1) : R(0)};
    Mat<R> ma, mb;
    R t;
    int root = resolve_root(h);
    if (split_material(root, h.pos, hc, &ma, &mb, &t)) {
      Sp<R> a = trace_hit(h, d, med, depth, ma, evals);
      Sp<R> b = trace_hit(h, d, med, depth, mb, evals);
      return lerp_sp(a, b, t);
    }
    Mat<R> m;
    if (!material_from_node(root, h.pos, hc, &m)) m = material_for_id<R>(S.desc(), h.mat);
    return trace_hit(h, d, med, depth, m, evals);
  }

 private:
  const Scene<R>& S;
  const Accel<R>& A;
  Opts op_;
  uint32_t max_depth_;

  Sp<R> env_radiance() const {  // R:4318-4326 over path lights
    Sp<R> s = black<R>();
    const ft_scene_desc& d = S.desc();
    bool any = false;
    for (uint32_t i = 0; i < d.n_lights; ++i)
      if (d.lights[i].kind == FT_LIGHT_ENV) {
        s = s + sp(R(d.lights[i].intensity[0]), R(d.lights[i].intensity[1]), R(d.lights[i].intensity[2]));
        any = true;
      }
    (void)any;
    return s;
  }

  // environment_color (R:4328-4333) with the env_radiance fallback
  Sp<R> environment(V<R> dir) const {
    const ft_scene_desc& d = S.desc();
    if (d.environment_program >= 0) {
      V<R> out;
      S.run_program(d.environment_program, &dir, &out);
      return sp(out.x, out.y, out.z);
    }
    return env_radiance();
  }

  static Sp<R> attenuate(Sp<R> c, const Medium<R>& m, R dist) {  // apply_medium_attenuation (R:5121-5123)
    return c * medium_transmittance(m, dist);
  }

  // estimate_node_normal (R:4554-4570)
  V<R> node_normal(int idx, V<R> p, R eps) const {
    R e = rmax(eps, R(1.0e-5));
    V<R> k1 = mk(R(1), R(-1), R(-1)), k2 = mk(R(-1), R(-1), R(1)), k3 = mk(R(-1), R(1), R(-1)),
         k4 = mk(R(1), R(1), R(1));
    V<R> n = k1 * S.info(idx, p + k1 * e).d + k2 * S.info(idx, p + k2 * e).d + k3 * S.info(idx, p + k3 * e).d +
             k4 * S.info(idx, p + k4 * e).d;
    return len(n) > R(1.0e-6) ? normalize(n) : mk(R(0), R(1), R(0));
  }

  static bool blend_kind(int k, bool* diff, R* radius, const ft_node& n) {
    *diff = false;
    switch (k) {
      case FT_NODE_UNION_ROUND: case FT_NODE_UNION_CHAMFER: case FT_NODE_UNION_SOFT: case FT_NODE_INTERSECT_ROUND:
      case FT_NODE_INTERSECT_CHAMFER: case FT_NODE_UNION_COLUMNS: case FT_NODE_UNION_STAIRS:
      case FT_NODE_INTERSECT_COLUMNS: case FT_NODE_INTERSECT_STAIRS:
        *radius = R(n.f[0]);
        return true;
      case FT_NODE_DIFF_ROUND: case FT_NODE_DIFF_CHAMFER: case FT_NODE_DIFF_COLUMNS: case FT_NODE_DIFF_STAIRS:
      case FT_NODE_PIPE: case FT_NODE_ENGRAVE:
        *diff = true;
        *radius = R(n.f[0]);
        return true;
      case FT_NODE_GROOVE: case FT_NODE_TONGUE:
        *diff = true;
        *radius = rmax(R(n.f[0]), R(n.f[1]));
        return true;
      default: return false;
    }
  }

  R blend_t(const ft_node& n, V<R> p, bool diff, R radius) const {
    Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
    R k = rmax(std::fabs(radius), R(1.0e-6));
    if (diff) return smoothstepf(R(0), R(1), R(0.5) + R(0.5) * (((-r.d) - l.d) / k));
    return smoothstepf(R(0), R(1), R(0.5) + R(0.5) * ((l.d - r.d) / k));
  }

  // resolve_surface_normal_from_node (R:4462-4527) / blend_surface_normals (R:4529-4552)
  bool surface_normal(int idx, V<R> p, R eps, V<R>* out) const {
    const ft_node& n = S.node(idx);
    if (n.kind <= FT_NODE_NOISE || n.kind == FT_NODE_CUSTOM) {  // primitives, Custom and modifiers
      *out = node_normal(idx, p, eps);
      return true;
    }
    switch (n.kind) {
      case FT_NODE_UNION: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return surface_normal(l.d <= r.d ? n.a : n.b, p, eps, out);
      }
      case FT_NODE_INTERSECT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return surface_normal(l.d >= r.d ? n.a : n.b, p, eps, out);
      }
      case FT_NODE_SUBTRACT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        if (l.d >= -r.d) return surface_normal(n.a, p, eps, out);
        if (!surface_normal(n.b, p, eps, out)) return false;
        *out = *out * R(-1);
        return true;
      }
      case FT_NODE_SLICE:
      case FT_NODE_SMOOTH: return surface_normal(n.a, p, eps, out);
      default: break;
    }
    bool diff;
    R radius;
    blend_kind(n.kind, &diff, &radius, n);
    Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
    (void)l;
    (void)r;
    V<R> left, right;
    if (!surface_normal(n.a, p, eps, &left) || !surface_normal(n.b, p, eps, &right)) return false;
    R t = blend_t(n, p, diff, radius);
    if (diff) right = right * R(-1);
    V<R> m = left * (R(1) - t) + right * t;
    if (len(m) > R(1.0e-6)) *out = normalize(m);
    else *out = t < R(0.5) ? left : right;
    return true;
  }

  struct HookCtx {
    V<R> pos, normal, view;
    R front;
  };

  // resolve_leaf_material (R:7164-7600) for a leaf primitive: the colour,
  // roughness, IOR and thin_walled hooks of its material evaluated on the
  // hit in the primitive's frame (to_local with its transform, R:7172-7177);
  // roughness clamped to [0, 1], IOR to [1, 3] and neither IOR nor
  // thin_walled for a Metal (R:7472-7530); a numeric colour grey.
  Mat<R> leaf_material(const ft_node& n, const HookCtx& hc) const {
    Mat<R> m = material_for_id<R>(S.desc(), n.material_id);
    const ft_scene_desc& d = S.desc();
    if (d.n_materials == 0) return m;
    const ft_material& fm = d.materials[n.material_id < d.n_materials ? n.material_id : 0];
    bool any = fm.color_program >= 0 || fm.roughness_program >= 0 || fm.ior_program >= 0 || fm.thin_walled_program >= 0;
    for (int k = FT_HOOK_EMISSION_COLOR; k <= FT_HOOK_COAT_MASK; ++k) any = any || fm.hook_program[k] >= 0;
    for (int k = FT_HOOK_MEDIUM_IOR; k <= FT_HOOK_MEDIUM_DENSITY; ++k) any = any || fm.hook_program[k] >= 0;
    if (!any) return m;
    const R obj = R(n.object_id), mid = R(n.material_id);
    V<R> args[FT_MATERIAL_HOOK_PARAMS] = {hc.pos, S.to_local(hc.pos, n), hc.normal, hc.view,
                                          mk(hc.front, hc.front, hc.front), mk(obj, obj, obj), mk(mid, mid, mid)};
    V<R> o;
    if (fm.color_program >= 0) {
      S.run_program(fm.color_program, args, &o);
      m.p.color = d.programs[fm.color_program].result_is_vec3 ? sp(o.x, o.y, o.z) : sp(o.x, o.x, o.x);
    }
    if (fm.roughness_program >= 0) {
      S.run_program(fm.roughness_program, args, &o);
      m.p.roughness = rclamp(o.x, R(0), R(1));
    }
    if (fm.kind != FT_MAT_METAL && fm.ior_program >= 0) {
      S.run_program(fm.ior_program, args, &o);
      m.p.ior = rclamp(o.x, R(1), R(3));
    }
    if (fm.kind != FT_MAT_METAL && fm.thin_walled_program >= 0) {
      S.run_program(fm.thin_walled_program, args, &o);
      m.p.thin_walled = o.x >= R(0.5);
    }
    // The further property hooks (R:7258-7470): emission for every
    // definition; metallic, specular, specular_weight, transmission and the
    // coat (compiled for Standard / Layered definitions only), the coat's
    // colour, roughness and IOR replacing the specular colour, clearcoat
    // roughness and IOR and its weight x mask the clearcoat.
    const int32_t* hp = fm.hook_program;
    auto num = [&](int slot) {
      S.run_program(hp[slot], args, &o);
      return o.x;
    };
    auto colour = [&](int slot) {
      S.run_program(hp[slot], args, &o);
      return d.programs[hp[slot]].result_is_vec3 ? sp(o.x, o.y, o.z) : sp(o.x, o.x, o.x);
    };
    if (hp[FT_HOOK_EMISSION_COLOR] >= 0) m.p.emission_color = colour(FT_HOOK_EMISSION_COLOR);
    if (hp[FT_HOOK_EMISSION_STRENGTH] >= 0) m.p.emission_strength = rmax(num(FT_HOOK_EMISSION_STRENGTH), R(0));
    if (hp[FT_HOOK_METALLIC] >= 0) m.p.metallic = rclamp(num(FT_HOOK_METALLIC), R(0), R(1));
    if (hp[FT_HOOK_SPECULAR] >= 0) m.p.specular = rclamp(num(FT_HOOK_SPECULAR), R(0), R(1));
    if (hp[FT_HOOK_SPECULAR_WEIGHT] >= 0) m.p.specular_weight = rclamp(num(FT_HOOK_SPECULAR_WEIGHT), R(0), R(1));
    if (hp[FT_HOOK_TRANSMISSION] >= 0) m.p.transmission = rclamp(num(FT_HOOK_TRANSMISSION), R(0), R(1));
    if (hp[FT_HOOK_COAT_COLOR] >= 0) m.p.specular_color = colour(FT_HOOK_COAT_COLOR);
    if (hp[FT_HOOK_COAT_ROUGHNESS] >= 0) m.p.clearcoat_roughness = rclamp(num(FT_HOOK_COAT_ROUGHNESS), R(0), R(1));
    if (hp[FT_HOOK_COAT_IOR] >= 0) m.p.ior = rclamp(num(FT_HOOK_COAT_IOR), R(1), R(3));
    if (hp[FT_HOOK_COAT_WEIGHT] >= 0 || hp[FT_HOOK_COAT_MASK] >= 0) {
      R w = hp[FT_HOOK_COAT_WEIGHT] >= 0 ? rclamp(num(FT_HOOK_COAT_WEIGHT), R(0), R(1)) : m.p.clearcoat;
      R k = hp[FT_HOOK_COAT_MASK] >= 0 ? rclamp(num(FT_HOOK_COAT_MASK), R(0), R(1)) : R(1);
      m.p.clearcoat = rclamp(w * k, R(0), R(1));
    }
    // `fn medium(ctx)`: runtime_medium.or(base.medium) with medium_from_value's
    // defaults and clamps (R:7217-7226, R:6834-6845)
    if (hp[FT_HOOK_MEDIUM_IOR] >= 0 || hp[FT_HOOK_MEDIUM_ABSORPTION] >= 0 || hp[FT_HOOK_MEDIUM_DENSITY] >= 0) {
      m.p.has_medium = true;
      m.p.medium_ior = hp[FT_HOOK_MEDIUM_IOR] >= 0 ? rclamp(num(FT_HOOK_MEDIUM_IOR), R(1), R(3)) : R(1);
      m.p.medium_absorption = hp[FT_HOOK_MEDIUM_ABSORPTION] >= 0 ? colour(FT_HOOK_MEDIUM_ABSORPTION) : sp(R(1), R(1), R(1));
      m.p.medium_density = hp[FT_HOOK_MEDIUM_DENSITY] >= 0 ? rmax(num(FT_HOOK_MEDIUM_DENSITY), R(0)) : R(0);
    }
    return m;
  }

  int resolve_root(const Hit<R>& h) const {
    if (g_resolve_mode == 1) {
      const int leaf = S.object_leaf(h.obj);
      if (leaf >= 0) return leaf;
    }
    return S.desc().root;
  }

  // ---------------------------------------------------------------- BSDF context and hooks
  // The BSDF context of a hit: the geometric normal through the hit
  // material's bump and normal hooks.
  BsdfCtx bsdf_context(const Hit<R>& h, bool front, V<R> geometric_normal, V<R> view_dir, R current_ior) const {
    BsdfCtx c;
    c.pos = h.pos;
    int ni = S.object_node(h.obj);
    c.local = ni >= 0 ? S.to_local(h.pos, S.node(ni)) : h.pos;
    c.normal = geometric_normal;
    c.wo = normalize(view_dir);
    c.front = front ? R(1) : R(0);
    c.obj = R(h.obj);
    c.mat = R(h.mat);
    c.current_ior = current_ior;
    c.normal = hooked_normal(c, view_dir, h.mat);
    return c;
  }
  // resolve_dynamic_bump then resolve_dynamic_normal (R:7749-7818) of the
  // hit's material (material_for_id, R:4418): a forward-difference gradient
  // of the bump height (step 0.01) along the normal's tangent frame, then the
  // normal hook; each normalised, turned to its input's side, dropped when
  // degenerate.
  V<R> hooked_normal(const BsdfCtx& c, V<R> view_dir, uint32_t hit_mat) const {
    const ft_scene_desc& d = S.desc();
    V<R> n = c.normal;
    if (d.n_materials == 0) return n;
    const ft_material& fm = d.materials[hit_mat < d.n_materials ? hit_mat : 0];
    const int bump = fm.hook_program[FT_HOOK_BUMP], nrm = fm.hook_program[FT_HOOK_NORMAL];
    V<R> a[FT_MATERIAL_HOOK_PARAMS] = {c.pos, c.local, n, view_dir, mk(c.front, c.front, c.front),
                                       mk(c.obj, c.obj, c.obj), mk(c.mat, c.mat, c.mat)};
    V<R> o;
    if (bump >= 0) {
      const R eps = R(0.01);
      S.run_program(bump, a, &o);
      const R center = o.x;
      V<R> up = std::fabs(n.y) < R(0.999) ? mk(R(0), R(1), R(0)) : mk(R(1), R(0), R(0));
      V<R> tangent = normalize(cross(n, up));
      V<R> bitangent = normalize(cross(n, tangent));
      a[1] = c.local + tangent * eps;
      S.run_program(bump, a, &o);
      const R dx = o.x - center;
      a[1] = c.local + bitangent * eps;
      S.run_program(bump, a, &o);
      const R dy = o.x - center;
      a[1] = c.local;
      V<R> b = normalize((n - tangent * (dx / eps)) - bitangent * (dy / eps));
      if (len(b) > R(1.0e-6)) n = dot(b, n) < R(0) ? b * R(-1) : b;
      a[2] = n;
    }
    if (nrm >= 0) {
      S.run_program(nrm, a, &o);
      V<R> b = normalize(o);
      if (len(b) > R(1.0e-6)) n = dot(b, n) < R(0) ? b * R(-1) : b;
    }
    return n;
  }
  // bsdf_context_value (R:5006-5030) as hook arguments
  static void bsdf_args(const BsdfCtx& c, V<R> wi, R u1, R u2, R u3, V<R>* a) {
    a[0] = c.pos; a[1] = c.local; a[2] = c.normal; a[3] = c.wo;
    a[4] = mk(c.front, c.front, c.front); a[5] = mk(c.obj, c.obj, c.obj); a[6] = mk(c.mat, c.mat, c.mat);
    a[7] = c.wo; a[8] = wi; a[9] = mk(c.current_ior, c.current_ior, c.current_ior);
    a[10] = mk(u1, u1, u1); a[11] = mk(u2, u2, u2); a[12] = mk(u3, u3, u3);
  }
  int bsdf_hook(const Mat<R>& m, int slot) const {
    const int dyn = dominant_params(m).dyn;
    return dyn >= 0 && S.desc().n_materials ? S.desc().materials[dyn].hook_program[slot] : -1;
  }
  // eval_bsdf (R:4905-4920)
  Sp<R> bsdf_eval(const Mat<R>& m, const BsdfCtx& c, V<R> wi) const {
    const int prog = bsdf_hook(m, FT_HOOK_EVAL);
    if (prog < 0) return mat_eval(m, c.normal, wi, c.wo);
    V<R> a[FT_BSDF_HOOK_PARAMS], o;
    bsdf_args(c, wi, R(0), R(0), R(0), a);
    S.run_program(prog, a, &o);
    return S.desc().programs[prog].result_is_vec3 ? sp(o.x, o.y, o.z) : sp(o.x, o.x, o.x);
  }
 public:
  // Test probe (oracle_bsdf_hit): the context of one hit with the given
  // geometric normal, and the hooks of the material resolved at the hit
  // (resolve_material_at_hit, R:6926-6935).
  int bsdf_probe(const Hit<R>& h, bool front, V<R> gn, V<R> view, R current_ior, V<R> wi, const float* u,
                 float* out) const {
    const HookCtx hc{h.pos, gn, normalize(view), front ? R(1) : R(0)};
    Mat<R> m;
    if (!material_from_node(S.desc().root, h.pos, hc, &m)) m = material_for_id<R>(S.desc(), h.mat);
    const BsdfCtx c = bsdf_context(h, front, gn, view, current_ior);
    const Sp<R> f = bsdf_eval(m, c, wi);
    const R pdf = bsdf_pdf(m, c, wi);
    SampleInputT<R> in{front, current_ior, R(u[0]), R(u[1]), R(u[2])};
    const BsdfSampleT<R> smp = bsdf_sample(m, c, in);
    const float vals[19] = {float(c.normal.x), float(c.normal.y), float(c.normal.z), float(f.r), float(f.g),
                            float(f.b), float(pdf), float(smp.wi.x), float(smp.wi.y), float(smp.wi.z),
                            float(smp.f.r), float(smp.f.g), float(smp.f.b), float(smp.pdf), smp.delta ? 1.0f : 0.0f,
                            smp.apply_cos ? 1.0f : 0.0f, smp.transmission ? 1.0f : 0.0f,
                            smp.thin_walled ? 1.0f : 0.0f, float(smp.next_ior)};
    for (int k = 0; k < 19; ++k) out[k] = vals[k];
    return 0;
  }

 private:

  // pdf_bsdf (R:4922-4933)
  R bsdf_pdf(const Mat<R>& m, const BsdfCtx& c, V<R> wi) const {
    const int prog = bsdf_hook(m, FT_HOOK_PDF);
    if (prog < 0) return mat_pdf(m, c.normal, wi, c.wo);
    V<R> a[FT_BSDF_HOOK_PARAMS], o;
    bsdf_args(c, wi, R(0), R(0), R(0), a);
    S.run_program(prog, a, &o);
    return rmax(o.x, R(0));
  }
  // sample_bsdf_lobe (R:4869-4903) with sample_bsdf_ft / bsdf_sample_from_value
  // (R:4934-4950, R:5032-5060)
  BsdfSampleT<R> bsdf_sample(const Mat<R>& m, const BsdfCtx& c, const SampleInputT<R>& in) const {
    const int dyn = dominant_params(m).dyn;
    const int32_t* hp = dyn >= 0 && S.desc().n_materials ? S.desc().materials[dyn].hook_program : nullptr;
    if (!hp || hp[FT_HOOK_SAMPLE_WI] < 0 || hp[FT_HOOK_SAMPLE_F] < 0) return mat_sample(m, c.normal, c.wo, in);
    V<R> a[FT_BSDF_HOOK_PARAMS], o;
    bsdf_args(c, c.normal, in.u1, in.u2, in.u3, a);
    auto num = [&](int slot, R dflt) {
      if (hp[slot] < 0) return dflt;
      S.run_program(hp[slot], a, &o);
      return o.x;
    };
    BsdfSampleT<R> r;
    S.run_program(hp[FT_HOOK_SAMPLE_WI], a, &o);
    r.wi = o;
    S.run_program(hp[FT_HOOK_SAMPLE_F], a, &o);
    r.f = S.desc().programs[hp[FT_HOOK_SAMPLE_F]].result_is_vec3 ? sp(o.x, o.y, o.z) : sp(o.x, o.x, o.x);
    r.pdf = rmax(num(FT_HOOK_SAMPLE_PDF, R(0)), R(0));
    r.delta = num(FT_HOOK_SAMPLE_DELTA, R(0)) >= R(0.5);
    r.apply_cos = num(FT_HOOK_SAMPLE_APPLY_COS, R(1)) >= R(0.5);
    r.transmission = num(FT_HOOK_SAMPLE_TRANSMISSION, R(0)) >= R(0.5);
    r.thin_walled = num(FT_HOOK_SAMPLE_THIN_WALLED, R(0)) >= R(0.5);
    r.next_ior = rclamp(num(FT_HOOK_SAMPLE_NEXT_IOR, R(1)), R(1), R(3));
    return r;
  }

  // resolve_material_from_node (R:6945-7050) / blend_node_materials (R:7093-7113)
  bool material_from_node(int idx, V<R> p, const HookCtx& hc, Mat<R>* out) const {
    const ft_node& n = S.node(idx);
    if (n.kind <= FT_NODE_EXTRUDE_POLYGON || n.kind == FT_NODE_CUSTOM) {
      *out = leaf_material(n, hc);
      return true;
    }
    switch (n.kind) {
      case FT_NODE_DOMAIN: case FT_NODE_DISTANCE_POST: case FT_NODE_NOISE: case FT_NODE_SLICE: case FT_NODE_SMOOTH:
        return material_from_node(n.a, p, hc, out);
      case FT_NODE_UNION: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return material_from_node(l.d <= r.d ? n.a : n.b, p, hc, out);
      }
      case FT_NODE_INTERSECT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return material_from_node(l.d >= r.d ? n.a : n.b, p, hc, out);
      }
      case FT_NODE_SUBTRACT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return material_from_node(l.d >= -r.d ? n.a : n.b, p, hc, out);
      }
      default: break;
    }
    bool diff;
    R radius;
    blend_kind(n.kind, &diff, &radius, n);
    Mat<R> left, right;
    if (!material_from_node(n.a, p, hc, &left) || !material_from_node(n.b, p, hc, &right)) return false;
    *out = blend_materials(left, right, blend_t(n, p, diff, radius));
    return true;
  }

  // resolve_split_material_from_node (R:7052-7091)
  bool split_material(int idx, V<R> p, const HookCtx& hc, Mat<R>* a, Mat<R>* b, R* t) const {
    const ft_node& n = S.node(idx);
    switch (n.kind) {
      case FT_NODE_UNION: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return split_material(l.d <= r.d ? n.a : n.b, p, hc, a, b, t);
      }
      case FT_NODE_INTERSECT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return split_material(l.d >= r.d ? n.a : n.b, p, hc, a, b, t);
      }
      case FT_NODE_SUBTRACT: {
        Info<R> l = S.info(n.a, p), r = S.info(n.b, p);
        return split_material(l.d >= -r.d ? n.a : n.b, p, hc, a, b, t);
      }
      case FT_NODE_SMOOTH:
      case FT_NODE_NOISE: return split_material(n.a, p, hc, a, b, t);
      default: break;
    }
    bool diff;
    R radius;
    if (!blend_kind(n.kind, &diff, &radius, n)) return false;
    if (!material_from_node(n.a, p, hc, a) || !material_from_node(n.b, p, hc, b)) return false;
    *t = blend_t(n, p, diff, radius);
    return true;
  }

  // offset_ray_origin (R:5067-5078)
  static V<R> offset_origin(V<R> pos, V<R> gn, V<R> dir, R eps) {
    V<R> n = len(gn) > R(1.0e-8) ? normalize(gn) : normalize(dir);
    R sign = dot(dir, n) >= R(0) ? R(1) : R(-1);
    V<R> no = n * (sign * rmax(eps * R(16), R(2.0e-4)));
    R step = rmax(eps * R(8), R(1.0e-4));
    return pos + no + normalize(dir) * step;
  }

  // shadow_visibility (R:4706-4733)
  R shadow(V<R> o, V<R> d, R max_t, uint64_t* evals) const {
    R eps = R(op_.epsilon);
    R t = eps * R(2);
    R vis = R(1);
    for (int i = 0; i < 80; ++i) {
      if (t >= max_t) return rclamp(vis, R(0), R(1));
      V<R> p = o + d * t;
      R lower = std::fabs(A.lower_bound(p));
      R h;
      if (lower > rmax(eps * R(8), R(0.02))) {
        h = lower;
      } else {
        h = std::fabs(A.distance(p));
        ++*evals;
      }
      if (h < eps * R(4)) return R(0);
      vis = rmin(vis, rclamp(R(10) * h / t, R(0), R(1)));
      t += rmax(h, eps * R(2));
    }
    return rclamp(vis, R(0), R(1));
  }

  // Light::sample_li_indexed (render_api.rs:172-259)
  void sample_light(const ft_light& L, V<R> p, uint32_t idx, uint32_t count, V<R>* wi, Sp<R>* rad, R* dist) const {
    Sp<R> inten = sp(R(L.intensity[0]), R(L.intensity[1]), R(L.intensity[2]));
    V<R> lp = mk(R(L.position[0]), R(L.position[1]), R(L.position[2]));
    if (L.kind == FT_LIGHT_ENV) {
      *wi = mk(R(0), R(1), R(0));
      *rad = inten;
      *dist = std::numeric_limits<R>::infinity();
      return;
    }
    V<R> target = lp;
    if (L.kind == FT_LIGHT_SPHERE && R(L.radius) > R(1.0e-5)) {
      V<R> nrm = normalize(p - lp);
      V<R> up = std::fabs(nrm.y) < R(0.99) ? mk(R(0), R(1), R(0)) : mk(R(1), R(0), R(0));
      V<R> tangent = normalize(cross(nrm, up));
      V<R> bit = normalize(cross(tangent, nrm));
      uint32_t n = std::max(count, 1u);
      R u = (R(idx) + R(0.5)) / R(n);
      uint32_t bits = idx;
      bits = (bits >> 16) | (bits << 16);
      bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
      bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
      bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
      bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
      R v = R(float(bits) * 2.3283064e-10f);
      R sx = R(2) * u - R(1), sy = R(2) * v - R(1);
      R dx = 0, dy = 0;
      if (!(std::fabs(sx) <= R(1.1920929e-7) && std::fabs(sy) <= R(1.1920929e-7))) {
        R rr, th;
        if (std::fabs(sx) > std::fabs(sy)) {
          rr = sx;
          th = R(0.78539816339744830962) * (sy / sx);
        } else {
          rr = sy;
          th = R(1.57079632679489661923) - R(0.78539816339744830962) * (sx / sy);
        }
        dx = rr * std::cos(th);
        dy = rr * std::sin(th);
      }
      target = lp + tangent * (dx * R(L.radius)) + bit * (dy * R(L.radius));
    }
    V<R> to = target - p;
    R dd = rmax(len(to), R(1.0e-4));
    R att = R(1) / (dd * dd);
    *wi = to * (R(1) / dd);
    *rad = scale(inten, att);
    *dist = dd;
  }

  // shade_color (R:4217-4276)
  Sp<R> shade(const Mat<R>& mat, const Hit<R>& h, bool front, const BsdfCtx& bc, uint64_t* evals) const {
    const V<R> n_shade = bc.normal;
    const ft_scene_desc& d = S.desc();
    if (d.n_lights == 0) return sp(R(1), R(1), R(1));
    V<R> n = normalize(n_shade);
    V<R> gn = front ? normalize(h.normal) : normalize(h.normal * R(-1));
    Sp<R> color = black<R>();
    R eps = R(op_.epsilon);
    for (uint32_t li = 0; li < d.n_lights; ++li) {
      const ft_light& L = d.lights[li];
      uint32_t samples = L.kind == FT_LIGHT_SPHERE ? std::max(L.samples, 1u) : 1u;
      R inv = R(1) / R(samples);
      for (uint32_t s = 0; s < samples; ++s) {
        V<R> wi;
        Sp<R> rad;
        R dist;
        sample_light(L, h.pos, s, samples, &wi, &rad, &dist);
        wi = normalize(wi);
        R ndotl = n.x * wi.x + n.y * wi.y + n.z * wi.z;
        if (ndotl <= R(0)) continue;
        V<R> so = offset_origin(h.pos, gn, wi, eps);
        R max_t = std::isfinite(dist) ? rmax(dist - eps * R(8), R(0)) : R(op_.max_dist);
        if (max_t <= R(0)) continue;
        R vis = shadow(so, wi, max_t, evals);
        if (vis <= R(0)) continue;
        // eval_bsdf passes the context normal as stored (R:4905-4919)
        Sp<R> f = bsdf_eval(mat, bc, wi);
        color = color + scale(f * rad, ndotl * vis * inv);
      }
    }
    return color;
  }

  static R fresnel_dielectric(R ci, R eta_i, R eta_t) {  // R:5188-5204
    R ei = rmax(eta_i, R(1.0e-4)), et = rmax(eta_t, R(1.0e-4));
    if (std::fabs(ei - et) < R(1.0e-6)) return R(0);
    ci = rclamp(ci, R(0), R(1));
    R eta = ei / et;
    R sin2 = eta * eta * (R(1) - ci * ci);
    if (sin2 >= R(1)) return R(1);
    R ct = std::sqrt(R(1) - sin2);
    R rs = ((ei * ci) - (et * ct)) / rmax((ei * ci) + (et * ct), R(1.0e-6));
    R rp = ((et * ci) - (ei * ct)) / rmax((et * ci) + (ei * ct), R(1.0e-6));
    return R(0.5) * (rs * rs + rp * rp);
  }

  // trace_hit_with_material (ray.rs:41-222)
  Sp<R> trace_hit(const Hit<R>& h, V<R> dir, Medium<R> med, uint32_t depth, const Mat<R>& mat,
                  uint64_t* evals) const {
    bool front = dot(h.normal, dir) < R(0);
    V<R> normal = front ? normalize(h.normal) : normalize(h.normal * R(-1));
    V<R> wo = normalize(dir * R(-1));
    // build_bsdf_context: tree-resolved geometric normal (epsilon 1e-4)
    V<R> gnode;
    V<R> shading_n = normal;
    if (surface_normal(resolve_root(h), h.pos, R(1.0e-4), &gnode)) {
      gnode = front ? gnode : gnode * R(-1);
      shading_n = normalize(gnode);
    }
    // the bump and normal hooks of the hit's material, and the BSDF context
    const BsdfCtx bc = bsdf_context(h, front, shading_n, dir * R(-1), med.ior);
    shading_n = bc.normal;
    Params<R> P = dominant_params(mat);
    R rough = rclamp(P.roughness, R(0), R(1));
    int model = dominant_model(mat);
    R transmission, ior, specular_strength, metallic, clearcoat;
    bool thin;
    Sp<R> spec_color, base_color;
    switch (model) {
      case kStandard:
        transmission = rclamp(P.transmission, R(0), R(1));
        ior = rclamp(P.ior, R(1), R(3));
        thin = P.thin_walled;
        spec_color = P.specular_color;
        base_color = P.color;
        metallic = rclamp(P.metallic, R(0), R(1));
        clearcoat = rclamp(P.clearcoat, R(0), R(1));
        specular_strength = rclamp(P.specular * P.specular_weight, R(0), R(1));
        break;
      case kLambert:
        transmission = 0; ior = 1; thin = false; spec_color = black<R>(); base_color = P.color;
        metallic = 0; clearcoat = 0; specular_strength = 0;
        break;
      case kMetal:
        transmission = 0; ior = 1; thin = false; spec_color = P.color; base_color = P.color;
        metallic = 1; clearcoat = 0; specular_strength = 1;
        break;
      default:  // dielectric
        transmission = 1; ior = rclamp(P.ior, R(1), R(3)); thin = P.thin_walled; spec_color = sp(R(1), R(1), R(1));
        base_color = P.color; metallic = 0; clearcoat = 0; specular_strength = 1;
        break;
    }
    R eta_i, eta_t, next_ior;
    if (thin) { eta_i = 1; eta_t = 1; next_ior = med.ior; }
    else if (front) { eta_i = med.ior; eta_t = ior; next_ior = ior; }
    else { eta_i = med.ior; eta_t = 1; next_ior = 1; }
    V<R> gn = normal;  // geometric normal (hit normal oriented to the viewer)
    R cosv = std::fabs(dot(normal, wo));
    R fresnel;
    if (transmission > R(1.0e-4)) {
      fresnel = fresnel_dielectric(cosv, eta_i, eta_t);
    } else {
      R f0 = rclamp(f0_from_ior(ior), R(0), R(1));
      R x = R(1) - rclamp(cosv, R(0), R(1));
      R m5 = x * x * x * x * x;
      fresnel = rclamp(f0 + (R(1) - f0) * m5, R(0), R(1));
    }
    R reflect_w;
    if (transmission > R(1.0e-4)) {
      reflect_w = rclamp(fresnel, R(0), R(1));
    } else {
      R base = metallic > R(0.5) ? R(1) : rclamp(specular_strength, R(0), R(1));
      reflect_w = rclamp(base * fresnel + metallic * R(0.8) + clearcoat * R(0.2), R(0), R(1));
    }
    R local_w = rclamp((R(1) - transmission) * (R(1) - reflect_w), R(0), R(1));
    Sp<R> color = scale(shade(mat, h, front, bc, evals), local_w);
    color = color + emission(mat);
    R eps = R(op_.epsilon);
    if (reflect_w > R(1.0e-4)) {
      V<R> rd = normalize(dir - normal * (R(2) * dot(dir, normal)));
      Sp<R> refl;
      if (transmission > R(1.0e-4) && rough > R(0.06)) {
        // trace_rough_dielectric_reflection (ray.rs:296-322)
        refl = lobe_average(h.pos, gn, rd, med, depth, rough, rough_reflection_samples(rough), evals);
      } else {
        V<R> ro = offset_origin(h.pos, gn, rd, eps * (R(1) + rough * R(6)));
        refl = trace(ro, rd, med, depth + 1, evals);
      }
      Sp<R> tint = lerp_sp(spec_color, base_color, rclamp(metallic, R(0), R(1)));
      color = color + scale(refl * tint, reflect_w);
    }
    if (transmission > R(1.0e-4)) {
      Medium<R> next = med;
      if (!thin) next = transition(mat, front, med);
      next.ior = rclamp(next_ior, R(1), R(3));
      Sp<R> refr = black<R>();
      V<R> td;
      if (refract_dir(dir, normal, eta_i / eta_t, &td)) {
        if (rough > R(0.06)) {
          // trace_rough_dielectric_refraction (ray.rs:324-352)
          refr = lobe_average(h.pos, gn, normalize(td), next, depth, rough, rough_refraction_samples(rough), evals);
        } else {
          V<R> to = offset_origin(h.pos, gn, td, eps * (R(8) + rough * R(12)));
          refr = trace(to, normalize(td), next, depth + 1, evals);
        }
      }
      if (!(refr.r == R(0) && refr.g == R(0) && refr.b == R(0))) {
        R tt = rclamp(transmission, R(0), R(1));
        Sp<R> tint = sp(R(1) - (R(1) - rclamp(base_color.r, R(0), R(1))) * tt,
                        R(1) - (R(1) - rclamp(base_color.g, R(0), R(1))) * tt,
                        R(1) - (R(1) - rclamp(base_color.b, R(0), R(1))) * tt);
        color = color + scale(refr * tint, transmission * (R(1) - fresnel));
      }
    }
    return attenuate(color, med, h.t);
  }

  static bool refract_dir(V<R> inc, V<R> nrm, R eta, V<R>* out) {  // R:5080-5095
    V<R> i = normalize(inc);
    V<R> n = normalize(nrm);
    R cosi = rclamp(dot(i, n), R(-1), R(1));
    if (cosi > R(0)) n = n * R(-1);
    else cosi = -cosi;
    R sin2 = eta * eta * (R(1) - cosi * cosi);
    if (sin2 > R(1)) return false;
    R cost = std::sqrt(R(1) - sin2);
    *out = normalize(i * eta + n * (eta * cosi - cost));
    return true;
  }

  static Medium<R> transition(const Mat<R>& m, bool front, Medium<R> cur) {  // R:5147-5166
    return transition_medium(m, front, cur);
  }
};

// spectrum_to_rgb8_reinhard (R:5229-5239)
uint8_t reinhard_u8(float v) {
  float x = std::fmax(v, 0.0f);
  float t = x / (1.0f + x);
  float mapped = std::min(std::pow(t, 1.0f / 2.2f), 1.0f);
  return static_cast<uint8_t>(mapped * 255.0f);
}

template <class R>
int render_trace(const ft_scene_desc* desc, const ft_render_options* options, int accel, uint32_t aa,
                 uint32_t max_depth, int threads, uint32_t row_begin, uint32_t row_end, uint32_t row_step,
                 float* rgb_out, uint8_t* rgb8_out, uint64_t* evals_out, uint32_t col_begin = 0,
                 uint32_t col_step = 1, int64_t jitter_seed = -1) {
  Opts op = resolve(options);
  Scene<R> scene(*desc);
  Accel<R> acc(scene, accel);
  Camera<R> cam(*desc, op);
  Tracer<R> tracer(scene, acc, op, max_depth);
  aa = std::max(aa, 1u);
  auto offs = sample_offsets(aa);
  float aspect = static_cast<float>(op.width) / static_cast<float>(op.height);
  if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  row_step = std::max(row_step, 1u);
  row_end = std::min(row_end, op.height);
  std::vector<uint32_t> rows;
  for (uint32_t y = row_begin; y < row_end; y += row_step) rows.push_back(y);
  std::vector<uint32_t> cols = sample_columns(op.width, col_begin, col_step);
  const size_t segs = (cols.size() + kSegment - 1) / kSegment;  // work item: one row segment
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> total{0};
  auto worker = [&]() {
    uint64_t evals = 0;
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= rows.size() * segs) break;
      uint32_t y = rows[k / segs];
      size_t c0 = (k % segs) * kSegment, c1 = std::min(c0 + kSegment, cols.size());
      for (size_t ci = c0; ci < c1; ++ci) {
        const uint32_t x = cols[ci];
        Sp<float> sum = sp(0.0f, 0.0f, 0.0f);
        for (uint32_t s = 0; s < aa; ++s) {
          float px, py;
          sample_ndc(x, y, s, op.width, op.height, offs, jitter_seed, &px, &py);
          V<R> d = cam.dir(R(px * aspect), R(py));
          Sp<R> c = tracer.trace(cam.origin, d, Medium<R>::air(), 0, &evals);
          sum = sum + sp(float(c.r), float(c.g), float(c.b));
        }
        Sp<float> avg = scale(sum, 1.0f / static_cast<float>(aa));
        size_t pi = (static_cast<size_t>(y) * op.width + x) * 3;
        if (rgb_out) {
          rgb_out[pi] = avg.r;
          rgb_out[pi + 1] = avg.g;
          rgb_out[pi + 2] = avg.b;
        }
        if (rgb8_out) {
          rgb8_out[pi] = reinhard_u8(avg.r);
          rgb8_out[pi + 1] = reinhard_u8(avg.g);
          rgb8_out[pi + 2] = reinhard_u8(avg.b);
        }
      }
    }
    total.fetch_add(evals);
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (evals_out) *evals_out = total.load();
  return 0;
}

// The progressive MIS path tracer (render_pathtrace_with_accel_progressive,
// R:3974-4045): per pixel, samples 0, 1, ... each with its own XorShift64
// seeded by seed_pixel_sample and jittered, until spp or until the pixel's
// relative error falls to noise_threshold after min_spp samples
// (PixelAccumulator R:4778-4817).  Pixels are independent, so one pass per
// pixel gives the reference's result.  Outputs: the average (linear), its
// spectrum_to_rgb8 (R:5221-5227) and the sample count per pixel.
template <class R>
int render_path(const ft_scene_desc* desc, const ft_render_options* options, int accel, uint32_t spp,
                uint32_t max_bounces, uint32_t min_spp, float noise_threshold, int threads, uint32_t row_begin,
                uint32_t row_end, uint32_t row_step, uint32_t col_begin, uint32_t col_step, float* rgb_out,
                uint8_t* rgb8_out, uint32_t* count_out, uint64_t* evals_out) {
  Opts op = resolve(options);
  Scene<R> scene(*desc);
  Accel<R> acc(scene, accel);
  Camera<R> cam(*desc, op);
  Tracer<R> tracer(scene, acc, op, 1);
  spp = std::max(spp, 1u);
  max_bounces = std::max(max_bounces, 1u);
  min_spp = std::min(std::max(min_spp, 1u), spp);
  const float threshold = std::max(noise_threshold, 0.0f);
  float aspect = static_cast<float>(op.width) / static_cast<float>(op.height);
  if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  row_step = std::max(row_step, 1u);
  row_end = std::min(row_end, op.height);
  std::vector<uint32_t> rows;
  for (uint32_t y = row_begin; y < row_end; y += row_step) rows.push_back(y);
  std::vector<uint32_t> cols = sample_columns(op.width, col_begin, col_step);
  const size_t segs = (cols.size() + kSegment - 1) / kSegment;
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> total{0};
  auto worker = [&]() {
    uint64_t evals = 0;
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= rows.size() * segs) break;
      uint32_t y = rows[k / segs];
      size_t c0 = (k % segs) * kSegment, c1 = std::min(c0 + kSegment, cols.size());
      for (size_t ci = c0; ci < c1; ++ci) {
        const uint32_t x = cols[ci];
        Sp<float> sum = sp(0.0f, 0.0f, 0.0f);
        uint32_t count = 0;
        float mean = 0.0f, m2 = 0.0f;
        for (uint32_t s = 0; s < spp; ++s) {
          XorShift64 rng(seed_pixel_sample(x, y, op.width, s));
          const float jx = rng.next_f32() - 0.5f;
          const float jy = rng.next_f32() - 0.5f;
          float px = (((static_cast<float>(x) + 0.5f + jx) / static_cast<float>(op.width)) * 2.0f - 1.0f) * aspect;
          float py = 1.0f - ((static_cast<float>(y) + 0.5f + jy) / static_cast<float>(op.height)) * 2.0f;
          V<R> d = cam.dir(R(px), R(py));
          Sp<R> c = tracer.trace_path(cam.origin, d, max_bounces, rng, &evals);
          Sp<float> cs = sp(float(c.r), float(c.g), float(c.b));
          // PixelAccumulator::add_sample
          sum = sum + cs;
          count += 1;
          float xl = luminance(cs);
          float delta = xl - mean;
          mean += delta / static_cast<float>(count);
          m2 += delta * (xl - mean);
          if (threshold > 0.0f && count >= min_spp && count >= 2) {
            float n = static_cast<float>(count);
            float var = std::max(m2 / (n - 1.0f), 0.0f);
            float rel = std::sqrt(var / n) / std::max(std::fabs(mean), 1.0e-4f);
            if (rel <= threshold) break;
          }
        }
        Sp<float> avg = count ? scale(sum, 1.0f / static_cast<float>(count)) : sp(0.0f, 0.0f, 0.0f);
        size_t pi = static_cast<size_t>(y) * op.width + x;
        if (rgb_out) {
          rgb_out[3 * pi] = avg.r;
          rgb_out[3 * pi + 1] = avg.g;
          rgb_out[3 * pi + 2] = avg.b;
        }
        if (rgb8_out) {
          rgb8_out[3 * pi] = depth_to_u8(avg.r);
          rgb8_out[3 * pi + 1] = depth_to_u8(avg.g);
          rgb8_out[3 * pi + 2] = depth_to_u8(avg.b);
        }
        if (count_out) count_out[pi] = count;
      }
    }
    total.fetch_add(evals);
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (evals_out) *evals_out = total.load();
  return 0;
}

// ============================================================ differentiation
// Multi-view depth + soft silhouette and its adjoint: the definitions of
// ft_render_views / ft_render_backward (include/forgedthoughts_gb300.h),
// restated on the CPU so the GPU adjoint has an FP64 reference and finite
// differences have an FP64 forward.

// Parameter slot of every (node, field) pair; a tree's radius slot is shared
// by all union_round nodes below the node named in the layout.
struct ParamSlots {
  std::vector<int32_t> slot;  // node * 8 + field -> parameter index, -1 if none
  ParamSlots(const ft_scene_desc& d, const ft_param* ps, uint32_t n) : slot(static_cast<size_t>(d.n_nodes) * 8, -1) {
    for (uint32_t i = 0; i < n; ++i) {
      if (ps[i].node < 0 || static_cast<uint32_t>(ps[i].node) >= d.n_nodes || ps[i].field < 0 || ps[i].field > 7)
        continue;
      if (ps[i].field == FT_PARAM_RADIUS) {
        std::vector<int> stack{ps[i].node};
        while (!stack.empty()) {
          int k = stack.back();
          stack.pop_back();
          const ft_node& nd = d.nodes[k];
          if (nd.kind != FT_NODE_UNION_ROUND) continue;
          slot[static_cast<size_t>(k) * 8 + FT_PARAM_RADIUS] = static_cast<int32_t>(i);
          stack.push_back(nd.a);
          stack.push_back(nd.b);
        }
      } else {
        slot[static_cast<size_t>(ps[i].node) * 8 + ps[i].field] = static_cast<int32_t>(i);
      }
    }
  }
  int at(int node, int field) const { return slot[static_cast<size_t>(node) * 8 + field]; }
};

// adj * d(value of subtree idx at p) / d(parameters, p), accumulated.
template <class R>
struct Backprop {
  const Scene<R>& sc;
  const ParamSlots& ps;
  std::vector<R>& g;
  V<R> gp = mk(R(0), R(0), R(0));
  bool unsupported = false;

  R value(int idx, V<R> p) const { return sc.info(idx, p).d; }

  void add(int node, int field, R v) {
    int k = ps.at(node, field);
    if (k >= 0) g[k] += v;
  }

  void run(int idx, V<R> p, R adj) {
    const ft_node& n = sc.node(idx);
    switch (n.kind) {
      case FT_NODE_SPHERE:
      case FT_NODE_BOX: {
        // q = rotate_y(p - c, -rot_y) (x / z rotations are zero for parameter primitives)
        V<R> dpc = p - sc.center(n);
        R a = to_radians(-R(n.rot_deg[1])), s = std::sin(a), c = std::cos(a);
        V<R> q = mk(c * dpc.x + s * dpc.z, dpc.y, -s * dpc.x + c * dpc.z);
        V<R> dq;  // d value / d q
        if (n.kind == FT_NODE_SPHERE) {
          R l = len(q);
          dq = l > R(0) ? q * (R(1) / l) : mk(R(0), R(0), R(0));
          add(idx, FT_PARAM_S0, -adj);
        } else {
          R h[3] = {R(n.f[0]), R(n.f[1]), R(n.f[2])};
          R qv[3] = {q.x, q.y, q.z};
          R qa[3], o[3];
          for (int i = 0; i < 3; ++i) {
            qa[i] = std::fabs(qv[i]) - h[i];
            o[i] = rmax(qa[i], R(0));
          }
          R outside = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
          R dqa[3] = {R(0), R(0), R(0)};
          if (outside > R(0)) {
            for (int i = 0; i < 3; ++i) dqa[i] = o[i] / outside;
          } else {
            int m = 0;
            for (int i = 1; i < 3; ++i)
              if (qa[i] > qa[m]) m = i;
            dqa[m] = R(1);
          }
          R sg[3];
          for (int i = 0; i < 3; ++i) sg[i] = qv[i] < R(0) ? R(-1) : R(1);
          dq = mk(dqa[0] * sg[0], dqa[1] * sg[1], dqa[2] * sg[2]);
          add(idx, FT_PARAM_S0, -adj * dqa[0]);
          add(idx, FT_PARAM_S1, -adj * dqa[1]);
          add(idx, FT_PARAM_S2, -adj * dqa[2]);
        }
        // d q / d p = rotation; d value / d p = R^T dq
        V<R> dp = mk(c * dq.x - s * dq.z, dq.y, s * dq.x + c * dq.z);
        gp = gp + dp * adj;
        add(idx, FT_PARAM_CX, -adj * dp.x);
        add(idx, FT_PARAM_CY, -adj * dp.y);
        add(idx, FT_PARAM_CZ, -adj * dp.z);
        // d q / d rot_y = (q.z, 0, -q.x) * d a / d rot_y, d a / d rot_y = -pi / 180
        add(idx, FT_PARAM_ROT_Y, adj * (dq.x * q.z - dq.z * q.x) * (-pi<R>() / R(180)));
        return;
      }
      case FT_NODE_UNION_ROUND: {
        R a = value(n.a, p), b = value(n.b, p);
        R r0 = R(n.f[0]);
        R r = rmax(std::fabs(r0), R(1.0e-6));
        R ux = rmax(r - a, R(0)), uy = rmax(r - b, R(0));
        R l = std::sqrt(ux * ux + uy * uy);
        R pa, pb, pr;
        if (l > R(0)) {
          pa = ux / l;
          pb = uy / l;
          pr = R(1) - (ux + uy) / l;
        } else {
          pa = a < b ? R(1) : R(0);
          pb = a < b ? R(0) : R(1);
          pr = R(0);
        }
        if (std::fabs(r0) > R(1.0e-6)) add(idx, FT_PARAM_RADIUS, adj * pr * (r0 < R(0) ? R(-1) : R(1)));
        if (pa != R(0)) run(n.a, p, adj * pa);
        if (pb != R(0)) run(n.b, p, adj * pb);
        return;
      }
      case FT_NODE_UNION: {
        // the culled min of the Union arm: the gradient follows the winner
        Info<R> l = sc.info(n.a, p), rr = sc.info(n.b, p);
        run(l.d <= rr.d ? n.a : n.b, p, adj);
        return;
      }
      default:
        unsupported = true;
        return;
    }
  }
};

constexpr int kGoldenSteps = 40;  // golden-section steps of the silhouette minimum

template <class R>
struct ViewRay {
  bool hit = false;
  R t = R(0);      // depth (zero of f) on a hit
  R sil = R(0);
  R tm = R(0);     // position of the refined minimum on a miss
  R m = R(0);      // refined minimum value
};

template <class R>
struct ViewCamera {
  V<R> origin, forward, right, up;
  R tan_fov;
  explicit ViewCamera(const ft_view& v) {
    origin = mk(R(v.origin[0]), R(v.origin[1]), R(v.origin[2]));
    V<R> tgt = mk(R(v.target[0]), R(v.target[1]), R(v.target[2]));
    forward = normalize(tgt - origin);
    right = normalize(cross(forward, mk(R(0), R(1), R(0))));
    up = normalize(cross(right, forward));
    tan_fov = std::tan(R(0.5) * to_radians(R(v.fov_y_degrees)));
  }
  V<R> dir(uint32_t x, uint32_t y, const Opts& op) const {
    float aspect = static_cast<float>(op.width) / static_cast<float>(op.height);
    float px = ((static_cast<float>(x) + 0.5f) / static_cast<float>(op.width)) * 2.0f - 1.0f;
    float py = 1.0f - ((static_cast<float>(y) + 0.5f) / static_cast<float>(op.height)) * 2.0f;
    V<R> d = normalize(forward + right * (R(px * aspect) * tan_fov) + up * (R(py) * tan_fov));
    return normalize(d);
  }
};

template <class R>
ViewRay<R> view_ray(const Accel<R>& acc, V<R> o, V<R> d, const Opts& op, R tau) {
  ViewRay<R> out;
  R t0, t1;
  if (!ray_aabb(o, d, acc.scene_bounds, &t0, &t1)) return out;  // sil 0: nothing along the ray
  R max_t = rmin(R(op.max_dist), t1);
  R traveled = rmax(t0, R(0)), prev = traveled;
  R eps = R(op.epsilon);
  R best = std::numeric_limits<R>::infinity(), tb_prev = traveled, tb = traveled, tb_next = traveled;
  bool need_next = false;
  auto f = [&](R t) { return acc.distance(o + d * t); };
  for (uint32_t s = 0; s < op.max_steps; ++s) {
    if (traveled > max_t) break;
    R dv = f(traveled);
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
    if (std::fabs(dv) < eps) {
      R lo = prev, hi = traveled;
      for (int k = 0; k < 10; ++k) {
        R mid = R(0.5) * (lo + hi);
        if (std::fabs(f(mid)) < eps) hi = mid;
        else lo = mid;
      }
      // secant steps from the bisection bracket onto the zero of f
      R fa = f(lo), fb = f(hi);
      for (int k = 0; k < 3; ++k) {
        if (fb == fa) break;
        R tn = hi - fb * (hi - lo) / (fb - fa);
        lo = hi;
        fa = fb;
        hi = tn;
        fb = f(hi);
      }
      out.hit = true;
      out.t = hi;
      out.sil = R(1);
      return out;
    }
    prev = traveled;
    traveled += rmax(std::fabs(dv) * rclamp(R(op.step_scale), R(0.05), R(1)), rmax(eps * R(0.5), R(1.0e-5)));
  }
  if (!(best < std::numeric_limits<R>::infinity())) return out;
  // Bracket a local minimum around the smallest sample: continue the descent
  // past the end of the march while f keeps falling, then golden-section
  // search on the triple (a, x, b) with f(x) <= f(a), f(b).
  auto step_of = [&](R fv) {
    return rmax(std::fabs(fv) * rclamp(R(op.step_scale), R(0.05), R(1)), rmax(eps * R(0.5), R(1.0e-5)));
  };
  // (the samples start at the scene box, so the descent may also continue
  // towards the camera when the first sample is the smallest)
  R a = tb_prev, x = tb, fx = best;
  R b = need_next ? x + step_of(fx) : tb_next;
  R fb = f(b);
  for (int k = 0; k < 64 && fb < fx && b < R(op.max_dist); ++k) {
    a = x;
    x = b;
    fx = fb;
    b = x + step_of(fx);
    fb = f(b);
  }
  if (!(a < x)) a = rmax(x - step_of(fx), R(0));
  R fa = f(a);
  for (int k = 0; k < 64 && fa < fx && a > R(0); ++k) {
    b = x;
    x = a;
    fx = fa;
    a = rmax(x - step_of(fx), R(0));
    fa = f(a);
  }
  for (int k = 0; k < kGoldenSteps; ++k) {
    R u = (b - x > x - a) ? x + R(0.3819660112501051) * (b - x) : x - R(0.3819660112501051) * (x - a);
    R fu = f(u);
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
  out.sil = std::exp(-rmax(out.m, R(0)) / tau);
  return out;
}

template <class R>
int render_views(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views, const ft_render_options* options,
                 R tau, int threads, double* t_out, uint8_t* mask_out, double* sil_out, const ft_param* params,
                 uint32_t n_params, const float* dl_dt, const float* dl_dsil, double* grad_out,
                 uint32_t stride = 1, uint32_t offset = 0) {
  Opts op = resolve(options);
  stride = std::max(stride, 1u);
  offset %= stride;
  const uint32_t rows_per_view = (op.height - std::min(offset, op.height) + stride - 1) / stride;
  Scene<R> scene(*desc);
  Accel<R> acc(scene, FT_ACCEL_BVH);
  ParamSlots slots(*desc, params, n_params);
  if (threads <= 0) threads = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
  const uint64_t per_view = static_cast<uint64_t>(op.width) * op.height;
  const uint64_t rows = static_cast<uint64_t>(n_views) * rows_per_view;
  std::atomic<uint64_t> next{0};
  std::atomic<bool> bad{false};
  std::vector<std::vector<R>> partial(threads, std::vector<R>(n_params, R(0)));
  auto worker = [&](int w) {
    std::vector<R>& g = partial[w];
    for (;;) {
      uint64_t row = next.fetch_add(1);
      if (row >= rows) break;
      uint32_t v = static_cast<uint32_t>(row / rows_per_view);
      uint32_t y = offset + static_cast<uint32_t>(row % rows_per_view) * stride;
      ViewCamera<R> cam(views[v]);
      for (uint32_t x = offset; x < op.width; x += stride) {
        size_t i = v * per_view + static_cast<size_t>(y) * op.width + x;
        V<R> d = cam.dir(x, y, op);
        ViewRay<R> r = view_ray(acc, cam.origin, d, op, tau);
        if (t_out) t_out[i] = r.hit ? static_cast<double>(r.t) : 0.0;
        if (mask_out) mask_out[i] = r.hit ? 1 : 0;
        if (sil_out) sil_out[i] = static_cast<double>(r.sil);
        if (!grad_out) continue;
        R wt = dl_dt ? R(dl_dt[i]) : R(0), ws = dl_dsil ? R(dl_dsil[i]) : R(0);
        std::vector<R> gl(n_params, R(0));
        if (r.hit && wt != R(0)) {
          Backprop<R> bp{scene, slots, gl};
          bp.run(desc->root, cam.origin + d * r.t, R(1));
          if (bp.unsupported) bad = true;
          R den = dot(bp.gp, d);
          if (std::fabs(den) > R(1.0e-8))
            for (uint32_t k = 0; k < n_params; ++k) g[k] += wt * (-gl[k] / den);
        } else if (!r.hit && ws != R(0) && r.m > R(0) && r.sil > R(0)) {
          // polish the minimum's position: secant steps on grad_p f . d = 0
          auto slope = [&](R tt) {
            std::vector<R> scratch(n_params, R(0));
            Backprop<R> probe{scene, slots, scratch};
            probe.run(desc->root, cam.origin + d * tt, R(1));
            return dot(probe.gp, d);
          };
          R tm = r.tm;
          const R dt0 = R(1.0e-3) * rmax(R(1), tm);
          const R g0 = slope(tm);
          R ta = tm - dt0, tb = tm + dt0, ga = slope(ta), gb = slope(tb);
          for (int k = 0; k < 4 && gb != ga; ++k) {
            R tn = tb - gb * (tb - ta) / (gb - ga);
            tn = rmin(rmax(tn, tm - R(4) * dt0), tm + R(4) * dt0);
            ta = tb;
            ga = gb;
            tb = tn;
            gb = slope(tb);
          }
          if (std::fabs(gb) < std::fabs(g0)) tm = tb;
          Backprop<R> bp{scene, slots, gl};
          bp.run(desc->root, cam.origin + d * tm, R(1));
          if (bp.unsupported) bad = true;
          for (uint32_t k = 0; k < n_params; ++k) g[k] += ws * (-(r.sil / tau) * gl[k]);
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(worker, i);
  worker(0);
  for (auto& t : pool) t.join();
  if (grad_out) {
    for (uint32_t k = 0; k < n_params; ++k) {
      double s = 0.0;
      for (int w = 0; w < threads; ++w) s += static_cast<double>(partial[w][k]);
      grad_out[k] = s;
    }
  }
  if (bad) {
    g_error = "scene has node kinds the adjoint does not differentiate";
    return FT_ERR_UNSUPPORTED;
  }
  return 0;
}

int check_desc(const ft_scene_desc* d) {
  if (!d || d->abi_version != FT_ABI_VERSION || d->root < 0 || static_cast<uint32_t>(d->root) >= d->n_nodes) {
    g_error = "invalid scene description";
    return FT_ERR_INVALID_ARGUMENT;
  }
  return 0;
}

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_error.c_str(); }

int oracle_render_depth(const ft_scene_desc* desc, const ft_render_options* options, int accel, uint32_t aa_samples,
                        int precision, int threads, uint32_t row_begin, uint32_t row_end, uint32_t row_step,
                        float* t_out, uint8_t* mask_out, uint32_t* material_out, float* normal_out,
                        uint8_t* rgb8_out, uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_depth<double>(desc, options, accel, aa_samples, threads, row_begin, row_end, row_step, t_out,
                                mask_out, material_out, normal_out, rgb8_out, evals_out);
  return render_depth<float>(desc, options, accel, aa_samples, threads, row_begin, row_end, row_step, t_out,
                             mask_out, material_out, normal_out, rgb8_out, evals_out);
}

int oracle_distance(const ft_scene_desc* desc, int accel, int precision, const float* points, size_t n,
                    double* distance_out, uint32_t* object_out, uint32_t* material_out) {
  if (int e = check_desc(desc)) return e;
  auto run = [&](auto tag) {
    using R = decltype(tag);
    Scene<R> scene(*desc);
    Accel<R> acc(scene, accel);
    for (size_t i = 0; i < n; ++i) {
      Info<R> info = acc.distance_info(mk(R(points[3 * i]), R(points[3 * i + 1]), R(points[3 * i + 2])));
      if (distance_out) distance_out[i] = static_cast<double>(info.d);
      if (object_out) object_out[i] = info.obj;
      if (material_out) material_out[i] = info.mat;
    }
  };
  if (precision == 64) run(0.0);
  else run(0.0f);
  return 0;
}

int oracle_eval_program(const ft_scene_desc* desc, int program, int precision, const float* args, size_t n,
                        double* out) {
  if (int e = check_desc(desc)) return e;
  if (program < 0 || static_cast<uint32_t>(program) >= desc->n_programs) {
    g_error = "invalid program index";
    return FT_ERR_INVALID_ARGUMENT;
  }
  auto run = [&](auto tag) {
    using R = decltype(tag);
    Scene<R> scene(*desc);
    uint32_t np = desc->programs[program].n_params;
    for (size_t i = 0; i < n; ++i) {
      V<R> a[16];
      for (uint32_t k = 0; k < np && k < 16; ++k) {
        const float* s = args + (i * np + k) * 3;
        a[k] = mk(R(s[0]), R(s[1]), R(s[2]));
      }
      V<R> o;
      scene.run_program(program, a, &o);
      out[3 * i] = double(o.x);
      out[3 * i + 1] = double(o.y);
      out[3 * i + 2] = double(o.z);
    }
  };
  if (precision == 64) run(0.0);
  else run(0.0f);
  return 0;
}

}  // extern "C"

extern "C" int oracle_render_trace(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                   uint32_t aa_samples, uint32_t max_depth, int precision, int threads,
                                   uint32_t row_begin, uint32_t row_end, uint32_t row_step, float* rgb_out,
                                   uint8_t* rgb8_out, uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_trace<double>(desc, options, accel, aa_samples, max_depth, threads, row_begin, row_end, row_step,
                                rgb_out, rgb8_out, evals_out);
  return render_trace<float>(desc, options, accel, aa_samples, max_depth, threads, row_begin, row_end, row_step,
                             rgb_out, rgb8_out, evals_out);
}

// The depth preview / Whitted trace over every row_step-th row and
// col_step-th column (a band of a full frame for the parity tests); outputs
// are full-frame arrays of which only the sampled pixels are written.
// jitter_seed >= 0 takes the jittered AA offsets instead of the grid.
extern "C" int oracle_render_depth_strided(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                           uint32_t aa_samples, int precision, int threads, uint32_t row_begin,
                                           uint32_t row_end, uint32_t row_step, uint32_t col_begin,
                                           uint32_t col_step, int64_t jitter_seed, float* t_out,
                                           uint8_t* mask_out, uint32_t* material_out, float* normal_out,
                                           uint8_t* rgb8_out, uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_depth<double>(desc, options, accel, aa_samples, threads, row_begin, row_end, row_step, t_out,
                                mask_out, material_out, normal_out, rgb8_out, evals_out, col_begin, col_step,
                                jitter_seed);
  return render_depth<float>(desc, options, accel, aa_samples, threads, row_begin, row_end, row_step, t_out,
                             mask_out, material_out, normal_out, rgb8_out, evals_out, col_begin, col_step,
                             jitter_seed);
}

extern "C" int oracle_render_trace_strided(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                           uint32_t aa_samples, uint32_t max_depth, int precision, int threads,
                                           uint32_t row_begin, uint32_t row_end, uint32_t row_step,
                                           uint32_t col_begin, uint32_t col_step, int64_t jitter_seed,
                                           float* rgb_out, uint8_t* rgb8_out, uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_trace<double>(desc, options, accel, aa_samples, max_depth, threads, row_begin, row_end, row_step,
                                rgb_out, rgb8_out, evals_out, col_begin, col_step, jitter_seed);
  return render_trace<float>(desc, options, accel, aa_samples, max_depth, threads, row_begin, row_end, row_step,
                             rgb_out, rgb8_out, evals_out, col_begin, col_step, jitter_seed);
}

extern "C" int oracle_render_path(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                  uint32_t spp, uint32_t max_bounces, uint32_t min_spp, float noise_threshold,
                                  int precision, int threads, uint32_t row_begin, uint32_t row_end,
                                  uint32_t row_step, uint32_t col_begin, uint32_t col_step, float* rgb_out,
                                  uint8_t* rgb8_out, uint32_t* count_out, uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_path<double>(desc, options, accel, spp, max_bounces, min_spp, noise_threshold, threads, row_begin,
                               row_end, row_step, col_begin, col_step, rgb_out, rgb8_out, count_out, evals_out);
  return render_path<float>(desc, options, accel, spp, max_bounces, min_spp, noise_threshold, threads, row_begin,
                            row_end, row_step, col_begin, col_step, rgb_out, rgb8_out, count_out, evals_out);
}

// Strided pixel sample (rows row_begin, +row_step ..; columns col_begin,
// +col_step ..) of the depth march or the Whitted trace: the timed CPU
// baseline's sample of a full frame.  mode 0: depth, else trace of max_depth.
extern "C" int oracle_render_sample(const ft_scene_desc* desc, const ft_render_options* options, int accel,
                                    uint32_t aa_samples, uint32_t max_depth, int mode, int threads,
                                    uint32_t row_begin, uint32_t row_step, uint32_t col_begin, uint32_t col_step,
                                    uint64_t* evals_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0) {
    g_error = "invalid render options";
    return FT_ERR_INVALID_ARGUMENT;
  }
  const uint32_t w = options->width, h = options->height, aa = std::max(aa_samples, 1u);
  if (mode == 0) {
    std::vector<float> t(static_cast<size_t>(w) * h * aa);
    std::vector<uint8_t> m(t.size());
    return render_depth<float>(desc, options, accel, aa, threads, row_begin, h, row_step, t.data(), m.data(),
                               nullptr, nullptr, nullptr, evals_out, col_begin, col_step);
  }
  std::vector<float> rgb(static_cast<size_t>(w) * h * 3);
  return render_trace<float>(desc, options, accel, aa, max_depth, threads, row_begin, h, row_step, rgb.data(),
                             nullptr, evals_out, col_begin, col_step);
}

extern "C" int oracle_render_views(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                   const ft_render_options* options, float tau, int precision, int threads,
                                   double* t_out, uint8_t* mask_out, double* sil_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0 || !views || !(tau > 0.0f)) {
    g_error = "invalid view render arguments";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_views<double>(desc, views, n_views, options, double(tau), threads, t_out, mask_out, sil_out,
                                nullptr, 0, nullptr, nullptr, nullptr);
  return render_views<float>(desc, views, n_views, options, tau, threads, t_out, mask_out, sil_out, nullptr, 0,
                             nullptr, nullptr, nullptr);
}

// render_views over the pixels (offset + i * stride, offset + j * stride) of
// every view: a sparse sample for finite differences at full resolution.
extern "C" int oracle_render_views_strided(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                           const ft_render_options* options, float tau, int precision, int threads,
                                           uint32_t stride, uint32_t offset, double* t_out, uint8_t* mask_out,
                                           double* sil_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0 || !views || !(tau > 0.0f)) {
    g_error = "invalid view render arguments";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_views<double>(desc, views, n_views, options, double(tau), threads, t_out, mask_out, sil_out,
                                nullptr, 0, nullptr, nullptr, nullptr, stride, offset);
  return render_views<float>(desc, views, n_views, options, tau, threads, t_out, mask_out, sil_out, nullptr, 0,
                             nullptr, nullptr, nullptr, stride, offset);
}

extern "C" int oracle_render_backward(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                      const ft_render_options* options, float tau, const ft_param* params,
                                      uint32_t n_params, const float* dl_dt, const float* dl_dsil, int precision,
                                      int threads, double* grad_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0 || !views || !(tau > 0.0f) || !grad_out ||
      (n_params && !params)) {
    g_error = "invalid backward arguments";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_views<double>(desc, views, n_views, options, double(tau), threads, nullptr, nullptr, nullptr,
                                params, n_params, dl_dt, dl_dsil, grad_out);
  return render_views<float>(desc, views, n_views, options, tau, threads, nullptr, nullptr, nullptr, params, n_params,
                             dl_dt, dl_dsil, grad_out);
}

// oracle_render_backward over the pixels (offset + i * stride, offset + j *
// stride) of every view (the upstream gradients elsewhere are not read).
extern "C" int oracle_render_backward_strided(const ft_scene_desc* desc, const ft_view* views, uint32_t n_views,
                                              const ft_render_options* options, float tau, const ft_param* params,
                                              uint32_t n_params, const float* dl_dt, const float* dl_dsil,
                                              int precision, int threads, uint32_t stride, uint32_t offset,
                                              double* grad_out) {
  if (int e = check_desc(desc)) return e;
  if (!options || options->width == 0 || options->height == 0 || !views || !(tau > 0.0f) || !grad_out ||
      (n_params && !params)) {
    g_error = "invalid backward arguments";
    return FT_ERR_INVALID_ARGUMENT;
  }
  if (precision == 64)
    return render_views<double>(desc, views, n_views, options, double(tau), threads, nullptr, nullptr, nullptr,
                                params, n_params, dl_dt, dl_dsil, grad_out, stride, offset);
  return render_views<float>(desc, views, n_views, options, tau, threads, nullptr, nullptr, nullptr, params, n_params,
                             dl_dt, dl_dsil, grad_out, stride, offset);
}

extern "C" void oracle_medium_transmittance(const float medium[5], float distance, float out_rgb[3]) {
  const Medium<float> m{medium[0], sp(medium[1], medium[2], medium[3]), medium[4]};
  const Sp<float> t = medium_transmittance(m, distance);
  out_rgb[0] = t.r;
  out_rgb[1] = t.g;
  out_rgb[2] = t.b;
}

extern "C" void oracle_transition_medium(const ft_material* material, int front_face, const float current[5],
                                         float out[5]) {
  Mat<float> m;
  m.kind = material->kind;
  m.p = params_from<float>(*material);
  const Medium<float> cur{current[0], sp(current[1], current[2], current[3]), current[4]};
  const Medium<float> next = transition_medium(m, front_face != 0, cur);
  out[0] = next.ior;
  out[1] = next.absorption.r;
  out[2] = next.absorption.g;
  out[3] = next.absorption.b;
  out[4] = next.density;
}

// Test-only: the BSDF context of one hit and the BSDF hooks (or built-in
// BSDF) of the material resolved there, for the reference's unit tests of
// build_bsdf_context (R:4397-4449), eval_bsdf, pdf_bsdf and sample_bsdf_lobe
// (R:4869-4950).  hit = position (3), normal (3), front_face, object_id,
// material_id; out = shading normal (3), eval (3), pdf, then the sample: wi
// (3), f (3), pdf, delta, apply_cos, transmission, thin_walled, next_ior.
extern "C" int oracle_bsdf_hit(const ft_scene_desc* desc, const float hit[9], const float view_dir[3],
                               float current_ior, const float wi[3], const float u[3], float out[19]) {
  if (int e = check_desc(desc)) return e;
  Scene<float> scene(*desc);
  Accel<float> acc(scene, FT_ACCEL_NAIVE);
  const Opts op{1, 1, 128, 40.0f, 1.0e-3f, 0.7f, 6.0f, 45.0f};
  Tracer<float> tr(scene, acc, op, 1);
  Hit<float> h;
  h.t = 1.0f;
  h.pos = mk(hit[0], hit[1], hit[2]);
  h.normal = mk(hit[3], hit[4], hit[5]);
  h.obj = static_cast<uint32_t>(hit[7]);
  h.mat = static_cast<uint32_t>(hit[8]);
  const bool front = hit[6] >= 0.5f;
  const V<float> view = mk(view_dir[0], view_dir[1], view_dir[2]);
  const V<float> gn = front ? normalize(h.normal) : normalize(h.normal * -1.0f);
  return tr.bsdf_probe(h, front, gn, view, current_ior, mk(wi[0], wi[1], wi[2]), u, out);
}

// Test-only: where hits resolve their normal and material (g_resolve_mode).
extern "C" void oracle_set_resolve_mode(int mode) { g_resolve_mode = mode; }
