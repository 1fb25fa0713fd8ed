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
  explicit Scene(const ft_scene_desc& d) : d_(d) {}

  const ft_scene_desc& desc() const { return d_; }
  const ft_node& node(int i) const { return d_.nodes[i]; }

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

  // accel_leaf_distance_info (R:635-657); Custom leaves are not in the IR.
  Info<R> leaf_info(const Leaf<R>& l, V<R> p) const { return scene.info(l.node, p); }

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

// depth_preview_value + spectrum_to_rgb8 (R:5215-5227)
uint8_t depth_to_u8(float v) {
  float mapped = std::min(std::pow(std::fmax(v, 0.0f), 1.0f / 2.2f), 1.0f);
  return static_cast<uint8_t>(mapped * 255.0f);
}

Opts resolve(const ft_render_options* o) {
  return Opts{o->width, o->height, o->max_steps, o->max_dist, o->epsilon, o->step_scale, o->camera_z, o->fov_y_degrees};
}

template <class R>
int render_depth(const ft_scene_desc* desc, const ft_render_options* options, int accel, uint32_t aa, int threads,
                 uint32_t row_begin, uint32_t row_end, uint32_t row_step, float* t_out, uint8_t* mask_out,
                 uint32_t* mat_out, float* normal_out, uint8_t* rgb_out, uint64_t* evals_out) {
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
  std::atomic<size_t> next{0};
  std::atomic<uint64_t> total{0};
  auto worker = [&]() {
    uint64_t evals = 0;
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= rows.size()) break;
      uint32_t y = rows[k];
      for (uint32_t x = 0; x < op.width; ++x) {
        float sum = 0.0f;
        for (uint32_t s = 0; s < aa; ++s) {
          float px = ((static_cast<float>(x) + offs[s].first) / static_cast<float>(op.width)) * 2.0f - 1.0f;
          float py = 1.0f - ((static_cast<float>(y) + offs[s].second) / static_cast<float>(op.height)) * 2.0f;
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
      V<R> a[8];
      for (uint32_t k = 0; k < np && k < 8; ++k) {
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
