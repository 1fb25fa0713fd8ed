// Device-side SDF arithmetic for sm_103a: primitives, hg_sdf operators, the
// noise modifier, point transforms and the hook-program interpreter.
//
// Each function restates the reference's CPU arithmetic
// (crates/forgedthoughts/src/renderer.rs, "R") so that a GPU evaluation and the
// reference's f32 evaluation agree to rounding.  No fast-math: sin/cos of hook
// arguments such as sin(p.y * 120) need full-range accuracy.
#pragma once

#include <cstdint>

#include "forgedthoughts_gb300.h"

#define FT_DEV __device__ __forceinline__

namespace ftd {

struct F3 {
  float x, y, z;
};
FT_DEV F3 f3(float x, float y, float z) { return F3{x, y, z}; }
FT_DEV F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
FT_DEV F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
FT_DEV F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
FT_DEV float dot3(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
FT_DEV float len3(F3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
// Vec3::cross
FT_DEV F3 cross3(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
// Vec3::normalize (R:414-420)
FT_DEV F3 normalize3(F3 a) {
  float l = len3(a);
  if (l <= 1.1920929e-7f) return a;
  return a * (1.0f / l);
}

// Rust f32::max / f32::min / f32::clamp.
FT_DEV float rmax(float a, float b) { return fmaxf(a, b); }
FT_DEV float rmin(float a, float b) { return fminf(a, b); }
FT_DEV float rclamp(float x, float lo, float hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}
FT_DEV float rem_euclid(float a, float b) {
  float r = fmodf(a, b);
  return r < 0.0f ? r + fabsf(b) : r;
}

struct Info {  // DistanceInfo (R:454-459)
  float d;
  uint32_t obj, mat;
};

// Scene node as laid out in device memory: the IR node plus the sin/cos of
// the inverse rotation angles, computed once on the host with the same f32
// sin/cos the reference evaluates per call in to_local (R:6216-6240).
struct DevNode {
  int32_t kind, a, b, program;
  uint32_t object_id, material_id;
  int32_t ival, has_rot;
  float c[3];
  float sz, cz, sy, cy, sx, cx;  // sin/cos of radians(-rot.z), (-rot.y), (-rot.x)
  float f[6];
  float bmin[3], bmax[3];
  float pad[3];
};
static_assert(sizeof(DevNode) == 128, "DevNode is one 128-byte line");

// to_local (R:6216-6222): translate, then rotate_z, rotate_y, rotate_x.
FT_DEV F3 to_local(F3 p, const DevNode& n) {
  F3 q = f3(p.x - n.c[0], p.y - n.c[1], p.z - n.c[2]);
  if (!n.has_rot) return q;
  q = f3(n.cz * q.x - n.sz * q.y, n.sz * q.x + n.cz * q.y, q.z);
  q = f3(n.cy * q.x + n.sy * q.z, q.y, -n.sy * q.x + n.cy * q.z);
  q = f3(q.x, n.cx * q.y - n.sx * q.z, n.sx * q.y + n.cx * q.z);
  return q;
}

FT_DEV float shell(float d, float sh) { return sh > 0.0f ? rmax(d, -(d + sh)) : d; }

// sd_regular_ngon (R:6206-6214).  Out of line: its trigonometry would
// otherwise be inlined at every primitive evaluation site of the march loops,
// whose bodies have to stay within the instruction cache.
__device__ __noinline__ float sd_regular_ngon(float px, float pz, int sides, float radius) {
  float n = (float)(sides > 3 ? sides : 3);
  float an = 3.14159265358979323846f / n;
  float apothem = radius * cosf(an);
  float angle = atan2f(pz, px);
  float sector = 2.0f * an;
  float wrapped = rem_euclid(angle + an, sector) - an;
  return hypotf(px, pz) * cosf(wrapped) - apothem;
}

__device__ __noinline__ float prim_local_rare(int kind, const float* f, int ival, F3 q);

// Primitive arms of sdf_distance_info (R:5547-5663), point already local.
// Spheres and boxes inline; the other kinds out of line.
FT_DEV float prim_local(int kind, const float* f, int ival, F3 q) {
  switch (kind) {
    case FT_NODE_SPHERE: return shell(len3(q) - f[0], f[1]);
    case FT_NODE_BOX: {
      float rd = f[3];
      float ix = rmax(f[0] - rd, 0.0f), iy = rmax(f[1] - rd, 0.0f), iz = rmax(f[2] - rd, 0.0f);
      float qx = fabsf(q.x) - ix, qy = fabsf(q.y) - iy, qz = fabsf(q.z) - iz;
      float ox = rmax(qx, 0.0f), oy = rmax(qy, 0.0f), oz = rmax(qz, 0.0f);
      float outside = sqrtf(ox * ox + oy * oy + oz * oz);
      float inside = rmin(rmax(rmax(qx, qy), qz), 0.0f);
      return shell(outside + inside - rd, f[4]);
    }
    default: return prim_local_rare(kind, f, ival, q);
  }
}

__device__ __noinline__ float prim_local_rare(int kind, const float* f, int ival, F3 q) {
  switch (kind) {
    case FT_NODE_SPHERE: return shell(len3(q) - f[0], f[1]);
    case FT_NODE_BOX: {
      float rd = f[3];
      float ix = rmax(f[0] - rd, 0.0f), iy = rmax(f[1] - rd, 0.0f), iz = rmax(f[2] - rd, 0.0f);
      float qx = fabsf(q.x) - ix, qy = fabsf(q.y) - iy, qz = fabsf(q.z) - iz;
      float ox = rmax(qx, 0.0f), oy = rmax(qy, 0.0f), oz = rmax(qz, 0.0f);
      float outside = sqrtf(ox * ox + oy * oy + oz * oz);
      float inside = rmin(rmax(rmax(qx, qy), qz), 0.0f);
      return shell(outside + inside - rd, f[4]);
    }
    case FT_NODE_CYLINDER: {
      float rd = f[2];
      float radial = sqrtf(q.x * q.x + q.z * q.z);
      float dx = radial - rmax(f[0] - rd, 0.0f);
      float dy = fabsf(q.y) - rmax(f[1] - rd, 0.0f);
      float ox = rmax(dx, 0.0f), oy = rmax(dy, 0.0f);
      float outside = sqrtf(ox * ox + oy * oy);
      float inside = rmin(rmax(dx, dy), 0.0f);
      return shell(outside + inside - rd, f[3]);
    }
    case FT_NODE_TORUS: {
      float qx = sqrtf(q.x * q.x + q.z * q.z) - f[0];
      return sqrtf(qx * qx + q.y * q.y) - f[1];
    }
    case FT_NODE_EXTRUDE_POLYGON: {
      float rd = f[2];
      float radial = sd_regular_ngon(q.x, q.z, ival, rmax(f[0] - rd, 0.0f));
      float dy = fabsf(q.y) - rmax(f[1] - rd, 0.0f);
      float ox = rmax(radial, 0.0f), oy = rmax(dy, 0.0f);
      float outside = sqrtf(ox * ox + oy * oy);
      float inside = rmin(rmax(radial, dy), 0.0f);
      return shell(outside + inside - rd, f[3]);
    }
  }
  return 0.0f;
}

FT_DEV float prim_distance(const DevNode& n, F3 p) { return prim_local(n.kind, n.f, n.ival, to_local(p, n)); }

// Device-wide nanosecond timer (%globaltimer), for time limits of long loops.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// point_aabb_lower_bound (R:5388-5411)
FT_DEV float aabb_lb(F3 p, const float* mn, const float* mx) {
  float dx = p.x < mn[0] ? mn[0] - p.x : (p.x > mx[0] ? p.x - mx[0] : 0.0f);
  float dy = p.y < mn[1] ? mn[1] - p.y : (p.y > mx[1] ? p.y - mx[1] : 0.0f);
  float dz = p.z < mn[2] ? mn[2] - p.z : (p.z > mx[2] ? p.z - mx[2] : 0.0f);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// ---------------------------------------------------------- hg_sdf operators
constexpr float kFrac1Sqrt2 = 0.70710678118654752440f;

FT_DEV float op_union_round(float a, float b, float r) {
  r = rmax(fabsf(r), 1.0e-6f);
  float ux = rmax(r - a, 0.0f), uy = rmax(r - b, 0.0f);
  return rmax(r, rmin(a, b)) - sqrtf(ux * ux + uy * uy);
}
FT_DEV float op_intersect_round(float a, float b, float r) {
  r = rmax(fabsf(r), 1.0e-6f);
  float ux = rmax(r + a, 0.0f), uy = rmax(r + b, 0.0f);
  return rmin(-r, rmax(a, b)) + sqrtf(ux * ux + uy * uy);
}
FT_DEV float op_union_chamfer(float a, float b, float r) { return rmin(rmin(a, b), (a - r + b) * kFrac1Sqrt2); }
FT_DEV float op_intersect_chamfer(float a, float b, float r) { return rmax(rmax(a, b), (a + r + b) * kFrac1Sqrt2); }
FT_DEV float repeat_centered(float p, float size) {
  size = rmax(size, 1.0e-6f);
  return rem_euclid(p + size * 0.5f, size) - size * 0.5f;
}
FT_DEV float op_union_columns(float a, float b, float r, float n) {
  if (a < r && b < r) {
    n = rmax(roundf(n), 2.0f);
    const float sq2 = 1.41421356237309504880f;
    float col = r * sq2 / ((n - 1.0f) * 2.0f + sq2);
    float x = a + col, y = b + col;
    bool odd = (((int)n) % 2) == 1;
    if (odd) x += col;
    float rx = (x + y) * kFrac1Sqrt2, ry = (y - x) * kFrac1Sqrt2;
    x = rx;
    y = ry;
    x -= sq2 * 0.5f * r;
    x += -col * sq2;
    if (odd) y += col;
    y = repeat_centered(y, col * 2.0f);
    return sqrtf(x * x + y * y) - col;
  }
  return rmin(a, b);
}
FT_DEV float op_union_stairs(float a, float b, float r, float n) {
  n = rmax(roundf(n), 1.0f);
  float s = r / n;
  float u = b - r;
  return rmin(rmin(a, b), 0.5f * (u + a + fabsf(rem_euclid(u - a + s, 2.0f * s) - s)));
}
FT_DEV float op_union_soft(float a, float b, float r) {
  r = rmax(fabsf(r), 1.0e-6f);
  float e = rmax(r - fabsf(a - b), 0.0f);
  return rmin(a, b) - e * e * 0.25f / r;
}
FT_DEV float op_smax(float a, float b, float k) {
  float h = rmax(k - fabsf(a - b), 0.0f);
  return rmax(a, b) + h * h * 0.25f / rmax(k, 1.0e-6f);
}
FT_DEV float op_smin(float a, float b, float k) {
  float h = rmax(k - fabsf(a - b), 0.0f);
  return rmin(a, b) - h * h * 0.25f / rmax(k, 1.0e-6f);
}

// Combine two child results of a binary node (R:5700-5931).
FT_DEV Info combine(int kind, float ra, float rb, Info l, Info r) {
  float d;
  switch (kind) {
    case FT_NODE_UNION: return l.d <= r.d ? l : r;
    case FT_NODE_INTERSECT: return l.d >= r.d ? l : r;
    case FT_NODE_SUBTRACT: {
      float rd = -r.d;
      if (l.d >= rd) return l;
      return Info{rd, r.obj, r.mat};
    }
    case FT_NODE_UNION_ROUND: d = op_union_round(l.d, r.d, ra); break;
    case FT_NODE_UNION_CHAMFER: d = op_union_chamfer(l.d, r.d, ra); break;
    case FT_NODE_UNION_COLUMNS: d = op_union_columns(l.d, r.d, ra, rb); break;
    case FT_NODE_UNION_STAIRS: d = op_union_stairs(l.d, r.d, ra, rb); break;
    case FT_NODE_UNION_SOFT: d = op_union_soft(l.d, r.d, ra); break;
    case FT_NODE_INTERSECT_ROUND: d = op_intersect_round(l.d, r.d, ra); break;
    case FT_NODE_INTERSECT_CHAMFER: d = op_intersect_chamfer(l.d, r.d, ra); break;
    case FT_NODE_INTERSECT_COLUMNS: d = -op_union_columns(-l.d, -r.d, ra, rb); break;
    case FT_NODE_INTERSECT_STAIRS: d = -op_union_stairs(-l.d, -r.d, ra, rb); break;
    case FT_NODE_DIFF_ROUND: d = op_intersect_round(l.d, -r.d, ra); break;
    case FT_NODE_DIFF_CHAMFER: d = op_intersect_chamfer(l.d, -r.d, ra); break;
    case FT_NODE_DIFF_COLUMNS: d = -op_union_columns(-l.d, r.d, ra, rb); break;
    case FT_NODE_DIFF_STAIRS: d = -op_union_stairs(-l.d, r.d, ra, rb); break;
    case FT_NODE_PIPE: return Info{sqrtf(l.d * l.d + r.d * r.d) - fabsf(ra), l.obj, l.mat};
    case FT_NODE_ENGRAVE: return Info{rmax(l.d, (l.d + fabsf(ra) - fabsf(r.d)) * kFrac1Sqrt2), l.obj, l.mat};
    case FT_NODE_GROOVE: return Info{rmax(l.d, rmin(l.d + fabsf(ra), fabsf(rb) - fabsf(r.d))), l.obj, l.mat};
    case FT_NODE_TONGUE: return Info{rmin(l.d, rmax(l.d - fabsf(ra), fabsf(r.d) - fabsf(rb))), l.obj, l.mat};
    default: return l;
  }
  if (kind <= FT_NODE_UNION_SOFT) return l.d <= r.d ? Info{d, l.obj, l.mat} : Info{d, r.obj, r.mat};
  if (kind <= FT_NODE_INTERSECT_STAIRS) return l.d >= r.d ? Info{d, l.obj, l.mat} : Info{d, r.obj, r.mat};
  return l.d >= -r.d ? Info{d, l.obj, l.mat} : Info{d, r.obj, r.mat};
}

// ---------------------------------------------------------- noise (R:5957-6017)
FT_DEV float fractf_(float x) { return x - floorf(x); }
FT_DEV float hash_noise(F3 p) {
  const float f1pi = 0.31830988618379067154f;
  F3 q = f3(fractf_(p.x * f1pi + 0.11f), fractf_(p.y * f1pi + 0.17f), fractf_(p.z * f1pi + 0.13f)) * 17.0f;
  return fractf_(q.x * q.y * q.z * (q.x + q.y + q.z));
}
FT_DEV float sd_base_noise(F3 p) {
  p = p + f3(0.5f, 0.5f, 0.5f);
  F3 i = f3(floorf(p.x), floorf(p.y), floorf(p.z));
  F3 f = f3(fractf_(p.x), fractf_(p.y), fractf_(p.z));
  float d = __int_as_float(0x7f800000);
  for (int ix = 0; ix <= 1; ++ix)
    for (int iy = 0; iy <= 1; ++iy)
      for (int iz = 0; iz <= 1; ++iz) {
        F3 c = f3((float)ix, (float)iy, (float)iz);
        float r = hash_noise(i + c);
        r = r * r * 0.7f;
        d = rmin(d, len3(f - c) - r);
      }
  return d;
}
FT_DEV float apply_noise(F3 p, float d, int octaves, float scale, float lac) {
  F3 q = p * rmax(scale, 1.0e-4f);
  float os = rmax(lac, 1.0e-4f);
  float s = 1.0f, t = 0.0f;
  int n = octaves > 1 ? octaves : 1;
  for (int o = 0; o < n; ++o) {
    float nn = s * sd_base_noise(q);
    nn = op_smax(nn, d - 0.1f * s, 0.3f * s);
    d = op_smin(nn, d, 0.3f * s);
    t += d;
    q = f3(0.00f * q.x + 1.60f * q.y + 1.20f * q.z, -1.60f * q.x + 0.72f * q.y - 0.96f * q.z,
           -1.20f * q.x - 0.96f * q.y + 1.28f * q.z) * os;
    s *= 0.415f;
    q.z += -4.33f * t * s;
  }
  return d;
}

// ---------------------------------------------------------- hook programs
// Interpreter for ft_instr programs (the role of the reference's JIT'd hook
// functions, E:2011-2146 / jit.rs:2931-3016).  Registers live in local memory.
FT_DEV float deg2rad(float d) { return d * (3.14159265358979323846f / 180.0f); }

FT_DEV F3 run_program(const ft_program& pg, const ft_instr* __restrict__ code, const F3* args,
                      unsigned long long* instr_count) {
  F3 regs[FT_MAX_PROGRAM_REGS];
  for (uint32_t i = 0; i < pg.n_params; ++i) regs[i] = args[i];
  const float eps = 1.1920929e-7f;
  for (uint32_t k = 0; k < pg.n_instr; ++k) {
    const ft_instr in = code[pg.first_instr + k];
    F3 a = regs[in.a], b = regs[in.b], c = regs[in.c];
    if (in.flags & FT_INSTR_A_SCALAR) a = f3(a.x, a.x, a.x);
    if (in.flags & FT_INSTR_B_SCALAR) b = f3(b.x, b.x, b.x);
    if (in.flags & FT_INSTR_C_SCALAR) c = f3(c.x, c.x, c.x);
    const bool v = (in.flags & FT_INSTR_VEC3) != 0;
    F3 o = f3(0.0f, 0.0f, 0.0f);
#define FT_LANES1(EXPR_X, EXPR_Y, EXPR_Z) \
  o.x = (EXPR_X);                          \
  if (v) {                                 \
    o.y = (EXPR_Y);                        \
    o.z = (EXPR_Z);                        \
  }
    switch (in.op) {
      case FT_OP_CONST: o = f3(in.imm[0], in.imm[1], in.imm[2]); break;
      case FT_OP_MOV: o = a; break;
      case FT_OP_ADD: FT_LANES1(a.x + b.x, a.y + b.y, a.z + b.z); break;
      case FT_OP_SUB: FT_LANES1(a.x - b.x, a.y - b.y, a.z - b.z); break;
      case FT_OP_MUL: FT_LANES1(a.x * b.x, a.y * b.y, a.z * b.z); break;
      case FT_OP_DIV: FT_LANES1(a.x / b.x, a.y / b.y, a.z / b.z); break;
      case FT_OP_NEG: FT_LANES1(-a.x, -a.y, -a.z); break;
      case FT_OP_GETX: o.x = a.x; break;
      case FT_OP_GETY: o.x = a.y; break;
      case FT_OP_GETZ: o.x = a.z; break;
      case FT_OP_VEC3: o = f3(a.x, b.x, c.x); break;
      case FT_OP_ABS: FT_LANES1(fabsf(a.x), fabsf(a.y), fabsf(a.z)); break;
      case FT_OP_FLOOR: FT_LANES1(floorf(a.x), floorf(a.y), floorf(a.z)); break;
      case FT_OP_CEIL: FT_LANES1(ceilf(a.x), ceilf(a.y), ceilf(a.z)); break;
      case FT_OP_FRACT: FT_LANES1(a.x - floorf(a.x), a.y - floorf(a.y), a.z - floorf(a.z)); break;
      case FT_OP_SQRT: FT_LANES1(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); break;
      case FT_OP_SIN: FT_LANES1(sinf(a.x), sinf(a.y), sinf(a.z)); break;
      case FT_OP_COS: FT_LANES1(cosf(a.x), cosf(a.y), cosf(a.z)); break;
      case FT_OP_SATURATE:
        FT_LANES1(rclamp(a.x, 0.0f, 1.0f), rclamp(a.y, 0.0f, 1.0f), rclamp(a.z, 0.0f, 1.0f));
        break;
      case FT_OP_MIN: FT_LANES1(rmin(a.x, b.x), rmin(a.y, b.y), rmin(a.z, b.z)); break;
      case FT_OP_MAX: FT_LANES1(rmax(a.x, b.x), rmax(a.y, b.y), rmax(a.z, b.z)); break;
      case FT_OP_POW: FT_LANES1(powf(a.x, b.x), powf(a.y, b.y), powf(a.z, b.z)); break;
      case FT_OP_CLAMP:
        FT_LANES1(b.x <= c.x ? rclamp(a.x, b.x, c.x) : rclamp(a.x, c.x, b.x),
                  b.y <= c.y ? rclamp(a.y, b.y, c.y) : rclamp(a.y, c.y, b.y),
                  b.z <= c.z ? rclamp(a.z, b.z, c.z) : rclamp(a.z, c.z, b.z));
        break;
      case FT_OP_MIX:
        FT_LANES1(a.x * (1.0f - c.x) + b.x * c.x, a.y * (1.0f - c.y) + b.y * c.y, a.z * (1.0f - c.z) + b.z * c.z);
        break;
      case FT_OP_STEP: o.x = b.x < a.x ? 0.0f : 1.0f; break;
      case FT_OP_SMOOTHSTEP: {
        float span = b.x - a.x;
        float t = fabsf(span) < eps ? (c.x < a.x ? 0.0f : 1.0f) : rclamp((c.x - a.x) / span, 0.0f, 1.0f);
        o.x = t * t * (3.0f - 2.0f * t);
        break;
      }
      case FT_OP_DOT: o.x = a.x * b.x + a.y * b.y + a.z * b.z; break;
      case FT_OP_LENGTH: o.x = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); break;
      case FT_OP_NORMALIZE: {
        float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
        o = l <= eps ? f3(0.0f, 0.0f, 0.0f) : f3(a.x / l, a.y / l, a.z / l);
        break;
      }
      case FT_OP_ROTX: {
        float s, cc;
        sincosf(deg2rad(b.x), &s, &cc);
        o = f3(a.x, cc * a.y - s * a.z, s * a.y + cc * a.z);
        break;
      }
      case FT_OP_ROTY: {
        float s, cc;
        sincosf(deg2rad(b.x), &s, &cc);
        o = f3(cc * a.x + s * a.z, a.y, -s * a.x + cc * a.z);
        break;
      }
      case FT_OP_ROTZ: {
        float s, cc;
        sincosf(deg2rad(b.x), &s, &cc);
        o = f3(cc * a.x - s * a.y, s * a.x + cc * a.y, a.z);
        break;
      }
      case FT_OP_RET:
        if (instr_count) *instr_count += k + 1;
        return a;
    }
#undef FT_LANES1
    regs[in.dst] = o;
  }
  if (instr_count) *instr_count += pg.n_instr;
  return f3(0.0f, 0.0f, 0.0f);
}

}  // namespace ftd
