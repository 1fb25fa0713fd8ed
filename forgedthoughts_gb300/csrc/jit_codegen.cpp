// Lowering of a scene's hook programs to CUDA C++ for run-time compilation
// (NVRTC): the role the Cranelift JIT plays in the reference (J:607-747,
// J:2931-3016), with CUDA source as the target.
//
// Each program becomes one straight-line device function whose registers are
// plain locals (the interpreter keeps them in a per-thread array indexed at
// run time).  Every instruction is emitted with the interpreter's arithmetic,
// operand broadcasting and lane rules (ft_device.cuh, run_program), so the
// two evaluate the same expressions.  Immediates are written as their exact
// bit patterns.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "jit.h"

namespace ftgpu {
namespace {

std::string fbits(float v) {
  uint32_t u;
  std::memcpy(&u, &v, sizeof(u));
  char buf[48];
  std::snprintf(buf, sizeof(buf), "__int_as_float(0x%08x)", u);
  return buf;
}

std::string reg(int r) { return "r" + std::to_string(r); }

// Operand as the interpreter reads it: scalar operands broadcast lane x.
std::string operand(int r, bool scalar) {
  return scalar ? "f3(" + reg(r) + ".x, " + reg(r) + ".x, " + reg(r) + ".x)" : reg(r);
}

void emit_instr(const ft_instr& in, std::string* out) {
  const bool v = (in.flags & FT_INSTR_VEC3) != 0;
  std::string a = operand(in.a, in.flags & FT_INSTR_A_SCALAR);
  std::string b = operand(in.b, in.flags & FT_INSTR_B_SCALAR);
  std::string c = operand(in.c, in.flags & FT_INSTR_C_SCALAR);
  std::string& s = *out;
  s += "  {\n    const F3 a = " + a + ", b = " + b + ", c = " + c + ";\n    (void)a; (void)b; (void)c;\n"
       "    F3 o = f3(0.0f, 0.0f, 0.0f);\n";
  auto lanes = [&](const char* x, const char* y, const char* z) {
    s += std::string("    o.x = ") + x + ";\n";
    if (v) s += std::string("    o.y = ") + y + ";\n    o.z = " + z + ";\n";
  };
  switch (in.op) {
    case FT_OP_CONST:
      s += "    o = f3(" + fbits(in.imm[0]) + ", " + fbits(in.imm[1]) + ", " + fbits(in.imm[2]) + ");\n";
      break;
    case FT_OP_MOV: s += "    o = a;\n"; break;
    case FT_OP_ADD: lanes("a.x + b.x", "a.y + b.y", "a.z + b.z"); break;
    case FT_OP_SUB: lanes("a.x - b.x", "a.y - b.y", "a.z - b.z"); break;
    case FT_OP_MUL: lanes("a.x * b.x", "a.y * b.y", "a.z * b.z"); break;
    case FT_OP_DIV: lanes("a.x / b.x", "a.y / b.y", "a.z / b.z"); break;
    case FT_OP_NEG: lanes("-a.x", "-a.y", "-a.z"); break;
    case FT_OP_GETX: s += "    o.x = a.x;\n"; break;
    case FT_OP_GETY: s += "    o.x = a.y;\n"; break;
    case FT_OP_GETZ: s += "    o.x = a.z;\n"; break;
    case FT_OP_VEC3: s += "    o = f3(a.x, b.x, c.x);\n"; break;
    case FT_OP_ABS: lanes("fabsf(a.x)", "fabsf(a.y)", "fabsf(a.z)"); break;
    case FT_OP_FLOOR: lanes("floorf(a.x)", "floorf(a.y)", "floorf(a.z)"); break;
    case FT_OP_CEIL: lanes("ceilf(a.x)", "ceilf(a.y)", "ceilf(a.z)"); break;
    case FT_OP_FRACT: lanes("a.x - floorf(a.x)", "a.y - floorf(a.y)", "a.z - floorf(a.z)"); break;
    case FT_OP_SQRT: lanes("sqrtf(a.x)", "sqrtf(a.y)", "sqrtf(a.z)"); break;
    case FT_OP_SIN: lanes("sinf(a.x)", "sinf(a.y)", "sinf(a.z)"); break;
    case FT_OP_COS: lanes("cosf(a.x)", "cosf(a.y)", "cosf(a.z)"); break;
    case FT_OP_SATURATE:
      lanes("rclamp(a.x, 0.0f, 1.0f)", "rclamp(a.y, 0.0f, 1.0f)", "rclamp(a.z, 0.0f, 1.0f)");
      break;
    case FT_OP_MIN: lanes("rmin(a.x, b.x)", "rmin(a.y, b.y)", "rmin(a.z, b.z)"); break;
    case FT_OP_MAX: lanes("rmax(a.x, b.x)", "rmax(a.y, b.y)", "rmax(a.z, b.z)"); break;
    case FT_OP_POW: lanes("powf(a.x, b.x)", "powf(a.y, b.y)", "powf(a.z, b.z)"); break;
    case FT_OP_CLAMP:
      lanes("b.x <= c.x ? rclamp(a.x, b.x, c.x) : rclamp(a.x, c.x, b.x)",
            "b.y <= c.y ? rclamp(a.y, b.y, c.y) : rclamp(a.y, c.y, b.y)",
            "b.z <= c.z ? rclamp(a.z, b.z, c.z) : rclamp(a.z, c.z, b.z)");
      break;
    case FT_OP_MIX:
      lanes("a.x * (1.0f - c.x) + b.x * c.x", "a.y * (1.0f - c.y) + b.y * c.y", "a.z * (1.0f - c.z) + b.z * c.z");
      break;
    case FT_OP_STEP: s += "    o.x = b.x < a.x ? 0.0f : 1.0f;\n"; break;
    case FT_OP_SMOOTHSTEP:
      s += "    { float span = b.x - a.x;\n"
           "      float t = fabsf(span) < kEps ? (c.x < a.x ? 0.0f : 1.0f) : rclamp((c.x - a.x) / span, 0.0f, 1.0f);\n"
           "      o.x = t * t * (3.0f - 2.0f * t); }\n";
      break;
    case FT_OP_DOT: s += "    o.x = a.x * b.x + a.y * b.y + a.z * b.z;\n"; break;
    case FT_OP_LENGTH: s += "    o.x = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);\n"; break;
    case FT_OP_NORMALIZE:
      s += "    { float l = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);\n"
           "      o = l <= kEps ? f3(0.0f, 0.0f, 0.0f) : f3(a.x / l, a.y / l, a.z / l); }\n";
      break;
    case FT_OP_ROTX:
      s += "    { float sn, cs; sincosf(deg2rad(b.x), &sn, &cs);\n"
           "      o = f3(a.x, cs * a.y - sn * a.z, sn * a.y + cs * a.z); }\n";
      break;
    case FT_OP_ROTY:
      s += "    { float sn, cs; sincosf(deg2rad(b.x), &sn, &cs);\n"
           "      o = f3(cs * a.x + sn * a.z, a.y, -sn * a.x + cs * a.z); }\n";
      break;
    case FT_OP_ROTZ:
      s += "    { float sn, cs; sincosf(deg2rad(b.x), &sn, &cs);\n"
           "      o = f3(cs * a.x - sn * a.y, sn * a.x + cs * a.y, a.z); }\n";
      break;
    case FT_OP_RET: s += "    return a;\n"; break;
    default: s += "    return f3(0.0f, 0.0f, 0.0f);\n"; break;
  }
  if (in.op != FT_OP_RET) s += "    " + reg(in.dst) + " = o;\n";
  s += "  }\n";
}

}  // namespace

std::string jit_hook_source(const ft_program* programs, uint32_t n_programs, const ft_instr* instrs) {
  std::string s;
  s += "// hook programs lowered by the scene JIT\n";
  s += "using namespace ftd;\n";
  s += "constexpr float kEps = 1.1920929e-7f;\n";
  for (uint32_t p = 0; p < n_programs; ++p) {
    const ft_program& pg = programs[p];
    s += "__device__ __forceinline__ F3 ft_jit_p" + std::to_string(p) + "(const F3* args) {\n";
    for (uint32_t r = 0; r < pg.n_regs && r < FT_MAX_PROGRAM_REGS; ++r) {
      if (r < pg.n_params) s += "  F3 " + reg(static_cast<int>(r)) + " = args[" + std::to_string(r) + "];\n";
      else s += "  F3 " + reg(static_cast<int>(r)) + " = f3(0.0f, 0.0f, 0.0f);\n";
    }
    for (uint32_t k = 0; k < pg.n_instr; ++k) emit_instr(instrs[pg.first_instr + k], &s);
    s += "  return f3(0.0f, 0.0f, 0.0f);\n}\n";
  }
  s += "__device__ F3 ft_jit_program(int index, const F3* args) {\n  switch (index) {\n";
  for (uint32_t p = 0; p < n_programs; ++p)
    s += "    case " + std::to_string(p) + ": return ft_jit_p" + std::to_string(p) + "(args);\n";
  s += "    default: return f3(0.0f, 0.0f, 0.0f);\n  }\n}\n";
  return s;
}

}  // namespace ftgpu
