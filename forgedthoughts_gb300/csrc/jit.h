// Run-time compilation of a scene's kernels (NVRTC): hook-program lowering
// and the device headers the compile unit includes, embedded at build time.
#pragma once

#include <cstdint>
#include <string>

#include "forgedthoughts_gb300.h"

namespace ftgpu {

// CUDA C++ for the hook programs: one device function per program and the
// dispatch `ft_jit_program(index, args)` the kernels call under FT_JIT.
std::string jit_hook_source(const ft_program* programs, uint32_t n_programs, const ft_instr* instrs);

// The device headers (name, contents), generated into the library by the
// build from the sources it compiles.
int jit_header_count();
const char* jit_header_name(int i);
const char* jit_header_text(int i);

}  // namespace ftgpu
