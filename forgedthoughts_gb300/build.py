"""In-tree build of the native libraries.

* ``forgedthoughts_gb300/_build/libforgedthoughts_gb300.so`` — the product:
  the `.ft` front-end, the scene builder and the sm_103a kernels behind the C
  ABI of ``include/forgedthoughts_gb300.h``.
* ``oracle/_build/libftoracle.so`` — the CPU oracle used by the tests and the
  benchmark's CPU-baseline leg (test infrastructure, never linked by the
  product).

Translation units compile in parallel; no CMake.  Run ``python -m
forgedthoughts_gb300.build`` or call :func:`build_all`.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "forgedthoughts_gb300"
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
ORACLE = ROOT / "oracle"
ORACLE_BUILD = ORACLE / "_build"

LIB_NAME = "libforgedthoughts_gb300.so"
ORACLE_NAME = "libftoracle.so"

GENCODE = "arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]

CPP_SOURCES = ["frontend_parse.cpp", "frontend_eval.cpp", "frontend_lower.cpp", "frontend_import.cpp",
               "frontend_layout.cpp", "frontend_api.cpp", "scene_build.cpp", "jit_codegen.cpp"]
CU_SOURCES = ["ft_render.cu"]
HEADERS = ["frontend.h", "common.h", "scene_build.h", "ft_device.cuh", "ft_trace.cuh", "ft_bricks.cuh", "ft_diff.cuh",
           "ft_kernels.cuh", "ft_layout.h", "jit.h", "ft_wavefront.cuh", "ft_path.cuh"]
# Device headers embedded for run-time compilation (NVRTC) of scene kernels.
JIT_HEADERS = ["ft_kernels.cuh", "ft_device.cuh", "ft_layout.h", "ft_bricks.cuh", "ft_trace.cuh", "ft_diff.cuh",
               "ft_wavefront.cuh", "ft_path.cuh"]

# Minimal C headers for the run-time compile unit (NVRTC ships no C library).
_JIT_SHIMS = {
    "stdint.h": (
        "#pragma once\n"
        "typedef signed char int8_t; typedef short int16_t; typedef int int32_t; typedef long long int64_t;\n"
        "typedef unsigned char uint8_t; typedef unsigned short uint16_t; typedef unsigned int uint32_t;\n"
        "typedef unsigned long long uint64_t;\n"),
    "stddef.h": "#pragma once\n",  # size_t and ptrdiff_t are built into the run-time compiler
    "cstdint": (
        "#pragma once\n#include <stdint.h>\nnamespace std { using ::int8_t; using ::int16_t; using ::int32_t;\n"
        "using ::int64_t; using ::uint8_t; using ::uint16_t; using ::uint32_t; using ::uint64_t; }\n"),
}


def _c_string(text: str) -> str:
    # raw string literal chunks (MSVC-style limits do not apply; keep lines short anyway)
    parts = []
    for i in range(0, len(text), 16000):
        parts.append('R"FTJIT(' + text[i:i + 16000] + ')FTJIT"')
    return "\n".join(parts)


def _write_jit_headers(path: Path) -> None:
    entries = [(name, (CSRC / name).read_text()) for name in JIT_HEADERS]
    entries.append(("forgedthoughts_gb300.h", (INCLUDE / "forgedthoughts_gb300.h").read_text()))
    entries += list(_JIT_SHIMS.items())
    out = ["// Generated by forgedthoughts_gb300/build.py: device headers for run-time compilation.",
           '#include "jit.h"', "namespace ftgpu {", "namespace {",
           "const char* const kNames[] = {" + ", ".join('"%s"' % n for n, _ in entries) + "};",
           "const char* const kTexts[] = {"]
    for _, text in entries:
        out.append(_c_string(text) + ",")
    out += ["};", "}  // namespace",
            "int jit_header_count() { return %d; }" % len(entries),
            "const char* jit_header_name(int i) { return kNames[i]; }",
            "const char* jit_header_text(int i) { return kTexts[i]; }",
            "}  // namespace ftgpu", ""]
    path.write_text("\n".join(out))


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the GPU library")
    return cand


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + proc.stdout)
    if proc.stdout.strip() and os.environ.get("FT_BUILD_VERBOSE"):
        print(proc.stdout)


def _digest(paths: list[Path], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in paths:
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def _up_to_date(out: Path, stamp: Path, digest: str) -> bool:
    return out.exists() and stamp.exists() and stamp.read_text() == digest


def build_library(force: bool = False) -> Path:
    """Compile the product library for sm_103a."""
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / LIB_NAME
    stamp = BUILD / (LIB_NAME + ".stamp")
    inputs = [CSRC / s for s in CPP_SOURCES + CU_SOURCES + HEADERS] + [INCLUDE / "forgedthoughts_gb300.h"]
    digest = _digest(inputs, GENCODE + " ".join(CXXFLAGS))
    if not force and _up_to_date(out, stamp, digest):
        return out
    nvcc = _nvcc()
    jobs = []
    objs = []
    gen = BUILD / "ft_jit_headers.cpp"
    _write_jit_headers(gen)
    for src in [CSRC / s for s in CPP_SOURCES] + [gen]:
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        jobs.append(["g++", *CXXFLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(obj)])
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        # -split-compile 0: cicc and ptxas work on the kernels in parallel on
        # every host core (ptxas alone is ~3 minutes single-threaded)
        jobs.append([nvcc, "-gencode", GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-O3", "-split-compile", "0", "-I", str(INCLUDE), "-I", str(CSRC), "-c",
                     str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    tmp = BUILD / (LIB_NAME + ".tmp")
    _run([nvcc, "-shared", "-gencode", GENCODE, "-cudart", "static", "-o", str(tmp), *map(str, objs),
          "-Xlinker", "--no-undefined", "-lnvrtc", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, out)
    stamp.write_text(digest)
    return out


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure)."""
    ORACLE_BUILD.mkdir(parents=True, exist_ok=True)
    out = ORACLE_BUILD / ORACLE_NAME
    stamp = ORACLE_BUILD / (ORACLE_NAME + ".stamp")
    inputs = [ORACLE / "oracle.cpp", ORACLE / "oracle.h", INCLUDE / "forgedthoughts_gb300.h"]
    # -ffp-contract=off keeps the f32 oracle's rounding identical to the
    # reference's separate multiply/add on every host architecture.
    flags = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", "-shared"]
    digest = _digest(inputs, " ".join(flags))
    if not force and _up_to_date(out, stamp, digest):
        return out
    tmp = ORACLE_BUILD / (ORACLE_NAME + ".tmp")
    _run(["g++", *flags, "-I", str(INCLUDE), "-I", str(ORACLE), str(ORACLE / "oracle.cpp"), "-o", str(tmp)])
    os.replace(tmp, out)
    stamp.write_text(digest)
    return out


def build_all(force: bool = False) -> tuple[Path, Path]:
    with ThreadPoolExecutor(max_workers=2) as ex:
        lib = ex.submit(build_library, force)
        orc = ex.submit(build_oracle, force)
        return lib.result(), orc.result()


if __name__ == "__main__":
    paths = build_all(force="--force" in sys.argv)
    for p in paths:
        print(p)
