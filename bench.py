#!/usr/bin/env python3
"""Benchmark of the GB300 sphere-tracing path.

Workload (default, ``--mode trace``): the 512-primitive union_round field
(balanced union_round(0.1) tree of spheres and rotated boxes over a ground box,
Lambert / Metal / Dielectric materials, one point light, an environment light
and a sky environment), rendered as a Whitted trace at 1920x1080 with a 2x2
deterministic AA grid (8,294,400 primary samples per step), max bounce depth 6,
Bricks accelerator semantics, march max 256 steps / eps 1e-4 / max dist 100 /
step scale 0.7.  A step is one full frame: every bounce, shadow ray, blended
normal and material, the per-pixel AA average (linear RGB) and the Reinhard
RGB8 image.

``--mode depth`` times the plain depth march of the same scene (refined hit
distance, hit mask, material id, estimate_normal and the gray preview).  The
trace line carries the depth march as a secondary figure.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode trace|depth]

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference's path (the oracle) on the host cores over a row sample of the same
workload.
"""
from __future__ import annotations

import argparse
import csv
import ctypes
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s at 1080p: plain FP32 vs FP16-brick+batched at depth err ≤1e-4; grads/s"
UNIT = "Mrays/s"

# Algorithmic FP32 work per counted event (FMA = 2 FLOP; sqrt/sin/cos = 1).
# aabb lower bound: 3 axis distances (3 FLOP each incl. select) + dot (5) + sqrt
FLOP_BOX = 15.0
# primitive: to_local translate (3) + rotation (15, most primitives are
# rotated) + sphere/box body (~16 average incl. sqrt)
FLOP_PRIM = 34.0
# march step bookkeeping: point (6), |d| test, step (4)
FLOP_STEP = 12.0
# union_round combine (op_union_round R:6024-6029): two max, two squares, sum,
# sqrt, min and a subtraction = 9 + 1 sqrt
FLOP_BLEND = 10.0
# candidate-list entry: running limit max(r, min(best, cutoff)) and the gap compare
FLOP_CAND = 3.0
# hook program instruction (interpreted or compiled): one operation
FLOP_HOOK = 1.0


def flop_count(s) -> float:
    """FP32 operations of the counted work (an ft_render_stats)."""
    return (s.box_tests * FLOP_BOX + s.primitive_evals * FLOP_PRIM + s.march_steps * FLOP_STEP
            + s.blend_ops * FLOP_BLEND + s.candidate_entries * FLOP_CAND + s.hook_instrs * FLOP_HOOK)

L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
_T0 = time.perf_counter()


def _log(what: str) -> None:
    """Progress on stderr (the JSON line is the only stdout)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f}s] {what}", file=sys.stderr, flush=True)


def _env_int(name: str, default: int) -> int:
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def workload(name: str):
    from forgedthoughts_gb300 import workloads

    if name == "union_round":
        return workloads.union_round_field()
    if name == "spheres":
        return workloads.spheres_on_ground()
    if name == "twisted":
        return workloads.twisted_shells()
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.file.read())) if len(r) >= 9]
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


CPU_ROW_STEP = 8  # every 8th row of the frame


def _oracle_sample(st, w, mode: str, threads: int, accel: int, col_first: int, col_step: int) -> int:
    """The oracle over every 8th row (from row 4) and every col_step-th column
    (from col_first) of the full frame; returns the samples traced."""
    import oracle

    oracle.render_sample(st, w.options, accel, w.aa, w.max_depth, mode, threads, rows=(CPU_ROW_STEP // 2, CPU_ROW_STEP),
                         cols=(col_first, col_step))
    return len(range(CPU_ROW_STEP // 2, w.options.height, CPU_ROW_STEP)) * \
        len(range(col_first, w.options.width, col_step)) * w.aa


def _col_step(st, w, mode: str, threads: int, accel: int, budget_s: float) -> int:
    """Column stride (a power of two, at least 64) for which one sample of
    every 8th row takes about budget_s, from a small timed probe."""
    import oracle

    t0 = time.perf_counter()
    oracle.render_sample(st, w.options, accel, w.aa, w.max_depth, mode, threads, rows=(32, 64), cols=(32, 256))
    probe_s = max(time.perf_counter() - t0, 1e-3)
    probe_n = len(range(32, w.options.height, 64)) * len(range(32, w.options.width, 256)) * w.aa
    per_sample = probe_s / max(probe_n, 1)
    rows = len(range(CPU_ROW_STEP // 2, w.options.height, CPU_ROW_STEP))
    step = 64
    while step < w.options.width and rows * (w.options.width / step) * w.aa * per_sample > budget_s:
        step *= 2
    return step


def _sample_text(w, mode: str, col_step: int, n: int) -> str:
    what = (f"Whitted trace depth {w.max_depth}" if mode == "trace" else "depth march")
    frac = CPU_ROW_STEP * col_step
    return (f"every {CPU_ROW_STEP}th row x every {col_step}th column of the {w.options.width}x{w.options.height} "
            f"frame x {w.aa} AA samples ({n} samples, 1/{frac} of the frame; the rate extrapolates to the full "
            f"frame), f32 C++ restatement of the reference {what}, {w.accel.name} accel")


def cpu_baseline(w, mode: str, budget_s: float = 20.0) -> dict:
    """Oracle (f32 restatement of the reference CPU path) on all host cores
    over a strided sample of the frame: every 8th row, strided columns.  Also
    the depth march under each accelerator mode, as `ftc bench` times
    Naive / Bvh / Bricks (crates/ftc/src/main.rs:508-548)."""
    import forgedthoughts_gb300 as ft

    st = ft.parse_and_eval(w.source)
    threads = os.cpu_count() or 1
    step = _col_step(st, w, mode, threads, int(w.accel), budget_s)
    t0 = time.perf_counter()
    n = _oracle_sample(st, w, mode, threads, int(w.accel), (step // 2) % step, step)
    dt = time.perf_counter() - t0
    out = {"value": n / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": _sample_text(w, mode, step, n) + f", {dt:.1f} s"}
    per_accel = {}
    for accel in (ft.AccelMode.Naive, ft.AccelMode.Bvh, ft.AccelMode.Bricks):
        dstep = _col_step(st, w, "depth", threads, int(accel), 4.0)
        t0 = time.perf_counter()
        dn = _oracle_sample(st, w, "depth", threads, int(accel), (dstep // 2) % dstep, dstep)
        ddt = time.perf_counter() - t0
        per_accel[accel.name] = {"value": dn / ddt / 1e6, "unit": UNIT, "samples": dn, "seconds": ddt,
                                 "col_step": dstep}
    out["depth_march_per_accel"] = per_accel
    return out


def run_reference(args, w) -> None:
    """`--impl reference`: the reference algorithm on the host cores, each
    step a strided sample of the frame (every 8th row; the column offset
    moves from step to step so the steps together cover more of the frame)."""
    import forgedthoughts_gb300 as ft

    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    st = ft.parse_and_eval(w.source)
    threads = os.cpu_count() or 1
    budget = 150.0 / max(args.steps + args.warmup, 1)
    step = _col_step(st, w, args.mode, threads, int(w.accel), budget)
    offsets = [(k * 37 + step // 2) % step for k in range(args.warmup + args.steps)]
    for k in range(args.warmup):
        _oracle_sample(st, w, args.mode, threads, int(w.accel), offsets[k], step)
    times, samples = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        samples += _oracle_sample(st, w, args.mode, threads, int(w.accel), offsets[args.warmup + k], step)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = samples / total / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": _config(w, args.mode, 1) | {"sample_col_step": step, "sample_row_step": CPU_ROW_STEP},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": _sample_text(w, args.mode, step, samples // max(len(times), 1))
                             + " per step, column offset moving per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _config(w, mode: str, world: int) -> dict:
    cfg = {"workload": w.name, "mode": mode, "width": w.options.width, "height": w.options.height, "aa": w.aa,
           "primary_samples_per_step": w.options.width * w.options.height * w.aa, "accel": w.accel.name,
           "variant": "plain_fp32", "l2": "flushed between steps (256 MiB write)",
           "parallelism": f"replicas x{world}"}
    if mode == "trace":
        cfg["max_depth"] = w.max_depth
        cfg["outputs"] = "linear rgb f32 + rgb8 (device)"
    else:
        cfg["outputs"] = "t, mask, material, normal, rgb8 (device)"
    return cfg


class Renderer:
    """One render step through the C ABI with device outputs."""

    def __init__(self, lib, scene, w, mode: str, dev, stream, extra_flags: int = 0):
        import torch

        from forgedthoughts_gb300 import _native

        self.lib, self.scene, self.w, self.mode = lib, scene, w, mode
        self.extra_flags = extra_flags
        self.native = _native
        self.opts = w.options.to_c()
        self.pixels = w.options.width * w.options.height
        self.items = self.pixels * w.aa
        self.sptr = ctypes.c_void_p(stream.cuda_stream)
        e = lambda n, dt: torch.empty(n, dtype=dt, device=dev)  # noqa: E731
        if mode == "trace":
            self.rgbf = e(self.pixels * 3, torch.float32)
            self.rgb8 = e(self.pixels * 3, torch.uint8)
        else:
            self.t = e(self.items, torch.float32)
            self.m = e(self.items, torch.uint8)
            self.mat = e(self.items, torch.int32)
            self.n = e(self.items * 3, torch.float32)
            self.rgb8 = e(self.pixels * 3, torch.uint8)

    def __call__(self, full_outputs: bool = True):
        p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
        w = self.w
        if self.mode == "trace":
            rc = self.lib.ft_render_trace(self.scene.handle, ctypes.byref(self.opts), int(w.accel), w.aa, w.max_depth,
                                          p(self.rgbf) if full_outputs else None,
                                          p(self.rgb8) if full_outputs else None,
                                          self.native.FT_FLAG_DEVICE_POINTERS, self.sptr)
        else:
            rc = self.lib.ft_render_depth(self.scene.handle, ctypes.byref(self.opts), int(w.accel), w.aa, p(self.t),
                                          p(self.m), p(self.mat), p(self.n), p(self.rgb8) if full_outputs else None,
                                          self.native.FT_FLAG_DEVICE_POINTERS | self.extra_flags, self.sptr)
        if rc != 0:
            raise RuntimeError(self.native.last_error())
        n = ctypes.c_uint32(0)
        self.lib.ft_scene_last_launches(self.scene.handle, ctypes.byref(n))
        self.launches += n.value

    launches = 0  # kernels launched by the calls so far

    def stats(self):
        s = self.native.RenderStatsC()
        w = self.w
        if self.mode == "trace":
            rc = self.lib.ft_render_trace_stats(self.scene.handle, ctypes.byref(self.opts), int(w.accel), w.aa,
                                                w.max_depth, ctypes.byref(s))
        else:
            rc = self.lib.ft_render_depth_stats(self.scene.handle, ctypes.byref(self.opts), int(w.accel), w.aa,
                                                self.extra_flags, ctypes.byref(s))
        if rc != 0:
            raise RuntimeError(self.native.last_error())
        return s


def replica_throughput(total_ms: float, items: int, steps: int, world: int, dist=None, device="cpu"):
    """Whole-job throughput of `world` replicas: the slowest rank's time (a
    MAX all-reduce when `dist` is given) and every rank's primary samples.
    Returns (total ms, Mrays/s)."""
    import torch

    if dist is not None:
        tt = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    return total_ms, items * steps * world / (total_ms * 1e-3) / 1e6


def _time_steps(fn, steps: int, stream, flush) -> list[float]:
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.fill_(k & 0xFF)  # evict L2 between steps (outside the timed events)
        starts[k].record(stream)
        fn()
        stops[k].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in zip(starts, stops)]


def _counts(s) -> dict:
    return {"distance_evals": s.distance_evals, "primitive_evals": s.primitive_evals, "box_tests": s.box_tests,
            "march_steps": s.march_steps, "blend_ops": s.blend_ops, "candidate_entries": s.candidate_entries,
            "hook_instrs": s.hook_instrs, "far_steps": s.far_steps, "brick_fetches": s.brick_fetches}


def _fp32_line(flops: float, kernel_ms: float, peak: float) -> dict:
    achieved = flops / (kernel_ms * 1e-3) / 1e12 if kernel_ms > 0 else 0.0
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
            "flop": flops, "kernel_ms": kernel_ms}


PEAK_SOURCE = "measured dependent-FMA kernel (ft_measure_fp32_peak), of measured"


def kernel_times(lib, scene, steps: int) -> dict:
    """Per-kernel CUDA-event times the library recorded on the launch stream
    since profiling started, per step: {kind: (ms per step, launches per step)}."""
    from forgedthoughts_gb300 import _native

    kt = _native.KernelTimesC()
    if lib.ft_scene_kernel_times(scene.handle, ctypes.byref(kt)) != 0:
        raise RuntimeError(_native.last_error())
    return {name: (kt.ms[k] / steps, kt.launches[k] / steps) for k, name in enumerate(_native.KERNEL_KIND_NAMES)
            if kt.launches[k]}


def trace_roofline(r: "Renderer", times: dict, peak: float) -> dict:
    """FP32 roofline of the Whitted trace's dominant kernel (the wavefront ray
    march), with the shade and shadow kernels and the whole wavefront beside
    it.  FLOPs: the op counts of the counting variants of the same kernels on
    the same frame; time: their CUDA-event times inside the timed steps."""
    from forgedthoughts_gb300 import _native

    m, sh, sd = _native.RenderStatsC(), _native.RenderStatsC(), _native.RenderStatsC()
    w = r.w
    if r.lib.ft_render_trace_kernel_stats(r.scene.handle, ctypes.byref(r.opts), int(w.accel), w.aa, w.max_depth,
                                          ctypes.byref(m), ctypes.byref(sh), ctypes.byref(sd)) != 0:
        raise RuntimeError(_native.last_error())
    per = {}
    total_flop = total_ms = 0.0
    for name, st in (("wf_march_persistent", m), ("wf_shade_kernel", sh), ("wf_shadow_persistent", sd)):
        ms, launches = times.get(name, (0.0, 0.0))
        per[name] = _fp32_line(flop_count(st), ms, peak) | {"launches_per_step": launches,
                                                              "avg_launch_ms": ms / launches if launches else None,
                                                              "counts": _counts(st)}
        total_flop += flop_count(st)
        total_ms += ms
    dom = per["wf_march_persistent"]
    line = {"bound": "fp32", "achieved": dom["achieved"], "peak": peak, "unit": "TFLOP/s", "frac": dom["frac"],
            "kernel": "wf_march_persistent", "kernel_ms_per_step": dom["kernel_ms"],
            "avg_launch_ms": dom["avg_launch_ms"], "flop_per_step": dom["flop"], "peak_source": PEAK_SOURCE,
            "flop_model": {"box": FLOP_BOX, "primitive": FLOP_PRIM, "march_step": FLOP_STEP, "blend": FLOP_BLEND,
                           "candidate_entry": FLOP_CAND, "hook_instr": FLOP_HOOK},
            "per_kernel": per, "wavefront": _fp32_line(total_flop, total_ms, peak)}
    return line


def depth_roofline(r: "Renderer", times: dict, peak: float) -> dict:
    s = r.stats()
    ms, launches = times.get("march_depth_persistent", (0.0, 0.0))
    line = {"bound": "fp32", "kernel": "march_depth_persistent", "peak_source": PEAK_SOURCE,
            "launches_per_step": launches} | _fp32_line(flop_count(s), ms, peak)
    line["counts"] = _counts(s)
    if s.brick_fetches:
        # one trilinear FP16 fetch reads 8 lattice corners x 2 B
        line["brick_fetch_gbs"] = s.brick_fetches * 16.0 / (ms * 1e-3) / 1e9 if ms > 0 else None
    return line


def _depth_figures(lib, scene, w, dev, stream, flush, peak: float, flags: int) -> dict:
    import torch

    d = Renderer(lib, scene, w, "depth", dev, stream, flags)
    for _ in range(3):
        d()
    torch.cuda.synchronize()
    lib.ft_scene_profile(scene.handle, 1)
    d_ms = _time_steps(d, 20, stream, flush)
    times = kernel_times(lib, scene, 20)
    lib.ft_scene_profile(scene.handle, 0)
    dl = depth_roofline(d, times, peak)
    dl["traffic"], note = _traffic_summary("march_depth_persistent" + ("_fp16_bricks" if flags else ""), w)
    if note:
        dl["traffic_source"] = note
    return {"value": d.items * len(d_ms) / (sum(d_ms) * 1e-3) / 1e6, "unit": UNIT,
            "ms_per_step": statistics.mean(d_ms), "roofline": dl, "gpu_launches_per_step": 2}


def _brick_figures(lib, scene, w, dev, stream, flush, peak: float) -> dict:
    """Build the FP16 brick cache, time the precision-form depth march, and
    compare its frame with the plain march's (mask agreement, depth error)."""
    import numpy as np
    import torch

    from forgedthoughts_gb300 import _native

    info = _native.BrickInfoC()
    o = _native.BrickOptionsC(0.02, 0.0, 0.0, 0)
    if lib.ft_scene_build_bricks(scene.handle, ctypes.byref(o), ctypes.byref(info)) != 0:
        raise RuntimeError(_native.last_error())
    out = _depth_figures(lib, scene, w, dev, stream, flush, peak, _native.FT_FLAG_FP16_BRICKS)
    a = Renderer(lib, scene, w, "depth", dev, stream, 0)
    b = Renderer(lib, scene, w, "depth", dev, stream, _native.FT_FLAG_FP16_BRICKS)
    a()
    b()
    torch.cuda.synchronize()
    ma, mb = a.m.cpu().numpy(), b.m.cpu().numpy()
    ta, tb = a.t.cpu().numpy().astype(np.float64), b.t.cpu().numpy().astype(np.float64)
    both = (ma == 1) & (mb == 1)
    err = np.abs(ta[both] - tb[both]) if both.any() else np.zeros(1)
    out["vs_plain_fp32"] = {"mask_agreement": float((ma == mb).mean()),
                            "depth_err_max": float(err.max()), "depth_err_q999": float(np.quantile(err, 0.999)),
                            "depth_within_1e-4": float((err <= 1e-4).mean())}
    out["bricks"] = {"voxel_size": 0.02, "brick_voxels": 8, "storage": "fp16 9^3 texels, trilinear texture fetch",
                     "near_bricks": info.near_bricks, "cells": list(info.bricks), "exact_leaves": info.exact_leaves,
                     "band": info.band, "max_lipschitz": info.max_lipschitz, "device_bytes": info.device_bytes,
                     "build_ms": info.build_ms}
    return out


def _cuda_ms(fn, reps: int) -> float:
    """Median CUDA-event time of fn() on the current stream (fn synchronises)."""
    import torch

    s = torch.cuda.current_stream()
    out = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        fn()
        b.record(s)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return float(statistics.median(out))


def precision_form(reps: int = 2) -> dict:
    """Hooked 4096-shell scene (domain rotate_y(p, p.y*18), distance_post
    abs(d + sin(p.y*120)*0.004) - 0.03 on every sphere), 1920x1080 depth:
    the plain FP32 march with the hook interpreter, the run-time compiled
    (NVRTC) kernels, and the FP16 brick form on top of them."""
    import numpy as np

    import forgedthoughts_gb300 as ft
    from forgedthoughts_gb300 import workloads

    w = workloads.twisted_shells()
    st = ft.parse_and_eval(w.source)
    g = st.gpu()
    items = w.options.width * w.options.height * w.aa
    ft.render_depth(st, w.options, w.accel, 1)  # warm-up
    plain_ms = _cuda_ms(lambda: ft.render_depth(st, w.options, w.accel, 1, want_rgb8=False), reps)
    ref = ft.render_depth(st, w.options, w.accel, 1)
    _log(f"  plain {plain_ms:.1f} ms; NVRTC compile")
    t0 = time.perf_counter()
    jit = g.jit()
    jit["wall_ms"] = 1000.0 * (time.perf_counter() - t0)
    _log(f"  compiled in {jit['wall_ms']:.0f} ms")
    ft.render_depth(st, w.options, w.accel, 1)
    jit_ms = _cuda_ms(lambda: ft.render_depth(st, w.options, w.accel, 1, want_rgb8=False), reps)
    jimg = ft.render_depth(st, w.options, w.accel, 1)
    # 1-bounce shading (Whitted depth 2) of the compiled scene
    shade = lambda bricks: ft.render_trace(st, w.options, w.accel, 1, 2, fp16_bricks=bricks)  # noqa: E731
    shade(False)
    jit_shaded_ms = _cuda_ms(lambda: shade(False), reps)
    jlin = shade(False)[0]
    info = g.build_bricks()
    ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    b_ms = _cuda_ms(lambda: ft.render_depth(st, w.options, w.accel, 1, want_rgb8=False, fp16_bricks=True), reps)
    bimg = ft.render_depth(st, w.options, w.accel, 1, fp16_bricks=True)
    shade(True)
    b_shaded_ms = _cuda_ms(lambda: shade(True), reps)
    blin = shade(True)[0]
    _log(f"  shaded: compiled {jit_shaded_ms:.0f} ms, compiled + bricks {b_shaded_ms:.0f} ms")

    def agree(a, b):
        both = (a.mask == 1) & (b.mask == 1)
        err = np.abs(a.t[both].astype(np.float64) - b.t[both]) if both.any() else np.zeros(1)
        return {"mask_agreement": float((a.mask == b.mask).mean()), "depth_err_q999": float(np.quantile(err, 0.999)),
                "depth_within_1e-4": float((err <= 1e-4).mean())}

    mr = lambda ms: items / (ms * 1e-3) / 1e6  # noqa: E731
    return {"workload": w.name, "primary_samples": items, "unit": UNIT,
            "plain_fp32_interpreter": {"value": mr(plain_ms), "ms": plain_ms},
            "jit_nvrtc": {"value": mr(jit_ms), "ms": jit_ms, "speedup_vs_plain": plain_ms / jit_ms,
                          "vs_plain": agree(ref, jimg), "compile": jit},
            "jit_fp16_bricks": {"value": mr(b_ms), "ms": b_ms, "speedup_vs_plain": plain_ms / b_ms,
                                "vs_plain": agree(ref, bimg),
                                "bricks": {"build_ms": info.build_ms, "device_bytes": info.device_bytes,
                                           "max_lipschitz": info.max_lipschitz, "near_bricks": info.near_bricks}},
            "shaded_1_bounce": {
                "what": "Whitted depth 2 (primary hit, lights, shadows, one bounce), 1 spp",
                "jit_nvrtc": {"value": mr(jit_shaded_ms), "ms": jit_shaded_ms},
                "jit_fp16_bricks": {"value": mr(b_shaded_ms), "ms": b_shaded_ms,
                                    "speedup_vs_jit": jit_shaded_ms / b_shaded_ms,
                                    "radiance_rmse_vs_jit": float(np.sqrt(np.mean(
                                        (blin.astype(np.float64) - jlin) ** 2)))}}}


def batched_form(reps: int = 3) -> dict:
    """256 independent scenes (8..2048 spheres, 64^2..512^2, half depth
    previews, half Whitted depth 2) in one CUDA-graph launch, autotuned, FP32
    and FP16-brick; against the same renders launched one by one."""
    import forgedthoughts_gb300 as ft
    from forgedthoughts_gb300 import workloads

    ws = workloads.batch_scenes()
    t0 = time.perf_counter()
    states = [ft.parse_and_eval(w.source) for w in ws]
    for st in states:
        st.gpu()
    setup_ms = 1000.0 * (time.perf_counter() - t0)
    _log(f"  {len(ws)} scenes set up in {setup_ms:.0f} ms")
    items = [(st, w.options, w.aa, w.max_depth) for st, w in zip(states, ws)]

    import torch

    from forgedthoughts_gb300 import _native

    lib = _native.lib()
    big = max(w.options.width * w.options.height * w.aa for w in ws)
    d_t = torch.empty(big, dtype=torch.float32, device="cuda")
    d_m = torch.empty(big, dtype=torch.uint8, device="cuda")
    d_rgb = torch.empty(big * 3, dtype=torch.float32, device="cuda")
    d_rgb8 = torch.empty(big * 3, dtype=torch.uint8, device="cuda")
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    copts = [w.options.to_c() for w in ws]

    def one_by_one():
        # the same renders through the C ABI, one call per scene, device outputs
        for st, w, o in zip(states, ws, copts):
            if w.max_depth == 0:
                rc = lib.ft_render_depth(st.gpu().handle, ctypes.byref(o), int(w.accel), w.aa, p(d_t), p(d_m), None,
                                         None, p(d_rgb8), _native.FT_FLAG_DEVICE_POINTERS, None)
            else:
                rc = lib.ft_render_trace(st.gpu().handle, ctypes.byref(o), int(w.accel), w.aa, w.max_depth, p(d_rgb),
                                         p(d_rgb8), _native.FT_FLAG_DEVICE_POINTERS, None)
            if rc != 0:
                raise RuntimeError(_native.last_error())

    one_by_one()
    seq_ms = _cuda_ms(one_by_one, 1)
    _log(f"  one by one {seq_ms:.1f} ms; autotune")
    b32 = ft.Batch(items)
    n = b32.samples()
    tune32 = b32.autotune()
    ms32 = _cuda_ms(lambda: (b32.launch(), __import__("torch").cuda.synchronize()), reps)
    t0 = time.perf_counter()
    for st, w in zip(states, ws):
        if w.max_depth == 0:
            st.gpu().build_bricks()
    bricks_ms = 1000.0 * (time.perf_counter() - t0)
    b16 = ft.Batch(items, fp16_bricks=True)
    tune16 = b16.autotune()
    ms16 = _cuda_ms(lambda: (b16.launch(), __import__("torch").cuda.synchronize()), reps)
    mr = lambda ms: n / (ms * 1e-3) / 1e6  # noqa: E731
    return {"scenes": len(ws), "primary_samples": n, "unit": UNIT, "host_setup_ms": setup_ms,
            "one_by_one": {"value": mr(seq_ms), "ms": seq_ms, "how": "one C-ABI call per scene, device outputs"},
            "batched_fp32": {"value": mr(ms32), "ms": ms32, "tuning": tune32, "speedup_vs_one_by_one": seq_ms / ms32},
            "batched_fp16_bricks": {"value": mr(ms16), "ms": ms16, "tuning": tune16,
                                    "speedup_vs_one_by_one": seq_ms / ms16, "brick_build_ms": bricks_ms}}


def differentiation_form(adam_steps: int = 200, reps: int = 3) -> dict:
    """Inverse shape fitting: 64 primitives (32 spheres, 32 boxes) in a
    union_round(0.15) tree, 449 parameters, 64 views at 256^2 on a ring of
    radius 5 at height 1.5; loss = L2(depth on pixels both renders hit) +
    L2(soft silhouette).  Times the forward + adjoint march (gradient
    evaluations per second) and runs Adam from the seed-7 init towards the
    target (init + N(0, 0.05))."""
    import numpy as np

    import forgedthoughts_gb300 as ft
    from forgedthoughts_gb300 import workloads

    src = workloads.shape_fit()
    ps = ft.ParamScene(src)
    opts = workloads.shape_fit_options(256)
    views = ft.ring_views(64)
    theta0 = ps.get_params()
    rng = np.random.default_rng(7)
    target_params = (theta0 + rng.normal(0.0, 0.05, size=theta0.shape)).astype(np.float32)
    ps.set_params(target_params)
    tt, tm, ts = ps.render(views, opts)
    ps.set_params(theta0)

    def loss_and_grad(theta):
        ps.set_params(theta)
        t, m, s = ps.render(views, opts)
        both = (m == 1) & (tm == 1)
        dt = np.where(both, 2.0 * (t - tt), 0.0).astype(np.float32)
        ds = (2.0 * (s - ts)).astype(np.float32)
        loss = float(np.sum(np.where(both, (t - tt) ** 2, 0.0)) + np.sum((s - ts) ** 2))
        return loss, ps.backward(views, opts, dt, ds)

    loss_and_grad(theta0)
    rays = len(views) * opts.width * opts.height
    t0 = time.perf_counter()
    for _ in range(reps):
        loss_and_grad(theta0)
    step_s = (time.perf_counter() - t0) / reps
    # Adam with a cosine-decayed step and an epsilon tied to the largest
    # gradient scale: Adam's per-parameter normalisation would otherwise move
    # weakly observed parameters (rotations in degrees, primitives hidden by
    # others) as fast as well observed ones, and they drift.
    _, g0 = loss_and_grad(theta0)
    active = np.abs(g0) > 0
    theta = theta0.astype(np.float64).copy()
    mom, vel = np.zeros_like(theta), np.zeros_like(theta)
    lr, b1, b2, eps_rel = 0.003, 0.9, 0.999, 1e-2
    losses = []
    _log(f"  forward + adjoint {1000 * step_s:.1f} ms; Adam")
    for k in range(1, adam_steps + 1):
        if k % 50 == 0:
            _log(f"  Adam step {k}")
        loss, g = loss_and_grad(theta.astype(np.float32))
        losses.append(loss)
        mom = b1 * mom + (1 - b1) * g
        vel = b2 * vel + (1 - b2) * g * g
        step = lr * 0.5 * (1 + np.cos(np.pi * (k - 1) / adam_steps))
        vhat = vel / (1 - b2 ** k)
        theta -= step * (mom / (1 - b1 ** k)) / (np.sqrt(vhat) + eps_rel * np.sqrt(vhat.max()) + 1e-12)
    final, _ = loss_and_grad(theta.astype(np.float32))
    err0 = float(np.sqrt(np.mean((theta0 - target_params) ** 2)))
    err1 = float(np.sqrt(np.mean((theta - target_params) ** 2)))
    err0a = float(np.sqrt(np.mean((theta0 - target_params)[active] ** 2)))
    err1a = float(np.sqrt(np.mean((theta - target_params)[active] ** 2)))
    return {"params": ps.n_params, "views": len(views), "rays_per_pass": rays,
            "forward_backward_s": step_s, "gradient_evaluations_per_s": 1.0 / step_s,
            "grads_per_s": rays * ps.n_params / step_s,
            "grads_per_s_definition": "rays x parameters per second of forward + adjoint march",
            "adam": {"steps": adam_steps, "lr": lr, "schedule": "cosine decay", "eps": "1e-2 x largest gradient scale",
                     "loss_first": losses[0], "loss_last": final,
                     "param_rmse_to_target_init": err0, "param_rmse_to_target_final": err1,
                     "params_with_gradient": int(active.sum()),
                     "param_rmse_with_gradient_init": err0a, "param_rmse_with_gradient_final": err1a}}


def _traffic_summary(kernel: str, w) -> tuple:
    """Per-launch DRAM bytes of a kernel from its committed ncu summary, and
    the summary's own note on the state it was captured in (None, None when
    there is no summary for this workload)."""
    prof = ROOT / "profiles" / f"{kernel}_traffic.txt"
    if not prof.exists() or not w.name.startswith("union_round512"):
        return None, None
    full = w.options.width * w.options.height * w.aa
    lines = prof.read_text().splitlines()
    state = next((ln[2:].strip() for ln in lines if ln.startswith("# State captured:")), None)
    for ln in lines:
        if ln.startswith(f"bytes_per_full_launch[{full}]:"):
            return int(ln.split(":", 1)[1]), state
    return None, None



def _e2e(lib, st, w, mode: str, steps: int):
    """The same render through the public C ABI with host buffers: scene upload
    (host -> device), render, outputs copied back to pinned host memory."""
    import torch

    from forgedthoughts_gb300 import _native

    opts = w.options.to_c()
    pixels = w.options.width * w.options.height
    items = pixels * w.aa
    pin = lambda n, dt: torch.empty(n, dtype=dt, pin_memory=True)  # noqa: E731
    p = lambda x: ctypes.c_void_p(x.data_ptr())  # noqa: E731
    if mode == "trace":
        h_rgbf, h_rgb = pin(pixels * 3, torch.float32), pin(pixels * 3, torch.uint8)
        d2h = pixels * 3 * 4 + pixels * 3
    else:
        h_t, h_m, h_mat = pin(items, torch.float32), pin(items, torch.uint8), pin(items, torch.int32)
        h_n, h_rgb = pin(items * 3, torch.float32), pin(pixels * 3, torch.uint8)
        d2h = items * (4 + 1 + 4 + 12) + pixels * 3
    times, h2d = [], 0
    for k in range(steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        handle = ctypes.c_void_p()
        if lib.ft_scene_create(st.desc_ptr, ctypes.byref(handle)) != 0:
            raise RuntimeError(_native.last_error())
        if mode == "trace":
            rc = lib.ft_render_trace(handle, ctypes.byref(opts), int(w.accel), w.aa, w.max_depth, p(h_rgbf), p(h_rgb),
                                     0, None)
        else:
            rc = lib.ft_render_depth(handle, ctypes.byref(opts), int(w.accel), w.aa, p(h_t), p(h_m), p(h_mat), p(h_n),
                                     p(h_rgb), 0, None)
        nbytes = ctypes.c_uint64(0)
        lib.ft_scene_device_bytes(handle, ctypes.byref(nbytes))
        lib.ft_scene_destroy(handle)
        if rc != 0:
            raise RuntimeError(_native.last_error())
        if k > 0:  # first call pays one-time CUDA module and allocator set-up
            times.append(time.perf_counter() - t0)
        h2d = int(nbytes.value) + ctypes.sizeof(opts)
    value = items / statistics.mean(times) / 1e6 if times else None
    return {"value": value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "includes": "scene upload + accelerator build + render + output copy to pinned host"}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0, help="timed steps (default 10 trace / 30 depth)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["trace", "depth"], default="trace")
    ap.add_argument("--workload", default="union_round")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the precision, batched and differentiation forms")
    ap.add_argument("--adam-steps", type=int, default=200)
    ap.add_argument("--width", type=int, default=0, help="override the workload's width (profiling runs)")
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--aa", type=int, default=0)
    ap.add_argument("--max-depth", type=int, default=0)
    args = ap.parse_args()
    if args.steps <= 0:
        args.steps = 10 if args.mode == "trace" else 30
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    from forgedthoughts_gb300.build import build_all

    build_all()
    w = workload(args.workload)
    if args.width:
        w.options.width = args.width
    if args.height:
        w.options.height = args.height
    if args.aa:
        w.aa = args.aa
    if args.width or args.height or args.aa:
        w.name = f"{w.name}_resized_to_{w.options.width}x{w.options.height}_aa{w.aa}"
    if args.max_depth:
        w.max_depth = args.max_depth
    if args.mode == "trace" and w.max_depth <= 0:
        w.max_depth = 6
    if args.impl == "reference":
        run_reference(args, w)
        return

    import torch

    import forgedthoughts_gb300 as ft
    from forgedthoughts_gb300 import _native

    rank, world, local = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1), _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    lib = _native.lib()
    st = ft.parse_and_eval(w.source)
    scene = st.gpu()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    r = Renderer(lib, scene, w, args.mode, dev, stream)
    items = r.items

    clocks = ClockSampler(local)
    _log(f"{args.mode}: {args.warmup} warm-up + {args.steps} timed steps")
    clocks.start()
    for _ in range(args.warmup):
        r()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    r.launches = 0
    lib.ft_scene_profile(scene.handle, 1)  # CUDA events around every launch of the timed steps
    step_ms = _time_steps(r, args.steps, stream, flush)
    times = kernel_times(lib, scene, args.steps)
    lib.ft_scene_profile(scene.handle, 0)
    timed_launches = r.launches
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms, value = replica_throughput(sum(step_ms), items, args.steps, world, dist, dev)
    ms_per_step = total_ms / args.steps

    peak = ctypes.c_double(0.0)
    if lib.ft_measure_fp32_peak(ctypes.byref(peak)) != 0:
        raise RuntimeError(_native.last_error())

    # Dominant kernel: the trace's wavefront ray march (or the depth march),
    # timed by the CUDA events of the timed steps, FLOPs from the counting
    # variants of the same kernels.
    if args.mode == "trace":
        roofline = trace_roofline(r, times, peak.value)
    else:
        roofline = depth_roofline(r, times, peak.value)
    roofline["traffic"], note = _traffic_summary(roofline["kernel"], w)
    if note:
        roofline["traffic_source"] = note
    roofline["kernel_times_per_step"] = {k: {"ms": v[0], "launches": v[1]} for k, v in times.items()}

    _log("roofline done; end-to-end steps")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
        "config": _config(w, args.mode, world),
        "roofline": roofline,
        "e2e": None if args.no_e2e else _e2e(lib, st, w, args.mode, min(args.steps, 5)),
        "clocks": clk,
        "gpu_launches": timed_launches,
    }
    _log("secondary figures")
    if not args.no_secondary:
        plain = None
        if args.mode == "trace":
            # The plain depth march of the same frame: the plain FP32 form.
            plain = _depth_figures(lib, scene, w, dev, stream, flush, peak.value, 0)
            line["depth_march"] = plain
        else:
            plain = {"value": value}
        # The FP16 brick precision form of the same depth march.
        fp16 = _brick_figures(lib, scene, w, dev, stream, flush, peak.value)
        fp16["speedup_vs_plain_fp32"] = fp16["value"] / plain["value"]
        line["depth_march_fp16_bricks"] = fp16
    if rank == 0 and not args.no_forms:
        # the precision, batching and differentiation forms beside the plain method
        forms = {}
        for name, fn in (("precision_fp16_bricks_and_jit", precision_form), ("batched", batched_form),
                         ("differentiation", lambda: differentiation_form(args.adam_steps))):
            _log(name)
            try:
                forms[name] = fn()
            except Exception as exc:  # a failing form is reported, the line still printed
                forms[name] = {"error": f"{type(exc).__name__}: {exc}"}
                _log(f"  {name} failed: {exc}")
        line["forms"] = forms
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        _log("cpu baseline")
        line["cpu_baseline"] = cpu_baseline(w, args.mode)
    _log("done")
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    st.close()


if __name__ == "__main__":
    main()
