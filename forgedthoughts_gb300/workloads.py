"""Seeded synthetic `.ft` scenes for the benchmark and parity workloads.

There is no public benchmark suite for this renderer; each workload is a
generated scene with the shapes, sizes and value distributions of the
configuration it stands for.  All randomness comes from
``numpy.random.default_rng(seed)`` with a fixed draw order per primitive.

Number literals are printed in positional notation: the `.ft` lexer accepts
only digit/dot runs (crates/forgedthoughts/src/lexer.rs:152-171) and the
evaluator rounds each literal to f32, so the shortest f32-round-tripping
decimal is emitted.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import AccelMode, RenderOptions


def num(v: float) -> str:
    s = np.format_float_positional(np.float32(v), unique=True, trim="-")
    return s


def v3(x: float, y: float, z: float) -> str:
    return f"vec3({num(x)}, {num(y)}, {num(z)})"


@dataclasses.dataclass
class Workload:
    name: str
    source: str
    options: RenderOptions
    accel: AccelMode
    aa: int
    max_depth: int = 0  # Whitted bounce depth (0: depth preview)


GROUND = "var ground = Box { size: vec3(220, 1, 220) };\nground.pos.y = -0.5;\n"

SKY = """environment Sky {
  let zenith = #6ea3ff;
  let horizon = #dfeeff;

  fn color(dir) {
    return mix(horizon, zenith, clamp(dir.y * 0.5 + 0.5, 0.0, 1.0));
  }
};
"""


def _march_options(width: int, height: int) -> RenderOptions:
    # max 256 steps, hit epsilon 1e-4, max distance 100, step scale 0.7
    return RenderOptions(width=width, height=height, max_steps=256, max_dist=100.0, epsilon=0.0001, step_scale=0.7,
                         camera_z=6.0, fov_y_degrees=45.0)


def spheres_on_ground(n: int = 8, seed: int = 0, width: int = 256, height: int = 256) -> Workload:
    """Ground box (top face at y = 0) hard-unioned with n spheres.

    Radius U[0.2, 0.6], centre U([-2, 2] x [0.2, 1.5] x [-2, 2]); camera at
    (0, 1, -5) looking at the origin, vertical fov 45 degrees; Naive accel.
    """
    rng = np.random.default_rng(seed)
    lines = [f"let camera = Camera {{ origin: {v3(0, 1, -5)}, target: {v3(0, 0, 0)}, fov_y: 45.0 }};", GROUND]
    names = []
    for i in range(n):
        r = rng.uniform(0.2, 0.6)
        c = (rng.uniform(-2, 2), rng.uniform(0.2, 1.5), rng.uniform(-2, 2))
        lines.append(f"let s{i} = Sphere {{ radius: {num(r)}, pos: {v3(*c)} }};")
        names.append(f"s{i}")
    lines.append("let scene = ground + " + " + ".join(names) + ";")
    return Workload(f"spheres{n}_ground_{width}x{height}", "\n".join(lines) + "\n", _march_options(width, height),
                    AccelMode.Naive, 1)


def union_round_field(n: int = 512, seed: int = 1, width: int = 1920, height: int = 1080, aa: int = 4,
                      k: float = 0.1, accel: AccelMode = AccelMode.Bricks, max_depth: int = 6) -> Workload:
    """n primitives in a balanced pairwise union_round(k) tree over a ground box.

    Even i: Sphere r U[0.1, 0.4]; odd i: Box with half size U[0.1, 0.35]^3.
    Centres U([-6, 6] x [0, 3] x [-6, 6]); rot.y U[0, 360) degrees.  Material
    Lambert (p 0.6, albedo U[0.2, 0.9]^3), Metal (p 0.25, roughness U[0, 0.4])
    or Dielectric (p 0.15, ior 1.5, roughness 0.02).  One PointLight at
    (4, 8, -4) with intensity 150, an EnvLight of radiance 0.2 and a sky
    gradient environment; camera (0, 4, -12) -> (0, 1, 0), fov 45.
    """
    rng = np.random.default_rng(seed)
    lines = [f"let camera = Camera {{ origin: {v3(0, 4, -12)}, target: {v3(0, 1, 0)}, fov_y: 45.0 }};",
             f"let key = PointLight {{ position: {v3(4, 8, -4)}, color: vec3(1, 1, 1), intensity: 150.0 }};",
             "let fill = EnvLight { color: vec3(1, 1, 1), intensity: 0.2 };", SKY, GROUND]
    prims = []
    for i in range(n):
        c = (rng.uniform(-6, 6), rng.uniform(0, 3), rng.uniform(-6, 6))
        if i % 2 == 0:
            size = f"radius: {num(rng.uniform(0.1, 0.4))}"
            kind = "Sphere"
        else:
            h = rng.uniform(0.1, 0.35, 3)
            size = f"size: {v3(2 * h[0], 2 * h[1], 2 * h[2])}"
            kind = "Box"
        rot = rng.uniform(0, 360)
        m = rng.choice(3, p=[0.6, 0.25, 0.15])
        if m == 0:
            a = rng.uniform(0.2, 0.9, 3)
            mat = f"Lambert {{ color: {v3(*a)} }}"
        elif m == 1:
            mat = f"Metal {{ roughness: {num(rng.uniform(0, 0.4))} }}"
        else:
            mat = "Dielectric { ior: 1.5, roughness: 0.02 }"
        lines.append(f"let p{i} = {kind} {{ {size}, pos: {v3(*c)}, rot: {v3(0, rot, 0)}, material: {mat} }};")
        prims.append(f"p{i}")
    level = 0
    while len(prims) > 1:
        nxt = []
        for j in range(0, len(prims) - 1, 2):
            name = f"u{level}_{j // 2}"
            lines.append(f"let {name} = {prims[j]}.union_round({prims[j + 1]}, {num(k)});")
            nxt.append(name)
        if len(prims) % 2:
            nxt.append(prims[-1])
        prims = nxt
        level += 1
    lines.append(f"let scene = ground + {prims[0]};")
    return Workload(f"union_round{n}_ground_{width}x{height}_aa{aa}", "\n".join(lines) + "\n",
                    _march_options(width, height), accel, aa, max_depth)


def twisted_shells(n: int = 4096, seed: int = 0, width: int = 1920, height: int = 1080) -> Workload:
    """As spheres_on_ground with n spheres, each carrying the hooks

    domain(p) = rotate_y(p, p.y * 18) and
    distance_post(d, p) = abs(d + sin(p.y * 120) * 0.004) - 0.03.
    """
    base = spheres_on_ground(0, seed, width, height)
    rng = np.random.default_rng(seed)
    lines = [base.source.split("let scene")[0],
             "let twist = fn(p) { return rotate_y(p, p.y * 18.0); };",
             "let ripple = fn(d, p) { return abs(d + sin(p.y * 120.0) * 0.004) - 0.03; };"]
    names = []
    for i in range(n):
        r = rng.uniform(0.2, 0.6)
        c = (rng.uniform(-2, 2), rng.uniform(0.2, 1.5), rng.uniform(-2, 2))
        lines.append(f"let s{i} = Sphere {{ radius: {num(r)}, pos: {v3(*c)}, domain: twist, distance_post: ripple }};")
        names.append(f"s{i}")
    lines.append("let scene = ground + " + " + ".join(names) + ";")
    return Workload(f"twisted_shells{n}_{width}x{height}", "\n".join(lines) + "\n", _march_options(width, height),
                    AccelMode.Bvh, 1, 2)


def batch_scenes(n: int = 256, first_seed: int = 0) -> list:
    """Independent scenes of uneven size for the batched launch.

    Scene i uses seed first_seed + i: primitive count round(exp(U[ln 8,
    ln 2048])) spheres drawn as in spheres_on_ground (radius U[0.2, 0.6],
    centre U([-2, 2] x [0.2, 1.5] x [-2, 2])) over the ground box; resolution
    uniform from {64^2, 128^2, 256^2, 512^2}; camera on the ring of radius 5 at
    height 1 around the origin at azimuth U[0, 2 pi), looking at the origin,
    fov 45; depth-only (p 0.5) or a Whitted trace of max depth 2.  One
    sample per pixel, Bvh accelerator.
    """
    out = []
    for i in range(n):
        rng = np.random.default_rng(first_seed + i)
        count = int(round(np.exp(rng.uniform(np.log(8), np.log(2048)))))
        res = int(rng.choice([64, 128, 256, 512]))
        az = rng.uniform(0, 2 * np.pi)
        trace = bool(rng.uniform() < 0.5)
        eye = (5.0 * np.sin(az), 1.0, -5.0 * np.cos(az))
        lines = [f"let camera = Camera {{ origin: {v3(*eye)}, target: {v3(0, 0, 0)}, fov_y: 45.0 }};", GROUND]
        names = []
        for j in range(count):
            r = rng.uniform(0.2, 0.6)
            c = (rng.uniform(-2, 2), rng.uniform(0.2, 1.5), rng.uniform(-2, 2))
            lines.append(f"let s{j} = Sphere {{ radius: {num(r)}, pos: {v3(*c)} }};")
            names.append(f"s{j}")
        lines.append("let scene = ground + " + " + ".join(names) + ";")
        out.append(Workload(f"batch{i}_spheres{count}_{res}x{res}_{'trace2' if trace else 'depth'}",
                            "\n".join(lines) + "\n", _march_options(res, res), AccelMode.Bvh, 1,
                            2 if trace else 0))
    return out


def shape_fit(n: int = 64, seed: int = 7, k: float = 0.15) -> str:
    """Inverse shape fitting scene: n primitives (even i sphere, odd i box) in a
    balanced pairwise union_round(k) tree, no ground.

    Centre U([-1.2, 1.2] x [-0.6, 0.8] x [-1.2, 1.2]); sphere radius
    U[0.15, 0.35]; box half size U[0.1, 0.3]^3; rot.y U[0, 360) degrees.  The
    parameter layout is 7 per primitive plus the shared radius (449 for 64).
    """
    rng = np.random.default_rng(seed)
    lines = []
    prims = []
    for i in range(n):
        c = (rng.uniform(-1.2, 1.2), rng.uniform(-0.6, 0.8), rng.uniform(-1.2, 1.2))
        if i % 2 == 0:
            size = f"radius: {num(rng.uniform(0.15, 0.35))}"
            kind = "Sphere"
        else:
            h = rng.uniform(0.1, 0.3, 3)
            size = f"size: {v3(2 * h[0], 2 * h[1], 2 * h[2])}"
            kind = "Box"
        rot = rng.uniform(0, 360)
        lines.append(f"let p{i} = {kind} {{ {size}, pos: {v3(*c)}, rot: {v3(0, rot, 0)} }};")
        prims.append(f"p{i}")
    level = 0
    while len(prims) > 1:
        nxt = []
        for j in range(0, len(prims) - 1, 2):
            name = f"u{level}_{j // 2}"
            lines.append(f"let {name} = {prims[j]}.union_round({prims[j + 1]}, {num(k)});")
            nxt.append(name)
        if len(prims) % 2:
            nxt.append(prims[-1])
        prims = nxt
        level += 1
    lines.append(f"let scene = {prims[0]};")
    return "\n".join(lines) + "\n"


def shape_fit_options(size: int = 256) -> RenderOptions:
    return _march_options(size, size)
