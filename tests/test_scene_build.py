"""Host-side culling structures (no device needed): leaf classification, the
union_round candidate grid, and rejection of malformed scene descriptions."""
import ctypes

import pytest

import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native, workloads


def build_info(desc_ptr):
    info = _native.BuildInfoC()
    rc = _native.lib().ft_scene_build_info(desc_ptr, ctypes.byref(info))
    return rc, info


def test_leaf_classification():
    st = ft.parse_and_eval(workloads.spheres_on_ground().source)
    rc, info = build_info(st.desc_ptr)
    assert rc == 0 and info.leaves == 9 and info.primitive_leaves == 9 and info.grid_cells == 0
    st = ft.parse_and_eval(workloads.twisted_shells(n=64, width=8, height=8).source)
    rc, info = build_info(st.desc_ptr)
    assert rc == 0 and info.generic_leaves == 64 and info.primitive_leaves == 1


def test_union_round_candidate_grid():
    st = ft.parse_and_eval(workloads.union_round_field().source)
    rc, info = build_info(st.desc_ptr)
    assert rc == 0
    assert info.union_round_leaves == 1 and info.primitive_leaves == 1
    assert info.grid_cells > 10000
    assert info.grid_entries / info.grid_cells < 16  # short candidate lists
    assert 0 < info.grid_max_list <= 64


@pytest.mark.parametrize("n,seed,cells,entries,max_list", [
    (512, 1, 135050, 639791, 23),
    (200, 5, 54450, 218559, 17),
    (64, 3, 18252, 54592, 12),
])
def test_candidate_grid_matches_the_full_scan(n, seed, cells, entries, max_list):
    """The grid is built in blocks whose primitive subsets are pruned by
    bounds; every cell's list must still be the one a scan of all primitives
    gives.  The expected counts are those of that full scan (every cell
    against every primitive) on the same trees."""
    st = ft.parse_and_eval(workloads.union_round_field(n=n, seed=seed).source)
    rc, info = build_info(st.desc_ptr)
    assert rc == 0
    assert (info.grid_cells, info.grid_entries, info.grid_max_list) == (cells, entries, max_list)


def _overlapping_spheres(n: int) -> str:
    """A balanced union_round tree of n nearly concentric spheres: every grid
    cell would list every primitive."""
    lines = [f"let p{i} = Sphere {{ radius: {0.5 + 0.0001 * i:.6f}, pos: vec3({0.001 * (i % 7):.4f}, 1, 0) }};"
             for i in range(n)]
    cur, lvl = [f"p{i}" for i in range(n)], 0
    while len(cur) > 1:
        nxt = []
        for j in range(0, len(cur) - 1, 2):
            lines.append(f"let v{lvl}_{j // 2} = {cur[j]}.union_round({cur[j + 1]}, 0.1);")
            nxt.append(f"v{lvl}_{j // 2}")
        cur, lvl = nxt + cur[len(cur) - len(cur) % 2:], lvl + 1
    lines.append(f"let scene = {cur[0]};")
    return "\n".join(lines)


def test_candidate_grid_is_dropped_past_its_entry_cap():
    """1200 overlapping spheres would give about 93 M list entries.  Past 2^26
    entries the tree keeps no grid and is evaluated through its BVH."""
    st = ft.parse_and_eval(_overlapping_spheres(1200))
    rc, info = build_info(st.desc_ptr)
    assert rc == 0 and info.union_round_leaves == 1
    assert info.grid_cells == 0 and info.grid_entries == 0


_OOM_CHILD = r"""
import ctypes, resource, sys
sys.path.insert(0, sys.argv[1])
import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native
sys.path.insert(0, sys.argv[2])
from test_scene_build import _overlapping_spheres
st = ft.parse_and_eval(_overlapping_spheres(1200))
info = _native.BuildInfoC()
lib = _native.lib()
soft, hard = resource.getrlimit(resource.RLIMIT_AS)
vm = int(open("/proc/self/statm").read().split()[0]) * resource.getpagesize()
resource.setrlimit(resource.RLIMIT_AS, (vm + (256 << 20), hard))
rc = lib.ft_scene_build_info(st.desc_ptr, ctypes.byref(info))
resource.setrlimit(resource.RLIMIT_AS, (soft, hard))
print(rc, _native.last_error())
"""


def test_host_allocation_failure_returns_a_status():
    """A failed host allocation inside the scene builder, here in its worker
    threads, comes back as FT_ERR_OUT_OF_MEMORY: no C++ exception crosses the
    C ABI (an escaping one would abort the process).  The child process caps
    its address space 256 MB above its size, and the tree's grid needs more
    than 500 MB before it reaches its entry cap.  The child's allocator keeps
    one arena: with one per worker thread, each reserving 64 MB of address
    space under the cap, the allocation of a new thread's thread-local block
    could be the one that fails, which glibc answers by ending the process
    ("cannot allocate memory for thread-local data") rather than with a
    status.  The builder's workers and its calling thread touch that block
    before any of them allocates for the grid."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    if not Path("/proc/self/statm").exists():
        pytest.skip("needs /proc")
    here = Path(__file__).resolve().parent
    env = dict(os.environ, MALLOC_ARENA_MAX="1", GLIBC_TUNABLES="glibc.malloc.arena_max=1")
    p = subprocess.run([sys.executable, "-c", _OOM_CHILD, str(here.parent), str(here)],
                       capture_output=True, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    rc, msg = p.stdout.strip().split(" ", 1)
    assert int(rc) == _native.FT_ERR_OUT_OF_MEMORY, p.stdout
    assert "host" in msg


def test_polygon_trees_take_the_generic_path():
    src = "let scene = " + ".union_round(".join(
        f"ExtrudePolygon {{ sides: 5, radius: 0.3, pos: vec3({i}, 0, 0) }}" for i in range(4)) + ", 0.1)" * 3 + ";"
    st = ft.parse_and_eval(src)
    rc, info = build_info(st.desc_ptr)
    assert rc == 0 and info.union_round_leaves == 0 and info.generic_leaves == 1


@pytest.mark.parametrize("field,value", [("root", 10 ** 6), ("abi_version", 99), ("n_nodes", 0)])
def test_malformed_descriptions_are_rejected(field, value):
    st = ft.parse_and_eval(workloads.spheres_on_ground().source)
    bad = _native.SceneDescC.from_buffer_copy(st.desc)
    setattr(bad, field, value)
    rc, _ = build_info(ctypes.pointer(bad))
    assert rc == _native.FT_ERR_INVALID_ARGUMENT
    assert _native.last_error()


def test_bad_child_index_is_rejected():
    st = ft.parse_and_eval(workloads.union_round_field(n=8, width=8, height=8).source)
    d = st.desc
    nodes = (_native.NodeC * d.n_nodes)()
    ctypes.memmove(nodes, d.nodes, ctypes.sizeof(nodes))
    for i in range(d.n_nodes):
        if nodes[i].kind == 11:
            nodes[i].b = 10 ** 6
            break
    bad = _native.SceneDescC.from_buffer_copy(d)
    bad.nodes = ctypes.cast(nodes, ctypes.POINTER(_native.NodeC))
    rc, _ = build_info(ctypes.pointer(bad))
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "child" in _native.last_error()


def _with_materials(st, mutate):
    d = st.desc
    mats = (_native.MaterialC * d.n_materials)()
    ctypes.memmove(mats, d.materials, ctypes.sizeof(mats))
    mutate(mats, d)
    bad = _native.SceneDescC.from_buffer_copy(d)
    bad.materials = ctypes.cast(mats, ctypes.POINTER(_native.MaterialC))
    return build_info(ctypes.pointer(bad))


def test_material_hook_programs_are_validated():
    """A material hook program must exist and map the shading context to a
    colour (colour hook) or a number (the others)."""
    from test_frontend import HOOK_MATERIALS

    st = ft.parse_and_eval(HOOK_MATERIALS + "let scene = Sphere { material: Stripe {} } + "
                           "Sphere { pos: vec3(3.0, 0.0, 0.0), material: RoughStripe {} };\n")
    rc, _ = build_info(st.desc_ptr)
    assert rc == 0

    def bad_index(mats, d):
        for i in range(d.n_materials):
            if mats[i].color_program >= 0:
                mats[i].color_program = d.n_programs + 5

    rc, _ = _with_materials(st, bad_index)
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "hook program" in _native.last_error()

    def colour_as_roughness(mats, d):
        for i in range(d.n_materials):
            if mats[i].color_program >= 0:
                mats[i].roughness_program = mats[i].color_program  # returns a vec3

    rc, _ = _with_materials(st, colour_as_roughness)
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "number" in _native.last_error()


def test_custom_sdf_nodes_are_validated():
    """A Custom node needs a distance program mapping vec3 to a number,
    optional domain / distance_post programs of the right shape and positive
    bounds."""
    from test_frontend import CUSTOM_SCENE

    st = ft.parse_and_eval(CUSTOM_SCENE)
    d = st.desc
    rc, info = build_info(st.desc_ptr)
    assert rc == 0 and info.generic_leaves == 3

    def mutated(fn):
        nodes = (_native.NodeC * d.n_nodes)()
        ctypes.memmove(nodes, d.nodes, ctypes.sizeof(nodes))
        for i in range(d.n_nodes):
            if nodes[i].kind == 30 and nodes[i].ival >= 0:
                fn(nodes[i])
                break
        bad = _native.SceneDescC.from_buffer_copy(d)
        bad.nodes = ctypes.cast(nodes, ctypes.POINTER(_native.NodeC))
        return build_info(ctypes.pointer(bad))

    for fn in (lambda n: setattr(n, "program", n.ival),      # distance returning a vec3
               lambda n: setattr(n, "reserved", n.program),  # distance_post with one parameter
               lambda n: setattr(n, "program", -1)):         # no distance
        rc, _ = mutated(fn)
        assert rc == _native.FT_ERR_INVALID_ARGUMENT and "custom sdf" in _native.last_error()

    def no_bounds(n):
        n.f[0] = 0.0

    rc, _ = mutated(no_bounds)
    assert rc == _native.FT_ERR_INVALID_ARGUMENT and "bounds" in _native.last_error()
