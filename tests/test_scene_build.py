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
