"""The C ABI library loads and exports every symbol include/*.h declares."""
import ctypes
import re

import pytest

from conftest import ROOT
from forgedthoughts_gb300 import _native


def declared_symbols():
    names = set()
    for header in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        for m in re.finditer(r"\b(ft_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("ft_scene_create", "ft_scene_destroy", "ft_render_depth", "ft_last_error",
                     "ft_scene_desc_from_source", "ft_scene_desc_free"):
        assert required in names


@pytest.mark.parametrize("name", declared_symbols())
def test_library_exports_symbol(name):
    lib = _native.lib()
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_python_binding_covers_header():
    assert set(declared_symbols()) <= set(_native.SIGNATURES)


def test_abi_version():
    assert _native.lib().ft_abi_version() == _native.FT_ABI_VERSION


def test_null_arguments_are_rejected():
    lib = _native.lib()
    assert lib.ft_scene_desc_from_source(None, None) == _native.FT_ERR_INVALID_ARGUMENT
    assert "non-null" in _native.last_error()
    assert lib.ft_scene_create(None, None) == _native.FT_ERR_INVALID_ARGUMENT
    assert lib.ft_render_depth(None, None, 0, 1, None, None, None, None, None, 0, None) == \
        _native.FT_ERR_INVALID_ARGUMENT
    lib.ft_scene_destroy(None)
    lib.ft_scene_desc_free(None)


def test_description_view_keeps_its_state_alive():
    """`parse_and_eval(src).desc` outlives the temporary state: the view holds
    the state that owns the native description."""
    import gc

    import forgedthoughts_gb300 as ft

    d = ft.parse_and_eval("var a = Sphere{}; var b = Box { size: vec3(1.0) }; let scene = a & b;").desc
    gc.collect()
    others = [ft.parse_and_eval("let scene = Torus {};") for _ in range(20)]  # reuse freed memory, if any
    root = d.nodes[d.root]
    assert root.kind == 9 and d.nodes[root.a].kind == _native.FT_NODE_SPHERE  # FT_NODE_INTERSECT
    assert d.nodes[root.b].kind == _native.FT_NODE_BOX and len(others) == 20
