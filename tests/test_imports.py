"""Scene files with imports (no device needed).

The cases follow the reference's loader tests (crates/forgedthoughts/src/
lib.rs tests loads_relative_imports_once, loads_namespaced_imports,
loads_same_import_under_multiple_aliases, loads_namespaced_imported_functions,
imports_only_exported_names, namespaced_import_keeps_private_dependencies_
working, rejects_import_cycles).  The reference checks the spliced program's
bindings; this front-end returns only the lowered scene, so each multi-file
scene is compared byte for byte with the single-file scene the splice must
equal.  The reference's namespaced-import test loads its built-in library;
here the same definitions come from files beside the scene.
"""
import ctypes

import pytest

import forgedthoughts_gb300 as ft
from forgedthoughts_gb300 import _native


def _write(root, files):
    for name, text in files.items():
        p = root / name
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(text)
    return root


def _dump(st):
    """Every array and scalar of the lowered scene, as bytes."""
    d = st.desc

    def arr(ptr, n, ctype):
        return ctypes.string_at(ptr, n * ctypes.sizeof(ctype)) if n else b""

    return (arr(d.nodes, d.n_nodes, _native.NodeC), arr(d.instrs, d.n_instrs, _native.InstrC),
            arr(d.programs, d.n_programs, _native.ProgramC), arr(d.lights, d.n_lights, _native.LightC),
            arr(d.materials, d.n_materials, _native.MaterialC), d.root, d.environment_program,
            bytes(d.camera), d.has_camera, tuple(d.scene_center), d.settings_mask, bytes(d.settings),
            d.settings_accel)


def _same_scene(path, single_source):
    assert _dump(ft.load_and_eval_scene(path)) == _dump(ft.parse_and_eval(single_source))


def test_loads_relative_imports_once(tmp_path):
    """`shared.ft` is imported by both `a.ft` and `b.ft` but spliced once: the
    mutable radius it declares keeps the increment `a.ft` made when `b.ft`
    reads it."""
    _write(tmp_path, {
        "shared.ft": "let gold = Metal { color: vec3(0.9, 0.7, 0.3), roughness: 0.2 };\nvar r = 0.5;\n",
        "a.ft": 'import "./shared.ft"; r = r + 0.25; let left = Sphere { radius: r, material: gold };\n',
        "b.ft": 'import "./shared.ft";\nlet right = Sphere { radius: r, pos: vec3(2.0, 0.0, 0.0), material: gold };\n',
        "main.ft": 'import "./a.ft"; import "./b.ft"; let scene = left + right;\n',
    })
    single = ("let gold = Metal { color: vec3(0.9, 0.7, 0.3), roughness: 0.2 };\nvar r = 0.5;\n"
              "r = r + 0.25; let left = Sphere { radius: r, material: gold };\n"
              "let right = Sphere { radius: r, pos: vec3(2.0, 0.0, 0.0), material: gold };\n"
              "let scene = left + right;\n")
    _same_scene(tmp_path / "main.ft", single)
    radii = {round(n.f[0], 4) for n in ft.load_and_eval_scene(tmp_path / "main.ft").desc.nodes[:3]
             if n.kind == 0}
    assert radii == {0.75}


GOLD = """
material Gold {
  model: Metal;
  let warm = vec3(0.92, 0.72, 0.3);
  color = warm;
  roughness = 0.18;
  fn roughness(ctx) {
    return mix(0.1, 0.3, step(0.0, sin(ctx.local_position.x * 8.0)));
  }
};
"""

SOFT_BLOB = """
sdf SoftBlob {
  let warp_scale = 0.25;
  fn bounds() {
    return vec3(1.2, 1.2, 1.2);
  }
  fn warp(p) {
    return vec3(p.x, p.y + sin(p.x * 3.0) * warp_scale, p.z);
  }
  fn distance(p) {
    let q = warp(p);
    return length(q) - 1.0;
  }
};
"""


def test_loads_namespaced_imports(tmp_path):
    """Material and sdf definitions of aliased imports are reached as
    `alias.Name { ... }`, from files in subdirectories."""
    _write(tmp_path, {
        "materials/gold.ft": GOLD,
        "objects/soft_blob.ft": SOFT_BLOB,
        "main.ft": 'import "./materials/gold.ft" as gold;\nimport "./objects/soft_blob.ft" as blob;\n'
                   "let scene = blob.SoftBlob {\n  material: gold.Gold {}\n};\n",
    })
    single = GOLD + SOFT_BLOB + "let scene = SoftBlob {\n  material: Gold {}\n};\n"
    _same_scene(tmp_path / "main.ft", single)
    d = ft.load_and_eval_scene(tmp_path / "main.ft").desc
    assert d.n_programs >= 2  # the custom distance and the roughness hook


def test_loads_same_import_under_multiple_aliases(tmp_path):
    _write(tmp_path, {
        "shared.ft": "let mat = Metal { color: vec3(0.9, 0.7, 0.3), roughness: 0.2 };\n",
        "main.ft": 'import "./shared.ft" as warm;\nimport "./shared.ft" as copy;\n'
                   "let left = Sphere { material: warm.mat };\n"
                   "let right = Sphere { pos: vec3(2.0, 0.0, 0.0), material: copy.mat };\n"
                   "let scene = left + right;\n",
    })
    single = ("let mat = Metal { color: vec3(0.9, 0.7, 0.3), roughness: 0.2 };\n"
              "let left = Sphere { material: mat };\n"
              "let right = Sphere { pos: vec3(2.0, 0.0, 0.0), material: mat };\n"
              "let scene = left + right;\n")
    _same_scene(tmp_path / "main.ft", single)


HELPERS = """
fn accent() {
  return #ebc757;
}

fn make_gold() {
  return Metal { color: accent(), roughness: 0.2 };
}

export { make_gold };
"""


def test_loads_namespaced_imported_functions(tmp_path):
    """`palette.make_gold()` calls an exported function, which calls the
    file's private `accent()` under its qualified name."""
    _write(tmp_path, {
        "helpers.ft": HELPERS,
        "main.ft": 'import "./helpers.ft" as palette;\nlet scene = Sphere { material: palette.make_gold() };\n',
    })
    single = HELPERS.replace("export { make_gold };", "") + "let scene = Sphere { material: make_gold() };\n"
    _same_scene(tmp_path / "main.ft", single)


def test_material_hooks_call_qualified_functions(tmp_path):
    """A material hook of the scene file calls `lib.stripe(...)` and reads
    `lib.dark`; a hook inside the imported file calls its own helper, which
    the alias qualifies.  Both compile to the programs of the single-file
    scene."""
    lib = ("let dark = vec3(0.12, 0.14, 0.18);\n"
           "fn stripe(x) {\n  return step(0.0, sin(x * 8.0));\n}\n"
           "material Banded {\n  model: Lambert;\n"
           "  fn color(ctx) {\n    return mix(vec3(0.9), dark, stripe(ctx.local_position.y));\n  }\n};\n")
    main_mat = ("material Striped {\n  model: Lambert;\n"
                "  fn color(ctx) {\n    return mix(vec3(0.9, 0.7, 0.3), @DARK@, @STRIPE@(ctx.local_position.x));\n"
                "  }\n};\n")
    scene = ("let scene = Sphere { material: Striped {} } + "
             "Sphere { pos: vec3(3.0, 0.0, 0.0), material: @BANDED@ {} };\n")
    _write(tmp_path, {
        "lib.ft": lib,
        "main.ft": 'import "./lib.ft" as lib;\n' + main_mat.replace("@DARK@", "lib.dark").replace("@STRIPE@", "lib.stripe")
                   + scene.replace("@BANDED@", "lib.Banded"),
    })
    single = lib + main_mat.replace("@DARK@", "dark").replace("@STRIPE@", "stripe") + scene.replace("@BANDED@", "Banded")
    _same_scene(tmp_path / "main.ft", single)
    d = ft.load_and_eval_scene(tmp_path / "main.ft").desc
    assert d.n_materials >= 2 and all(d.materials[i].color_program >= 0 for i in range(d.n_materials))


MODULE = """
let private_color = #ebc757;
let public_mat = Metal { color: private_color, roughness: 0.2 };
let unused = 5.0;
export { public_mat };
"""


def test_imports_only_exported_names(tmp_path):
    """An exported binding brings what it reads (`private_color`); a binding
    that is neither exported nor read by an export is not imported."""
    _write(tmp_path, {
        "module.ft": MODULE,
        "main.ft": 'import "./module.ft";\nlet scene = Sphere { material: public_mat };\n',
        "bad.ft": 'import "./module.ft";\nlet scene = Sphere { radius: unused, material: public_mat };\n',
    })
    single = MODULE.replace("export { public_mat };", "") + "let scene = Sphere { material: public_mat };\n"
    _same_scene(tmp_path / "main.ft", single)
    with pytest.raises(ft.EvalError, match="undefined identifier 'unused'"):
        ft.load_and_eval_scene(tmp_path / "bad.ft")


def test_namespaced_import_keeps_private_dependencies_working(tmp_path):
    _write(tmp_path, {
        "module.ft": MODULE,
        "main.ft": 'import "./module.ft" as lib;\nlet scene = Sphere { material: lib.public_mat };\n',
        "bad.ft": 'import "./module.ft" as lib;\nlet scene = Sphere { radius: lib.unused, material: lib.public_mat };\n',
    })
    single = MODULE.replace("export { public_mat };", "") + "let scene = Sphere { material: public_mat };\n"
    _same_scene(tmp_path / "main.ft", single)
    with pytest.raises(ft.EvalError):
        ft.load_and_eval_scene(tmp_path / "bad.ft")


def test_exported_binding_keeps_its_assignments(tmp_path):
    """An assignment stays with the exported binding it writes; one to a
    dropped binding goes with it (lib.rs:976-984)."""
    _write(tmp_path, {
        "module.ft": "var size = 0.5;\nsize = size * 2.0;\nvar other = 1.0;\nother = 3.0;\n"
                     "let ball = Sphere { radius: size };\nexport { ball };\n",
        "main.ft": 'import "./module.ft" as m;\nlet scene = m.ball;\n',
    })
    _same_scene(tmp_path / "main.ft", "let scene = Sphere { radius: 1.0 };\n")


def test_scene_file_export_list_filters_the_scene_file(tmp_path):
    """The loader applies a file's export list to the file it was asked to
    load as well (lib.rs:354-373): a scene file exporting only `ball` loses
    its `scene` binding."""
    _write(tmp_path, {"main.ft": "let ball = Sphere {};\nlet scene = ball;\nexport { ball };\n"})
    with pytest.raises(ft.MissingSceneRoot):
        ft.load_and_eval_scene(tmp_path / "main.ft")


def test_rejects_import_cycles(tmp_path):
    _write(tmp_path, {
        "a.ft": 'import "./b.ft"; let a = 1.0; let scene = Sphere {};\n',
        "b.ft": 'import "./a.ft"; let b = 2.0;\n',
    })
    with pytest.raises(ft.ImportCycle) as e:
        ft.load_and_eval_scene(tmp_path / "a.ft")
    msg = str(e.value)
    assert msg.startswith("import cycle detected: ")
    chain = msg[len("import cycle detected: "):].split(" -> ")
    assert [p.rsplit("/", 1)[-1] for p in chain] == ["a.ft", "b.ft", "a.ft"]
    assert e.value.status == _native.FT_ERR_IMPORT_CYCLE


def test_missing_and_unsupported_imports(tmp_path):
    _write(tmp_path, {
        "missing.ft": 'import "./nowhere.ft";\nlet scene = Sphere {};\n',
        "library.ft": 'import "materials/gold.ft" as gold;\nlet scene = Sphere {};\n',
        "sub/up.ft": 'import "../shared.ft";\nlet scene = Sphere { material: mat };\n',
        "shared.ft": "let mat = Lambert { color: vec3(0.2, 0.4, 0.8) };\n",
    })
    with pytest.raises(ft.MissingImport, match="missing import './nowhere.ft' from "):
        ft.load_and_eval_scene(tmp_path / "missing.ft")
    with pytest.raises(ft.RenderError) as e:
        ft.load_and_eval_scene(tmp_path / "library.ft")
    assert e.value.status == _native.FT_ERR_UNSUPPORTED and "built-in library" in str(e.value)
    with pytest.raises(ft.SceneIoError, match="failed to read scene file"):
        ft.load_and_eval_scene(tmp_path / "absent.ft")
    _same_scene(tmp_path / "sub" / "up.ft",
                "let mat = Lambert { color: vec3(0.2, 0.4, 0.8) };\nlet scene = Sphere { material: mat };\n")
    # A source string has no directory to resolve an import from.
    with pytest.raises(ft.RenderError) as e:
        ft.parse_and_eval('import "./shared.ft";\nlet scene = Sphere {};\n')
    assert e.value.status == _native.FT_ERR_UNSUPPORTED


def test_parse_errors_name_the_file(tmp_path):
    _write(tmp_path, {"broken.ft": "let x = ;\n", "main.ft": 'import "./broken.ft";\nlet scene = Sphere {};\n'})
    with pytest.raises(ft.ParseError, match="broken.ft"):
        ft.load_and_eval_scene(tmp_path / "main.ft")


def test_c_entry_point_rejects_null_arguments():
    lib = _native.lib()
    out = ctypes.POINTER(_native.SceneDescC)()
    assert lib.ft_scene_desc_from_file(None, ctypes.byref(out)) == _native.FT_ERR_INVALID_ARGUMENT
    assert lib.ft_scene_desc_from_file(b"x.ft", None) == _native.FT_ERR_INVALID_ARGUMENT


LIB_GOLD = "material Gold {\n  model: Metal;\n  color = vec3(0.95, 0.75, 0.3);\n  roughness = 0.2;\n};\nexport { Gold };\n"
LIB_FLOOR = ("let floor_mat = Lambert { color: vec3(0.8) };\n"
             "let Floor = Box { size: vec3(8.0, 0.5, 8.0), pos: vec3(0.0, -0.25, 0.0), material: floor_mat };\n"
             "export { Floor };\n")


def _library():
    return [ft.LibraryItem("Gold", "materials/gold.ft", LIB_GOLD),
            ft.LibraryItem("StageFloor", "objects/stage_floor.ft", LIB_FLOOR)]


def test_library_imports_by_path_and_by_name(tmp_path):
    """Imports that are not relative paths select a library item by path or
    by name (resolve_import, lib.rs:385-416); the caller supplies the items,
    as the reference supplies its built-in table."""
    _write(tmp_path, {
        "by_path.ft": 'import "materials/gold.ft" as gold;\nimport "objects/stage_floor.ft";\n'
                      "let scene = Floor + Sphere { pos: vec3(0.0, 1.0, 0.0), material: gold.Gold {} };\n",
        "by_name.ft": 'import "Gold";\nimport "StageFloor";\n'
                      "let scene = Floor + Sphere { pos: vec3(0.0, 1.0, 0.0), material: Gold {} };\n",
    })
    single = (LIB_GOLD.replace("export { Gold };", "") + LIB_FLOOR.replace("export { Floor };", "")
              + "let scene = Floor + Sphere { pos: vec3(0.0, 1.0, 0.0), material: Gold {} };\n")
    ref = _dump(ft.parse_and_eval(single))
    assert _dump(ft.load_and_eval_scene(tmp_path / "by_path.ft", library=_library())) == ref
    assert _dump(ft.load_and_eval_scene(tmp_path / "by_name.ft", library=_library())) == ref


def test_library_directory_naming(tmp_path, monkeypatch):
    """library_from_dir names each file's item by its stem in CamelCase;
    FT_LIBRARY_DIR supplies the directory when no library is passed."""
    _write(tmp_path / "lib", {"materials/gold.ft": LIB_GOLD, "objects/stage_floor.ft": LIB_FLOOR})
    items = ft.library_from_dir(tmp_path / "lib")
    assert [(i.name, i.path) for i in items] == [("Gold", "materials/gold.ft"),
                                                ("StageFloor", "objects/stage_floor.ft")]
    _write(tmp_path, {"main.ft": 'import "Gold";\nlet scene = Sphere { material: Gold {} };\n'})
    monkeypatch.setenv("FT_LIBRARY_DIR", str(tmp_path / "lib"))
    _same_scene(tmp_path / "main.ft", LIB_GOLD.replace("export { Gold };", "")
                + "let scene = Sphere { material: Gold {} };\n")


def test_library_import_errors(tmp_path):
    twin = _library() + [ft.LibraryItem("Gold", "materials/gold_leaf.ft", LIB_GOLD)]
    loop = [ft.LibraryItem("Loop", "scenes/loop.ft", 'import "Loop";\nlet x = 1.0;\n')]
    _write(tmp_path, {
        "twin.ft": 'import "Gold";\nlet scene = Sphere {};\n',
        "unknown.ft": 'import "Silver";\nlet scene = Sphere {};\n',
        "loop.ft": 'import "Loop";\nlet scene = Sphere {};\n',
    })
    with pytest.raises(ft.AmbiguousImport,
                       match="ambiguous built-in import 'Gold' matches: materials/gold.ft, materials/gold_leaf.ft"):
        ft.load_and_eval_scene(tmp_path / "twin.ft", library=twin)
    with pytest.raises(ft.MissingImport, match="missing import 'Silver' from "):
        ft.load_and_eval_scene(tmp_path / "unknown.ft", library=_library())
    with pytest.raises(ft.ImportCycle, match="builtin:scenes/loop.ft -> builtin:scenes/loop.ft"):
        ft.load_and_eval_scene(tmp_path / "loop.ft", library=loop)
    lib = _native.lib()
    out = ctypes.POINTER(_native.SceneDescC)()
    bad = (_native.LibraryItemC * 1)(_native.LibraryItemC(b"X", None, b""))
    assert lib.ft_scene_desc_from_file_with_library(str(tmp_path / "loop.ft").encode(), bad, 1,
                                                    ctypes.byref(out)) == _native.FT_ERR_INVALID_ARGUMENT
