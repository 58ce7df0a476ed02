"""The C++ host loaders (rust-sloth_gb300/host/loaders.cpp, run through sloth_meshdump:
no GPU) against the Python restatement of the same tobj/stl_io rules and against the
golden summaries of the reference's own model files (tests/golden/models.json)."""
import json
import os
import struct
from pathlib import Path

import numpy as np
import pytest

import workloads as W
from loader_helpers import MESHDUMP, ROOT, cpp_meshes, summary

# The reference's models/ folder: SLOTH_MODELS_DIR, else a `reference` checkout beside
# this repository.  Where neither exists only the golden-summary test is skipped (it says
# so); every other loader test runs on the synthetic files it writes.
REF_MODELS = Path(os.environ.get("SLOTH_MODELS_DIR", str(ROOT.parent / "reference" / "models")))
GOLDEN = json.loads((ROOT / "tests" / "golden" / "models.json").read_text())


def test_meshdump_is_built():
    # conftest builds it for every run: the loader tests below must not skip silently
    assert MESHDUMP.exists(), MESHDUMP


def py_meshes(path: Path):
    try:
        return W.read_obj(path) if path.suffix.lower() == ".obj" else [W.read_stl(path)]
    except W.LoadError as e:
        return str(e)


def same(cpp, py):
    assert isinstance(cpp, list) and isinstance(py, list), (cpp, py)
    assert len(cpp) == len(py)
    for a, b in zip(cpp, py):
        for k in ("x", "y", "z"):
            assert np.array_equal(np.asarray(a[k], np.float32).view(np.uint32),
                                  np.asarray(b[k], np.float32).view(np.uint32)), k
        assert np.array_equal(a["rgb"], b["rgb"])
        assert np.array_equal(a["bbox_max"].view(np.uint32), np.asarray(b["bbox_max"], np.float32).view(np.uint32))


@pytest.mark.skipif(not REF_MODELS.exists(), reason="the reference's models/ folder is absent: set SLOTH_MODELS_DIR")
@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_reference_models_match_python_and_golden(name):
    path = REF_MODELS / name
    cpp, py = cpp_meshes(str(path)), py_meshes(path)
    same(cpp, py)
    assert [summary(m) for m in cpp] == GOLDEN[name]


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_obj_quads_groups_materials_and_vertex_colours(tmp_path):
    write(tmp_path, "m.mtl", "newmtl red one\nKd 1.0 0.0 0.0\nnewmtl half\nKd 0.5 0.5 0.25\n")
    obj = write(tmp_path, "a.obj", "\n".join([
        "mtllib m.mtl",
        "v 0 0 0", "v 1 0 0", "v 1 1 0", "v 0 1 0", "v 0.5 2 1",
        "usemtl red one",
        "f 1 2 3 4",               # quad -> 2 triangles
        "f -5/1 -4//2 -1/3/3",     # negative indices, texture/normal parts
        "usemtl red one",          # same material: no new mesh
        "f 1 3 5",
        "usemtl half",             # material change: new mesh
        "f 2 3 5 4 1",             # pentagon -> 3 triangles
        "g second",
        "f 1 2 5",
        "o third",
        "usemtl missing",          # unknown material: no new mesh, no material
        "usemtl half",
        "f 3 4 5",
    ]) + "\n")
    cpp, py = cpp_meshes(str(obj)), py_meshes(obj)
    same(cpp, py)
    assert [m["rgb"].shape[0] for m in cpp] == [4, 3, 1, 1]
    assert cpp[0]["rgb"][0].tolist() == [255, 0, 0]
    assert cpp[1]["rgb"][0].tolist() == [127, 127, 63]
    # vertex colours replace the material colour (first corner's colour)
    obj2 = write(tmp_path, "b.obj", "mtllib m.mtl\nv 0 0 0 0.2 0.4 1.0\nv 1 0 0 1 1 1\nv 0 1 0 0 0 0\n"
                                    "usemtl half\nf 1 2 3\nf 2 3 1\n")
    cpp, py = cpp_meshes(str(obj2)), py_meshes(obj2)
    same(cpp, py)
    assert cpp[0]["rgb"].tolist() == [[51, 102, 255], [255, 255, 255]]


def test_obj_without_materials_is_white_one_and_bbox_from_origin(tmp_path):
    obj = write(tmp_path, "c.obj", "v -3 -2 -1\nv -1 -2 -3\nv -2 -1 -3\nf 1 2 3\n")
    cpp = cpp_meshes(str(obj))
    same(cpp, py_meshes(obj))
    assert cpp[0]["rgb"].tolist() == [[1, 1, 1]]
    assert cpp[0]["bbox_max"].tolist() == [0.0, 0.0, 0.0]      # grown from the origin
    assert cpp[0]["bbox_min"].tolist() == [-3.0, -2.0, -3.0]


@pytest.mark.parametrize("text,needle", [
    ("mtllib nowhere.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "Expected to have materials."),
    ("v 0 0 0\nv 1 0 0\nf 1 2 3\n", "FaceVertexOutOfBounds"),
    ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "FaceParseError"),
])
def test_obj_errors(tmp_path, text, needle):
    obj = write(tmp_path, "e.obj", text)
    err = cpp_meshes(str(obj))
    assert isinstance(err, str) and needle in err, err
    assert isinstance(py_meshes(obj), str)


def test_obj_face_without_material_when_materials_exist(tmp_path):
    write(tmp_path, "m.mtl", "newmtl a\nKd 1 1 1\n")
    obj = write(tmp_path, "f.obj", "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    assert isinstance(cpp_meshes(str(obj)), str)
    assert isinstance(py_meshes(obj), str)


def test_stl_ascii_and_binary(tmp_path):
    tris = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0.1, 0.2, 0.3], [-1.5, 2.25, 3], [4, -5, 6.5]]], np.float32)
    ascii_text = "solid x\n" + "".join(
        "facet normal 0 0 1\nouter loop\n" + "".join(f"vertex {a:.9g} {b:.9g} {c:.9g}\n" for a, b, c in t) +
        "endloop\nendfacet\n" for t in tris) + "endsolid x\n"
    pa = write(tmp_path, "a.stl", ascii_text)
    pb = tmp_path / "b.stl"
    body = b"".join(struct.pack("<3f", 0, 0, 1) + t.astype("<f4").tobytes() + b"\0\0" for t in tris)
    pb.write_bytes(b"binary header".ljust(80, b"\0") + struct.pack("<I", len(tris)) + body)
    for p in (pa, pb):
        cpp = cpp_meshes(str(p))
        same(cpp, py_meshes(p))
        assert cpp[0]["rgb"].tolist() == [[255, 255, 0]] * 2
        assert np.array_equal(np.stack([cpp[0]["x"], cpp[0]["y"], cpp[0]["z"]], 1), tris.reshape(-1, 3))
        assert cpp[0]["bbox_max"].tolist() == tris.reshape(-1, 3).max(0).tolist()


def test_match_meshes_splits_on_spaces_and_checks_extensions(tmp_path):
    a = write(tmp_path, "one.obj", "v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    b = write(tmp_path, "two.OBJ", "v 0 0 1\nv 1 0 1\nv 0 1 1\nf 1 2 3\nf 3 2 1\n")
    ms = cpp_meshes(f"{a} {b}")
    assert [m["rgb"].shape[0] for m in ms] == [1, 2]
    err = cpp_meshes(str(tmp_path / "x.ply"))
    assert err.startswith("filename: [") and "unknown filename extension" in err
    err = cpp_meshes(str(tmp_path / "noext"))
    assert "couldn't determine filename extension" in err
