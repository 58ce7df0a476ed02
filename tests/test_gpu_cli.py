"""The C++ `sloth` command (rust-sloth_gb300/host): stdout byte for byte against the
oracle's frames and flush emitter, for the image path of the reference's main
(src/main.rs:27-111): one frame (ANSI colour or -b plain) and the -j N JS export."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CLI = Path(__file__).resolve().parents[1] / "rust-sloth_gb300" / "_build" / "sloth"
F32 = np.float32


def run(*args):
    r = subprocess.run([str(CLI), *map(str, args)], capture_output=True, timeout=120)
    return r.returncode, r.stdout, r.stderr


def expected(meshes, w, h, rot, fmt):
    """One frame as the reference prints it: update (utransform from the meshes' boxes),
    clear, draw every mesh in order, flush."""
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"] for m in meshes]))
    o = O.Oracle(w, h, True, U)
    R = O.euler_rotation(*rot)
    for m in meshes:
        o.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], R, m.get("idx"))
    return O.flush(o.frame().cells, True, fmt)


@pytest.fixture(scope="module")
def models(tmp_path_factory):
    d = tmp_path_factory.mktemp("models")
    (d / "col.mtl").write_text("newmtl warm\nKd 0.9 0.55 0.2\nnewmtl cool\nKd 0.2 0.6 0.95\n")
    sph = W.uv_sphere()
    lines = ["mtllib col.mtl"] + [f"v {a:.9g} {b:.9g} {c:.9g}" for a, b, c in zip(sph["x"], sph["y"], sph["z"])]
    faces = sph["idx"] + 1
    half = len(faces) // 2
    lines += ["usemtl warm"] + [f"f {a} {b} {c}" for a, b, c in faces[:half]]
    lines += ["usemtl cool"] + [f"f {a} {b} {c}" for a, b, c in faces[half:]]
    (d / "sphere.obj").write_text("\n".join(lines) + "\n")
    soup = W.soup(400, seed=12, n_large=3)
    tris = np.stack([soup["x"], soup["y"], soup["z"]], 1).reshape(-1, 3, 3)
    (d / "soup.stl").write_text("solid s\n" + "".join(
        "facet normal 0 0 1\nouter loop\n" + "".join(f"vertex {a:.9g} {b:.9g} {c:.9g}\n" for a, b, c in t) +
        "endloop\nendfacet\n" for t in tris) + "endsolid s\n")
    return d


def test_image_frame_colour_and_plain(models):
    obj = models / "sphere.obj"
    meshes = W.read_obj(obj)
    rc, out, err = run(obj, "image", "-w", 160, "-h", 48, "-x", 0.5)
    assert rc == 0, err
    assert out == expected(meshes, 160, 48, W.cli_rotation(yaw=0.5), O.FLUSH_ANSI)
    rc, out, err = run(obj, "-b", "image", "-w", 161, "-h", 40, "-y", -0.3, "-z", 0.2)
    assert rc == 0, err
    assert out == expected(meshes, 161, 40, W.cli_rotation(pitch=-0.3, roll=0.2), O.FLUSH_PLAIN)
    # -w alone: height = width; -b after `image` is not the colour switch the reference reads
    rc, out, err = run(obj, "image", "-w", 64, "-b")
    assert rc == 0, err
    assert out == expected(meshes, 64, 64, W.cli_rotation(), O.FLUSH_ANSI)


def test_several_files_in_one_argument(models):
    obj, stl = models / "sphere.obj", models / "soup.stl"
    meshes = W.read_obj(obj) + [W.read_stl(stl)]
    rc, out, err = run(f"{obj} {stl}", "-b", "image", "-w", 200, "-h", 60, "-x", 1.1)
    assert rc == 0, err
    assert out == expected(meshes, 200, 60, W.cli_rotation(yaw=1.1), O.FLUSH_PLAIN)


@pytest.mark.parametrize("n", [1, 3, 7])
def test_js_export(models, n):
    """-j N: `let frames = [`, then per frame "`" + the HTML flush, closed by "`," or
    "`];", the pitch stepping by (2 pi) * (1/N) in f32 (src/main.rs:55-58,85-106)."""
    obj = models / "sphere.obj"
    meshes = W.read_obj(obj)
    rc, out, err = run(obj, "image", "-w", 80, "-h", 24, "-j", n, "-x", 0.25)
    assert rc == 0, err
    want = [b"let frames = [\n"]
    t0, t1, t2 = W.cli_rotation(yaw=0.25)
    t1 = F32(t1)
    step = F32(F32(2.0) * W.PI_F32) * F32(F32(1.0) / F32(n))
    count = 0
    while True:
        want.append(b"`\n" + expected(meshes, 80, 24, (t0, float(t1), t2), O.FLUSH_HTML))
        t1 = F32(t1 + step)
        if t1 > F32(9.42477) or n - 1 == count:
            want.append(b"`];\n")
            break
        want.append(b"`,\n")
        count += 1
    assert out == b"".join(want)


def test_errors(models, tmp_path):
    rc, out, err = run(tmp_path / "model.ply", "image", "-w", 10)
    assert rc == 1 and b"unknown filename extension" in err and out == b""
    (tmp_path / "m.obj").write_text("mtllib none.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    rc, out, err = run(tmp_path / "m.obj", "image", "-w", 10)
    assert rc == 101 and b"Expected to have materials." in err
    rc, out, err = run(models / "sphere.obj")
    assert rc == 2                                       # the interactive terminal mode
