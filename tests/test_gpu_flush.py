"""Context::flush bytes formatted on the GPU (sloth_ctx_flush / sloth_batch_flush) against
the oracle's emitter, byte for byte."""
import hashlib

import numpy as np
import pytest

import sloth_gpu as S
import workloads as W
from oracle import oracle as O
from gpu_helpers import gpu_render, oracle_render

pytestmark = pytest.mark.gpu

FORMATS = (O.FLUSH_PLAIN, O.FLUSH_ANSI, O.FLUSH_HTML)


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def render_and_flush(ctx, meshes, R, w, h, image):
    ref = oracle_render(meshes, R, w, h, image)
    cells, _, _, _ = gpu_render(ctx, meshes, R, w, h, image, depth_cull=True)
    assert np.array_equal(cells, ref.cells)
    return ref, {f: ctx.flush(f) for f in FORMATS}


@pytest.mark.parametrize("w,h,image", [(160, 48, True), (160, 48, False), (640, 360, True), (1, 1, True),
                                       (1, 7, True), (5, 1, False), (33, 9, True)])
def test_sphere_flush_matches_oracle(ctx, w, h, image):
    R = O.euler_rotation(*W.cli_rotation(yaw=0.5))
    ref, out = render_and_flush(ctx, [W.uv_sphere()], R, w, h, image)
    for f in FORMATS:
        assert out[f] == O.flush(ref.cells, image, f), f"format {f} {w}x{h} image={image}"


def test_large_soup_html_and_ansi(ctx):
    """A 1920x1080 colourful soup: about 60 MB of HTML formatted in chunks."""
    m = W.soup(200000, seed=8, n_large=20)
    R = O.euler_rotation(*W.cli_rotation(yaw=1.1))
    ref, out = render_and_flush(ctx, [m], R, 1920, 1080, True)
    for f in FORMATS:
        want = O.flush(ref.cells, True, f)
        assert len(out[f]) == len(want)
        assert hashlib.sha256(out[f]).digest() == hashlib.sha256(want).digest(), f"format {f}"


def test_batch_flush_matches_oracle(ctx):
    ico = W.displaced_icosphere(3, seed=3)
    soup = W.soup(3000, seed=4, n_large=5)
    mi, ms = S.Mesh(ctx, ico["x"], ico["y"], ico["z"], ico["rgb"], ico["idx"], ico["bbox_max"]), \
        S.Mesh(ctx, soup["x"], soup["y"], soup["z"], soup["rgb"], None, soup["bbox_max"])
    specs = [(80, 24, True, ico, mi), (161, 47, False, soup, ms), (64, 64, True, soup, ms)]
    frames, refs = [], []
    for i, (w, h, image, m, dm) in enumerate(specs):
        R = O.euler_rotation(*W.cli_rotation(yaw=0.3 * i))
        U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
        frames.append({"w": w, "h": h, "image": image, "U": U, "draws": [(dm, R)]})
        refs.append((oracle_render([m], R, w, h, image, U=U), image))
    b = S.Batch(ctx, frames)
    b.render()
    for i, (ref, image) in enumerate(refs):
        for f in FORMATS:
            assert b.flush(i, f) == O.flush(ref.cells, image, f), f"frame {i} format {f}"
    b.close()


def test_flush_errors(ctx):
    ctx.set_viewport(8, 4, True)
    ctx.clear()
    with pytest.raises(S.SlothError):
        ctx.flush(7)
    n = S.C.c_uint64()
    buf = S.C.create_string_buffer(4)
    assert ctx.lib.sloth_ctx_flush(ctx.h, S.FLUSH_HTML, buf, 4, S.C.byref(n)) == S.ERR_LIMIT
    assert n.value > 4
