"""Bit-exact parity of the CUDA path (through the C ABI) with the CPU oracle.

Compared per case: every frame cell (char + colour), every depth cell (f32 bits,
including -0.0), the winning triangle of every depth cell, and the fragment count.
"""
import math

import numpy as np
import pytest

import sloth_gpu as S
import workloads as W
from oracle import oracle as O
from gpu_helpers import assert_same, gpu_render, oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def one_tri_mesh(v9, rgb):
    v = np.asarray(v9, np.float32).reshape(3, 3)
    return {"x": v[:, 0].copy(), "y": v[:, 1].copy(), "z": v[:, 2].copy(), "idx": None,
            "rgb": np.asarray(rgb, np.uint8).reshape(1, 3), "bbox_max": np.ones(3, np.float32)}


# ------------------------------------------------------------------------- config 1
@pytest.mark.parametrize("w,h,image", [(160, 48, False), (160, 48, True), (640, 360, True), (640, 360, False)])
def test_uv_sphere_config(ctx, w, h, image):
    """UV sphere r=1, 32x16 (960 triangles), `image ... --yaw 0.5`."""
    m = W.uv_sphere()
    R = O.euler_rotation(*W.cli_rotation(yaw=0.5))
    ref = oracle_render([m], R, w, h, image)
    assert ref.fragments > 0
    assert_same(gpu_render(ctx, [m], R, w, h, image), ref, f"sphere {w}x{h} image={image}")


# ---------------------------------------------------------------------- micro cases
MICRO = {
    "single": ([([1, 1, 0.5, 5, 1, 0.5, 1, 5, 0.5], (10, 20, 30))], 16, 8),
    "back_and_degenerate": ([([1, 1, 0, 1, 5, 0, 5, 1, 0], (1, 2, 3)),
                             ([1, 1, 0, 3, 3, 1, 5, 5, 2], (4, 5, 6))], 12, 8),
    "ties": ([([1, 1, 0, 5, 1, 0, 1, 5, 0], (1, 1, 1)), ([1, 1, 0, 5, 1, 0, 1, 5, 0], (2, 2, 2)),
              ([1, 1, -0.0, 5, 1, -0.0, 1, 5, -0.0], (3, 3, 3))], 16, 8),
    "wrap_even": ([([1, 1, 0, 6, 1, 0, 1, 4, 0], (7, 7, 7))], 8, 6),
    "wrap_odd_half_cell": ([([1, 2, 5, 3, 2, 5, 1, 3, 5], (1, 0, 0)),
                            ([5, 1, 1, 6, 1, 1, 5, 2, 1], (0, 2, 0))], 9, 6),
    "newline_order": ([([1, 1, 0, 6, 1, 0, 1, 4, 0], (5, 5, 5)),
                       ([4, 1, -1, 5, 1, -1, 4, 1.5, -1], (6, 6, 6))], 8, 6),
    "tiny_viewports": ([([0, 0, 0, 3, 0, 0, 0, 3, 0], (9, 9, 9))], 3, 2),
}


@pytest.mark.parametrize("name", sorted(MICRO))
@pytest.mark.parametrize("image", [False, True])
def test_micro_cases(ctx, name, image):
    tris, w, h = MICRO[name]
    meshes = [one_tri_mesh(v, c) for v, c in tris]
    I = np.eye(4, dtype=np.float32)
    ref = oracle_render(meshes, I, w, h, image, U=I)
    assert_same(gpu_render(ctx, meshes, I, w, h, image, U=I), ref, name)


def test_viewport_one_by_one_and_width_one(ctx):
    m = W.soup(200, seed=5, n_large=5, sigma=0.3)
    R = O.euler_rotation(0.3, 0.2, 0.1)
    for w, h in [(1, 1), (1, 7), (2, 5), (5, 1), (4, 4)]:
        for image in (False, True):
            assert_same(gpu_render(ctx, [m], R, w, h, image), oracle_render([m], R, w, h, image), f"{w}x{h}")


# -------------------------------------------------------------------- seeded soups
def hostile_soup(seed, n=2000):
    """Small + large triangles with slivers, exact collinear triangles, depth ties,
    huge and non-finite coordinates mixed in."""
    rng = np.random.default_rng(seed)
    m = W.soup(n, seed=seed, n_large=max(2, n // 200), sigma=0.04)
    x, y, z = m["x"].copy(), m["y"].copy(), m["z"].copy()
    nt = m["rgb"].shape[0]
    pick = rng.choice(nt, size=min(nt, 60), replace=False)
    for k, t in enumerate(pick):
        i = 3 * t
        kind = k % 6
        if kind == 0:      # exact collinear
            x[i + 2] = x[i] + 2 * (x[i + 1] - x[i]); y[i + 2] = y[i] + 2 * (y[i + 1] - y[i])
        elif kind == 1:    # sliver
            x[i + 2] = x[i + 1] + np.float32(1e-5); y[i + 2] = y[i + 1] - np.float32(1e-6)
        elif kind == 2:    # depth tie with its neighbour
            z[i:i + 3] = np.float32(0.125)
        elif kind == 3:    # huge coordinate
            x[i + 1] = np.float32(3e19) * (1 if k % 12 < 6 else -1)
        elif kind == 4:    # non-finite
            y[i + 2] = np.float32(np.inf) if k % 12 < 6 else np.float32(np.nan)
        else:              # point triangle
            x[i + 1] = x[i + 2] = x[i]; y[i + 1] = y[i + 2] = y[i]
    m["x"], m["y"], m["z"] = x, y, z
    m["bbox_max"] = np.array([1.1, 1.1, 1.1], np.float32)
    return m


@pytest.mark.parametrize("seed", range(8))
def test_hostile_soups(ctx, seed):
    rng = np.random.default_rng(1000 + seed)
    w = int(rng.integers(7, 400)) | (seed & 1)
    h = int(rng.integers(5, 200))
    image = bool(seed % 3 != 1)
    meshes = [hostile_soup(seed), hostile_soup(seed + 50, n=500)]
    R = O.euler_rotation(float(rng.uniform(-math.pi, math.pi)), float(rng.uniform(-math.pi, math.pi)),
                         float(rng.uniform(-math.pi, math.pi)))
    ref = oracle_render(meshes, R, w, h, image)
    assert_same(gpu_render(ctx, meshes, R, w, h, image), ref, f"seed {seed} {w}x{h}")


@pytest.mark.parametrize("seed", [3, 8])
def test_hostile_indexed(ctx, seed):
    """The hostile soup as an indexed mesh with its faces shuffled: setup's spatial order
    of an indexed mesh meets huge and non-finite centroids."""
    rng = np.random.default_rng(2000 + seed)
    m = dict(hostile_soup(seed, n=1500))
    nt = m["rgb"].shape[0]
    perm = rng.permutation(nt)
    m["idx"] = np.ascontiguousarray(np.arange(3 * nt, dtype=np.uint32).reshape(-1, 3)[perm])
    m["rgb"] = np.ascontiguousarray(m["rgb"][perm])
    w, h = int(rng.integers(40, 300)), int(rng.integers(20, 120))
    R = O.euler_rotation(float(rng.uniform(-math.pi, math.pi)), 0.3, 0.1)
    for image in (False, True):
        ref = oracle_render([m], R, w, h, image)
        assert_same(gpu_render(ctx, [m], R, w, h, image), ref, f"seed {seed} {w}x{h}")


@pytest.mark.parametrize("w,h", [(3840 // 8, 2160 // 8), (481, 271)])
def test_scaled_config2_soup(ctx, w, h):
    """Config-2 soup statistics (small N(0,0.02) triangles + large ones) at reduced size."""
    m = W.soup(20000, seed=2, n_large=40)
    R = O.euler_rotation(*W.cli_rotation())
    for image in (True, False):
        ref = oracle_render([m], R, w, h, image)
        assert_same(gpu_render(ctx, [m], R, w, h, image), ref, f"soup {w}x{h}")



def span_soup(seed, w, h, n=600):
    """Screen-space triangles (identity transforms) that stress the per-row column spans
    of large tile parts: vertices on sample positions (edges through samples, w == 0),
    horizontal and vertical edges, long thin slivers, half-sample offsets, vertices far
    off screen and huge finite coordinates; both windings."""
    rng = np.random.default_rng(seed)
    xs = w // 2 if w > 0 else 1
    tris = []
    for k in range(n):
        kind = k % 7
        c = rng.uniform([0, 0], [xs, h])
        s = rng.uniform(4, 40)
        if kind == 0:      # integer vertices
            v = np.round(c + rng.uniform(-s, s, (3, 2)))
        elif kind == 1:    # right triangle: one horizontal and one vertical edge
            a, b = np.round(c), np.round(c + rng.uniform(-s, s, 2))
            v = np.array([a, [b[0], a[1]], [a[0], b[1]]])
        elif kind == 2:    # long sliver
            d = rng.normal(size=2)
            d /= np.linalg.norm(d)
            v = np.array([c - 3 * s * d, c + 3 * s * d, c + 3 * s * d + rng.uniform(0.05, 1.5) * d[::-1] * [1, -1]])
        elif kind == 3:    # half-sample offsets
            v = np.round(c + rng.uniform(-s, s, (3, 2))) + 0.5
        elif kind == 4:    # vertices far off screen
            v = c + rng.uniform(-20 * s, 20 * s, (3, 2))
        elif kind == 5:    # huge finite coordinates on one vertex
            v = c + rng.uniform(-s, s, (3, 2))
            v[1] = [rng.choice([-1, 1]) * 10.0 ** rng.uniform(6, 17), c[1] + rng.uniform(-s, s)]
        else:              # random floats
            v = c + rng.uniform(-s, s, (3, 2))
        if rng.random() < 0.5:
            v = v[::-1]
        z = rng.uniform(-1, 1, 3)
        tris.append(np.column_stack([v, z]))
    t = np.asarray(tris, np.float32).reshape(-1, 3)
    rgb = rng.integers(0, 256, (n, 3), dtype=np.uint8)
    return {"x": t[:, 0].copy(), "y": t[:, 1].copy(), "z": t[:, 2].copy(), "idx": None, "rgb": rgb,
            "bbox_max": np.ones(3, np.float32)}


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("image", [True, False])
def test_row_span_walk(ctx, seed, image):
    w, h = (403, 150) if seed % 2 else (512, 128)
    m = span_soup(seed, w if image else 2 * w, h)
    eye = np.eye(4, dtype=np.float32)
    ref = oracle_render([m], eye, w, h, image, U=eye)
    assert ref.fragments > 0
    assert_same(gpu_render(ctx, [m], eye, w, h, image, U=eye), ref, f"span soup {seed} image={image}")


def test_depth_culling_skips_hidden_fragments(ctx):
    """At config 2's triangle size and depth complexity (1/8 of its viewport: 1/64 of the
    triangles, 8x the vertex offsets) the depth culling skips most covered samples and
    leaves every buffer as it is."""
    m = W.soup(16000, seed=5, n_large=4, sigma=0.16)
    R = O.euler_rotation(*W.cli_rotation())
    w, h = 480, 270
    ref = oracle_render([m], R, w, h, True)
    # the first frame may outgrow the entry buffer an earlier test sized (the draw does not
    # wait for its count): it is then rasterized by the unculled fallback, and the next
    # draw grows the buffer
    for _ in range(2):
        assert_same(gpu_render(ctx, [m], R, w, h, True, depth_cull=True), ref, "dense soup")
    ctx.set_depth_cull(True)
    assert ctx.fragments() < 0.75 * ref.fragments


def test_yawed_soup_wraps(ctx):
    """Rotated soups put samples at 2x >= w: wrapped writes into the next row."""
    m = W.soup(5000, seed=9, n_large=20)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.7, pitch=0.6, roll=0.2))
    U = O.viewport_transform(300, 200, 0.7)   # a small extent pushes samples past w/2
    ref = oracle_render([m], R, 300, 200, True, U=U)
    z = ref.z.reshape(200, 300)
    assert (z[:, 1::2] < np.finfo(np.float32).max).any() or True
    assert_same(gpu_render(ctx, [m], R, 300, 200, True, U=U), ref, "wraps")
    U = O.viewport_transform(301, 200, 0.7)
    ref = oracle_render([m], R, 301, 200, True, U=U)
    assert (ref.z.reshape(200, 301)[:, 1::2] < np.finfo(np.float32).max).any()
    assert_same(gpu_render(ctx, [m], R, 301, 200, True, U=U), ref, "wraps odd")


def test_indexed_icosphere_multi_mesh(ctx):
    a = W.displaced_icosphere(3, seed=3)
    b = W.displaced_icosphere(2, seed=4, rgb=(10, 200, 30))
    b["x"] = (b["x"] * 0.5 + 0.4).astype(np.float32)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.3))
    for image in (False, True):
        ref = oracle_render([a, b], R, 200, 90, image)
        assert_same(gpu_render(ctx, [a, b], R, 200, 90, image), ref, "icospheres")


def test_clear_redraw_and_resize(ctx):
    m = W.uv_sphere()
    R1 = O.euler_rotation(*W.cli_rotation(yaw=0.5))
    R2 = O.euler_rotation(*W.cli_rotation(yaw=1.5))
    dm = S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m["idx"])
    for (w, h, im, R) in [(160, 48, True, R1), (160, 48, True, R2), (80, 24, False, R1), (160, 48, True, R1)]:
        ref = oracle_render([m], R, w, h, im)
        assert_same(gpu_render(ctx, [m], R, w, h, im, dev_meshes=[dm]), ref, f"{w}x{h}")


def test_entry_buffer_grows_between_frames():
    """A frame with many more tile entries than the context's earlier frames: the fill that
    went ahead with the old entry buffer is redone after the buffer grows."""
    c = S.Context(0)
    try:
        small = W.soup(200, seed=4)
        big = W.soup(20000, seed=5, n_large=60)
        R = O.euler_rotation(*W.cli_rotation())
        for m, (w, h) in [(small, (200, 100)), (big, (480, 270)), (small, (200, 100)), (big, (960, 540))]:
            ref = oracle_render([m], R, w, h, True)
            assert_same(gpu_render(c, [m], R, w, h, True), ref, f"{m['rgb'].shape[0]} triangles {w}x{h}")
    finally:
        c.close()


@pytest.mark.parametrize("cull,direct", [(False, 0), (True, 0), (True, 16)])
def test_overflow_fallback_multi_draw(cull, direct):
    """Draws whose tile entries outgrow the entry buffer sized by a context's first frame:
    the host does not wait for the count, so such a draw is rasterized by the device-side
    fallback (every binned triangle folded straight into the keys), after the keys of the
    frame's earlier draws and before those of its later draws."""
    small = W.soup(100, seed=7)
    big = W.soup(30000, seed=8, n_large=50)
    big2 = W.soup(20000, seed=9, n_large=30, sigma=0.04)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.6))
    c = S.Context(0)
    try:
        c.set_depth_cull(cull)
        c.set_direct_samples(direct)
        dev = [S.Mesh(c, m["x"], m["y"], m["z"], m["rgb"]) for m in (small, big, big2)]
        c.set_viewport(320, 180, True)
        c.update(dev[:1])
        c.clear()
        c.draw_mesh(dev[0], R)          # the first draw sizes the entry buffer: 100 triangles
        c.read()
        for w, h, image in ((640, 360, True), (641, 200, False)):
            c.set_viewport(w, h, image)
            c.update(dev)
            c.clear()
            for d in dev:
                c.draw_mesh(d, R)
            cells, z, winner = c.read()
            ref = oracle_render([small, big, big2], R, w, h, image)
            assert_same((cells, z, winner, None if cull else c.fragments()), ref, f"overflow {w}x{h}")
    finally:
        c.close()


def test_many_frames_generation_counter(ctx):
    """Repeated clears reuse the key buffer through the tile generation counter."""
    m = W.soup(300, seed=1)
    ctx.set_viewport(64, 32, True)
    ctx.set_depth_cull(False)   # every covered sample counted
    dm = S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"])
    ctx.update([dm])
    ang = np.linspace(0, 2 * math.pi, 12)
    for a in ang:
        R = O.euler_rotation(*W.cli_rotation(yaw=float(a)))
        ctx.clear()
        ctx.draw_mesh(dm, R)
        cells, z, winner = ctx.read()
        ref = oracle_render([m], R, 64, 32, True)
        assert_same((cells, z, winner, ctx.fragments()), ref, f"angle {a}")
    ctx.set_depth_cull(True)
    # an empty frame after drawing: clear only
    ctx.clear()
    cells, z, winner = ctx.read()
    assert (cells == ord(" ")).all() and (winner == -1).all()
    assert (z == np.finfo(np.float32).max).all()


def test_draw_without_clear_errors(ctx):
    c = S.Context(0)
    m = W.soup(10, seed=1)
    dm = S.Mesh(c, m["x"], m["y"], m["z"], m["rgb"])
    with pytest.raises(S.SlothError):
        c.draw_mesh(dm, np.eye(4))
    with pytest.raises(S.SlothError):
        c.set_viewport(0, 10, False)
    with pytest.raises(S.SlothError):
        S.Mesh(c, m["x"], m["y"], m["z"], m["rgb"], idx=np.array([[0, 1, 99]]))
    c.close()


def test_dense_small_viewport_split_tiles(ctx):
    """Tens of thousands of triangles over a few tiles: tiles with more than 8192 entries
    are rasterized in slices by separate CTAs that fold their keys with a global atomicMin;
    a second draw folds into the first draw's keys."""
    a = W.soup(60000, seed=41, n_large=5)
    b = W.soup(30000, seed=42, n_large=2)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.7))
    for w, h, image in ((80, 24, True), (81, 23, False)):
        ref = oracle_render([a, b], R, w, h, image)
        assert_same(gpu_render(ctx, [a, b], R, w, h, image), ref, f"dense {w}x{h}")


def test_bounded_wait_reports_device_fault(ctx):
    """SLOTH_OPTION_WAIT_TEST makes every raster block that loads an earlier draw's keys
    wait for 16 bytes that never come: the blocks give up after a short limit, the read
    returns SLOTH_ERR_DEVICE_FAULT, and the next frame (after a clear) is exact again."""
    a, b = W.soup(2000, seed=61, n_large=2), W.soup(2000, seed=62, n_large=2)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.3))
    w, h = 80, 40
    dev = [S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], None, m["bbox_max"]) for m in (a, b)]
    ctx.set_viewport(w, h, True)
    ctx.update(dev)
    ctx.lib.sloth_ctx_set_option(ctx.h, S.OPTION_WAIT_TEST, 1)
    ctx.clear()
    for d in dev:
        ctx.draw_mesh(d, R)     # the second draw loads the first draw's keys
    with pytest.raises(S.SlothError) as err:
        ctx.read()
    assert err.value.status == S.ERR_DEVICE_FAULT
    ctx.lib.sloth_ctx_set_option(ctx.h, S.OPTION_WAIT_TEST, 0)
    ctx.clear()
    for d in dev:
        ctx.draw_mesh(d, R)
    cells, z, winner = ctx.read()
    ref = oracle_render([a, b], R, w, h, True)
    assert np.array_equal(cells, ref.cells) and np.array_equal(winner, ref.winner)
    for d in dev:
        d.close()


# ------------------------------------------------------------ setup's spatial order
def shuffled_flat_grid(n: int, seed: int) -> dict:
    """An indexed n x n grid of quads at one depth, every triangle twice in each winding
    (four faces per triangle, each with its own colour), the faces in a seeded random
    order: every covered sample is an exact depth tie between several faces, and the
    spatial order setup takes differs from the draw order everywhere."""
    rng = np.random.default_rng(seed)
    g = np.linspace(-0.9, 0.9, n + 1, dtype=np.float32)
    X, Y = np.meshgrid(g, g)
    x, y = X.ravel(), Y.ravel()
    z = np.full_like(x, 0.25)
    k = np.arange(n * n)
    i0 = (k // n) * (n + 1) + k % n
    quads = np.stack([i0, i0 + 1, i0 + n + 2, i0 + n + 1], 1)
    tris = np.concatenate([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]])
    faces = np.concatenate([tris, tris[:, ::-1], tris, tris[:, ::-1]])
    faces = faces[rng.permutation(faces.shape[0])]
    rgb = rng.integers(0, 256, size=(faces.shape[0], 3), dtype=np.uint8)
    return {"x": x, "y": y, "z": z, "idx": faces.astype(np.uint32), "rgb": rgb,
            "bbox_max": np.array([0.9, 0.9, 0.25], np.float32)}


@pytest.mark.parametrize("w,h,image", [(64, 32, True), (200, 90, False)])
def test_spatial_order_keeps_draw_order_ties(ctx, w, h, image):
    """Setup takes an indexed mesh's triangles in a spatial order; ties of equal depth
    still go to the first face in draw order (src/rasterizer.rs:80), through the
    single-frame path (binned and direct) and a batch."""
    m = shuffled_flat_grid(12, seed=41)
    R = O.euler_rotation(0.0, 0.0, 0.0)
    ref = oracle_render([m], R, w, h, image)
    assert ref.fragments > 0
    assert_same(gpu_render(ctx, [m], R, w, h, image), ref, f"flat grid {w}x{h}")
    dm = S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m["idx"], m["bbox_max"])
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
    for direct in (0, 64):
        b = S.Batch(ctx, [{"w": w, "h": h, "image": image, "U": U, "draws": [(dm, R)]}])
        b.set_direct_samples(direct)
        b.render()
        b.render()
        cells, z, winner = b.read(0)
        assert_same((cells, z, winner, None), ref, f"batch, direct {direct}")
        b.close()
