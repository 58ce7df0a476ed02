"""The batched path (sloth_batch_*): many frames of uneven meshes and viewports in one
pass of each stage, one persistent raster pass and a CUDA graph.  Every frame must be
bit-identical to the oracle drawing that frame alone; so must the single-frame path
with every tile shape."""
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


def dev_mesh(ctx, m):
    return S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m.get("idx"), m.get("bbox_max"))


def mixed_frames(ctx):
    """Host meshes + a frame list mixing sizes, image modes, wraps and multi-draw frames."""
    sphere = W.uv_sphere()
    ico = W.displaced_icosphere(3, seed=3)
    soup_a = W.soup(4000, seed=31, n_large=12)
    soup_b = W.soup(1500, seed=32, n_large=4, sigma=0.06)
    meshes = {"sphere": sphere, "ico": ico, "a": soup_a, "b": soup_b}
    dev = {k: dev_mesh(ctx, m) for k, m in meshes.items()}
    rng = np.random.default_rng(5)
    frames = []
    specs = [(160, 48, True, ["sphere"]), (640, 360, True, ["ico"]), (80, 24, False, ["a"]),
             (161, 47, True, ["a", "b"]), (300, 200, True, ["b", "sphere"]), (64, 64, False, ["ico", "a"]),
             (1, 1, True, ["a"]), (33, 9, True, ["b"])]
    for i in range(20):
        w, h, image, names = specs[i % len(specs)]
        ang = W.cli_rotation(yaw=float(rng.uniform(0, 2 * math.pi)), pitch=float(rng.uniform(-0.5, 0.5)))
        R = O.euler_rotation(*ang)
        ext = 0.7 if i % 3 == 0 else O.scene_extent([meshes[n]["bbox_max"] for n in names])
        U = O.viewport_transform(w, h, ext)
        frames.append({"w": w, "h": h, "image": image, "U": U, "names": names, "R": R,
                       "draws": [(dev[n], R) for n in names]})
    return meshes, dev, frames


def check_frames(batch, meshes, frames, label):
    for i, f in enumerate(frames):
        ref = oracle_render([meshes[n] for n in f["names"]], f["R"], f["w"], f["h"], f["image"], U=f["U"])
        cells, z, winner = batch.read(i)
        assert_same((cells, z, winner, None), ref, f"{label} frame {i} {f['w']}x{f['h']}")


@pytest.mark.parametrize("direct,persistent", [(0, True), (16, True), (0, False)])
def test_batch_matches_oracle_and_replays(ctx, direct, persistent):
    meshes, dev, frames = mixed_frames(ctx)
    b = S.Batch(ctx, frames)
    b.set_direct_samples(direct)
    b.set_persistent(persistent)
    b.render()                                   # planned render (sizes the entries)
    check_frames(b, meshes, frames, "planned")
    for k in range(3):                           # graph capture + replays
        b.render()
    check_frames(b, meshes, frames, "graph")
    # new transforms for every draw, replayed through the same graph
    rng = np.random.default_rng(9)
    mats = []
    for f in frames:
        R = O.euler_rotation(*W.cli_rotation(yaw=float(rng.uniform(0, 6.28))))
        f["R"] = R
        mats += [R] * len(f["draws"])
    b.set_transforms(np.stack(mats))
    b.render()
    check_frames(b, meshes, frames, "new transforms")
    b.close()


def test_batch_every_tile_shape_and_autotune(ctx):
    meshes, dev, frames = mixed_frames(ctx)
    frames = frames[:8]
    b = S.Batch(ctx, frames)
    for shape in range(len(S.tile_shapes())):
        b.set_tile_shape(shape)
        b.render()
        check_frames(b, meshes, frames, f"shape {S.tile_shapes()[shape]}")
    for direct in (4, 64):
        b.set_direct_samples(direct)
        b.render()
        check_frames(b, meshes, frames, f"direct {direct}")
    for tpb in (128, 4096):
        b.set_triangles_per_block(tpb)
        b.render()
        check_frames(b, meshes, frames, f"{tpb} triangles per block")
    best = b.autotune(reps=2)
    assert 0 <= best["shape"] < len(S.tile_shapes()) and best["direct"] in (0, 4, 16, 64)
    assert best["tpb"] in (128, 256, 1024, 4096) and best["ms"] > 0
    b.render()
    check_frames(b, meshes, frames, "autotuned")
    b.close()


def test_batch_entry_overflow_replans(ctx):
    """Transforms that list far more tile entries than the first render sized: the
    raster reports the overflow and the read re-plans and re-renders."""
    m = W.soup(3000, seed=41, n_large=10)
    dm = dev_mesh(ctx, m)
    small = np.diag([0.05, 0.05, 0.05, 1.0]).astype(np.float32)
    R0 = O.mat4_mul(O.euler_rotation(*W.cli_rotation()), small)
    U = O.viewport_transform(640, 360, 1.0)
    frames = [{"w": 640, "h": 360, "image": True, "U": U, "draws": [(dm, R0)]} for _ in range(3)]
    b = S.Batch(ctx, frames)
    b.render()
    b.render()                      # graph captured with the small entry buffer
    R1 = O.euler_rotation(*W.cli_rotation(yaw=0.3))
    b.set_transforms(np.stack([R1] * 3))
    b.render()                      # the graph overflows the entry buffer
    ref = oracle_render([m], R1, 640, 360, True, U=U)
    for i in range(3):
        assert_same((*b.read(i), None), ref, f"overflow frame {i}")
    b.close()


def test_batch_exact_across_setting_changes(ctx):
    """One batch through graph replays, new transforms, the direct path switched off and
    on, a tile-shape change and an entry overflow with the direct path on, on even- and
    odd-width frames: every frame exact after every render (the keys the direct folds
    need are cleared at the right renders, the graph is captured again when it must)."""
    meshes, dev, frames = mixed_frames(ctx)
    frames = frames[:10]
    b = S.Batch(ctx, frames)
    rng = np.random.default_rng(17)

    def new_transforms():
        mats = []
        for f in frames:
            R = O.euler_rotation(*W.cli_rotation(yaw=float(rng.uniform(0, 6.28))))
            f["R"] = R
            mats += [R] * len(f["draws"])
        b.set_transforms(np.stack(mats))

    steps = [("direct 64", lambda: b.set_direct_samples(64)), ("replay", None), ("replay", None),
             ("transforms", new_transforms), ("direct 0", lambda: b.set_direct_samples(0)),
             ("direct 16", lambda: b.set_direct_samples(16)), ("replay", None),
             ("shape 1", lambda: b.set_tile_shape(1)), ("replay", None), ("transforms", new_transforms)]
    for name, change in steps:
        if change:
            change()
        b.render()
        check_frames(b, meshes, frames, name)
    # a transform that overflows the entry buffer, with the direct path on
    big = np.diag([4.0, 4.0, 4.0, 1.0]).astype(np.float32)
    mats = []
    for f in frames:
        f["R"] = O.mat4_mul(f["R"], big)
        mats += [f["R"]] * len(f["draws"])
    b.set_transforms(np.stack(mats))
    b.render()
    check_frames(b, meshes, frames, "overflow")
    b.render()
    check_frames(b, meshes, frames, "after the overflow")
    b.close()


@pytest.mark.parametrize("direct,tpb", [(0, 128), (16, 4096), (4, 256)])
def test_context_tuning_settings(ctx, direct, tpb):
    """Every value of the autotuner's other dimensions renders the same frame."""
    m = W.soup(6000, seed=52, n_large=15)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.2, pitch=0.4))
    ctx.set_triangles_per_block(tpb)
    try:
        ctx.set_direct_samples(direct)
        ctx.set_depth_cull(True)
        for w, h, image in [(321, 181, True), (200, 90, False)]:
            U = O.viewport_transform(w, h, 0.75)
            ref = oracle_render([m], R, w, h, image, U=U)
            assert_same(gpu_render(ctx, [m], R, w, h, image, U=U, depth_cull=True), ref, f"{direct}/{tpb} {w}x{h}")
    finally:
        ctx.set_triangles_per_block(256)
        ctx.set_direct_samples(0)


def test_context_autotune_renders_the_same_frame(ctx):
    m = W.soup(8000, seed=53, n_large=20)
    R = O.euler_rotation(*W.cli_rotation(yaw=1.1))
    dm = dev_mesh(ctx, m)
    w, h = 480, 270
    ctx.set_viewport(w, h, True)
    ctx.update([dm])
    best = ctx.autotune([(dm, R)], reps=2)
    assert 0 <= best["shape"] < len(S.tile_shapes()) and best["direct"] in (0, 4, 16, 64)
    assert best["tpb"] in (128, 256, 1024, 4096) and best["ms"] > 0
    ctx.clear()
    ctx.draw_mesh(dm, R)
    cells, z, winner = ctx.read()
    assert_same((cells, z, winner, None), oracle_render([m], R, w, h, True), "autotuned context")
    ctx.set_tile_shape(0)
    ctx.set_direct_samples(0)
    ctx.set_triangles_per_block(256)


@pytest.mark.parametrize("shape", range(5))
def test_context_every_tile_shape(ctx, shape):
    m = W.soup(6000, seed=51, n_large=15)
    R = O.euler_rotation(*W.cli_rotation(yaw=0.9, pitch=0.3))
    ctx.set_tile_shape(shape)
    try:
        for w, h, image in [(321, 181, True), (640, 360, False)]:
            U = O.viewport_transform(w, h, 0.75)
            ref = oracle_render([m], R, w, h, image, U=U)
            assert_same(gpu_render(ctx, [m], R, w, h, image, U=U), ref, f"shape {shape} {w}x{h}")
    finally:
        ctx.set_tile_shape(0)


@pytest.mark.parametrize("direct,persistent", [(0, True), (64, True), (0, False)])
def test_batch_dense_frames_split_tiles(ctx, direct, persistent):
    """Frames whose tiles hold more than 8192 entries (rasterized in slices) next to
    ordinary frames, planned and replayed."""
    dense = W.soup(50000, seed=43, n_large=3)
    ico = W.displaced_icosphere(3, seed=3)
    meshes = {"dense": dense, "ico": ico}
    dev = {k: dev_mesh(ctx, m) for k, m in meshes.items()}
    frames = []
    for i, (w, h, image, names) in enumerate([(80, 24, True, ["dense"]), (160, 48, False, ["ico"]),
                                              (64, 32, True, ["dense", "ico"]), (33, 9, False, ["dense"])]):
        R = O.euler_rotation(*W.cli_rotation(yaw=0.4 * i, pitch=0.2 * i))
        U = O.viewport_transform(w, h, O.scene_extent([meshes[n]["bbox_max"] for n in names]))
        frames.append({"w": w, "h": h, "image": image, "U": U, "names": names, "R": R,
                       "draws": [(dev[n], R) for n in names]})
    b = S.Batch(ctx, frames)
    b.set_direct_samples(direct)
    b.set_persistent(persistent)
    b.render()
    check_frames(b, meshes, frames, "planned")
    b.render()
    b.render()
    check_frames(b, meshes, frames, "graph")
    b.close()


def test_context_destroyed_before_its_batch_and_mesh():
    """Destroying a context detaches its batches and meshes: later calls on the batch
    fail cleanly and destroying the handles is safe (the meshes' buffers stay usable)."""
    c = S.Context(0)
    m = W.soup(300, seed=51)
    dm = dev_mesh(c, m)
    U = O.viewport_transform(40, 20, O.scene_extent([m["bbox_max"]]))
    b = S.Batch(c, [{"w": 40, "h": 20, "image": True, "U": U, "draws": [(dm, O.euler_rotation(0.0, 3.1, 0.0))]}])
    b.render()
    c2 = S.Context(0)
    c.close()
    with pytest.raises(S.SlothError):
        b.render()
    # the mesh still draws on another context of the same device
    c2.set_viewport(40, 20, True)
    c2.set_utransform(U)
    c2.clear()
    c2.draw_mesh(dm, O.euler_rotation(0.0, 3.1, 0.0))
    ref = oracle_render([m], O.euler_rotation(0.0, 3.1, 0.0), 40, 20, True, U=U)
    assert np.array_equal(c2.read()[0], ref.cells)
    b.close()
    dm.close()
    c2.close()
