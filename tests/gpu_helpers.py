"""Shared helpers of the GPU parity tests: render the same meshes through the C ABI
(libsloth_gpu.so on the GPU) and through the CPU oracle, and compare bit for bit."""
import numpy as np

import sloth_gpu as S
from oracle import oracle as O


def _render_once(ctx, dev_meshes, Rs, w, h, image, U, depth_cull, direct=0):
    ctx.set_depth_cull(depth_cull)
    ctx.set_direct_samples(direct)
    ctx.set_viewport(w, h, image)
    if U is None:
        ctx.update(dev_meshes)
    else:
        ctx.set_utransform(U)
    ctx.clear()
    for dm, Rm in zip(dev_meshes, Rs):
        ctx.draw_mesh(dm, Rm)
    cells, z, winner = ctx.read()
    return cells, z, winner, ctx.fragments()


def gpu_render(ctx, meshes, R, w, h, image, U=None, dev_meshes=None, depth_cull=None):
    """Clear, draw every mesh in order, read back: (cells, z, winner, fragments).

    depth_cull None renders four times: without depth culling (where every covered sample
    is counted, so the fragment count is compared) and with it, each with every triangle
    binned and with the small ones folded straight into the keys by setup (direct limits 64
    and 16); all four buffers must be identical, and so must the two unculled fragment
    counts.  The returned tuple is the culled, binned render with the unculled count."""
    if dev_meshes is None:
        dev_meshes = [S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m.get("idx"), m.get("bbox_max"))
                      for m in meshes]
    Rs = R if isinstance(R, list) else [R] * len(dev_meshes)
    if depth_cull is not None:
        out = _render_once(ctx, dev_meshes, Rs, w, h, image, U, depth_cull)
        return out if not depth_cull else (*out[:3], None)
    plain = _render_once(ctx, dev_meshes, Rs, w, h, image, U, False)
    culled = _render_once(ctx, dev_meshes, Rs, w, h, image, U, True)
    direct = _render_once(ctx, dev_meshes, Rs, w, h, image, U, False, direct=64)
    direct_culled = _render_once(ctx, dev_meshes, Rs, w, h, image, U, True, direct=16)
    for other, what in ((culled, "depth culling"), (direct, "the direct path"),
                        (direct_culled, "the direct path with depth culling")):
        for a, b, name in zip(plain[:3], other[:3], ("cells", "z", "winner")):
            assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                                  b.view(np.uint32) if b.dtype == np.float32 else b), \
                f"{what} changed the {name} buffer"
    assert culled[3] <= plain[3] and direct_culled[3] <= plain[3]
    assert direct[3] == plain[3], f"fragments: direct path {direct[3]}, binned {plain[3]}"
    ctx.set_depth_cull(True)
    ctx.set_direct_samples(0)
    return (*culled[:3], plain[3])


def oracle_render(meshes, R, w, h, image, U=None, threads=1):
    if U is None:
        U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"] for m in meshes]))
    o = O.Oracle(w, h, image, U)
    Rs = R if isinstance(R, list) else [R] * len(meshes)
    for m, Rm in zip(meshes, Rs):
        o.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], Rm, m.get("idx"), threads=threads)
    return o.frame()


def assert_same(gpu, ref, label=""):
    cells, z, winner, frags = gpu
    bad_c = np.nonzero(cells != ref.cells)[0]
    bad_z = np.nonzero(z.view(np.uint32) != ref.z.view(np.uint32))[0]
    bad_w = np.nonzero(winner != ref.winner)[0]
    msg = (f"{label}: {bad_c.size} frame cells, {bad_z.size} depth cells, {bad_w.size} winners differ; "
           f"first cells {bad_c[:5].tolist()} gpu {cells[bad_c[:5]].tolist()} ref {ref.cells[bad_c[:5]].tolist()}; "
           f"first z {bad_z[:5].tolist()} gpu {z[bad_z[:5]].tolist()} ref {ref.z[bad_z[:5]].tolist()}; "
           f"winners gpu {winner[bad_w[:5]].tolist()} ref {ref.winner[bad_w[:5]].tolist()}")
    assert bad_c.size == 0 and bad_z.size == 0 and bad_w.size == 0, msg
    if frags is not None:
        assert frags == ref.fragments, f"{label}: fragments gpu {frags} ref {ref.fragments}"
