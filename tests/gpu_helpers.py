"""Shared helpers of the GPU parity tests: render the same meshes through the C ABI
(libsloth_gpu.so on the GPU) and through the CPU oracle, and compare bit for bit."""
import numpy as np

import sloth_gpu as S
from oracle import oracle as O


def gpu_render(ctx, meshes, R, w, h, image, U=None, dev_meshes=None):
    """Clear, draw every mesh in order, read back.  Returns (cells, z, winner, fragments)."""
    ctx.set_viewport(w, h, image)
    if dev_meshes is None:
        dev_meshes = [S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m.get("idx"), m.get("bbox_max"))
                      for m in meshes]
    if U is None:
        ctx.update(dev_meshes)
    else:
        ctx.set_utransform(U)
    ctx.clear()
    Rs = R if isinstance(R, list) else [R] * len(dev_meshes)
    for dm, Rm in zip(dev_meshes, Rs):
        ctx.draw_mesh(dm, Rm)
    cells, z, winner = ctx.read()
    return cells, z, winner, ctx.fragments()


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
    assert frags == ref.fragments, f"{label}: fragments gpu {frags} ref {ref.fragments}"
