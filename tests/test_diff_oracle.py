"""The f64 CPU adjoint of the differentiable shading (oracle/diff_shade.py) against
central finite differences of its own forward, with the oracle's visibility (winner and
winner sample per depth cell) held fixed.  CPU only."""
import numpy as np
import pytest

import workloads as W
from oracle import diff_shade as D
from oracle import oracle as O

LIGHT = np.array([0.577, 0.577, 0.577])


def scene(subdiv=2, w=96, h=64, thetas=(0.3, 2.0), seed=1, image=False):
    m = W.displaced_icosphere(subdiv, seed=seed, amplitude=0.1)
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
    views = []
    for th in thetas:
        R = O.euler_rotation(*W.cli_rotation(pitch=th))
        f = O.render([m], R, w, h, image, U=U)
        views.append(D.View(O.mat4_mul(U, R), f.winner, f.winner_xy))
    pos = np.stack([m["x"], m["y"], m["z"]], 1).astype(np.float64)
    return m, pos, views


def loss(pos, vrgb, light, idx, views, grads):
    return sum(float((g * D.shade(pos, vrgb, light, idx, v)).sum()) for v, g in zip(views, grads))


@pytest.mark.parametrize("image", [False, True])
def test_adjoint_matches_central_differences(image):
    m, pos, views = scene(image=image)
    rng = np.random.default_rng(7)
    vrgb = rng.uniform(0, 1, (pos.shape[0], 3))
    grads = [rng.normal(size=(v.winner.size, 3)) for v in views]
    gp = np.zeros_like(pos)
    gc = np.zeros_like(vrgb)
    gl = np.zeros(3)
    for v, g in zip(views, grads):
        a, b, c = D.shade_vjp(pos, vrgb, LIGHT, m["idx"], v, g)
        gp += a
        gc += b
        gl += c
    h = 1e-6
    for _ in range(3):
        dp = rng.normal(size=pos.shape)
        dc = rng.normal(size=vrgb.shape)
        dl = rng.normal(size=3)
        fd = (loss(pos + h * dp, vrgb + h * dc, LIGHT + h * dl, m["idx"], views, grads)
              - loss(pos - h * dp, vrgb - h * dc, LIGHT - h * dl, m["idx"], views, grads)) / (2 * h)
        an = (gp * dp).sum() + (gc * dc).sum() + (gl * dl).sum()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)
    # each block on its own
    for which in range(3):
        d = [np.zeros_like(pos), np.zeros_like(vrgb), np.zeros(3)]
        d[which] = rng.normal(size=d[which].shape)
        fd = (loss(pos + h * d[0], vrgb + h * d[1], LIGHT + h * d[2], m["idx"], views, grads)
              - loss(pos - h * d[0], vrgb - h * d[1], LIGHT - h * d[2], m["idx"], views, grads)) / (2 * h)
        an = (gp * d[0]).sum() + (gc * d[1]).sum() + (gl * d[2]).sum()
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (which, fd, an)


def test_light_along_z_gives_the_reference_normal_z():
    """With L = (0,0,1) and white vertices the shade is clamp(normal z) of the reference's
    triangle (src/rasterizer.rs:76), the quantity its shader maps to a char."""
    m, pos, views = scene(thetas=(0.9,))
    v = views[0]
    img = D.shade(pos, np.ones_like(pos), np.array([0.0, 0.0, 1.0]), m["idx"], v)
    cells = np.nonzero(v.winner >= 0)[0]
    idx = m["idx"].reshape(-1, 3)
    for c in cells[:: max(1, len(cells) // 50)]:
        t = v.winner[c]
        tri = np.concatenate([np.r_[pos[i].astype(np.float32), np.float32(1.0)] for i in idx[t]])
        n = O.triangle_normal(O.triangle_mul(tri, v.M))
        exp = min(max(float(n[2]), 0.0), 1.0)
        assert np.allclose(img[c], exp, atol=1e-5), (c, img[c], exp)


def test_interior_mask_keeps_samples_inside_their_triangle():
    m, pos, views = scene()
    v = views[0]
    mask = D.interior_cells(pos, m["idx"], v)
    assert mask.sum() > 50
    assert not (mask & (v.winner < 0)).any()
    # a 2-pixel margin keeps a subset of the 1-pixel one
    m2 = D.interior_cells(pos, m["idx"], v, margin=2.0)
    assert not (m2 & ~mask).any()


def test_oracle_winner_sample_matches_depth_cell():
    """winner_xy is the sample whose depth cell id = y*w + 2x holds the winner, and the
    banded oracle records the same samples."""
    m = W.displaced_icosphere(2, seed=4)
    w, h = 81, 40
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
    R = O.euler_rotation(*W.cli_rotation(yaw=0.4, pitch=1.1))
    f = O.render([m], R, w, h, True, U=U)
    hit = np.nonzero(f.winner >= 0)[0]
    assert hit.size > 100
    xy = f.winner_xy[hit].astype(np.int64)
    x, y = xy & 0xFFFF, xy >> 16
    assert np.array_equal(y * w + 2 * x, hit)
    assert (f.winner_xy[f.winner < 0] == 0xFFFFFFFF).all()
    fb = O.render([m], R, w, h, True, U=U, threads=4)
    assert np.array_equal(fb.winner_xy, f.winner_xy)
