"""Differentiable shading on the GPU (sloth_batch_shade / sloth_batch_shade_backward)
against the f64 CPU reference (oracle/diff_shade.py) on the oracle's visibility, plus
central finite differences through the whole GPU render on interior pixels."""
import numpy as np
import pytest

import sloth_gpu as S
import workloads as W
from oracle import diff_shade as D
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

LIGHT = (0.577, 0.577, 0.577)


@pytest.fixture(scope="module")
def env():
    stream = torch.cuda.Stream(torch.device("cuda", 0))
    ctx = S.Context(0, stream=stream.cuda_stream)
    yield ctx, stream
    torch.cuda.synchronize()
    ctx.close()


def views_of(m, specs):
    """specs: (w, h, image, pitch) -> view dicts sharing the mesh's utransform extent."""
    ext = O.scene_extent([m["bbox_max"]])
    out = []
    for w, h, image, th in specs:
        U = O.viewport_transform(w, h, ext)
        R = O.euler_rotation(*W.cli_rotation(pitch=th, yaw=0.2 * th))
        out.append({"w": w, "h": h, "image": image, "U": U, "R": R})
    return out


def oracle_views(m, views, pos=None):
    mm = dict(m)
    if pos is not None:
        p32 = np.asarray(pos, np.float32)
        mm.update(x=p32[:, 0].copy(), y=p32[:, 1].copy(), z=p32[:, 2].copy())
    out = []
    for v in views:
        f = O.render([mm], v["R"], v["w"], v["h"], v["image"], U=v["U"])
        out.append(D.View(O.mat4_mul(v["U"], v["R"]), f.winner, f.winner_xy))
    return out


def host_pos(m):
    return np.stack([m["x"], m["y"], m["z"]], 1).astype(np.float32)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


SPECS = [(160, 96, False, 0.4), (161, 95, True, 2.2), (64, 64, False, 4.0)]


@pytest.mark.parametrize("store", [True, False])
def test_forward_and_backward_match_f64(env, store):
    import diff_render as DR
    ctx, stream = env
    m = W.displaced_icosphere(3, seed=11, amplitude=0.1)
    views = views_of(m, SPECS)
    rng = np.random.default_rng(3)
    vrgb = rng.uniform(0, 1, (m["x"].size, 3)).astype(np.float32)
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        sv = DR.ShadedViews(ctx, m, views, stream, store_visibility=store)
        pos_t = torch.from_numpy(host_pos(m)).to(dev)
        vrgb_t = torch.from_numpy(vrgb).to(dev)
        light_t = torch.tensor(LIGHT, dtype=torch.float32, device=dev)
        sv.render(pos_t)
        rgb = sv.shade(vrgb_t, light_t)
        grads = torch.from_numpy(rng.normal(size=(sv.ncells, 3)).astype(np.float32)).to(dev)
        gp, gc, gl = sv.shade_backward(vrgb_t, light_t, grads)
        torch.cuda.synchronize()
    rgb_h, g_h = rgb.cpu().numpy(), grads.cpu().numpy()
    pos64 = host_pos(m).astype(np.float64)
    ref_p, ref_c, ref_l = np.zeros_like(pos64), np.zeros_like(pos64), np.zeros(3)
    for i, ov in enumerate(oracle_views(m, views)):
        a, n = sv.cells[i]
        ref = D.shade(pos64, vrgb.astype(np.float64), np.array(LIGHT), m["idx"], ov)
        assert np.abs(rgb_h[a:a + n] - ref).max() <= 1e-4, f"view {i}"
        # cells the oracle leaves empty are 0 on the GPU too
        assert not rgb_h[a:a + n][ov.winner < 0].any()
        p, c, l = D.shade_vjp(pos64, vrgb.astype(np.float64), np.array(LIGHT), m["idx"], ov, g_h[a:a + n])
        ref_p += p
        ref_c += c
        ref_l += l
    assert rel(gp.cpu().numpy(), ref_p) <= 1e-4
    assert rel(gc.cpu().numpy(), ref_c) <= 1e-4
    assert rel(gl.cpu().numpy(), ref_l) <= 1e-4
    sv.close()


def test_autograd_function_and_finite_differences_on_interior_pixels(env):
    """loss = sum over interior cells of (rgb - target)^2, target rendered from vertices
    perturbed by N(0, 0.01); autograd gradient vs central differences (h = 1e-3) of the
    GPU render, on cells whose sample is >= 1 px inside its triangle and whose winner is
    the same at +h and -h."""
    import diff_render as DR
    ctx, stream = env
    m = W.displaced_icosphere(3, seed=12, amplitude=0.1)
    views = views_of(m, [(192, 128, False, 0.7), (128, 128, True, 3.1)])
    rng = np.random.default_rng(5)
    dev = torch.device("cuda", 0)
    pos0 = host_pos(m)
    vrgb = rng.uniform(0, 1, (pos0.shape[0], 3)).astype(np.float32)
    with torch.cuda.stream(stream):
        sv = DR.ShadedViews(ctx, m, views, stream)
        light = torch.tensor(LIGHT, dtype=torch.float32, device=dev)
        vrgb_t = torch.from_numpy(vrgb).to(dev)
        tgt_pos = torch.from_numpy(pos0 + rng.normal(0, 0.01, pos0.shape).astype(np.float32)).to(dev)
        target = DR.shade_views(tgt_pos, vrgb_t, light, sv).detach().clone()
        pos_t = torch.from_numpy(pos0).to(dev)
        d = torch.from_numpy(rng.normal(size=pos0.shape).astype(np.float32)).to(dev)
        h = 1e-3

        def winners():
            torch.cuda.synchronize()
            return np.concatenate([sv.batch.read(i)[2] for i in range(len(views))])

        DR.shade_views(pos_t + h * d, vrgb_t, light, sv)
        w_plus = winners()
        DR.shade_views(pos_t - h * d, vrgb_t, light, sv)
        w_minus = winners()
        DR.shade_views(pos_t, vrgb_t, light, sv)
        w0 = winners()
        interior = np.concatenate([D.interior_cells(pos0.astype(np.float64), m["idx"], ov)
                                   for ov in oracle_views(m, views)])
        mask_np = interior & (w_plus == w0) & (w_minus == w0)
        assert mask_np.sum() > 1000
        mask = torch.from_numpy(mask_np).to(dev)[:, None].float()

        def loss_at(p, v, l):
            rgb = DR.shade_views(p, v, l, sv)
            return (((rgb - target) ** 2) * mask).double().sum()

        p = pos_t.clone().requires_grad_(True)
        v = vrgb_t.clone().requires_grad_(True)
        l = light.clone().requires_grad_(True)
        loss_at(p, v, l).backward()
        an = float((p.grad * d).sum())
        with torch.no_grad():
            fd = float((loss_at(pos_t + h * d, vrgb_t, light) - loss_at(pos_t - h * d, vrgb_t, light)) / (2 * h))
        assert abs(fd - an) <= 2e-2 * abs(an) + 1e-3, (fd, an)
        # colours and light enter linearly / smoothly: same check
        dc = torch.from_numpy(rng.normal(size=vrgb.shape).astype(np.float32)).to(dev)
        an_c = float((v.grad * dc).sum())
        with torch.no_grad():
            fd_c = float((loss_at(pos_t, vrgb_t + h * dc, light) - loss_at(pos_t, vrgb_t - h * dc, light)) / (2 * h))
        assert abs(fd_c - an_c) <= 1e-2 * abs(an_c) + 1e-3, (fd_c, an_c)
        dl = torch.tensor([0.3, -0.2, 0.5], device=dev)
        an_l = float((l.grad * dl).sum())
        with torch.no_grad():
            fd_l = float((loss_at(pos_t, vrgb_t, light + h * dl) - loss_at(pos_t, vrgb_t, light - h * dl)) / (2 * h))
        assert abs(fd_l - an_l) <= 1e-2 * abs(an_l) + 1e-3, (fd_l, an_l)
        torch.cuda.synchronize()
    sv.close()


def test_multi_draw_frame_and_soup(env):
    """A frame drawing the same soup twice with different transforms: the second draw's
    triangles follow the first's in draw order."""
    ctx, stream = env
    m = W.soup(600, seed=21, n_large=3)
    dev = torch.device("cuda", 0)
    w, h = 120, 80
    U = O.viewport_transform(w, h, O.scene_extent([m["bbox_max"]]))
    Ra = O.euler_rotation(*W.cli_rotation(yaw=0.3))
    Rb = O.euler_rotation(*W.cli_rotation(yaw=1.9, pitch=0.4))
    rng = np.random.default_rng(8)
    nv = m["x"].size
    vrgb = rng.uniform(0, 1, (nv, 3)).astype(np.float32)
    with torch.cuda.stream(stream):
        mesh = S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], None, m["bbox_max"])
        b = S.Batch(ctx, [{"w": w, "h": h, "image": True, "U": U, "draws": [(mesh, Ra), (mesh, Rb)]}])
        b.render()
        _, n = b.depth_cells(0)
        out = torch.empty(n, 3, device=dev)
        vt = torch.from_numpy(vrgb).to(dev)
        lt = torch.tensor(LIGHT, device=dev)
        b.shade(vt.data_ptr(), lt.data_ptr(), out.data_ptr(), False)
        g = torch.from_numpy(rng.normal(size=(n, 3)).astype(np.float32)).to(dev)
        gp = torch.zeros(nv, 3, device=dev)
        gc = torch.zeros(nv, 3, device=dev)
        b.shade_backward(vt.data_ptr(), lt.data_ptr(), g.data_ptr(), gp.data_ptr(), gc.data_ptr(), 0)
        torch.cuda.synchronize()
    o = O.Oracle(w, h, True, U)
    o.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], Ra)
    o.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], Rb)
    f = o.frame()
    ntri = m["rgb"].shape[0]
    pos64 = host_pos(m).astype(np.float64)
    ref = np.zeros((n, 3))
    ref_p, ref_c = np.zeros_like(pos64), np.zeros_like(pos64)
    gh = g.cpu().numpy()
    for R, lo, hi in ((Ra, 0, ntri), (Rb, ntri, 2 * ntri)):
        sel = (f.winner >= lo) & (f.winner < hi)
        v = D.View(O.mat4_mul(U, R), np.where(sel, f.winner - lo, -1), f.winner_xy)
        ref += D.shade(pos64, vrgb.astype(np.float64), np.array(LIGHT), None, v)
        p, c, _ = D.shade_vjp(pos64, vrgb.astype(np.float64), np.array(LIGHT), None, v, gh)
        ref_p += p
        ref_c += c
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-4
    assert rel(gp.cpu().numpy(), ref_p) <= 1e-4
    assert rel(gc.cpu().numpy(), ref_c) <= 1e-4
    b.close()
    mesh.close()


def test_shading_needs_one_mesh(env):
    ctx, stream = env
    a, b_ = W.soup(50, seed=1), W.soup(50, seed=2)
    dev = torch.device("cuda", 0)
    with torch.cuda.stream(stream):
        ma = S.Mesh(ctx, a["x"], a["y"], a["z"], a["rgb"])
        mb = S.Mesh(ctx, b_["x"], b_["y"], b_["z"], b_["rgb"])
        U = O.viewport_transform(40, 20, 1.0)
        R = O.euler_rotation(0.0, 0.0, 0.0)
        batch = S.Batch(ctx, [{"w": 40, "h": 20, "image": False, "U": U, "draws": [(ma, R)]},
                              {"w": 40, "h": 20, "image": False, "U": U, "draws": [(mb, R)]}])
        buf = torch.zeros(2 * 800, 3, device=dev)
        with pytest.raises(S.SlothError):
            batch.shade(buf.data_ptr(), buf.data_ptr(), buf.data_ptr())   # before any render
        batch.render()
        with pytest.raises(S.SlothError):
            batch.shade(buf.data_ptr(), buf.data_ptr(), buf.data_ptr())
        torch.cuda.synchronize()
    batch.close()
