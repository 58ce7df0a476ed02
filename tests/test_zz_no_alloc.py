"""sloth_render_noalloc: one frame without any device allocation by the library.

Callers that cannot let a library allocate device memory use this entry point instead of
the context API: hosts that fix the renderer's memory at start-up and forbid allocation
afterwards, frame loops that cannot afford cudaMalloc/cudaFree's device-wide
synchronisation, and programs whose device memory is held by a framework's caching pool.
The test gives it caller-owned device buffers (allocated here by torch, not by the
library) and checks its frames bit for bit against the oracle and against the context
path (sloth_ctx_clear + sloth_draw_mesh + sloth_ctx_read) on calls in a row: a smaller
frame, then a larger one (keys the first call left in the shared scratch array must not
show through), then an empty soup (the frame of a bare clear).
"""
import ctypes as C

import numpy as np
import pytest

import sloth_gpu as S
import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

LIMIT = 4


def context_frame(m, R, U, w, h, image):
    with S.Context(0) as ctx:
        dm = S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"])
        ctx.set_viewport(w, h, image)
        ctx.set_utransform(U)
        ctx.clear()
        ctx.draw_mesh(dm, R)
        return ctx.read()


def noalloc_frame(torch, m, R, U, w, h, image):
    lib = S.load_library()
    dev = torch.device("cuda", 0)
    ntri = int(m["rgb"].shape[0])
    ins = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (m["x"], m["y"], m["z"], m["rgb"].reshape(-1))]
    ptrs = [t.data_ptr() if ntri else None for t in ins]
    ncells = w * h + (h if image else 0)
    cells = torch.full((ncells,), -1, dtype=torch.int32, device=dev)
    zbuf = torch.full((w * h,), float("nan"), dtype=torch.float32, device=dev)
    winner = torch.full((w * h,), 7, dtype=torch.int32, device=dev)
    M = np.ascontiguousarray(O.mat4_mul(U, R).reshape(16), np.float32)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = lib.sloth_render_noalloc(ptrs[0], ptrs[1], ptrs[2], ntri, ptrs[3], M.ctypes.data_as(C.POINTER(C.c_float)),
                                  w, h, 1 if image else 0, cells.data_ptr(), zbuf.data_ptr(), winner.data_ptr(),
                                  C.c_void_p(stream))
    assert st == S.OK, st
    torch.cuda.synchronize()
    return cells.cpu().numpy().view(np.uint32), zbuf.cpu().numpy(), winner.cpu().numpy()


def assert_frames_equal(got, ref, label):
    for a, b, name in zip(got, ref, ("cells", "z", "winner")):
        av = a.view(np.uint32) if a.dtype == np.float32 else a
        bv = b.view(np.uint32) if b.dtype == np.float32 else b
        assert np.array_equal(av, bv), f"{label}: {name} differ at {np.nonzero(av != bv)[0][:5]}"


def empty_soup():
    z = np.zeros(0, np.float32)
    return {"x": z, "y": z, "z": z, "rgb": np.zeros((0, 3), np.uint8)}


def test_noalloc_matches_oracle_and_context_path():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cases = [
        # a smaller frame first, then a larger one with another mesh: the second call must
        # not see keys, tile generations or newlines the first one left in the scratch
        # array; then an empty soup, whose frame is a bare clear
        (W.soup(3000, seed=22, n_large=10, sigma=0.05), W.cli_rotation(yaw=1.3, pitch=0.2), 161, 48, False),
        (W.soup(12000, seed=21, n_large=30), W.cli_rotation(yaw=0.4), 640, 360, True),
        (empty_soup(), W.cli_rotation(), 320, 200, True),
    ]
    for m, ang, w, h, image in cases:
        R = O.euler_rotation(*ang)
        U = O.viewport_transform(w, h, 0.8)     # an extent below the soup's: wrapped cells
        got = noalloc_frame(torch, m, R, U, w, h, image)
        ntri = int(m["rgb"].shape[0])
        label = f"{ntri} triangles at {w}x{h}"
        orc = O.Oracle(w, h, image, U)
        if ntri:
            orc.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], R)
        ref = orc.frame()
        assert_frames_equal(got, (ref.cells, ref.z, ref.winner), label + " vs the oracle")
        if ntri:
            assert_frames_equal(got, context_frame(m, R, U, w, h, image), label + " vs the context path")
            assert (ref.winner >= 0).any()
        else:
            with S.Context(0) as ctx:
                ctx.set_viewport(w, h, image)
                ctx.clear()
                assert_frames_equal(got, ctx.read(), label + " vs a cleared context")


def test_noalloc_rejects_sizes_beyond_its_limits():
    lib = S.load_library()
    M = np.eye(4, dtype=np.float32).reshape(16)
    p = C.c_void_p(16)   # never dereferenced: the limits are checked before any GPU work
    mp = M.ctypes.data_as(C.POINTER(C.c_float))
    too_many = int(np.uint32(32768)) + 1
    assert lib.sloth_render_noalloc(p, p, p, too_many, p, mp, 64, 32, 0, p, p, p, None) == LIMIT
    assert lib.sloth_render_noalloc(p, p, p, 10, p, mp, 64, 4097, 0, p, p, p, None) == LIMIT
    assert lib.sloth_render_noalloc(p, p, p, 10, p, mp, 1024, 1024, 0, p, p, p, None) == LIMIT
    assert lib.sloth_render_noalloc(p, p, p, 10, p, None, 64, 32, 0, p, p, p, None) == 1
