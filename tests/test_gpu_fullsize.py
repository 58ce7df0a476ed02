"""The benchmarked workloads at their full sizes, bit for bit against the oracle.

- config 2: 1,000,000 small + 2,000 large soup triangles at 3840x2160 in image mode, the
  frame every headline number is quoted on (rendered with depth culling off, where every
  covered sample is counted, and on);
- config 3: all 320 frames of the batched workload (256 views of the 81,920-triangle
  displaced icosphere at 640x360 and 64 soups of 1k-500k triangles at 80x24 .. 1920x1080),
  rendered in one batch, first with the planned render, then through the graph replay.

The oracle renders the config-2 frame banded over every host thread, and the config-3
frames one per host thread (bench.check_frames_vs_oracle).
"""
import os

import numpy as np
import pytest

import bench
import sloth_gpu as S
import workloads as W
from oracle import oracle as O
from gpu_helpers import assert_same, gpu_render

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def test_config2_full_frame():
    m = W.soup(1_000_000, seed=2, n_large=2000)
    R = O.euler_rotation(*W.cli_rotation())
    ref = O.render([m], R, 3840, 2160, True, threads=THREADS)
    with S.Context(0) as ctx:
        got = gpu_render(ctx, [m], R, 3840, 2160, True)
    assert ref.fragments > 100_000_000
    assert_same(got, ref, "config 2, 1,002,000 triangles at 3840x2160")


def test_config3_every_frame():
    meshes, specs = bench.config3_frames()
    jobs = [([meshes[mi]], R, w, h, im, U) for mi, w, h, im, U, R in specs]
    with S.Context(0) as ctx:
        dev = [S.Mesh(ctx, m["x"], m["y"], m["z"], m["rgb"], m["idx"], m["bbox_max"]) for m in meshes]
        frames = [{"w": w, "h": h, "image": im, "U": U, "draws": [(dev[mi], R)]} for mi, w, h, im, U, R in specs]
        b = S.Batch(ctx, frames)
        try:
            b.render()                                   # planned render (sizes the entries)
            planned = bench.check_frames_vs_oracle(jobs, b.read, THREADS)
            b.render()                                   # graph capture
            b.render()                                   # graph replay
            replayed = bench.check_frames_vs_oracle(jobs, b.read, THREADS)
        finally:
            b.close()
    for name, res in (("planned", planned), ("graph", replayed)):
        assert res["frames_checked"] == 320
        assert res["frames_bitexact"] == 320, f"{name}: {res['mismatches']}"
    assert sum(np.asarray(m["rgb"]).shape[0] for m in meshes) > 5_000_000
