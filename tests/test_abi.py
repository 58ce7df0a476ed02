"""The C ABI library on a machine without a GPU: it loads, exports every function that
include/sloth_gpu.h declares, its host math equals the oracle's, and device calls fail
loudly (no CPU fallback) when there is no GPU."""
import re
from pathlib import Path

import numpy as np
import pytest

import sloth_gpu as S
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(sloth_\w+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not S.LIB_PATH.exists():
        import build  # rust-sloth_gb300/build.py
        build.build_library()
    return S.load_library()


def test_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(S.SIGNATURES), set(names) ^ set(S.SIGNATURES)


def test_version(lib):
    assert b"sm_103a" in lib.sloth_version()


def test_host_math_matches_oracle(lib):
    rng = np.random.default_rng(7)
    for _ in range(50):
        a = rng.normal(size=(4, 4)).astype(np.float32)
        b = rng.normal(size=(4, 4)).astype(np.float32)
        assert np.array_equal(S.mat4_mul(a, b), O.mat4_mul(a, b))
        ang = rng.uniform(-7, 7, size=3)
        assert np.array_equal(S.euler_rotation(*ang), O.euler_rotation(*ang))
        w, h = int(rng.integers(1, 4000)), int(rng.integers(1, 3000))
        e = float(rng.uniform(0.01, 10))
        assert np.array_equal(S.viewport_transform(w, h, e), O.viewport_transform(w, h, e))
        bb = rng.normal(size=(3, 3)).astype(np.float32)
        assert S.scene_extent(bb) == O.scene_extent(bb)
    for s in [-1.0, 0.2, 0.25, 0.5, 0.95, 1.0, 1.5, float("nan")]:
        assert S.default_shader(s) == O.default_shader(s)
    t = np.zeros(9, np.float32)
    ch = S.C.create_string_buffer(10)
    lib.sloth_shader_thresholds(t.ctypes.data_as(S._f32p), ch)
    assert t.tolist() == [np.float32(v) for v in (0.2, 0.3, 0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0)]
    assert ch.raw == b".:-=+*#%@ "


def test_no_cpu_fallback_without_gpu(lib):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(S.SlothError):
        S.Context()


def test_null_arguments_are_rejected(lib):
    assert lib.sloth_ctx_clear(None) == 1
    assert lib.sloth_draw_mesh(None, None, None) == 1
    assert lib.sloth_ctx_create(None, 0, None) == 1
