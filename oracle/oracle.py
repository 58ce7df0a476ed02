"""ctypes wrapper of the CPU oracle (oracle/sloth_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline, always as the checker or the baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsloth_oracle.so"


class OrcCtx(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("image", C.c_int32),
        ("U", C.c_float * 16),
        ("z", C.POINTER(C.c_float)), ("cells", C.POINTER(C.c_uint32)),
        ("winner", C.POINTER(C.c_int32)),
        ("fragments", C.c_uint64), ("candidates", C.c_uint64), ("next_tri", C.c_uint32),
        ("winner_xy", C.POINTER(C.c_uint32)),
    ]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from oracle.build import build_oracle  # noqa: F401  (repo root on sys.path)
            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        f32p, u32p, u8p = C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_uint8)
        L.orc_default_shader.restype = C.c_char
        L.orc_default_shader.argtypes = [C.c_float]
        L.orc_clear.argtypes = [C.POINTER(OrcCtx)]
        L.orc_mat4_mul.argtypes = [f32p, f32p, f32p]
        L.orc_mat4_vec.argtypes = [f32p, f32p, f32p]
        L.orc_euler_rotation.argtypes = [C.c_float, C.c_float, C.c_float, f32p]
        L.orc_scene_extent.restype = C.c_float
        L.orc_scene_extent.argtypes = [f32p, C.c_uint32]
        L.orc_viewport_transform.argtypes = [C.c_uint16, C.c_uint16, C.c_float, f32p]
        L.orc_triangle_mul.argtypes = [f32p, f32p]
        L.orc_triangle_aabb.argtypes = [f32p, f32p, f32p]
        L.orc_triangle_normal.argtypes = [f32p, f32p]
        L.orc_draw_triangle.argtypes = [C.POINTER(OrcCtx), f32p, u8p, f32p]
        L.orc_draw_mesh.argtypes = [C.POINTER(OrcCtx), f32p, f32p, f32p, u32p, u8p, C.c_uint32, f32p]
        L.orc_draw_mesh_banded.argtypes = [C.POINTER(OrcCtx), f32p, f32p, f32p, u32p, u8p, C.c_uint32,
                                           f32p, C.c_int]
        L.orc_flush.restype = C.c_uint64
        L.orc_flush.argtypes = [u32p, C.c_uint64, C.c_int, C.c_int, C.c_char_p]
        _lib = L
    return _lib


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def _m(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, np.float32).reshape(16))


def mat4_mul(a, b) -> np.ndarray:
    a, b = _m(a), _m(b)
    out = np.zeros(16, np.float32)
    lib().orc_mat4_mul(_p(a, C.c_float), _p(b, C.c_float), _p(out, C.c_float))
    return out.reshape(4, 4)


def mat4_vec(m, v) -> np.ndarray:
    m = _m(m)
    v = np.ascontiguousarray(np.asarray(v, np.float32).reshape(4))
    out = np.zeros(4, np.float32)
    lib().orc_mat4_vec(_p(m, C.c_float), _p(v, C.c_float), _p(out, C.c_float))
    return out


def euler_rotation(roll, pitch, yaw) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_euler_rotation(C.c_float(roll), C.c_float(pitch), C.c_float(yaw), _p(out, C.c_float))
    return out.reshape(4, 4)


def scene_extent(bbox_max) -> float:
    b = np.ascontiguousarray(np.asarray(bbox_max, np.float32).reshape(-1, 3))
    return float(lib().orc_scene_extent(_p(b, C.c_float), b.shape[0]))


def viewport_transform(w, h, ext) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_viewport_transform(w, h, C.c_float(ext), _p(out, C.c_float))
    return out.reshape(4, 4)


def triangle_mul(v12, M) -> np.ndarray:
    v = np.ascontiguousarray(np.asarray(v12, np.float32).reshape(12)).copy()
    M = _m(M)
    lib().orc_triangle_mul(_p(v, C.c_float), _p(M, C.c_float))
    return v.reshape(3, 4)


def triangle_aabb(v12) -> tuple[np.ndarray, np.ndarray]:
    v = np.ascontiguousarray(np.asarray(v12, np.float32).reshape(12))
    mn, mx = np.zeros(4, np.float32), np.zeros(4, np.float32)
    lib().orc_triangle_aabb(_p(v, C.c_float), _p(mn, C.c_float), _p(mx, C.c_float))
    return mn, mx


def triangle_normal(v12) -> np.ndarray:
    v = np.ascontiguousarray(np.asarray(v12, np.float32).reshape(12))
    n = np.zeros(4, np.float32)
    lib().orc_triangle_normal(_p(v, C.c_float), _p(n, C.c_float))
    return n


def default_shader(s: float) -> str:
    return lib().orc_default_shader(C.c_float(s)).decode()


FLUSH_PLAIN, FLUSH_ANSI, FLUSH_HTML = 0, 1, 2


def flush(cells, image: bool, fmt: int) -> bytes:
    """Context::flush's stdout bytes for a frame of cells (src/context.rs:50-92)."""
    c = np.ascontiguousarray(cells, np.uint32)
    n = int(lib().orc_flush(_p(c, C.c_uint32), c.size, 1 if image else 0, fmt, None))
    buf = C.create_string_buffer(n)
    lib().orc_flush(_p(c, C.c_uint32), c.size, 1 if image else 0, fmt, buf)
    return buf.raw[:n]


@dataclass
class Frame:
    cells: np.ndarray     # uint32 per frame cell (char | r<<8 | g<<16 | b<<24)
    z: np.ndarray         # float32 per depth cell
    winner: np.ndarray    # int32 per depth cell
    fragments: int
    candidates: int
    winner_xy: np.ndarray = None   # uint32 per depth cell: sample x | y << 16 (0xffffffff: none)


class Oracle:
    """A CPU render context (Context of src/context.rs) with caller-visible buffers."""

    def __init__(self, width: int, height: int, image: bool, U):
        self.w, self.h, self.image = width, height, bool(image)
        n = width * height
        self.z = np.empty(n, np.float32)
        self.cells = np.empty(n + (height if image else 0), np.uint32)
        self.winner = np.empty(n, np.int32)
        self.winner_xy = np.empty(n, np.uint32)
        self.c = OrcCtx()
        self.c.width, self.c.height, self.c.image = width, height, 1 if image else 0
        for i, v in enumerate(_m(U)):
            self.c.U[i] = float(v)
        self.c.z = _p(self.z, C.c_float)
        self.c.cells = _p(self.cells, C.c_uint32)
        self.c.winner = _p(self.winner, C.c_int32)
        self.c.winner_xy = _p(self.winner_xy, C.c_uint32)
        self.clear()

    def clear(self):
        lib().orc_clear(C.byref(self.c))

    def draw_mesh(self, x, y, z, rgb, R, idx=None, threads: int = 1):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1)
        ix = None if idx is None else np.ascontiguousarray(idx, np.uint32).reshape(-1)
        R = _m(R)
        ntri = rgb.size // 3
        args = (C.byref(self.c), _p(x, C.c_float), _p(y, C.c_float), _p(z, C.c_float),
                _p(ix, C.c_uint32), _p(rgb, C.c_uint8), ntri, _p(R, C.c_float))
        if threads > 1:
            lib().orc_draw_mesh_banded(*args, threads)
        else:
            lib().orc_draw_mesh(*args)

    def draw_triangle(self, v9, rgb, M):
        v = np.ascontiguousarray(np.asarray(v9, np.float32).reshape(9))
        c = np.ascontiguousarray(np.asarray(rgb, np.uint8).reshape(3))
        M = _m(M)
        lib().orc_draw_triangle(C.byref(self.c), _p(v, C.c_float), _p(c, C.c_uint8), _p(M, C.c_float))

    def frame(self) -> Frame:
        return Frame(self.cells.copy(), self.z.copy(), self.winner.copy(),
                     int(self.c.fragments), int(self.c.candidates), self.winner_xy.copy())


def render(meshes, R, width, height, image, U=None, threads: int = 1) -> Frame:
    """Clear, draw every mesh in order with rotation R, return the frame.

    meshes: list of dicts with x, y, z, rgb (and optional idx, bbox_max).
    U: utransform; default = Context::update over the meshes' bbox_max."""
    if U is None:
        ext = scene_extent([m["bbox_max"] for m in meshes])
        U = viewport_transform(width, height, ext)
    o = Oracle(width, height, image, U)
    for m in meshes:
        o.draw_mesh(m["x"], m["y"], m["z"], m["rgb"], R, m.get("idx"), threads=threads)
    return o.frame()
