"""ctypes binding of libsloth_gpu.so (include/sloth_gpu.h).

A thin Python mirror of the reference's draw-path interface, for tests and benchmarks:

    Context  ~ Context (src/context.rs:12-141): set_viewport/update/clear/read
    Mesh     ~ SimpleMesh (src/geometry.rs:78-81), uploaded once
    ctx.draw_mesh(mesh, transform) ~ draw_mesh(&mut ctx, &mesh, transform, default_shader)

There is no CPU fallback: importing works anywhere, but creating a Context needs the
built library and a CUDA device, and every failure raises SlothError.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsloth_gpu.so"

OK = 0
ERR_INVALID_ARGUMENT, ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_LIMIT, ERR_DEVICE_FAULT = 1, 2, 3, 4, 5
OPTION_DEPTH_CULL = 1
OPTION_TILE_SHAPE = 2
OPTION_WAIT_TEST = 3
OPTION_DIRECT_SAMPLES = 4
OPTION_TRIANGLES_PER_BLOCK = 5
STATUS ={0: "OK", 1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "CUDA", 4: "LIMIT", 5: "DEVICE_FAULT"}

# Every symbol declared in include/sloth_gpu.h, with (restype, argtypes).
_f32p = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u8p = C.POINTER(C.c_uint8)
_u64p = C.POINTER(C.c_uint64)
_vp = C.c_void_p
SIGNATURES = {
    "sloth_version": (C.c_char_p, []),
    "sloth_shader_thresholds": (None, [_f32p, C.c_char_p]),
    "sloth_default_shader": (C.c_char, [C.c_float]),
    "sloth_euler_rotation": (None, [C.c_float, C.c_float, C.c_float, _f32p]),
    "sloth_mat4_mul": (None, [_f32p, _f32p, _f32p]),
    "sloth_scene_extent": (C.c_float, [_f32p, C.c_uint32]),
    "sloth_viewport_transform": (None, [C.c_uint16, C.c_uint16, C.c_float, _f32p]),
    "sloth_spatial_order": (C.c_int, [_f32p, _f32p, _f32p, C.c_uint32, _u32p, C.c_uint32, _u32p]),
    "sloth_ctx_create": (C.c_int, [C.POINTER(_vp), C.c_int, _vp]),
    "sloth_ctx_destroy": (None, [_vp]),
    "sloth_ctx_last_error": (C.c_char_p, [_vp]),
    "sloth_ctx_set_viewport": (C.c_int, [_vp, C.c_uint32, C.c_uint32, C.c_int]),
    "sloth_ctx_set_utransform": (C.c_int, [_vp, _f32p]),
    "sloth_ctx_update": (C.c_int, [_vp, C.POINTER(_vp), C.c_uint32]),
    "sloth_ctx_clear": (C.c_int, [_vp]),
    "sloth_ctx_sizes": (C.c_int, [_vp, _u64p, _u64p]),
    "sloth_ctx_read": (C.c_int, [_vp, _u32p, _f32p, _i32p]),
    "sloth_ctx_device_buffers": (C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    "sloth_ctx_fragments": (C.c_int, [_vp, _u64p]),
    "sloth_mesh_create": (C.c_int, [_vp, _f32p, _f32p, _f32p, C.c_uint32, _u32p, C.c_uint32,
                                    _u8p, _f32p, C.POINTER(_vp)]),
    "sloth_mesh_destroy": (None, [_vp]),
    "sloth_mesh_info": (C.c_int, [_vp, _u32p, _f32p]),
    "sloth_mesh_update": (C.c_int, [_vp, _f32p, _f32p, _f32p, _u8p]),
    "sloth_draw_mesh": (C.c_int, [_vp, _vp, _f32p]),
    "sloth_ctx_set_option": (C.c_int, [_vp, C.c_int, C.c_int64]),
    "sloth_ctx_autotune": (C.c_int, [_vp, C.POINTER(_vp), _f32p, C.c_uint32, C.c_int, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "sloth_render_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_uint32, _vp, _f32p, C.c_uint32, C.c_uint32,
                                       C.c_int, _vp, _vp, _vp, _vp]),
    "sloth_tile_shape": (C.c_int, [C.c_int, _u32p, _u32p]),
    "sloth_batch_create": (C.c_int, [_vp, _vp, C.c_uint32, _vp, C.c_uint32, C.POINTER(_vp)]),
    "sloth_batch_destroy": (None, [_vp]),
    "sloth_batch_set_transforms": (C.c_int, [_vp, _f32p]),
    "sloth_batch_render": (C.c_int, [_vp]),
    "sloth_batch_read": (C.c_int, [_vp, C.c_uint32, _u32p, _f32p, _i32p]),
    "sloth_batch_frame_buffers": (C.c_int, [_vp, C.c_uint32, C.POINTER(_vp), C.POINTER(_vp)]),
    "sloth_batch_fragments": (C.c_int, [_vp, _u64p]),
    "sloth_batch_set_tile_shape": (C.c_int, [_vp, C.c_int]),
    "sloth_batch_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "sloth_batch_set_triangles_per_block": (C.c_int, [_vp, C.c_int]),
    "sloth_batch_set_direct_samples": (C.c_int, [_vp, C.c_int]),
    "sloth_batch_set_persistent": (C.c_int, [_vp, C.c_int]),
    "sloth_batch_depth_cells": (C.c_int, [_vp, C.c_uint32, _u64p, _u64p]),
    "sloth_ctx_flush": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_uint64, _u64p]),
    "sloth_ctx_read_async": (C.c_int, [_vp, _u32p, _f32p, _i32p]),
    "sloth_ctx_synchronize": (C.c_int, [_vp]),
    "sloth_ctx_flush_device": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_void_p), _u64p]),
    "sloth_batch_flush": (C.c_int, [_vp, C.c_uint32, C.c_int, C.c_char_p, C.c_uint64, _u64p]),
    "sloth_batch_shade": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int]),
    "sloth_batch_shade_backward": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sloth_ctx_set_timing": (C.c_int, [_vp, C.c_int]),
    "sloth_ctx_kernel_time": (C.c_int, [_vp, C.c_char_p, C.POINTER(C.c_double), _u64p]),
    "sloth_ctx_launch_count": (C.c_uint64, [_vp]),
}


class SlothError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_lib = None


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load the built library (raises FileNotFoundError if it was not built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is not built; run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a: np.ndarray | None, ct):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ct))


def _mat(m) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float32).reshape(16))
    return a


# ---- host math -----------------------------------------------------------------------
def euler_rotation(roll: float, pitch: float, yaw: float) -> np.ndarray:
    out = np.zeros(16, np.float32)
    load_library().sloth_euler_rotation(C.c_float(roll), C.c_float(pitch), C.c_float(yaw), _ptr(out, C.c_float))
    return out.reshape(4, 4)


def mat4_mul(a, b) -> np.ndarray:
    a, b = _mat(a), _mat(b)
    out = np.zeros(16, np.float32)
    load_library().sloth_mat4_mul(_ptr(a, C.c_float), _ptr(b, C.c_float), _ptr(out, C.c_float))
    return out.reshape(4, 4)


def scene_extent(bbox_max) -> float:
    b = np.ascontiguousarray(np.asarray(bbox_max, np.float32).reshape(-1, 3))
    return float(load_library().sloth_scene_extent(_ptr(b, C.c_float), b.shape[0]))


def spatial_order(x, y, z, idx) -> np.ndarray:
    """The order in which setup takes an indexed mesh's triangles (sloth_spatial_order)."""
    x, y, z = (np.ascontiguousarray(a, np.float32) for a in (x, y, z))
    idx = np.ascontiguousarray(idx, np.uint32).reshape(-1)
    ntri = idx.size // 3
    out = np.zeros(max(ntri, 1), np.uint32)
    if not (x.size == y.size == z.size):
        raise ValueError("x, y and z differ in length")
    st = load_library().sloth_spatial_order(_ptr(x, C.c_float), _ptr(y, C.c_float), _ptr(z, C.c_float), x.size,
                                            _ptr(idx, C.c_uint32), ntri, _ptr(out, C.c_uint32))
    if st != 0:
        raise SlothError(st, "sloth_spatial_order")
    return out[:ntri]


def viewport_transform(width: int, height: int, extent: float) -> np.ndarray:
    out = np.zeros(16, np.float32)
    load_library().sloth_viewport_transform(width, height, C.c_float(extent), _ptr(out, C.c_float))
    return out.reshape(4, 4)


def default_shader(shade: float) -> str:
    return load_library().sloth_default_shader(C.c_float(shade)).decode()


# ---- context and meshes -----------------------------------------------------------------
class Context:
    """A render context on one GPU (the reference's Context)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.sloth_ctx_create(C.byref(h), device, C.c_void_p(stream) if stream else None)
        if st != OK:
            raise SlothError(st, "sloth_ctx_create failed (no CUDA device?)")
        self.h = h
        self.device = device
        self.width = self.height = 0
        self.image = False

    def _check(self, st: int):
        if st != OK:
            raise SlothError(st, self.lib.sloth_ctx_last_error(self.h).decode())

    def flush(self, fmt: int = 1) -> bytes:
        """Context::flush's stdout bytes for the current frame (FLUSH_PLAIN / _ANSI / _HTML),
        formatted on the GPU."""
        return _flush_bytes(lambda out, cap, n: self._check(self.lib.sloth_ctx_flush(self.h, fmt, out, cap, n)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.sloth_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_viewport(self, width: int, height: int, image: bool):
        self._check(self.lib.sloth_ctx_set_viewport(self.h, width, height, 1 if image else 0))
        self.width, self.height, self.image = width, height, bool(image)

    def set_utransform(self, u):
        u = _mat(u)
        self._check(self.lib.sloth_ctx_set_utransform(self.h, _ptr(u, C.c_float)))

    def update(self, meshes):
        arr = (C.c_void_p * len(meshes))(*[m.h for m in meshes])
        self._check(self.lib.sloth_ctx_update(self.h, arr, len(meshes)))

    def clear(self):
        self._check(self.lib.sloth_ctx_clear(self.h))

    def draw_mesh(self, mesh: "Mesh", transform):
        t = _mat(transform)
        self._check(self.lib.sloth_draw_mesh(self.h, mesh.h, _ptr(t, C.c_float)))

    def sizes(self):
        f, z = C.c_uint64(), C.c_uint64()
        self._check(self.lib.sloth_ctx_sizes(self.h, C.byref(f), C.byref(z)))
        return f.value, z.value

    def read(self, cells=True, z=True, winner=True):
        nf, nz = self.sizes()
        c = np.empty(nf, np.uint32) if cells else None
        zz = np.empty(nz, np.float32) if z else None
        w = np.empty(nz, np.int32) if winner else None
        self._check(self.lib.sloth_ctx_read(self.h, _ptr(c, C.c_uint32), _ptr(zz, C.c_float), _ptr(w, C.c_int32)))
        return c, zz, w

    def read_into(self, cells: np.ndarray | None, z: np.ndarray | None):
        self._check(self.lib.sloth_ctx_read(self.h, _ptr(cells, C.c_uint32), _ptr(z, C.c_float), None))

    def read_into_async(self, cells: np.ndarray | None, z: np.ndarray | None):
        """Queue the copies (complete at the next synchronize); keep the arrays alive."""
        self._pending = (cells, z)
        self._check(self.lib.sloth_ctx_read_async(self.h, _ptr(cells, C.c_uint32), _ptr(z, C.c_float), None))

    def synchronize(self):
        self._check(self.lib.sloth_ctx_synchronize(self.h))

    def device_buffers(self):
        c, z = C.c_void_p(), C.c_void_p()
        self._check(self.lib.sloth_ctx_device_buffers(self.h, C.byref(c), C.byref(z)))
        return c.value, z.value

    def fragments(self) -> int:
        f = C.c_uint64()
        self._check(self.lib.sloth_ctx_fragments(self.h, C.byref(f)))
        return f.value

    def set_tile_shape(self, shape: int):
        """SLOTH_OPTION_TILE_SHAPE (index into tile_shapes()); applies at the next clear."""
        self._check(self.lib.sloth_ctx_set_option(self.h, OPTION_TILE_SHAPE, shape))

    def set_depth_cull(self, on: bool):
        """SLOTH_OPTION_DEPTH_CULL: skip triangles proven hidden (same results)."""
        self._check(self.lib.sloth_ctx_set_option(self.h, OPTION_DEPTH_CULL, 1 if on else 0))

    def set_direct_samples(self, samples: int):
        """SLOTH_OPTION_DIRECT_SAMPLES: triangles of at most this many samples are folded
        straight into the depth keys by setup (same results); applies at the next clear."""
        self._check(self.lib.sloth_ctx_set_option(self.h, OPTION_DIRECT_SAMPLES, samples))

    def set_triangles_per_block(self, tpb: int):
        """SLOTH_OPTION_TRIANGLES_PER_BLOCK: 128, 256, 1024 or 4096 triangles per setup block."""
        self._check(self.lib.sloth_ctx_set_option(self.h, OPTION_TRIANGLES_PER_BLOCK, tpb))

    def autotune(self, draws, reps: int = 3) -> dict:
        """sloth_ctx_autotune over draws [(Mesh, transform), ...]: the fastest (tile shape,
        direct limit, triangles per block), now the context's options, and its frame time."""
        arr = (C.c_void_p * max(1, len(draws)))(*[m.h for m, _ in draws])
        mats = np.ascontiguousarray(np.stack([_mat(t) for _, t in draws]) if draws else np.zeros(16, np.float32))
        s, d, t, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        self._check(self.lib.sloth_ctx_autotune(self.h, arr, _ptr(mats, C.c_float), len(draws), reps, C.byref(s),
                                                C.byref(d), C.byref(t), C.byref(ms)))
        return {"shape": s.value, "direct": d.value, "tpb": t.value, "ms": ms.value}

    def set_timing(self, on: bool):
        self._check(self.lib.sloth_ctx_set_timing(self.h, 1 if on else 0))

    def kernel_time(self, name: str):
        ms, n = C.c_double(), C.c_uint64()
        self._check(self.lib.sloth_ctx_kernel_time(self.h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def launch_count(self) -> int:
        return int(self.lib.sloth_ctx_launch_count(self.h))


FLUSH_PLAIN, FLUSH_ANSI, FLUSH_HTML = 0, 1, 2


def _flush_bytes(call) -> bytes:
    n = C.c_uint64()
    call(None, 0, C.byref(n))
    buf = C.create_string_buffer(max(1, n.value))
    call(buf, n.value, C.byref(n))
    return buf.raw[:n.value]


class Mesh:
    """A mesh uploaded to a context's device (the reference's SimpleMesh)."""

    def __init__(self, ctx: Context, x, y, z, rgb, idx=None, bbox_max=None):
        self.lib = ctx.lib
        self.ctx = ctx
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        z = np.ascontiguousarray(z, np.float32)
        rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1)
        ntri = rgb.size // 3
        ix = None if idx is None else np.ascontiguousarray(idx, np.uint32).reshape(-1)
        bb = None if bbox_max is None else np.ascontiguousarray(bbox_max, np.float32).reshape(3)
        h = C.c_void_p()
        st = self.lib.sloth_mesh_create(ctx.h, _ptr(x, C.c_float), _ptr(y, C.c_float), _ptr(z, C.c_float),
                                        x.size, _ptr(ix, C.c_uint32), ntri, _ptr(rgb, C.c_uint8),
                                        _ptr(bb, C.c_float), C.byref(h))
        ctx._check(st)
        self.h = h
        self.ntri = ntri
        self.nvert = x.size

    def update(self, x, y, z, rgb):
        """Overwrite positions and colours in place (async; keep the arrays alive)."""
        self._keep = (x, y, z, rgb)
        st = self.lib.sloth_mesh_update(self.h, _ptr(x, C.c_float), _ptr(y, C.c_float), _ptr(z, C.c_float),
                                        _ptr(rgb, C.c_uint8))
        self.ctx._check(st)

    def update_device(self, x: int, y: int, z: int, rgb: int):
        """Overwrite positions and colours from device pointers (ints), asynchronously on
        the context's stream."""
        fp, bp = C.POINTER(C.c_float), C.POINTER(C.c_uint8)
        st = self.lib.sloth_mesh_update(self.h, C.cast(x, fp), C.cast(y, fp), C.cast(z, fp), C.cast(rgb, bp))
        self.ctx._check(st)

    @property
    def bbox_max(self) -> np.ndarray:
        out = np.zeros(3, np.float32)
        n = C.c_uint32()
        self.lib.sloth_mesh_info(self.h, C.byref(n), _ptr(out, C.c_float))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.lib.sloth_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FrameDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("image", C.c_int32),
                ("utransform", C.c_float * 16), ("first_draw", C.c_uint32), ("ndraws", C.c_uint32)]


class DrawDesc(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("transform", C.c_float * 16)]


def tile_shapes() -> list[tuple[int, int]]:
    lib = load_library()
    out, i = [], 0
    w, h = C.c_uint32(), C.c_uint32()
    while lib.sloth_tile_shape(i, C.byref(w), C.byref(h)) == OK:
        out.append((w.value, h.value))
        i += 1
    return out


class Batch:
    """Many frames rendered together (sloth_batch_*).

    frames: list of dicts {w, h, image, U, draws: [(Mesh, R), ...]}; each frame is drawn
    like ctx.clear() + ctx.draw_mesh(mesh, R) for its draws in order."""

    def __init__(self, ctx: Context, frames):
        self.ctx, self.lib = ctx, ctx.lib
        draws = [d for f in frames for d in f["draws"]]
        self._meshes = [m for m, _ in draws]   # keep alive
        fa = (FrameDesc * len(frames))()
        first = 0
        self.sizes = []
        for i, f in enumerate(frames):
            fa[i].width, fa[i].height, fa[i].image = f["w"], f["h"], 1 if f["image"] else 0
            for k, v in enumerate(_mat(f["U"])):
                fa[i].utransform[k] = float(v)
            fa[i].first_draw, fa[i].ndraws = first, len(f["draws"])
            first += len(f["draws"])
            nz = f["w"] * f["h"]
            self.sizes.append((nz + (f["h"] if f["image"] else 0), nz))
        da = (DrawDesc * max(1, len(draws)))()
        for i, (m, R) in enumerate(draws):
            da[i].mesh = m.h
            for k, v in enumerate(_mat(R)):
                da[i].transform[k] = float(v)
        h = C.c_void_p()
        ctx._check(self.lib.sloth_batch_create(ctx.h, C.cast(fa, C.c_void_p), len(frames), C.cast(da, C.c_void_p),
                                               len(draws), C.byref(h)))
        self.h = h
        self.ndraws = len(draws)

    def close(self):
        if getattr(self, "h", None):
            self.lib.sloth_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self):
        self.ctx._check(self.lib.sloth_batch_render(self.h))

    def set_transforms(self, mats):
        a = np.ascontiguousarray(np.asarray(mats, np.float32).reshape(self.ndraws * 16))
        self.ctx._check(self.lib.sloth_batch_set_transforms(self.h, _ptr(a, C.c_float)))

    def read(self, frame: int):
        nf, nz = self.sizes[frame]
        c, z, w = np.empty(nf, np.uint32), np.empty(nz, np.float32), np.empty(nz, np.int32)
        self.ctx._check(self.lib.sloth_batch_read(self.h, frame, _ptr(c, C.c_uint32), _ptr(z, C.c_float),
                                                  _ptr(w, C.c_int32)))
        return c, z, w

    def fragments(self) -> int:
        f = C.c_uint64()
        self.ctx._check(self.lib.sloth_batch_fragments(self.h, C.byref(f)))
        return f.value

    def set_tile_shape(self, shape: int):
        self.ctx._check(self.lib.sloth_batch_set_tile_shape(self.h, shape))

    def set_direct_samples(self, samples: int):
        self.ctx._check(self.lib.sloth_batch_set_direct_samples(self.h, samples))

    def set_persistent(self, on: bool):
        """Persistent raster over the device-side item queue (default) or one CTA per item."""
        self.ctx._check(self.lib.sloth_batch_set_persistent(self.h, 1 if on else 0))

    def set_triangles_per_block(self, tpb: int):
        self.ctx._check(self.lib.sloth_batch_set_triangles_per_block(self.h, tpb))

    def autotune(self, reps: int = 3) -> dict:
        """The fastest (tile shape, direct limit, triangles per block, persistent) setting,
        now set, and its mean render time."""
        s, d, t, p, ms = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_float()
        self.ctx._check(self.lib.sloth_batch_autotune(self.h, reps, C.byref(s), C.byref(d), C.byref(t), C.byref(p),
                                                      C.byref(ms)))
        return {"shape": s.value, "direct": d.value, "tpb": t.value, "persistent": bool(p.value), "ms": ms.value}

    def flush(self, frame: int, fmt: int = 1) -> bytes:
        """Context::flush's stdout bytes for one frame, formatted on the GPU."""
        return _flush_bytes(lambda out, cap, n: self.ctx._check(
            self.lib.sloth_batch_flush(self.h, frame, fmt, out, cap, n)))

    # ---- differentiable shading (device pointers as ints, e.g. torch data_ptr()) ----
    def depth_cells(self, frame: int) -> tuple[int, int]:
        """(first depth cell, count) of a frame in the shaded image's cell order."""
        a, n = C.c_uint64(), C.c_uint64()
        self.ctx._check(self.lib.sloth_batch_depth_cells(self.h, frame, C.byref(a), C.byref(n)))
        return a.value, n.value

    def shade(self, vertex_rgb: int, light: int, rgb: int, store_visibility: bool = True):
        self.ctx._check(self.lib.sloth_batch_shade(self.h, C.c_void_p(vertex_rgb), C.c_void_p(light),
                                                   C.c_void_p(rgb), 1 if store_visibility else 0))

    def shade_backward(self, vertex_rgb: int, light: int, grad_rgb: int, grad_pos: int = 0,
                       grad_vertex_rgb: int = 0, grad_light: int = 0):
        self.ctx._check(self.lib.sloth_batch_shade_backward(
            self.h, C.c_void_p(vertex_rgb), C.c_void_p(light), C.c_void_p(grad_rgb),
            C.c_void_p(grad_pos or None), C.c_void_p(grad_vertex_rgb or None), C.c_void_p(grad_light or None)))


def cells_to_text(cells: np.ndarray) -> str:
    """The chars of a frame buffer as one string (Context::flush without colour)."""
    return (cells & 0xFF).astype(np.uint8).tobytes().decode("ascii")
