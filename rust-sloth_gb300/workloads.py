"""Seeded synthetic meshes for the sloth rasterization path, and minimal OBJ/STL I/O.

Meshes are dicts of numpy arrays in the C ABI's layout:
    x, y, z : float32 vertex positions (structure of arrays)
    idx     : uint32 (ntri, 3) vertex indices, or None for an unindexed soup
    rgb     : uint8 (ntri, 3) face colours (Triangle.color)
    bbox_max: float32 (3,) SimpleMesh bounding_box.max

The generators stand in for the model files the reference CLI loads (the reference ships
no benchmark meshes); every one is a pure function of its seed.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

PI_F32 = np.float32(math.pi)


def obj_bbox_max(x, y, z, idx) -> np.ndarray:
    """bounding_box.max of an OBJ-loaded mesh: grown from the origin over every triangle's
    vertices (src/geometry.rs:86-89,128-135)."""
    if idx is None:
        vx, vy, vz = x, y, z
    else:
        used = np.asarray(idx).reshape(-1)
        vx, vy, vz = x[used], y[used], z[used]
    b = np.zeros(3, np.float32)
    if vx.size:
        b = np.maximum(b, np.array([np.nanmax(vx), np.nanmax(vy), np.nanmax(vz)], np.float32))
    return b.astype(np.float32)


def _mesh(x, y, z, idx, rgb) -> dict:
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    z = np.ascontiguousarray(z, np.float32)
    idx = None if idx is None else np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
    rgb = np.ascontiguousarray(rgb, np.uint8).reshape(-1, 3)
    return {"x": x, "y": y, "z": z, "idx": idx, "rgb": rgb, "bbox_max": obj_bbox_max(x, y, z, idx)}


def ntri(m: dict) -> int:
    return m["rgb"].shape[0]


def _orient_outward(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Reorder each face so that it winds counter-clockwise seen from outside (normal
    along the centroid direction)."""
    a, b, c = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, (a + b + c)) < 0
    f = faces.copy()
    f[flip, 1], f[flip, 2] = faces[flip, 2], faces[flip, 1]
    return f


def uv_sphere(lon: int = 32, lat: int = 16, radius: float = 1.0, rgb=(1, 1, 1)) -> dict:
    """UV sphere: two polar fans of `lon` triangles and (lat-2) bands of 2*lon triangles
    (32 x 16 -> 960 triangles).  Faces CCW from outside; y is the polar axis.  The
    default colour is the loader's colour for an OBJ without materials (1,1,1)."""
    pos = [(0.0, radius, 0.0)]
    for i in range(1, lat):
        th = math.pi * i / lat
        for j in range(lon):
            ph = 2.0 * math.pi * j / lon
            pos.append((radius * math.sin(th) * math.cos(ph), radius * math.cos(th),
                        radius * math.sin(th) * math.sin(ph)))
    pos.append((0.0, -radius, 0.0))
    pos = np.array(pos, np.float64)
    south = len(pos) - 1

    def ring(i, j):
        return 1 + (i - 1) * lon + (j % lon)

    faces = []
    for j in range(lon):
        faces.append((0, ring(1, j), ring(1, j + 1)))
    for i in range(1, lat - 1):
        for j in range(lon):
            a, b, c, d = ring(i, j), ring(i, j + 1), ring(i + 1, j), ring(i + 1, j + 1)
            faces.append((a, c, b))
            faces.append((b, c, d))
    for j in range(lon):
        faces.append((south, ring(lat - 1, j + 1), ring(lat - 1, j)))
    faces = _orient_outward(pos, np.array(faces, np.int64))
    p32 = pos.astype(np.float32)
    col = np.tile(np.array(rgb, np.uint8), (len(faces), 1))
    return _mesh(p32[:, 0], p32[:, 1], p32[:, 2], faces, col)


def soup(n_small: int, seed: int, n_large: int = 0, sigma: float = 0.02) -> dict:
    """Triangle soup: centroids U[-1,1]^3, vertices = centroid + N(0, sigma) per axis;
    plus `n_large` triangles with vertices U[-1,1]^3 (appended after the small ones).
    Vertex colours are uniform u8; a face takes its first vertex's colour, as the
    reference's OBJ loader does (src/geometry.rs:118-126)."""
    rng = np.random.default_rng(seed)
    cen = rng.uniform(-1.0, 1.0, size=(n_small, 1, 3))
    off = rng.normal(0.0, sigma, size=(n_small, 3, 3))
    small = (cen + off).reshape(-1, 3)
    large = rng.uniform(-1.0, 1.0, size=(n_large * 3, 3))
    pos = np.concatenate([small, large]).astype(np.float32)
    vcol = rng.integers(0, 256, size=(pos.shape[0], 3), dtype=np.uint8)
    face_rgb = vcol[0::3].copy()
    return _mesh(pos[:, 0], pos[:, 1], pos[:, 2], None, face_rgb)


def icosphere(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (positions float64 (V,3), faces int64 (F,3)), F = 20*4^subdiv."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
                  (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
                  (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
                  (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e_sorted = np.sort(e, axis=1)
        uniq, inv = np.unique(e_sorted, axis=0, return_inverse=True)
        mids = v[uniq[:, 0]] + v[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mids])
        nf = f.shape[0]
        inv = inv.reshape(-1)
        m01, m12, m20 = base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    f = _orient_outward(v, f)
    return v, f


def value_noise3(p: np.ndarray, seed: int, freq: float = 2.0, lattice: int = 16) -> np.ndarray:
    """Seeded 3-D value noise in [-1,1]: random values on an integer lattice (periodic),
    trilinear interpolation with smoothstep weights."""
    rng = np.random.default_rng(seed)
    table = rng.uniform(-1.0, 1.0, size=(lattice, lattice, lattice))
    q = (p + 1.0) * freq
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    s = f * f * (3.0 - 2.0 * f)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = ((s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) *
                     (s[:, 2] if dz else 1 - s[:, 2]))
                val = table[(i0[:, 0] + dx) % lattice, (i0[:, 1] + dy) % lattice, (i0[:, 2] + dz) % lattice]
                out += w * val
    return out


def displaced_icosphere(subdiv: int, seed: int, amplitude: float = 0.1, rgb=(200, 180, 90)) -> dict:
    """Icosphere whose vertices are pushed along the radius by amplitude * value noise."""
    v, f = icosphere(subdiv)
    if amplitude:
        v = v * (1.0 + amplitude * value_noise3(v, seed))[:, None]
    p32 = v.astype(np.float32)
    col = np.tile(np.array(rgb, np.uint8), (f.shape[0], 1))
    return _mesh(p32[:, 0], p32[:, 1], p32[:, 2], f, col)


def vertex_colours(m: dict, seed: int, freq: float = 1.5) -> np.ndarray:
    """(nvert, 3) f32 vertex colours in [0, 1]: one seeded value-noise field per channel."""
    p = np.stack([m["x"], m["y"], m["z"]], 1).astype(np.float64)
    c = np.stack([0.5 + 0.5 * value_noise3(p, seed + k, freq) for k in range(3)], 1)
    return np.clip(c, 0.0, 1.0).astype(np.float32)


def cli_rotation(yaw: float = 0.0, pitch: float = 0.0, roll: float = 0.0) -> tuple[float, float, float]:
    """The Euler angles (roll, pitch, yaw slots of from_euler_angles) that the CLI builds
    from `-x/--yaw`, `-y/--pitch`, `-z/--roll` (src/inputs.rs:131-149): the yaw flag feeds
    the roll slot and pi is added to the pitch in f32."""
    return (float(np.float32(yaw)), float(np.float32(np.float32(pitch) + PI_F32)), float(np.float32(roll)))


# ---- OBJ I/O (a subset of tobj 3.2.2 with GPU_LOAD_OPTIONS) --------------------------------
def write_obj(path: Path | str, m: dict) -> None:
    """Triangle-only OBJ with %.9g floats (exact f32 round trip), no materials."""
    x, y, z = m["x"], m["y"], m["z"]
    idx = m["idx"] if m["idx"] is not None else np.arange(x.size, dtype=np.uint32).reshape(-1, 3)
    with open(path, "w") as fh:
        fh.write("# sloth-gb300 synthetic mesh\n")
        fh.writelines(f"v {a:.9g} {b:.9g} {c:.9g}\n" for a, b, c in zip(x.tolist(), y.tolist(), z.tolist()))
        fh.writelines(f"f {a + 1} {b + 1} {c + 1}\n" for a, b, c in idx.tolist())


class LoadError(Exception):
    """A file the reference's loaders would reject."""


_libc = None


def _strtof(tok: str) -> float:
    """C strtof: the correctly rounded float32 of a decimal (Rust's f32::from_str), without
    the double rounding of float() followed by a float32 cast."""
    global _libc
    import ctypes
    try:
        float(tok)
    except ValueError:
        raise LoadError(f"bad number {tok!r}")
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.strtof.restype = ctypes.c_float
        _libc.strtof.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    return _libc.strtof(tok.encode(), None)


def _rest(line: str, tag: str) -> str:
    return line.split(tag, 1)[1].strip() if tag in line else ""


def read_obj(path: Path | str) -> list[dict]:
    """Read an OBJ the way the reference's loader sees it (tobj 3.2.2 load_obj with
    GPU_LOAD_OPTIONS, then to_simple_mesh_with_materials, src/geometry.rs:83-148): a new
    mesh at every object or group, and at a change to a different known material; polygons
    fan-triangulated (v0, vi, vi+1); colour = material Kd*255 as u8, replaced by the first
    corner's vertex colour when `v` lines carry colours, (1,1,1) when the file has no
    materials.  A missing material library or a face without a material when there are
    materials are errors, as they are for the reference.  Restates tobj's published
    behaviour for the features the reference models use; parity with tobj itself is not
    pinned.  Every mesh is an unindexed soup with its origin-grown bounding box."""
    path = Path(path)
    pos, vcol = [], []
    materials: list[tuple[str, list]] = []
    mtl_failed = False
    groups = []   # (material index or None, [corner position indices])
    cur: list = []
    cur_mat = None

    def flush():
        nonlocal cur
        if cur:
            groups.append((cur_mat, cur))
        cur = []

    for line in path.read_text(errors="replace").splitlines():
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        tag = parts[0]
        if tag == "v":
            if len(parts) < 4:
                raise LoadError("PositionParseError")
            pos.append([_strtof(t) for t in parts[1:4]])
            if len(parts) >= 7:
                vcol.append([_strtof(t) for t in parts[4:7]])
        elif tag == "f":
            ids = []
            for tok in parts[1:]:
                head = tok.split("/")[0]
                try:
                    i = int(head)
                except ValueError:
                    raise LoadError("FaceParseError")
                if i == 0:
                    raise LoadError("FaceParseError")
                j = i - 1 if i > 0 else len(pos) + i
                if not 0 <= j < len(pos):
                    raise LoadError("FaceVertexOutOfBounds")
                ids.append(j)
            for k in range(1, len(ids) - 1):
                cur += [ids[0], ids[k], ids[k + 1]]
        elif tag in ("o", "g"):
            flush()
        elif tag == "usemtl":
            name = _rest(line, "usemtl")
            if not name:
                raise LoadError("MaterialParseError")
            found = next((k for k, (n, _) in enumerate(materials) if n == name), None)
            if found is not None and found != cur_mat:
                flush()
            cur_mat = found
        elif tag == "mtllib" and len(parts) > 1:
            mp = path.parent / parts[1]
            if not mp.exists():
                mtl_failed = True
                continue
            for ml in mp.read_text(errors="replace").splitlines():
                mt = ml.split()
                if not mt or mt[0].startswith("#"):
                    continue
                if mt[0] == "newmtl":
                    materials.append((_rest(ml, "newmtl"), [0.0, 0.0, 0.0]))
                elif mt[0] == "Kd" and materials and len(mt) >= 4:
                    materials[-1] = (materials[-1][0], [_strtof(t) for t in mt[1:4]])
    flush()
    if mtl_failed:
        raise LoadError("Expected to have materials.")
    P = np.array(pos, np.float32).reshape(-1, 3)
    VC = np.array(vcol, np.float32).reshape(-1, 3)
    meshes = []
    for mat, corners in groups:
        F = np.array(corners, np.int64).reshape(-1, 3)
        col = np.ones((F.shape[0], 3), np.uint8)
        if materials:
            if mat is None:
                raise LoadError("a face without a material")
            col[:] = _f32_to_u8(np.array(materials[mat][1], np.float32) * np.float32(255.0))
            if VC.size:
                if F[:, 0].max() >= VC.shape[0]:
                    raise LoadError("vertex colour index out of range")
                col = _f32_to_u8(VC[F[:, 0]] * np.float32(255.0))
        flat = P[F].reshape(-1, 3)
        meshes.append(_mesh(flat[:, 0], flat[:, 1], flat[:, 2], None, col))
    return meshes


def _f32_to_u8(a: np.ndarray) -> np.ndarray:
    """Rust `f32 as u8`: truncation, saturating at 0 and 255, NaN -> 0."""
    a = np.nan_to_num(np.asarray(a, np.float32), nan=0.0)
    return np.clip(np.trunc(a), 0, 255).astype(np.uint8)


def read_stl(path: Path | str) -> dict:
    """Binary or ASCII STL, the way the reference sees it (stl_io 0.4.2 read_stl then
    to_simple_mesh, src/geometry.rs:150-189): ASCII when the file starts with "solid ",
    binary otherwise; facets in file order, colour (255,255,0), bounding box grown from
    (+MAX, -MAX) over the facets."""
    data = Path(path).read_bytes()
    if data.startswith(b"solid "):
        verts = [[_strtof(t) for t in line.split()[1:4]] for line in data.decode(errors="replace").splitlines()
                 if line.split()[:1] == ["vertex"]]
        if len(verts) % 3:
            raise LoadError("incomplete facet")
        tris = np.array(verts, np.float32).reshape(-1, 3, 3)
    else:
        if len(data) < 84:
            raise LoadError("short header")
        n = int.from_bytes(data[80:84], "little")
        if len(data) < 84 + 50 * n:
            raise LoadError("short file")
        rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]),
                            count=n, offset=84)
        tris = rec["v"].astype(np.float32)
    flat = tris.reshape(-1, 3)
    m = _mesh(flat[:, 0], flat[:, 1], flat[:, 2], None, np.tile(np.array([255, 255, 0], np.uint8), (tris.shape[0], 1)))
    m["bbox_max"] = np.max(tris.reshape(-1, 3), axis=0).astype(np.float32) if tris.size else \
        np.full(3, -np.finfo(np.float32).max, np.float32)
    return m
