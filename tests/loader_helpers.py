"""Shared helpers for the loader tests: run the C++ loaders (sloth_meshdump, no GPU) and
summarise meshes."""
import hashlib
import struct
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
MESHDUMP = ROOT / "rust-sloth_gb300" / "_build" / "sloth_meshdump"


def cpp_meshes(files: str):
    """Meshes the C++ host loaders read from one `sloth` file argument, or the error text."""
    r = subprocess.run([str(MESHDUMP), files], capture_output=True)
    if r.returncode != 0:
        return r.stderr.decode().strip()
    b, off = r.stdout, 4
    out = []
    for _ in range(struct.unpack_from("<I", b, 0)[0]):
        n = struct.unpack_from("<I", b, off)[0]
        off += 4
        arr = lambda cnt, dt: np.frombuffer(b, dt, cnt, off)
        x = arr(3 * n, "<f4"); off += 12 * n
        y = arr(3 * n, "<f4"); off += 12 * n
        z = arr(3 * n, "<f4"); off += 12 * n
        rgb = arr(3 * n, np.uint8).reshape(-1, 3); off += 3 * n
        bmin = arr(3, "<f4"); off += 12
        bmax = arr(3, "<f4"); off += 12
        out.append({"x": x, "y": y, "z": z, "rgb": rgb, "bbox_min": bmin, "bbox_max": bmax})
    return out


def summary(m: dict) -> dict:
    h = hashlib.sha256()
    for k in ("x", "y", "z"):
        h.update(np.ascontiguousarray(m[k], np.float32).tobytes())
    h.update(np.ascontiguousarray(m["rgb"], np.uint8).tobytes())
    return {"triangles": int(np.asarray(m["rgb"]).reshape(-1, 3).shape[0]), "sha256": h.hexdigest(),
            "bbox_max": [float(v) for v in np.asarray(m["bbox_max"], np.float32)]}
