"""Writes tests/golden/models.json: for every OBJ and STL under the reference's models/
folder, what the Python restatement of its loaders (rust-sloth_gb300/workloads.py:
read_obj, read_stl) reads -- per mesh the triangle count, a SHA-256 of the positions and
colours, and the bounding box maximum -- or the error text.  Run where the reference tree
is present:  python tests/golden/make_model_fixtures.py <reference checkout>/models
(or with SLOTH_MODELS_DIR set)."""
import os
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent), str(HERE.parents[1] / "rust-sloth_gb300")]

import workloads as W  # noqa: E402
from loader_helpers import summary  # noqa: E402


def main(models_dir: str):
    out = {}
    for p in sorted(Path(models_dir).iterdir()):
        ext = p.suffix.lower()
        if ext not in (".obj", ".stl"):
            continue
        try:
            meshes = W.read_obj(p) if ext == ".obj" else [W.read_stl(p)]
            out[p.name] = [summary(m) for m in meshes]
        except W.LoadError as e:
            out[p.name] = {"error": str(e)}
    (HERE / "models.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{len(out)} model files -> {HERE / 'models.json'}")


if __name__ == "__main__":
    d = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SLOTH_MODELS_DIR")
    if not d:
        sys.exit("usage: make_model_fixtures.py <models dir>  (or set SLOTH_MODELS_DIR)")
    main(d)
