"""Build the CPU oracle (test infrastructure) into oracle/_build/libsloth_oracle.so.

gcc -O2 -ffp-contract=off -fno-fast-math: every f32 operation separately rounded, as in
Rust.  The product library never links this.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "libsloth_oracle.so"
SRC = [HERE / "sloth_oracle.c"]
HDR = [HERE / "sloth_oracle.h"]
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
          "-std=c11", "-Wall"]


def build_oracle(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    deps = SRC + HDR + [Path(__file__)]
    if force or not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in deps):
        cmd = ["gcc"] + CFLAGS + [str(s) for s in SRC] + ["-o", str(OUT), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return OUT


if __name__ == "__main__":
    print(build_oracle(force=True))
