"""Build libsloth_gpu.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Every translation unit is compiled by nvcc for `-gencode arch=compute_103a,code=sm_103a`
only, in parallel, then linked into `_build/libsloth_gpu.so` next to this file.
Device code is built with `-fmad=false` (no contraction, like Rust) and without
flush-to-zero; host code with `-ffp-contract=off` (gcc contracts by default on Arm).
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
INCLUDE = HERE.parent / "include"
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "libsloth_gpu.so"

SOURCES = ["setup.cu", "bin.cu", "raster.cu", "resolve.cu", "sloth_api.cu", "noalloc.cu", "batch.cu",
           "batch_api.cu", "diff.cu", "flush.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-ftz=false",
    "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
    "-I", str(INCLUDE), "-I", str(CSRC),
]


def _nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libsloth_gpu.so; returns its path.  Raises on failure."""
    OUT_DIR.mkdir(exist_ok=True)
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    nvcc = _nvcc()

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = obj_dir / (Path(src).stem + ".o")
        if force or _stale(o, [s] + headers + [Path(__file__)]):
            cmd = [nvcc] + NVCC_FLAGS + ["-c", str(s), "-o", str(o)]
            if verbose:
                print(" ".join(cmd))
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


HOST = HERE / "host"
HOST_SOURCES = ["loaders.cpp", "context.cpp", "main.cpp"]
CLI = OUT_DIR / "sloth"
MESHDUMP = OUT_DIR / "sloth_meshdump"
HOST_FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-I", str(INCLUDE)]


def _meshdump_job(force: bool) -> list[str] | None:
    dump_deps = [HOST / "meshdump.cpp", HOST / "loaders.cpp", HOST / "sloth_host.hpp", Path(__file__)]
    if force or _stale(MESHDUMP, dump_deps):
        # the loaders alone, no GPU library: usable where there is no CUDA device
        return ["g++"] + HOST_FLAGS + [str(HOST / "meshdump.cpp"), str(HOST / "loaders.cpp"), "-o", str(MESHDUMP)]
    return None


def build_meshdump(force: bool = False, verbose: bool = False) -> Path:
    """Compile `sloth_meshdump`, the C++ loaders without the GPU library (g++ only, a few
    seconds); returns its path."""
    OUT_DIR.mkdir(exist_ok=True)
    job = _meshdump_job(force)
    if job:
        if verbose:
            print(" ".join(job))
        r = subprocess.run(job, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"meshdump build failed:\n{r.stdout}\n{r.stderr}")
    return MESHDUMP


def build_host(force: bool = False, verbose: bool = False) -> Path:
    """Compile the C++ host side (loaders, Context mirror, the `sloth` command) against
    libsloth_gpu.so; returns the command's path."""
    lib = build_library(force=force, verbose=verbose)
    deps = [HOST / s for s in HOST_SOURCES] + [HOST / "sloth_host.hpp", INCLUDE / "sloth_gpu.h", lib, Path(__file__)]
    jobs = []
    if force or _stale(CLI, deps):
        jobs.append(["g++"] + HOST_FLAGS + [str(HOST / s) for s in HOST_SOURCES] + [
            "-o", str(CLI), "-L", str(OUT_DIR), "-lsloth_gpu", "-Wl,-rpath,$ORIGIN"])
    dump = _meshdump_job(force)
    if dump:
        jobs.append(dump)
    procs = [subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for c in jobs]
    for c, p in zip(jobs, procs):
        out, err = p.communicate()
        if verbose:
            print(" ".join(c))
        if p.returncode != 0:
            raise RuntimeError(f"host build failed:\n{out}\n{err}")
    return CLI


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
    print(build_host(verbose=True))
