"""Build of the compositor's shared library (libhdsr.so) for sm_103a.

Each CUDA translation unit under csrc/ is compiled by nvcc in parallel and
linked into one shared library next to this file. Every unit is compiled with
-fmad=false: the kernels spell out each fused multiply-add (fmaf) they use, so
that the frame's arithmetic is a fixed sequence of IEEE operations.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
LIB_NAME = "libhdsr.so"
SOURCES = ["hdsr_api.cu", "hdsr_project.cu", "hdsr_scan.cu", "hdsr_sort.cu", "hdsr_dsort.cu", "hdsr_raster.cu",
           "hdsr_static.cu", "hdsr_backward.cu", "hdsr_backward_prep.cu", "hdsr_serve.cu",
           "hdsr_post.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhdsr.so")


def library_path() -> Path:
    return PKG_DIR / LIB_NAME


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile csrc/*.cu into libhdsr.so (incremental unless force)."""
    build_dir = PKG_DIR / "_build"
    build_dir.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [PKG_DIR.parent / "include" / "hdsr.h"]
    sources = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    exe = nvcc()
    extra = os.environ.get("HDSR_NVCC_FLAGS", "").split()  # tuning overrides (-D...)

    def compile_one(src: Path) -> Path:
        obj = build_dir / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [exe, *ARCH, *FLAGS, *extra, "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stderr}")
            if verbose and res.stderr:
                print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(sources)) as pool:
        objs = list(pool.map(compile_one, sources))
    lib = library_path()
    if force or _stale(lib, objs):
        cmd = [exe, *ARCH, "-shared", "-o", str(lib), *map(str, objs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
