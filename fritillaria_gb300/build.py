"""Builds the native parts in-tree: the CUDA library for sm_103a, the synthetic
data generator and (when asked) the oracle.  Objects go to ``_build/``; the
shared libraries sit beside the code that loads them.  A target is rebuilt only
when one of its sources or headers is newer than it."""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                     f"-I{INCLUDE}", "-diag-suppress", "550"]

CUDA_SOURCES = ["inflate.cu", "bam.cu", "runtime.cu", "decoder.cu", "engine.cu", "formats.cu", "noalloc.cu", "bai.cpp", "tune.cpp", "fields.cu",
                "serve.cu", "deflate.cu"]
LIB = PKG / "libfrt_gb300.so"
SYNTH_LIB = PKG / "libfrt_synth.so"


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [INCLUDE / "frt.h"]


def build_cuda(jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = [CSRC / s for s in CUDA_SOURCES if (CSRC / s).exists()]
    headers = _headers()
    objs = []
    steps = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            steps.append([NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, steps))
    if _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *map(str, objs),
              "-Xlinker", f"-rpath,{CUDA_HOME / 'lib64'}"])
    return LIB


def build_synth() -> Path:
    src = CSRC / "synth.cpp"
    if _newer(SYNTH_LIB, [src]):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-o", str(SYNTH_LIB), str(src), "-lz", "-pthread"])
    return SYNTH_LIB


def build_all() -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_cuda)
        f2 = ex.submit(build_synth)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all()
    print("built", LIB, SYNTH_LIB, file=sys.stderr)
