"""TEST INFRASTRUCTURE ONLY.  Builds the oracle (``libfrt_oracle.so``, plain C
plus zlib) and, where the reference tree is present, the reference's own
kernels compiled as host C++ into ``oracle/_ref/`` (from the sources where they
lie; nothing is copied)."""

from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "libfrt_oracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libfrt_ref.so"
# the reference's CUDA kernels for the GPU (device code: built here from the
# reference's sources, it travels with the tree) and the host driver that
# loads them (built wherever it runs, from this directory's source)
REF_CUBIN = REF_DIR / "ref_kernels_sm103a.cubin"
REF_CUDA_LIB = REF_DIR / "libfrt_ref_cuda.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
# The reference checkout the oracle is pinned against: FRT_REFERENCE_ROOT, by
# default the read-only tree this project was built beside.  Only test
# infrastructure reads it; where it is absent the reference-backed pins skip.
REFERENCE_ROOT = Path(os.environ.get("FRT_REFERENCE_ROOT", "/root/reference"))
REFERENCE_TESTDATA = REFERENCE_ROOT / "testdata"
REFERENCE_KERNELS = REFERENCE_ROOT / "crates" / "fritillaria-cuda" / "kernels"


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def build_oracle() -> Path:
    c_files = [HERE / "frt_oracle.c", HERE / "frt_oracle_formats.c"]
    if _newer(ORACLE_LIB, c_files + [HERE / "frt_oracle.h"]):
        _run(["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-o", str(ORACLE_LIB),
              *map(str, c_files), "-lz", "-pthread"])
    return ORACLE_LIB


def build_ref() -> Path | None:
    """The reference's kernels as host code; only where the reference exists."""
    if not REFERENCE_KERNELS.is_dir():
        return None
    REF_DIR.mkdir(exist_ok=True)
    deps = [HERE / "ref_driver.cpp", HERE / "ref_shim.h"] + [REFERENCE_KERNELS / f for f in
                                                            ("inflate.cu", "crc32.cu", "bam_decode.cu", "fastq_scan.cu", "bcf_scan.cu",
                                                             "fasta_compact.cu", "text_scan.cu")]
    if _newer(REF_LIB, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", f"-I{HERE}", f"-I{REFERENCE_KERNELS}",
              "-o", str(REF_LIB), str(HERE / "ref_driver.cpp")])
    return REF_LIB


def build_ref_cubin() -> Path | None:
    """The reference's inflate and BAM kernels as an sm_103a cubin; only where
    the reference tree is present (elsewhere a cubin built earlier is used)."""
    if not REFERENCE_KERNELS.is_dir():
        return REF_CUBIN if REF_CUBIN.exists() else None
    REF_DIR.mkdir(exist_ok=True)
    deps = [HERE / "ref_cuda_kernels.cu", REFERENCE_KERNELS / "inflate.cu", REFERENCE_KERNELS / "bam_decode.cu"]
    if _newer(REF_CUBIN, deps):
        _run([str(CUDA_HOME / "bin" / "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
              f"-I{REFERENCE_KERNELS}", "-o", str(REF_CUBIN), str(HERE / "ref_cuda_kernels.cu")])
    return REF_CUBIN


def build_ref_cuda() -> Path | None:
    """The host driver of the reference's CUDA kernels (needs the cubin)."""
    if not REF_CUBIN.exists():
        return None
    lib = build_oracle()
    src = HERE / "ref_cuda_driver.cpp"
    if _newer(REF_CUDA_LIB, [src, HERE / "frt_oracle.h", lib]):
        _run([str(CUDA_HOME / "bin" / "nvcc"), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", f"-I{HERE}",
              "-o", str(REF_CUDA_LIB), str(src), f"-L{HERE}", "-lfrt_oracle", "-lcuda", "-Xlinker",
              f"-rpath,{HERE}"])
    return REF_CUDA_LIB


if __name__ == "__main__":
    print(build_oracle(), build_ref(), build_ref_cubin(), build_ref_cuda())
