"""TEST INFRASTRUCTURE ONLY.  Builds the oracle (``libfrt_oracle.so``, plain C
plus zlib) and, where the reference tree is present, the reference's own
kernels compiled as host C++ into ``oracle/_ref/`` (from the sources where they
lie; nothing is copied)."""

from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "libfrt_oracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libfrt_ref.so"
REFERENCE_KERNELS = Path("/root/reference/crates/fritillaria-cuda/kernels")


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


if __name__ == "__main__":
    print(build_oracle(), build_ref())
