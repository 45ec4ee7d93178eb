"""TEST INFRASTRUCTURE ONLY -- the reference's own CUDA kernels run on the GPU
in the reference's launch order (``ref_cuda_driver.cpp`` over the cubin that
``build.py`` compiles from the reference's ``inflate.cu`` and
``bam_decode.cu``).  Only the benchmark's baseline legs and the tests use it:
it times the reference's CUDA path beside this library's and checks its
results against the oracle.  It is never the product."""

from __future__ import annotations

import ctypes as C

import numpy as np

from oracle.build import REF_CUBIN, build_ref_cuda


class RefCudaResult(C.Structure):
    _fields_ = [("records", C.c_uint64), ("inflated_bytes", C.c_uint64), ("members", C.c_uint64),
                ("consumed_bytes", C.c_uint64), ("batches", C.c_uint64), ("seconds", C.c_double), ("inflate_ms", C.c_double),
                ("reconcile_ms", C.c_double), ("kernels_ms", C.c_double), ("status", C.c_int32)]


class RefCudaColumns(C.Structure):
    _fields_ = [("record_offsets", C.c_void_p), ("ref_id", C.c_void_p), ("pos", C.c_void_p), ("flags", C.c_void_p),
                ("seq_len", C.c_void_p), ("cap", C.c_uint64)]


_lib = None


def available() -> str | None:
    """None when the reference's CUDA path can run here, else why not."""
    if not REF_CUBIN.exists():
        return "the reference's kernels were not compiled (no reference tree where the build ran)"
    try:
        _load()
    except Exception as e:  # noqa: BLE001 - reported, not hidden
        return f"the reference CUDA driver did not build or load: {e}"
    return None


def _load():
    global _lib
    if _lib is None:
        path = build_ref_cuda()
        if path is None:
            raise RuntimeError("no reference cubin")
        lib = C.CDLL(str(path))
        lib.refcu_open.argtypes = [C.c_char_p, C.c_int]
        lib.refcu_run_bam.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]
        lib.refcu_last_error.restype = C.c_char_p
        if lib.refcu_open(str(REF_CUBIN).encode(), 0):
            raise RuntimeError(lib.refcu_last_error().decode())
        _lib = lib
    return _lib


def run_bam(bgzf: np.ndarray, blocks_per_batch: int = 256, columns_cap: int = 0, stop_after: int = 0):
    """The reference's reader + CudaCodec + BamDecoder loop over a whole BGZF
    BAM in host memory (with stop_after, only the batches that start before
    that compressed offset: a bounded sample).  Returns (result, columns or
    None); with columns_cap the record offsets (whole-file inflated
    coordinates), ref_id, pos, flags and seq_len come back for comparison
    with the oracle."""
    lib = _load()
    b = np.ascontiguousarray(bgzf, dtype=np.uint8)
    res = RefCudaResult()
    cols = None
    spec = None
    if columns_cap:
        cols = {"record_offsets": np.zeros(columns_cap, np.uint64), "ref_id": np.zeros(columns_cap, np.int32),
                "pos": np.zeros(columns_cap, np.int32), "flags": np.zeros(columns_cap, np.uint16),
                "seq_len": np.zeros(columns_cap, np.uint32)}
        spec = RefCudaColumns(*(cols[k].ctypes.data for k in ("record_offsets", "ref_id", "pos", "flags",
                                                               "seq_len")), columns_cap)
    rc = lib.refcu_run_bam(b.ctypes.data, b.size, blocks_per_batch, stop_after, C.byref(res),
                           C.byref(spec) if spec is not None else None)
    if rc:
        raise RuntimeError(f"reference CUDA path failed ({rc}): {lib.refcu_last_error().decode()}")
    if cols is not None:
        cols = {k: v[: res.records] for k, v in cols.items()}
    return res, cols
