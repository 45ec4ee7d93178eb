"""GB300-native BGZF -> device columns.

A Python mirror of the reference's surface for this path, over the C ABI in
``include/frt.h`` (``libfrt_gb300.so``):

  * :class:`CudaCodec` -- ``CudaCodec`` as ``BlockCodec`` / ``DeviceBlockCodec``
    (crates/fritillaria-cuda/src/lib.rs:152-293);
  * :func:`select_codec` / :class:`Backend` (crates/fritillaria/src/lib.rs:151-260);
  * :class:`DeviceBgzfReader` -- ``next_batch`` / ``carry_from``
    (crates/fritillaria-bgzf/src/device_read.rs:57-280);
  * :class:`BamDecoder` / :class:`DeviceRecordBatch` -- ``decode`` / ``tail``
    (crates/fritillaria-cuda/src/bam.rs:113-187, crates/fritillaria-bam/src/columnar/device.rs);
  * :class:`BatchEngine` -- the batched, device-resident form.

There is no CPU fallback: if the library or a GB300 is missing, constructors
raise.  Device memory, streams and events belong to the CUDA runtime the
library links; torch is only used by callers that want tensors.
"""

from __future__ import annotations

import ctypes as C
import enum
import re
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libfrt_gb300.so"
HEADER = _PKG.parent / "include" / "frt.h"

# ---------------------------------------------------------------------------
# errors (crates/fritillaria-core/src/error.rs:14-67)
# ---------------------------------------------------------------------------


class FrtError(Exception):
    code = -1

    def __init__(self, err=None, message: str | None = None):
        if err is not None:
            self.offset = err.offset
            self.expected = err.expected
            self.actual = err.actual
            self.position = err.position
            self.format = err.format.decode(errors="replace")
            self.reason = err.reason.decode(errors="replace")
        else:
            self.offset = self.expected = self.actual = self.position = 0
            self.format = ""
            self.reason = message or ""
        super().__init__(self._describe())

    def _describe(self):
        return self.reason


class IoError(FrtError):
    code = 1


class InvalidBlock(FrtError):
    code = 2

    def _describe(self):
        return f"invalid BGZF block at offset {self.offset}: {self.reason}"


class ChecksumMismatch(FrtError):
    code = 3

    def _describe(self):
        return (f"checksum mismatch in block at offset {self.offset}: expected crc32 {self.expected:#010x}, "
                f"got {self.actual:#010x}")


class SizeMismatch(FrtError):
    code = 4

    def _describe(self):
        return (f"size mismatch in block at offset {self.offset}: ISIZE says {self.expected} bytes, "
                f"inflated {self.actual}")


class InflateError(FrtError):
    code = 5

    def _describe(self):
        return f"inflate failed for block at offset {self.offset}: {self.reason}"


class Malformed(FrtError):
    code = 6

    def _describe(self):
        return f"malformed {self.format} at position {self.position}: {self.reason}"


class InvalidDeviceBatch(FrtError):
    code = 7


class CudaUnavailable(FrtError):
    code = 8


class CudaError(FrtError):
    code = 9


class InvalidArgument(FrtError):
    code = 10


_ERRORS = {c.code: c for c in (IoError, InvalidBlock, ChecksumMismatch, SizeMismatch, InflateError, Malformed,
                               InvalidDeviceBatch, CudaUnavailable, CudaError, InvalidArgument)}


class _Err(C.Structure):
    _fields_ = [("code", C.c_int32), ("offset", C.c_uint64), ("expected", C.c_uint64), ("actual", C.c_uint64),
                ("position", C.c_uint64), ("format", C.c_char * 16), ("reason", C.c_char * 200)]


class Span(C.Structure):
    """BlockSpan (crates/fritillaria-core/src/codec.rs:17-41)."""
    _fields_ = [("compressed_offset", C.c_uint64), ("payload_start", C.c_uint64), ("payload_len", C.c_uint64),
                ("isize", C.c_uint32), ("crc32", C.c_uint32)]


SPAN_DTYPE = np.dtype([("compressed_offset", "<u8"), ("payload_start", "<u8"), ("payload_len", "<u8"),
                       ("isize", "<u4"), ("crc32", "<u4")])


class EngineConfig(C.Structure):
    _fields_ = [("warps_per_cta", C.c_uint32), ("queue_chunk", C.c_uint32), ("use_graph", C.c_uint32),
                ("sort_queue", C.c_uint32)]


class InflateTuning(C.Structure):
    """A tuning of the member inflate: a compiled variant, warps per CTA (one
    member per warp), CTAs per SM (0: as many as fit), members per queue pop,
    and the one-chain variant for small launches (-1: the same variant)."""
    _fields_ = [("variant", C.c_int32), ("warps_per_cta", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("queue_chunk", C.c_int32), ("spread_variant", C.c_int32)]

    def __init__(self, variant: int = 0, warps_per_cta: int = 3, ctas_per_sm: int = 0, queue_chunk: int = 1,
                 spread_variant: int = -1):
        super().__init__(variant, warps_per_cta, ctas_per_sm, queue_chunk, spread_variant)

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class InflateVariant(C.Structure):
    _fields_ = [("lit_bits", C.c_int32), ("dist_bits", C.c_int32), ("window", C.c_int32), ("queue", C.c_int32),
                ("max_registers", C.c_int32), ("chains", C.c_int32), ("stage_half", C.c_int32),
                ("smem_per_warp", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class AutotuneResult(C.Structure):
    _fields_ = [("tuning", InflateTuning), ("ms", C.c_double), ("gbs", C.c_double), ("members", C.c_uint64),
                ("from_cache", C.c_int32), ("candidates", C.c_int32), ("key", C.c_char * 192)]

    def as_dict(self) -> dict:
        d = self.tuning.as_dict()
        d.update(variant_shape=inflate_variants()[self.tuning.variant], sample_ms=float(self.ms),
                 sample_gbs=float(self.gbs), sample_members=int(self.members), from_cache=bool(self.from_cache),
                 candidates=int(self.candidates), key=self.key.decode())
        return d


class EngineStats(C.Structure):
    _fields_ = [("members", C.c_uint64), ("compressed_bytes", C.c_uint64), ("inflated_bytes", C.c_uint64),
                ("records", C.c_uint64), ("tail", C.c_uint64), ("aux_fields", C.c_uint64),
                ("fallbacks", C.c_uint64), ("status", C.c_int32), ("error_member", C.c_uint32)]


def _raise(rc: int, err: _Err):
    if rc:
        raise _ERRORS.get(rc, FrtError)(err)


_lib = None
_P = C.c_void_p


def header_functions() -> list[str]:
    """Every function `include/frt.h` declares."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(frt_[a-z0-9_]+)\s*\(", text)
    seen = []
    for n in names:
        if n not in seen and n != "frt_read_fn":
            seen.append(n)
    return seen


def lib():
    """The native library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                           " (there is no CPU fallback)")
    L = C.CDLL(str(LIB_PATH))
    sig = {
        "frt_cuda_is_usable": (C.c_int, []),
        "frt_select_codec": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_codec_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_codec_destroy": (None, [_P]),
        "frt_codec_name": (C.c_char_p, [_P]),
        "frt_codec_device_ordinal": (C.c_int, [_P]),
        "frt_codec_stream": (_P, [_P]),
        "frt_codec_inflate_batch_device": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P, _P]),
        "frt_codec_inflate_batch_host": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P, C.c_size_t, _P, _P]),
        "frt_codec_crc32_device": (C.c_int, [_P, _P, _P, _P, C.c_size_t, _P, _P]),
        "frt_inflate_batch_len": (C.c_size_t, [_P]),
        "frt_inflate_batch_byte_len": (C.c_size_t, [_P]),
        "frt_inflate_batch_data": (_P, [_P]),
        "frt_inflate_batch_offsets": (C.POINTER(C.c_uint64), [_P]),
        "frt_inflate_batch_compressed_offsets": (C.POINTER(C.c_uint64), [_P]),
        "frt_inflate_batch_device_ordinal": (C.c_int, [_P]),
        "frt_inflate_batch_ready_event": (_P, [_P]),
        "frt_inflate_batch_to_host": (C.c_int, [_P, _P, C.c_size_t, _P]),
        "frt_inflate_batch_free": (None, [_P]),
        "frt_reader_open_memory": (C.c_int, [_P, C.c_size_t, _P, _P, _P]),
        "frt_reader_open_path": (C.c_int, [C.c_char_p, _P, _P, _P]),
        "frt_reader_set_blocks_per_batch": (None, [_P, C.c_size_t]),
        "frt_reader_next_batch": (C.c_int, [_P, _P, _P, _P, _P]),
        "frt_reader_carry_from": (C.c_int, [_P, C.c_uint64, _P]),
        "frt_reader_codec_name": (C.c_char_p, [_P]),
        "frt_reader_device_ordinal": (C.c_int, [_P]),
        "frt_reader_close": (None, [_P]),
        "frt_bgzf_discover": (C.c_int, [_P, C.c_size_t, C.c_uint64, _P, C.c_size_t, _P, _P, _P]),
        "frt_bam_parse_header": (C.c_int, [_P, C.c_size_t, _P, _P, _P]),
        "frt_bam_decoder_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_bam_decoder_set_reference_count": (None, [_P, C.c_int32]),
        "frt_bam_decoder_destroy": (None, [_P]),
        "frt_bam_decode": (C.c_int, [_P, _P, C.c_uint64, _P, _P]),
        "frt_bam_decoder_last_fallbacks": (C.c_uint64, [_P]),
        "frt_bam_scan_noalloc": (C.c_int, [_P, C.c_uint64, _P, C.c_uint32, C.c_uint64, C.c_int32, _P, C.c_uint64, _P,
                                           _P, _P, _P]),
        "frt_record_batch_len": (C.c_uint64, [_P]),
        "frt_record_batch_tail": (C.c_uint64, [_P]),
        "frt_record_batch_aux_fields": (C.c_uint64, [_P]),
        "frt_record_batch_device_ordinal": (C.c_int, [_P]),
        "frt_record_batch_column": (C.c_int, [_P, C.c_int, _P, _P, _P]),
        "frt_record_batch_column_to_host": (C.c_int, [_P, C.c_int, _P, C.c_size_t, _P]),
        "frt_record_batch_ready_event": (_P, [_P]),
        "frt_record_batch_free": (None, [_P]),
        "frt_engine_create": (C.c_int, [C.c_int, _P, _P, _P, _P]),
        "frt_engine_destroy": (None, [_P]),
        "frt_engine_bind_bam": (C.c_int, [_P, _P, C.c_size_t, _P]),
        "frt_engine_run": (C.c_int, [_P, _P]),
        "frt_engine_finish": (C.c_int, [_P, _P, _P]),
        "frt_engine_run_host": (C.c_int, [_P, _P, C.c_size_t, _P, _P]),
        "frt_engine_column": (C.c_int, [_P, C.c_int, _P, _P, _P]),
        "frt_engine_inflated": (_P, [_P, _P]),
        "frt_engine_column_to_host": (C.c_int, [_P, C.c_int, _P, C.c_size_t, _P]),
        "frt_engine_stream": (_P, [_P]),
        "frt_engine_time_stages": (C.c_int, [_P, _P, C.c_int, _P]),
        "frt_engine_launches": (C.c_uint64, [_P]),
        "frt_engine_bind_files": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P]),
        "frt_engine_file_count": (C.c_size_t, [_P]),
        "frt_engine_get_file_info": (C.c_int, [_P, C.c_size_t, _P]),
        "frt_engine_file_bam": (_P, [_P, C.c_size_t]),
        "frt_engine_file_columns": (_P, [_P, C.c_size_t]),
        "frt_record_batch_aux_lookup": (C.c_int, [_P, C.c_char_p, _P, _P]),
        "frt_record_batch_cigar_resolved": (C.c_int, [_P, _P, _P]),
        "frt_record_batch_unpack_sequences": (C.c_int, [_P, _P, _P]),
        "frt_record_batch_compact": (C.c_int, [_P, _P, _P]),
        "frt_engine_aux_lookup": (C.c_int, [_P, C.c_char_p, _P, _P]),
        "frt_engine_cigar_resolved": (C.c_int, [_P, _P, _P]),
        "frt_engine_unpack_sequences": (C.c_int, [_P, _P, _P]),
        "frt_engine_compact": (C.c_int, [_P, _P, _P]),
        "frt_engine_inflated_to_host": (C.c_int, [_P, _P, C.c_size_t, _P]),
        "frt_engine_get_tuning": (C.c_int, [_P, _P]),
        "frt_engine_set_tuning": (C.c_int, [_P, _P, _P]),
        "frt_engine_time_inflate": (C.c_int, [_P, _P, C.c_uint64, C.c_int32, _P, _P, _P]),
        "frt_autotune": (C.c_int, [_P, C.c_char_p, C.c_int32, _P, _P]),
        "frt_inflate_variant_count": (C.c_int, []),
        "frt_inflate_variant_info": (C.c_int, [C.c_int32, _P, _P]),
        "frt_inflate_get_default_tuning": (None, [_P]),
        "frt_inflate_set_default_tuning": (C.c_int, [C.c_int, _P, _P]),
        "frt_inflate_tuning_ctas_per_sm": (C.c_int, [C.c_int, _P]),
        "frt_bai_parse": (C.c_int, [_P, C.c_size_t, _P, _P]),
        "frt_bai_free": (None, [_P]),
        "frt_bai_reference_count": (C.c_int32, [_P]),
        "frt_bai_query": (C.c_int, [_P, C.c_int32, C.c_uint64, C.c_uint64, _P, C.c_size_t, _P, _P]),
        "frt_server_create": (C.c_int, [C.c_int, _P, C.c_uint64, _P, _P]),
        "frt_server_destroy": (None, [_P]),
        "frt_server_set_limits": (None, [_P, C.c_uint32, C.c_uint32]),
        "frt_server_clock_ms": (C.c_double, [_P]),
        "frt_server_get_stats": (C.c_int, [_P, _P, C.c_int32]),
        "frt_server_add_bam": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P, _P]),
        "frt_server_submit": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_uint64, C.c_uint64, C.c_double, _P, _P]),
        "frt_server_progress": (C.c_int, [_P, _P, _P]),
        "frt_server_drain": (C.c_int, [_P, _P]),
        "frt_server_request_info": (C.c_int, [_P, C.c_uint64, _P]),
        "frt_server_request_error": (C.c_int, [_P, C.c_uint64, _P]),
        "frt_server_request_column": (C.c_int, [_P, C.c_uint64, C.c_int, _P, _P, _P]),
        "frt_server_request_column_to_host": (C.c_int, [_P, C.c_uint64, C.c_int, _P, C.c_size_t, _P]),
        "frt_server_request_inflated": (_P, [_P, C.c_uint64, _P]),
        "frt_server_release": (None, [_P, C.c_uint64]),
        "frt_fastq_scanner_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_fastq_scanner_destroy": (None, [_P]),
        "frt_fastq_decode": (C.c_int, [_P, _P, C.c_uint64, _P, _P]),
        "frt_text_scanner_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_text_scanner_destroy": (None, [_P]),
        "frt_text_scan": (C.c_int, [_P, _P, C.c_uint64, C.c_int32, C.c_int32, _P, _P]),
        "frt_vcf_decoder_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_vcf_decoder_destroy": (None, [_P]),
        "frt_vcf_set_contigs": (C.c_int, [_P, _P, _P, C.c_size_t, _P]),
        "frt_vcf_set_contigs_from_header": (C.c_int, [_P, _P, C.c_size_t, _P, _P]),
        "frt_vcf_decode": (C.c_int, [_P, _P, _P, _P]),
        "frt_vcf_genotypes": (C.c_int, [_P, _P, _P, _P]),
        "frt_compressor_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_compressor_destroy": (None, [_P]),
        "frt_compressor_name": (C.c_char_p, [_P]),
        "frt_compressor_device_ordinal": (C.c_int, [_P]),
        "frt_choose_framing": (C.c_int, [C.c_size_t, C.c_size_t]),
        "frt_framed_size": (C.c_size_t, [C.c_size_t, C.c_size_t]),
        "frt_compress_bound": (C.c_size_t, [C.c_size_t]),
        "frt_compress_batch_device": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P, C.c_size_t, _P, _P, _P]),
        "frt_bgzf_writer_open": (C.c_int, [_P, _P, _P, _P, _P]),
        "frt_bgzf_writer_set_chunks_per_batch": (None, [_P, C.c_size_t]),
        "frt_bgzf_writer_set_payload_size": (None, [_P, C.c_size_t]),
        "frt_bgzf_writer_write_batch": (C.c_int, [_P, _P, C.c_size_t, _P, C.c_size_t, _P]),
        "frt_bgzf_writer_write_device": (C.c_int, [_P, _P, C.c_size_t, _P]),
        "frt_bgzf_writer_finish": (C.c_int, [_P, _P]),
        "frt_bgzf_writer_stats": (None, [_P, _P, _P, _P, _P]),
        "frt_bgzf_writer_destroy": (None, [_P]),
        "frt_bcf_parse_header": (C.c_int, [_P, C.c_size_t, _P, _P, _P, _P]),
        "frt_bcf_scanner_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_bcf_scanner_destroy": (None, [_P]),
        "frt_bcf_decode": (C.c_int, [_P, _P, C.c_uint64, C.c_uint32, C.c_uint32, _P, _P]),
        "frt_fasta_compactor_create": (C.c_int, [C.c_int, _P, _P, _P]),
        "frt_fasta_compactor_destroy": (None, [_P]),
        "frt_fasta_compact": (C.c_int, [_P, _P, _P, _P]),
        "frt_columns_len": (C.c_uint64, [_P]),
        "frt_columns_tail": (C.c_uint64, [_P]),
        "frt_columns_total_bases": (C.c_uint64, [_P]),
        "frt_columns_count": (C.c_int, [_P]),
        "frt_columns_device_ordinal": (C.c_int, [_P]),
        "frt_columns_scan_info": (None, [_P, _P, _P, _P]),
        "frt_columns_column": (C.c_int, [_P, C.c_int, _P, _P, _P]),
        "frt_columns_column_to_host": (C.c_int, [_P, C.c_int, _P, C.c_size_t, _P]),
        "frt_columns_ready_event": (_P, [_P]),
        "frt_columns_free": (None, [_P]),
    }
    for name, (res, args) in sig.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def cuda_is_usable() -> bool:
    """cuda_is_usable (crates/fritillaria/src/lib.rs:183-186)."""
    try:
        return bool(lib().frt_cuda_is_usable())
    except RuntimeError:
        return False


class Backend(enum.IntEnum):
    """Backend (crates/fritillaria/src/lib.rs:151-176)."""
    AUTO = 0
    CPU = 1
    CUDA = 2
    NVCOMP = 3


def _u8(data) -> np.ndarray:
    if isinstance(data, np.ndarray):
        return np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    return np.frombuffer(bytes(data), dtype=np.uint8)


# ---------------------------------------------------------------------------
# codec
# ---------------------------------------------------------------------------
class CudaCodec:
    """CudaCodec: inflate BGZF members on the GB300, CRC32 + ISIZE verified."""

    def __init__(self, device: int = 0, stream: int | None = None, _handle=None):
        L = lib()
        if _handle is not None:
            self._h = _handle
        else:
            h = _P()
            err = _Err()
            _raise(L.frt_codec_create(device, stream, C.byref(h), C.byref(err)), err)
            self._h = h

    @property
    def handle(self):
        return self._h

    def name(self) -> str:
        return lib().frt_codec_name(self._h).decode()

    def device_ordinal(self) -> int:
        return lib().frt_codec_device_ordinal(self._h)

    @property
    def stream(self) -> int:
        return lib().frt_codec_stream(self._h) or 0

    def inflate_batch_device(self, batch, spans) -> "DeviceInflateBatch":
        """DeviceBlockCodec::inflate_batch_device."""
        b = _u8(batch)
        s = np.ascontiguousarray(spans, dtype=SPAN_DTYPE)
        out = _P()
        err = _Err()
        _raise(lib().frt_codec_inflate_batch_device(self._h, b.ctypes.data, b.size, s.ctypes.data, len(s),
                                                    C.byref(out), C.byref(err)), err)
        return DeviceInflateBatch(out)

    def inflate_batch(self, batch, spans):
        """BlockCodec::inflate_batch: (bytes, offsets) on the host."""
        b = _u8(batch)
        s = np.ascontiguousarray(spans, dtype=SPAN_DTYPE)
        total = int(s["isize"].astype(np.uint64).sum())
        out = np.empty(total + 1, dtype=np.uint8)
        offs = np.empty(len(s) + 1, dtype=np.uint64)
        err = _Err()
        _raise(lib().frt_codec_inflate_batch_host(self._h, b.ctypes.data, b.size, s.ctypes.data, len(s),
                                                  out.ctypes.data, out.size, offs.ctypes.data, C.byref(err)), err)
        return out[:total], offs

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_codec_destroy(h)
            self._h = None


def select_codec(backend: Backend = Backend.AUTO):
    """select_codec: (codec, resolved backend).  No CPU fallback."""
    h = _P()
    resolved = C.c_int()
    err = _Err()
    _raise(lib().frt_select_codec(int(backend), C.byref(h), C.byref(resolved), C.byref(err)), err)
    return CudaCodec(_handle=h), Backend(resolved.value)


def discover_blocks(data, base_offset: int = 0):
    """BGZF member spans (host walk, discover.rs:51-109) and bytes consumed."""
    b = _u8(data)
    cap = b.size // 28 + 2
    spans = np.zeros(cap, dtype=SPAN_DTYPE)
    n = C.c_size_t()
    used = C.c_size_t()
    err = _Err()
    _raise(lib().frt_bgzf_discover(b.ctypes.data, b.size, base_offset, spans.ctypes.data, cap, C.byref(n),
                                   C.byref(used), C.byref(err)), err)
    return spans[: n.value].copy(), used.value


def parse_header(data):
    """parse_header (crates/fritillaria-bam/src/columnar/header.rs:43-101):
    (records_start, n_ref).  Raises Malformed when the bytes do not hold a
    whole header yet."""
    b = _u8(data)
    rs = C.c_uint64()
    nr = C.c_int32()
    err = _Err()
    _raise(lib().frt_bam_parse_header(b.ctypes.data, b.size, C.byref(rs), C.byref(nr), C.byref(err)), err)
    return rs.value, nr.value


class DeviceInflateBatch:
    """DeviceInflateBatch: inflated bytes on the device plus member offsets."""

    def __init__(self, handle):
        self._h = handle

    @property
    def handle(self):
        return self._h

    def __len__(self):
        return lib().frt_inflate_batch_len(self._h)

    def byte_len(self) -> int:
        return lib().frt_inflate_batch_byte_len(self._h)

    def data_ptr(self) -> int:
        return lib().frt_inflate_batch_data(self._h) or 0

    def offsets(self) -> np.ndarray:
        n = len(self) + 1
        p = lib().frt_inflate_batch_offsets(self._h)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def compressed_offsets(self) -> np.ndarray:
        n = len(self)
        if n == 0:
            return np.zeros(0, dtype=np.uint64)
        p = lib().frt_inflate_batch_compressed_offsets(self._h)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def device_ordinal(self) -> int:
        return lib().frt_inflate_batch_device_ordinal(self._h)

    def ready_event(self) -> int:
        return lib().frt_inflate_batch_ready_event(self._h) or 0

    def to_host(self) -> np.ndarray:
        out = np.empty(self.byte_len(), dtype=np.uint8)
        err = _Err()
        _raise(lib().frt_inflate_batch_to_host(self._h, out.ctypes.data, out.size, C.byref(err)), err)
        return out

    def free(self):
        if self._h and _lib is not None:
            _lib.frt_inflate_batch_free(self._h)
        self._h = None

    def __del__(self):
        self.free()


class DeviceBatch:
    """DeviceBatch {data, start} (device_read.rs:47-56)."""

    def __init__(self, data: DeviceInflateBatch, start: int):
        self.data = data
        self.start = start


class DeviceBgzfReader:
    """DeviceBgzfReader over a file path, bytes or a numpy buffer."""

    def __init__(self, source, codec: CudaCodec, blocks_per_batch: int | None = None):
        self._codec = codec  # must outlive the reader
        h = _P()
        err = _Err()
        if isinstance(source, (str, Path)):
            rc = lib().frt_reader_open_path(str(source).encode(), codec.handle, C.byref(h), C.byref(err))
            self._src = None
        else:
            self._src = _u8(source)
            rc = lib().frt_reader_open_memory(self._src.ctypes.data, self._src.size, codec.handle, C.byref(h),
                                              C.byref(err))
        _raise(rc, err)
        self._h = h
        if blocks_per_batch is not None:
            self.with_blocks_per_batch(blocks_per_batch)

    def with_blocks_per_batch(self, blocks: int) -> "DeviceBgzfReader":
        lib().frt_reader_set_blocks_per_batch(self._h, max(0, int(blocks)))
        return self

    def codec_name(self) -> str:
        return lib().frt_reader_codec_name(self._h).decode()

    def device_ordinal(self) -> int:
        return lib().frt_reader_device_ordinal(self._h)

    def next_batch(self) -> DeviceBatch | None:
        out = _P()
        start = C.c_uint64()
        has = C.c_int()
        err = _Err()
        _raise(lib().frt_reader_next_batch(self._h, C.byref(out), C.byref(start), C.byref(has), C.byref(err)), err)
        if not has.value:
            return None
        return DeviceBatch(DeviceInflateBatch(out), start.value)

    def carry_from(self, tail: int) -> None:
        err = _Err()
        _raise(lib().frt_reader_carry_from(self._h, int(tail), C.byref(err)), err)

    def __iter__(self):
        while True:
            b = self.next_batch()
            if b is None:
                return
            yield b

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_reader_close(h)
            self._h = None


# Column ids (frt_bam_column) and dtypes.
BAM_COLUMNS = {
    "ref_id": (0, np.int32), "pos": (1, np.int32), "flags": (2, np.uint16), "mapq": (3, np.uint8),
    "seq_len": (4, np.uint32), "mate_ref_id": (5, np.int32), "mate_pos": (6, np.int32), "tlen": (7, np.int32),
    "record_offsets": (8, np.uint64), "cigar_start": (9, np.uint32), "sequence_start": (10, np.uint32),
    "quality_start": (11, np.uint32), "aux_start": (12, np.uint32), "record_end": (13, np.uint32),
    "bin": (14, np.uint16), "n_cigar": (15, np.uint16), "name_len": (16, np.uint8),
    "virtual_offset": (17, np.uint64), "aux_count": (18, np.uint32), "aux_status": (19, np.uint8),
    "aux_first": (20, np.uint32),
}
AUX_DTYPE = np.dtype([("tag", "u1", (2,)), ("type", "u1"), ("subtype", "u1"), ("value_offset", "<u4"),
                      ("count", "<u4")])


class BamDecoder:
    """BamDecoder: record boundaries and columns on device."""

    def __init__(self, device: int = 0, stream: int | None = None):
        h = _P()
        err = _Err()
        _raise(lib().frt_bam_decoder_create(device, stream, C.byref(h), C.byref(err)), err)
        self._h = h

    def set_reference_count(self, n_ref: int) -> "BamDecoder":
        lib().frt_bam_decoder_set_reference_count(self._h, int(n_ref))
        return self

    def decode(self, batch: DeviceInflateBatch | None, start: int) -> "DeviceRecordBatch":
        out = _P()
        err = _Err()
        _raise(lib().frt_bam_decode(self._h, batch.handle if batch is not None else None, int(start), C.byref(out),
                                    C.byref(err)), err)
        return DeviceRecordBatch(out)

    def last_fallbacks(self) -> int:
        return lib().frt_bam_decoder_last_fallbacks(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_bam_decoder_destroy(h)
            self._h = None


NOALLOC_MAX_MEMBERS = 1024


def bam_scan_noalloc(data_ptr: int, length: int, member_offsets_ptr: int, n_members: int, start: int,
                     record_offsets_ptr: int, record_cap: int, n_ref: int = -1, stream: int | None = None):
    """Record boundaries of device-resident inflated bytes without any
    allocation by the library (frt_bam_scan_noalloc): the caller's device
    arrays hold the member offsets (n_members + 1) and receive the record
    offsets.  Returns (n_records, tail)."""
    n = C.c_uint64()
    tail = C.c_uint64()
    err = _Err()
    _raise(lib().frt_bam_scan_noalloc(data_ptr, length, member_offsets_ptr, n_members, start, n_ref,
                                      record_offsets_ptr, record_cap, C.byref(n), C.byref(tail), stream,
                                      C.byref(err)), err)
    return n.value, tail.value


# Record fields: opt-in device kernels over decoded BAM records (one aux tag for
# every record, CIGARs resolved through CG, bases unpacked, payloads compacted).
AUX_VALUE_COLUMNS = {"status": (0, np.uint8), "type": (1, np.uint8), "subtype": (2, np.uint8),
                     "count": (3, np.uint32), "value": (4, np.int64), "offset": (5, np.uint64)}
CIGAR_COLUMNS = {"offset": (0, np.uint64), "ops": (1, np.uint32), "status": (2, np.uint8)}
BASES_COLUMNS = {"offsets": (0, np.uint64), "data": (1, np.uint8)}
COMPACT_COLUMNS = {"name_offsets": (0, np.uint64), "name_data": (1, np.uint8),
                   "cigar_offsets": (2, np.uint64), "cigar_data": (3, np.uint32),
                   "sequence_offsets": (4, np.uint64), "sequence_data": (5, np.uint8),
                   "quality_offsets": (6, np.uint64), "quality_data": (7, np.uint8),
                   "aux_offsets": (8, np.uint64), "aux_data": (9, np.uint8)}


def _tag(tag) -> bytes:
    t = tag.encode() if isinstance(tag, str) else bytes(tag)
    if len(t) != 2:
        raise InvalidArgument(message=f"an aux tag is two bytes, got {t!r}")
    return t


def _fields_call(prefix: str, handle, op: str, tag=None) -> "ColumnBatch":
    cols = {"aux_lookup": AUX_VALUE_COLUMNS, "cigar_resolved": CIGAR_COLUMNS,
            "unpack_sequences": BASES_COLUMNS, "compact": COMPACT_COLUMNS}[op]
    h, err = _P(), _Err()
    fn = getattr(lib(), f"{prefix}_{op}")
    if op == "aux_lookup":
        _raise(fn(handle, _tag(tag), C.byref(h), C.byref(err)), err)
    else:
        _raise(fn(handle, C.byref(h), C.byref(err)), err)
    return ColumnBatch(h, cols)


class _RecordFields:
    """The record-field kernels, for classes whose handle names decoded records."""
    _fields_prefix = ""

    def aux_lookup(self, tag) -> "ColumnBatch":
        """One aux tag for every record (Record::aux_get): AUX_VALUE_COLUMNS."""
        return _fields_call(self._fields_prefix, self._h, "aux_lookup", tag)

    def cigar_resolved(self) -> "ColumnBatch":
        """Where each record's CIGAR ops are, following CG for the long-CIGAR placeholder."""
        return _fields_call(self._fields_prefix, self._h, "cigar_resolved")

    def unpack_sequences(self) -> "ColumnBatch":
        """The bases as ASCII, one byte each, records back to back."""
        return _fields_call(self._fields_prefix, self._h, "unpack_sequences")

    def compact(self) -> "ColumnBatch":
        """The name, CIGAR, sequence, quality and aux payloads copied out of the inflated batch."""
        return _fields_call(self._fields_prefix, self._h, "compact")


class DeviceRecordBatch(_RecordFields):
    """DeviceRecordBatch: device columns; keeps its inflate batch alive."""
    _fields_prefix = "frt_record_batch"

    def __init__(self, handle, owned: bool = True):
        self._h = handle
        self._owned = owned

    def __len__(self):
        return lib().frt_record_batch_len(self._h)

    def tail(self) -> int:
        return lib().frt_record_batch_tail(self._h)

    def aux_fields(self) -> int:
        return lib().frt_record_batch_aux_fields(self._h)

    def device_ordinal(self) -> int:
        return lib().frt_record_batch_device_ordinal(self._h)

    def column_ptr(self, name: str):
        cid = BAM_COLUMNS[name][0] if name != "aux_entries" else 21
        p = _P()
        nb = C.c_size_t()
        w = C.c_size_t()
        lib().frt_record_batch_column(self._h, cid, C.byref(p), C.byref(nb), C.byref(w))
        return p.value or 0, nb.value, w.value

    def column(self, name: str) -> np.ndarray:
        if name == "aux_entries":
            cid, dt = 21, AUX_DTYPE
        else:
            cid, dt = BAM_COLUMNS[name]
        _, nb, _ = self.column_ptr(name)
        out = np.empty(nb // np.dtype(dt).itemsize, dtype=dt)
        err = _Err()
        _raise(lib().frt_record_batch_column_to_host(self._h, cid, out.ctypes.data, out.nbytes, C.byref(err)), err)
        return out

    def to_host(self) -> dict:
        return {name: self.column(name) for name in BAM_COLUMNS}

    def free(self):
        if self._h and self._owned and _lib is not None:
            _lib.frt_record_batch_free(self._h)
        self._h = None

    def __del__(self):
        self.free()


# ---------------------------------------------------------------------------
# FASTQ, BCF, FASTA
# ---------------------------------------------------------------------------

FASTQ_COLUMNS = {"record_offsets": (0, np.uint64), "sequence_start": (1, np.uint32), "plus_start": (2, np.uint32),
                 "quality_start": (3, np.uint32), "sequence_len": (4, np.uint32), "record_end": (5, np.uint32)}
BCF_COLUMNS = {"chromosome_id": (0, np.int32), "position": (1, np.int32), "reference_span": (2, np.int32),
               "quality": (3, np.uint32), "info_count": (4, np.uint16), "allele_count": (5, np.uint16),
               "sample_count": (6, np.uint32), "format_count": (7, np.uint8), "record_offsets": (8, np.uint64),
               "alleles_start": (9, np.uint32), "filters_start": (10, np.uint32), "info_start": (11, np.uint32),
               "genotypes_start": (12, np.uint32), "record_end": (13, np.uint32)}
FASTA_COLUMNS = {"sequence": (0, np.uint8), "sequence_offsets": (1, np.uint64), "sequence_lengths": (2, np.uint64),
                 "record_offsets": (3, np.uint64)}


class Proof(enum.IntEnum):
    """How a scan's boundaries were established (speculative.rs, Proof)."""
    TILED = 0
    WALKED = 1


class SpeculativeScan:
    """SpeculativeScan: offsets, tail, survivors and the proof."""

    def __init__(self, offsets, tail, survivors, validated, proof):
        self.offsets = offsets
        self.tail = tail
        self.survivors = survivors
        self.validated = validated
        self.proof = Proof(proof)


class ColumnBatch:
    """Device columns of a FASTQ or BCF batch, or a compacted FASTA reference
    (DeviceRecordBatch / DeviceReference); keeps its inflate batch alive."""

    def __init__(self, handle, columns: dict, owned: bool = True):
        self._h = handle
        self._cols = columns
        self._owned = owned

    def __len__(self):
        return lib().frt_columns_len(self._h)

    def is_empty(self) -> bool:
        return len(self) == 0

    def tail(self) -> int:
        return lib().frt_columns_tail(self._h)

    def total_bases(self) -> int:
        return lib().frt_columns_total_bases(self._h)

    def device_ordinal(self) -> int:
        return lib().frt_columns_device_ordinal(self._h)

    def scan_info(self):
        proof, surv, val = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().frt_columns_scan_info(self._h, C.byref(proof), C.byref(surv), C.byref(val))
        return proof.value, surv.value, val.value

    def column_ptr(self, name: str):
        cid = self._cols[name][0]
        p, nb, w = _P(), C.c_size_t(), C.c_size_t()
        lib().frt_columns_column(self._h, cid, C.byref(p), C.byref(nb), C.byref(w))
        return p.value or 0, nb.value, w.value

    def column(self, name: str) -> np.ndarray:
        cid, dt = self._cols[name]
        _, nb, _ = self.column_ptr(name)
        out = np.empty(nb // np.dtype(dt).itemsize, dtype=dt)
        err = _Err()
        _raise(lib().frt_columns_column_to_host(self._h, cid, out.ctypes.data, out.nbytes, C.byref(err)), err)
        return out

    def to_host(self) -> dict:
        return {name: self.column(name) for name in self._cols}

    def free(self):
        if self._h and self._owned and _lib is not None:
            _lib.frt_columns_free(self._h)
        self._h = None

    def __del__(self):
        self.free()


class _Scanner:
    _create = _destroy = None

    def __init__(self, device: int = 0, stream: int | None = None):
        h = _P()
        err = _Err()
        _raise(getattr(lib(), self._create)(device, stream, C.byref(h), C.byref(err)), err)
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            getattr(_lib, self._destroy)(h)
            self._h = None


class FastqScanner(_Scanner):
    """FastqScanner (crates/fritillaria-cuda/src/fastq.rs:46-140)."""
    _create, _destroy = "frt_fastq_scanner_create", "frt_fastq_scanner_destroy"

    def decode(self, batch: DeviceInflateBatch | None, start: int) -> ColumnBatch:
        out = _P()
        err = _Err()
        _raise(lib().frt_fastq_decode(self._h, batch.handle if batch is not None else None, int(start), C.byref(out),
                                      C.byref(err)), err)
        return ColumnBatch(out, FASTQ_COLUMNS)

    def scan(self, batch: DeviceInflateBatch | None, start: int) -> SpeculativeScan:
        cb = self.decode(batch, start)
        proof, surv, val = cb.scan_info()
        return SpeculativeScan(cb.column("record_offsets"), cb.tail(), surv, val, proof)


TEXT_COLUMNS = {"record_offsets": (0, np.uint64), "record_ends": (1, np.uint64), "header_offsets": (2, np.uint64),
                "tabs": (3, np.uint64), "field_starts": (4, np.uint64)}


class Dialect:
    """Which leading bytes mark a header line (batch.rs:23-76): (comment, secondary or None)."""
    SAM = (ord("@"), None)
    VCF = (ord("#"), None)
    GFF = (ord("#"), None)
    BED = (ord("#"), None)


class TextScanner(_Scanner):
    """TextScanner (crates/fritillaria-cuda/src/text.rs:33-96) for SAM, VCF, BED,
    GFF and GTF: records, header lines and each record's tab offsets."""
    _create, _destroy = "frt_text_scanner_create", "frt_text_scanner_destroy"

    def scan(self, batch: DeviceInflateBatch | None, start: int, dialect=Dialect.SAM) -> ColumnBatch:
        comment, secondary = dialect
        out, err = _P(), _Err()
        _raise(lib().frt_text_scan(self._h, batch.handle if batch is not None else None, int(start), int(comment),
                                   -1 if secondary is None else int(secondary), C.byref(out), C.byref(err)), err)
        return ColumnBatch(out, TEXT_COLUMNS)


VCF_COLUMNS = {"chrom": (0, np.int32), "pos": (1, np.uint64), "bounds": (2, np.uint32), "n_alt": (3, np.uint32),
               "qual": (4, np.uint32), "flags": (5, np.uint16), "status": (6, np.uint8)}
VCF_BOUNDS = 9  # ends of CHROM, POS, ID, REF, ALT, QUAL, FILTER, INFO, and of the line


class VcfFlag(enum.IntFlag):
    """FRT_VCF_FLAG_*: missing fields ("."), FILTER PASS, QUAL parsed on the
    device, the telomere start."""
    ID_MISSING = 1
    ALT_MISSING = 2
    QUAL_MISSING = 4
    FILTER_MISSING = 8
    INFO_MISSING = 16
    SAMPLES_MISSING = 32
    FILTER_PASS = 64
    QUAL_PARSED = 128
    TELOMERE = 256


class VcfStatus(enum.IntEnum):
    OK = 0
    UNEXPECTED_EOL = 1     # fewer than eight fields (read_record's "unexpected EOL")
    INVALID_POSITION = 2   # POS is not a usize, or is 0 written other than "0"


class VcfColumns(ColumnBatch):
    """The fixed fields of a text scan's VCF records; `bounds` comes back as
    (records, VCF_BOUNDS) and `quality()` as float32 (NaN where not parsed)."""

    def column(self, name: str) -> np.ndarray:
        out = super().column(name)
        return out.reshape(-1, VCF_BOUNDS) if name == "bounds" else out

    def quality(self) -> np.ndarray:
        return self.column("qual").view(np.float32)


class VcfDecoder(_Scanner):
    """Columnar VCF on the device over the text framing -- the step the
    reference's README names after its text scan (README.md, "What's next"),
    with the vendored lazy reader's field semantics
    (crates/fritillaria-vcf/src/io/reader/record.rs:9-118,
    src/record/fields.rs:20-103).  CHROM becomes an index into the contig
    dictionary set here."""
    _create, _destroy = "frt_vcf_decoder_create", "frt_vcf_decoder_destroy"

    def set_contigs(self, names) -> None:
        bufs = [bytes(n, "ascii") if isinstance(n, str) else bytes(n) for n in names]
        arr = (C.c_char_p * max(1, len(bufs)))(*bufs)
        lens = (C.c_size_t * max(1, len(bufs)))(*[len(b) for b in bufs])
        err = _Err()
        _raise(lib().frt_vcf_set_contigs(self._h, arr, lens, len(bufs), C.byref(err)), err)

    def set_contigs_from_header(self, text) -> int:
        """The contigs of a header's "##contig=<ID=...>" lines; returns how many."""
        b = _u8(text)
        n = C.c_size_t()
        err = _Err()
        _raise(lib().frt_vcf_set_contigs_from_header(self._h, b.ctypes.data if b.size else None, b.size, C.byref(n),
                                                     C.byref(err)), err)
        return n.value

    def decode(self, text: ColumnBatch) -> VcfColumns:
        out, err = _P(), _Err()
        _raise(lib().frt_vcf_decode(self._h, text._h, C.byref(out), C.byref(err)), err)
        return VcfColumns(out, VCF_COLUMNS)

    def genotypes(self, text: ColumnBatch) -> "VcfGenotypes":
        """Every sample's GT (value/genotype/iter.rs), one call per tab."""
        out, err = _P(), _Err()
        _raise(lib().frt_vcf_genotypes(self._h, text._h, C.byref(out), C.byref(err)), err)
        return VcfGenotypes(out, VCF_GT_COLUMNS)


VCF_GT_COLUMNS = {"calls": (0, np.uint32), "key": (1, np.int32)}


class GtStatus(enum.IntEnum):
    """FRT_VCF_GT_*: bits 28-31 of a call."""
    CALLED = 0
    MISSING = 1        # the value is "."
    NONE = 2           # no value: no GT key, a shorter or empty sample, no samples
    INVALID = 3        # the reader's error
    UNREPRESENTED = 4  # valid but more than two alleles, or an index above 4093


class VcfGenotypes(ColumnBatch):
    """Every sample's GT: `calls` has one u32 per tab of the text scan, the
    call of the sample that tab opens; `unpack()` splits calls into status,
    ploidy, phasing and allele indices (-1 for ".")."""

    @staticmethod
    def unpack(calls: np.ndarray) -> dict:
        c = calls.astype(np.uint32)
        return {"status": (c >> 28).astype(np.uint8), "ploidy": ((c >> 26) & 3).astype(np.uint8),
                "phased": np.stack([(c >> 24) & 1, (c >> 25) & 1], -1).astype(np.uint8),
                "alleles": np.stack([(c & 0xFFF).astype(np.int32) - 1, ((c >> 12) & 0xFFF).astype(np.int32) - 1], -1)}

    def matrix(self, text: ColumnBatch) -> np.ndarray:
        """The calls as (records, samples), when every record has as many samples."""
        fs = text.column("field_starts").astype(np.int64)
        if len(fs) < 2:
            return np.zeros((0, 0), np.uint32)
        ns = np.diff(fs) - 8
        if (ns != ns[0]).any() or ns[0] < 0:
            raise ValueError("records have different numbers of samples")
        calls = self.column("calls")
        return calls[(fs[:-1, None] + 8 + np.arange(ns[0])[None, :])]


# ---------------------------------------------------------------------------
# the write side
# ---------------------------------------------------------------------------
MAX_COMPRESSIBLE_PAYLOAD = 65505  # crates/fritillaria-core/src/compress.rs:51-65
DEFAULT_PAYLOAD_SIZE = 0xFF00     # crates/fritillaria-bgzf/src/write.rs:19
EOF_BLOCK = bytes([0x1F, 0x8B, 8, 4, 0, 0, 0, 0, 0, 0xFF, 6, 0, 0x42, 0x43, 2, 0, 0x1B, 0, 3, 0, 0, 0, 0, 0, 0, 0, 0, 0])


class Framing(enum.IntEnum):
    """How a block's payload is encoded (compress.rs:82-98)."""
    DEFLATED = 0
    STORED = 1
    EMPTY = 2


def choose_framing(payload_len: int, deflate_len: int) -> Framing:
    """choose_framing (compress.rs:115-128)."""
    return Framing(lib().frt_choose_framing(payload_len, deflate_len))


def framed_size(payload_len: int, deflate_len: int) -> int:
    """framed_size (compress.rs:134-142)."""
    return lib().frt_framed_size(payload_len, deflate_len)


class CompressedBatch:
    """Framed BGZF blocks back to back (compress.rs:157-226): block i is
    data[offsets[i]:offsets[i + 1]]; no EOF block."""

    def __init__(self, data: np.ndarray, offsets: np.ndarray):
        self.data, self.offsets = data, offsets

    def __len__(self):
        return len(self.offsets) - 1

    def block(self, i: int) -> np.ndarray:
        return self.data[int(self.offsets[i]):int(self.offsets[i + 1])]

    def byte_len(self) -> int:
        return int(self.data.size)


class DeviceCompressor:
    """DeviceBlockCompressor (crates/fritillaria-core/src/device.rs:326-372) on
    the GB300: each range of device bytes becomes one BGZF block, inflating back
    to it exactly."""

    def __init__(self, device: int = 0, stream: int | None = None):
        h, err = _P(), _Err()
        _raise(lib().frt_compressor_create(device, stream, C.byref(h), C.byref(err)), err)
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_compressor_destroy(h)
            self._h = None

    def name(self) -> str:
        return lib().frt_compressor_name(self._h).decode()

    def device_ordinal(self) -> int:
        return lib().frt_compressor_device_ordinal(self._h)

    def compress_batch_device(self, data_ptr: int, data_len: int, bounds, out: np.ndarray | None = None
                              ) -> CompressedBatch:
        """The blocks of bounds[i]..bounds[i + 1]; into `out` (a uint8 host
        array, pinned for a fast copy back) when given, as a view of it."""
        b = np.ascontiguousarray(bounds, dtype=np.uint64)
        n = max(0, b.size - 1)
        own = out is None
        if own:
            out = np.empty(max(1, lib().frt_compress_bound(n)), np.uint8)
        offs = np.zeros(n + 1, np.uint64)
        got, err = C.c_size_t(), _Err()
        _raise(lib().frt_compress_batch_device(self._h, data_ptr, data_len, b.ctypes.data, b.size, out.ctypes.data,
                                               out.size, offs.ctypes.data, C.byref(got), C.byref(err)), err)
        return CompressedBatch(out[:got.value].copy() if own else out[:got.value], offs)


_WRITE_FN = C.CFUNCTYPE(C.c_int64, C.c_void_p, C.c_void_p, C.c_size_t)


class DeviceBgzfWriter:
    """DeviceBgzfWriter (crates/fritillaria-bgzf/src/device_write.rs): device
    bytes compressed a batch of chunks at a time into `sink` (anything with
    write(bytes)); finish() appends the EOF block."""

    def __init__(self, sink, compressor: DeviceCompressor, chunks_per_batch: int | None = None,
                 payload_size: int | None = None):
        self._sink, self._compressor = sink, compressor

        def _write(_ctx, buf, n):
            try:
                self._sink.write(C.string_at(buf, n))
                return n
            except Exception:  # the library reports the refusal as Io
                return -1

        self._cb = _WRITE_FN(_write)
        h, err = _P(), _Err()
        _raise(lib().frt_bgzf_writer_open(self._cb, None, compressor._h, C.byref(h), C.byref(err)), err)
        self._h = h
        if chunks_per_batch is not None:
            lib().frt_bgzf_writer_set_chunks_per_batch(h, chunks_per_batch)
        if payload_size is not None:
            lib().frt_bgzf_writer_set_payload_size(h, payload_size)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_bgzf_writer_destroy(h)
            self._h = None

    def write_batch(self, data_ptr: int, data_len: int, bounds) -> None:
        b = np.ascontiguousarray(bounds, dtype=np.uint64)
        err = _Err()
        _raise(lib().frt_bgzf_writer_write_batch(self._h, data_ptr, data_len, b.ctypes.data if b.size else None,
                                                 b.size, C.byref(err)), err)

    def write_device(self, data_ptr: int, data_len: int) -> None:
        err = _Err()
        _raise(lib().frt_bgzf_writer_write_device(self._h, data_ptr, data_len, C.byref(err)), err)

    def finish(self) -> None:
        err = _Err()
        _raise(lib().frt_bgzf_writer_finish(self._h, C.byref(err)), err)

    def stats(self) -> dict:
        v = [C.c_uint64() for _ in range(4)]
        lib().frt_bgzf_writer_stats(self._h, *[C.byref(x) for x in v])
        return dict(zip(("blocks", "batches", "compressed_bytes", "uncompressed_bytes"), (x.value for x in v)))


def parse_bcf_header(data):
    """BCF parse_header (header.rs:111-160): (records_start, samples, contigs).
    Raises Malformed when the bytes do not hold the whole header."""
    b = _u8(data)
    rs, ns, nc = C.c_uint64(), C.c_uint32(), C.c_uint32()
    err = _Err()
    _raise(lib().frt_bcf_parse_header(b.ctypes.data, b.size, C.byref(rs), C.byref(ns), C.byref(nc), C.byref(err)),
           err)
    return rs.value, ns.value, nc.value


class BcfScanner(_Scanner):
    """BcfScanner (crates/fritillaria-cuda/src/bcf.rs:38-150)."""
    _create, _destroy = "frt_bcf_scanner_create", "frt_bcf_scanner_destroy"

    def decode(self, batch: DeviceInflateBatch | None, start: int, samples: int, contigs: int) -> ColumnBatch:
        out = _P()
        err = _Err()
        _raise(lib().frt_bcf_decode(self._h, batch.handle if batch is not None else None, int(start), int(samples),
                                    int(contigs), C.byref(out), C.byref(err)), err)
        return ColumnBatch(out, BCF_COLUMNS)

    def scan(self, batch: DeviceInflateBatch | None, start: int, samples: int, contigs: int) -> SpeculativeScan:
        cb = self.decode(batch, start, samples, contigs)
        proof, surv, val = cb.scan_info()
        return SpeculativeScan(cb.column("record_offsets"), cb.tail(), surv, val, proof)


class FastaCompactor(_Scanner):
    """FastaCompactor (crates/fritillaria-cuda/src/fasta.rs:30-80)."""
    _create, _destroy = "frt_fasta_compactor_create", "frt_fasta_compactor_destroy"

    def compact(self, batch: DeviceInflateBatch | None) -> ColumnBatch:
        out = _P()
        err = _Err()
        _raise(lib().frt_fasta_compact(self._h, batch.handle if batch is not None else None, C.byref(out),
                                       C.byref(err)), err)
        return ColumnBatch(out, FASTA_COLUMNS)


class Format(enum.IntEnum):
    """File formats of a multi-file engine bind (frt_format)."""
    BAM = 0
    BCF = 1
    FASTQ = 2
    FASTA = 3


class EngineFile(C.Structure):
    _fields_ = [("offset", C.c_uint64), ("length", C.c_uint64), ("format", C.c_int32)]


class EngineFileInfo(C.Structure):
    _fields_ = [("format", C.c_int32), ("members", C.c_uint64), ("compressed_bytes", C.c_uint64),
                ("inflated_offset", C.c_uint64), ("inflated_bytes", C.c_uint64), ("records", C.c_uint64),
                ("tail", C.c_uint64), ("proof", C.c_uint64), ("decode_ms", C.c_double), ("launches", C.c_uint64)]


class Bai:
    """A BAI index (crates/fritillaria-bam/src/bai.rs) with the region query of
    the csi BinningIndex (binning_index/index.rs:93-119)."""

    def __init__(self, data):
        self._buf = _u8(data)
        h = _P()
        err = _Err()
        _raise(lib().frt_bai_parse(self._buf.ctypes.data, self._buf.size, C.byref(h), C.byref(err)), err)
        self._h = h

    @property
    def handle(self):
        return self._h

    def reference_count(self) -> int:
        return int(lib().frt_bai_reference_count(self._h))

    def query(self, ref: int, start: int = 0, end: int = 0):
        """Chunks (start, end virtual offsets) for [start, end], 1-based inclusive."""
        n = C.c_size_t()
        err = _Err()
        rc = lib().frt_bai_query(self._h, ref, start, end, None, 0, C.byref(n), C.byref(err))
        if rc and n.value == 0:
            _raise(rc, err)
        out = np.zeros(max(n.value, 1), dtype=[("start", "<u8"), ("end", "<u8")])
        _raise(lib().frt_bai_query(self._h, ref, start, end, out.ctypes.data, len(out), C.byref(n), C.byref(err)), err)
        return [(int(a), int(b)) for a, b in out[: n.value]]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_bai_free(h)
            self._h = None


REGION_COLUMNS = {"virtual_offset": (0, np.uint64), "record_offset": (1, np.uint64), "ref_id": (2, np.int32),
                  "pos": (3, np.int32), "flags": (4, np.uint16), "mapq": (5, np.uint8), "seq_len": (6, np.uint32)}


class RegionInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("records", C.c_uint64), ("arrival_ms", C.c_double),
                ("done_ms", C.c_double), ("inflated_bytes", C.c_uint64), ("chunks", C.c_uint32),
                ("members", C.c_uint64), ("retries", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("ticks", C.c_uint64), ("requests", C.c_uint64), ("members", C.c_uint64), ("host_ms", C.c_double),
                ("upload_ms", C.c_double), ("inflate_ms", C.c_double), ("scan_ms", C.c_double),
                ("max_inflate_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: (round(getattr(self, k), 3) if t is C.c_double else int(getattr(self, k))) for k, t in self._fields_}


class RegionServer:
    """Region queries over resident BAMs with their BAIs, batched continuously
    into one persistent inflate per tick (frt_server_*)."""

    def __init__(self, device: int = 0, budget_bytes: int = 150 << 30, stream: int | None = None):
        h = _P()
        err = _Err()
        _raise(lib().frt_server_create(device, stream, int(budget_bytes), C.byref(h), C.byref(err)), err)
        self._h = h

    def set_limits(self, max_requests_per_tick: int = 0, max_ticks_in_flight: int = 4) -> None:
        """Requests per tick (0: no limit) and ticks in flight (the server
        starts with no limit and four; each tick in flight has its own stream)."""
        lib().frt_server_set_limits(self._h, max_requests_per_tick, max_ticks_in_flight)

    def stats(self, reset: bool = False) -> dict:
        """Per-stage totals over finished ticks (frt_server_get_stats)."""
        st = ServerStats()
        lib().frt_server_get_stats(self._h, C.byref(st), int(reset))
        return st.as_dict()

    def clock_ms(self) -> float:
        return lib().frt_server_clock_ms(self._h)

    def add_bam(self, bgzf, bai) -> int:
        b, x = _u8(bgzf), _u8(bai)
        fid = C.c_int32()
        err = _Err()
        _raise(lib().frt_server_add_bam(self._h, b.ctypes.data, b.size, x.ctypes.data, x.size, C.byref(fid),
                                        C.byref(err)), err)
        return fid.value

    def submit(self, file: int, ref: int, start: int, end: int, arrival_ms: float = -1.0) -> int:
        rid = C.c_uint64()
        err = _Err()
        _raise(lib().frt_server_submit(self._h, file, ref, start, end, arrival_ms, C.byref(rid), C.byref(err)), err)
        return rid.value

    def progress(self) -> int:
        n = C.c_uint32()
        err = _Err()
        _raise(lib().frt_server_progress(self._h, C.byref(n), C.byref(err)), err)
        return n.value

    def drain(self) -> None:
        err = _Err()
        _raise(lib().frt_server_drain(self._h, C.byref(err)), err)

    def info(self, request: int) -> RegionInfo:
        out = RegionInfo()
        if lib().frt_server_request_info(self._h, request, C.byref(out)):
            raise InvalidArgument(message=f"no request {request}")
        return out

    def check(self, request: int) -> None:
        """Raises the request's error, if it failed."""
        err = _Err()
        _raise(lib().frt_server_request_error(self._h, request, C.byref(err)), err)

    def column(self, request: int, name: str) -> np.ndarray:
        cid, dt = REGION_COLUMNS[name]
        p, nb, w = _P(), C.c_size_t(), C.c_size_t()
        if lib().frt_server_request_column(self._h, request, cid, C.byref(p), C.byref(nb), C.byref(w)):
            raise InvalidArgument(message=f"request {request} has no results")
        out = np.empty(nb.value // np.dtype(dt).itemsize, dtype=dt)
        err = _Err()
        _raise(lib().frt_server_request_column_to_host(self._h, request, cid, out.ctypes.data, out.nbytes,
                                                       C.byref(err)), err)
        return out

    def release(self, request: int) -> None:
        lib().frt_server_release(self._h, request)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_server_destroy(h)
            self._h = None


def inflate_variants() -> list[dict]:
    """The compiled variants of the member inflate: table roots, window buffer
    and match queue per warp, shared memory per warp."""
    out = []
    for v in range(int(lib().frt_inflate_variant_count())):
        info = InflateVariant()
        err = _Err()
        _raise(lib().frt_inflate_variant_info(v, C.byref(info), C.byref(err)), err)
        out.append(info.as_dict())
    return out


def inflate_ctas_per_sm(tuning: InflateTuning, device: int = 0) -> int:
    """CTAs of this tuning one SM holds (0: the tuning is invalid or does not fit)."""
    return int(lib().frt_inflate_tuning_ctas_per_sm(device, C.byref(tuning)))


def default_tuning() -> InflateTuning:
    t = InflateTuning()
    lib().frt_inflate_get_default_tuning(C.byref(t))
    return t


def set_default_tuning(tuning: InflateTuning, device: int = 0) -> None:
    """The tuning codecs, engines and servers created afterwards start from."""
    err = _Err()
    _raise(lib().frt_inflate_set_default_tuning(device, C.byref(tuning), C.byref(err)), err)


class BatchEngine(_RecordFields):
    """The batched form: a whole BGZF BAM resident on the device, inflated,
    verified, scanned and decoded by persistent kernels fed from a device work
    queue, the steady state replayed as a CUDA graph.  bind_files() takes
    several BGZF files of different formats laid out back to back: one inflate
    over all their members, then each file's decoder."""
    _fields_prefix = "frt_engine"

    def __init__(self, device: int = 0, stream: int | None = None, warps_per_cta: int = 0, queue_chunk: int = 0,
                 use_graph: bool = True, sort_queue: bool = True):
        cfg = EngineConfig(warps_per_cta, queue_chunk, int(use_graph), int(sort_queue))
        h = _P()
        err = _Err()
        _raise(lib().frt_engine_create(device, stream, C.byref(cfg), C.byref(h), C.byref(err)), err)
        self._h = h

    def bind_bam(self, dev_ptr: int, length: int) -> None:
        err = _Err()
        _raise(lib().frt_engine_bind_bam(self._h, dev_ptr, length, C.byref(err)), err)

    def bind_files(self, dev_ptr: int, length: int, files) -> None:
        """files: (offset, length, Format) for each file, back to back."""
        arr = (EngineFile * len(files))(*[EngineFile(int(o), int(n), int(f)) for o, n, f in files])
        err = _Err()
        _raise(lib().frt_engine_bind_files(self._h, dev_ptr, length, arr, len(files), C.byref(err)), err)

    def file_count(self) -> int:
        return int(lib().frt_engine_file_count(self._h))

    def file_info(self, i: int) -> EngineFileInfo:
        info = EngineFileInfo()
        if lib().frt_engine_get_file_info(self._h, i, C.byref(info)):
            raise InvalidArgument(message=f"no file {i}")
        return info

    def file_result(self, i: int):
        """The last run's result for file i: a DeviceRecordBatch (BAM) or a
        ColumnBatch (BCF, FASTQ, FASTA), owned by the engine."""
        fmt = Format(self.file_info(i).format)
        if fmt == Format.BAM:
            return DeviceRecordBatch(lib().frt_engine_file_bam(self._h, i), owned=False)
        cols = {Format.BCF: BCF_COLUMNS, Format.FASTQ: FASTQ_COLUMNS, Format.FASTA: FASTA_COLUMNS}[fmt]
        return ColumnBatch(lib().frt_engine_file_columns(self._h, i), cols, owned=False)

    def run(self) -> None:
        err = _Err()
        _raise(lib().frt_engine_run(self._h, C.byref(err)), err)

    @property
    def tuning(self) -> InflateTuning:
        t = InflateTuning()
        lib().frt_engine_get_tuning(self._h, C.byref(t))
        return t

    def set_tuning(self, tuning: InflateTuning) -> None:
        err = _Err()
        _raise(lib().frt_engine_set_tuning(self._h, C.byref(tuning), C.byref(err)), err)

    def time_inflate(self, tuning: InflateTuning, members: int = 0, reps: int = 3) -> tuple[float, int]:
        """Best time (ms) of the persistent inflate alone under a tuning over the
        first `members` members (0: all), and the bytes they inflate to."""
        ms, nbytes, err = C.c_double(), C.c_uint64(), _Err()
        _raise(lib().frt_engine_time_inflate(self._h, C.byref(tuning), members, reps, C.byref(ms), C.byref(nbytes),
                                             C.byref(err)), err)
        return ms.value, nbytes.value

    def autotune(self, cache_path: str | None = None, force: bool = False) -> dict:
        """Picks the inflate tuning for this engine's workload: from the JSON
        cache, or by timing the candidates and caching the winner.  The winner
        becomes this engine's tuning and the process default."""
        res, err = AutotuneResult(), _Err()
        path = None if cache_path is None else str(cache_path).encode()
        _raise(lib().frt_autotune(self._h, path, int(force), C.byref(res), C.byref(err)), err)
        return res.as_dict()

    def finish(self) -> EngineStats:
        st = EngineStats()
        err = _Err()
        _raise(lib().frt_engine_finish(self._h, C.byref(st), C.byref(err)), err)
        return st

    def run_host(self, data) -> EngineStats:
        b = _u8(data)
        st = EngineStats()
        err = _Err()
        _raise(lib().frt_engine_run_host(self._h, b.ctypes.data, b.size, C.byref(st), C.byref(err)), err)
        return st

    def column_ptr(self, name: str):
        cid = BAM_COLUMNS[name][0] if name != "aux_entries" else 21
        p = _P()
        nb = C.c_size_t()
        w = C.c_size_t()
        lib().frt_engine_column(self._h, cid, C.byref(p), C.byref(nb), C.byref(w))
        return p.value or 0, nb.value, w.value

    def column(self, name: str) -> np.ndarray:
        if name == "aux_entries":
            cid, dt = 21, AUX_DTYPE
        else:
            cid, dt = BAM_COLUMNS[name]
        _, nb, _ = self.column_ptr(name)
        out = np.empty(nb // np.dtype(dt).itemsize, dtype=dt)
        err = _Err()
        _raise(lib().frt_engine_column_to_host(self._h, cid, out.ctypes.data, out.nbytes, C.byref(err)), err)
        return out

    def inflated_ptr(self):
        n = C.c_size_t()
        p = lib().frt_engine_inflated(self._h, C.byref(n))
        return p or 0, n.value

    def inflated(self) -> np.ndarray:
        """The last run's inflated bytes, copied to host memory."""
        _, n = self.inflated_ptr()
        out = np.empty(n, np.uint8)
        err = _Err()
        _raise(lib().frt_engine_inflated_to_host(self._h, out.ctypes.data, out.size, C.byref(err)), err)
        return out

    @property
    def stream(self) -> int:
        return lib().frt_engine_stream(self._h) or 0

    def time_stages(self, repeats: int = 3):
        """Milliseconds per stage (front, inflate, records), each the mean of
        `repeats` eager runs timed with CUDA events on the engine stream."""
        ms = (C.c_float * 3)()
        err = _Err()
        _raise(lib().frt_engine_time_stages(self._h, ms, repeats, C.byref(err)), err)
        return list(ms)

    def launches_per_run(self) -> int:
        return int(lib().frt_engine_launches(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.frt_engine_destroy(h)
            self._h = None
