"""TEST INFRASTRUCTURE ONLY -- ctypes access to the oracle (``frt_oracle.c``)
and to the reference's own kernels compiled as host code (``_ref/``).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It is the oracle the tests compare against, never the product."""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


class OrcError(C.Structure):
    _fields_ = [("code", C.c_int32), ("offset", C.c_uint64), ("expected", C.c_uint64), ("actual", C.c_uint64),
                ("position", C.c_uint64), ("reason", C.c_char * 128)]


class OrcSpan(C.Structure):
    _fields_ = [("compressed_offset", C.c_uint64), ("payload_start", C.c_uint64), ("payload_len", C.c_uint64),
                ("isize", C.c_uint32), ("crc32", C.c_uint32)]


class OrcFileDecode(C.Structure):
    _fields_ = [("members", C.c_uint64), ("inflated_bytes", C.c_uint64), ("records", C.c_uint64),
                ("aux_entries", C.c_uint64), ("tail", C.c_uint64), ("records_start", C.c_uint64),
                ("n_ref", C.c_int32), ("status", C.c_int32)]


class OrcBaseline(C.Structure):
    _fields_ = [("members", C.c_uint64), ("inflated_bytes", C.c_uint64), ("records", C.c_uint64),
                ("aux_tags", C.c_uint64), ("checksum", C.c_uint64), ("seconds", C.c_double), ("status", C.c_int32)]


_P = C.c_void_p
_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        from oracle.build import build_oracle
        path = build_oracle()
        _lib = C.CDLL(str(path))
        _lib.orc_crc32.restype = C.c_uint32
        _lib.orc_crc32.argtypes = [C.c_uint32, _P, C.c_size_t]
        _lib.orc_crc32_combine.restype = C.c_uint32
        _lib.orc_crc32_combine.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64]
        _lib.orc_bgzf_discover.argtypes = [_P, C.c_size_t, C.c_uint64, _P, C.c_size_t, _P, _P, _P]
        _lib.orc_inflate_batch.argtypes = [_P, C.c_size_t, _P, C.c_size_t, _P, C.c_size_t, _P, _P]
        _lib.orc_bam_header.argtypes = [_P, C.c_size_t, _P, _P, _P]
        _lib.orc_bam_scan.argtypes = [_P, C.c_size_t, C.c_uint64, _P, C.c_size_t, _P, _P, _P]
        _lib.orc_bam_scan_blocked.argtypes = [_P, C.c_size_t, _P, C.c_size_t, C.c_uint64, _P, C.c_size_t, _P, _P,
                                              _P, _P]
        _lib.orc_bam_decode.argtypes = [_P, _P, C.c_size_t, _P]
        _lib.orc_bam_aux.argtypes = [_P, C.c_uint32, C.c_uint32, _P, C.c_uint32, _P]
        _lib.orc_baseline_bam.argtypes = [_P, C.c_size_t, C.c_int, C.c_uint64, _P]
        _lib.orc_baseline_file.argtypes = [_P, C.c_size_t, C.c_int, C.c_int, _P]
        _lib.orc_inflate_file.argtypes = [_P, C.c_size_t, C.c_int, _P, C.c_uint64, _P, _P]
        _lib.orc_bam_file_decode.argtypes = [_P, C.c_size_t, C.c_int, _P, C.c_uint64, _P, _P, _P, _P, _P, C.c_uint64,
                                             C.c_uint64, _P]
        _lib.orc_region_records.restype = C.c_uint64
        _lib.orc_region_records.argtypes = [_P, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int32, C.c_uint64, C.c_uint64,
                                            _P, C.c_uint64]
        _lib.orc_fastq_scan.argtypes = [_P, C.c_uint64, C.c_uint64, _P, C.c_size_t, _P, _P, _P, _P]
        _lib.orc_fastq_decode.argtypes = [_P, C.c_uint64, _P, C.c_size_t, _P, _P, _P, _P, _P]
        _lib.orc_bcf_header.argtypes = [_P, C.c_uint64, _P, _P, _P, _P]
        _lib.orc_bcf_scan.argtypes = [_P, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _P, C.c_size_t, _P, _P,
                                      _P, _P, _P]
        _lib.orc_bcf_decode.argtypes = [_P, C.c_uint64, _P, C.c_size_t, _P]
        _lib.orc_fasta_compact.argtypes = [_P, C.c_uint64, _P, C.c_uint64, _P, _P, _P, _P, C.c_size_t, _P, _P]
    return _lib


def ref_lib():
    """The reference's kernels as host code, or None where not built."""
    global _ref
    if _ref is None:
        p = HERE / "_ref" / "libfrt_ref.so"
        if not p.exists():
            try:
                from oracle.build import build_ref
                build_ref()
            except Exception:
                return None
        if not p.exists():
            return None
        _ref = C.CDLL(str(p))
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _buf(data) -> np.ndarray:
    if isinstance(data, np.ndarray):
        return np.ascontiguousarray(data, dtype=np.uint8)
    return np.frombuffer(bytes(data), dtype=np.uint8)


class OracleError(Exception):
    def __init__(self, err: OrcError):
        self.code = err.code
        self.offset = err.offset
        self.expected = err.expected
        self.actual = err.actual
        self.position = err.position
        self.reason = err.reason.decode(errors="replace")
        super().__init__(f"code {self.code} offset {self.offset} position {self.position}: {self.reason}")


def crc32(data, crc: int = 0) -> int:
    b = _buf(data)
    return lib().orc_crc32(crc, _ptr(b), b.size)


def crc32_combine(a: int, b: int, len_b: int) -> int:
    return lib().orc_crc32_combine(a, b, len_b)


SPAN_DTYPE = np.dtype([("compressed_offset", "<u8"), ("payload_start", "<u8"), ("payload_len", "<u8"),
                       ("isize", "<u4"), ("crc32", "<u4")])


def discover(data, base_offset: int = 0):
    """BGZF member spans and the consumed length (discover.rs:51-109)."""
    b = _buf(data)
    cap = b.size // 28 + 2
    spans = np.zeros(cap, dtype=SPAN_DTYPE)
    n = C.c_size_t()
    used = C.c_size_t()
    err = OrcError()
    rc = lib().orc_bgzf_discover(_ptr(b), b.size, base_offset, _ptr(spans), cap, C.byref(n), C.byref(used),
                                 C.byref(err))
    if rc:
        raise OracleError(err)
    return spans[: n.value].copy(), used.value


def inflate_batch(data, spans):
    """(inflated bytes, n+1 offsets); raises OracleError like CpuCodec."""
    b = _buf(data)
    spans = np.ascontiguousarray(spans, dtype=SPAN_DTYPE)
    total = int(spans["isize"].astype(np.uint64).sum())
    out = np.zeros(total + 1, dtype=np.uint8)
    offs = np.zeros(len(spans) + 1, dtype=np.uint64)
    err = OrcError()
    rc = lib().orc_inflate_batch(_ptr(b), b.size, _ptr(spans), len(spans), _ptr(out), out.size, _ptr(offs),
                                 C.byref(err))
    if rc:
        raise OracleError(err)
    return out[:total], offs


def bam_header(buf):
    b = _buf(buf)
    rs = C.c_uint64()
    nr = C.c_int32()
    err = OrcError()
    rc = lib().orc_bam_header(_ptr(b), b.size, C.byref(rs), C.byref(nr), C.byref(err))
    if rc:
        raise OracleError(err)
    return rs.value, nr.value


def bam_scan(buf, start: int):
    """scan_records (record.rs:58-95): (offsets, tail)."""
    b = _buf(buf)
    cap = b.size // 36 + 1
    offs = np.zeros(cap, dtype=np.uint64)
    n = C.c_size_t()
    tail = C.c_uint64()
    err = OrcError()
    rc = lib().orc_bam_scan(_ptr(b), b.size, start, _ptr(offs), cap, C.byref(n), C.byref(tail), C.byref(err))
    if rc:
        raise OracleError(err)
    return offs[: n.value].copy(), tail.value


def bam_scan_blocked(buf, block_starts, start: int):
    """scan_records_blocked (blocked.rs:193-282): (offsets, tail, fallbacks)."""
    b = _buf(buf)
    bs = np.ascontiguousarray(block_starts, dtype=np.uint64)
    cap = b.size // 36 + 1
    offs = np.zeros(cap, dtype=np.uint64)
    n = C.c_size_t()
    tail = C.c_uint64()
    fb = C.c_size_t()
    err = OrcError()
    rc = lib().orc_bam_scan_blocked(_ptr(b), b.size, _ptr(bs), len(bs) - 1, start, _ptr(offs), cap, C.byref(n),
                                    C.byref(tail), C.byref(fb), C.byref(err))
    if rc:
        raise OracleError(err)
    return offs[: n.value].copy(), tail.value, fb.value


BAM_COLUMNS = [("ref_id", np.int32), ("pos", np.int32), ("flags", np.uint16), ("mapq", np.uint8),
               ("seq_len", np.uint32), ("mate_ref_id", np.int32), ("mate_pos", np.int32), ("tlen", np.int32),
               ("cigar_start", np.uint32), ("sequence_start", np.uint32), ("quality_start", np.uint32),
               ("aux_start", np.uint32), ("record_end", np.uint32), ("bin", np.uint16), ("n_cigar", np.uint16),
               ("name_len", np.uint8), ("aux_count", np.uint32), ("aux_status", np.uint8)]


def bam_decode(buf, offsets) -> dict:
    """RecordBatch::decode columns plus field bounds and aux counts."""
    b = _buf(buf)
    offs = np.ascontiguousarray(offsets, dtype=np.uint64)
    n = len(offs)
    cols = {name: np.zeros(n, dtype=dt) for name, dt in BAM_COLUMNS}
    ptrs = [_ptr(cols[name]) for name, _ in BAM_COLUMNS]
    struct = (C.c_void_p * len(ptrs))(*ptrs)
    lib().orc_bam_decode(_ptr(b), _ptr(offs), n, C.byref(struct))
    cols["record_offsets"] = offs.copy()
    return cols


AUX_DTYPE = np.dtype([("tag", "u1", (2,)), ("type", "u1"), ("subtype", "u1"), ("value_offset", "<u4"),
                      ("count", "<u4")])


def bam_aux(buf, record_offset: int, aux_start: int, record_end: int):
    """Aux fields of one record (aux.rs:301-479): (entries, status)."""
    b = _buf(buf)
    rec = b[record_offset:]
    cap = max(1, (record_end - aux_start) // 4 + 1)
    out = np.zeros(cap, dtype=AUX_DTYPE)
    n = C.c_uint32()
    st = lib().orc_bam_aux(_ptr(rec), aux_start, record_end, _ptr(out), cap, C.byref(n))
    return out[: n.value].copy(), st


def decode_bam_file(bgzf) -> dict:
    """Whole-file oracle: discover, inflate (verified), header, serial scan and
    columns.  Returns a dict with the inflated bytes, spans and columns."""
    spans, used = discover(bgzf)
    data, offs = inflate_batch(bgzf, spans)
    start, n_ref = bam_header(data)
    rec, tail = bam_scan(data, start)
    cols = bam_decode(data, rec)
    return {"spans": spans, "inflated": data, "offsets": offs, "records_start": start, "n_ref": n_ref,
            "tail": tail, "columns": cols, "consumed": used}


def virtual_offsets(spans, member_offsets, record_offsets):
    """Member compressed offset << 16 | in-member offset (virtual_offset.rs:24-70)."""
    mo = np.asarray(member_offsets, dtype=np.uint64)
    ro = np.asarray(record_offsets, dtype=np.uint64)
    m = np.searchsorted(mo, ro, side="right") - 1
    co = np.asarray(spans["compressed_offset"], dtype=np.uint64)[m]
    return (co << np.uint64(16)) | (ro - mo[m])


def baseline_file(bgzf, fmt: int, threads: int):
    """CPU baseline for a bgzipped BCF (1), FASTQ (2) or FASTA (3) file."""
    b = _buf(bgzf)
    res = OrcBaseline()
    lib().orc_baseline_file(_ptr(b), b.size, fmt, threads, C.byref(res))
    return res


def baseline_bam(bgzf, threads: int, max_members: int = 0):
    b = _buf(bgzf)
    res = OrcBaseline()
    lib().orc_baseline_bam(_ptr(b), b.size, threads, max_members, C.byref(res))
    return res


def inflate_file(bgzf, threads: int, total: int | None = None) -> np.ndarray:
    """Every member inflated and CRC/ISIZE-checked on `threads` host threads;
    `total` (the inflated size, when known) saves a discovery pass."""
    b = _buf(bgzf)
    members, got = C.c_uint64(), C.c_uint64()
    if total is None:
        lib().orc_inflate_file(_ptr(b), b.size, threads, None, 0, C.byref(members), C.byref(got))
        total = got.value
    out = np.empty(max(int(total), 1), np.uint8)
    rc = lib().orc_inflate_file(_ptr(b), b.size, threads, _ptr(out), out.size, C.byref(members), C.byref(got))
    if rc:
        raise RuntimeError(f"oracle inflate failed: code {rc}")
    return out[: got.value]


def decode_bam_file_mt(bgzf, threads: int, records: int, aux_entries: int, inflated_bytes: int) -> dict:
    """The whole BAM file decoded by the oracle on `threads` inflate threads:
    inflated bytes, the serial scan, every column, virtual offsets and the aux
    directory.  The capacities come from the run being checked; a file that
    needs more raises with the sizes the oracle found."""
    b = _buf(bgzf)
    inflated = np.empty(max(int(inflated_bytes), 1), np.uint8)
    rec_cap = int(records) + 1
    cols = {name: np.zeros(rec_cap, dtype=dt) for name, dt in BAM_COLUMNS}
    ptrs = [_ptr(cols[name]) for name, _ in BAM_COLUMNS]
    struct = (C.c_void_p * len(ptrs))(*ptrs)
    offs = np.zeros(rec_cap, np.uint64)
    vo = np.zeros(rec_cap, np.uint64)
    first = np.zeros(rec_cap + 1, np.uint32)
    aux = np.zeros(max(int(aux_entries), 1), dtype=AUX_DTYPE)
    res = OrcFileDecode()
    rc = lib().orc_bam_file_decode(_ptr(b), b.size, threads, _ptr(inflated), inflated.size, _ptr(offs), _ptr(vo),
                                   C.byref(struct), _ptr(first), _ptr(aux), rec_cap, aux.size, C.byref(res))
    if rc:
        raise RuntimeError(f"oracle decode failed: code {rc}; records {res.records}, aux entries {res.aux_entries}, "
                           f"inflated bytes {res.inflated_bytes}")
    n = int(res.records)
    out = {name: cols[name][:n] for name, _ in BAM_COLUMNS}
    out["record_offsets"] = offs[:n]
    out["virtual_offset"] = vo[:n]
    out["aux_first"] = first[: n + 1]
    return {"inflated": inflated[: res.inflated_bytes], "columns": out, "aux_entries": aux[: res.aux_entries],
            "tail": int(res.tail), "records_start": int(res.records_start), "members": int(res.members)}


# ---- FASTQ, BCF, FASTA (frt_oracle_formats.c) ------------------------------

TILED, WALKED = 0, 1

FASTQ_COLUMNS = [("sequence_start", np.uint32), ("plus_start", np.uint32), ("quality_start", np.uint32),
                 ("sequence_len", np.uint32), ("record_end", np.uint32)]


def fastq_scan(buf, start: int = 0, cap: int | None = None):
    """FastqScanner::scan semantics: (offsets, tail, survivors, proof).
    `cap` bounds the offsets list (default: one per four bytes)."""
    b = _buf(buf)
    cap = b.size // 4 + 1 if cap is None else int(cap)
    offs = np.zeros(cap, dtype=np.uint64)
    n, tail, surv, proof = C.c_size_t(), C.c_uint64(), C.c_uint64(), C.c_int()
    rc = lib().orc_fastq_scan(_ptr(b), b.size, start, _ptr(offs), cap, C.byref(n), C.byref(tail), C.byref(surv),
                              C.byref(proof))
    if rc:
        raise RuntimeError(f"orc_fastq_scan: {rc}")
    return offs[: n.value].copy(), tail.value, surv.value, proof.value


def fastq_decode(buf, start: int = 0, cap: int | None = None) -> dict:
    """Offsets, tail and the five line-bound columns of FastqScanner::decode."""
    b = _buf(buf)
    offs, tail, surv, proof = fastq_scan(b, start, cap)
    cols = {name: np.zeros(len(offs), dtype=dt) for name, dt in FASTQ_COLUMNS}
    errors = lib().orc_fastq_decode(_ptr(b), b.size, _ptr(offs), len(offs),
                                    *[_ptr(cols[name]) for name, _ in FASTQ_COLUMNS])
    if errors:
        raise RuntimeError(f"{errors} FASTQ records failed to decode")
    cols["record_offsets"] = offs
    return {"columns": cols, "tail": tail, "survivors": surv, "proof": proof}


BCF_COLUMNS = [("chromosome_id", np.int32), ("position", np.int32), ("reference_span", np.int32),
               ("quality", np.uint32), ("info_count", np.uint16), ("allele_count", np.uint16),
               ("sample_count", np.uint32), ("format_count", np.uint8), ("alleles_start", np.uint32),
               ("filters_start", np.uint32), ("info_start", np.uint32), ("genotypes_start", np.uint32),
               ("record_end", np.uint32)]


def bcf_header(buf):
    """(records_start, samples, contigs) of a BCF header (header.rs:111-160)."""
    b = _buf(buf)
    rs, ns, nc = C.c_uint64(), C.c_uint32(), C.c_uint32()
    err = OrcError()
    rc = lib().orc_bcf_header(_ptr(b), b.size, C.byref(rs), C.byref(ns), C.byref(nc), C.byref(err))
    if rc:
        raise OracleError(err)
    return rs.value, ns.value, nc.value


def bcf_scan(buf, start: int, samples: int, contigs: int):
    """BcfScanner::scan semantics: (offsets, tail, sieved, validated, proof)."""
    b = _buf(buf)
    cap = b.size // 32 + 1
    offs = np.zeros(cap, dtype=np.uint64)
    n, tail, sv, va, proof = C.c_size_t(), C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_int()
    rc = lib().orc_bcf_scan(_ptr(b), b.size, start, samples, contigs, _ptr(offs), cap, C.byref(n), C.byref(tail),
                            C.byref(sv), C.byref(va), C.byref(proof))
    if rc:
        raise RuntimeError(f"orc_bcf_scan: {rc}")
    return offs[: n.value].copy(), tail.value, sv.value, va.value, proof.value


def bcf_decode(buf, start: int, samples: int, contigs: int) -> dict:
    """Offsets, tail and the site-core columns of BcfScanner::decode."""
    b = _buf(buf)
    offs, tail, sv, va, proof = bcf_scan(b, start, samples, contigs)
    cols = {name: np.zeros(len(offs), dtype=dt) for name, dt in BCF_COLUMNS}
    ptrs = (C.c_void_p * len(BCF_COLUMNS))(*[_ptr(cols[name]) for name, _ in BCF_COLUMNS])
    errors = lib().orc_bcf_decode(_ptr(b), b.size, _ptr(offs), len(offs), C.byref(ptrs))
    if errors:
        raise RuntimeError(f"{errors} BCF records failed to decode")
    cols["record_offsets"] = offs
    return {"columns": cols, "tail": tail, "sieved": sv, "validated": va, "proof": proof}


FASTA_BOUNDS_DTYPE = np.dtype([("sequence_start", "<u4"), ("line_bases", "<u4"), ("line_width", "<u4"),
                               ("uniform", "u1"), ("sequence_len", "<u8"), ("record_end", "<u8")], align=True)


def fasta_compact(buf, cap: int | None = None) -> dict:
    """FastaCompactor::compact semantics: the bases of every contig without
    newlines, plus per-contig offsets, lengths, record offsets and layout.
    `cap` bounds the contig count (default: one per two bytes)."""
    b = _buf(buf)
    cap = b.size // 2 + 1 if cap is None else int(cap)
    so, sl, ro = (np.zeros(cap, dtype=np.uint64) for _ in range(3))
    bounds = np.zeros(cap, dtype=FASTA_BOUNDS_DTYPE)
    n, total = C.c_size_t(), C.c_uint64()
    rc = lib().orc_fasta_compact(_ptr(b), b.size, None, 0, _ptr(so), _ptr(sl), _ptr(ro), _ptr(bounds), cap,
                                 C.byref(n), C.byref(total))
    if rc:
        raise RuntimeError(f"orc_fasta_compact: {rc}")
    seq = np.zeros(total.value + 1, dtype=np.uint8)
    rc = lib().orc_fasta_compact(_ptr(b), b.size, _ptr(seq), seq.size, _ptr(so), _ptr(sl), _ptr(ro), _ptr(bounds),
                                 cap, C.byref(n), C.byref(total))
    if rc:
        raise RuntimeError(f"orc_fasta_compact: {rc}")
    k = n.value
    return {"sequence": seq[: total.value], "sequence_offsets": so[:k].copy(), "sequence_lengths": sl[:k].copy(),
            "record_offsets": ro[:k].copy(), "bounds": bounds[:k].copy()}


def region_query(bgzf, spans, index, ref: int, start: int, end: int):
    """The reference's indexed region query on the host: the BAI's chunks,
    each chunk's members inflated with zlib (plus the members a record
    starting in the chunk runs into), the chunk's records scanned and
    filtered.  Returns (kept record count, inflated bytes)."""
    from oracle import bai as obai

    coff = spans["compressed_offset"].astype(np.uint64)
    kept, inflated = 0, 0
    for c0, c1 in obai.query(index, ref, start, end or obai.MAX_POSITION):
        ma = int(np.searchsorted(coff, np.uint64(c0 >> 16), "right")) - 1
        me = int(np.searchsorted(coff, np.uint64(c1 >> 16), "right")) - 1
        mz = min(len(spans) - 1, me + 1)
        data, offs = inflate_batch(bgzf, spans[ma: mz + 1])
        inflated += data.size
        s0 = int(c0 & 0xFFFF)
        e0 = int(offs[me - ma]) + int(c1 & 0xFFFF)
        out = np.zeros(1, np.uint64)
        kept += lib().orc_region_records(_ptr(data), data.size, s0, e0, ref, start, end or obai.MAX_POSITION,
                                         _ptr(out), 0)
    return kept, inflated
