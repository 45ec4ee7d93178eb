"""TEST INFRASTRUCTURE ONLY.  Python drivers for the reference's own kernels
compiled as host code (oracle/_ref/libfrt_ref.so, built by oracle/build.py
from crates/fritillaria-cuda/kernels/*.cu where the reference tree is present).
Each function returns what the reference's launcher returns for the same
input; `lib()` is None where the library could not be built."""

from __future__ import annotations

import ctypes as C

import numpy as np

from oracle import oracle

_P = C.c_void_p


def lib():
    return oracle.ref_lib()


def _need():
    L = lib()
    if L is None:
        raise RuntimeError("the reference kernels (oracle/_ref) are not built")
    return L


def inflate(bgzf: np.ndarray, spans):
    """inflate_blocks over every member (backend.rs:635-700): (bytes, member
    offsets, status, produced, crc)."""
    L = _need()
    n = len(spans)
    in_off = np.ascontiguousarray(spans["payload_start"], dtype=np.uint64)
    in_len = np.ascontiguousarray(spans["payload_len"], dtype=np.uint32)
    caps = np.ascontiguousarray(spans["isize"], dtype=np.uint32)
    out_off = np.zeros(n + 1, dtype=np.uint64)
    out_off[1:] = np.cumsum(caps.astype(np.uint64))
    out = np.zeros(int(out_off[-1]) + 1, dtype=np.uint8)
    status = np.zeros(n, np.uint32)
    produced = np.zeros(n, np.uint32)
    crc = np.zeros(n, np.uint32)
    bgzf = np.ascontiguousarray(bgzf, dtype=np.uint8)
    L.ref_inflate_blocks(bgzf.ctypes.data_as(_P), in_off.ctypes.data_as(_P), in_len.ctypes.data_as(_P),
                         out.ctypes.data_as(_P), out_off.ctypes.data_as(_P), caps.ctypes.data_as(_P),
                         status.ctypes.data_as(_P), produced.ctypes.data_as(_P), crc.ctypes.data_as(_P), n)
    return out[: int(out_off[-1])], out_off, status, produced, crc


BAM_REF_COLUMNS = [("ref_id", np.int32), ("pos", np.int32), ("flags", np.uint16), ("mapq", np.uint8),
                   ("seq_len", np.uint32), ("mate_ref_id", np.int32), ("mate_pos", np.int32), ("tlen", np.int32),
                   ("cigar_start", np.uint32), ("sequence_start", np.uint32), ("quality_start", np.uint32),
                   ("aux_start", np.uint32), ("record_end", np.uint32)]


def bam(data: np.ndarray, member_starts, start: int):
    """The four BAM phases (bam.rs:368-573): (offsets, tail, 13 columns)."""
    L = _need()
    data = np.ascontiguousarray(data, dtype=np.uint8)
    cap = data.size // 36 + 1
    offs = np.zeros(cap, np.uint64)
    cols = {name: np.zeros(cap, dt) for name, dt in BAM_REF_COLUMNS}
    n = C.c_ulonglong()
    tail = C.c_ulonglong()
    bs = np.ascontiguousarray(member_starts, dtype=np.uint64)
    args = [data.ctypes.data_as(_P), C.c_ulonglong(data.size), bs.ctypes.data_as(_P), C.c_int(len(bs) - 1),
            C.c_ulonglong(start), offs.ctypes.data_as(_P), C.c_ulonglong(cap), C.byref(n), C.byref(tail)]
    args += [cols[name].ctypes.data_as(_P) for name, _ in BAM_REF_COLUMNS]
    rc = L.ref_bam_decode(*args)
    if rc != 0:
        raise RuntimeError(f"reference scan returned {rc}")
    k = n.value
    return offs[:k].copy(), tail.value, {name: c[:k].copy() for name, c in cols.items()}


def fastq(buf, start: int) -> dict:
    """FastqScanner::run + decode (fastq.rs:486-560) around fastq_scan.cu."""
    L = _need()
    b = np.ascontiguousarray(buf, dtype=np.uint8)
    cap = b.size // 4 + 2
    offs = np.zeros(cap, np.uint64)
    cols = {name: np.zeros(cap, dt) for name, dt in oracle.FASTQ_COLUMNS}
    n, tail, surv, proof = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong(), C.c_int()
    rc = L.ref_fastq_run(b.ctypes.data_as(_P), C.c_ulonglong(b.size), C.c_ulonglong(start), offs.ctypes.data_as(_P),
                         C.c_ulonglong(cap), C.byref(n), C.byref(tail), C.byref(surv), C.byref(proof),
                         *[cols[k].ctypes.data_as(_P) for k, _ in oracle.FASTQ_COLUMNS])
    if rc != 0:
        raise RuntimeError(f"reference FASTQ scan returned {rc}")
    k = n.value
    out = {name: c[:k].copy() for name, c in cols.items()}
    out["record_offsets"] = offs[:k].copy()
    return {"columns": out, "tail": tail.value, "survivors": surv.value, "proof": proof.value}


def bcf(buf, start: int, samples: int, contigs: int) -> dict:
    """BcfScanner::scan + decode (bcf.rs:280-420) around bcf_scan.cu."""
    L = _need()
    b = np.ascontiguousarray(buf, dtype=np.uint8)
    cap = b.size // 32 + 2
    offs = np.zeros(cap, np.uint64)
    n, tail, sv, va, proof = C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong(), C.c_ulonglong(), C.c_int()
    rc = L.ref_bcf_scan(b.ctypes.data_as(_P), C.c_ulonglong(b.size), C.c_ulonglong(start), C.c_uint(samples),
                        C.c_uint(contigs), offs.ctypes.data_as(_P), C.c_ulonglong(cap), C.byref(n), C.byref(tail),
                        C.byref(sv), C.byref(va), C.byref(proof))
    if rc != 0:
        raise RuntimeError(f"reference BCF scan returned {rc}")
    k = n.value
    offs = offs[:k].copy()
    cols = {name: np.zeros(max(k, 1), dt) for name, dt in oracle.BCF_COLUMNS}
    L.ref_bcf_decode.restype = C.c_uint
    errors = L.ref_bcf_decode(b.ctypes.data_as(_P), C.c_ulonglong(b.size), offs.ctypes.data_as(_P), C.c_uint(k),
                              *[cols[name].ctypes.data_as(_P) for name, _ in oracle.BCF_COLUMNS])
    if errors:
        raise RuntimeError(f"reference BCF decode reported {errors} failures")
    out = {name: c[:k] for name, c in cols.items()}
    out["record_offsets"] = offs
    return {"columns": out, "tail": tail.value, "sieved": sv.value, "validated": va.value, "proof": proof.value}


def fasta_compact(buf) -> dict:
    """FastaCompactor::compact (fasta.rs:212-300): fasta_find_contigs, the
    per-contig layout, then fasta_compact_uniform or fasta_compact_scan per
    contig.  The layout step runs the oracle's restatement of
    RecordBatch::decode (fasta record.rs), as the launcher runs the CPU one."""
    L = _need()
    b = np.ascontiguousarray(buf, dtype=np.uint8)
    starts = np.zeros(1 << 16, np.uint64)
    L.ref_fasta_find_contigs.restype = C.c_uint
    n = L.ref_fasta_find_contigs(b.ctypes.data_as(_P), C.c_ulonglong(b.size), starts.ctypes.data_as(_P),
                                 C.c_uint(len(starts)))
    layout = oracle.fasta_compact(b)
    if not np.array_equal(starts[:n], layout["record_offsets"]):
        raise RuntimeError("the reference's contig starts disagree with the layout")
    seq = np.zeros(int(layout["sequence_lengths"].sum()) + 1, np.uint8)
    for i in range(n):
        bd = layout["bounds"][i]
        src = b[int(starts[i]) + int(bd["sequence_start"]): int(starts[i]) + int(bd["record_end"])]
        dst = seq[int(layout["sequence_offsets"][i]):]
        if bd["uniform"]:
            L.ref_fasta_compact_uniform(src.ctypes.data_as(_P), C.c_ulonglong(src.size), dst.ctypes.data_as(_P),
                                        C.c_uint(int(bd["line_width"])))
        else:
            L.ref_fasta_compact_scan(src.ctypes.data_as(_P), C.c_ulonglong(src.size), dst.ctypes.data_as(_P))
    return {"sequence": seq[:-1], "sequence_offsets": layout["sequence_offsets"],
            "sequence_lengths": layout["sequence_lengths"], "record_offsets": starts[:n].copy()}


def text_scan(buf: np.ndarray, start: int, comment: int, secondary: int | None):
    """TextScanner::scan (text.rs:233-420) over text_scan.cu: dict of record
    offsets, record ends, header offsets, tabs, field starts and the tail;
    raises when the reference reports more lines than its slots."""
    L = _need()
    buf = np.ascontiguousarray(buf, dtype=np.uint8)
    cap_lines = buf.size + 1
    cap_tabs = int(np.count_nonzero(buf == 9)) + 1
    rec_off = np.zeros(cap_lines, np.uint64)
    rec_end = np.zeros(cap_lines, np.uint64)
    hdr_off = np.zeros(cap_lines, np.uint64)
    tabs = np.zeros(cap_tabs, np.uint64)
    starts = np.zeros(cap_lines + 1, np.uint64)
    n_rec, n_hdr, n_tabs, tail = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
    rc = L.ref_text_scan(buf.ctypes.data_as(_P), C.c_uint64(buf.size), C.c_uint64(start), C.c_uint(comment),
                         C.c_uint(0xFFFFFFFF if secondary is None else secondary), rec_off.ctypes.data_as(_P),
                         rec_end.ctypes.data_as(_P), hdr_off.ctypes.data_as(_P), tabs.ctypes.data_as(_P),
                         starts.ctypes.data_as(_P), C.c_uint64(cap_lines), C.c_uint64(cap_tabs), C.byref(n_rec),
                         C.byref(n_hdr), C.byref(n_tabs), C.byref(tail))
    if rc:
        raise RuntimeError(f"reference text scan failed ({rc})")
    n = n_rec.value
    return {"record_offsets": rec_off[:n], "record_ends": rec_end[:n], "header_offsets": hdr_off[:n_hdr.value],
            "tabs": tabs[:n_tabs.value], "field_starts": starts[:n + 1] if n else starts[:0], "tail": tail.value}
