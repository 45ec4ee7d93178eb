"""Generates the golden vectors under tests/golden/.

Inputs are seeded synthetic BGZF files (made by this package's generator and
by Python's zlib); outputs come from the reference's own kernels --
crates/fritillaria-cuda/kernels/inflate.cu (inflate_blocks), crc32.cu,
bam_decode.cu (bam_scan_blocks, bam_reconcile, bam_emit_offsets,
bam_decode_fields), fastq_scan.cu, bcf_scan.cu and fasta_compact.cu -- compiled as host code from the reference tree by
oracle/build.py into oracle/_ref/ and driven in the reference's launch order.
So the vectors pin the oracle and the GPU path to the reference's results on
machines that have no reference tree.

Each case is one .npz holding the input bytes, the member spans, the per-member
inflate status/produced/CRC from the reference kernel, a SHA-256 of every
member's output, and per format: for BAM the record offsets, tail and the 13
per-record columns of DeviceColumns; for FASTQ (fastq_scan.cu) and BCF
(bcf_scan.cu) the offsets, tail, proof and columns of the launchers' decode;
for FASTA (fasta_compact.cu) the contig offsets, lengths and a SHA-256 of the
compacted bases.

Run from the repository root with the reference tree present:
    python tests/golden/make_golden.py
"""

from __future__ import annotations

import hashlib
import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from oracle import ref  # noqa: E402
from fritillaria_gb300 import synth  # noqa: E402

def bgzf_member(payload: bytes, level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY) -> bytes:
    """One BGZF member (SAM spec 4.1): gzip header with the BC extra subfield,
    raw DEFLATE payload, CRC32 and ISIZE."""
    co = zlib.compressobj(level, zlib.DEFLATED, -15, 9, strategy)
    cdata = co.compress(payload) + co.flush()
    bsize = 18 + len(cdata) + 8
    if bsize > 65536:
        raise ValueError("member exceeds 64 KiB")
    head = b"\x1f\x8b\x08\x04\x00\x00\x00\x00\x00\xff\x06\x00BC\x02\x00" + struct.pack("<H", bsize - 1)
    return head + cdata + struct.pack("<II", zlib.crc32(payload), len(payload))


def deflate_cases() -> bytes:
    rng = np.random.default_rng(7)
    dna = bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), 60000).tobytes())
    text = (b"the quick brown fox jumps over the lazy dog; " * 1400)[:60000]
    rnd = rng.integers(0, 256, 32000, dtype=np.uint8).tobytes()
    members = [
        bgzf_member(bytes(65536), 6),                       # distance-1 runs of 258
        bgzf_member(rng.integers(0, 256, 60000, dtype=np.uint8).tobytes(), 6),  # zlib picks stored
        bgzf_member(text[:20000], 0),                        # stored blocks
        bgzf_member(dna, 1),
        bgzf_member(dna, 9),
        bgzf_member(dna, 6, zlib.Z_FIXED),
        bgzf_member(dna, 6, zlib.Z_HUFFMAN_ONLY),
        bgzf_member(dna, 6, zlib.Z_RLE),
        bgzf_member(text, 6, zlib.Z_FILTERED),
        bgzf_member(rnd + rnd, 9),                           # distance 32000, near the window end
        bgzf_member(b"A", 6),
        bgzf_member(b"", 6),                                 # the EOF member
    ]
    return b"".join(members)


def make_case(name: str, bgzf: bytes, kind: str) -> Path:
    b = np.frombuffer(bgzf, dtype=np.uint8).copy()
    spans, used = oracle.discover(b)
    assert used == b.size, "golden inputs hold whole members only"
    data, out_off, status, produced, crc = ref.inflate(b, spans)
    assert not status.any(), f"{name}: reference kernel status {status}"
    assert np.array_equal(produced, spans["isize"]), f"{name}: produced != ISIZE"
    assert np.array_equal(crc, spans["crc32"]), f"{name}: CRC mismatch"
    sha = np.array([hashlib.sha256(data[out_off[i]:out_off[i + 1]].tobytes()).digest() for i in range(len(spans))],
                   dtype="S32")
    rec = {"bgzf": b, "span_compressed_offset": spans["compressed_offset"], "span_payload_start": spans["payload_start"],
           "span_payload_len": spans["payload_len"], "span_isize": spans["isize"], "span_crc32": spans["crc32"],
           "ref_status": status, "ref_produced": produced, "ref_crc": crc, "member_sha256": sha,
           "inflated_len": np.uint64(data.size)}
    if kind == "bam":
        start, n_ref = oracle.bam_header(data)
        offs, tail, cols = ref.bam(data, out_off, start)
        rec.update({"records_start": np.uint64(start), "n_ref": np.int32(n_ref), "record_offsets": offs,
                    "tail": np.uint64(tail)})
        rec.update({f"col_{k}": v for k, v in cols.items()})
    elif kind == "fastq":
        r = ref.fastq(data, 0)
        rec.update({"tail": np.uint64(r["tail"]), "survivors": np.uint64(r["survivors"]), "proof": np.int32(r["proof"])})
        rec.update({f"col_{k}": v for k, v in r["columns"].items()})
    elif kind == "bcf":
        start, samples, contigs = oracle.bcf_header(data)
        r = ref.bcf(data, start, samples, contigs)
        rec.update({"records_start": np.uint64(start), "samples": np.uint32(samples), "contigs": np.uint32(contigs),
                    "tail": np.uint64(r["tail"]), "proof": np.int32(r["proof"])})
        rec.update({f"col_{k}": v for k, v in r["columns"].items()})
    elif kind == "fasta":
        r = ref.fasta_compact(data)
        rec.update({"sequence_sha256": np.frombuffer(hashlib.sha256(r["sequence"].tobytes()).digest(), np.uint8),
                    "total_bases": np.uint64(r["sequence"].size)})
        rec.update({f"col_{k}": r[k] for k in ("sequence_offsets", "sequence_lengths", "record_offsets")})
    path = HERE / f"{name}.npz"
    np.savez_compressed(path, **rec)
    return path


def main():
    if ref.lib() is None:
        sys.exit("the reference kernels (oracle/_ref) are not built; they need the reference tree")
    cases = [
        ("deflate_strategies", deflate_cases(), "inflate"),
        ("bam_short_full", synth.short_read_bam(1200, n_contigs=3, genome_len=2_000_000, seed=101, levels=(1, 6),
                                                member_payload=16000)[1].tobytes(), "bam"),
        ("bam_short_record_stored", synth.short_read_bam(400, n_contigs=2, genome_len=1_000_000, seed=102,
                                                         levels=(0, 9), packing="record")[1].tobytes(), "bam"),
        ("bam_ultra_long", synth.ultra_long_bam(3, 0, seed=103, levels=(6, 6),
                                                member_payload=8000)[1].tobytes(), "bam"),
        ("fastq_illumina", synth.fastq(500, seed=104, levels=(1, 6), member_payload=20000)[1].tobytes(), "fastq"),
        ("fastq_ultra_long", synth.fastq(2, kind="ont", seed=105, member_payload=9000)[1].tobytes(), "fastq"),
        ("bcf_sites", synth.bcf(500, n_samples=16, seed=106, member_payload=12000)[1].tobytes(), "bcf"),
        ("fasta_wrapped", synth.fasta(3, 120_000, 60, True, seed=107)[1].tobytes(), "fasta"),
    ]
    for name, data, kind in cases:
        p = make_case(name, data, kind)
        print(f"{p.name}: {p.stat().st_size} bytes")


if __name__ == "__main__":
    main()
