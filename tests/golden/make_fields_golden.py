"""Generates the golden inputs of the record-field tests under tests/golden/.

fields_htslib.npz: the header and first 1,000 records of the reference's
testdata/htslib_multiblock.bam (a samtools-written BAM), packed into BGZF by
this package's writer, with what `samtools view` printed for those records in
the reference's testdata/reads.sam (`samtools view -h htslib_multiblock.bam`,
testdata/README.md:405): name, flag, 1-based position, mapq, CIGAR text,
sequence, quality (Phred+33) and the NM:i value.

fields_cases.npz: hand-built records for what no fixture holds, after the
reference's own unit tests (crates/fritillaria-bam/src/columnar/record.rs:560-671):
a long CIGAR of 70,000 ops in CG:B:I behind the <l_seq>S<ref_len>N placeholder,
a genuine two-op S/N record, a placeholder with no CG and one with CG:Z, the
NM/XZ aux lookup; plus every scalar type and B subtype, a repeated tag, a
malformed aux block after a valid field, odd and empty sequences.  Their
expected fields come from oracle/fields.py at test time, which
tests/test_oracle_fields.py pins to those unit tests' assertions.

text_real.npz: the reference's text fixtures written by samtools, bcftools,
NCBI and UCSC (reads.sam cut at a line end after 120 KB, calls.vcf,
cytoband.bed, lambda.gff3, lambda.gtf), for the text scanner; its expected
tables come from oracle/text.py, which tests/test_oracle_text.py pins to the
reference's text_scan.cu compiled as host code.

Run from the repository root with the reference tree present:
    python tests/golden/make_fields_golden.py
"""

from __future__ import annotations

import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from fritillaria_gb300 import synth  # noqa: E402
from oracle import oracle  # noqa: E402

from oracle.build import REFERENCE_TESTDATA as TESTDATA  # noqa: E402
BASES = b"=ACMGRSVTWYHKDBN"
OPS = b"MIDNSHP=X"
N_HTSLIB = 1000


def op(length: int, kind: str) -> int:
    return (length << 4) | OPS.index(kind.encode())


def record(name: bytes, ops: list[int], seq: bytes, qual: bytes | None = None, aux: bytes = b"", flag: int = 0,
           ref_id: int = 0, pos: int = 100, mapq: int = 60) -> bytes:
    """One BAM record (SAM specification 4.2), block_size included."""
    l_seq = len(seq)
    packed = bytearray((l_seq + 1) // 2)
    for i, ch in enumerate(seq):
        nib = BASES.index(ch)
        packed[i // 2] |= nib << 4 if i % 2 == 0 else nib
    if qual is None:
        qual = bytes(30 for _ in range(l_seq))
    body = struct.pack("<iiBBHHHIiii", ref_id, pos, len(name) + 1, mapq, 4680, len(ops), flag, l_seq, -1, -1, 0)
    body += name + b"\0" + struct.pack(f"<{len(ops)}I", *ops) + bytes(packed) + qual + aux
    return struct.pack("<I", len(body)) + body


def header(refs=(("chr1", 5_000_000),)) -> bytes:
    text = b"@HD\tVN:1.6\n" + b"".join(f"@SQ\tSN:{n}\tLN:{l}\n".encode() for n, l in refs)
    out = b"BAM\x01" + struct.pack("<i", len(text)) + text + struct.pack("<i", len(refs))
    for n, l in refs:
        out += struct.pack("<i", len(n) + 1) + n.encode() + b"\0" + struct.pack("<i", l)
    return out


def cases() -> bytes:
    rng = np.random.default_rng(41)
    acgt = lambda n: bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), n).tobytes())  # noqa: E731
    cg = b"CGBI" + struct.pack("<I", 70_000) + struct.pack("<70000I", *([op(1, "M")] * 70_000))
    every = (b"Ac" + b"A" + b"x" + b"cc" + b"c" + struct.pack("<b", -5) + b"CC" + b"C" + bytes([200])
             + b"ss" + b"s" + struct.pack("<h", -300) + b"SS" + b"S" + struct.pack("<H", 60000)
             + b"ii" + b"i" + struct.pack("<i", -70000) + b"II" + b"I" + struct.pack("<I", 3_000_000_000)
             + b"ff" + b"f" + struct.pack("<f", 1.5) + b"ZZ" + b"Z" + b"text\0" + b"HH" + b"H" + b"1AE3\0"
             + b"Bc" + b"Bc" + struct.pack("<I", 2) + struct.pack("<2b", -1, 2)
             + b"BC" + b"BC" + struct.pack("<I", 3) + bytes([1, 2, 3])
             + b"Bs" + b"Bs" + struct.pack("<I", 2) + struct.pack("<2h", -7, 8)
             + b"BS" + b"BS" + struct.pack("<I", 1) + struct.pack("<H", 65535)
             + b"Bi" + b"Bi" + struct.pack("<I", 2) + struct.pack("<2i", -1, 1 << 30)
             + b"BI" + b"BI" + struct.pack("<I", 1) + struct.pack("<I", 4_000_000_000)
             + b"Bf" + b"Bf" + struct.pack("<I", 2) + struct.pack("<2f", 0.25, -2.0)
             + b"Bz" + b"BC" + struct.pack("<I", 0))
    recs = [
        record(b"long_cigar", [op(1000, "S"), op(500, "N")], acgt(1000), aux=cg),
        record(b"genuine_sn", [op(10, "S"), op(500, "N")], acgt(1000)),
        record(b"placeholder_no_cg", [op(1000, "S"), op(500, "N")], acgt(1000)),
        record(b"placeholder_cg_z", [op(1000, "S"), op(500, "N")], acgt(1000), aux=b"CGZnot an array\0"),
        record(b"read1", [op(4, "M")], b"ACGT", aux=b"NMC" + bytes([7]) + b"XZZhello\0"),
        record(b"every_type", [op(7, "M")], b"ACGTNAC", aux=every),
        record(b"repeated_tag", [op(5, "M")], b"ACMGR", aux=b"NMC" + bytes([1]) + b"NMC" + bytes([2])),
        record(b"malformed_aux", [op(6, "M")], b"SVTWYH", aux=b"XAi" + struct.pack("<i", 5) + b"YBBC"
               + struct.pack("<I", 10) + bytes([1, 2, 3])),
        record(b"no_sequence", [], b"", aux=b"RGZgroup\0"),
        record(b"odd_length", [op(3, "M"), op(2, "I"), op(4, "M")], b"KDBN=ACGT", aux=b"ZZZz\0"),
    ]
    for k in range(200):  # ordinary records after the cases, so every case is followed by records
        n = int(rng.integers(20, 200))
        recs.append(record(f"plain{k}".encode(), [op(n, "M")], acgt(n), aux=b"NMi" + struct.pack("<i", k)))
    return header() + b"".join(recs)


def text_fixture():
    """text_real.npz: the reference's real text fixtures written by samtools,
    bcftools, NCBI and UCSC (testdata/README.md): reads.sam cut at a line end
    after 120 KB, calls.vcf, cytoband.bed, lambda.gff3, lambda.gtf whole."""
    out = {}
    for name in ("reads.sam", "calls.vcf", "cytoband.bed", "lambda.gff3", "lambda.gtf"):
        b = (TESTDATA / name).read_bytes()
        if name == "reads.sam":
            b = b[: b.index(b"\n", 120_000) + 1]
        out[name.replace(".", "_")] = np.frombuffer(b, np.uint8)
    np.savez_compressed(HERE / "text_real.npz", **out)
    print("text_real", (HERE / "text_real.npz").stat().st_size)


def main():
    text_fixture()
    raw = np.frombuffer(cases(), np.uint8)
    np.savez_compressed(HERE / "fields_cases.npz", bgzf=synth.bgzf(raw, packing="full", levels=(6, 6)))

    bam = np.fromfile(TESTDATA / "htslib_multiblock.bam", np.uint8)
    r = oracle.decode_bam_file(bam)
    infl = r["inflated"]
    offs = r["columns"]["record_offsets"]
    first = int(offs[0])
    end = int(offs[N_HTSLIB])  # the next record's start ends the subset
    sub = np.concatenate([infl[:first], infl[first:end]])
    lines = [ln for ln in (TESTDATA / "reads.sam").read_text().split("\n") if ln and not ln.startswith("@")]
    cols = [ln.split("\t") for ln in lines[:N_HTSLIB]]
    nm = [int(next(t for t in c[11:] if t.startswith("NM:i:"))[5:]) for c in cols]
    np.savez_compressed(
        HERE / "fields_htslib.npz", bgzf=synth.bgzf(sub, packing="full", levels=(6, 6)),
        name="\n".join(c[0] for c in cols).encode(), flag=np.array([int(c[1]) for c in cols], np.uint16),
        pos=np.array([int(c[3]) for c in cols], np.int64), mapq=np.array([int(c[4]) for c in cols], np.uint8),
        cigar="\n".join(c[5] for c in cols).encode(), seq="\n".join(c[9] for c in cols).encode(),
        qual="\n".join(c[10] for c in cols).encode(), nm=np.array(nm, np.int64))
    print("fields_cases", (HERE / "fields_cases.npz").stat().st_size, "fields_htslib",
          (HERE / "fields_htslib.npz").stat().st_size)


if __name__ == "__main__":
    main()
