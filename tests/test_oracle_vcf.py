"""The columnar-VCF oracle (oracle/vcf.py) pinned to the vendored reader's
own tests and to the reference's real-file test, on the CPU:
  * crates/fritillaria-vcf/src/io/reader/record.rs:124-147 (test_read_record):
    ".\\t1\\t.\\tN\\t.\\t.\\t.\\t." with LF and with CRLF reads as
    Bounds::default() (src/record/fields/bounds.rs:54-67) over ".1.N....";
  * crates/fritillaria-text/tests/real_files.rs:78-107: every CHROM and POS of
    testdata/calls.vcf (bcftools) equals the vendored reader's, and :241-286:
    10 fields a record, 235 header lines;
  * f32::from_str's result is the nearest binary32 (ties to even), checked
    against numpy's binary32 conversion and at exact ties."""

from fractions import Fraction
from pathlib import Path
import random

import numpy as np
import pytest

from oracle import text, vcf

GOLDEN = Path(__file__).resolve().parent / "golden"


def decode(raw: bytes, contigs=()):
    buf = np.frombuffer(raw, np.uint8)
    scan = text.device_scan(buf, 0, text.VCF)
    return scan, vcf.decode(buf, scan, contigs)


def noodles_bounds(bounds_row):
    """Our bounds (ends in the line, tabs included) as the reader's Bounds
    (ends in the line with the tabs removed): field k has k tabs before it."""
    return [int(bounds_row[k]) - k for k in range(8)]


@pytest.mark.parametrize("eol", [b"\n", b"\r\n"])
def test_read_record_vectors(eol):
    scan, got = decode(b".\t1\t.\tN\t.\t.\t.\t." + eol)
    assert len(scan["record_offsets"]) == 1 and got["status"][0] == vcf.OK
    assert noodles_bounds(got["bounds"][0]) == [1, 2, 3, 4, 5, 6, 7, 8]  # Bounds::default()
    assert got["bounds"][0][8] == 15  # the line without its CR
    assert got["pos"][0] == 1
    missing = vcf.ID_MISSING | vcf.ALT_MISSING | vcf.QUAL_MISSING | vcf.FILTER_MISSING | vcf.INFO_MISSING
    assert got["flags"][0] == missing | vcf.SAMPLES_MISSING


def test_a_line_without_eight_fields_is_unexpected_eol():
    _, got = decode(b"chr1\t5\t.\tA\tC\t.\tPASS\nx\n")
    assert list(got["status"]) == [vcf.UNEXPECTED_EOL, vcf.UNEXPECTED_EOL]
    _, got = decode(b"chr1\t5\t.\tA\tC\t.\tPASS\t.\n")  # INFO at the end of the line is enough
    assert list(got["status"]) == [vcf.OK]


def test_calls_vcf_matches_the_text_fields():
    raw = bytes(np.load(GOLDEN / "text_real.npz")["calls_vcf"])
    header = b"\n".join(l for l in raw.split(b"\n") if l.startswith(b"#"))
    contigs = vcf.header_contigs(header)
    assert contigs[:3] == [b"chr1", b"chr2", b"chr3"]
    scan, got = decode(raw, contigs)
    assert len(scan["header_offsets"]) == 235 and len(got["pos"]) == 275
    assert all(np.diff(scan["field_starts"].astype(np.int64)) == 9)  # 10 fields
    assert (got["status"] == vcf.OK).all()
    lines = [l for l in raw.split(b"\n") if l and not l.startswith(b"#")]
    for r, line in enumerate(lines):
        f = line.split(b"\t")
        assert contigs[got["chrom"][r]] == f[0]
        assert got["pos"][r] == int(f[1])
        assert got["n_alt"][r] == len(f[4].split(b","))
        assert got["qual"][r] == vcf.f32_bits(float(f[5]))
        assert bool(got["flags"][r] & vcf.FILTER_PASS) == (f[6] == b"PASS")


def test_positions_follow_usize_from_str():
    cases = {b"+5": (5, vcf.OK), b"0": (0, vcf.OK), b"00": (0, vcf.INVALID_POSITION),
             b"-1": (0, vcf.INVALID_POSITION), b"": (0, vcf.INVALID_POSITION), b"+": (0, vcf.INVALID_POSITION),
             b"007": (7, vcf.OK), b"18446744073709551615": ((1 << 64) - 1, vcf.OK),
             b"18446744073709551616": (0, vcf.INVALID_POSITION), b"1e3": (0, vcf.INVALID_POSITION),
             b" 5": (0, vcf.INVALID_POSITION)}
    raw = b"".join(b"c\t" + p + b"\t.\tA\t.\t.\t.\t.\n" for p in cases)
    _, got = decode(raw)
    for r, (p, (pos, st)) in enumerate(cases.items()):
        assert (int(got["pos"][r]), int(got["status"][r])) == (pos, st), p
        assert bool(got["flags"][r] & vcf.TELOMERE) == (p == b"0")


def test_nearest_binary32():
    rng = random.Random(7)
    for _ in range(3000):
        s = f"{rng.randint(0, 10 ** rng.randint(1, 9))}.{rng.randint(0, 999999):06d}e{rng.randint(-12, 12)}"
        want = vcf.f32_bits(float(np.float32(s)))
        assert vcf.f32_nearest(vcf.decimal(s.encode())) == want, s
    # exact ties go to the even significand
    assert vcf.f32_nearest(Fraction(2 ** 24 + 1)) == vcf.f32_bits(2.0 ** 24)
    assert vcf.f32_nearest(Fraction(2 ** 24 + 3)) == vcf.f32_bits(2.0 ** 24 + 4)
    assert vcf.f32_nearest(Fraction(-1, 3)) == vcf.f32_bits(float(np.float32(-1 / 3)))
    assert vcf.f32_nearest(Fraction(10) ** 39) == 0x7F800000


def test_quality_fast_path():
    for s, parsed in [(b"50", True), (b"29.5", True), (b"1e3", True), (b"1E-2", True), (b".5", True),
                      (b"5.", True), (b"-0", True), (b"+7.25", True), (b"1e12", True), (b"16777216", True),
                      (b"16777217", False), (b"123456789.5", False), (b"1e11", True), (b"1e-11", False),
                      (b"3e40", False), (b"inf", False), (b"NaN", False), (b"abc", False), (b"", False),
                      (b"+", False), (b"1e", False), (b"e1", False), (b"1.2.3", False), (b"0e999999999", True),
                      (b"0.000000000000000000001", False), (b"0.0000000001", True), (b"12345678901234567890", False)]:
        ok, bits = vcf.qual_fast_path(s)
        assert ok == parsed, s
        if ok:
            v = vcf.decimal(s)  # a Fraction has no signed zero: f32::from_str("-0") is -0.0
            assert bits == (vcf.f32_nearest(v) if v else (0x80000000 if s[:1] == b"-" else 0)), s
    assert vcf.qual_fast_path(b"-0")[1] == 0x80000000
    assert vcf.qual_fast_path(b"0.1")[1] == vcf.f32_bits(float(np.float32(0.1)))


def test_fields_and_missing_markers():
    lines = [b"chr2\t10\trs1;rs2\tA\tC,G,T\t13.5\tq10;s50\tDP=3\tGT\t0|1",
             b"chrX\t11\t.\tAC\t\t.\tPASS\t.\t.\t0|1",
             b"chrX\t12\t.\tA\t.\t.\t.\tX=1\t",
             b"chrUn\t13\t.\tA\t<DEL>\t.\t.\t.\tGT",
             b"chr2\t14\t.\tA\tG\t.\t.\t.\r"]  # unterminated: the CR stays
    _, got = decode(b"\n".join(lines), [b"chr2", b"chrX", b"chr2"])
    assert list(got["chrom"]) == [0, 1, 1, -1, 0]
    assert list(got["n_alt"]) == [3, 0, 0, 1, 1]
    f = [int(x) for x in got["flags"]]
    assert f[0] & vcf.QUAL_PARSED and not f[0] & vcf.SAMPLES_MISSING and not f[0] & vcf.FILTER_PASS
    assert f[1] & vcf.ID_MISSING and not f[1] & vcf.ALT_MISSING and f[1] & vcf.FILTER_PASS
    assert f[1] & vcf.SAMPLES_MISSING  # FORMAT "."
    assert f[2] & vcf.ALT_MISSING and f[2] & vcf.SAMPLES_MISSING  # nothing after INFO's tab
    assert not f[3] & vcf.SAMPLES_MISSING
    assert got["bounds"][4][8] == len(lines[4]) and not f[4] & vcf.INFO_MISSING  # INFO is ".\r"


def test_genotype_iterator_vectors():
    """value/genotype/iter.rs test_next: each value's (position, phasing) list."""
    assert vcf.alleles(b"0|0") == [(0, True), (0, True)]
    assert vcf.alleles(b"0/1") == [(0, False), (1, False)]
    assert vcf.alleles(b"|0/1") == [(0, True), (1, False)]
    assert vcf.alleles(b"|1/2|3") == [(1, True), (2, False), (3, True)]
    assert vcf.alleles(b"./.") == [(None, False), (None, False)]
    assert vcf.alleles(b"") is None  # UnexpectedEof
    # test_is_implicitly_unphased / test_next_allele, through the first allele
    assert vcf.alleles(b"0") == [(0, True)]
    assert vcf.alleles(b"/0") == [(0, False)]


def test_genotype_packing_and_lookup():
    code = vcf.gt_code
    assert code(b"0|1") == (2 << 26) | (1 << 25) | (1 << 24) | (2 << 12) | 1
    assert code(b"./.") == 2 << 26
    assert code(b".") == vcf.GT_MISSING << 28 and code(b"") == vcf.GT_INVALID << 28
    assert code(b"0|") == vcf.GT_INVALID << 28 and code(b"-1|0") == vcf.GT_INVALID << 28
    assert code(b"0|1|2") == vcf.GT_UNREPRESENTED << 28 and code(b"4095|0") == vcf.GT_UNREPRESENTED << 28
    assert code(b"4094|0") & 0xFFF == 4095
    lines = [b"c\t1\t.\tA\tC\t.\t.\t.\tGT:DP\t0|1:5\t./.:.\t1:3",
             b"c\t2\t.\tA\tC\t.\t.\t.\tDP:GT\t5:0/1\t7\t\t.:.",
             b"c\t3\t.\tA\tC\t.\t.\t.\tDP\t5",
             b"c\t4\t.\tA\tC\t.\t.\t.\t.\t0|1",
             b"c\t5\t.\tA\tC\t.\t.\t."]
    buf = np.frombuffer(b"\n".join(lines) + b"\n", np.uint8)
    scan = text.device_scan(buf, 0, text.VCF)
    calls, key = vcf.genotypes(buf, scan)
    assert list(key) == [0, 1, -1, -1, -1]
    fs = scan["field_starts"].astype(int)
    row = lambda r: [int(c) for c in calls[fs[r] + 8:fs[r + 1]]]  # noqa: E731
    assert row(0) == [code(b"0|1"), code(b"./."), code(b"1")]
    assert row(1) == [code(b"0/1"), vcf.GT_NONE << 28, vcf.GT_NONE << 28, vcf.GT_MISSING << 28]
    assert row(2) == [vcf.GT_NONE << 28] and row(3) == [vcf.GT_NONE << 28] and row(4) == []
