"""Columnar VCF on the GB300 against the oracle (oracle/vcf.py, pinned to the
vendored reader's tests and the reference's real-file test in
tests/test_oracle_vcf.py): the reference's calls.vcf (bcftools), the
benchmark's synthetic population VCF, hand-built records at every edge the
reader has (short lines, CR before LF and at the batch end, missing markers,
positions usize::from_str rejects, empty ALT, FORMAT "."), and a sweep of
QUAL spellings -- bgzipped, inflated on the device, framed and decoded."""

from pathlib import Path
import random

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import text, vcf

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
COLS = ["chrom", "pos", "bounds", "n_alt", "qual", "flags", "status"]


def run(gpu, raw: bytes, contigs=None, header=None):
    buf = np.frombuffer(raw, np.uint8)
    bgzf = synth.bgzf(buf, "full", (6, 6))
    spans, _ = gpu.discover_blocks(bgzf)
    batch = gpu.CudaCodec(0).inflate_batch_device(bgzf, spans)
    tx = gpu.TextScanner(0).scan(batch, 0, gpu.Dialect.VCF)
    dec = gpu.VcfDecoder(0)
    if header is not None:
        contigs = vcf.header_contigs(header)
        assert dec.set_contigs_from_header(header) == len(contigs)
    elif contigs is not None:
        dec.set_contigs(contigs)
    got = dec.decode(tx)
    scan = text.device_scan(buf, 0, text.VCF)
    want = vcf.decode(buf, scan, contigs or ())
    assert len(got) == len(want["pos"]) == len(tx)
    assert got.tail() == tx.tail()
    for k in COLS:
        assert np.array_equal(got.column(k), want[k]), k
    gt = dec.genotypes(tx)
    calls, key = vcf.genotypes(buf, scan)
    assert np.array_equal(gt.column("calls"), calls) and np.array_equal(gt.column("key"), key)
    got.gt, got.text = gt, tx
    return got


def test_calls_vcf(gpu):
    raw = bytes(np.load(GOLDEN / "text_real.npz")["calls_vcf"])
    header = b"\n".join(l for l in raw.split(b"\n") if l.startswith(b"#"))
    got = run(gpu, raw, header=header)
    assert len(got) == 275 and (got.column("status") == 0).all() and (got.column("chrom") >= 0).all()
    assert (got.quality() == 50.0).all()


def test_synthetic_population_vcf(gpu):
    raw = bytes(synth.raw_vcf_text(600, 97, seed=3))
    header = b"\n".join(l for l in raw.split(b"\n") if l.startswith(b"#"))
    got = run(gpu, raw, header=header)
    assert len(got) == 600 and (got.column("flags") & gpu.VcfFlag.FILTER_PASS).all()
    m = got.gt.matrix(got.text)
    assert m.shape == (600, 97)
    u = gpu.VcfGenotypes.unpack(m)
    assert (u["status"] == 0).all() and (u["ploidy"] == 2).all() and (u["phased"] == 1).all()
    # the generator's genotypes, read back from the text
    lines = [l for l in raw.split(b"\n") if l and not l.startswith(b"#")]
    want = np.array([[[int(g[0:1]), int(g[2:3])] for g in l.split(b"\t")[9:]] for l in lines])
    assert np.array_equal(u["alleles"], want)


def test_wide_records_take_several_warps(gpu):
    """1,200 samples a record: the genotype kernel spreads each record over
    eight warps; short records and lines without samples mixed in after them
    keep their own counts."""
    raw = bytes(synth.raw_vcf_text(40, 1200, seed=5))
    raw += (b"chr1\t5\t.\tA\tC\t.\tPASS\t.\tGT:DP\t0|1:3\t1/1:2\n"
            b"chr1\t6\t.\tA\tC\t.\tPASS\n"
            b"chr2\t7\t.\tA\tC\t.\tPASS\t.\tDP:GT\t" + b"\t".join(b"4:%d|%d" % (i % 3, i % 2) for i in range(700)) + b"\n")
    header = b"\n".join(l for l in raw.split(b"\n") if l.startswith(b"#"))
    got = run(gpu, raw, header=header)
    assert len(got) == 43
    fs = got.text.column("field_starts").astype(np.int64)
    u = gpu.VcfGenotypes.unpack(got.gt.column("calls")[fs[:40, None] + 8 + np.arange(1200)[None, :]])
    assert u["alleles"].shape == (40, 1200, 2) and (u["status"] == 0).all()
    assert list(got.gt.column("key")[40:]) == [0, -1, 1]


EDGE = [b".\t1\t.\tN\t.\t.\t.\t.",
        b".\t1\t.\tN\t.\t.\t.\t.\r",
        b"chr1\t5\t.\tA\tC\t.\tPASS",
        b"x",
        b"chr2\t10\trs1;rs2\tA\tC,G,T\t13.5\tq10;s50\tDP=3\tGT\t0|1",
        b"chrX\t11\t.\tAC\t\t.\tPASS\t.\t.\t0|1",
        b"chrX\t12\t.\tA\t.\t.\t.\tX=1\t",
        b"chrUn\t13\t.\tA\t<DEL>\t1e3\t.\t.\tGT",
        b"chr2\t+14\t.\tA\tG\t-0\t.\t.\tGT:DP\t0/1:3\t./.:.",
        b"chr2\t0\t.\tA\tG\t.5\t.\t.",
        b"chr2\t00\t.\tA\tG\t5.\t.\t.",
        b"chr2\t18446744073709551616\t.\tA\tG\tinf\t.\t.",
        b"chr2\t18446744073709551615\t.\tA\tG\t16777217\t.\t.",
        b"chr_" + b"n" * 300 + b"\t7\t.\tA\tG\t1e-11\t.\t.",
        b"chr2\t7\t.\tA\tG\t1.0000000000000000001\t\t\r",
        b"\t\t\t\t\t\t\t",
        b"chrM\t9\t.\tA\tG\t29.5\tPASS\t.\t.\t.\t."]


@pytest.mark.parametrize("last_newline", [True, False])
def test_edge_records(gpu, last_newline):
    raw = b"##fileformat=VCFv4.2\n#CHROM\n" + b"\n".join(EDGE) + (b"\n" if last_newline else b"")
    got = run(gpu, raw, contigs=[b"chr1", b"chr2", b"chrX", b"chr2", b"chr_" + b"n" * 300, b""])
    st = got.column("status")
    assert st[3] == gpu.VcfStatus.UNEXPECTED_EOL and st[2] == gpu.VcfStatus.UNEXPECTED_EOL
    assert st[10] == gpu.VcfStatus.INVALID_POSITION and st[11] == gpu.VcfStatus.INVALID_POSITION


def test_quality_spellings(gpu):
    rng = random.Random(11)
    quals = [b"50", b"0", b"-0", b"+3", b"3.25", b".001", b"99999999", b"16777216", b"1e10", b"1E+10", b"1e-10",
             b"2.5e-3", b"123456.7", b"0.1", b"nan", b"Infinity", b"1..2", b"", b"+", b"-", b"1e", b"e5"]
    for _ in range(400):
        quals.append(f"{rng.randint(0, 10 ** rng.randint(0, 9))}.{rng.randint(0, 10 ** rng.randint(0, 4))}"
                     f"{'e' + str(rng.randint(-12, 12)) if rng.random() < 0.3 else ''}".encode())
    raw = b"".join(b"chr1\t%d\t.\tA\tC\t%s\t.\t.\n" % (i + 1, q) for i, q in enumerate(quals))
    got = run(gpu, raw, contigs=[b"chr1"])
    parsed = (got.column("flags") & gpu.VcfFlag.QUAL_PARSED) != 0
    # both kinds occur: decimals of up to 8 significant digits parse, longer ones are left to the caller
    want = sum(vcf.qual_fast_path(q)[0] for q in quals)
    assert parsed.sum() == want and 200 < want < len(quals)


def test_empty_and_header_only(gpu):
    dec = gpu.VcfDecoder(0)
    ts = gpu.TextScanner(0)
    empty = dec.decode(ts.scan(None, 0, gpu.Dialect.VCF))
    assert len(empty) == 0 and empty.column("bounds").shape == (0, 9)
    run(gpu, b"##fileformat=VCFv4.2\n#CHROM\tPOS\n")


def test_dictionary_changes_and_errors(gpu):
    raw = b"chr1\t1\t.\tA\t.\t.\t.\t.\nchr9\t2\t.\tA\t.\t.\t.\t.\n"
    buf = np.frombuffer(raw, np.uint8)
    bgzf = synth.bgzf(buf, "full", (6, 6))
    spans, _ = gpu.discover_blocks(bgzf)
    batch = gpu.CudaCodec(0).inflate_batch_device(bgzf, spans)
    tx = gpu.TextScanner(0).scan(batch, 0, gpu.Dialect.VCF)
    dec = gpu.VcfDecoder(0)
    assert list(dec.decode(tx).column("chrom")) == [-1, -1]
    dec.set_contigs(["chr9", "chr1"])
    assert list(dec.decode(tx).column("chrom")) == [1, 0]
    dec.set_contigs([])
    assert list(dec.decode(tx).column("chrom")) == [-1, -1]
    fq = gpu.FastqScanner(0).decode(None, 0)  # columns, but not a text scan's
    with pytest.raises(gpu.InvalidArgument):
        dec.decode(fq)


def test_genotype_spellings(gpu):
    gts = [b"0|0", b"0/1", b"|0/1", b"|1/2|3", b"./.", b".|.", b".", b"", b"1", b"/1", b"0|", b"+1|2", b"-1|2",
           b"4094|0", b"4095|0", b"12|7", b"0/.", b"0|1|2", b"a|b", b"0:1", b"01|00"]
    samples = b"\t".join(g + b":9" for g in gts)
    raw = (b"chr1\t1\t.\tA\tC\t.\t.\t.\tGT:DP\t" + samples + b"\n"
           b"chr1\t2\t.\tA\tC\t.\t.\t.\tDP:GT\t" + b"\t".join(b"9:" + g for g in gts) + b"\n"
           b"chr1\t3\t.\tA\tC\t.\t.\t.\tGT\t\t.\t0|1\r\n"
           b"chr1\t4\t.\tA\tC\t.\t.\t.\tGT\t0/1\r")
    run(gpu, raw, contigs=[b"chr1"])
