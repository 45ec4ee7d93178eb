"""The FASTQ, BCF and FASTA oracles pinned before they are trusted (CPU only).

Anchors:
  * the reference's fixture facts (testdata/README.md:187-380): FASTQ record
    counts and read lengths, BCF record/sample counts, controls.fa against its
    committed samtools .fai;
  * the reference's hand-built FASTQ cases (crates/fritillaria-fastq/src/
    columnar/record.rs tests: the '@' decoy in a quality line, the
    length-matched decoy only the '+' check rejects, a final record without a
    newline, a short quality line);
  * the reference's own kernels (fastq_scan.cu, bcf_scan.cu, fasta_compact.cu)
    compiled as host code and driven in their launchers' order, on the
    fixtures, on batch seams cut through them, and on synthetic data.
"""

from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle
from oracle.build import REFERENCE_TESTDATA as TESTDATA
from oracle import ref as ref_kernels



def fixture(name):
    p = TESTDATA / name
    if not p.exists():
        pytest.skip(f"reference fixture {name} not present")
    return np.fromfile(p, dtype=np.uint8)


def inflated(name):
    raw = fixture(name)
    spans, _ = oracle.discover(raw)
    data, offs = oracle.inflate_batch(raw, spans)
    return data, offs


def ref():
    if ref_kernels.lib() is None:
        pytest.skip("reference kernels (oracle/_ref) not built: no reference tree")
    return ref_kernels.lib()


def ref_fastq(buf, start):
    ref()
    return ref_kernels.fastq(buf, start)


def ref_bcf(buf, start, samples, contigs):
    ref()
    return ref_kernels.bcf(buf, start, samples, contigs)


def same(a, b, keys):
    for k in keys:
        assert np.array_equal(a["columns"][k], b["columns"][k]), k
    assert a["tail"] == b["tail"]


FQ_KEYS = [k for k, _ in oracle.FASTQ_COLUMNS] + ["record_offsets"]
BCF_KEYS = [k for k, _ in oracle.BCF_COLUMNS] + ["record_offsets"]


# ---- FASTQ --------------------------------------------------------------------


@pytest.mark.parametrize("name,records,lo,hi", [("illumina.fastq.gz", 4000, 100, 100),
                                               ("pacbio_hifi.fastq.gz", 8, 13_661, 20_499),
                                               ("ont_ultralong.fastq.gz", 3, 5_556, 162_932)])
def test_fastq_fixture_facts(name, records, lo, hi):
    data, _ = inflated(name)
    r = oracle.fastq_decode(data, 0)
    lens = r["columns"]["sequence_len"]
    assert len(lens) == records and lens.min() == lo and lens.max() == hi
    assert r["tail"] == data.size and r["proof"] == oracle.TILED and r["survivors"] == records


def test_illumina_fixture_holds_its_decoys():
    data, _ = inflated("illumina.fastq.gz")
    r = oracle.fastq_decode(data, 0)
    c = r["columns"]
    q = c["record_offsets"] + c["quality_start"]
    assert int((data[q.astype(np.int64)] == ord("@")).sum()) == 83


def _rec(name, seq, plus=b""):
    return b"@" + name + b"\n" + seq + b"\n+" + plus + b"\n" + b"I" * len(seq) + b"\n"


def test_fastq_hand_built_cases():
    # an '@' opening a quality line is not a record start
    buf = bytearray(_rec(b"r0", b"ACGT"))
    qs = len(buf) - 5
    buf[qs] = ord("@")
    buf += _rec(b"r1", b"TTTT")
    r = oracle.fastq_decode(bytes(buf), 0)
    assert len(r["columns"]["record_offsets"]) == 2 and r["tail"] == len(buf)
    # a length-matched decoy that only the '+' check rejects
    buf = b"@A\nACG\n+\n@BC\n" + b"@XY\nACGT\n+ab\nIIII\n"
    r = oracle.fastq_decode(buf, 0)
    assert r["columns"]["record_offsets"].tolist() == [0, 13]
    # the final record may lack its newline
    buf = _rec(b"r0", b"ACGT")[:-1]
    r = oracle.fastq_decode(buf, 0)
    assert r["columns"]["record_end"].tolist() == [len(buf)] and r["tail"] == len(buf)
    # a quality line one byte short is a partial record: the tail
    buf = _rec(b"r0", b"ACGT") + _rec(b"r1", b"ACGT")[:-2]
    r = oracle.fastq_decode(buf, 0)
    assert len(r["columns"]["record_offsets"]) == 1 and r["tail"] == len(_rec(b"r0", b"ACGT"))


EDGE_FASTQ = {
    "blank_lines_between": _rec(b"a", b"ACGT") + b"\n\n" + _rec(b"b", b"GG") + b"\n" + _rec(b"c", b"T"),
    "trailing_blank_lines": _rec(b"a", b"ACGT") + _rec(b"b", b"GG") + b"\n\n",
    "leading_newline": b"\n" + _rec(b"a", b"ACGT") + _rec(b"b", b"GG"),
    "garbage_mid": _rec(b"a", b"ACGT") + b"xyz\n" + _rec(b"b", b"GG"),
    "partial_tail": _rec(b"a", b"ACGT") + b"@b\nAC",
    "only_partial": b"@b\nACGT\n+\nII",
    "only_newlines": b"\n\n\n",
    "decoy_in_chain": b"@A\nACG\n+\nIII\n@BC\n+\n@B\nII\n" + _rec(b"z", b"AC"),
    "no_newline_end": _rec(b"a", b"ACGT") + _rec(b"b", b"GG")[:-1],
    "empty_sequence": b"@a\n\n+\n\n" + _rec(b"b", b"G"),
}


@pytest.mark.parametrize("case", sorted(EDGE_FASTQ))
def test_fastq_edge_cases_match_the_reference_kernels(case):
    buf = np.frombuffer(EDGE_FASTQ[case], dtype=np.uint8)
    for start in range(0, min(len(buf), 12)):
        got = oracle.fastq_decode(buf, start)
        want = ref_fastq(buf, start)
        same(got, want, FQ_KEYS)
        assert got["proof"] == want["proof"] and got["survivors"] == want["survivors"], (case, start)


@pytest.mark.parametrize("name", ["illumina.fastq.gz", "pacbio_hifi.fastq.gz", "ont_ultralong.fastq.gz"])
def test_fastq_oracle_matches_reference_kernels_across_seams(name):
    data, offs = inflated(name)
    same(oracle.fastq_decode(data, 0), ref_fastq(data, 0), FQ_KEYS)
    # the reader's carry: batches of members, each resuming at the last tail
    for per in (1, 3):
        start_file = 0
        for i in range(0, len(offs) - 1, per):
            lo = int(min(start_file, offs[i]))
            hi = int(offs[min(i + per, len(offs) - 1)])
            batch = data[lo:hi]
            got = oracle.fastq_decode(batch, start_file - lo)
            want = ref_fastq(batch, start_file - lo)
            same(got, want, FQ_KEYS)
            start_file = lo + got["tail"]


def test_fastq_synthetic_matches_reference_kernels():
    raw, _ = synth.fastq(3000, seed=11)
    same(oracle.fastq_decode(raw, 0), ref_fastq(raw, 0), FQ_KEYS)
    raw, _ = synth.fastq(6, kind="ont", seed=12)
    same(oracle.fastq_decode(raw, 0), ref_fastq(raw, 0), FQ_KEYS)


# ---- BCF ----------------------------------------------------------------------


@pytest.mark.parametrize("name,records,samples", [("kg_phase3.bcf", 715, 2504), ("giab_hg002.bcf", 275, 1),
                                                  ("giab_hg002_idx_gap.bcf", 275, 1)])
def test_bcf_fixture_facts(name, records, samples):
    data, _ = inflated(name)
    rs, ns, nc = oracle.bcf_header(data)
    assert ns == samples
    r = oracle.bcf_decode(data, rs, ns, nc)
    assert len(r["columns"]["record_offsets"]) == records and r["tail"] == data.size
    assert r["proof"] == oracle.TILED and r["sieved"] == records and r["validated"] == records
    assert (r["columns"]["sample_count"] == samples).all()


@pytest.mark.parametrize("name", ["kg_phase3.bcf", "giab_hg002.bcf", "giab_hg002_idx_gap.bcf"])
def test_bcf_oracle_matches_reference_kernels_across_seams(name):
    data, offs = inflated(name)
    rs, ns, nc = oracle.bcf_header(data)
    got, want = oracle.bcf_decode(data, rs, ns, nc), ref_bcf(data, rs, ns, nc)
    same(got, want, BCF_KEYS)
    assert (got["sieved"], got["validated"], got["proof"]) == (want["sieved"], want["validated"], want["proof"])
    start_file = rs
    for i in range(len(offs) - 1):
        lo = int(min(start_file, offs[i]))
        hi = int(offs[i + 1])
        batch = data[lo:hi]
        got = oracle.bcf_decode(batch, start_file - lo, ns, nc)
        want = ref_bcf(batch, start_file - lo, ns, nc)
        same(got, want, BCF_KEYS)
        assert got["proof"] == want["proof"]
        start_file = lo + got["tail"]
    assert start_file == data.size


def test_bcf_header_edges():
    data, _ = inflated("giab_hg002.bcf")
    assert oracle.bcf_header(data)[2] == 195
    for bad in (data[:5], b"BAM\x02\x02" + bytes(10), b"BCF\x03\x02" + bytes(10), data[:100]):
        with pytest.raises(oracle.OracleError):
            oracle.bcf_header(np.frombuffer(bytes(bad), np.uint8))


def test_bcf_walk_fallback_matches_the_reference():
    raw, _ = synth.bcf(400, n_samples=8, seed=21)
    rs, ns, nc = oracle.bcf_header(raw)
    good = oracle.bcf_decode(raw, rs, ns, nc)
    # a sample count the records do not carry: nothing survives the sieve and
    # the walk gives the same chain
    got, want = oracle.bcf_decode(raw, rs, ns + 1, nc), ref_bcf(raw, rs, ns + 1, nc)
    same(got, want, BCF_KEYS)
    assert got["proof"] == want["proof"] == oracle.WALKED
    assert np.array_equal(got["columns"]["record_offsets"], good["columns"]["record_offsets"])
    # a record whose l_shared is below the site core stops the walk there
    bad = raw.copy()
    at = int(good["columns"]["record_offsets"][100])
    bad[at:at + 4] = np.frombuffer(np.uint32(10).tobytes(), np.uint8)
    got, want = oracle.bcf_decode(bad, rs, ns, nc), ref_bcf(bad, rs, ns, nc)
    same(got, want, BCF_KEYS)
    assert got["tail"] == at and len(got["columns"]["record_offsets"]) == 100


def test_bcf_synthetic_matches_reference_kernels():
    raw, _ = synth.bcf(1500, n_samples=30, seed=22)
    rs, ns, nc = oracle.bcf_header(raw)
    assert (ns, nc) == (30, 24)
    got, want = oracle.bcf_decode(raw, rs, ns, nc), ref_bcf(raw, rs, ns, nc)
    same(got, want, BCF_KEYS)
    assert len(got["columns"]["record_offsets"]) == 1500 and got["tail"] == raw.size


# ---- FASTA --------------------------------------------------------------------


def test_controls_fa_matches_its_fai():
    fa = fixture("controls.fa")
    fai = [line.split("\t") for line in (TESTDATA / "controls.fa.fai").read_text().splitlines()]
    r = oracle.fasta_compact(fa)
    assert len(r["record_offsets"]) == len(fai) == 2
    for i, (name, length, offset, linebases, linewidth) in enumerate(fai):
        b = r["bounds"][i]
        assert r["sequence_lengths"][i] == int(length)
        assert int(r["record_offsets"][i]) + int(b["sequence_start"]) == int(offset)
        assert b["line_bases"] == int(linebases) and b["line_width"] == int(linewidth) and b["uniform"] == 1
        s = r["sequence"][r["sequence_offsets"][i]: r["sequence_offsets"][i] + r["sequence_lengths"][i]]
        assert np.isin(s, np.frombuffer(b"ACGT", np.uint8)).all()


def _ref_compact(buf):
    ref()
    r = ref_kernels.fasta_compact(buf)
    return r["sequence"], oracle.fasta_compact(buf)


@pytest.mark.parametrize("blank", [False, True])
@pytest.mark.parametrize("width", [60, 70])
def test_fasta_oracle_matches_reference_kernels(blank, width):
    fa = synth.raw_fasta(5, 2_000_000, width, blank, seed=31)
    seq, r = _ref_compact(fa)
    assert np.array_equal(seq, r["sequence"])
    assert (r["bounds"]["uniform"] == 1).all()


def test_fasta_controls_through_the_reference_kernels():
    seq, r = _ref_compact(fixture("controls.fa"))
    assert np.array_equal(seq, r["sequence"])


def test_fasta_edges():
    # ragged wrapping goes the byte-wise way and still drops only newlines
    fa = b">a desc\nACG\nT\nACGTA\n>b\n\n>c\nGG"
    r = oracle.fasta_compact(np.frombuffer(fa, np.uint8))
    assert r["record_offsets"].tolist() == [0, 20, 24]
    assert r["sequence_lengths"].tolist() == [9, 0, 2]
    assert bytes(r["sequence"]) == b"ACGTACGTAGG"
    assert r["bounds"]["uniform"].tolist() == [0, 1, 1]
    # text before the first record is not a record; a final definition line
    # without a newline is not one either
    r = oracle.fasta_compact(np.frombuffer(b"junk\n>a\nAC\n>b", np.uint8))
    assert r["record_offsets"].tolist() == [5] and bytes(r["sequence"]) == b"AC"
    r = oracle.fasta_compact(np.frombuffer(b"no records here\n", np.uint8))
    assert len(r["record_offsets"]) == 0


# ---- golden vectors (the reference's kernels on seeded synthetic inputs) -------

GOLDEN = Path(__file__).resolve().parent / "golden"


def _golden(name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    spans, _ = oracle.discover(g["bgzf"])
    data, _ = oracle.inflate_batch(g["bgzf"], spans)
    return g, data


@pytest.mark.parametrize("name", ["fastq_illumina", "fastq_ultra_long"])
def test_fastq_oracle_matches_golden(name):
    g, data = _golden(name)
    r = oracle.fastq_decode(data, 0)
    for k in FQ_KEYS:
        assert np.array_equal(r["columns"][k], g[f"col_{k}"]), k
    assert r["tail"] == int(g["tail"]) and r["proof"] == int(g["proof"]) and r["survivors"] == int(g["survivors"])


def test_bcf_oracle_matches_golden():
    g, data = _golden("bcf_sites")
    rs, ns, nc = oracle.bcf_header(data)
    assert (rs, ns, nc) == (int(g["records_start"]), int(g["samples"]), int(g["contigs"]))
    r = oracle.bcf_decode(data, rs, ns, nc)
    for k in BCF_KEYS:
        assert np.array_equal(r["columns"][k], g[f"col_{k}"]), k
    assert r["tail"] == int(g["tail"]) and r["proof"] == int(g["proof"])


def test_fasta_oracle_matches_golden():
    import hashlib

    g, data = _golden("fasta_wrapped")
    r = oracle.fasta_compact(data)
    assert hashlib.sha256(r["sequence"].tobytes()).digest() == g["sequence_sha256"].tobytes()
    for k in ("sequence_offsets", "sequence_lengths", "record_offsets"):
        assert np.array_equal(r[k], g[f"col_{k}"]), k
