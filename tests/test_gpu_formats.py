"""FASTQ, BCF and FASTA on the GB300 against the reference's kernels (golden
vectors) and the oracle: whole batches, every edge case the reference's tests
build by hand, batch seams through the reader (records that span batches, the
carry of the tail), the fallback walks, and empty batches.  Modelled on
crates/fritillaria-cuda/tests/fastq_decode.rs, bcf_decode.rs and fasta.rs."""

import hashlib
from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FQ = ["record_offsets", "sequence_start", "plus_start", "quality_start", "sequence_len", "record_end"]
BCF = ["chromosome_id", "position", "reference_span", "quality", "info_count", "allele_count", "sample_count",
       "format_count", "record_offsets", "alleles_start", "filters_start", "info_start", "genotypes_start",
       "record_end"]


def device_batch(frt, codec, raw):
    """The bytes as a device inflate batch (compressed, then inflated by the codec)."""
    bgzf = synth.bgzf(np.frombuffer(bytes(raw), np.uint8), "full", (6, 6))
    spans, _ = frt.discover_blocks(bgzf)
    return codec.inflate_batch_device(bgzf, spans)


def golden_batch(frt, codec, name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    spans, _ = frt.discover_blocks(g["bgzf"])
    return g, codec.inflate_batch_device(g["bgzf"], spans)


# ---- FASTQ ----------------------------------------------------------------------


@pytest.mark.parametrize("name", ["fastq_illumina", "fastq_ultra_long"])
def test_fastq_matches_the_reference_kernels(gpu, name):
    codec, scanner = gpu.CudaCodec(0), gpu.FastqScanner(0)
    g, batch = golden_batch(gpu, codec, name)
    cb = scanner.decode(batch, 0)
    for k in FQ:
        assert np.array_equal(cb.column(k), g[f"col_{k}"]), k
    assert cb.tail() == int(g["tail"])
    proof, survivors, _ = cb.scan_info()
    assert proof == int(g["proof"]) == 0 and survivors == int(g["survivors"])


def _rec(name, seq, plus=b""):
    return b"@" + name + b"\n" + seq + b"\n+" + plus + b"\n" + b"I" * len(seq) + b"\n"


EDGE_FASTQ = {
    "decoy_quality_line": bytes(_rec(b"r0", b"ACGT")[:-5]) + b"@III\n" + _rec(b"r1", b"TTTT"),
    "length_matched_decoy": b"@A\nACG\n+\n@BC\n" + b"@XY\nACGT\n+ab\nIIII\n",
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
    "short_quality_line": _rec(b"r0", b"ACGT") + _rec(b"r1", b"ACGT")[:-2],
}


@pytest.mark.parametrize("case", sorted(EDGE_FASTQ))
def test_fastq_edge_cases(gpu, case):
    codec, scanner = gpu.CudaCodec(0), gpu.FastqScanner(0)
    raw = EDGE_FASTQ[case]
    batch = device_batch(gpu, codec, raw)
    for start in range(0, min(len(raw), 10)):
        want = oracle.fastq_decode(raw, start)
        cb = scanner.decode(batch, start)
        for k in FQ:
            assert np.array_equal(cb.column(k), want["columns"][k]), (case, start, k)
        assert cb.tail() == want["tail"], (case, start)
        proof, survivors, _ = cb.scan_info()
        assert (proof, survivors) == (want["proof"], want["survivors"]), (case, start)


def test_fastq_tiles_denser_than_the_index_slots(gpu):
    """The newline index keeps up to 1,024 newlines of each 16 KiB tile from
    its one read of the bytes; a denser tile (records of a few bytes, runs of
    blank lines) is read again.  Dense and ordinary tiles side by side, at
    starts on and off a tile."""
    codec, scanner = gpu.CudaCodec(0), gpu.FastqScanner(0)
    normal, _ = synth.fastq(400, seed=5)
    normal = bytes(normal)
    tiny = b"".join(_rec(b"", b"ACGT"[i % 4:i % 4 + 1]) for i in range(6000))  # 8 bytes, 4 newlines
    n = len(normal)
    cases = [(normal + tiny + normal + tiny + normal, (0, 3, n, n + 8000, 2 * n + len(tiny) + 40)),
             (normal + tiny + b"\n" * 20000 + normal + tiny[:30001] + normal, (0, n + 16, 16384))]
    for raw, starts in cases:
        batch = device_batch(gpu, codec, raw)
        for start in starts:
            want = oracle.fastq_decode(raw, start)
            cb = scanner.decode(batch, start)
            for k in FQ:
                assert np.array_equal(cb.column(k), want["columns"][k]), (start, k)
            assert cb.tail() == want["tail"], start
            assert cb.scan_info()[:2] == (want["proof"], want["survivors"]), start


def test_fastq_scanner_reuses_and_grows_its_index_slots(gpu):
    """One scanner over a one-tile batch, a batch of many tiles (its kept
    slot array grows) and the one-tile batch again: each equals the oracle."""
    codec, scanner = gpu.CudaCodec(0), gpu.FastqScanner(0)
    small, _ = synth.fastq(20, seed=8)
    big, _ = synth.fastq(6000, seed=9)
    for raw in (bytes(small), bytes(big), bytes(small), bytes(big)[:500_001]):
        batch = device_batch(gpu, codec, raw)
        want = oracle.fastq_decode(raw, 0)
        cb = scanner.decode(batch, 0)
        for k in FQ:
            assert np.array_equal(cb.column(k), want["columns"][k]), (len(raw), k)
        assert cb.tail() == want["tail"]


def test_fastq_empty_batch_decodes_to_an_empty_column_set(gpu):
    codec, scanner = gpu.CudaCodec(0), gpu.FastqScanner(0)
    raw, _ = synth.fastq(50, seed=2)
    batch = device_batch(gpu, codec, raw)
    cb = scanner.decode(batch, raw.size)
    assert cb.is_empty() and cb.tail() == raw.size
    assert all(cb.column(k).size == 0 for k in FQ)
    cb = scanner.decode(batch, raw.size + 7)
    assert cb.is_empty() and cb.tail() == raw.size


def _fastq_through_reader(frt, bgzf, blocks):
    codec, scanner = frt.CudaCodec(0), frt.FastqScanner(0)
    reader = frt.DeviceBgzfReader(bgzf, codec, blocks_per_batch=blocks)
    lens, seams = [], 0
    while (item := reader.next_batch()) is not None:
        cb = scanner.decode(item.data, item.start)
        lens.append(cb.column("sequence_len"))
        # the tiling holds on well-formed FASTQ whenever the batch holds a
        # record (with none the reference reports the walk, fastq.rs:500-520)
        assert cb.scan_info()[0] == (0 if len(cb) else 1)
        reader.carry_from(cb.tail())
        seams += 1
    return np.concatenate(lens), seams


@pytest.mark.parametrize("kind,n,blocks", [("illumina", 20000, 1), ("illumina", 20000, 4), ("ont", 40, 1),
                                           ("ont", 40, 3)])
def test_fastq_across_batch_seams(gpu, kind, n, blocks):
    raw, bgzf = synth.fastq(n, kind=kind, seed=7)
    want = oracle.fastq_decode(raw, 0)["columns"]["sequence_len"]
    got, seams = _fastq_through_reader(gpu, bgzf, blocks)
    assert np.array_equal(got, want)
    assert seams >= 3


# ---- BCF ------------------------------------------------------------------------


def test_bcf_matches_the_reference_kernels(gpu):
    codec, scanner = gpu.CudaCodec(0), gpu.BcfScanner(0)
    g, batch = golden_batch(gpu, codec, "bcf_sites")
    rs, ns, nc = gpu.parse_bcf_header(batch.to_host())
    assert (rs, ns, nc) == (int(g["records_start"]), int(g["samples"]), int(g["contigs"]))
    cb = scanner.decode(batch, rs, ns, nc)
    for k in BCF:
        assert np.array_equal(cb.column(k), g[f"col_{k}"]), k
    assert cb.tail() == int(g["tail"]) and cb.scan_info()[0] == int(g["proof"]) == 0


def _bcf_through_reader(frt, bgzf, blocks):
    codec, scanner = frt.CudaCodec(0), frt.BcfScanner(0)
    reader = frt.DeviceBgzfReader(bgzf, codec, blocks_per_batch=blocks)
    header = None
    out = {k: [] for k in ("record_offsets_len", "position", "genotypes_start", "record_end")}
    proofs = []
    while (item := reader.next_batch()) is not None:
        if header is None:
            try:
                header = frt.parse_bcf_header(item.data.to_host())
            except frt.Malformed:
                reader.carry_from(0)
                continue
            start = header[0]
        else:
            start = item.start
        cb = scanner.decode(item.data, start, header[1], header[2])
        for k in ("position", "genotypes_start", "record_end"):
            out[k].append(cb.column(k))
        proofs.append(cb.scan_info()[0])
        reader.carry_from(cb.tail())
    return {k: np.concatenate(v) for k, v in out.items() if v}, proofs


@pytest.mark.parametrize("sites,samples,blocks", [(3000, 12, 1), (3000, 12, 4), (120, 2000, 1), (120, 2000, 2)])
def test_bcf_across_batch_seams(gpu, sites, samples, blocks):
    raw, bgzf = synth.bcf(sites, n_samples=samples, seed=8)
    rs, ns, nc = oracle.bcf_header(raw)
    want = oracle.bcf_decode(raw, rs, ns, nc)["columns"]
    got, proofs = _bcf_through_reader(gpu, bgzf, blocks)
    for k in ("position", "genotypes_start", "record_end"):
        assert np.array_equal(got[k], want[k]), k
    assert all(p == 0 for p in proofs)


def test_bcf_walk_fallback(gpu):
    codec, scanner = gpu.CudaCodec(0), gpu.BcfScanner(0)
    raw, _ = synth.bcf(400, n_samples=8, seed=21)
    rs, ns, nc = oracle.bcf_header(raw)
    batch = device_batch(gpu, codec, raw)
    # the wrong sample count: nothing survives the sieve, the walk finds the chain
    want = oracle.bcf_decode(raw, rs, ns + 1, nc)
    cb = scanner.decode(batch, rs, ns + 1, nc)
    assert cb.scan_info()[0] == want["proof"] == 1
    for k in BCF:
        assert np.array_equal(cb.column(k), want["columns"][k]), k
    # a record whose l_shared is below the site core stops the chain there
    good = oracle.bcf_decode(raw, rs, ns, nc)
    bad = raw.copy()
    at = int(good["columns"]["record_offsets"][100])
    bad[at:at + 4] = np.frombuffer(np.uint32(10).tobytes(), np.uint8)
    want = oracle.bcf_decode(bad, rs, ns, nc)
    cb = scanner.decode(device_batch(gpu, codec, bad), rs, ns, nc)
    assert cb.tail() == want["tail"] == at and len(cb) == 100
    assert np.array_equal(cb.column("record_offsets"), want["columns"]["record_offsets"])


def test_bcf_empty_and_partial_batches(gpu):
    codec, scanner = gpu.CudaCodec(0), gpu.BcfScanner(0)
    raw, _ = synth.bcf(50, n_samples=4, seed=3)
    rs, ns, nc = oracle.bcf_header(raw)
    batch = device_batch(gpu, codec, raw)
    cb = scanner.decode(batch, raw.size, ns, nc)
    assert cb.is_empty() and cb.tail() == raw.size
    cut = raw[: raw.size - 10]
    want = oracle.bcf_decode(cut, rs, ns, nc)
    cb = scanner.decode(device_batch(gpu, codec, cut), rs, ns, nc)
    assert len(cb) == 49 and cb.tail() == want["tail"] and cb.scan_info()[0] == want["proof"] == 0


# ---- FASTA ----------------------------------------------------------------------


def _check_fasta(cb, want):
    assert len(cb) == len(want["record_offsets"])
    for k in ("sequence_offsets", "sequence_lengths", "record_offsets"):
        assert np.array_equal(cb.column(k), want[k]), k
    assert cb.total_bases() == want["sequence"].size
    assert np.array_equal(cb.column("sequence"), want["sequence"])


def test_fasta_matches_the_reference_kernels(gpu):
    codec, comp = gpu.CudaCodec(0), gpu.FastaCompactor(0)
    g, batch = golden_batch(gpu, codec, "fasta_wrapped")
    cb = comp.compact(batch)
    seq = cb.column("sequence")
    assert hashlib.sha256(seq.tobytes()).digest() == g["sequence_sha256"].tobytes()
    for k in ("sequence_offsets", "sequence_lengths", "record_offsets"):
        assert np.array_equal(cb.column(k), g[f"col_{k}"]), k


@pytest.mark.parametrize("contigs,bases,width,blank", [(24, 30_000_000, 60, False), (3, 2_000_000, 70, True),
                                                       (2, 3_000_000, 1_000_000, False), (1, 100, 7, False)])
def test_fasta_synthetic(gpu, contigs, bases, width, blank):
    codec, comp = gpu.CudaCodec(0), gpu.FastaCompactor(0)
    raw = synth.raw_fasta(contigs, bases, width, blank, seed=9)
    _check_fasta(comp.compact(device_batch(gpu, codec, raw)), oracle.fasta_compact(raw))


EDGE_FASTA = {
    "ragged": b">a desc\nACG\nT\nACGTA\n>b\n\n>c\nGG",
    "junk_before": b"junk\n>a\nAC\n>b",
    "no_records": b"no records here\n",
    "header_only_no_newline": b">only",
    "crlf": b">a\r\nAC\r\nGT\r\n",
    "interior_blank": b">a\nACGT\n\nACGT\nAC\n",
    "gt_inside_header": b">a >b >c\nAAAA\n>d\nC\n",
    # a record start every other byte: 8,192 in a 16 KiB tile, the most a tile's count holds
    "dense_headers": b">\n" * 20000 + b">a\nACGT\n",
    "tiny_records": b">x\nA\n" * 9000,
}


@pytest.mark.parametrize("case", sorted(EDGE_FASTA))
def test_fasta_edges(gpu, case):
    codec, comp = gpu.CudaCodec(0), gpu.FastaCompactor(0)
    raw = EDGE_FASTA[case]
    _check_fasta(comp.compact(device_batch(gpu, codec, raw)), oracle.fasta_compact(np.frombuffer(raw, np.uint8)))
