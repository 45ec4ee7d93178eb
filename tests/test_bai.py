"""BAI region resolution on the host (CPU only): the library's frt_bai_query
against the oracle's restatement of BinningIndex::query on the reference's
own htslib-written index (testdata/htslib_multiblock.bam.bai) and on
synthetic multi-contig indexes, the records those chunks reach against a
brute-force overlap scan, the reference's merge/optimize known answers
(crates/fritillaria-csi/src/binning_index.rs tests), and the error paths."""

from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import bai as obai
from oracle import oracle
from oracle.build import REFERENCE_TESTDATA as TESTDATA



@pytest.fixture(scope="module")
def frt():
    import fritillaria_gb300 as frt
    from fritillaria_gb300 import build

    if not build.LIB.exists():
        build.build_cuda()
    frt.lib()
    return frt


def _table(bgzf):
    r = oracle.decode_bam_file(bgzf)
    vo = oracle.virtual_offsets(r["spans"], r["offsets"][:-1], r["columns"]["record_offsets"])
    return obai.record_table(r["inflated"], r["columns"]["record_offsets"], vo)


def test_chunk_merge_known_answers():
    chunks = [(2, 5), (3, 4), (5, 7), (9, 12), (10, 15), (16, 21)]
    assert obai.optimize_chunks(chunks) == [(2, 7), (9, 15), (16, 21)]
    assert obai.optimize_chunks(chunks, 10) == [(9, 15), (16, 21)]
    assert obai.optimize_chunks([]) == []


def test_fixture_index_queries(frt):
    p = TESTDATA / "htslib_multiblock.bam.bai"
    if not p.exists():
        pytest.skip("reference fixture not present")
    data = np.fromfile(p, np.uint8)
    idx, lib_idx = obai.parse(data), frt.Bai(data)
    assert lib_idx.reference_count() == len(idx["refs"]) == 1
    t = _table(np.fromfile(TESTDATA / "htslib_multiblock.bam", np.uint8))
    rng = np.random.default_rng(3)
    for _ in range(200):
        s = int(rng.integers(1, 420_000))
        e = s + int(rng.integers(0, 60_000))
        want = obai.query(idx, 0, s, e)
        assert lib_idx.query(0, s, e) == want
        assert np.array_equal(obai.via_chunks(t, want, 0, s, e), obai.brute_force(t, 0, s, e))
    # unbounded
    assert lib_idx.query(0) == obai.query(idx, 0)


def test_synthetic_indexes(frt):
    raw, bgzf = synth.short_read_bam(40_000, n_contigs=24, genome_len=60_000_000, seed=9, levels=(1, 6))
    data = synth.bai(raw, bgzf)
    idx, lib_idx = obai.parse(data), frt.Bai(data)
    assert lib_idx.reference_count() == len(idx["refs"]) == 24
    t = _table(bgzf)
    rng = np.random.default_rng(4)
    total = 0
    for _ in range(300):
        ref = int(rng.integers(0, 24))
        s = int(rng.integers(1, 5_000_000))
        e = s + int(np.exp(rng.uniform(np.log(1_000), np.log(10_000_000))))
        want = obai.query(idx, ref, s, e)
        assert lib_idx.query(ref, s, e) == want
        got = obai.via_chunks(t, want, ref, s, e)
        assert np.array_equal(got, obai.brute_force(t, ref, s, e))
        total += len(got)
    assert total > 1000


def test_index_and_query_errors(frt):
    raw, bgzf = synth.short_read_bam(2000, n_contigs=2, genome_len=5_000_000, seed=2)
    data = synth.bai(raw, bgzf)
    with pytest.raises(frt.Malformed):
        frt.Bai(b"BAM\x01" + bytes(20))
    with pytest.raises(frt.Malformed):
        frt.Bai(data[: len(data) // 2])
    b = frt.Bai(data)
    with pytest.raises(frt.InvalidArgument):
        b.query(5, 1, 100)
    with pytest.raises(frt.InvalidArgument):
        b.query(0, 1 << 30, (1 << 30) + 5)
    with pytest.raises(frt.InvalidArgument):
        b.query(0, 500, 100)


def test_host_region_query_matches_brute_force():
    raw, bgzf = synth.short_read_bam(20_000, n_contigs=24, genome_len=100_000_000, seed=12)
    idx = obai.parse(synth.bai(raw, bgzf))
    spans = oracle.discover(bgzf)[0]
    t = _table(bgzf)
    rng = np.random.default_rng(6)
    for _ in range(60):
        ref = int(rng.integers(0, 24))
        s = int(rng.integers(1, 3_000_000))
        e = s + int(rng.integers(1_000, 2_000_000))
        kept, _ = oracle.region_query(bgzf, spans, idx, ref, s, e)
        assert kept == len(obai.brute_force(t, ref, s, e))
