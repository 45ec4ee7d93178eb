"""The oracle pinned before it is trusted (CPU only).

Three independent anchors:
  * the reference's own known answers -- CRC-32 values
    (crates/fritillaria-bgzf/src/deflate.rs:117-118) and the fixture facts its
    tests assert (crates/fritillaria-bam/tests/htslib.rs:83-108, 283-314,
    tests/ont.rs, tests/pacbio.rs:206-221, testdata/README.md:141-152) -- read
    from the reference's testdata where that tree is present;
  * the golden vectors of tests/golden/, produced by the reference's kernels
    (inflate.cu, bam_decode.cu) compiled as host code (tests/golden/make_golden.py);
  * the same reference kernels run live where oracle/_ref was built, and
    Python's zlib for raw DEFLATE and CRC-32.
Planted mistakes (a flipped CRC, a wrong ISIZE, a cut payload, a broken
header) check that the oracle fails with the reference's error variant and
member offset.
"""

import ctypes as C
import hashlib
import zlib
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from oracle.build import REFERENCE_TESTDATA as TESTDATA

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("fields_", "text_")))  # record-field and text inputs have their own tests

# frt_status / Error variants (crates/fritillaria-core/src/error.rs:14-67)
INVALID_BLOCK, CHECKSUM, SIZE, INFLATE, MALFORMED = 2, 3, 4, 5, 6


def fixture(name):
    p = TESTDATA / name
    if not p.exists():
        pytest.skip(f"reference fixture {name} not present")
    return np.fromfile(p, dtype=np.uint8)


def golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def spans_of(g):
    s = np.zeros(len(g["span_isize"]), dtype=oracle.SPAN_DTYPE)
    for f in ("compressed_offset", "payload_start", "payload_len", "isize", "crc32"):
        s[f] = g[f"span_{f}"]
    return s


# ---- CRC-32 -------------------------------------------------------------


def test_crc32_known_answers():
    assert oracle.crc32(b"") == 0
    assert oracle.crc32(b"noodles") == 0x802A58A1


def test_crc32_matches_zlib_and_combines():
    rng = np.random.default_rng(5)
    for n in (1, 7, 64, 1000, 65536):
        a = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        b = rng.integers(0, 256, n // 3 + 1, dtype=np.uint8).tobytes()
        assert oracle.crc32(a) == zlib.crc32(a)
        assert oracle.crc32_combine(zlib.crc32(a), zlib.crc32(b), len(b)) == zlib.crc32(a + b)


# ---- golden vectors from the reference kernels --------------------------


@pytest.mark.parametrize("case", CASES)
def test_oracle_discovers_the_golden_members(case):
    g = golden(case)
    spans, used = oracle.discover(g["bgzf"])
    assert used == g["bgzf"].size
    want = spans_of(g)
    for f in ("compressed_offset", "payload_start", "payload_len", "isize", "crc32"):
        assert np.array_equal(spans[f], want[f]), f


@pytest.mark.parametrize("case", CASES)
def test_oracle_inflates_like_the_reference_kernel(case):
    g = golden(case)
    data, offs = oracle.inflate_batch(g["bgzf"], spans_of(g))
    assert data.size == int(g["inflated_len"])
    assert np.array_equal(g["ref_produced"], np.diff(offs).astype(np.uint32))
    for i in range(len(offs) - 1):
        member = data[offs[i]:offs[i + 1]].tobytes()
        assert hashlib.sha256(member).digest() == g["member_sha256"][i], f"member {i}"
        assert oracle.crc32(member) == g["ref_crc"][i]


@pytest.mark.parametrize("case", [c for c in CASES if c.startswith("bam_")])
def test_oracle_scans_and_decodes_like_the_reference_kernels(case):
    g = golden(case)
    data, offs = oracle.inflate_batch(g["bgzf"], spans_of(g))
    start, n_ref = oracle.bam_header(data)
    assert start == int(g["records_start"]) and n_ref == int(g["n_ref"])
    rec, tail = oracle.bam_scan(data, start)
    assert np.array_equal(rec, g["record_offsets"])
    assert tail == int(g["tail"])
    brec, btail, _ = oracle.bam_scan_blocked(data, offs, start)
    assert np.array_equal(brec, g["record_offsets"]) and btail == int(g["tail"])
    cols = oracle.bam_decode(data, rec)
    for key in g:
        if key.startswith("col_"):
            assert np.array_equal(cols[key[4:]], g[key]), key


# ---- planted mistakes ---------------------------------------------------


def _one_member_file():
    g = golden("deflate_strategies")
    spans = spans_of(g)
    k = 3  # a dynamic-Huffman DNA member
    s = spans[k]
    lo = int(s["compressed_offset"])
    hi = int(s["payload_start"] + s["payload_len"]) + 8
    return g["bgzf"][lo:hi].copy()


def test_flipped_crc_is_a_checksum_mismatch_at_the_member():
    base = _one_member_file()
    two = np.concatenate([base, base])
    two[-8] ^= 1  # the second member's stored CRC
    spans, _ = oracle.discover(two)
    with pytest.raises(oracle.OracleError) as ei:
        oracle.inflate_batch(two, spans)
    assert ei.value.code == CHECKSUM
    assert ei.value.offset == base.size


def test_wrong_isize_is_a_size_mismatch():
    m = _one_member_file()
    m[-4:] = np.frombuffer(np.uint32(int(np.frombuffer(m[-4:].tobytes(), "<u4")[0]) - 1).tobytes(), np.uint8)
    spans, _ = oracle.discover(m)
    with pytest.raises(oracle.OracleError) as ei:
        oracle.inflate_batch(m, spans)
    # one byte more is produced than ISIZE allows: an inflate overrun
    assert ei.value.code in (INFLATE, SIZE)
    assert ei.value.offset == 0


def test_cut_payload_is_an_inflate_error():
    m = _one_member_file()
    spans, _ = oracle.discover(m)
    spans["payload_len"] -= 200
    with pytest.raises(oracle.OracleError) as ei:
        oracle.inflate_batch(m, spans)
    assert ei.value.code in (INFLATE, SIZE)


def test_broken_header_is_an_invalid_block_at_its_offset():
    m = _one_member_file()
    two = np.concatenate([m, m])
    two[m.size + 3] = 0  # FLG without FEXTRA
    with pytest.raises(oracle.OracleError) as ei:
        oracle.discover(two)
    assert ei.value.code == INVALID_BLOCK
    assert ei.value.offset == m.size


def test_partial_trailing_member_is_left_for_the_next_window():
    m = _one_member_file()
    two = np.concatenate([m, m[:-10]])
    spans, used = oracle.discover(two)
    assert len(spans) == 1 and used == m.size


# ---- the reference's fixtures and known answers --------------------------


def _bam_fixture(name):
    raw = fixture(name)
    spans, used = oracle.discover(raw)
    assert used == raw.size
    data, offs = oracle.inflate_batch(raw, spans)
    start, n_ref = oracle.bam_header(data)
    rec, tail = oracle.bam_scan(data, start)
    return raw, spans, data, offs, start, n_ref, rec, tail, oracle.bam_decode(data, rec)


def test_htslib_bam_known_answers():
    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture("htslib.bam")
    assert n_ref == 2
    assert len(rec) == 8 and tail == data.size
    assert cols["pos"].tolist() == [6, 8, 8, 15, 28, 36, -1, 0]
    assert cols["flags"].tolist() == [99, 0, 0, 0, 0, 83, 4, 0]
    assert cols["mapq"].tolist() == [60, 30, 30, 30, 30, 60, 0, 40]
    assert cols["seq_len"].tolist() == [17, 14, 6, 11, 6, 9, 9, 5]
    assert cols["ref_id"].tolist() == [0, 0, 0, 0, 0, 0, -1, 1]
    assert cols["n_cigar"][6] == 0  # r007: unmapped, `*` CIGAR
    name0 = data[rec[0] + 36: rec[0] + 36 + cols["name_len"][0] - 1].tobytes()
    assert name0 == b"r001"


def test_htslib_multiblock_known_answers():
    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture("htslib_multiblock.bam")
    assert len(rec) == 4000 and tail == data.size
    assert cols["pos"][0] == 0 and cols["pos"][1] == 100 and cols["pos"][3999] == 399_900
    assert (cols["seq_len"] == 100).all() and (cols["mapq"] == 60).all()
    i = 3999
    assert data[rec[i] + 36: rec[i] + 36 + cols["name_len"][i] - 1].tobytes() == b"read003999"


def test_ont_ultralong_records_span_members():
    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture("ont_ultralong.bam")
    assert n_ref == 195 and len(rec) == 4 and tail == data.size
    ends = np.append(rec[1:], data.size)
    assert (ends - rec).tolist() == [254_293, 113_876, 4_277, 9_535]
    assert cols["seq_len"].tolist() == [162_932, 73_028, 0, 5_556]
    assert cols["n_cigar"].tolist() == [2_251, 967, 1_037, 267]
    crossed = [int(np.searchsorted(offs, e, "left") - np.searchsorted(offs, s, "right")) for s, e in zip(rec, ends)]
    assert crossed[0] == 3


def test_pacbio_aux_types_and_counts():
    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture("pacbio_hifi.bam")
    assert len(rec) == 20 and n_ref == 86
    types, subtypes, total = set(), set(), 0
    for i in range(len(rec)):
        ent, st = oracle.bam_aux(data, int(rec[i]), int(cols["aux_start"][i]), int(cols["record_end"][i]))
        assert st == 0
        assert 25 <= len(ent) <= 29
        assert cols["aux_count"][i] == len(ent)
        types |= {chr(t) for t in ent["type"]}
        subtypes |= {chr(s) for t, s in zip(ent["type"], ent["subtype"]) if t == ord("B")}
        total += len(ent)
    assert types == set("BCISZf")
    assert subtypes == set("CSfi")
    assert total > 500


@pytest.mark.parametrize("name", ["htslib.bam", "htslib_multiblock.bam", "pacbio_hifi.bam", "ont_ultralong.bam"])
def test_blocked_scan_equals_serial_scan_on_fixtures(name):
    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture(name)
    brec, btail, _ = oracle.bam_scan_blocked(data, offs, start)
    assert np.array_equal(brec, rec) and btail == tail
    # re-blocked at arbitrary cut points, records straddling every block
    cuts = np.unique(np.concatenate([[0], np.arange(start, data.size, 777), [data.size]]).astype(np.uint64))
    brec, btail, _ = oracle.bam_scan_blocked(data, cuts, start)
    assert np.array_equal(brec, rec) and btail == tail


def test_oracle_inflate_matches_zlib_on_fixtures():
    for name in ("htslib.bam", "htslib_multiblock.bam", "pacbio_hifi.bam", "ont_ultralong.bam",
                 "illumina.fastq.gz", "kg_phase3.bcf"):
        raw = fixture(name)
        spans, used = oracle.discover(raw)
        data, offs = oracle.inflate_batch(raw, spans)
        for i, s in enumerate(spans):
            p = raw[int(s["payload_start"]): int(s["payload_start"] + s["payload_len"])].tobytes()
            assert zlib.decompress(p, -15) == data[offs[i]:offs[i + 1]].tobytes()


# ---- the reference's kernels, run live ----------------------------------


def _ref():
    lib = oracle.ref_lib()
    if lib is None:
        pytest.skip("reference kernels (oracle/_ref) not built: no reference tree")
    return lib


@pytest.mark.parametrize("name", ["htslib.bam", "htslib_multiblock.bam", "pacbio_hifi.bam", "ont_ultralong.bam"])
def test_oracle_matches_the_reference_kernels_on_fixtures(name):
    _ref()
    from oracle import ref

    raw, spans, data, offs, start, n_ref, rec, tail, cols = _bam_fixture(name)
    rdata, roffs, status, produced, crc = ref.inflate(raw, spans)
    assert not status.any()
    assert np.array_equal(rdata, data)
    assert np.array_equal(crc, spans["crc32"])
    rrec, rtail, rcols = ref.bam(data, roffs, start)
    assert np.array_equal(rrec, rec) and rtail == tail
    for k, v in rcols.items():
        assert np.array_equal(cols[k], v), k


def test_reference_crc_kernel_matches_oracle():
    lib = _ref()
    g = golden("deflate_strategies")
    data, offs = oracle.inflate_batch(g["bgzf"], spans_of(g))
    n = len(offs) - 1
    off = np.ascontiguousarray(offs[:-1], dtype=np.uint64)
    ln = np.diff(offs).astype(np.uint32)
    out = np.zeros(n, np.uint32)
    buf = np.concatenate([data, np.zeros(1, np.uint8)])
    lib.ref_crc32_blocks(buf.ctypes.data_as(C.c_void_p), off.ctypes.data_as(C.c_void_p),
                         ln.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p), n)
    assert np.array_equal(out, g["span_crc32"])


def test_threaded_whole_file_decode_equals_the_serial_oracle():
    """The whole-file decode the benchmark checks its full-size run against
    (threaded inflate, scan, columns, virtual offsets, aux directory) gives
    what the serial oracle functions give on the same file."""
    from fritillaria_gb300 import synth

    _, bgzf = synth.short_read_bam(3000, n_contigs=3, genome_len=3_000_000, seed=9, levels=(1, 6))
    want = oracle.decode_bam_file(bgzf)
    n = len(want["columns"]["pos"])
    entries = sum(oracle.bam_aux(want["inflated"], int(o), int(want["columns"]["aux_start"][i]),
                                 int(want["columns"]["record_end"][i]))[0].size
                  for i, o in enumerate(want["columns"]["record_offsets"]))
    got = oracle.decode_bam_file_mt(bgzf, 4, n, entries, want["inflated"].size)
    assert np.array_equal(got["inflated"], want["inflated"])
    assert got["tail"] == want["tail"] and got["records_start"] == want["records_start"]
    for k, _ in oracle.BAM_COLUMNS:
        assert np.array_equal(got["columns"][k], want["columns"][k]), k
    assert np.array_equal(got["columns"]["record_offsets"], want["columns"]["record_offsets"])
    vo = oracle.virtual_offsets(want["spans"], want["offsets"][:-1], want["columns"]["record_offsets"])
    assert np.array_equal(got["columns"]["virtual_offset"], vo)
    first = got["columns"]["aux_first"]
    for i in (0, 1, n // 2, n - 1):
        e, _ = oracle.bam_aux(want["inflated"], int(want["columns"]["record_offsets"][i]),
                              int(want["columns"]["aux_start"][i]), int(want["columns"]["record_end"][i]))
        assert np.array_equal(got["aux_entries"][first[i]:first[i + 1]], e)
    assert int(first[-1]) == entries
    # a capacity one record short is refused with the sizes found
    with pytest.raises(RuntimeError, match="records"):
        oracle.decode_bam_file_mt(bgzf, 2, n - 2, entries, want["inflated"].size)
    assert np.array_equal(oracle.inflate_file(bgzf, 3), want["inflated"])
