"""BAM record scan and columns on the GB300 against the oracle, through the
reader/decoder consumer loop of crates/fritillaria-cuda/tests/bam_reader.rs:76-115:
every batch size, records straddling members and batches, ultra-long reads,
members packed full (noodles) and record-aligned (htslib)."""

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

COLS = ["ref_id", "pos", "flags", "mapq", "seq_len", "mate_ref_id", "mate_pos", "tlen", "cigar_start",
        "sequence_start", "quality_start", "aux_start", "record_end", "bin", "n_cigar", "name_len", "aux_count",
        "aux_status"]


def drive(frt, bgzf, blocks):
    codec = frt.CudaCodec(0)
    decoder = frt.BamDecoder(0)
    reader = frt.DeviceBgzfReader(bgzf, codec, blocks_per_batch=blocks)
    out = {k: [] for k in COLS + ["virtual_offset"]}
    header = None
    while True:
        batch = reader.next_batch()
        if batch is None:
            break
        if header is None:
            host = batch.data.to_host()
            try:
                header = frt.parse_header(host)
            except frt.Malformed:
                reader.carry_from(0)
                continue
            decoder.set_reference_count(header[1])
            begin = header[0]
        else:
            begin = batch.start
        records = decoder.decode(batch.data, begin)
        for k in out:
            out[k].append(records.column(k))
        tail = records.tail()
        records.free()
        reader.carry_from(tail)
    return {k: np.concatenate(v) if v else np.zeros(0) for k, v in out.items()}


def expected(bgzf):
    r = oracle.decode_bam_file(bgzf)
    vo = oracle.virtual_offsets(r["spans"], r["offsets"][:-1], r["columns"]["record_offsets"])
    return r, vo


@pytest.mark.parametrize("packing", ["full", "record"])
@pytest.mark.parametrize("blocks", [1, 4, 256])
def test_short_reads_columns(gpu, packing, blocks):
    raw, bgzf = synth.short_read_bam(6000, seed=21, levels=(1, 6), packing=packing)
    r, vo = expected(bgzf)
    got = drive(gpu, bgzf, blocks)
    for k in COLS:
        assert np.array_equal(got[k], r["columns"][k]), k
    assert np.array_equal(got["virtual_offset"], vo)


@pytest.mark.parametrize("blocks", [1, 2, 3, 8, 256])
def test_ultra_long_reads_span_batches(gpu, blocks):
    raw, bgzf = synth.ultra_long_bam(12, n_long_extra=1, seed=4)
    r, vo = expected(bgzf)
    got = drive(gpu, bgzf, blocks)
    for k in COLS:
        assert np.array_equal(got[k], r["columns"][k]), k
    assert np.array_equal(got["virtual_offset"], vo)


def test_aux_directory_matches_oracle(gpu):
    raw, bgzf = synth.ultra_long_bam(6, seed=8)
    codec = gpu.CudaCodec(0)
    decoder = gpu.BamDecoder(0)
    spans, _ = oracle.discover(bgzf)
    data, offs = oracle.inflate_batch(bgzf, spans)
    start, n_ref = oracle.bam_header(data)
    batch = codec.inflate_batch_device(bgzf, spans)
    rb = decoder.decode(batch, start)
    cols = rb.to_host()
    entries = rb.column("aux_entries")
    first = cols["aux_first"]
    for i, off in enumerate(cols["record_offsets"]):
        e, st = oracle.bam_aux(data, int(off), int(cols["aux_start"][i]), int(cols["record_end"][i]))
        got = entries[first[i]:first[i + 1]]
        assert st == cols["aux_status"][i]
        assert np.array_equal(got, e.astype(got.dtype))


def test_whole_file_single_batch_matches_serial_scan(gpu):
    raw, bgzf = synth.short_read_bam(20000, seed=5, levels=(6, 6))
    r, _ = expected(bgzf)
    codec = gpu.CudaCodec(0)
    decoder = gpu.BamDecoder(0)
    batch = codec.inflate_batch_device(bgzf, r["spans"])
    rb = decoder.decode(batch, r["records_start"])
    assert len(rb) == len(r["columns"]["pos"])
    assert rb.tail() == r["tail"]
    assert np.array_equal(rb.column("record_offsets"), r["columns"]["record_offsets"])
