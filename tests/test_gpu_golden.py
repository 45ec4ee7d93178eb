"""The CUDA path against the golden vectors of tests/golden/, which hold the
outputs of the reference's own kernels (inflate.cu, bam_decode.cu) on the
same inputs: member bytes (SHA-256), CRC-32, record offsets, tail and the 13
per-record columns of DeviceColumns -- through the codec, the reader/decoder
loop at several batch sizes, and the batched engine."""

import hashlib
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("fields_", "text_")))  # record-field and text inputs have their own tests
BAM_CASES = [c for c in CASES if c.startswith("bam_")]
REF_COLS = ["ref_id", "pos", "flags", "mapq", "seq_len", "mate_ref_id", "mate_pos", "tlen", "cigar_start",
            "sequence_start", "quality_start", "aux_start", "record_end"]


def golden(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def spans_of(frt, g):
    s = np.zeros(len(g["span_isize"]), dtype=frt.SPAN_DTYPE)
    for f in ("compressed_offset", "payload_start", "payload_len", "isize", "crc32"):
        s[f] = g[f"span_{f}"]
    return s


@pytest.mark.parametrize("case", CASES)
def test_codec_inflates_the_golden_members(gpu, case):
    g = golden(case)
    codec = gpu.CudaCodec(0)
    batch = codec.inflate_batch_device(g["bgzf"], spans_of(gpu, g))
    data = batch.to_host()
    offs = batch.offsets()
    assert data.size == int(g["inflated_len"])
    for i in range(len(offs) - 1):
        assert hashlib.sha256(data[offs[i]:offs[i + 1]].tobytes()).digest() == g["member_sha256"][i], f"member {i}"


@pytest.mark.parametrize("case", BAM_CASES)
@pytest.mark.parametrize("blocks", [1, 3, 256])
def test_reader_and_decoder_match_the_reference_kernels(gpu, case, blocks):
    g = golden(case)
    codec = gpu.CudaCodec(0)
    decoder = gpu.BamDecoder(0)
    reader = gpu.DeviceBgzfReader(g["bgzf"], codec, blocks_per_batch=blocks)
    got = {k: [] for k in REF_COLS + ["record_offsets"]}
    header = None
    base = 0  # inflated offset of the current batch's first byte
    tail = 0
    while (item := reader.next_batch()) is not None:
        if header is None:
            try:
                header = gpu.parse_header(item.data.to_host())
            except gpu.Malformed:
                reader.carry_from(0)
                continue
            begin = header[0]
        else:
            begin = item.start
        rb = decoder.decode(item.data, begin)
        for k in REF_COLS:
            got[k].append(rb.column(k))
        got["record_offsets"].append(rb.column("record_offsets").astype(np.uint64))
        tail = rb.tail()
        # the batch starts at the compressed member holding `tail` next time;
        # translate in-batch offsets to whole-file offsets with the batch's
        # first member (compressed offsets are unique per member)
        co = item.data.compressed_offsets()
        first = int(np.searchsorted(g["span_compressed_offset"], co[0]))
        base_file = int(np.concatenate([[0], np.cumsum(g["span_isize"].astype(np.uint64))])[first])
        got["record_offsets"][-1] = got["record_offsets"][-1] + np.uint64(base_file)
        tail_file = base_file + tail
        rb.free()
        reader.carry_from(tail)
    for k in REF_COLS:
        assert np.array_equal(np.concatenate(got[k]), g[f"col_{k}"]), k
    assert np.array_equal(np.concatenate(got["record_offsets"]), g["record_offsets"])
    assert tail_file == int(g["tail"])


@pytest.mark.parametrize("case", BAM_CASES)
def test_engine_matches_the_reference_kernels(gpu, case):
    torch = pytest.importorskip("torch")
    g = golden(case)
    dev = torch.from_numpy(np.ascontiguousarray(g["bgzf"])).to("cuda")
    torch.cuda.synchronize()
    eng = gpu.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream)
    eng.bind_bam(dev.data_ptr(), dev.numel())
    eng.run()
    st = eng.finish()
    assert st.status == 0
    assert st.records == len(g["record_offsets"]) and st.tail == int(g["tail"])
    assert np.array_equal(eng.column("record_offsets"), g["record_offsets"])
    for k in REF_COLS:
        assert np.array_equal(eng.column(k), g[f"col_{k}"]), k
