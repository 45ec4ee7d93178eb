"""Several files of different formats in one persistent inflate: a BAM, a BCF,
a bgzipped FASTQ and a bgzipped FASTA laid out back to back in device memory,
discovered and inflated as one population of members, then each decoded by its
format's decoder -- every file's bytes and columns equal to the oracle's
whole-file result, with and without the graph, across replays."""

import hashlib

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def _files():
    bam_raw, bam = synth.short_read_bam(8000, n_contigs=24, genome_len=3_100_000_000, seed=41, levels=(1, 6))
    bcf_raw, bcf = synth.bcf(1500, n_samples=40, seed=42)
    fq_raw, fq = synth.fastq(6000, seed=43)
    fa_raw, fa = synth.fasta(4, 1_500_000, 60, True, seed=44)
    return [("bam", bam_raw, bam), ("bcf", bcf_raw, bcf), ("fastq", fq_raw, fq), ("fasta", fa_raw, fa)]


def _bind(frt, torch, files, **kw):
    blob = np.concatenate([f[2] for f in files])
    dev = torch.from_numpy(blob).to("cuda")
    torch.cuda.synchronize()
    eng = frt.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream, **kw)
    fmt = {"bam": frt.Format.BAM, "bcf": frt.Format.BCF, "fastq": frt.Format.FASTQ, "fasta": frt.Format.FASTA}
    layout, at = [], 0
    for name, _, bgzf in files:
        layout.append((at, bgzf.size, fmt[name]))
        at += bgzf.size
    eng.bind_files(dev.data_ptr(), dev.numel(), layout)
    return eng, dev, layout


def _check(frt, eng, files, layout):
    assert eng.file_count() == len(files)
    inflated_ptr, inflated_len = eng.inflated_ptr()
    for i, (name, raw, bgzf) in enumerate(files):
        info = eng.file_info(i)
        assert info.compressed_bytes == bgzf.size
        assert info.inflated_bytes == raw.size, name
        res = eng.file_result(i)
        if name == "bam":
            want = oracle.decode_bam_file(bgzf)
            assert info.records == len(want["columns"]["pos"]) and info.tail == want["tail"]
            for k in ("ref_id", "pos", "flags", "seq_len", "cigar_start", "aux_start", "record_end", "aux_count",
                      "record_offsets"):
                assert np.array_equal(res.column(k), want["columns"][k]), k
            vo = oracle.virtual_offsets(want["spans"], want["offsets"][:-1], want["columns"]["record_offsets"])
            assert np.array_equal(res.column("virtual_offset"), vo)
        elif name == "bcf":
            rs, ns, nc = oracle.bcf_header(raw)
            want = oracle.bcf_decode(raw, rs, ns, nc)
            assert info.records == 1500 and info.tail == raw.size and info.proof == 0
            for k, _ in oracle.BCF_COLUMNS:
                assert np.array_equal(res.column(k), want["columns"][k]), k
            assert np.array_equal(res.column("record_offsets"), want["columns"]["record_offsets"])
        elif name == "fastq":
            want = oracle.fastq_decode(raw, 0)
            assert info.records == 6000 and info.tail == raw.size and info.proof == 0
            for k in ("record_offsets", "sequence_start", "plus_start", "quality_start", "sequence_len",
                      "record_end"):
                assert np.array_equal(res.column(k), want["columns"][k]), k
        else:
            want = oracle.fasta_compact(raw)
            assert info.records == len(want["record_offsets"]) and info.tail == want["sequence"].size
            seq = res.column("sequence")
            assert hashlib.sha256(seq.tobytes()).digest() == hashlib.sha256(want["sequence"].tobytes()).digest()
            for k in ("sequence_offsets", "sequence_lengths", "record_offsets"):
                assert np.array_equal(res.column(k), want[k]), k


@pytest.mark.parametrize("graph", [True, False])
def test_mixed_formats_in_one_inflate(gpu, graph):
    torch = pytest.importorskip("torch")
    files = _files()
    eng, dev, layout = _bind(gpu, torch, files, use_graph=graph)
    _check(gpu, eng, files, layout)
    for _ in range(2):
        eng.run()
        st = eng.finish()
        assert st.status == 0
        assert st.inflated_bytes == sum(f[1].size for f in files)
        _check(gpu, eng, files, layout)


def test_mixed_bind_rejects_a_bad_layout(gpu):
    torch = pytest.importorskip("torch")
    files = _files()[:2]
    blob = np.concatenate([f[2] for f in files])
    dev = torch.from_numpy(blob).to("cuda")
    eng = gpu.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream)
    with pytest.raises(gpu.InvalidArgument):
        eng.bind_files(dev.data_ptr(), dev.numel(), [(0, files[0][2].size, gpu.Format.BAM)])
    with pytest.raises(gpu.InvalidArgument):
        eng.bind_files(dev.data_ptr(), dev.numel(), [(0, files[0][2].size - 10, gpu.Format.BAM),
                                                     (files[0][2].size - 10, files[1][2].size + 10, gpu.Format.BCF)])


def test_mixed_reports_the_first_bad_member(gpu):
    torch = pytest.importorskip("torch")
    files = _files()
    eng, dev, layout = _bind(gpu, torch, files)
    # flip a CRC byte in the FASTQ file's second member; the error names that
    # member's offset in the bound buffer
    fq_off = layout[2][0]
    spans, _ = oracle.discover(files[2][2])
    second = int(spans[1]["compressed_offset"])
    crc_at = fq_off + int(spans[1]["payload_start"] + spans[1]["payload_len"])
    blob = dev.cpu().numpy()
    blob[crc_at] ^= 0xFF
    dev.copy_(torch.from_numpy(blob))
    torch.cuda.synchronize()
    with pytest.raises(gpu.ChecksumMismatch) as ei:
        eng.run()
        eng.finish()
    assert ei.value.offset == fq_off + second


def test_mixed_run_host_overlaps_the_upload_and_matches(gpu):
    """run_host on several files: the slices go up while the host plans, each
    group is inflated as it lands, then every file's decoder runs."""
    torch = pytest.importorskip("torch")
    files = _files()
    eng, dev, layout = _bind(gpu, torch, files)
    blob = np.concatenate([f[2] for f in files])
    pinned = torch.from_numpy(blob).pin_memory().numpy()
    for host in (pinned, pinned, np.array(blob)):
        dev.zero_()  # the run must bring the bytes itself
        torch.cuda.synchronize()
        st = eng.run_host(host)
        assert st.status == 0
        assert st.inflated_bytes == sum(f[1].size for f in files)
        _check(gpu, eng, files, layout)


def test_mixed_run_host_reports_the_first_bad_member(gpu):
    torch = pytest.importorskip("torch")
    files = _files()
    eng, dev, layout = _bind(gpu, torch, files)
    blob = np.concatenate([f[2] for f in files])
    fq_off = layout[2][0]
    spans, _ = oracle.discover(files[2][2])
    second = int(spans[1]["compressed_offset"])
    bad = blob.copy()
    bad[fq_off + int(spans[1]["payload_start"] + spans[1]["payload_len"])] ^= 0xFF
    with pytest.raises(gpu.ChecksumMismatch) as ei:
        eng.run_host(bad)
    assert ei.value.offset == fq_off + second
    st = eng.run_host(blob)  # and the good files afterwards are fine
    assert st.status == 0
    _check(gpu, eng, files, layout)
