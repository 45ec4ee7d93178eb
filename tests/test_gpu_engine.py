"""The batched, device-resident form against the oracle: whole file in HBM,
device discovery, size-sorted queue, persistent inflate, graph replay."""

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

COLS = ["ref_id", "pos", "flags", "mapq", "seq_len", "mate_ref_id", "mate_pos", "tlen", "record_offsets",
        "cigar_start", "sequence_start", "quality_start", "aux_start", "record_end", "bin", "n_cigar", "name_len",
        "aux_count", "aux_status"]


def _device_copy(torch, data):
    t = torch.from_numpy(np.ascontiguousarray(data)).to("cuda")
    torch.cuda.synchronize()
    return t


def run_engine(frt, torch, bgzf, **kw):
    dev = _device_copy(torch, bgzf)
    eng = frt.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream, **kw)
    eng.bind_bam(dev.data_ptr(), dev.numel())
    eng.run()
    st = eng.finish()
    return eng, st, dev


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("sort", [True, False])
def test_engine_matches_oracle(gpu, graph, sort):
    torch = pytest.importorskip("torch")
    raw, bgzf = synth.short_read_bam(30000, n_contigs=24, genome_len=3_100_000_000, seed=17, levels=(1, 6))
    r = oracle.decode_bam_file(bgzf)
    eng, st, dev = run_engine(gpu, torch, bgzf, use_graph=graph, sort_queue=sort)
    assert st.status == 0
    assert st.records == len(r["columns"]["pos"])
    assert st.inflated_bytes == r["inflated"].size
    assert st.tail == r["tail"]
    for k in COLS:
        assert np.array_equal(eng.column(k), r["columns"][k]), k
    vo = oracle.virtual_offsets(r["spans"], r["offsets"][:-1], r["columns"]["record_offsets"])
    assert np.array_equal(eng.column("virtual_offset"), vo)
    # replays give the same answer
    for _ in range(2):
        eng.run()
        st2 = eng.finish()
        assert st2.records == st.records and st2.status == 0
    assert np.array_equal(eng.column("pos"), r["columns"]["pos"])


def test_engine_ultra_long(gpu):
    torch = pytest.importorskip("torch")
    raw, bgzf = synth.ultra_long_bam(40, n_long_extra=2, seed=6)
    r = oracle.decode_bam_file(bgzf)
    eng, st, dev = run_engine(gpu, torch, bgzf)
    assert st.status == 0 and st.records == len(r["columns"]["pos"])
    for k in COLS:
        assert np.array_equal(eng.column(k), r["columns"][k]), k


def test_engine_reports_first_bad_member(gpu):
    torch = pytest.importorskip("torch")
    raw, bgzf = synth.short_read_bam(8000, seed=2)
    spans, _ = oracle.discover(bgzf)
    bad = bgzf.copy()
    k = 3
    end = int(spans[k]["payload_start"] + spans[k]["payload_len"])
    bad[end] ^= 0xff  # trailer CRC of member 3
    eng, st, dev = run_engine(gpu, torch, bgzf)
    assert st.status == 0
    dev.copy_(torch.from_numpy(bad).to("cuda"))
    torch.cuda.synchronize()
    eng.run()
    with pytest.raises(gpu.ChecksumMismatch) as ei:
        eng.finish()
    assert ei.value.offset == int(spans[k]["compressed_offset"])


@pytest.mark.parametrize("kind", ["short", "ultra_long"])
def test_run_host_overlaps_the_upload_and_matches(gpu, kind):
    """run_host uploads in slices while the host plans, inflating each group of
    members as its bytes land: the columns and stats equal the single-launch
    run's, replays included."""
    torch = pytest.importorskip("torch")
    if kind == "short":
        _, bgzf = synth.short_read_bam(40000, n_contigs=24, genome_len=3_100_000_000, seed=23, levels=(1, 6))
    else:
        _, bgzf = synth.ultra_long_bam(60, n_long_extra=2, seed=23)
    eng, st, dev = run_engine(gpu, torch, bgzf)
    want = {k: eng.column(k) for k in COLS + ["virtual_offset", "aux_entries"]}
    host = torch.from_numpy(bgzf).pin_memory().numpy()
    for _ in range(3):
        st2 = eng.run_host(host)
        assert (st2.status, st2.records, st2.members, st2.inflated_bytes, st2.tail, st2.aux_fields) == (
            st.status, st.records, st.members, st.inflated_bytes, st.tail, st.aux_fields)
        for k, v in want.items():
            assert np.array_equal(eng.column(k), v), k
    # pageable host memory too (no overlap, same answer)
    st3 = eng.run_host(np.array(bgzf))
    assert st3.records == st.records and np.array_equal(eng.column("pos"), want["pos"])


def test_run_host_reports_the_first_bad_member(gpu):
    torch = pytest.importorskip("torch")
    _, bgzf = synth.short_read_bam(30000, seed=4)
    spans, _ = oracle.discover(bgzf)
    eng, st, dev = run_engine(gpu, torch, bgzf)
    assert st.status == 0
    for k in (2, len(spans) // 2, len(spans) - 3):  # members in different upload groups
        bad = bgzf.copy()
        end = int(spans[k]["payload_start"] + spans[k]["payload_len"])
        bad[end] ^= 0xff  # that member's trailer CRC
        bad[int(spans[len(spans) - 2]["payload_start"] + spans[len(spans) - 2]["payload_len"])] ^= 0xff  # a later one
        with pytest.raises(gpu.ChecksumMismatch) as ei:
            eng.run_host(bad)
        assert ei.value.offset == int(spans[k]["compressed_offset"])
    # a file the plan cannot describe (a member header cut) takes the single-launch path's error
    cut = bgzf.copy()
    cut[int(spans[5]["compressed_offset"]) + 12] ^= 0x55  # corrupt the BC subfield id of member 5
    with pytest.raises(gpu.FrtError):
        eng.run_host(cut)
    st4 = eng.run_host(bgzf)  # and a good file afterwards is fine
    assert st4.status == 0 and st4.records == st.records
