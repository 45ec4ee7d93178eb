"""Inflate tunings on the GB300: every compiled variant (table roots, window
buffer, match queue) at several CTA widths and queue chunks gives the same
bytes, CRCs and columns -- on the golden members of the reference's kernels
and on a synthetic BAM through the batched engine -- invalid tunings are
refused, and the autotuner times candidates, caches the winner as JSON and
reads it back."""

import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
COLS = ["ref_id", "pos", "flags", "mapq", "seq_len", "mate_ref_id", "mate_pos", "tlen", "record_offsets",
        "cigar_start", "sequence_start", "quality_start", "aux_start", "record_end", "aux_count"]


@pytest.fixture
def frt(gpu):
    """The library, with the process default tuning put back afterwards."""
    saved = gpu.default_tuning()
    yield gpu
    gpu.set_default_tuning(saved)


def _tunings(frt):
    out = []
    for v in range(len(frt.inflate_variants())):
        for w, chunk in ((2, 1), (4, 2)):
            out.append(frt.InflateTuning(v, w, 0, chunk))
    return out


def _spans(frt, g):
    s = np.zeros(len(g["span_isize"]), dtype=frt.SPAN_DTYPE)
    for f in ("compressed_offset", "payload_start", "payload_len", "isize", "crc32"):
        s[f] = g[f"span_{f}"]
    return s


def test_every_variant_inflates_the_golden_members(frt):
    cases = sorted(p for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("fields_", "text_")))
    assert cases
    for t in _tunings(frt):
        frt.set_default_tuning(t)
        codec = frt.CudaCodec(0)  # a codec takes the default tuning when made
        for case in cases:
            g = dict(np.load(case))
            batch = codec.inflate_batch_device(g["bgzf"], _spans(frt, g))
            data, offs = batch.to_host(), batch.offsets()
            assert data.size == int(g["inflated_len"]), (t.as_dict(), case.stem)
            for i in range(len(offs) - 1):
                got = hashlib.sha256(data[offs[i]:offs[i + 1]].tobytes()).digest()
                assert got == g["member_sha256"][i], (t.as_dict(), case.stem, i)


def test_small_launches_take_the_spread_variant(frt):
    """A launch of fewer members than one wave of one-warp CTAs holds runs one
    warp per CTA with the tuning's spread variant: every one-chain variant in
    that role gives the golden members exactly, under a base variant of
    another shape."""
    cases = sorted(p for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("fields_", "text_")))
    one_chain = [i for i, v in enumerate(frt.inflate_variants()) if v["chains"] == 1]
    for sv in one_chain:
        base = one_chain[(one_chain.index(sv) + 3) % len(one_chain)]
        t = frt.InflateTuning(base, 4, 0, 2, spread_variant=sv)
        frt.set_default_tuning(t)
        codec = frt.CudaCodec(0)
        for case in cases:
            g = dict(np.load(case))
            batch = codec.inflate_batch_device(g["bgzf"], _spans(frt, g))
            data, offs = batch.to_host(), batch.offsets()
            assert data.size == int(g["inflated_len"]), (t.as_dict(), case.stem)
            for i in range(len(offs) - 1):
                got = hashlib.sha256(data[offs[i]:offs[i + 1]].tobytes()).digest()
                assert got == g["member_sha256"][i], (t.as_dict(), case.stem, i)


@pytest.fixture(scope="module")
def bam():
    raw, bgzf = synth.short_read_bam(12000, n_contigs=24, genome_len=3_100_000_000, seed=33, levels=(1, 6))
    return bgzf, oracle.decode_bam_file(bgzf)


def _engine(frt, torch, bgzf):
    dev = torch.from_numpy(np.ascontiguousarray(bgzf)).to("cuda")
    torch.cuda.synchronize()
    eng = frt.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream)
    eng.bind_bam(dev.data_ptr(), dev.numel())
    return eng, dev


def test_every_tuning_gives_the_same_columns(frt, bam):
    torch = pytest.importorskip("torch")
    bgzf, r = bam
    eng, dev = _engine(frt, torch, bgzf)
    want_inflated = r["inflated"]
    for t in _tunings(frt):
        eng.set_tuning(t)
        assert eng.tuning.as_dict() == t.as_dict()
        eng.run()
        st = eng.finish()
        assert st.status == 0 and st.records == len(r["columns"]["pos"]), t.as_dict()
        assert np.array_equal(eng.inflated(), want_inflated), t.as_dict()
        for k in COLS:
            assert np.array_equal(eng.column(k), r["columns"][k]), (t.as_dict(), k)


def test_invalid_tunings_are_refused(frt, bam):
    torch = pytest.importorskip("torch")
    eng, dev = _engine(frt, torch, bam[0])
    n = len(frt.inflate_variants())
    multi = next(i for i, v in enumerate(frt.inflate_variants()) if v["chains"] > 1)
    for bad in (frt.InflateTuning(n, 3, 0, 1), frt.InflateTuning(-1, 3, 0, 1), frt.InflateTuning(0, 0, 0, 1),
                frt.InflateTuning(0, 9, 0, 1), frt.InflateTuning(0, 3, 0, 0), frt.InflateTuning(0, 3, 0, 65),
                frt.InflateTuning(0, 3, -1, 1), frt.InflateTuning(0, 3, 0, 1, spread_variant=n),
                frt.InflateTuning(0, 3, 0, 1, spread_variant=-2), frt.InflateTuning(0, 3, 0, 1, spread_variant=multi)):
        with pytest.raises(frt.InvalidArgument):
            eng.set_tuning(bad)
        with pytest.raises(frt.InvalidArgument):
            frt.set_default_tuning(bad)
        with pytest.raises(frt.InvalidArgument):
            eng.time_inflate(bad)
    # a refused tuning leaves the engine as it was
    eng.run()
    assert eng.finish().status == 0


def test_time_inflate_reports_the_sample(frt, bam):
    torch = pytest.importorskip("torch")
    bgzf, r = bam
    eng, dev = _engine(frt, torch, bgzf)
    spans = r["spans"]
    ms, nbytes = eng.time_inflate(frt.InflateTuning(0, 3, 0, 1), members=40, reps=2)
    assert ms > 0
    assert nbytes == int(spans["isize"][:40].sum())
    ms, nbytes = eng.time_inflate(frt.InflateTuning(1, 4, 0, 2), members=0, reps=1)
    assert nbytes == r["inflated"].size
    # timing leaves the next run exact
    eng.run()
    st = eng.finish()
    assert st.status == 0
    assert np.array_equal(eng.column("pos"), r["columns"]["pos"])


def test_autotune_caches_and_reads_back(frt, bam, tmp_path):
    torch = pytest.importorskip("torch")
    bgzf, r = bam
    eng, dev = _engine(frt, torch, bgzf)
    cache = tmp_path / "tuning.json"
    first = eng.autotune(cache)
    assert not first["from_cache"]
    assert first["candidates"] >= len(frt.inflate_variants())
    assert first["sample_gbs"] > 0
    doc = json.loads(cache.read_text())
    entry = doc["entries"][first["key"]]
    assert entry["variant"] == first["variant"]
    assert entry["warps_per_cta"] == first["warps_per_cta"]
    assert entry["queue_chunk"] == first["queue_chunk"]
    shape = frt.inflate_variants()[first["variant"]]
    assert (entry["lit_bits"], entry["window"]) == (shape["lit_bits"], shape["window"])
    # the small-launch variant is a one-chain variant, timed and cached with the rest
    assert first["spread_variant"] >= 0 and entry["spread_variant"] == first["spread_variant"]
    assert frt.inflate_variants()[first["spread_variant"]]["chains"] == 1
    # the winner is the engine's tuning and the process default
    assert eng.tuning.as_dict() == {k: first[k] for k in ("variant", "warps_per_cta", "ctas_per_sm", "queue_chunk",
                                                          "spread_variant")}
    assert frt.default_tuning().as_dict() == eng.tuning.as_dict()
    eng.run()
    st = eng.finish()
    assert st.status == 0 and np.array_equal(eng.column("pos"), r["columns"]["pos"])
    # a second engine on the same workload reads the cache
    eng2, dev2 = _engine(frt, torch, bgzf)
    again = eng2.autotune(cache)
    assert again["from_cache"] and again["key"] == first["key"]
    assert eng2.tuning.as_dict() == eng.tuning.as_dict()
    # other entries survive a forced re-tune
    doc["entries"]["another device|sm1"] = dict(entry)
    cache.write_text(json.dumps(doc))
    forced = eng2.autotune(cache, force=True)
    assert not forced["from_cache"]
    doc2 = json.loads(cache.read_text())
    assert "another device|sm1" in doc2["entries"] and first["key"] in doc2["entries"]
    # an entry without a small-launch variant is completed on a hit and written back
    del doc2["entries"][first["key"]]["spread_variant"]
    cache.write_text(json.dumps(doc2))
    hit = eng2.autotune(cache)
    assert hit["from_cache"] and hit["spread_variant"] >= 0
    assert json.loads(cache.read_text())["entries"][first["key"]]["spread_variant"] == hit["spread_variant"]
    # a cache that names a variant of another shape is not trusted
    doc2["entries"][first["key"]]["lit_bits"] = 3
    cache.write_text(json.dumps(doc2))
    assert not eng2.autotune(cache)["from_cache"]


def _strategy_file():
    """Members of every zlib strategy and level over varied payloads, with
    stored, fixed and dynamic blocks, empty members and the EOF block."""
    from test_gpu_inflate import build_file

    return build_file(np.random.default_rng(5))


def _tampered(what: str):
    from test_gpu_inflate import member

    rng = np.random.default_rng(11)
    parts = [member(bytes(rng.integers(65, 70, 20000, dtype=np.uint8)), 6) for _ in range(5)]
    bad = bytearray(parts[3])
    if what == "crc":
        bad[-8] ^= 0xFF
    else:
        bad[40] ^= 0x55
    parts[3] = bytes(bad)
    return np.frombuffer(b"".join(parts), np.uint8)


def test_every_variant_inflates_every_block_kind(frt):
    """Plain form of every variant (one chain or several per warp) on stored,
    fixed and dynamic blocks of every zlib strategy, empty members and the EOF
    block: the oracle's bytes, and a tampered member fails with the oracle's
    error variant and member offset."""
    data = _strategy_file()
    spans, _ = oracle.discover(data)
    want, offs = oracle.inflate_batch(data, spans)
    for what in ("crc", "payload"):
        bad = _tampered(what)
        bspans, _ = oracle.discover(bad)
        with pytest.raises(oracle.OracleError) as oe:
            oracle.inflate_batch(bad, bspans)
        for t in _tunings(frt):
            frt.set_default_tuning(t)
            codec = frt.CudaCodec(0)
            if what == "crc":
                got, goffs = codec.inflate_batch(data, spans)
                assert np.array_equal(goffs, offs) and np.array_equal(got, want), t.as_dict()
            with pytest.raises(frt.FrtError) as ei:
                codec.inflate_batch_device(bad, bspans)
            assert (ei.value.code, ei.value.offset) == (oe.value.code, oe.value.offset), (t.as_dict(), what)


def test_every_variant_reports_the_first_bad_member_in_the_engine(frt, bam):
    """The batched (persistent) form of every variant: a tampered trailer or
    payload is reported for the first failing member in file order."""
    torch = pytest.importorskip("torch")
    bgzf, r = bam
    spans = r["spans"]
    eng, dev = _engine(frt, torch, bgzf)  # bound on good bytes, then overwritten
    for k, flip in ((5, "crc"), (2, "payload")):
        bad = bgzf.copy()
        if flip == "crc":
            bad[int(spans[k]["payload_start"] + spans[k]["payload_len"])] ^= 0xFF
        else:
            bad[int(spans[k]["payload_start"]) + 30] ^= 0x55
        with pytest.raises(oracle.OracleError) as oe:
            oracle.inflate_batch(bad, oracle.discover(bad)[0])
        dev.copy_(torch.from_numpy(bad).to("cuda"))
        torch.cuda.synchronize()
        for t in _tunings(frt):
            eng.set_tuning(t)
            eng.run()
            with pytest.raises(frt.FrtError) as ei:
                eng.finish()
            assert ei.value.code == oe.value.code and ei.value.offset == int(spans[k]["compressed_offset"]), \
                (t.as_dict(), flip)
