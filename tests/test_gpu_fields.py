"""Record fields on the GB300 against the oracle (oracle/fields.py, pinned in
tests/test_oracle_fields.py): one aux tag for every record (Record::aux_get),
CIGARs resolved through CG (Record::cigar_resolved), bases unpacked
(decode_sequence) and the payloads compacted (the Record accessors), through a
decoded record batch and through the batched engine, on the hand-built cases,
on the reference's samtools-written fixture (also against samtools' own text),
and on synthetic short and ultra-long reads."""

from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import fields as of

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
TAGS_CASES = [b"NM", b"XZ", b"ZZ", b"CG", b"Ac", b"cc", b"CC", b"ss", b"SS", b"ii", b"II", b"ff", b"HH", b"Bc",
              b"BC", b"Bs", b"BS", b"Bi", b"BI", b"Bf", b"Bz", b"XA", b"YB", b"RG"]


def decode_one_batch(frt, bgzf):
    """The whole file as one inflate batch and its record batch."""
    codec = frt.CudaCodec(0)
    reader = frt.DeviceBgzfReader(bgzf, codec, blocks_per_batch=1 << 16)
    item = reader.next_batch()
    buf = item.data.to_host()
    start, _ = frt.parse_header(buf)
    rb = frt.BamDecoder(0).decode(item.data, start)
    return rb, buf, rb.column("record_offsets"), item


def check_aux(res, buf, offs, tag):
    got = res.to_host()
    assert len(res) == len(offs)
    for i, o in enumerate(offs):
        want = of.aux_get(buf, int(o), tag)
        row = {k: int(got[k][i]) for k in ("status", "type", "subtype", "count", "value", "offset")}
        assert row == want, (tag, i, row, want)


def check_cigar(res, buf, offs):
    got = res.to_host()
    for i, o in enumerate(offs):
        want = of.cigar_resolved(buf, int(o))
        row = {"status": int(got["status"][i]), "offset": int(got["offset"][i]), "ops": int(got["ops"][i])}
        assert row == want, (i, row, want)


def check_bases(res, buf, offs):
    got = res.to_host()
    assert got["offsets"][0] == 0 and len(got["offsets"]) == len(offs) + 1
    assert res.total_bases() == got["offsets"][-1] == got["data"].size
    data = got["data"].tobytes()
    for i, o in enumerate(offs):
        assert data[got["offsets"][i]:got["offsets"][i + 1]] == of.decode_sequence(buf, int(o)), i


def check_compact(res, buf, offs):
    got = res.to_host()
    for part, cw in (("name", 1), ("cigar", 4), ("sequence", 1), ("quality", 1), ("aux", 1)):
        o_ = got[f"{part}_offsets"]
        data = got[f"{part}_data"].tobytes()
        assert o_[0] == 0 and o_[-1] == len(data), part
        for i, o in enumerate(offs):
            assert data[o_[i]:o_[i + 1]] == of.payloads(buf, int(o))[part], (part, i)


def test_cases_through_the_decoder(gpu):
    g = dict(np.load(GOLDEN / "fields_cases.npz"))
    rb, buf, offs, _ = decode_one_batch(gpu, g["bgzf"])
    assert len(offs) == 210
    for tag in TAGS_CASES:
        check_aux(rb.aux_lookup(tag), buf, offs, tag)
    cig = rb.cigar_resolved()
    check_cigar(cig, buf, offs)
    st = cig.column("status")
    assert st[0] == 1 and cig.column("ops")[0] == 70_000 and st[1] == 0 and st[2] == 2 and st[3] == 2
    check_bases(rb.unpack_sequences(), buf, offs)
    check_compact(rb.compact(), buf, offs)


def test_htslib_fixture_matches_samtools(gpu):
    g = dict(np.load(GOLDEN / "fields_htslib.npz"))
    rb, buf, offs, _ = decode_one_batch(gpu, g["bgzf"])
    assert len(offs) == 1000
    for tag in (b"NM", b"XX"):
        check_aux(rb.aux_lookup(tag), buf, offs, tag)
    nm = rb.aux_lookup("NM").to_host()
    assert (nm["status"] == 1).all() and np.array_equal(nm["value"], g["nm"])
    bases = rb.unpack_sequences().to_host()
    seqs = g["seq"].tobytes().split(b"\n")
    data = bases["data"].tobytes()
    assert [data[bases["offsets"][i]:bases["offsets"][i + 1]] for i in range(1000)] == seqs
    comp = rb.compact().to_host()
    names, quals = g["name"].tobytes().split(b"\n"), g["qual"].tobytes().split(b"\n")
    nd, qd = comp["name_data"].tobytes(), comp["quality_data"].tobytes()
    no, qo = comp["name_offsets"], comp["quality_offsets"]
    assert [nd[no[i]:no[i + 1]] for i in range(1000)] == names
    assert [bytes(b + 33 for b in qd[qo[i]:qo[i + 1]]) for i in range(1000)] == quals
    cig = rb.cigar_resolved().to_host()
    assert (cig["status"] == 0).all()
    texts = g["cigar"].tobytes().decode().split("\n")
    for i in range(1000):
        ops = np.frombuffer(buf[cig["offset"][i]:cig["offset"][i] + 4 * cig["ops"][i]].tobytes(), "<u4")
        assert "".join(f"{op >> 4}{'MIDNSHP=X'[op & 15]}" for op in ops) == texts[i]


@pytest.mark.parametrize("kind", ["short", "ultra_long", "ultra_long_many"])
def test_synthetic_reads(gpu, kind):
    if kind == "short":
        _, bgzf = synth.short_read_bam(6000, seed=8, levels=(1, 6))
        tags = [b"NM", b"MD", b"RG", b"XX"]
    elif kind == "ultra_long_many":
        # more records than one copy CTA takes, reads above and below the
        # length the long-record kernel takes over at, in one batch
        _, bgzf = synth.ultra_long_bam(1200, n_long_extra=2, seed=9, levels=(1, 1))
        tags = [b"MM", b"qs"]
    else:
        _, bgzf = synth.ultra_long_bam(30, n_long_extra=1, seed=8)
        tags = [b"MM", b"ML", b"qs", b"ch", b"NM"]
    rb, buf, offs, _ = decode_one_batch(gpu, bgzf)
    for tag in tags:
        check_aux(rb.aux_lookup(tag), buf, offs, tag)
    check_cigar(rb.cigar_resolved(), buf, offs)
    check_bases(rb.unpack_sequences(), buf, offs)
    check_compact(rb.compact(), buf, offs)


def test_engine_forms(gpu):
    torch = pytest.importorskip("torch")
    g = dict(np.load(GOLDEN / "fields_cases.npz"))
    dev = torch.from_numpy(np.ascontiguousarray(g["bgzf"])).to("cuda")
    torch.cuda.synchronize()
    eng = gpu.BatchEngine(0, stream=torch.cuda.current_stream().cuda_stream)
    eng.bind_bam(dev.data_ptr(), dev.numel())
    eng.run()
    assert eng.finish().status == 0
    buf, offs = eng.inflated(), eng.column("record_offsets")
    assert len(offs) == 210
    for tag in (b"CG", b"NM", b"ff", b"Bf", b"YB"):
        check_aux(eng.aux_lookup(tag), buf, offs, tag)
    check_cigar(eng.cigar_resolved(), buf, offs)
    check_bases(eng.unpack_sequences(), buf, offs)
    check_compact(eng.compact(), buf, offs)


def test_a_compacted_batch_outlives_its_source(gpu):
    g = dict(np.load(GOLDEN / "fields_cases.npz"))
    rb, buf, offs, item = decode_one_batch(gpu, g["bgzf"])
    comp = rb.compact()
    aux = rb.aux_lookup("NM")
    want = [of.payloads(buf, int(o))["aux"] for o in offs]
    del rb, item  # the record batch and its inflate batch go; the results stay valid
    import gc
    gc.collect()
    got = comp.to_host()
    data = got["aux_data"].tobytes()
    assert [data[got["aux_offsets"][i]:got["aux_offsets"][i + 1]] for i in range(len(offs))] == want
    assert aux.column("status")[4] == 1 and aux.column("value")[4] == 7


def test_argument_errors(gpu):
    g = dict(np.load(GOLDEN / "fields_cases.npz"))
    rb, _, _, _ = decode_one_batch(gpu, g["bgzf"])
    with pytest.raises(gpu.InvalidArgument):
        rb.aux_lookup("N")
    with pytest.raises(gpu.InvalidArgument):
        rb.aux_lookup(b"NMX")
