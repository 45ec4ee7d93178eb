"""The record-field oracle (oracle/fields.py) pinned on the CPU: to the
assertions of the reference's own unit tests for aux lookup and long CIGARs
(crates/fritillaria-bam/src/columnar/record.rs:588-671) on the hand-built
records of tests/golden/fields_cases.npz, to what samtools printed for the
first 1,000 records of the reference's htslib_multiblock.bam
(tests/golden/fields_htslib.npz, from testdata/reads.sam), and to the C
oracle's aux walk."""

import struct
from pathlib import Path

import numpy as np
import pytest

from oracle import fields as of
from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def _decode(name):
    g = dict(np.load(GOLDEN / name))
    r = oracle.decode_bam_file(g["bgzf"])
    return g, r["inflated"], [int(o) for o in r["columns"]["record_offsets"]]


@pytest.fixture(scope="module")
def cases():
    g, buf, offs = _decode("fields_cases.npz")
    names = [of.payloads(buf, o)["name"] for o in offs]
    return buf, dict(zip(names, offs))


def test_long_cigar_resolves_from_cg(cases):
    buf, at = cases
    o = at[b"long_cigar"]
    assert of.has_long_cigar_placeholder(buf, o)
    assert of.layout(buf, o)["n_cigar"] == 2  # the stored CIGAR is the placeholder
    r = of.cigar_resolved(buf, o)
    assert r["status"] == 1 and r["ops"] == 70_000
    ops = np.frombuffer(bytes(buf[r["offset"]:r["offset"] + 4 * r["ops"]]), "<u4")
    assert ops[0] == (1 << 4) and ops[-1] == (1 << 4) and (ops == (1 << 4)).all()


def test_genuine_two_op_record_is_not_a_placeholder(cases):
    buf, at = cases
    o = at[b"genuine_sn"]
    assert not of.has_long_cigar_placeholder(buf, o)
    r = of.cigar_resolved(buf, o)
    assert r["status"] == 0 and r["ops"] == 2


def test_placeholder_without_cg_or_with_wrong_type_is_an_error(cases):
    buf, at = cases
    for name in (b"placeholder_no_cg", b"placeholder_cg_z"):
        assert of.has_long_cigar_placeholder(buf, at[name])
        assert of.cigar_resolved(buf, at[name])["status"] == 2


def test_aux_lookup_finds_a_tag_and_reports_absence(cases):
    buf, at = cases
    o = at[b"read1"]
    nm = of.aux_get(buf, o, b"NM")
    assert (nm["status"], nm["type"], nm["value"]) == (of.PRESENT, ord("C"), 7)
    xz = of.aux_get(buf, o, b"XZ")
    assert xz["status"] == of.PRESENT and bytes(buf[xz["offset"]:xz["offset"] + xz["count"]]) == b"hello"
    assert of.aux_get(buf, o, b"ZZ")["status"] == of.ABSENT
    assert len(of.aux_fields(buf, o)[0]) == 2


def test_every_scalar_type_and_array_subtype(cases):
    buf, at = cases
    o = at[b"every_type"]
    want = {b"Ac": ("A", ord("x")), b"cc": ("c", -5), b"CC": ("C", 200), b"ss": ("s", -300), b"SS": ("S", 60000),
            b"ii": ("i", -70000), b"II": ("I", 3_000_000_000), b"ff": ("f", struct.unpack("<I", struct.pack("<f", 1.5))[0])}
    for tag, (ty, value) in want.items():
        v = of.aux_get(buf, o, tag)
        assert (v["status"], chr(v["type"]), v["value"], v["count"]) == (of.PRESENT, ty, value, 1), tag
    z = of.aux_get(buf, o, b"ZZ")
    assert bytes(buf[z["offset"]:z["offset"] + z["count"]]) == b"text"
    h = of.aux_get(buf, o, b"HH")
    assert chr(h["type"]) == "H" and bytes(buf[h["offset"]:h["offset"] + h["count"]]) == b"1AE3"
    arrays = {b"Bc": ("c", [-1, 2], "<b"), b"BC": ("C", [1, 2, 3], "<B"), b"Bs": ("s", [-7, 8], "<h"),
              b"BS": ("S", [65535], "<H"), b"Bi": ("i", [-1, 1 << 30], "<i"), b"BI": ("I", [4_000_000_000], "<I"),
              b"Bf": ("f", [0.25, -2.0], "<f"), b"Bz": ("C", [], "<B")}
    for tag, (sub, values, fmt) in arrays.items():
        v = of.aux_get(buf, o, tag)
        assert (chr(v["type"]), chr(v["subtype"]), v["count"]) == ("B", sub, len(values)), tag
        w = struct.calcsize(fmt)
        got = [struct.unpack_from(fmt, bytes(buf[v["offset"] + w * k:v["offset"] + w * (k + 1)]))[0]
               for k in range(len(values))]
        assert got == values, tag


def test_first_of_a_repeated_tag_and_malformed_blocks(cases):
    buf, at = cases
    assert of.aux_get(buf, at[b"repeated_tag"], b"NM")["value"] == 1
    o = at[b"malformed_aux"]
    fields, bad = of.aux_fields(buf, o)
    assert bad and [f[0] for f in fields] == [b"XA"]
    assert of.aux_get(buf, o, b"XA")["value"] == 5
    assert of.aux_get(buf, o, b"YB")["status"] == of.MALFORMED
    assert of.aux_get(buf, o, b"ZZ")["status"] == of.MALFORMED


def test_sequences(cases):
    buf, at = cases
    assert of.decode_sequence(buf, at[b"no_sequence"]) == b""
    assert of.decode_sequence(buf, at[b"odd_length"]) == b"KDBN=ACGT"
    assert of.decode_sequence(buf, at[b"read1"]) == b"ACGT"


def test_oracle_matches_samtools_on_the_htslib_fixture():
    g, buf, offs = _decode("fields_htslib.npz")
    names, cigars = g["name"].tobytes().split(b"\n"), g["cigar"].tobytes().decode().split("\n")
    seqs, quals = g["seq"].tobytes().split(b"\n"), g["qual"].tobytes().split(b"\n")
    assert len(offs) == len(names) == 1000
    for i, o in enumerate(offs):
        p = of.payloads(buf, o)
        assert p["name"] == names[i]
        assert of.cigar_text(buf, o) == cigars[i]
        assert of.decode_sequence(buf, o) == seqs[i]
        assert bytes(q + 33 for q in p["quality"]) == quals[i]
        nm = of.aux_get(buf, o, b"NM")
        assert nm["status"] == of.PRESENT and nm["value"] == g["nm"][i]
        L = of.layout(buf, o)
        flag, = struct.unpack_from("<H", bytes(buf[o + 18:o + 20]))
        pos, = struct.unpack_from("<i", bytes(buf[o + 8:o + 12]))
        assert (flag, pos + 1, buf[o + 13]) == (g["flag"][i], g["pos"][i], g["mapq"][i])
        assert L["record_end"] > L["aux_start"]


def test_aux_walk_matches_the_c_oracle():
    for name in ("fields_cases.npz", "fields_htslib.npz"):
        g, buf, offs = _decode(name)
        for o in offs[:400]:
            L = of.layout(buf, o)
            entries, status = oracle.bam_aux(buf, o, L["aux_start"], L["record_end"])
            fields, bad = of.aux_fields(buf, o)
            assert len(entries) == len(fields) and bool(status) == bad
