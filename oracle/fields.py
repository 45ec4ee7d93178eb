"""Record fields, restated on the CPU -- test infrastructure: the oracle for
the device record-field kernels, never called by the product.

Follows the reference's host accessors for one BAM record:
  * layout and payloads: Record::name / cigar_raw / sequence_packed /
    qualities / aux_raw (crates/fritillaria-bam/src/columnar/record.rs:222-270),
    the name without its trailing NUL (record.rs:227-228);
  * aux fields: Fields and read_value / read_array
    (crates/fritillaria-bam/src/columnar/aux.rs:301-479), fused at the first
    malformed field; Record::aux_get (record.rs:286-294) returns the first
    field with the tag, and an error when the walk fails before it;
  * has_long_cigar_placeholder / cigar_resolved (record.rs:316-357);
  * decode_sequence with BASES = "=ACMGRSVTWYHKDBN", high nibble first
    (crates/fritillaria-bam/src/columnar/seq.rs).
"""

import struct

BASES = b"=ACMGRSVTWYHKDBN"
CIGAR_OPS = b"MIDNSHP=X"
WIDTH = {ord("c"): 1, ord("C"): 1, ord("s"): 2, ord("S"): 2, ord("i"): 4, ord("I"): 4, ord("f"): 4}
SCALAR = {ord("A"): 1, ord("c"): 1, ord("C"): 1, ord("s"): 2, ord("S"): 2, ord("i"): 4, ord("I"): 4, ord("f"): 4}
HEX = set(b"0123456789abcdefABCDEF")

ABSENT, PRESENT, MALFORMED = 0, 1, 2


def layout(buf, off: int) -> dict:
    """Field boundaries of the record at `off` (record-relative offsets)."""
    b = memoryview(buf)
    block_size, = struct.unpack_from("<I", b, off)
    name_len = b[off + 12]
    n_cigar, = struct.unpack_from("<H", b, off + 16)
    l_seq, = struct.unpack_from("<I", b, off + 20)
    cs = 36 + name_len
    ss = cs + 4 * n_cigar
    qs = ss + (l_seq + 1) // 2
    a = qs + l_seq
    return {"name_len": name_len, "n_cigar": n_cigar, "l_seq": l_seq, "cigar_start": cs, "sequence_start": ss,
            "quality_start": qs, "aux_start": a, "record_end": 4 + block_size}


def payloads(buf, off: int) -> dict:
    """name (NUL stripped), cigar_raw, sequence_packed, qualities, aux_raw."""
    L = layout(buf, off)
    b = bytes(buf[off:off + L["record_end"]])
    name = b[36:L["cigar_start"]]
    if name.endswith(b"\0"):
        name = name[:-1]
    return {"name": name, "cigar": b[L["cigar_start"]:L["sequence_start"]],
            "sequence": b[L["sequence_start"]:L["quality_start"]], "quality": b[L["quality_start"]:L["aux_start"]],
            "aux": b[L["aux_start"]:L["record_end"]]}


def aux_fields(buf, off: int):
    """([(tag, type, subtype, count, value_offset)], malformed): the fields up to
    the first malformed one; value_offset is record-relative (for B, the
    subtype byte)."""
    L = layout(buf, off)
    b = bytes(buf[off:off + L["record_end"]])
    end = L["record_end"]
    pos = L["aux_start"]
    out = []
    while pos < end:
        if pos + 3 > end:
            return out, True
        tag, ty = b[pos:pos + 2], b[pos + 2]
        v = pos + 3
        sub, count = 0, 1
        if ty in SCALAR:
            nxt = v + SCALAR[ty]
        elif ty in (ord("Z"), ord("H")):
            q = b.find(b"\0", v, end)
            if q < 0:
                return out, True
            count = q - v
            if ty == ord("H") and (count % 2 or any(c not in HEX for c in b[v:q])):
                return out, True
            nxt = q + 1
        elif ty == ord("B"):
            if v + 5 > end:
                return out, True
            sub = b[v]
            count, = struct.unpack_from("<I", b, v + 1)
            if sub not in WIDTH:
                return out, True
            nxt = v + 5 + count * WIDTH[sub]
        else:
            return out, True
        if nxt > end:
            return out, True
        out.append((tag, ty, sub, count, v))
        pos = nxt
    return out, False


def aux_get(buf, off: int, tag: bytes) -> dict:
    """Record::aux_get for every column of an AUX_VALUE row: status, type,
    subtype, count, value (integer scalars extended, A its byte, f its bits),
    offset (absolute, B at its first element)."""
    fields, bad = aux_fields(buf, off)
    for t, ty, sub, count, v in fields:
        if t != tag:
            continue
        p = off + v
        raw = bytes(memoryview(buf)[p:p + 4])
        value = 0
        if ty in (ord("A"), ord("C")):
            value = raw[0]
        elif ty == ord("c"):
            value = struct.unpack("<b", raw[:1])[0]
        elif ty == ord("s"):
            value = struct.unpack("<h", raw[:2])[0]
        elif ty == ord("S"):
            value = struct.unpack("<H", raw[:2])[0]
        elif ty == ord("i"):
            value = struct.unpack("<i", raw[:4])[0]
        elif ty in (ord("I"), ord("f")):
            value = struct.unpack("<I", raw[:4])[0]
        return {"status": PRESENT, "type": ty, "subtype": sub, "count": count, "value": value,
                "offset": p + 5 if ty == ord("B") else p}
    return {"status": MALFORMED if bad else ABSENT, "type": 0, "subtype": 0, "count": 0, "value": 0, "offset": 0}


def has_long_cigar_placeholder(buf, off: int) -> bool:
    L = layout(buf, off)
    if L["n_cigar"] != 2:
        return False
    op0, op1 = struct.unpack_from("<II", bytes(buf[off + L["cigar_start"]:off + L["cigar_start"] + 8]))
    kind = lambda op: CIGAR_OPS[op & 15] if (op & 15) < len(CIGAR_OPS) else None  # noqa: E731
    return kind(op0) == ord("S") and op0 >> 4 == L["l_seq"] and kind(op1) == ord("N")


def cigar_resolved(buf, off: int) -> dict:
    """status 0 stored / 1 from CG / 2 error, absolute offset of the first op, op count."""
    L = layout(buf, off)
    if not has_long_cigar_placeholder(buf, off):
        return {"status": 0, "offset": off + L["cigar_start"], "ops": L["n_cigar"]}
    cg = aux_get(buf, off, b"CG")
    if cg["status"] == PRESENT and cg["type"] == ord("B") and cg["subtype"] == ord("I"):
        return {"status": 1, "offset": cg["offset"], "ops": cg["count"]}
    return {"status": 2, "offset": 0, "ops": 0}


def cigar_text(buf, off: int) -> str:
    """The resolved CIGAR as SAM text (the reference's pacbio test renders it so)."""
    r = cigar_resolved(buf, off)
    ops = struct.unpack_from(f"<{r['ops']}I", bytes(buf[r["offset"]:r["offset"] + 4 * r["ops"]])) if r["ops"] else ()
    return "".join(f"{op >> 4}{chr(CIGAR_OPS[op & 15])}" for op in ops) or "*"


def decode_sequence(buf, off: int) -> bytes:
    L = layout(buf, off)
    packed = bytes(buf[off + L["sequence_start"]:off + L["quality_start"]])
    out = bytearray()
    for i in range(L["l_seq"]):
        byte = packed[i // 2]
        out.append(BASES[byte >> 4 if i % 2 == 0 else byte & 15])
    return bytes(out)
