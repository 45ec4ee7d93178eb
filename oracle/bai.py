"""TEST INFRASTRUCTURE ONLY.  A restatement of the reference's BAI region
resolution and region filter, the oracle for the library's BAI query and
its region-serving path:

  * parse: the BAI layout (SAM specification 5.2; crates/fritillaria-bam/src/
    bai.rs:13-21 and its reader): per reference the bins with their chunks (the
    pseudo-bin 37450 is metadata, not a bin) and the 16 kb linear index;
  * query: BinningIndex::query (crates/fritillaria-csi/src/binning_index/
    index.rs:93-119): reg2bins over the 1-based inclusive interval
    (reference_sequence.rs:376-398), the chunks of the bins present, the linear
    index's minimum offset for the interval start (index/linear_index.rs:11-15),
    then optimize_chunks (binning_index.rs:33-62);
  * records: what the reference's indexed query yields (crates/fritillaria-bam/
    src/io/reader/query.rs:97-122): records whose start virtual offset lies in a
    chunk, kept when their reference matches and [pos+1, pos+span] (span from the
    CIGAR's M/D/N/=/X, at least 1) intersects the interval.
"""

from __future__ import annotations

import struct

import numpy as np

MIN_SHIFT = 14
DEPTH = 5
META_BIN = 37450
MAX_POSITION = (1 << (MIN_SHIFT + DEPTH * 3)) - 1


def parse(data) -> dict:
    b = bytes(data)
    if b[:4] != b"BAI\x01":
        raise ValueError("not a BAI")
    at = 4
    (n_ref,) = struct.unpack_from("<i", b, at)
    at += 4
    refs = []
    for _ in range(n_ref):
        (n_bin,) = struct.unpack_from("<i", b, at)
        at += 4
        bins, meta = {}, None
        for _ in range(n_bin):
            bin_id, n_chunk = struct.unpack_from("<Ii", b, at)
            at += 8
            chunks = [struct.unpack_from("<QQ", b, at + 16 * k) for k in range(n_chunk)]
            at += 16 * n_chunk
            if bin_id == META_BIN:
                meta = chunks
            else:
                bins.setdefault(bin_id, []).extend(chunks)
        (n_intv,) = struct.unpack_from("<i", b, at)
        at += 4
        lidx = list(struct.unpack_from(f"<{n_intv}Q", b, at))
        at += 8 * n_intv
        refs.append({"bins": bins, "lidx": lidx, "meta": meta})
    n_no_coor = struct.unpack_from("<Q", b, at)[0] if at + 8 <= len(b) else None
    return {"refs": refs, "n_no_coor": n_no_coor}


def reg2bins(start: int, end: int) -> set:
    """Bins overlapping the 1-based inclusive interval [start, end]."""
    beg, last = start - 1, end - 1
    out, t, s = set(), 0, MIN_SHIFT + DEPTH * 3
    for level in range(DEPTH + 1):
        out.update(range(t + (beg >> s), t + (last >> s) + 1))
        s -= 3
        t += 1 << (level * 3)
    return out


def optimize_chunks(chunks, min_offset: int = 0):
    cs = sorted((c for c in chunks if c[1] > min_offset), key=lambda c: c[0])
    if not cs:
        return []
    merged, cur = [], list(cs[0])
    for nxt in cs[1:]:
        if nxt[0] > cur[1]:
            merged.append(tuple(cur))
            cur = list(nxt)
        elif cur[1] < nxt[1]:
            cur[1] = nxt[1]
    merged.append(tuple(cur))
    return merged


def query(index: dict, ref: int, start: int = 1, end: int = MAX_POSITION):
    if ref < 0 or ref >= len(index["refs"]):
        raise IndexError(f"invalid reference sequence ID: {ref}")
    if start > MAX_POSITION or end > MAX_POSITION:
        raise ValueError("invalid interval bound")
    r = index["refs"][ref]
    want = reg2bins(start, end)
    chunks = [c for bid, cs in r["bins"].items() if bid in want for c in cs]
    w = (start - 1) >> MIN_SHIFT
    min_offset = r["lidx"][w] if w < len(r["lidx"]) else 0
    return optimize_chunks(chunks, min_offset)


def record_table(inflated, record_offsets, virtual_offsets) -> dict:
    """Per record: ref id, 0-based pos, span and start virtual offset."""
    buf = np.asarray(inflated, dtype=np.uint8)
    n = len(record_offsets)
    ref = np.zeros(n, np.int32)
    pos = np.zeros(n, np.int32)
    span = np.ones(n, np.int64)
    for i, o in enumerate(record_offsets):
        o = int(o)
        ref[i], pos[i] = struct.unpack_from("<ii", buf, o + 4)
        name_len = int(buf[o + 12])
        (n_cigar,) = struct.unpack_from("<H", buf, o + 16)
        s = 0
        for k in range(n_cigar):
            (op,) = struct.unpack_from("<I", buf, o + 36 + name_len + 4 * k)
            if op & 15 in (0, 2, 3, 7, 8):
                s += op >> 4
        span[i] = s if s > 0 else 1
    return {"ref": ref, "pos": pos, "span": span, "voff": np.asarray(virtual_offsets, np.uint64)}


def overlaps(t: dict, ref: int, start: int, end: int) -> np.ndarray:
    a0 = t["pos"].astype(np.int64) + 1
    a1 = a0 + t["span"] - 1
    return (t["ref"] == ref) & (t["pos"] >= 0) & (a0 <= end) & (start <= a1)


def brute_force(t: dict, ref: int, start: int, end: int) -> np.ndarray:
    """Start virtual offsets of every overlapping record, in file order."""
    return t["voff"][overlaps(t, ref, start, end)]


def via_chunks(t: dict, chunks, ref: int, start: int, end: int) -> np.ndarray:
    """What the indexed query yields: records starting inside a chunk, filtered."""
    keep = np.zeros(len(t["voff"]), bool)
    for c0, c1 in chunks:
        keep |= (t["voff"] >= np.uint64(c0)) & (t["voff"] < np.uint64(c1))
    return t["voff"][keep & overlaps(t, ref, start, end)]
