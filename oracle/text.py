"""Tab-delimited text framing, restated on the CPU -- test infrastructure: the
oracle for the device text scanner, never called by the product.

Two restatements, because the reference's CPU decode and its device launcher
differ on a batch whose last line has no newline:
  * cpu_decode: RecordBatch::decode over scan_lines
    (crates/fritillaria-text/src/columnar/batch.rs:98-125, 270-297): only lines
    ending in a newline are lines; the tail is where an unterminated last line
    starts (or the end);
  * device_scan: TextScanner::scan (crates/fritillaria-cuda/src/text.rs:233-420)
    over kernels/text_scan.cu: every line start is a line, an unterminated last
    one a record running to the end of the batch, and the tail is that
    record's start when it runs to the end, else the batch end.
Both skip blank lines and split header lines from records by the first byte
(Dialect, batch.rs:23-76).  The product follows device_scan.
"""

import numpy as np

SAM = (ord("@"), None)
VCF = (ord("#"), None)
GFF = (ord("#"), None)
BED = (ord("#"), None)


def _lines(buf: np.ndarray, start: int):
    """Starts and ends (newline excluded, or the batch end) of the non-blank
    lines from `start`: a line starts at `start` or one past a newline."""
    n = buf.size
    if start >= n:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    nl = np.flatnonzero(buf[start:] == 10).astype(np.int64) + start
    starts = np.concatenate([np.array([start], np.int64), nl + 1])
    starts = starts[starts < n]
    ends = np.append(nl, n)[np.searchsorted(nl, starts)]  # the first newline at or after the start
    keep = buf[starts] != 10
    return starts[keep], ends[keep]


def _fields(buf, starts, ends, comment, secondary) -> dict:
    """Records and header lines by first byte; each record's tabs in order."""
    first = buf[starts]
    hdr = first == comment
    if secondary is not None:
        hdr |= first == secondary
    r_off, r_end = starts[~hdr], ends[~hdr]
    tabs = np.flatnonzero(buf == 9).astype(np.int64)
    lo, hi = np.searchsorted(tabs, r_off), np.searchsorted(tabs, r_end)
    flat = np.concatenate([tabs[a:b] for a, b in zip(lo, hi)]) if r_off.size else np.zeros(0, np.int64)
    fs = np.zeros(r_off.size + 1, np.uint64)
    fs[1:] = np.cumsum(hi - lo)
    return {"record_offsets": r_off.astype(np.uint64), "record_ends": r_end.astype(np.uint64),
            "header_offsets": starts[hdr].astype(np.uint64), "tabs": flat.astype(np.uint64),
            "field_starts": fs if r_off.size else np.zeros(0, np.uint64)}


def device_scan(buf, start: int, dialect) -> dict:
    buf = np.asarray(buf, np.uint8)
    starts, ends = _lines(buf, start)
    out = _fields(buf, starts, ends, *dialect)
    r_off, r_end = out["record_offsets"], out["record_ends"]
    if start >= buf.size:
        out["tail"] = min(start, buf.size)
    elif r_off.size and int(r_end[-1]) >= buf.size:
        out["tail"] = int(r_off[-1])
    else:
        out["tail"] = int(buf.size)
    return out


def cpu_decode(buf, start: int, dialect) -> dict:
    buf = np.asarray(buf, np.uint8)
    starts, ends = _lines(buf, start)
    terminated = ends < buf.size
    out = _fields(buf, starts[terminated], ends[terminated], *dialect)
    # scan_lines stops at the first line without a newline; past the end it
    # returns where it started
    out["tail"] = int(starts[~terminated][0]) if (~terminated).any() else max(start, int(buf.size))
    return out
