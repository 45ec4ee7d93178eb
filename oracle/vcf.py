"""Columnar VCF restated on the CPU -- test infrastructure: the oracle for the
device VCF decoder, never called by the product.

Each record of a text scan (oracle/text.py device_scan, VCF dialect) is read
as the vendored lazy VCF reader reads a line:
  * read_record (crates/fritillaria-vcf/src/io/reader/record.rs:9-54): seven
    fields that must each end in a tab ("unexpected EOL" otherwise), then INFO
    up to a tab or the end of the line; read_field (:72-118) and read_line
    (src/io/reader.rs:400-422) drop a carriage return that precedes the line
    feed, so an unterminated last line keeps it;
  * the accessors (src/record/fields.rs:20-103, src/record.rs:35-79,147-150):
    "." is missing for ID, ALT, QUAL, FILTER and INFO; POS "0" is the
    telomere, anything else usize::from_str then Position::try_from (non-zero);
    QUAL f32::from_str; ALT split on ','
    (src/record/alternate_bases.rs:29-46); samples missing when empty or when
    their first tab-separated piece is ".".
QUAL values are the exact decimal rounded to the nearest binary32, ties to
even, which is what f32::from_str returns; whether the device parses a QUAL
at all follows its fast path (Clinger 1990), restated in qual_fast_path.
"""

from fractions import Fraction
import struct

import numpy as np

ID_MISSING, ALT_MISSING, QUAL_MISSING, FILTER_MISSING, INFO_MISSING = 1, 2, 4, 8, 16
SAMPLES_MISSING, FILTER_PASS, QUAL_PARSED, TELOMERE = 32, 64, 128, 256
OK, UNEXPECTED_EOL, INVALID_POSITION = 0, 1, 2
NAN_BITS = 0x7FC00000
BOUNDS = 9


def usize(s: bytes):
    """usize::from_str: an optional '+', then one or more ASCII digits, below 2^64."""
    t = s[1:] if s[:1] == b"+" else s
    if not t or any(c < 48 or c > 57 for c in t):
        return None
    v = int(t)
    return v if v < 1 << 64 else None


def f32_nearest(x: Fraction) -> int:
    """The binary32 nearest to x (ties to even) as bits; overflow to infinity."""
    sign = 0x80000000 if x < 0 else 0
    x = abs(x)
    if x == 0:
        return sign
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if Fraction(2) ** e > x:
        e -= 1
    e = max(e, -126)                        # subnormals share the minimum exponent
    q = x / Fraction(2) ** (e - 23)         # the significand in units of the last place
    m = q.numerator // q.denominator
    rem = q - m
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and m & 1):
        m += 1
    if m >= 1 << 24:                        # rounding carried into the next binade
        m >>= 1
        e += 1
    if e > 127:
        return sign | 0x7F800000
    if m < 1 << 23:                         # subnormal
        return sign | m
    return sign | ((e + 127) << 23) | (m - (1 << 23))


def decimal(s: bytes):
    """The exact value of a decimal in f32::from_str's grammar without inf/NaN,
    or None; a value whose leading digit lies beyond 10^40 or below 10^-50 is
    clamped there (binary32 rounds it to infinity or zero all the same)."""
    i, n, neg = 0, len(s), False
    if i < n and s[i] in b"+-":
        neg, i = s[i] == 45, i + 1
    j = i
    while j < n and 48 <= s[j] <= 57:
        j += 1
    ip = s[i:j]
    fp = b""
    if j < n and s[j] == 46:
        k = j + 1
        while k < n and 48 <= s[k] <= 57:
            k += 1
        fp, j = s[j + 1:k], k
    if not ip and not fp:
        return None
    ex = 0
    if j < n and s[j] in b"eE":
        k = j + 1
        if k < n and s[k] in b"+-":
            k += 1
        m = k
        while m < n and 48 <= s[m] <= 57:
            m += 1
        if m == k:
            return None
        ex, j = int(s[j + 1:m]), m
    if j != n:
        return None
    digits = (ip + fp).lstrip(b"0")
    if not digits:
        return Fraction(0)
    lead = ex - len(fp) + len(digits) - 1  # the power of ten of the leading digit
    if lead > 40:  # beyond binary32 either way: only the direction matters
        v = Fraction(10) ** 40
    elif lead < -50:
        v = Fraction(1, 10 ** 50)
    else:
        v = Fraction(int(digits)) * Fraction(10) ** (ex - len(fp))
    return -v if neg else v


def qual_fast_path(s: bytes):
    """(parsed, f32 bits) as the device decoder gives them: the digits of a
    decimal while its mantissa stays below 10^17 (a longer one is left
    unparsed), trailing zeros of the fraction moved to the exponent, a small
    mantissa absorbing an exponent above 10, then the value when the mantissa
    is at most 2^24 and the power of ten at most 10^10 either way."""
    v = decimal(s)
    if v is None:
        return False, NAN_BITS
    i, n, neg = 0, len(s), False
    if i < n and s[i] in b"+-":
        neg, i = s[i] == 45, i + 1
    m, e10, big = 0, 0, False
    while i < n and 48 <= s[i] <= 57:
        if m < 10 ** 17:
            m = m * 10 + s[i] - 48
        else:
            big, e10 = True, e10 + 1
        i += 1
    if i < n and s[i] == 46:
        i += 1
        while i < n and 48 <= s[i] <= 57:
            if m < 10 ** 17:
                m, e10 = m * 10 + s[i] - 48, e10 - 1
            else:
                big = True
            i += 1
    if i < n:  # exponent, saturated as the device saturates it
        i += 1
        eneg = i < n and s[i] == 45
        if i < n and s[i] in b"+-":
            i += 1
        x = 0
        while i < n:
            if x < 100000:
                x = x * 10 + s[i] - 48
            i += 1
        e10 += -x if eneg else x
    if big:
        return False, NAN_BITS
    if m == 0:
        return True, 0x80000000 if neg else 0
    while e10 < 0 and m % 10 == 0:
        m, e10 = m // 10, e10 + 1
    while e10 > 10 and m * 10 <= 1 << 24:
        m, e10 = m * 10, e10 - 1
    if m > 1 << 24 or not -10 <= e10 <= 10:
        return False, NAN_BITS
    return True, f32_nearest(v)


def f32_bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def header_contigs(text: bytes) -> list:
    """The ID of every "##contig=<...>" line of a header, in order."""
    out = []
    for line in text.split(b"\n"):
        if not line.startswith(b"##contig=<"):
            continue
        k, body = 0, line[len(b"##contig=<"):]
        while k < len(body):
            ke = k
            while ke < len(body) and body[ke] not in b"=,>":
                ke += 1
            if ke < len(body) and body[ke] == 61:
                ve = ke + 1
                if ve < len(body) and body[ve] == 34:
                    ve += 1
                    while ve < len(body) and body[ve] != 34:
                        ve += 1
                    ve = min(ve + 1, len(body))
                while ve < len(body) and body[ve] not in b",>":
                    ve += 1
                if body[k:ke] == b"ID":
                    out.append(body[ke + 1:ve])
                    break
                k = ve + 1
            else:
                k = ke + 1
    return out


def decode(buf, scan: dict, contigs=()) -> dict:
    """Columns of the records of a text scan (oracle/text.py device_scan)."""
    buf = bytes(np.asarray(buf, np.uint8))
    index = {}
    for i, c in enumerate(contigs):
        index.setdefault(bytes(c), i)
    offs, ends = scan["record_offsets"], scan["record_ends"]
    tabs, fs = scan["tabs"], scan["field_starts"]
    n = len(offs)
    out = {"chrom": np.full(n, -1, np.int32), "pos": np.zeros(n, np.uint64),
           "bounds": np.zeros((n, BOUNDS), np.uint32), "n_alt": np.zeros(n, np.uint32),
           "qual": np.full(n, NAN_BITS, np.uint32), "flags": np.zeros(n, np.uint16), "status": np.zeros(n, np.uint8)}
    for r in range(n):
        a, b = int(offs[r]), int(ends[r])
        line = buf[a:b]
        t = [int(x) - a for x in tabs[int(fs[r]):int(fs[r + 1])]]
        if len(t) < 7:
            out["status"][r] = UNEXPECTED_EOL
            continue
        content = len(line) - 1 if b < len(buf) and line.endswith(b"\r") else len(line)
        e = t[:7] + [t[7] if len(t) >= 8 else content, content]
        out["bounds"][r] = e
        field = lambda k: line[(e[k - 1] + 1 if k else 0):e[k]]  # noqa: E731
        fl, st = 0, OK
        out["chrom"][r] = index.get(field(0), -1)
        p = field(1)
        if p == b"0":
            fl |= TELOMERE
        else:
            v = usize(p)
            if not v:
                st = INVALID_POSITION
            else:
                out["pos"][r] = v
        if field(2) == b".":
            fl |= ID_MISSING
        alt = field(4)
        if alt == b".":
            fl |= ALT_MISSING
        elif alt:
            out["n_alt"][r] = alt.count(b",") + 1
        q = field(5)
        if q == b".":
            fl |= QUAL_MISSING
        else:
            ok, bits = qual_fast_path(q)
            if ok:
                fl |= QUAL_PARSED
                out["qual"][r] = bits
        f = field(6)
        if f == b".":
            fl |= FILTER_MISSING
        elif f == b"PASS":
            fl |= FILTER_PASS
        if field(7) == b".":
            fl |= INFO_MISSING
        samples = line[e[7] + 1:content] if len(t) >= 8 else b""
        if not samples or samples.split(b"\t")[0] == b".":
            fl |= SAMPLES_MISSING
        out["flags"][r] = fl
        out["status"][r] = st
    return out


GT_CALLED, GT_MISSING, GT_NONE, GT_INVALID, GT_UNREPRESENTED = 0, 1, 2, 3, 4


def alleles(v: bytes):
    """Genotype::iter over a GT value (value/genotype/iter.rs): [(position or
    None, phased)], or None where the iterator yields an error."""
    if not v:
        return None  # UnexpectedEof
    out, i = [], 0
    while i < len(v):
        j = i + 1  # next_allele searches from the second byte
        while j < len(v) and v[j] not in b"|/":
            j += 1
        a = i
        if v[a] in b"|/":  # explicit phasing (every allele after the first has one)
            ph, a = v[a] == 124, a + 1
        else:              # is_implicitly_unphased over what follows
            ph = b"/" not in v[j:]
        pos = v[a:j]
        if pos == b".":
            x = None
        else:
            x = usize(pos)
            if x is None:
                return None
        out.append((x, ph))
        i = j
    return out


def gt_code(v: bytes) -> int:
    """One GT value packed as the device packs it: "." is missing
    (src/record/samples/series/value.rs:26-27), else alleles()."""
    if v == b".":
        return GT_MISSING << 28
    al = alleles(v)
    if al is None:
        return GT_INVALID << 28
    if len(al) > 2 or any(x is not None and x >= 4095 for x, _ in al):
        return GT_UNREPRESENTED << 28
    code = [0 if x is None else x + 1 for x, _ in al] + [0]
    ph = [int(p) for _, p in al] + [0]
    return (len(al) << 26) | (ph[1] << 25) | (ph[0] << 24) | (code[1] << 12) | code[0]


def genotypes(buf, scan: dict):
    """(calls per tab, GT key index per record) for a text scan's records: the
    samples follow FORMAT (src/record/fields.rs:86-103 for when they are
    missing), each value is found at GT's position among the FORMAT keys
    (src/record/samples/sample.rs: keys zipped with the ':'-pieces of a
    non-empty sample)."""
    buf = bytes(np.asarray(buf, np.uint8))
    offs, ends = scan["record_offsets"], scan["record_ends"]
    tabs, fs = scan["tabs"], scan["field_starts"]
    calls = np.zeros(len(tabs), np.uint32)
    key = np.full(len(offs), -1, np.int32)
    for r in range(len(offs)):
        a, b = int(offs[r]), int(ends[r])
        line = buf[a:b]
        t = [int(x) - a for x in tabs[int(fs[r]):int(fs[r + 1])]]
        if len(t) < 8:
            continue
        content = len(line) - 1 if b < len(buf) and line.endswith(b"\r") else len(line)
        fmt = line[t[7] + 1:(t[8] if len(t) >= 9 else content)]
        g = -1
        if t[7] + 1 < content and fmt != b".":
            keys = fmt.split(b":")
            g = keys.index(b"GT") if b"GT" in keys else -1
        key[r] = g
        for j in range(len(t) - 8):
            code = GT_NONE << 28
            if g >= 0:
                s = line[t[8 + j] + 1:(t[9 + j] if 9 + j < len(t) else content)]
                pieces = s.split(b":") if s else []
                if g < len(pieces):
                    code = gt_code(pieces[g])
            calls[int(fs[r]) + 8 + j] = code
    return calls, key
