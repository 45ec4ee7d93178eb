"""Inflate + CRC/ISIZE verification on the GB300 against the oracle (zlib) on
the same members: dynamic, fixed-Huffman, stored, RLE/Huffman-only streams,
empty and EOF members, mixed levels; tampered CRC/ISIZE/payload must fail the
batch with the reference's error variant and member offset
(crates/fritillaria-cuda/tests/inflate.rs:37-233)."""

import zlib

import numpy as np
import pytest

from oracle import oracle

pytestmark = pytest.mark.gpu

EOF_BLOCK = bytes([0x1f, 0x8b, 0x08, 0x04, 0, 0, 0, 0, 0, 0xff, 0x06, 0, 0x42, 0x43, 0x02, 0, 0x1b, 0, 0x03, 0, 0, 0, 0,
                   0, 0, 0, 0, 0])


def member(payload: bytes, level=6, strategy=zlib.Z_DEFAULT_STRATEGY, memlevel=8) -> bytes:
    co = zlib.compressobj(level, zlib.DEFLATED, -15, memlevel, strategy)
    cdata = co.compress(payload) + co.flush()
    bsize = 18 + len(cdata) + 8
    if bsize > 65536:
        return None  # does not fit a BGZF member
    hdr = bytes([0x1f, 0x8b, 8, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, ord("B"), ord("C"), 2, 0]) + (bsize - 1).to_bytes(2, "little")
    return hdr + cdata + zlib.crc32(payload).to_bytes(4, "little") + len(payload).to_bytes(4, "little")


def payloads(rng):
    text = b"".join(b"r%09d\tchr1\t%d\tACGT\n" % (i, i * 7) for i in range(1500))
    yield b""
    yield b"a"
    yield bytes(rng.integers(0, 256, 60000, dtype=np.uint8))          # incompressible
    yield bytes(rng.integers(65, 69, 65280, dtype=np.uint8))          # 2-bit alphabet
    yield b"A" * 65536                                                 # one long run
    yield text[:65000]
    yield bytes(rng.choice(np.frombuffer(b"ACGTN", np.uint8), 40000, p=[.3, .2, .2, .29, .01]))


STRATEGIES = [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_DEFAULT_STRATEGY),
              (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_FIXED), (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE),
              (6, zlib.Z_FILTERED)]


def build_file(rng):
    parts = []
    for p in payloads(rng):
        for level, strat in STRATEGIES:
            m = member(p, level, strat)
            if m is not None:
                parts.append(m)
    parts.append(EOF_BLOCK)
    return b"".join(parts)


def test_inflate_matches_oracle(gpu):
    rng = np.random.default_rng(5)
    data = build_file(rng)
    spans, used = oracle.discover(data)
    assert used == len(data)
    expect, offs = oracle.inflate_batch(data, spans)
    codec = gpu.CudaCodec(0)
    got, goffs = codec.inflate_batch(data, spans)
    assert np.array_equal(goffs, offs)
    assert np.array_equal(got, expect)
    dev = codec.inflate_batch_device(data, spans)
    assert dev.byte_len() == expect.size
    assert np.array_equal(dev.to_host(), expect)
    assert np.array_equal(dev.offsets(), offs)


def test_inflate_single_members_each_type(gpu):
    rng = np.random.default_rng(9)
    codec = gpu.CudaCodec(0)
    for p in payloads(rng):
        for level, strat in STRATEGIES:
            m = member(p, level, strat)
            if m is None:
                continue
            spans, _ = oracle.discover(m)
            got, _ = codec.inflate_batch(m, spans)
            assert bytes(got) == p, (len(p), level, strat)


@pytest.mark.parametrize("what", ["crc", "isize", "payload"])
def test_tampered_member_fails_with_its_offset(gpu, what):
    rng = np.random.default_rng(11)
    parts = [member(bytes(rng.integers(65, 70, 20000, dtype=np.uint8)), 6) for _ in range(4)]
    offsets = np.cumsum([0] + [len(p) for p in parts])[:-1]
    bad = bytearray(parts[2])
    if what == "crc":
        bad[-8] ^= 0xff
    elif what == "isize":
        bad[-4] = (bad[-4] + 1) & 0xff
    else:
        bad[40] ^= 0x55
    parts[2] = bytes(bad)
    data = b"".join(parts)
    spans, _ = oracle.discover(data)
    codec = gpu.CudaCodec(0)
    with pytest.raises(gpu.FrtError) as ei:
        codec.inflate_batch_device(data, spans)
    try:
        oracle.inflate_batch(data, spans)
        raise AssertionError("oracle accepted a tampered member")
    except oracle.OracleError as oe:
        assert ei.value.code == oe.code, (ei.value, oe)
        assert ei.value.offset == oe.offset == offsets[2]
