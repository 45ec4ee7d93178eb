"""The write side's host rules, on the CPU: choose_framing and framed_size
pinned to the reference's own tests (crates/fritillaria-core/src/compress.rs,
tests a_chunk_at_the_limit_frames_to_exactly_one_maximal_block through
an_empty_payload_is_always_the_canonical_empty_block) and the EOF block to
crates/fritillaria-bgzf/src/block.rs:40-43."""

import zlib

import pytest

import fritillaria_gb300 as frt

HEADER, TRAILER, STORED = 18, 8, 5


def test_the_largest_chunk_frames_to_exactly_one_block():
    assert frt.MAX_COMPRESSIBLE_PAYLOAD == 65505
    assert frt.framed_size(frt.MAX_COMPRESSIBLE_PAYLOAD, (1 << 64) - 1) == 65536


def test_a_stream_too_large_to_frame_is_stored():
    assert frt.choose_framing(65_280, 148_256) == frt.Framing.STORED
    assert frt.framed_size(65_280, 148_256) == HEADER + 65_280 + STORED + TRAILER


def test_a_stream_that_would_grow_the_payload_is_stored():
    assert frt.choose_framing(1000, 1006) == frt.Framing.STORED
    assert frt.framed_size(1000, 1006) == HEADER + 1005 + TRAILER


def test_a_stream_no_larger_than_a_stored_block_is_used():
    assert frt.choose_framing(1000, 1005) == frt.Framing.DEFLATED
    assert frt.choose_framing(1000, 400) == frt.Framing.DEFLATED
    assert frt.framed_size(1000, 400) == HEADER + 400 + TRAILER


@pytest.mark.parametrize("claimed", [0, 2, 5, 999, 148_256])
def test_an_empty_payload_is_the_canonical_empty_block(claimed):
    assert frt.choose_framing(0, claimed) == frt.Framing.EMPTY
    assert frt.framed_size(0, claimed) == 28


def test_eof_block():
    assert frt.EOF_BLOCK == bytes([0x1f, 0x8b, 0x08, 0x04, 0x00, 0x00, 0x00, 0x00, 0x00, 0xff, 0x06, 0x00, 0x42,
                                   0x43, 0x02, 0x00, 0x1b, 0x00, 0x03, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00,
                                   0x00, 0x00])
    assert zlib.decompress(frt.EOF_BLOCK, 31) == b""
