"""The write side on the GB300: DeviceBlockCompressor.compress_batch_device
and DeviceBgzfWriter (crates/fritillaria-core/src/device.rs:326-372,
crates/fritillaria-bgzf/src/device_write.rs).  The contract is a round trip:
every block is a spec-valid BGZF member that gzip (zlib, which checks CRC32
and ISIZE) and this library's own device inflate turn back into its chunk;
empty chunks are the canonical empty block, incompressible ones stored, and
the writer's file ends with the EOF block."""

import gzip
import zlib

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def device(torch, raw: np.ndarray):
    t = torch.from_numpy(np.ascontiguousarray(raw, np.uint8)).to("cuda")
    torch.cuda.synchronize()
    return t


def check_block(frt, blk: bytes, chunk: bytes):
    assert blk[:4] == b"\x1f\x8b\x08\x04" and blk[12:14] == b"BC"
    assert int.from_bytes(blk[16:18], "little") + 1 == len(blk) <= 65536
    assert zlib.decompress(blk, 31) == chunk


def inputs():
    rng = np.random.default_rng(5)
    bam, _ = synth.short_read_bam(3000, seed=6, levels=(1, 1))
    fq, _ = synth.fastq(2000, seed=7)
    vcf = synth.raw_vcf_text(1500, 100, seed=8)
    return {"bam": bam, "fastq": fq, "vcf": vcf, "random": rng.integers(0, 256, 300_000, dtype=np.uint8),
            "zeros": np.zeros(200_000, np.uint8), "acgt": np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 250_000)]}


@pytest.mark.parametrize("name", ["bam", "fastq", "vcf", "random", "zeros", "acgt"])
def test_every_block_inflates_back(gpu, name):
    torch = pytest.importorskip("torch")
    raw = inputs()[name]
    dev = device(torch, raw)
    comp = gpu.DeviceCompressor(0)
    # chunks of the default size, the largest legal size, odd sizes, an empty one and a gap
    b = [0, 65280, 65280 + 65505, 65280 + 65505, 65280 + 65505 + 7, 65280 + 65505 + 7 + 1000]
    b += list(range(b[-1] + 3, raw.size, 40_000)) + [raw.size]
    bounds = np.array(b, np.uint64)
    cb = comp.compress_batch_device(dev.data_ptr(), dev.numel(), bounds)
    assert len(cb) == len(bounds) - 1 and cb.offsets[-1] == cb.byte_len()
    for i in range(len(cb)):
        chunk = bytes(raw[int(bounds[i]):int(bounds[i + 1])])
        blk = bytes(cb.block(i))
        check_block(gpu, blk, chunk)
        if not chunk:
            assert blk == gpu.EOF_BLOCK
        if name == "random" and len(chunk) >= 1000:  # fixed codes spend over 8 bits a random byte
            assert len(blk) == 18 + 5 + len(chunk) + 8  # stored
    if name in ("zeros", "acgt", "vcf"):
        assert cb.byte_len() < 0.7 * (bounds[-1] - bounds[0])
    # the library's own inflate of the same blocks
    stream = np.frombuffer(bytes(cb.data), np.uint8)
    spans, _ = gpu.discover_blocks(stream)
    batch = gpu.CudaCodec(0).inflate_batch_device(stream, spans)
    want = b"".join(bytes(raw[int(bounds[i]):int(bounds[i + 1])]) for i in range(len(cb)))
    assert bytes(batch.to_host()) == want


def test_writer_round_trip(gpu, tmp_path):
    torch = pytest.importorskip("torch")
    raw = inputs()["bam"]
    dev = device(torch, raw)
    comp = gpu.DeviceCompressor(0)
    path = tmp_path / "out.bgzf"
    with open(path, "wb") as f:
        w = gpu.DeviceBgzfWriter(f, comp, chunks_per_batch=7)
        w.write_device(dev.data_ptr(), dev.numel())
        w.write_batch(dev.data_ptr(), dev.numel(), [0, 100, 100, 5000])
        w.finish()
        w.finish()  # once
        st = w.stats()
    data = np.fromfile(path, np.uint8)
    assert bytes(data[-28:]) == gpu.EOF_BLOCK
    spans, consumed = oracle.discover(data)
    assert consumed == data.size
    n_write = -(-raw.size // 65280)
    assert len(spans) == n_write + 3 + 1 and st["blocks"] == n_write + 3
    assert st["batches"] == -(-n_write // 7) + 1
    assert st["compressed_bytes"] == data.size and st["uncompressed_bytes"] == raw.size + 5000
    assert gzip.decompress(bytes(data)) == bytes(raw) + bytes(raw[:5000])  # every member, in order


def test_bad_bounds_are_malformed(gpu):
    torch = pytest.importorskip("torch")
    dev = device(torch, np.zeros(200_000, np.uint8))
    comp = gpu.DeviceCompressor(0)
    for bad in ([0, 10, 5], [0, 65506], [0, 200_001], [5, 4]):
        with pytest.raises(gpu.Malformed):
            comp.compress_batch_device(dev.data_ptr(), dev.numel(), bad)
    assert len(comp.compress_batch_device(dev.data_ptr(), dev.numel(), [7])) == 0
    w = gpu.DeviceBgzfWriter(open("/dev/null", "wb"), comp)
    with pytest.raises(gpu.Malformed):
        w.write_batch(dev.data_ptr(), dev.numel(), [])
    w.finish()
    with pytest.raises(gpu.InvalidArgument):
        w.write_batch(dev.data_ptr(), dev.numel(), [0, 10])
