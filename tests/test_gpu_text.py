"""Tab-delimited text on the GB300 against the oracle (oracle/text.py, pinned
to the reference's text_scan.cu in tests/test_oracle_text.py): the reference's
real SAM, VCF, BED, GFF3 and GTF files and random text -- headers, blank
lines, empty fields, unterminated last lines, lines longer than a warp's
stride -- bgzipped, inflated on the device and scanned, at several starts;
modelled on crates/fritillaria-cuda/tests/text_scan.rs."""

from pathlib import Path

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import text

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
COLS = ["record_offsets", "record_ends", "header_offsets", "tabs", "field_starts"]
DIALECTS = {"reads_sam": text.SAM, "calls_vcf": text.VCF, "cytoband_bed": text.BED, "lambda_gff3": text.GFF,
            "lambda_gtf": text.GFF}


def device_batch(frt, codec, raw: np.ndarray):
    bgzf = synth.bgzf(np.ascontiguousarray(raw, np.uint8), "full", (6, 6))
    spans, _ = frt.discover_blocks(bgzf)
    return codec.inflate_batch_device(bgzf, spans)


def check(frt, scanner, batch, buf, start, dialect):
    got = scanner.scan(batch, start, dialect)
    want = text.device_scan(buf, start, dialect)
    assert len(got) == want["record_offsets"].size
    assert got.tail() == want["tail"]
    assert got.scan_info()[0] == want["header_offsets"].size
    for k in COLS:
        assert np.array_equal(got.column(k), want[k].astype(np.uint64)), (k, start)
    return got


@pytest.fixture(scope="module")
def scanner(gpu):
    return gpu.TextScanner(0)


@pytest.mark.parametrize("name", sorted(DIALECTS))
def test_real_files(gpu, scanner, name):
    buf = np.load(GOLDEN / "text_real.npz")[name]
    codec = gpu.CudaCodec(0)
    batch = device_batch(gpu, codec, buf)
    assert np.array_equal(batch.to_host(), buf)
    for start in (0, 1, 17, buf.size // 3, buf.size - 1, buf.size, buf.size + 4):
        check(gpu, scanner, batch, buf, start, DIALECTS[name])


def random_text(seed: int, n_lines: int, unterminated: bool, long_lines: bool = False) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lines = []
    for _ in range(n_lines):
        kind = rng.integers(0, 10)
        if kind == 0:
            lines.append(b"")
        elif kind == 1:
            lines.append(b"@" + b"\t".join(b"h" * int(rng.integers(0, 5)) for _ in range(int(rng.integers(1, 4)))))
        else:
            nf = int(rng.integers(1, 2600 if long_lines and kind == 9 else 30))
            fields = [bytes(rng.integers(33, 127, int(rng.integers(0, 12)), dtype=np.uint8)).replace(b"@", b"a")
                      for _ in range(nf)]
            lines.append(b"\t".join(fields))
    body = b"\n".join(lines)
    return np.frombuffer(body if unterminated else body + b"\n", np.uint8)


@pytest.mark.parametrize("seed", range(4))
def test_random_text(gpu, scanner, seed):
    codec = gpu.CudaCodec(0)
    for unterminated in (False, True):
        buf = random_text(seed, 6000 if seed < 3 else 200, unterminated, long_lines=seed == 3)
        batch = device_batch(gpu, codec, buf)
        for start in (0, 5, buf.size // 2):
            check(gpu, scanner, batch, buf, start, text.SAM)
            check(gpu, scanner, batch, buf, start, (ord("@"), ord("x")))


def test_synthetic_vcf(gpu, scanner):
    """The benchmark's VCF shape (meta lines, a #CHROM line naming every
    sample, a phased genotype per sample) at test size."""
    buf = synth.raw_vcf_text(300, 257, seed=5)
    codec = gpu.CudaCodec(0)
    batch = device_batch(gpu, codec, buf)
    got = check(gpu, scanner, batch, buf, 0, text.VCF)
    assert len(got) == 300 and got.scan_info()[0] == 32
    assert np.all(np.diff(got.column("field_starts").astype(np.int64)) == 8 + 257)


def test_edges(gpu, scanner):
    codec = gpu.CudaCodec(0)
    for raw in (b"\n", b"\n\n\n", b"@only\theaders\n@more\n", b"x", b"x\ty", b"a\tb\n\nc\t\td\n", b"@h\n@unterminated",
                b"\t", b"\t\n\t\n", b"r\n" * 5000):
        buf = np.frombuffer(raw, np.uint8)
        batch = device_batch(gpu, codec, buf)
        for start in range(0, min(len(raw), 4) + 2):
            check(gpu, scanner, batch, buf, start, text.SAM)
    empty = scanner.scan(None, 0, text.SAM)
    assert len(empty) == 0 and empty.tail() == 0


def test_tiles_denser_than_the_index_slots(gpu, scanner):
    """Tiles of 16 KiB with more than 1,024 newlines are read twice by the
    newline index, the others once: runs of two-byte lines between ordinary
    text."""
    codec = gpu.CudaCodec(0)
    dense = np.frombuffer(b"r\tx\n" * 9000 + b"\n" * 12000, np.uint8)
    buf = np.concatenate([random_text(11, 800, False), dense, random_text(12, 800, False), dense[:20001],
                          random_text(13, 300, True)])
    batch = device_batch(gpu, codec, buf)
    for start in (0, 7, 16384 + 3, buf.size // 2):
        check(gpu, scanner, batch, buf, start, text.SAM)


def test_a_batch_cut_mid_line_carries_the_line(gpu, scanner):
    buf = np.load(GOLDEN / "text_real.npz")["calls_vcf"]
    cut = buf[: buf.size // 2]
    assert cut[-1] != 10
    codec = gpu.CudaCodec(0)
    got = check(gpu, scanner, device_batch(gpu, codec, cut), cut, 0, text.VCF)
    # the cut line is the last record and the tail: the next batch starts there
    assert got.tail() == got.column("record_offsets")[-1] and got.column("record_ends")[-1] == cut.size


def test_argument_errors(gpu, scanner):
    codec = gpu.CudaCodec(0)
    batch = device_batch(gpu, codec, np.frombuffer(b"a\tb\n", np.uint8))
    with pytest.raises(gpu.InvalidArgument):
        scanner.scan(batch, 0, (300, None))
