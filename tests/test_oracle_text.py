"""The text-framing oracle (oracle/text.py) pinned on the CPU: its device
semantics against the reference's own text_scan.cu compiled as host code and
driven in the launcher's order (text.rs:233-420), on the reference's real SAM,
VCF, BED, GFF3 and GTF files (tests/golden/text_real.npz) at many starts and
on random text with headers, blank lines, empty fields and unterminated last
lines; and where the CPU decode (batch.rs:98-125, 270-297) and the launcher
agree -- every batch that ends in a newline -- the two restatements agree."""

from pathlib import Path

import numpy as np
import pytest

from oracle import ref as ref_kernels
from oracle import text

GOLDEN = Path(__file__).resolve().parent / "golden"
DIALECTS = {"reads_sam": text.SAM, "calls_vcf": text.VCF, "cytoband_bed": text.BED, "lambda_gff3": text.GFF,
            "lambda_gtf": text.GFF}


def ref():
    if ref_kernels.lib() is None:
        pytest.skip("reference kernels (oracle/_ref) not built: no reference tree")


def same(a: dict, b: dict):
    for k in ("record_offsets", "record_ends", "header_offsets", "tabs", "field_starts", "tail"):
        assert np.asarray(a[k]).tolist() == np.asarray(b[k]).tolist(), k


def random_text(seed: int, n_lines: int, unterminated: bool) -> np.ndarray:
    rng = np.random.default_rng(seed)
    lines = []
    for _ in range(n_lines):
        kind = rng.integers(0, 10)
        if kind == 0:
            lines.append(b"")  # blank
        elif kind == 1:
            lines.append(b"#" + b"\t".join(b"h" * int(rng.integers(0, 5)) for _ in range(int(rng.integers(1, 4)))))
        else:
            fields = [bytes(rng.integers(33, 127, int(rng.integers(0, 12)), dtype=np.uint8))
                      for _ in range(int(rng.integers(1, 30)))]
            lines.append(b"\t".join(f.replace(b"#", b"x") for f in fields))
    body = b"\n".join(lines)
    return np.frombuffer(body if unterminated else body + b"\n", np.uint8)


def test_fixture_facts():
    g = dict(np.load(GOLDEN / "text_real.npz"))
    facts = {k: text.device_scan(v, 0, DIALECTS[k]) for k, v in g.items()}
    assert facts["calls_vcf"]["record_offsets"].size == 275 and facts["calls_vcf"]["header_offsets"].size == 235
    assert facts["cytoband_bed"]["record_offsets"].size == 1549 and facts["cytoband_bed"]["header_offsets"].size == 0
    assert facts["lambda_gff3"]["record_offsets"].size == 308 and facts["lambda_gtf"]["record_offsets"].size == 357
    sam = facts["reads_sam"]
    fs = sam["field_starts"]
    assert sam["header_offsets"].size == 4 and ((fs[1:] - fs[:-1]) == 11).all()  # 12 SAM fields


@pytest.mark.parametrize("name", sorted(DIALECTS))
def test_fixtures_match_the_reference_kernels(name):
    ref()
    buf = np.load(GOLDEN / "text_real.npz")[name]
    for start in (0, 1, 17, buf.size // 3, buf.size - 5, buf.size - 1, buf.size, buf.size + 4):
        c, s2 = DIALECTS[name]
        same(text.device_scan(buf, start, DIALECTS[name]), ref_kernels.text_scan(buf, start, c, s2))
    # a batch cut in the middle of a line: the cut line is the tail
    cut = buf[: buf.size // 2]
    same(text.device_scan(cut, 0, DIALECTS[name]), ref_kernels.text_scan(cut, 0, *DIALECTS[name]))


@pytest.mark.parametrize("seed", range(6))
def test_random_text_matches_the_reference_kernels(seed):
    ref()
    for unterminated in (False, True):
        buf = random_text(seed, 400, unterminated)
        for start in (0, 3, buf.size // 2):
            same(text.device_scan(buf, start, text.VCF), ref_kernels.text_scan(buf, start, ord("#"), None))
            same(text.device_scan(buf, start, (ord("#"), ord("x"))),
                 ref_kernels.text_scan(buf, start, ord("#"), ord("x")))


def test_cpu_decode_agrees_on_terminated_batches():
    g = dict(np.load(GOLDEN / "text_real.npz"))
    for name, buf in g.items():
        assert buf[-1] == 10
        same(text.device_scan(buf, 0, DIALECTS[name]), text.cpu_decode(buf, 0, DIALECTS[name]))
    buf = random_text(9, 300, True)
    dev, cpu = text.device_scan(buf, 0, text.VCF), text.cpu_decode(buf, 0, text.VCF)
    # the launcher keeps the unterminated last line as a record; the CPU decode carries it
    assert dev["record_offsets"].size == cpu["record_offsets"].size + 1 and dev["tail"] == cpu["tail"]


def test_synthetic_vcf_matches_the_reference_kernels():
    """The benchmark's VCF generator: seeded, a #CHROM line naming every
    sample, and framed alike by the oracle, the reference's kernels and the
    reference's CPU decode."""
    from fritillaria_gb300 import synth

    buf = synth.raw_vcf_text(200, 100, seed=5)
    assert np.array_equal(buf, synth.raw_vcf_text(200, 100, seed=5))
    dev = text.device_scan(buf, 0, text.VCF)
    assert dev["record_offsets"].size == 200 and dev["tabs"].size == 200 * (8 + 100)
    chrom = bytes(buf[int(dev["header_offsets"][-1]):int(dev["record_offsets"][0]) - 1]).split(b"\t")
    assert chrom[:9] == [b"#CHROM", b"POS", b"ID", b"REF", b"ALT", b"QUAL", b"FILTER", b"INFO", b"FORMAT"]
    assert len(chrom) == 109
    same(dev, text.cpu_decode(buf, 0, text.VCF))
    ref()
    same(dev, ref_kernels.text_scan(buf, 0, ord("#"), None))
