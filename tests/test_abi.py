"""The C ABI without a GPU: the library loads, exports every function that
include/frt.h declares, refuses to run without a GB300 (no CPU fallback), and
its host-side parts -- BGZF member discovery (discover.rs:51-109) and the BAM
header parse (header.rs:43-101) -- agree with the oracle, including the errors
and their offsets."""

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("fields_", "text_")))  # record-field and text inputs have their own tests


@pytest.fixture(scope="module")
def frt():
    import fritillaria_gb300 as frt
    from fritillaria_gb300 import build

    if not build.LIB.exists():
        build.build_cuda()
    frt.lib()
    return frt


def test_library_exports_every_declared_function(frt):
    names = frt.header_functions()
    assert len(names) >= 50  # the parse found the declarations
    raw = C.CDLL(str(frt.LIB_PATH))
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing


def test_every_declared_function_has_a_binding(frt):
    L = frt.lib()
    for n in frt.header_functions():
        fn = getattr(L, n)
        assert fn.argtypes is not None or n == "frt_reader_open", n


def test_no_cpu_fallback_without_a_gpu(frt):
    if frt.cuda_is_usable():
        pytest.skip("a GPU is present")
    for backend in (frt.Backend.AUTO, frt.Backend.CUDA, frt.Backend.NVCOMP):
        with pytest.raises(frt.CudaUnavailable):
            frt.select_codec(backend)
    with pytest.raises(frt.InvalidArgument):
        frt.select_codec(frt.Backend.CPU)
    with pytest.raises(frt.CudaUnavailable):
        frt.CudaCodec(0)


@pytest.mark.parametrize("case", CASES)
def test_host_discovery_matches_oracle(frt, case):
    b = np.load(GOLDEN / f"{case}.npz")["bgzf"]
    got, used = frt.discover_blocks(b)
    want, wused = oracle.discover(b)
    assert used == wused
    for f in ("compressed_offset", "payload_start", "payload_len", "isize", "crc32"):
        assert np.array_equal(got[f], want[f]), f
    # a window that ends inside a member stops before it
    cut = b[: int(want["compressed_offset"][-1]) + 5]
    got, used = frt.discover_blocks(cut, base_offset=1000)
    assert used == int(want["compressed_offset"][-1])
    assert np.array_equal(got["compressed_offset"], want["compressed_offset"][:-1] + 1000)


def test_host_discovery_errors_match_oracle(frt):
    b = np.load(GOLDEN / "bam_short_full.npz")["bgzf"].copy()
    spans, _ = oracle.discover(b)
    at = int(spans["compressed_offset"][3])
    for pos, val in ((at + 2, 7), (at + 3, 0), (at + 12, 9), (at + 16, 0xFF)):
        bad = b.copy()
        bad[pos] = val
        with pytest.raises(oracle.OracleError) as want:
            oracle.discover(bad)
        with pytest.raises(frt.FrtError) as got:
            frt.discover_blocks(bad)
        assert got.value.code == want.value.code == 2
        assert got.value.offset == want.value.offset == at


@pytest.mark.parametrize("case", [c for c in CASES if c.startswith("bam_")])
def test_host_header_parse_matches_oracle(frt, case):
    g = np.load(GOLDEN / f"{case}.npz")
    data, _ = oracle.inflate_batch(g["bgzf"], oracle.discover(g["bgzf"])[0])
    assert frt.parse_header(data) == oracle.bam_header(data) == (int(g["records_start"]), int(g["n_ref"]))
    # a window ending inside the header is Malformed until more bytes arrive
    with pytest.raises(frt.Malformed):
        frt.parse_header(data[: int(g["records_start"]) - 1])
    with pytest.raises(frt.Malformed):
        frt.parse_header(b"BAM\x02")


@pytest.mark.parametrize("case", ["bcf_sites"])
def test_host_bcf_header_parse_matches_oracle(frt, case):
    g = np.load(GOLDEN / f"{case}.npz")
    data, _ = oracle.inflate_batch(g["bgzf"], oracle.discover(g["bgzf"])[0])
    want = oracle.bcf_header(data)
    assert frt.parse_bcf_header(data) == want == (int(g["records_start"]), int(g["samples"]), int(g["contigs"]))
    for cut in (4, 8, int(g["records_start"]) - 1):
        with pytest.raises(frt.Malformed):
            frt.parse_bcf_header(data[:cut])
    bad = data.copy()
    bad[3] = 3
    with pytest.raises(frt.Malformed):
        frt.parse_bcf_header(bad)


def test_format_scanners_refuse_without_a_gpu(frt):
    if frt.cuda_is_usable():
        pytest.skip("a GPU is present")
    for cls in (frt.FastqScanner, frt.BcfScanner, frt.FastaCompactor):
        with pytest.raises(frt.CudaUnavailable):
            cls(0)


def test_inflate_variants_and_default_tuning():
    import fritillaria_gb300 as frt

    frt.lib()
    vs = frt.inflate_variants()
    assert len(vs) >= 2
    for v in vs:
        assert 7 <= v["dist_bits"] <= v["lit_bits"] + 1 and v["lit_bits"] + v["dist_bits"] + 13 <= 33
        assert v["window"] % 32 == 0 and v["queue"] <= 1024 and v["smem_per_warp"] > v["window"]
        assert 32 <= v["max_registers"] <= 255
    t = frt.default_tuning().as_dict()
    assert t == {"variant": 0, "warps_per_cta": 3, "ctas_per_sm": 0, "queue_chunk": 1, "spread_variant": -1}
    with pytest.raises(frt.InvalidArgument):
        err = frt._Err()
        frt._raise(frt.lib().frt_inflate_variant_info(len(vs), frt.C.byref(frt.InflateVariant()), frt.C.byref(err)),
                   err)


def test_shipped_tuning_cache_names_compiled_variants():
    """Every entry of the committed tuning cache names a compiled variant of
    the shape it records (a stale entry would be ignored and re-tuned)."""
    import json

    import fritillaria_gb300 as frt

    frt.lib()
    path = Path(frt.__file__).resolve().parent / "inflate_tuning.json"
    doc = json.loads(path.read_text())
    assert doc["version"] == 1 and doc["entries"]
    vs = frt.inflate_variants()
    for key, e in doc["entries"].items():
        v = vs[e["variant"]]
        assert (e["lit_bits"], e["dist_bits"], e["window"], e["queue"], e["max_registers"]) == (
            v["lit_bits"], v["dist_bits"], v["window"], v["queue"], v["max_registers"]), key
        assert 1 <= e["warps_per_cta"] <= 8 and 1 <= e["queue_chunk"] <= 64 and e.get("chains", 1) >= 1
