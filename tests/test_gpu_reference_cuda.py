"""The reference's own CUDA kernels (inflate_blocks, bam_scan_blocks,
bam_reconcile, bam_emit_offsets, bam_decode_fields), compiled from the
reference's sources for sm_103a and driven in its launch order with its reader
batching and carry (oracle/ref_cuda_driver.cpp), give the oracle's record
offsets and columns -- so the oracle this library is checked against is also
the reference's own CUDA path where that runs.  Skipped only where the
reference's kernels could not be compiled (no reference tree where the build
ran)."""

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle
from oracle import ref_cuda

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refcu(gpu):
    why = ref_cuda.available()
    if why:
        pytest.skip(why)
    return ref_cuda


@pytest.mark.parametrize("kind,blocks", [("short", 256), ("short", 3), ("long", 2), ("long", 256)])
def test_reference_cuda_path_equals_the_oracle(refcu, kind, blocks):
    if kind == "short":
        _, bgzf = synth.short_read_bam(20000, n_contigs=24, genome_len=3_100_000_000, seed=71, levels=(1, 6))
    else:
        _, bgzf = synth.ultra_long_bam(30, n_long_extra=2, seed=72)
    want = oracle.decode_bam_file(bgzf)
    n = len(want["columns"]["pos"])
    res, cols = refcu.run_bam(bgzf, blocks, columns_cap=n + 16)
    assert res.status == 0
    assert res.records == n
    assert np.array_equal(cols["record_offsets"], want["columns"]["record_offsets"])
    for k in ("ref_id", "pos", "flags", "seq_len"):
        assert np.array_equal(cols[k], want["columns"][k]), k
    # carried members are inflated again at the front of the next batch
    assert res.inflated_bytes >= want["inflated"].size
