"""GPU test of frt_bam_scan_noalloc, the record-boundary scan that allocates
nothing.

It exists for callers that cannot let a library allocate device memory -- a
host that owns all device memory through its own arena, code that must not
allocate under a fixed budget or inside a capture, pipelines that preallocate
once.  The caller passes the inflated bytes, the member offsets and the output
array; the scan's scratch is one fixed device array inside the library, shared
by every call.  So the test checks that, called through the C ABI, it returns
exactly what the allocating entry point (frt_bam_decode) returns, on calls in a
row over different batches -- the shared scratch must not carry anything from
one call into the next.

This file sorts last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process (its first call on
the device performs the scratch set-up).
"""

import numpy as np
import pytest

from fritillaria_gb300 import synth

pytestmark = pytest.mark.gpu


def _reference(frt, codec, decoder, bgzf):
    spans, _ = frt.discover_blocks(bgzf)
    batch = codec.inflate_batch_device(bgzf, spans)
    start, n_ref = frt.parse_header(batch.to_host())
    rb = decoder.decode(batch, start)
    return batch, start, n_ref, rb.column("record_offsets"), rb.tail()


def test_noalloc_scan_matches_decode_on_calls_in_a_row(gpu):
    torch = pytest.importorskip("torch")
    codec = gpu.CudaCodec(0)
    decoder = gpu.BamDecoder(0)
    batches = []
    for seed, n in ((31, 12000), (32, 7000)):
        _, bgzf = synth.short_read_bam(n, seed=seed, levels=(1, 6))
        batches.append(_reference(gpu, codec, decoder, bgzf))
    # A, B, A: every call must match the allocating entry point exactly
    for idx in (0, 1, 0):
        batch, start, n_ref, want, want_tail = batches[idx]
        offs = torch.from_numpy(batch.offsets().astype(np.int64)).to("cuda")
        out = torch.full((len(want) + 16,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        n, tail = gpu.bam_scan_noalloc(batch.data_ptr(), batch.byte_len(), offs.data_ptr(), len(batch), start,
                                       out.data_ptr(), out.numel(), n_ref=n_ref)
        assert n == len(want)
        assert tail == want_tail
        got = out[:n].cpu().numpy().astype(np.uint64)
        assert np.array_equal(got, want)
        assert int(out[n].item()) == -1  # nothing written past the records


def test_noalloc_scan_rejects_batches_beyond_its_scratch(gpu):
    with pytest.raises(gpu.InvalidArgument) as ei:
        gpu.bam_scan_noalloc(0, 1, 0, gpu.NOALLOC_MAX_MEMBERS + 1, 0, 0, 0)
    assert "scratch" in str(ei.value)
