"""GPU test of frt_bam_scan_noalloc, the record-boundary scan that allocates
nothing.

It exists for callers that cannot let a library allocate device memory -- a
host that owns all device memory through its own arena, code that must not
allocate under a fixed budget or inside a capture, pipelines that preallocate
once.  The caller passes the inflated bytes, the member offsets and the output
array; the scan's scratch is one fixed device array inside the library, shared
by every call.  So the tests check, through the C ABI, that it returns exactly
what the oracle's serial scan (scan_records, record.rs:58-95) returns on the
same bytes -- on calls in a row over different batches (the shared scratch must
not carry anything from one call into the next), on a batch of exactly the
documented maximum of members, and on a batch cut inside its last record --
and that it refuses what its scratch cannot hold: too many members, a member
larger than BGZF's 64 KiB, too small an output array, a null output array with
room claimed, and a malformed record.

This file sorts last so that a run stopping at the first failure has run every
other test first; it also passes alone in a fresh process (its first call on
the device performs the scratch set-up).
"""

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import oracle

pytestmark = pytest.mark.gpu


def _inflated(frt, bgzf):
    """The file inflated on the device, its member offsets (host) and the
    oracle's view of the same bytes."""
    spans, _ = frt.discover_blocks(bgzf)
    batch = frt.CudaCodec(0).inflate_batch_device(bgzf, spans)
    host = batch.to_host()
    start, n_ref = oracle.bam_header(host)
    return batch, batch.offsets().astype(np.int64), host, start, n_ref


def _scan(frt, torch, data_ptr, length, member_offsets, start, n_ref, cap, extra=16):
    offs = torch.from_numpy(np.ascontiguousarray(member_offsets, dtype=np.int64)).to("cuda")
    out = torch.full((cap + extra,), -1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    n, tail = frt.bam_scan_noalloc(data_ptr, length, offs.data_ptr(), len(member_offsets) - 1, start,
                                   out.data_ptr(), cap, n_ref=n_ref)
    return n, tail, out.cpu().numpy()


def test_noalloc_scan_matches_the_oracle_on_calls_in_a_row(gpu):
    torch = pytest.importorskip("torch")
    files = []
    for seed, n in ((31, 12000), (32, 7000)):
        _, bgzf = synth.short_read_bam(n, seed=seed, levels=(1, 6))
        batch, moff, host, start, n_ref = _inflated(gpu, bgzf)
        want, want_tail = oracle.bam_scan(host, start)
        files.append((batch, moff, start, n_ref, want, want_tail))
    # A, B, A: every call must equal the oracle exactly
    for idx in (0, 1, 0):
        batch, moff, start, n_ref, want, want_tail = files[idx]
        n, tail, out = _scan(gpu, torch, batch.data_ptr(), batch.byte_len(), moff, start, n_ref, len(want))
        assert n == len(want)
        assert tail == want_tail
        assert np.array_equal(out[:n].astype(np.uint64), want)
        assert out[n] == -1  # nothing written past the records


def test_noalloc_scan_at_its_member_limit_and_cut_mid_record(gpu):
    """Exactly FRT_NOALLOC_MAX_MEMBERS small members, then the same bytes cut
    a few bytes into the last record: records and tail equal the oracle's
    scan of the same prefix."""
    torch = pytest.importorskip("torch")
    limit = gpu.NOALLOC_MAX_MEMBERS
    _, bgzf = synth.short_read_bam(30000, seed=33, levels=(1, 6), member_payload=8000)
    batch, moff, host, start, n_ref = _inflated(gpu, bgzf)
    assert len(moff) - 1 > limit
    moff = moff[: limit + 1]
    end = int(moff[-1])
    want, want_tail = oracle.bam_scan(host[:end], start)
    n, tail, out = _scan(gpu, torch, batch.data_ptr(), end, moff, start, n_ref, len(want))
    assert (n, tail) == (len(want), want_tail)
    assert np.array_equal(out[:n].astype(np.uint64), want)
    # cut 7 bytes into the last whole record: it becomes the tail
    cut = int(want[-1]) + 7
    moff_cut = moff.copy()
    k = int(np.searchsorted(moff_cut, cut, side="left"))
    moff_cut = np.append(moff_cut[:k], cut)
    want2, tail2 = oracle.bam_scan(host[:cut], start)
    assert tail2 == int(want[-1])
    n2, t2, out2 = _scan(gpu, torch, batch.data_ptr(), cut, moff_cut, start, n_ref, len(want2))
    assert (n2, t2) == (len(want2), tail2)
    assert np.array_equal(out2[:n2].astype(np.uint64), want2)


def test_noalloc_scan_refuses_what_its_scratch_cannot_hold(gpu):
    torch = pytest.importorskip("torch")
    with pytest.raises(gpu.InvalidArgument) as ei:
        gpu.bam_scan_noalloc(0, 1, 0, gpu.NOALLOC_MAX_MEMBERS + 1, 0, 0, 0)
    assert "scratch" in str(ei.value)
    _, bgzf = synth.short_read_bam(3000, seed=34, levels=(6, 6))
    batch, moff, host, start, n_ref = _inflated(gpu, bgzf)
    assert batch.byte_len() > 70_000
    # one member of about 70 KiB: more than BGZF allows, so refused
    with pytest.raises(gpu.InvalidArgument) as ei:
        _scan(gpu, torch, batch.data_ptr(), 70_000, [0, 70_000], start, n_ref, 1000)
    assert "65,536" in str(ei.value)
    # offsets past len are refused the same way
    with pytest.raises(gpu.InvalidArgument):
        _scan(gpu, torch, batch.data_ptr(), int(moff[1]) - 1, moff[:2], start, n_ref, 1000)
    want, want_tail = oracle.bam_scan(host, start)
    n = len(want)
    # one slot short: refused, and nothing is written at or past the cap
    with pytest.raises(gpu.InvalidArgument):
        _scan(gpu, torch, batch.data_ptr(), batch.byte_len(), moff, start, n_ref, n - 1)
    offs = torch.from_numpy(moff).to("cuda")
    out = torch.full((n + 4,), -1, dtype=torch.int64, device="cuda")
    with pytest.raises(gpu.InvalidArgument):
        gpu.bam_scan_noalloc(batch.data_ptr(), batch.byte_len(), offs.data_ptr(), len(moff) - 1, start,
                             out.data_ptr(), n - 1, n_ref=n_ref)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.array_equal(got[: n - 1].astype(np.uint64), want[: n - 1])
    assert np.all(got[n - 1:] == -1)
    # a null array with room claimed is refused; with no room it counts
    with pytest.raises(gpu.InvalidArgument):
        gpu.bam_scan_noalloc(batch.data_ptr(), batch.byte_len(), offs.data_ptr(), len(moff) - 1, start, 0, 10,
                             n_ref=n_ref)
    assert gpu.bam_scan_noalloc(batch.data_ptr(), batch.byte_len(), offs.data_ptr(), len(moff) - 1, start, 0, 0,
                                n_ref=n_ref) == (n, want_tail)
    # a block_size below 32 on the chain is Malformed, at that record
    bad = host.copy()
    at = int(want[n // 2])
    bad[at:at + 4] = np.frombuffer(np.uint32(20).tobytes(), np.uint8)
    dev = torch.from_numpy(bad).to("cuda")
    with pytest.raises(gpu.Malformed):
        _scan(gpu, torch, dev.data_ptr(), dev.numel(), moff, start, n_ref, n)
    # and the next call on good bytes is unaffected
    n3, t3, out3 = _scan(gpu, torch, batch.data_ptr(), batch.byte_len(), moff, start, n_ref, n)
    assert (n3, t3) == (n, want_tail) and np.array_equal(out3[:n].astype(np.uint64), want)
