"""Region serving on the GB300: BAI-resolved queries over resident BAMs,
batched into shared persistent inflates.  Every request's records equal the
reference's indexed query (chunks, then the overlap filter of
crates/fritillaria-bam/src/io/reader/query.rs:97-122), checked against a
brute-force scan of the whole file; a request gives the same bytes alone and
in a mix of concurrent requests; a budget smaller than the whole load still
serves everything, a few ticks at a time."""

import numpy as np
import pytest

from fritillaria_gb300 import synth
from oracle import bai as obai
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def files():
    out = []
    for seed, n in ((71, 60_000), (72, 25_000)):
        raw, bgzf = synth.short_read_bam(n, n_contigs=24, genome_len=200_000_000, seed=seed, levels=(1, 6))
        r = oracle.decode_bam_file(bgzf)
        vo = oracle.virtual_offsets(r["spans"], r["offsets"][:-1], r["columns"]["record_offsets"])
        t = obai.record_table(r["inflated"], r["columns"]["record_offsets"], vo)
        out.append({"bgzf": bgzf, "bai": synth.bai(raw, bgzf), "table": t, "cols": r["columns"]})
    return out


def _regions(n, seed):
    rng = np.random.default_rng(seed)
    regs = []
    for _ in range(n):
        f = int(rng.integers(0, 2))
        ref = int(rng.integers(0, 24))
        s = int(rng.integers(1, 8_000_000))
        e = s + int(np.exp(rng.uniform(np.log(1_000), np.log(10_000_000))))
        regs.append((f, ref, s, e))
    return regs


def _server(frt, files, budget=8 << 30):
    srv = frt.RegionServer(0, budget_bytes=budget)
    ids = [srv.add_bam(f["bgzf"], f["bai"]) for f in files]
    return srv, ids


def _want(files, f, ref, s, e):
    e = e or obai.MAX_POSITION  # 0: unbounded
    t = files[f]["table"]
    keep = obai.overlaps(t, ref, s, e)
    return t["voff"][keep], np.nonzero(keep)[0]


def _check(srv, rid, files, f, ref, s, e):
    srv.check(rid)
    info = srv.info(rid)
    assert info.state == 2
    voff, idx = _want(files, f, ref, s, e)
    assert np.array_equal(srv.column(rid, "virtual_offset"), voff), (f, ref, s, e)
    cols = files[f]["cols"]
    assert np.array_equal(srv.column(rid, "pos"), cols["pos"][idx])
    assert np.array_equal(srv.column(rid, "ref_id"), cols["ref_id"][idx])
    assert np.array_equal(srv.column(rid, "flags"), cols["flags"][idx])
    assert np.array_equal(srv.column(rid, "seq_len"), cols["seq_len"][idx])
    return srv.column(rid, "virtual_offset")


def test_regions_match_the_indexed_query(gpu, files):
    srv, ids = _server(gpu, files)
    regs = _regions(60, 5) + [(0, 3, 1, 0), (1, 23, 1, 200), (0, 0, 150_000_000, 150_001_000)]
    rids = [srv.submit(ids[f], ref, s, e) for f, ref, s, e in regs]
    srv.drain()
    total = 0
    for rid, (f, ref, s, e) in zip(rids, regs):
        total += len(_check(srv, rid, files, f, ref, s, e))
    assert total > 10_000


def test_same_alone_and_in_the_mix(gpu, files):
    srv, ids = _server(gpu, files)
    probe = (0, 5, 2_000_000, 2_600_000)
    alone = srv.submit(ids[0], *probe[1:])
    srv.drain()
    a = {k: srv.column(alone, k) for k in ("virtual_offset", "record_offset", "pos", "flags", "mapq", "seq_len")}
    # the same request among many others, submitted while ticks are running
    regs = _regions(40, 9)
    others = []
    for i, (f, ref, s, e) in enumerate(regs):
        others.append(srv.submit(ids[f], ref, s, e))
        if i == 20:
            mixed = srv.submit(ids[0], *probe[1:])
        srv.progress()
    srv.drain()
    for k, v in a.items():
        assert np.array_equal(srv.column(mixed, k), v), k
    for rid, (f, ref, s, e) in zip(others, regs):
        _check(srv, rid, files, f, ref, s, e)


def test_ticks_in_flight_on_their_own_streams(gpu, files):
    """Three ticks in flight, each on a stream of its own, with requests
    submitted while ticks run and results released as they are read: every
    request equals the indexed query."""
    srv, ids = _server(gpu, files)
    srv.set_limits(4, 3)
    regs = _regions(45, 13)
    rids = []
    for f, ref, s, e in regs:
        rids.append(srv.submit(ids[f], ref, s, e))
        srv.progress()
    srv.drain()
    for rid, reg in zip(rids, regs):
        _check(srv, rid, files, *reg)
        srv.release(rid)
    # and back to one tick in flight on the same server
    srv.set_limits(0, 1)
    rid = srv.submit(ids[1], *regs[0][1:])
    srv.drain()
    _check(srv, rid, files, 1, *regs[0][1:])


def test_small_budget_serves_everything(gpu, files):
    srv, ids = _server(gpu, files, budget=8 << 20)
    srv.set_limits(0, 1)
    regs = _regions(30, 11)
    rids = [srv.submit(ids[f], ref, s, e) for f, ref, s, e in regs]
    done = 0
    for _ in range(100000):
        done += srv.progress()
        # results are released as they are read, freeing the budget
        for rid, reg in zip(rids, regs):
            if rid is not None and srv.info(rid).state == 2:
                _check(srv, rid, files, *reg)
                srv.release(rid)
                rids[rids.index(rid)] = None
        if all(r is None for r in rids):
            break
    assert all(r is None for r in rids)


def test_empty_and_far_regions(gpu, files):
    srv, ids = _server(gpu, files)
    r1 = srv.submit(ids[0], 0, 199_000_000, 199_000_100)   # past the contig's reads
    r2 = srv.submit(ids[1], 7, 10, 10)
    srv.drain()
    for rid, reg in ((r1, (0, 0, 199_000_000, 199_000_100)), (r2, (1, 7, 10, 10))):
        _check(srv, rid, files, *reg)
    with pytest.raises(gpu.InvalidArgument):
        srv.submit(ids[0], 40, 1, 100)
