#!/usr/bin/env python3
"""BAM -> device columns, decompressed GB/s on GB300.

One step = one pass of the path over the whole synthetic file: BGZF member
discovery, inflate, CRC32/ISIZE verification, BAM record scan and every
column, ending with the device error word read back and checked.

  value   batched form, compressed bytes already resident in HBM
  e2e     the same through the C ABI from pinned host memory (H2D of the
          compressed file and D2H of the run's stats inside the timed region)
  plain   the reference-shaped per-batch form (DeviceBgzfReader +
          BamDecoder, 256 members per batch, host syncs per batch) on the
          same GPU and the same host bytes
  cpu_baseline  the oracle's multithreaded restatement of the noodles CPU
          path (zlib inflate + CRC on all host cores, serial record scan,
          columns and aux walk)
  roofline  the inflate kernel's HBM fraction (algorithmic bytes over its
          CUDA-event time), and beside it, for short reads, its issue
          roofline: warp instructions per second over the SMs' issue
          capacity, with warps in flight and symbols per warp per second

Inputs are seeded synthetic data (no dataset is available offline); the
workload is larger than L2, so no flush is needed between steps.
Multi-GPU: the path shards by file, so N GPUs run N replicas of the workload
(weak scaling); value = all ranks' bytes / the slowest rank's time.
"""

from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "short_reads_20m": dict(kind="short", n_records=20_000_000, n_contigs=24, genome_len=3_100_000_000,
                            levels=(1, 6), seed=20,
                            desc="20M paired-end 2x150 bp records over 24 contigs (3.1 Gb), BGZF members "
                                 "alternating zlib level 1/6, packed full (records straddle members)"),
    "short_reads_2m": dict(kind="short", n_records=2_000_000, n_contigs=24, genome_len=3_100_000_000,
                           levels=(1, 6), seed=20,
                           desc="2M records of the 20M workload's shape (profiling size: inputs above L2, "
                                "under 1 GB on the device)"),
    "short_reads_100k": dict(kind="short", n_records=100_000, n_contigs=1, genome_len=50_000_000, levels=(6, 6),
                             seed=1, desc="100k 2x150 bp records on one 50 Mb contig, BGZF level 6, packed full"),
    "ultra_long_50k": dict(kind="long", n_records=50_000, n_long_extra=20, levels=(6, 6), seed=3,
                           desc="50k unaligned ultra-long reads (log-normal, median 15 kb) + 20 of 250-800 kb, "
                                "MM/ML/qs/ch tags, BGZF level 6 packed full"),
}

# Several formats in one persistent inflate: (a) BCF, (b) bgzipped FASTQ,
# (c) bgzipped FASTA, decoded by their scanners after one inflate of all members.
MIXED = {
    "mixed_formats": dict(bcf_sites=2_000_000, bcf_samples=500, fastq_reads=10_000_000, fasta_bases=3_100_000_000,
                          vcf_sites=20_000, vcf_samples=2504,
                          desc="one persistent inflate over (a) BCF 2M sites x 500 samples over 24 contigs, "
                               "(b) bgzipped FASTQ 10M x 150 bp, (c) bgzipped FASTA 3.1 Gb (60-column lines, "
                               "soft-masked runs, N runs); each then decoded by its scanner. Text framing is "
                               "timed beside it on a bgzipped VCF of 20k sites x 2,504 phased genotypes"),
    "mixed_formats_small": dict(bcf_sites=200_000, bcf_samples=500, fastq_reads=1_000_000, fasta_bases=310_000_000,
                                vcf_sites=2_000, vcf_samples=2504,
                                desc="the mixed-format workload at one tenth size (profiling size)"),
}

# Region serving: BAI-indexed BAMs resident on the device, a Poisson stream of
# region queries, continuous batching into shared persistent inflates.
SERVING = {
    "serving": dict(files=32, min_records=50_000, max_records=2_500_000, rate=2000.0, requests=4000,
                    plain_requests=300, budget=150 << 30,
                    desc="32 BAI-indexed short-read BAMs (24 contigs, 3.1 Gb; record counts log-uniform "
                         "50k-2.5M, one twentieth of 1M-50M), Poisson arrivals at 2,000 req/s, regions on a "
                         "random contig with uniform start and log-uniform length 1 kb-10 Mb, 150 GB budget"),
    "serving_quarter": dict(files=32, min_records=250_000, max_records=12_500_000, rate=2000.0, requests=4000,
                            plain_requests=300, budget=150 << 30,
                            desc="32 BAI-indexed short-read BAMs (24 contigs, 3.1 Gb; record counts log-uniform "
                                 "250k-12.5M, one quarter of 1M-50M), Poisson arrivals at 2,000 req/s, regions on a "
                                 "random contig with uniform start and log-uniform length 1 kb-10 Mb, 150 GB budget"),
    "serving_full": dict(files=32, min_records=1_000_000, max_records=50_000_000, rate=2000.0, requests=4000,
                         plain_requests=300, budget=150 << 30,
                         desc="32 BAI-indexed short-read BAMs (24 contigs, 3.1 Gb; record counts log-uniform 1M-50M), "
                              "Poisson arrivals at 2,000 req/s, regions on a random contig with uniform start and "
                              "log-uniform length 1 kb-10 Mb, 150 GB budget"),
    "serving_small": dict(files=8, min_records=20_000, max_records=200_000, rate=2000.0, requests=800,
                          plain_requests=100, budget=150 << 30, desc="the serving workload at test size"),
}

METRIC = "BAM->device-column decompressed GB/s, batched vs plain, 1 GB300, bit-exact"
# members per batch of the plain per-batch loop: the reference's default
# (crates/fritillaria-bgzf/src/read.rs:37) first, then larger batches
PLAIN_BATCHES = (256, 1024, 4096, 16384)


def bam_config(workload: str, records: int, members: int, compressed: int, inflated: int, world: int) -> dict:
    """The workload as both arms report it (the same keys and values)."""
    return {"workload": workload, "description": WORKLOADS[workload]["desc"], "records": int(records),
            "members": int(members), "compressed_bytes": int(compressed), "inflated_bytes": int(inflated),
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}
# Inflate tunings measured on GB300 (written by the autotuner, one entry per
# device and workload class); a miss is tuned at start-up and added.
TUNING_CACHE = ROOT / "fritillaria_gb300" / "inflate_tuning.json"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(MIXED) + sorted(SERVING), default="short_reads_20m")
    p.add_argument("--no-plain", action="store_true", help="skip the per-batch comparison")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-fields", action="store_true", help="skip timing the record-field kernels")
    p.add_argument("--no-write", action="store_true", help="skip timing the BGZF compressor")
    p.add_argument("--tuning-cache", default=str(TUNING_CACHE),
                   help="JSON cache of inflate tunings (read, and written on a miss)")
    p.add_argument("--retune", action="store_true", help="time the inflate tunings again even on a cache hit")
    return p.parse_args()


def generate(name: str):
    from fritillaria_gb300 import synth

    w = WORKLOADS[name]
    if w["kind"] == "short":
        _, bgzf = synth.short_read_bam(w["n_records"], n_contigs=w["n_contigs"], genome_len=w["genome_len"],
                                       seed=w["seed"], levels=w["levels"])
    else:
        _, bgzf = synth.ultra_long_bam(w["n_records"], n_long_extra=w["n_long_extra"], seed=w["seed"],
                                       levels=w["levels"])
    return bgzf


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = list(csv.reader(io.StringIO(open(self.path).read())))
        os.unlink(self.path)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(value: float, dist=None, device="cpu") -> float:
    """The slowest rank's figure (an all-reduce MAX); the value itself on one
    rank.  Every rank must call it."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gbs(bytes_per_rank: int, world: int, steps: int, ms: float) -> float:
    """Aggregate GB/s of N replicas that each processed `bytes_per_rank` per
    step, over the slowest rank's time."""
    return world * bytes_per_rank * steps / (ms / 1e3) / 1e9


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(bgzf, inflated_bytes: int):
    """The oracle's CPU restatement of the reference's CPU path: all host
    threads over the whole file (seconds of work on 16 cores), and one thread
    over the file's first quarter of members (a bounded sample)."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    res = oracle.baseline_bam(bgzf, threads)
    gbs = res.inflated_bytes / res.seconds / 1e9 if res.seconds > 0 else 0.0
    quarter = max(1, res.members // 4)
    one = oracle.baseline_bam(bgzf, 1, quarter)
    one_gbs = one.inflated_bytes / one.seconds / 1e9 if one.seconds > 0 else 0.0
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"whole file: {res.members} members, {res.inflated_bytes} inflated bytes, {res.records} "
                      f"records, {res.seconds:.2f} s; C restatement of the noodles multithreaded BGZF reader "
                      f"(zlib 1.3 inflate + CRC32) and the serial record scan/columns/aux walk",
            "records": res.records, "status": res.status, "cpu_model": cpu_model(), "nproc": threads,
            "one_thread": {"value": round(one_gbs, 3), "unit": "GB/s", "cores": 1,
                           "sample": f"the first {one.members} members ({one.inflated_bytes} inflated bytes, "
                                     f"{one.records} records), {one.seconds:.2f} s"}}


class _DeviceBytes:
    """A device byte range as a torch tensor view (no copy), through the CUDA
    array interface."""

    def __init__(self, ptr: int, n: int):
        self.__cuda_array_interface__ = {"shape": (int(n),), "typestr": "|u1", "data": (int(ptr), False),
                                         "version": 2, "strides": None}


def same_bytes(ptr: int, n: int, host) -> bool:
    """Whether n device bytes at ptr equal the host array, compared in
    256 MiB slices (no full-size host copy)."""
    import numpy as np
    import torch

    if host.size != n:
        return False
    if n == 0:
        return True
    view = torch.as_tensor(_DeviceBytes(ptr, n), device="cuda")
    step = 1 << 28
    for a in range(0, n, step):
        if not np.array_equal(view[a:a + step].cpu().numpy(), host[a:a + step]):
            return False
    return True


def oracle_bam(st, bgzf):
    """The oracle's decode of the whole file (threaded inflate with CRC32/ISIZE
    checks, serial scan, columns, virtual offsets, aux directory), sized from
    the run it will check; (decode or None, error, seconds)."""
    from oracle import oracle

    t0 = time.perf_counter()
    try:
        want = oracle.decode_bam_file_mt(bgzf, os.cpu_count() or 1, st.records, st.aux_fields, st.inflated_bytes)
        return want, None, time.perf_counter() - t0
    except RuntimeError as e:
        return None, str(e), time.perf_counter() - t0


def parity_bam(eng, st, want, error: str | None, oracle_s: float) -> dict:
    """Bit-exactness of the timed run at its full size: the engine's inflated
    bytes, every column, the virtual offsets, the aux directory and the tail
    against the oracle's decode of the same file.  Runs after the timed
    region."""
    import numpy as np

    import fritillaria_gb300 as frt

    t0 = time.perf_counter()
    if want is None:
        return {"checked": True, "match": False, "mismatch": [error], "seconds": round(oracle_s, 1)}
    bad = []
    ptr, n = eng.inflated_ptr()
    if not same_bytes(ptr, n, want["inflated"]):
        bad.append("inflated bytes")
    if st.records != len(want["columns"]["pos"]):
        bad.append("record count")
    if st.tail != want["tail"]:
        bad.append("tail")
    names = list(frt.BAM_COLUMNS)
    for name in names:
        if not np.array_equal(eng.column(name), want["columns"][name]):
            bad.append(name)
    if not np.array_equal(eng.column("aux_entries"), want["aux_entries"]):
        bad.append("aux_entries")
    return {"checked": True, "match": not bad, "columns": len(names) + 1, "records": len(want["columns"]["pos"]),
            "inflated_bytes": int(want["inflated"].size), "aux_entries": int(want["aux_entries"].size),
            "mismatch": bad, "seconds": round(oracle_s + time.perf_counter() - t0, 1),
            "against": "oracle whole-file decode (zlib inflate + CRC32/ISIZE on every member, serial scan_records, "
                       "RecordBatch::decode columns, virtual offsets, aux directory)"}


def reference_cuda(hbuf, want, inflated: int, blocks_per_batch: int = 256, sample_gb: float = 0.5) -> dict:
    """The reference's own CUDA kernels, compiled from its sources for sm_103a
    and driven in its launch order (reader batches of blocks_per_batch x 64 KiB
    compressed, inflate_blocks a thread per member, host verification,
    bam_scan_blocks, bam_reconcile<<<1,1>>>, emit, decode_fields) from the same
    pinned host bytes as the plain arm.  Its one-thread-per-member inflate
    runs at tens of MB/s, so it takes a bounded sample: the batches that start
    within the first sample_gb of inflated bytes' worth of compressed input
    (the whole file when it is smaller).  One run is checked against the
    oracle's records of that prefix, then one is timed."""
    import numpy as np

    from oracle import ref_cuda

    why = ref_cuda.available()
    if why:
        return {"unavailable": why}
    ratio = inflated / max(1, hbuf.size)
    stop = 0 if inflated <= sample_gb * 1e9 else int(sample_gb * 1e9 / ratio)
    out = {"unit": "GB/s", "members_per_batch": blocks_per_batch,
           "form": "reference kernels inflate.cu + bam_decode.cu (nvcc, sm_103a) under a C++ restatement of "
                   "DeviceBgzfReader + CudaCodec + BamDecoder (oracle/ref_cuda_driver.cpp); wall time of the "
                   "loop from pinned host memory",
           "sample": "whole file" if not stop else f"the batches starting in the first {stop} compressed bytes"}
    try:
        n = 0 if want is None else len(want["columns"]["pos"])
        res, cols = ref_cuda.run_bam(hbuf, blocks_per_batch, columns_cap=n + 16 if n else 0, stop_after=stop)
        if want is not None:
            k = int(res.records)
            ok = k <= n and np.array_equal(cols["record_offsets"], want["columns"]["record_offsets"][:k])
            for c in ("ref_id", "pos", "flags", "seq_len"):
                ok = ok and np.array_equal(cols[c], want["columns"][c][:k])
            out["matches_oracle"] = bool(ok and (stop or k == n))
            del cols
        res, _ = ref_cuda.run_bam(hbuf, blocks_per_batch, stop_after=stop)
    except RuntimeError as e:
        return {"unavailable": f"the reference's CUDA path failed: {e}"}
    out.update({"value": round(res.consumed_bytes / res.seconds / 1e9, 4), "seconds": round(res.seconds, 3),
                "records": int(res.records), "inflated_bytes": int(res.consumed_bytes), "batches": int(res.batches),
                "inflate_kernel_ms": round(res.inflate_ms, 2), "reconcile_kernel_ms": round(res.reconcile_ms, 2),
                "kernels_ms": round(res.kernels_ms, 2),
                "reinflated_bytes": int(res.inflated_bytes - res.consumed_bytes)})
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import oracle

    threads = os.cpu_count() or 1
    if args.workload in SERVING:
        import numpy as np

        from oracle import bai as obai

        w = SERVING[args.workload]
        files, reqs = generate_serving(args.workload)
        idx = [obai.parse(x) for _, x, _ in files]
        spans = [oracle.discover(b)[0] for b, _, _ in files]
        sample = reqs[: w["plain_requests"]]
        svc, nbytes = [], 0
        for a, f, ref, s0, e0 in sample:
            t = time.perf_counter()
            _, nb = oracle.region_query(files[f][0], spans[f], idx[f], ref, s0, e0)
            svc.append(1e3 * (time.perf_counter() - t))
            nbytes += nb
        total_s = sum(svc) / 1e3
        line = {"impl": "reference", "metric": METRIC, "value": round(nbytes / total_s / 1e9, 3), "unit": "GB/s",
                "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": round(1e3 * total_s, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
                "config": {"workload": args.workload, "description": w["desc"], "requests": len(sample)},
                "serving": {"requests_per_s": round(len(sample) / total_s, 1),
                            "service_p50_ms": round(float(np.percentile(svc, 50)), 3),
                            "service_p99_ms": round(float(np.percentile(svc, 99)), 3)},
                "cpu_baseline": {"value": round(nbytes / total_s / 1e9, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                                 "sample": f"the first {len(sample)} requests of the stream, served one at a time: "
                                           "BAI chunks, zlib inflate of the chunk members, record scan and filter"},
                "e2e": {"value": round(nbytes / total_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.workload in MIXED:
        files = generate_mixed(args.workload)
        fmt = {"bcf": 1, "fastq": 2, "fasta": 3}
        times, total = [], 0
        for i in range(args.warmup + args.steps):
            secs, total, records, members = 0.0, 0, 0, 0
            for name, _, bgzf in files:
                r = oracle.baseline_file(bgzf, fmt[name], threads)
                secs, total, records = secs + r.seconds, total + r.inflated_bytes, records + r.records
                members += r.members
            if i >= args.warmup:
                times.append(secs)
        gbs = total * len(times) / sum(times) / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * sum(times) / len(times), 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
                "config": mixed_config(args.workload, members, sum(f[2].size for f in files), total, world),
                "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                                 "cpu_model": cpu_model(), "nproc": threads, "records": records,
                                 "sample": "the three whole files per step; C restatement of the noodles CPU path "
                                           "(multithreaded BGZF inflate + serial scan/decode per format)"},
                "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                        "note": "a CPU arm: the input and the columns stay in host memory, so no copy is declared"}}
        print(json.dumps(line), flush=True)
        return
    bgzf = generate(args.workload)
    times = []
    res = None
    for i in range(args.warmup + args.steps):
        res = oracle.baseline_bam(bgzf, threads)
        if i >= args.warmup:
            times.append(res.seconds)
    total = sum(times)
    gbs = res.inflated_bytes * len(times) / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * total / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": bam_config(args.workload, res.records, res.members, len(bgzf), res.inflated_bytes, world),
        "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(), "nproc": threads,
                         "sample": "whole file per step; C restatement of the noodles CPU path (the reference's "
                                   "Rust CPU path cannot be built here: no Rust toolchain)"},
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                "note": "a CPU arm: the input and the columns stay in host memory, so no copy is declared"},
    }
    print(json.dumps(line), flush=True)


def run_plain(frt, host_bytes, blocks_per_batch=256):
    """The drop-in per-batch loop (crates/fritillaria-cuda/tests/bam_reader.rs:76-115)."""
    codec = frt.CudaCodec(0)
    decoder = frt.BamDecoder(0)
    t0 = time.perf_counter()
    reader = frt.DeviceBgzfReader(host_bytes, codec, blocks_per_batch=blocks_per_batch)
    header = None
    records = 0
    inflated = 0
    batches = 0
    while True:
        batch = reader.next_batch()
        if batch is None:
            break
        batches += 1
        inflated += batch.data.byte_len()
        if header is None:
            # the header is parsed on the host from the first batch, as the
            # reference's consumer loop does
            try:
                header = frt.parse_header(batch.data.to_host())
            except frt.Malformed:
                reader.carry_from(0)
                continue
            decoder.set_reference_count(header[1])
            begin = header[0]
        else:
            begin = batch.start
        rb = decoder.decode(batch.data, begin)
        records += len(rb)
        tail = rb.tail()
        rb.free()
        reader.carry_from(tail)
    dt = time.perf_counter() - t0
    return records, inflated, dt, batches


def record_fields(eng, records: int, peak: float) -> dict:
    """The opt-in record-field kernels over the engine's records, each timed
    once after a warm-up call (wall time of the call, result allocation and
    totals read-back included), with the bytes each must read and write."""
    import numpy as np
    import torch

    out = {}
    seq = eng.column("seq_len").astype(np.uint64)
    n_fields = int(eng.column("aux_count").astype(np.uint64).sum())
    bases = int(seq.sum())
    payload = int((eng.column("record_end").astype(np.int64) - 36).sum())
    # per record: the columns read (record offset, starts, counts), the aux
    # directory entries scanned (12 B each), the value or op bytes, the row written
    algo = {"aux_lookup NM": records * (8 + 4 + 4 + 1 + 4 + 23) + 12 * n_fields,
            "cigar_resolved": records * (8 + 2 + 4 + 4 + 8 + 13),
            "unpack_sequences": bases // 2 + bases + records * (8 + 4 + 4 + 8 + 8),
            "compact": 2 * payload + records * (8 + 6 * 4 + 5 * 8)}
    calls = {"aux_lookup NM": lambda: eng.aux_lookup("NM"), "cigar_resolved": eng.cigar_resolved,
             "unpack_sequences": eng.unpack_sequences, "compact": eng.compact}
    for name, fn in calls.items():
        fn().free()  # warm: allocator pools, module load
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = fn()
        res.column_ptr(next(iter(res._cols)))
        torch.cuda.synchronize()
        ms = 1e3 * (time.perf_counter() - t0)
        res.free()
        gbs = algo[name] / (ms / 1e3) / 1e9
        out[name] = {"ms": round(ms, 3), "algorithmic_bytes": algo[name], "gbs": round(gbs, 2),
                     "hbm_frac": round(gbs / peak, 4)}
    return out


def write_side(frt, eng, bgzf, no_cpu: bool) -> dict:
    """The write side over the engine's inflated bytes: DeviceCompressor
    (the reference's DeviceBlockCompressor contract) in 65,280-byte chunks,
    16,384 chunks a call into pinned host memory, wall time of the calls; and
    zlib on the host cores over a sample of the same chunks."""
    import concurrent.futures
    import zlib

    import numpy as np
    import torch

    ptr, n = eng.inflated_ptr()
    comp = frt.DeviceCompressor(0)
    bounds = np.append(np.arange(0, n, frt.DEFAULT_PAYLOAD_SIZE, dtype=np.uint64), np.uint64(n))
    per = 16384
    pinned = torch.empty(per * 65536, dtype=torch.uint8).pin_memory().numpy()
    comp.compress_batch_device(ptr, n, bounds[:1025], out=pinned)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    total = 0
    for s0 in range(0, len(bounds) - 1, per):
        total += comp.compress_batch_device(ptr, n, bounds[s0:s0 + per + 1], out=pinned).byte_len()
    secs = time.perf_counter() - t0
    out = {"input_bytes": int(n), "output_bytes": int(total), "ratio": round(n / total, 3), "ms": round(1e3 * secs, 2),
           "gbs": round(n / secs / 1e9, 2), "blocks": int(len(bounds) - 1),
           "form": "DeviceCompressor.compress_batch_device over the engine's inflated bytes, 65,280-byte chunks, "
                   "16,384 chunks a call, framed blocks copied to pinned host memory, wall time"}
    if not no_cpu:
        # the same bytes on the host: the file's first members, inflated by zlib
        spans, _ = frt.discover_blocks(bgzf[: 600 * 65536])
        parts, size = [], 0
        for sp in spans:
            a = int(sp["payload_start"])
            parts.append(zlib.decompress(bytes(bgzf[a:a + int(sp["payload_len"])]), -15))
            size += len(parts[-1])
            if size >= 512 * 65280:
                break
        host = np.frombuffer(b"".join(parts), np.uint8)[: 512 * 65280]
        chunks = [host[i:i + 65280].tobytes() for i in range(0, host.size, 65280)]
        threads = os.cpu_count() or 1
        res = {}
        for level in (1, 6):
            with concurrent.futures.ThreadPoolExecutor(threads) as ex:
                t0 = time.perf_counter()
                sizes = list(ex.map(lambda c: len(zlib.compress(c, level)), chunks))
                dt = time.perf_counter() - t0
            res[f"zlib{level}"] = {"gbs": round(host.size / dt / 1e9, 3), "ratio": round(host.size / sum(sizes), 3)}
        out["cpu_baseline"] = {"kind": "port", "cores": threads, "levels": res,
                               "sample": f"{len(chunks)} chunks of 65,280 bytes of the same inflated BAM, zlib "
                                         f"(Python's, releasing the GIL) on a pool of {threads} threads"}
    return out


def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import fritillaria_gb300 as frt

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    bgzf = generate(args.workload)
    host = torch.from_numpy(bgzf).pin_memory()
    dev = host.to("cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    eng = frt.BatchEngine(0, stream=stream.cuda_stream)
    eng.bind_bam(dev.data_ptr(), dev.numel())
    # the inflate tuning for this device and workload (from the cache, or
    # timed now); it also becomes the default the plain arm's codec starts from
    tuning = eng.autotune(args.tuning_cache, force=args.retune)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            eng.run()
            st = eng.finish()
        assert st.status == 0
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with Clocks(local) as clocks:
            t0 = time.perf_counter()
            ev0.record(stream)
            for _ in range(args.steps):
                eng.run()
                st = eng.finish()  # reads and checks the device error word
                if st.status != 0:
                    raise RuntimeError(f"engine status {st.status}")
            ev1.record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        ms = ev0.elapsed_time(ev1)
    ms = max_over_ranks(ms, dist, "cuda")
    if dist:
        dist.barrier()
    ms_step = ms / args.steps
    inflated = st.inflated_bytes
    value = whole_job_gbs(inflated, world, args.steps, ms)

    # stage breakdown and the roofline of the dominant kernel (inflate)
    front_ms, inflate_ms, records_ms = eng.time_stages(3)
    spans = frt.discover_blocks(bgzf)[0]
    payload = int(spans["payload_len"].astype(np.uint64).sum())
    col_bytes = 0
    for name in frt.BAM_COLUMNS:
        col_bytes += eng.column_ptr(name)[1]
    col_bytes += eng.column_ptr("aux_entries")[1]
    peak, peak_kind = peaks()
    inflate_bytes = payload + inflated
    achieved = inflate_bytes / (inflate_ms / 1e3) / 1e9
    traffic = None
    tp = ROOT / "profiles" / "inflate_traffic.json"
    if tp.exists():
        d = json.loads(tp.read_text())
        if d.get("workload") == args.workload:
            traffic = d.get("traffic_bytes_per_launch")
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": traffic, "issue": issue_model(frt, eng, inflated, inflate_ms) if args.workload.startswith("short_reads") else None,
                "kernel": "k_inflate_persistent (persistent warp-per-member inflate + CRC32/ISIZE verify)",
                "algorithmic_bytes_per_launch": inflate_bytes, "kernel_ms": round(inflate_ms, 3),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "pipeline": {"bytes": len(bgzf) + inflated + col_bytes, "ms": round(ms_step, 3),
                             "frac": round((len(bgzf) + inflated + col_bytes) / (ms_step / 1e3) / 1e9 / peak, 5)},
                "stages_ms": {"discover_plan_queue": round(front_ms, 3), "inflate_verify": round(inflate_ms, 3),
                              "records_columns": round(records_ms, 3)}}

    # e2e through the C ABI from pinned host memory
    e2e_steps = max(3, min(args.steps, 5))
    hbuf = host.numpy()
    for _ in range(1):
        eng.run_host(hbuf)
    torch.cuda.synchronize()
    steps_ms = []
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        st2 = eng.run_host(hbuf)
        steps_ms.append(round(1e3 * (time.perf_counter() - t1), 3))
        assert st2.status == 0
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist, "cuda")
    e2e = {"value": round(whole_job_gbs(inflated, world, 1, 1e3 * e2e_s), 3), "unit": "GB/s", "h2d_bytes_per_step": len(bgzf),
           "d2h_bytes_per_step": 128, "ms_per_step": round(1e3 * e2e_s, 3), "step_ms": steps_ms}

    fields = record_fields(eng, st.records, peak) if rank == 0 and not args.no_fields else None
    write = write_side(frt, eng, bgzf, args.no_cpu) if rank == 0 and not args.no_write else None

    plain = None
    if not args.no_plain:
        sweep = []
        for bpb in PLAIN_BATCHES:
            run_plain(frt, hbuf, bpb)  # warm
            recs, infl, dt, batches = run_plain(frt, hbuf, bpb)
            # the file's inflated bytes (members carried into the next batch
            # are inflated twice; that work is not counted as output)
            sweep.append({"members_per_batch": bpb, "value": round(inflated / dt / 1e9, 3), "batches": batches,
                          "records": recs, "reinflated_bytes": int(infl - inflated)})
        head = sweep[0]
        plain = {"value": head["value"], "unit": "GB/s", "records": head["records"], "batches": head["batches"],
                 "members_per_batch": PLAIN_BATCHES[0], "note": "per-batch reader+decoder from pinned host memory; "
                                                                "compare with e2e",
                 "batched_e2e_over_plain": round((inflated / e2e_s) / (head["value"] * 1e9), 2),
                 "sweep": sweep,
                 "sweep_note": "the same loop with larger batches (more members in flight per launch): what the "
                               "batch size alone buys, against what the persistent kernel, the sorted queue and "
                               "the graph add on top"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(bgzf, inflated)
    parity = ref_cu = None
    if rank == 0:
        want, error, oracle_s = oracle_bam(st, bgzf)
        parity = parity_bam(eng, st, want, error, oracle_s)
        if not args.no_plain:
            ref_cu = reference_cuda(hbuf, want, inflated)
        del want

    if rank == 0:
        w = WORKLOADS[args.workload]
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": bam_config(args.workload, st.records, st.members, len(bgzf), inflated, world),
            "engine": {"aux_fields": st.aux_fields, "column_bytes": col_bytes, "speculation_fallbacks": st.fallbacks,
                       "queue": "sorted by compressed size", "graph": True,
                       "records_per_s": round(world * st.records * args.steps / (ms / 1e3), 1), "tuning": tuning},
            "parity": parity,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "plain": plain,
            "reference_cuda": ref_cu,
            "record_fields": fields,
            "write_side": write,
            "gpu_launches": eng.launches_per_run() * args.steps,
            "clocks": clocks.summary(),
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)
        if parity is not None and not parity["match"]:
            print(f"parity mismatch: {parity['mismatch']}", file=sys.stderr, flush=True)
            sys.exit(1)
    if dist:
        dist.destroy_process_group()


def parity_mixed(eng, files) -> dict:
    """Bit-exactness of the mixed-format run at its full size: each file's
    inflated bytes and every column of its decoder against the oracle (the
    threaded inflate with CRC32/ISIZE checks, then the format's CPU scan and
    decode).  Runs after the timed region."""
    import numpy as np

    from oracle import oracle

    t0 = time.perf_counter()
    threads = os.cpu_count() or 1
    ptr, _ = eng.inflated_ptr()
    bad, per = [], {}
    for i, (name, _, bgzf) in enumerate(files):
        info = eng.file_info(i)
        try:
            raw = oracle.inflate_file(bgzf, threads, int(info.inflated_bytes))
        except RuntimeError as e:
            bad.append(f"{name}: {e}")
            continue
        if not same_bytes(ptr + int(info.inflated_offset), int(info.inflated_bytes), raw):
            bad.append(f"{name}: inflated bytes")
        res = eng.file_result(i)
        if name == "bcf":
            rs, ns, nc = oracle.bcf_header(raw)
            want = oracle.bcf_decode(raw, rs, ns, nc)
            cols, tail, n = want["columns"], want["tail"], len(want["columns"]["position"])
        elif name == "fastq":
            want = oracle.fastq_decode(raw, 0, cap=4 * int(info.records) + 1024)
            cols, tail, n = want["columns"], want["tail"], len(want["columns"]["record_offsets"])
        else:
            want = oracle.fasta_compact(raw, cap=int(info.records) + 1024)
            cols = {k: want[k] for k in ("sequence", "sequence_offsets", "sequence_lengths", "record_offsets")}
            tail, n = want["sequence"].size, len(want["record_offsets"])
        if info.records != n:
            bad.append(f"{name}: record count")
        if info.tail != tail:
            bad.append(f"{name}: tail")
        for k, v in cols.items():
            if k == "sequence":
                p, nb, _ = res.column_ptr(k)
                ok = same_bytes(p, nb, v)
            else:
                ok = np.array_equal(res.column(k), v)
            if not ok:
                bad.append(f"{name}: {k}")
        per[name] = {"records": int(n), "columns": len(cols), "inflated_bytes": int(raw.size)}
        del raw, want, cols
    return {"checked": True, "match": not bad, "files": per, "columns": sum(v["columns"] for v in per.values()),
            "mismatch": bad, "seconds": round(time.perf_counter() - t0, 1),
            "against": "oracle: threaded zlib inflate + CRC32/ISIZE of every member, then the reference's CPU scan "
                       "and decode per format (BCF chain + site core, FASTQ scan + bounds, FASTA compaction)"}


def mixed_config(workload: str, members: int, compressed: int, inflated: int, world: int) -> dict:
    """The mixed workload as both arms report it (the same keys and values)."""
    return {"workload": workload, "description": MIXED[workload]["desc"], "members": int(members),
            "compressed_bytes": int(compressed), "inflated_bytes": int(inflated),
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}


def generate_mixed(name: str):
    """[(format name, raw bytes, bgzf bytes)] for the mixed-format workload."""
    from fritillaria_gb300 import synth

    w = MIXED[name]
    files = []
    raw, bgzf = synth.bcf(w["bcf_sites"], n_samples=w["bcf_samples"], n_contigs=24, seed=61, levels=(6, 6))
    files.append(("bcf", raw.size, bgzf))
    del raw
    raw, bgzf = synth.fastq(w["fastq_reads"], seed=62, levels=(6, 6))
    files.append(("fastq", raw.size, bgzf))
    del raw
    raw, bgzf = synth.fasta(24, w["fasta_bases"], 60, False, seed=63, levels=(6, 6))
    files.append(("fasta", raw.size, bgzf))
    del raw
    return files


def text_framing(args, frt, w, peak):
    """TextScanner over a bgzipped VCF inflated on the device: the scan's wall
    time per batch (its read-backs make it host-synchronous), the HBM
    fraction of its algorithmic bytes (the text read once, the five columns
    written) and the oracle's numpy restatement on the same bytes."""
    import numpy as np
    import torch

    from fritillaria_gb300 import synth

    raw, bgz = synth.vcf_text(w["vcf_sites"], w["vcf_samples"], seed=64)
    spans, _ = frt.discover_blocks(bgz)
    batch = frt.CudaCodec(0).inflate_batch_device(bgz, spans)
    scanner = frt.TextScanner(0)
    for _ in range(3):
        out = scanner.scan(batch, 0, frt.Dialect.VCF)
    torch.cuda.synchronize()
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        out = scanner.scan(batch, 0, frt.Dialect.VCF)
    torch.cuda.synchronize()
    ms = 1e3 * (time.perf_counter() - t0) / reps
    col_bytes = sum(out.column_ptr(k)[1] for k in out._cols)
    algo = raw.size + col_bytes
    # columnar VCF over the scan: the fixed fields of every record
    dec = frt.VcfDecoder(0)
    head = bytes(raw[: int(out.column("record_offsets")[0])]) if len(out) else b""
    n_contigs = dec.set_contigs_from_header(head)
    cols = dec.decode(out)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        cols = dec.decode(out)
    torch.cuda.synchronize()
    vcf_ms = 1e3 * (time.perf_counter() - t0) / reps
    vcf_ok = int((cols.column("status") == 0).sum())
    gt = dec.genotypes(out)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        gt = dec.genotypes(out)
    torch.cuda.synchronize()
    gt_ms = 1e3 * (time.perf_counter() - t0) / reps
    n_calls = int(out.column_ptr("tabs")[1] // 8) - 8 * len(out)
    called = int(((gt.column("calls") >> 28) == 0).sum()) - 8 * len(out)  # tabs before FORMAT hold 0
    # per call: the sample's bytes read (about 4) and its u32 written; per record its tabs read
    gt_algo = raw.size + 4 * n_calls + 8 * n_calls
    res = {"text_bytes": int(raw.size), "compressed_bytes": int(bgz.size), "records": len(out),
           "header_lines": int(out.scan_info()[0]), "tabs": int(out.column_ptr("tabs")[1] // 8),
           "column_bytes": int(col_bytes), "scan_ms": round(ms, 3),
           "scan_gbs": round(raw.size / (ms / 1e3) / 1e9, 2),
           "hbm_frac": round(algo / (ms / 1e3) / 1e9 / peak, 4),
           "form": "wall time per TextScanner.scan on a resident inflated batch, 20 scans after 3 warm-ups",
           "vcf_decode": {"ms": round(vcf_ms, 4), "records_ok": vcf_ok, "contigs": n_contigs,
                          "records_per_s": round(len(out) / (vcf_ms / 1e3)),
                          "form": "wall time per VcfDecoder.decode over the scan's columns (CHROM index, POS, "
                                  "field bounds, ALT count, QUAL, flags, status)"},
           "genotypes": {"ms": round(gt_ms, 4), "calls": n_calls, "called": called,
                         "calls_per_s": round(n_calls / (gt_ms / 1e3)),
                         "hbm_frac": round(gt_algo / (gt_ms / 1e3) / 1e9 / peak, 4),
                         "algorithmic_bytes": gt_algo,
                         "form": "wall time per VcfDecoder.genotypes: every sample's GT as a packed u32 "
                                 "(algorithmic bytes: the text read, the 8-byte tabs read, a u32 per call)"}}
    if not args.no_cpu:
        from oracle import text

        t0 = time.perf_counter()
        want = text.device_scan(raw, 0, text.VCF)
        secs = time.perf_counter() - t0
        assert len(out) == want["record_offsets"].size and np.array_equal(out.column("tabs"), want["tabs"])
        res["cpu_baseline"] = {"value": round(raw.size / secs / 1e9, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                               "sample": "the whole VCF text through oracle/text.py device_scan (numpy)"}
    return res


def run_mixed(args, rank, world, local):
    import numpy as np
    import torch

    import fritillaria_gb300 as frt

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    files = generate_mixed(args.workload)
    blob = np.concatenate([f[2] for f in files])
    host = torch.from_numpy(blob).pin_memory()
    dev = host.to("cuda")
    fmt = {"bam": frt.Format.BAM, "bcf": frt.Format.BCF, "fastq": frt.Format.FASTQ, "fasta": frt.Format.FASTA}
    layout, at = [], 0
    for name, _, bgzf in files:
        layout.append((at, bgzf.size, fmt[name]))
        at += bgzf.size
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    eng = frt.BatchEngine(0, stream=stream.cuda_stream)
    eng.bind_files(dev.data_ptr(), dev.numel(), layout)
    tuning = eng.autotune(args.tuning_cache, force=args.retune)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            eng.run()
            st = eng.finish()
        assert st.status == 0
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        with Clocks(local) as clocks:
            t0 = time.perf_counter()
            ev0.record(stream)
            for _ in range(args.steps):
                eng.run()
                st = eng.finish()
                if st.status != 0:
                    raise RuntimeError(f"engine status {st.status}")
            ev1.record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        ms = ev0.elapsed_time(ev1)
    ms = max_over_ranks(ms, dist, "cuda")
    if dist:
        dist.barrier()
    ms_step = ms / args.steps
    inflated = st.inflated_bytes
    value = whole_job_gbs(inflated, world, args.steps, ms)

    # each stage and each file's decode: the median of five eager runs
    stage_runs, file_runs = [], [[] for _ in files]
    for _ in range(5):
        stage_runs.append(eng.time_stages(1))
        for i in range(len(files)):
            file_runs[i].append(eng.file_info(i).decode_ms)
    front_ms, inflate_ms, decode_ms = (statistics.median(x) for x in zip(*stage_runs))
    per = {}
    col_bytes = 0
    launches = 0
    for i, (name, raw_size, bgzf) in enumerate(files):
        info = eng.file_info(i)
        info.decode_ms = statistics.median(file_runs[i])
        res = eng.file_result(i)
        cb = sum(res.column_ptr(k)[1] for k in res._cols)
        col_bytes += cb
        launches += info.launches
        algo = info.inflated_bytes + cb  # read the inflated file, write its columns
        per[name] = {"compressed_bytes": int(info.compressed_bytes), "inflated_bytes": int(info.inflated_bytes),
                     "records": int(info.records), "decode_ms": round(info.decode_ms, 3),
                     "decode_gbs": round(info.inflated_bytes / (info.decode_ms / 1e3) / 1e9, 2) if info.decode_ms else None,
                     "column_bytes": int(cb), "proof": int(info.proof),
                     "decode_hbm_frac": round(algo / (info.decode_ms / 1e3) / 1e9 / peaks()[0], 4) if info.decode_ms else None}
    peak, peak_kind = peaks()
    payload = sum(int(frt.discover_blocks(f[2])[0]["payload_len"].astype(np.uint64).sum()) for f in files)
    inflate_bytes = payload + inflated
    achieved = inflate_bytes / (inflate_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "traffic": None,
                "kernel": "k_inflate_persistent (one persistent inflate over the members of all three files)",
                "algorithmic_bytes_per_launch": inflate_bytes, "kernel_ms": round(inflate_ms, 3),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "pipeline": {"bytes": blob.size + inflated + col_bytes, "ms": round(ms_step, 3),
                             "frac": round((blob.size + inflated + col_bytes) / (ms_step / 1e3) / 1e9 / peak, 5)},
                "stages_ms": {"discover_plan_queue": round(front_ms, 3), "inflate_verify": round(inflate_ms, 3),
                              "decoders": round(decode_ms, 3)}}

    e2e_steps = max(3, min(args.steps, 5))
    hbuf = host.numpy()
    eng.run_host(hbuf)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        st2 = eng.run_host(hbuf)
        assert st2.status == 0
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist, "cuda")
    e2e = {"value": round(whole_job_gbs(inflated, world, 1, 1e3 * e2e_s), 3), "unit": "GB/s",
           "h2d_bytes_per_step": int(blob.size), "d2h_bytes_per_step": 128, "ms_per_step": round(1e3 * e2e_s, 3)}

    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle

        threads = os.cpu_count() or 1
        secs, nbytes, parts = 0.0, 0, {}
        for name, _, bgzf in files:
            r = oracle.baseline_file(bgzf, int(fmt[name]), threads)
            secs += r.seconds
            nbytes += r.inflated_bytes
            parts[name] = {"seconds": round(r.seconds, 3), "records": int(r.records)}
        cpu = {"value": round(nbytes / secs / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"whole files: {parts}; C restatement of the noodles multithreaded BGZF reader (zlib 1.3 "
                         f"inflate + CRC32 on all cores) then the reference's serial CPU scan/decode per format"}

    parity = parity_mixed(eng, files) if rank == 0 else None

    if rank == 0:
        w = MIXED[args.workload]
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": mixed_config(args.workload, st.members, blob.size, inflated, world),
            "engine": {"records": int(st.records), "column_bytes": int(col_bytes), "files": per,
                       "queue": "sorted by compressed size", "graph": "discovery + plan + inflate", "tuning": tuning},
            "parity": parity,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "text_framing": text_framing(args, frt, w, peak),
            "gpu_launches": eng.launches_per_run() * args.steps,
            "clocks": clocks.summary(),
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)
        if not parity["match"]:
            print(f"parity mismatch: {parity['mismatch']}", file=sys.stderr, flush=True)
            sys.exit(1)
    if dist:
        dist.destroy_process_group()


def generate_serving(name: str):
    """Files (bgzf, bai, contig lengths) and the request stream."""
    import numpy as np

    from fritillaria_gb300 import synth

    w = SERVING[name]
    rng = np.random.default_rng(2024)
    lo, hi = np.log(w["min_records"]), np.log(w["max_records"])
    sizes = np.exp(rng.uniform(lo, hi, w["files"])).astype(np.int64)
    files = []
    for i, n in enumerate(sizes):
        raw, bgzf = synth.short_read_bam(int(n), n_contigs=24, genome_len=3_100_000_000, seed=300 + i, levels=(1, 6))
        files.append((bgzf, synth.bai(raw, bgzf), int(n)))
        del raw
    # contig lengths of the generator (human proportions over 3.1 Gb)
    human = np.array([248956422, 242193529, 198295559, 190214555, 181538259, 170805979, 159345973, 145138636,
                      138394717, 133797422, 135086622, 133275309, 114364328, 107043718, 101991189, 90338345,
                      83257441, 80373285, 58617616, 64444167, 46709983, 50818468, 156040895, 57227415], float)
    contig_len = (3_100_000_000 * human / human.sum()).astype(np.int64)
    n = w["requests"]
    arrivals = np.cumsum(rng.exponential(1000.0 / w["rate"], n))  # ms
    reqs = []
    for k in range(n):
        f = int(rng.integers(0, w["files"]))
        ref = int(rng.integers(0, 24))
        length = int(np.exp(rng.uniform(np.log(1_000), np.log(10_000_000))))
        start = int(rng.integers(1, max(2, contig_len[ref] - length)))
        reqs.append((float(arrivals[k]), f, ref, start, start + length - 1))
    return files, reqs


def serve_stream(frt, srv, ids, reqs):
    """Submits each request at its arrival time and drives the server until
    all complete; returns per-request (arrival, done, bytes, records)."""
    t0 = srv.clock_ms()
    rids, k = [], 0
    while k < len(reqs):
        now = srv.clock_ms() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            a, f, ref, s, e = reqs[k]
            rids.append(srv.submit(ids[f], ref, s, e, arrival_ms=t0 + a))
            k += 1
        srv.progress()
    srv.drain()
    out = []
    for rid in rids:
        srv.check(rid)
        i = srv.info(rid)
        out.append((i.arrival_ms, i.done_ms, i.inflated_bytes, i.records, i.retries))
    for rid in rids:
        srv.release(rid)
    return out


def latency_summary(rows):
    import numpy as np

    lat = np.array([d - a for a, d, _, _, _ in rows])
    span = max(d for _, d, _, _, _ in rows) - min(a for a, _, _, _, _ in rows)
    nbytes = sum(b for _, _, b, _, _ in rows)
    return {"requests": len(rows), "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3), "mean_ms": round(float(lat.mean()), 3),
            "span_ms": round(span, 3), "inflated_bytes": int(nbytes),
            "gbs": round(nbytes / (span / 1e3) / 1e9, 3) if span > 0 else None,
            "records": int(sum(r for _, _, _, r, _ in rows)), "retries": int(sum(t for *_, t in rows)),
            "completed_per_s": round(len(rows) / (span / 1e3), 1) if span > 0 else None}


def tick_breakdown(st: dict) -> dict:
    """Mean per-tick stage times of a serving run (frt_server_get_stats)."""
    n = max(1, st["ticks"])
    return {"ticks": st["ticks"], "requests_per_tick": round(st["requests"] / n, 1),
            "members_per_tick": round(st["members"] / n, 1), "host_ms": round(st["host_ms"] / n, 3),
            "upload_and_wait_ms": round(st["upload_ms"] / n, 3), "inflate_ms": round(st["inflate_ms"] / n, 3),
            "scan_emit_ms": round(st["scan_ms"] / n, 3), "max_inflate_ms": st["max_inflate_ms"]}


def issue_model(frt, eng, inflated: int, inflate_ms: float) -> dict | None:
    """The inflate's second roofline: it is a serial Huffman chain per member,
    so its bound is instruction issue, not HBM.  Warp instructions and DEFLATE
    symbols per inflated byte come from the ncu capture and the symbol count in
    profiles/inflate_issue.json; the issue peak is SMs x 4 schedulers x the SM
    clock.  Also the chain model: warps in flight times each warp's symbol
    rate, against one warp alone on an SM."""
    ip = ROOT / "profiles" / "inflate_issue.json"
    if not ip.exists() or inflate_ms <= 0:
        return None
    d = json.loads(ip.read_text())
    per_byte = d["warp_instructions_per_launch"] / d["inflated_bytes_per_launch"]
    sym_per_byte = d["deflate_symbols_per_launch"] / d["inflated_bytes_per_launch"]
    secs = inflate_ms / 1e3
    peak = d["sms"] * d["schedulers_per_sm"] * d["sm_clock_hz"]
    instr = per_byte * inflated / secs
    t = eng.tuning
    warps = int(d["sms"]) * int(t.warps_per_cta) * max(1, frt.inflate_ctas_per_sm(t))
    sym = sym_per_byte * inflated / secs
    return {"achieved": round(instr / 1e12, 4), "peak": round(peak / 1e12, 4), "unit": "T warp instructions/s",
            "frac": round(instr / peak, 4), "instructions_per_symbol": round(per_byte / sym_per_byte, 1),
            "chain": {"warps_in_flight": warps, "symbols_per_s": round(sym / 1e9, 3),
                      "per_warp_symbols_per_s": round(sym / warps / 1e6, 3),
                      "lone_warp_symbols_per_s": round(d["lone_warp_symbols_per_s"] / 1e6, 3),
                      "unit": "G symbols/s (total), M symbols/s (per warp)"},
            "source": "profiles/inflate_issue.json (instructions and symbols per inflated byte of the 2M capture)"}


def run_serving(args, rank, world, local):
    import torch

    import fritillaria_gb300 as frt

    torch.cuda.set_device(local)
    w = SERVING[args.workload]
    files, reqs = generate_serving(args.workload)
    # the inflate tuning, from an engine over the first file: servers made
    # afterwards start from it
    dev0 = torch.from_numpy(files[0][0]).to("cuda")
    torch.cuda.synchronize()
    tune_eng = frt.BatchEngine(0)
    tune_eng.bind_bam(dev0.data_ptr(), dev0.numel())
    tuning = tune_eng.autotune(args.tuning_cache, force=args.retune)
    del tune_eng, dev0
    srv = frt.RegionServer(0, budget_bytes=w["budget"])
    ids = [srv.add_bam(b, x) for b, x, _ in files]
    # warm-up: a few requests through every stage
    serve_stream(frt, srv, ids, [(0.0,) + r[1:] for r in reqs[: max(3, args.warmup)]])
    srv.stats(reset=True)
    with Clocks(local) as clocks:
        t0 = time.perf_counter()
        rows = serve_stream(frt, srv, ids, reqs)
        wall = time.perf_counter() - t0
    batched = latency_summary(rows)
    batched["ticks"] = tick_breakdown(srv.stats(reset=True))
    # capacity: the whole stream offered at once
    cap_rows = serve_stream(frt, srv, ids, [(0.0,) + r[1:] for r in reqs])
    capacity = latency_summary(cap_rows)
    capacity["ticks"] = tick_breakdown(srv.stats(reset=True))
    # fewer ticks in flight than the server's default of four (each tick on
    # its own stream): one, where a request waits for the running tick, and two
    srv.set_limits(0, 1)
    one_rows = serve_stream(frt, srv, ids, reqs)
    one_tick = latency_summary(one_rows)
    one_tick["ticks"] = tick_breakdown(srv.stats(reset=True))
    srv.set_limits(0, 2)
    two_rows = serve_stream(frt, srv, ids, reqs)
    two_ticks = latency_summary(two_rows)
    two_ticks["ticks"] = tick_breakdown(srv.stats(reset=True))
    srv.set_limits(0, 4)
    # the plain per-request form: one request per tick, one tick in flight,
    # the same arrivals (a prefix of the stream: it cannot keep up)
    plain_srv = frt.RegionServer(0, budget_bytes=w["budget"])
    plain_ids = [plain_srv.add_bam(b, x) for b, x, _ in files]
    plain_srv.set_limits(1, 1)
    serve_stream(frt, plain_srv, plain_ids, [(0.0,) + r[1:] for r in reqs[:3]])
    prow = serve_stream(frt, plain_srv, plain_ids, reqs[: w["plain_requests"]])
    plain = latency_summary(prow)
    if rank == 0:
        line = {
            "metric": METRIC, "value": batched["gbs"], "unit": "GB/s", "n_gpus": world, "steps": 1,
            "warmup": args.warmup, "ms_per_step": batched["span_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": args.workload, "description": w["desc"], "files": len(files),
                       "records": int(sum(n for *_, n in files)),
                       "compressed_bytes": int(sum(b.size for b, _, _ in files)),
                       "offered_req_per_s": w["rate"], "budget_bytes": w["budget"],
                       "l2": "region requests are independent (no flush)", "parallelism": f"replicas x{world}",
                       "tuning": tuning},
            "serving": {"batched": batched, "capacity": capacity, "one_tick_in_flight": one_tick,
                        "two_ticks_in_flight": two_ticks,
                        "plain_per_request": plain,
                        "note": "latency = device completion of the request's tick - arrival; batched = every queued "
                                "request that fits the budget in a tick, four ticks in flight; plain = one request "
                                "per tick, one tick in flight, on the first requests of the same stream"},
            "roofline": None, "cpu_baseline": None,
            "e2e": {"value": batched["gbs"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "files resident on the device; results stay on the device"},
            "gpu_launches": None,
            "clocks": clocks.summary(),
            "wall_s": round(wall, 3),
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload in MIXED:
        run_mixed(args, rank, world, local)
        return
    if args.workload in SERVING:
        run_serving(args, rank, world, local)
        return
    run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
