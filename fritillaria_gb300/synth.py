"""Seeded synthetic inputs (native generator in ``csrc/synth.cpp``).

Workloads:
  * ``short_reads``: paired-end 2x150 bp, coordinate-sorted, NM/MD/RG tags --
    100k records on one 50 Mb contig, or 20M records over 24 contigs
    proportional to the human chromosomes (3.1 Gb);
  * ``ultra_long``: unaligned reads with log-normal lengths (median 15 kb,
    sigma 1.0, capped at 1 Mb) plus extra 250-800 kb reads, MM/ML/qs/ch tags.
Members are packed "full" (records straddle members, as the noodles writer
does) or "record" aligned (as htslib does), at one or two alternating levels.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent


class _Params(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_contigs", C.c_int32), ("n_records", C.c_uint64),
                ("genome_len", C.c_uint64), ("seed", C.c_uint64), ("threads", C.c_int32),
                ("n_long_extra", C.c_int32)]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _PKG / "libfrt_synth.so"
        if not path.exists():
            from fritillaria_gb300.build import build_synth
            build_synth()
        _lib = C.CDLL(str(path))
        _lib.frt_synth_bam.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.frt_synth_bgzf.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_uint32, C.c_void_p, C.c_size_t,
                                        C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.frt_synth_free.argtypes = [C.c_void_p]
        _lib.frt_synth_bai.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
        _lib.frt_synth_fastq.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
        _lib.frt_synth_bcf.argtypes = [C.c_uint64, C.c_uint32, C.c_int, C.c_uint64, C.c_int, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.frt_synth_fasta.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_int, C.c_uint64, C.c_int, C.c_void_p,
                                         C.c_void_p]
    return _lib


def _take(ptr: C.c_void_p, n: int) -> np.ndarray:
    arr = np.empty(n, dtype=np.uint8)
    if n:
        C.memmove(arr.ctypes.data, ptr, n)
    _load().frt_synth_free(ptr)
    return arr


def raw_bam(kind: str = "short_reads", n_records: int = 1000, n_contigs: int = 1, genome_len: int = 50_000_000,
            seed: int = 1, n_long_extra: int = 0, threads: int | None = None):
    """Uncompressed BAM bytes and the end offset of the header and of each
    record."""
    lib = _load()
    p = _Params(0 if kind == "short_reads" else 1, n_contigs, n_records, genome_len, seed,
                threads or os.cpu_count() or 1, n_long_extra)
    raw = C.c_void_p()
    raw_len = C.c_size_t()
    ends = C.c_void_p()
    n_ends = C.c_size_t()
    if lib.frt_synth_bam(C.byref(p), C.byref(raw), C.byref(raw_len), C.byref(ends), C.byref(n_ends)) != 0:
        raise MemoryError("synthetic BAM generation failed")
    data = _take(raw, raw_len.value)
    e = np.empty(n_ends.value, dtype=np.uint64)
    C.memmove(e.ctypes.data, ends, 8 * n_ends.value)
    lib.frt_synth_free(ends)
    return data, e


def bgzf(raw: np.ndarray, packing: str = "full", levels=(6, 6), record_ends=None, member_payload: int = 65495,
         threads: int | None = None) -> np.ndarray:
    """BGZF-compress `raw` into members (plus the EOF member)."""
    lib = _load()
    raw = np.ascontiguousarray(raw, dtype=np.uint8)
    mode = 0 if packing == "full" else 1
    if mode == 1 and record_ends is None:
        raise ValueError("record packing needs record_ends")
    ends = np.ascontiguousarray(record_ends if record_ends is not None else np.zeros(1), dtype=np.uint64)
    out = C.c_void_p()
    out_len = C.c_size_t()
    nm = C.c_uint64()
    payload = member_payload if mode == 0 else 65280
    rc = lib.frt_synth_bgzf(raw.ctypes.data, raw.size, mode, payload, ends.ctypes.data,
                            len(ends) if record_ends is not None else 0, levels[0], levels[1],
                            threads or os.cpu_count() or 1, C.byref(out), C.byref(out_len), C.byref(nm))
    if rc != 0:
        raise MemoryError("BGZF compression failed")
    return _take(out, out_len.value)


def short_read_bam(n_records: int, n_contigs: int = 1, genome_len: int = 50_000_000, seed: int = 1,
                   levels=(6, 6), packing: str = "full", member_payload: int = 65495):
    raw, ends = raw_bam("short_reads", n_records, n_contigs, genome_len, seed)
    return raw, bgzf(raw, packing, levels, ends, member_payload)


def ultra_long_bam(n_records: int, n_long_extra: int = 0, seed: int = 3, levels=(6, 6), packing: str = "full",
                   member_payload: int = 65495):
    raw, ends = raw_bam("ultra_long", n_records, 1, 0, seed, n_long_extra)
    return raw, bgzf(raw, packing, levels, ends, member_payload)


def bai(raw: np.ndarray, bgzf_bytes: np.ndarray) -> np.ndarray:
    """A BAI for a coordinate-sorted BAM: `raw` its uncompressed bytes,
    `bgzf_bytes` the BGZF file they were written as."""
    lib = _load()
    raw = np.ascontiguousarray(raw, dtype=np.uint8)
    bg = np.ascontiguousarray(bgzf_bytes, dtype=np.uint8)
    out = C.c_void_p()
    n = C.c_size_t()
    rc = lib.frt_synth_bai(raw.ctypes.data, raw.size, bg.ctypes.data, bg.size, C.byref(out), C.byref(n))
    if rc != 0:
        raise ValueError(f"BAI generation failed ({rc})")
    return _take(out, n.value)


def _with_ends(fn, *args):
    lib = _load()
    raw = C.c_void_p()
    raw_len = C.c_size_t()
    ends = C.c_void_p()
    n_ends = C.c_size_t()
    if fn(*args, C.byref(raw), C.byref(raw_len), C.byref(ends), C.byref(n_ends)) != 0:
        raise MemoryError("synthetic generation failed")
    data = _take(raw, raw_len.value)
    e = np.empty(n_ends.value, dtype=np.uint64)
    C.memmove(e.ctypes.data, ends, 8 * n_ends.value)
    lib.frt_synth_free(ends)
    return data, e


def raw_fastq(n_records: int, kind: str = "illumina", seed: int = 1, threads: int | None = None):
    """FASTQ text and the end offset of every record (first entry 0)."""
    return _with_ends(_load().frt_synth_fastq, 0 if kind == "illumina" else 1, n_records, seed,
                      threads or os.cpu_count() or 1)


def fastq(n_records: int, kind: str = "illumina", seed: int = 1, levels=(6, 6), packing: str = "full",
          member_payload: int = 65495):
    """(FASTQ text, bgzipped FASTQ)."""
    raw, ends = raw_fastq(n_records, kind, seed)
    return raw, bgzf(raw, packing, levels, ends, member_payload)


def raw_bcf(n_sites: int, n_samples: int = 500, n_contigs: int = 24, seed: int = 1, threads: int | None = None):
    """Uncompressed BCF (header + records) and the end offsets of the header
    and of every record."""
    return _with_ends(_load().frt_synth_bcf, n_sites, n_samples, n_contigs, seed, threads or os.cpu_count() or 1)


def bcf(n_sites: int, n_samples: int = 500, n_contigs: int = 24, seed: int = 1, levels=(6, 6),
        packing: str = "full", member_payload: int = 65280):
    """(uncompressed BCF, BGZF-compressed BCF); bcftools packs members full."""
    raw, ends = raw_bcf(n_sites, n_samples, n_contigs, seed)
    return raw, bgzf(raw, packing, levels, ends, member_payload)


def raw_fasta(n_contigs: int = 24, total_bases: int = 3_100_000_000, line_width: int = 60, blank_lines: bool = False,
              seed: int = 1, threads: int | None = None) -> np.ndarray:
    """FASTA text wrapped at `line_width` bases per line."""
    lib = _load()
    raw = C.c_void_p()
    raw_len = C.c_size_t()
    rc = lib.frt_synth_fasta(n_contigs, total_bases, line_width, int(blank_lines), seed,
                             threads or os.cpu_count() or 1, C.byref(raw), C.byref(raw_len))
    if rc != 0:
        raise ValueError("synthetic FASTA generation failed")
    return _take(raw, raw_len.value)


def fasta(n_contigs: int = 24, total_bases: int = 3_100_000_000, line_width: int = 60, blank_lines: bool = False,
          seed: int = 1, levels=(6, 6)):
    """(FASTA text, bgzipped FASTA)."""
    raw = raw_fasta(n_contigs, total_bases, line_width, blank_lines, seed)
    return raw, bgzf(raw, "full", levels)


def raw_vcf_text(n_sites: int, n_samples: int = 2504, n_contigs: int = 24, seed: int = 1) -> np.ndarray:
    """VCF 4.2 text of phased biallelic genotypes, shaped like a population
    panel: `##` meta lines, a `#CHROM` line naming every sample, then one line
    per site -- CHROM, sorted POS, ID, REF, ALT, QUAL, FILTER, INFO (AC, AN,
    AF, DP), FORMAT GT and a `a|b` genotype per sample, alleles drawn with the
    site's allele frequency (log-uniform 1e-4..0.5)."""
    rng = np.random.default_rng(seed)
    contigs = [f"chr{k + 1}" for k in range(n_contigs)]
    head = ["##fileformat=VCFv4.2", "##source=fritillaria_gb300.synth"]
    head += [f"##contig=<ID={c},length={250_000_000 - 7_000_000 * k}>" for k, c in enumerate(contigs)]
    head += ['##INFO=<ID=AC,Number=A,Type=Integer,Description="Alternate allele count">',
             '##INFO=<ID=AN,Number=1,Type=Integer,Description="Total allele number">',
             '##INFO=<ID=AF,Number=A,Type=Float,Description="Alternate allele frequency">',
             '##INFO=<ID=DP,Number=1,Type=Integer,Description="Combined depth">',
             '##FORMAT=<ID=GT,Number=1,Type=String,Description="Phased genotype">',
             "\t".join(["#CHROM", "POS", "ID", "REF", "ALT", "QUAL", "FILTER", "INFO", "FORMAT"]
                       + [f"S{i:05d}" for i in range(n_samples)])]
    parts = [np.frombuffer(("\n".join(head) + "\n").encode(), np.uint8)]
    per = np.bincount(np.sort(rng.integers(0, n_contigs, n_sites)), minlength=n_contigs)
    af = np.exp(rng.uniform(np.log(1e-4), np.log(0.5), n_sites))
    bases = "ACGT"
    chunk = 1024
    site = 0
    for k, c in enumerate(contigs):
        pos = np.sort(rng.choice(200_000_000, int(per[k]), replace=False)) + 1 if per[k] else []
        for lo in range(0, int(per[k]), chunk):
            m = min(chunk, int(per[k]) - lo)
            alt = (rng.random((m, 2 * n_samples)) < af[site:site + m, None]).astype(np.uint8)
            gt = np.empty((m, n_samples, 4), np.uint8)
            gt[:, :, 0] = alt[:, 0::2] + ord("0")
            gt[:, :, 1] = ord("|")
            gt[:, :, 2] = alt[:, 1::2] + ord("0")
            gt[:, :, 3] = ord("\t")
            gt[:, -1, 3] = ord("\n")
            gt = gt.reshape(m, 4 * n_samples)
            ac = alt.sum(axis=1)
            refs = rng.integers(0, 4, m)
            alts = (refs + rng.integers(1, 4, m)) % 4
            qual = rng.integers(20, 10_000, m)
            dp = rng.integers(5_000, 40_000, m)
            for i in range(m):
                p = int(pos[lo + i])
                line = (f"{c}\t{p}\trs{1_000_000 + site + i}\t{bases[refs[i]]}\t{bases[alts[i]]}\t{qual[i]}\tPASS\t"
                        f"AC={ac[i]};AN={2 * n_samples};AF={ac[i] / (2 * n_samples):.4g};DP={dp[i]}\tGT\t")
                parts.append(np.frombuffer(line.encode(), np.uint8))
                parts.append(gt[i])
            site += m
    return np.concatenate(parts)


def vcf_text(n_sites: int, n_samples: int = 2504, n_contigs: int = 24, seed: int = 1, levels=(6, 6)):
    """(VCF text, bgzipped VCF text), members packed full as bgzip does."""
    raw = raw_vcf_text(n_sites, n_samples, n_contigs, seed)
    return raw, bgzf(raw, "full", levels)


# The benchmark configurations.
CONFIGS = {
    "short_reads_100k": dict(n_records=100_000, n_contigs=1, genome_len=50_000_000, levels=(6, 6)),
    "short_reads_20m": dict(n_records=20_000_000, n_contigs=24, genome_len=3_100_000_000, levels=(1, 6)),
}
