/*
 * TEST INFRASTRUCTURE ONLY.  Drives the reference's kernels, compiled as host
 * C++ from their own sources (crates/fritillaria-cuda/kernels/*.cu), one
 * "thread" at a time, in the launch order of the reference's launchers
 * (crates/fritillaria-cuda/src/backend.rs:635-720, src/bam.rs:368-573).
 * Built by oracle/build.py into oracle/_ref/ only where the reference tree is
 * present; never shipped.
 */
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <utility>
#include <vector>

#include "ref_shim.h"

thread_local RefDim3 blockIdx = {0, 0, 0}, threadIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};

namespace ref_inflate {
#include "inflate.cu"
}
namespace ref_crc {
#include "crc32.cu"
}
namespace ref_bam {
#include "bam_decode.cu"
}
namespace ref_fastq {
#include "fastq_scan.cu"
}
namespace ref_bcf {
#include "bcf_scan.cu"
}
namespace ref_fasta {
#include "fasta_compact.cu"
}
namespace ref_text {
#include "text_scan.cu"
}

namespace {

/* One "thread" per index, as a grid of single-thread blocks. */
template <class F> void for_threads(unsigned long long n, F &&f)
{
    blockDim.x = 1;
    threadIdx.x = 0;
    for (unsigned long long i = 0; i < n; ++i) {
        blockIdx.x = (unsigned)i;
        f();
    }
}

} // namespace

extern "C" {

void ref_inflate_blocks(const unsigned char *in, const unsigned long long *in_off, const unsigned int *in_len,
                        unsigned char *out, const unsigned long long *out_off, const unsigned int *caps,
                        unsigned int *status, unsigned int *produced, unsigned int *crc, int n)
{
    blockDim.x = 1;
    for (int i = 0; i < n; ++i) {
        blockIdx.x = (unsigned)i;
        threadIdx.x = 0;
        ref_inflate::inflate_blocks(in, in_off, in_len, out, out_off, caps, status, produced, crc, n);
    }
}

void ref_crc32_blocks(const unsigned char *data, const unsigned long long *off, const unsigned int *len,
                      unsigned int *out, int n)
{
    blockDim.x = 1;
    for (int i = 0; i < n; ++i) {
        blockIdx.x = (unsigned)i;
        threadIdx.x = 0;
        ref_crc::crc32_blocks(data, off, len, out, n);
    }
}

/* The four BAM phases.  Returns status (0 ok, 1 malformed); offsets holds
 * n_records entries (cap permitting); columns are filled for the records. */
int ref_bam_decode(const unsigned char *buf, unsigned long long len, const unsigned long long *block_starts,
                   int n_blocks, unsigned long long start, unsigned long long *record_offsets, unsigned long long cap,
                   unsigned long long *n_records, unsigned long long *tail, int *ref_id, int *pos,
                   unsigned short *flags, unsigned char *mapq, unsigned int *seq_len, int *mate_ref, int *mate_pos,
                   int *tlen, unsigned int *cigar_start, unsigned int *seq_start, unsigned int *qual_start,
                   unsigned int *aux_start, unsigned int *record_end)
{
    std::vector<unsigned int> spec_counts(n_blocks), counts(n_blocks), first(n_blocks);
    std::vector<unsigned long long> lands(n_blocks), entries(n_blocks), totals(3);
    std::vector<unsigned char> complete(n_blocks), valid(n_blocks);
    blockDim.x = 1;
    for (int b = 0; b < n_blocks; ++b) {
        blockIdx.x = (unsigned)b;
        threadIdx.x = 0;
        ref_bam::bam_scan_blocks(buf, len, block_starts, n_blocks, spec_counts.data(), lands.data(), complete.data(),
                                 valid.data());
    }
    blockIdx.x = 0;
    threadIdx.x = 0;
    ref_bam::bam_reconcile(buf, len, block_starts, n_blocks, start, spec_counts.data(), lands.data(), complete.data(),
                           valid.data(), entries.data(), counts.data(), first.data(), totals.data());
    *n_records = totals[0];
    *tail = totals[1];
    if (totals[2] != 0) return (int)totals[2];
    if (totals[0] > cap) return -1;
    for (int b = 0; b < n_blocks; ++b) {
        blockIdx.x = (unsigned)b;
        ref_bam::bam_emit_offsets(buf, entries.data(), counts.data(), first.data(), n_blocks, record_offsets);
    }
    unsigned int n = (unsigned int)totals[0];
    for (unsigned int i = 0; i < n; ++i) {
        blockIdx.x = i;
        ref_bam::bam_decode_fields(buf, record_offsets, n, ref_id, pos, flags, mapq, seq_len, mate_ref, mate_pos,
                                   tlen, cigar_start, seq_start, qual_start, aux_start, record_end);
    }
    return 0;
}

/* FastqScanner::run + decode (crates/fritillaria-cuda/src/fastq.rs:486-560)
 * around the reference's fastq_sieve / fastq_decode / fastq_walk kernels,
 * with the launcher's capacity rule (len / 64, at least 1024).  Returns 0, or
 * 1 when decode reported failures, 2 when the walk overflowed. */
int ref_fastq_run(const unsigned char *buf, unsigned long long len, unsigned long long start,
                  unsigned long long *offsets, unsigned long long cap, unsigned long long *n_out,
                  unsigned long long *tail_out, unsigned long long *survivors_out, int *proof_out,
                  unsigned int *seq_start, unsigned int *plus_start, unsigned int *qual_start,
                  unsigned int *seq_len, unsigned int *rec_end)
{
    *n_out = 0;
    *survivors_out = 0;
    *proof_out = 0;
    if (start >= len) {
        *tail_out = start < len ? start : len;
        return 0;
    }
    unsigned long long capacity = len / 64 > 1024 ? len / 64 : 1024;
    std::vector<unsigned long long> sieved(capacity);
    unsigned int count = 0, overflow = 0;
    unsigned long long anchor = 0;
    unsigned long long span = len - start;
    /* thread i covers byte start + i; blockIdx carries the high part */
    blockDim.x = 256;
    for (unsigned long long i = 0; i < span; ++i) {
        blockIdx.x = (unsigned)(i / 256);
        threadIdx.x = (unsigned)(i % 256);
        ref_fastq::fastq_sieve(buf, len, start, sieved.data(), &count, (unsigned)capacity, &overflow, &anchor);
    }
    std::vector<unsigned long long> offs;
    bool ok = overflow == 0;
    if (ok) {
        offs.assign(sieved.begin(), sieved.begin() + count);
        std::sort(offs.begin(), offs.end());
    }
    *survivors_out = ok ? offs.size() : 0;
    unsigned int errors = 0;
    auto decode = [&](const std::vector<unsigned long long> &o) {
        for_threads(o.size(), [&] {
            ref_fastq::fastq_decode(buf, len, o.data(), (unsigned)o.size(), seq_start, plus_start, qual_start,
                                    seq_len, rec_end, &errors);
        });
    };
    if (ok && !offs.empty() && offs[0] == anchor && offs.size() <= cap) {
        decode(offs);
        if (errors) return 1; /* decode_offsets fails the call (fastq.rs:395-402) */
        unsigned long long at = anchor;
        bool tiled = true;
        for (size_t k = 0; k < offs.size() && tiled; ++k) {
            unsigned long long next = at + rec_end[k];
            if (offs[k] != at || next <= at || next > len) tiled = false;
            else at = next;
        }
        if (tiled) {
            std::copy(offs.begin(), offs.end(), offsets);
            *n_out = offs.size();
            *tail_out = at;
            return 0;
        }
    }
    *proof_out = 1;
    std::vector<unsigned long long> walked(capacity);
    unsigned int wn = 0, wover = 0;
    unsigned long long tail = 0;
    blockIdx.x = 0;
    threadIdx.x = 0;
    blockDim.x = 1;
    ref_fastq::fastq_walk(buf, len, start, walked.data(), &wn, (unsigned)capacity, &wover, &tail);
    if (wover || wn > cap) return 2;
    walked.resize(wn);
    decode(walked);
    std::copy(walked.begin(), walked.end(), offsets);
    *n_out = wn;
    *tail_out = tail;
    return errors ? 1 : 0;
}

/* BcfScanner::scan (crates/fritillaria-cuda/src/bcf.rs:280-372) around
 * bcf_sieve / bcf_validate / bcf_probe_tail / bcf_walk, with the launcher's
 * capacity rule.  Returns 0, or 2 when the walk overflowed. */
int ref_bcf_scan(const unsigned char *buf, unsigned long long len, unsigned long long start, unsigned int samples,
                 unsigned int contigs, unsigned long long *offsets, unsigned long long cap,
                 unsigned long long *n_out, unsigned long long *tail_out, unsigned long long *sieved_out,
                 unsigned long long *validated_out, int *proof_out)
{
    *n_out = 0;
    *sieved_out = *validated_out = 0;
    *proof_out = 0;
    if (start >= len) {
        *tail_out = start < len ? start : len;
        return 0;
    }
    unsigned long long capacity = len / 64 > 1024 ? len / 64 : 1024;
    std::vector<unsigned long long> sv(capacity), se(capacity);
    unsigned int ns = 0, overflow = 0;
    unsigned long long span = len - start;
    blockDim.x = 256;
    for (unsigned long long i = 0; i < span; ++i) {
        blockIdx.x = (unsigned)(i / 256);
        threadIdx.x = (unsigned)(i % 256);
        ref_bcf::bcf_sieve(buf, len, start, samples, contigs, sv.data(), se.data(), &ns, (unsigned)capacity,
                           &overflow);
    }
    *sieved_out = ns;
    bool walk = overflow != 0 || ns > capacity;
    if (!walk) {
        std::vector<unsigned long long> vv(capacity), ve(capacity);
        unsigned int nv = 0;
        for_threads(ns, [&] {
            ref_bcf::bcf_validate(buf, len, sv.data(), se.data(), ns, vv.data(), ve.data(), &nv);
        });
        *validated_out = nv;
        std::vector<std::pair<unsigned long long, unsigned long long>> pairs;
        for (unsigned int k = 0; k < nv; ++k) pairs.emplace_back(vv[k], ve[k]);
        std::sort(pairs.begin(), pairs.end());
        unsigned long long at = start;
        bool tiled = true;
        for (auto &pe : pairs) {
            if (pe.first != at || pe.second > len || pe.second <= pe.first) {
                tiled = false;
                break;
            }
            at = pe.second;
        }
        if (tiled) {
            unsigned int whole = 0;
            blockIdx.x = 0;
            threadIdx.x = 0;
            ref_bcf::bcf_probe_tail(buf, len, at, &whole);
            if (!whole && pairs.size() <= cap) {
                for (size_t k = 0; k < pairs.size(); ++k) offsets[k] = pairs[k].first;
                *n_out = pairs.size();
                *tail_out = at;
                return 0;
            }
        }
    }
    *proof_out = 1;
    unsigned long long wcap = (len - start) / 32 + 1;
    if (wcap < 1024) wcap = 1024;
    std::vector<unsigned long long> out(wcap);
    unsigned int wn = 0, wover = 0;
    unsigned long long tail = 0;
    blockIdx.x = 0;
    threadIdx.x = 0;
    blockDim.x = 1;
    ref_bcf::bcf_walk(buf, len, start, out.data(), &wn, (unsigned)wcap, &wover, &tail);
    if (wover || wn > cap) return 2;
    std::copy(out.begin(), out.begin() + wn, offsets);
    *n_out = wn;
    *tail_out = tail;
    return 0;
}

/* bcf_decode over n records; returns its error count. */
unsigned int ref_bcf_decode(const unsigned char *buf, unsigned long long len, const unsigned long long *offsets,
                            unsigned int n, int *chrom, int *pos, int *rlen, unsigned int *qual,
                            unsigned short *n_info, unsigned short *n_allele, unsigned int *n_sample,
                            unsigned char *n_fmt, unsigned int *alleles, unsigned int *filters, unsigned int *info,
                            unsigned int *genotypes, unsigned int *end)
{
    unsigned int errors = 0;
    for_threads(n, [&] {
        ref_bcf::bcf_decode(buf, len, offsets, n, chrom, pos, rlen, qual, n_info, n_allele, n_sample, n_fmt,
                            alleles, filters, info, genotypes, end, &errors);
    });
    return errors;
}

/* fasta_find_contigs (sorted, as the launcher sorts), fasta_compact_uniform
 * and fasta_compact_scan (crates/fritillaria-cuda/kernels/fasta_compact.cu). */
unsigned int ref_fasta_find_contigs(const unsigned char *buf, unsigned long long len, unsigned long long *out,
                                    unsigned int cap)
{
    unsigned int count = 0, overflow = 0;
    blockDim.x = 256;
    for (unsigned long long i = 0; i < len; ++i) {
        blockIdx.x = (unsigned)(i / 256);
        threadIdx.x = (unsigned)(i % 256);
        ref_fasta::fasta_find_contigs(buf, len, 0, out, &count, cap, &overflow);
    }
    std::sort(out, out + (count < cap ? count : cap));
    return overflow ? 0xFFFFFFFFu : count;
}

void ref_fasta_compact_uniform(const unsigned char *src, unsigned long long span, unsigned char *dst,
                               unsigned int line_width)
{
    blockDim.x = 256;
    for (unsigned long long i = 0; i < span; ++i) {
        blockIdx.x = (unsigned)(i / 256);
        threadIdx.x = (unsigned)(i % 256);
        ref_fasta::fasta_compact_uniform(src, span, dst, line_width);
    }
}

void ref_fasta_compact_scan(const unsigned char *src, unsigned long long span, unsigned char *dst)
{
    blockIdx.x = 0;
    threadIdx.x = 0;
    blockDim.x = 1;
    ref_fasta::fasta_compact_scan(src, span, dst);
}

/*
 * TextScanner::scan (crates/fritillaria-cuda/src/text.rs:233-420): text_find_lines
 * over every byte from start into max(len / 8, 1024) slots (overflow is an
 * error), the offsets sorted and split by kind, text_count_fields per record,
 * the host prefix sum, text_write_fields, and the tail rule.  Returns 0, 1 when
 * the line slots overflow, 2 when the caller's arrays are too small.
 */
int ref_text_scan(const unsigned char *buf, unsigned long long len, unsigned long long start, unsigned int comment,
                  unsigned int secondary, unsigned long long *rec_off, unsigned long long *rec_end,
                  unsigned long long *hdr_off, unsigned long long *tabs, unsigned long long *starts,
                  unsigned long long cap_lines, unsigned long long cap_tabs, unsigned long long *n_rec,
                  unsigned long long *n_hdr, unsigned long long *n_tabs, unsigned long long *tail)
{
    *n_rec = *n_hdr = *n_tabs = 0;
    if (start >= len) {
        *tail = start < len ? start : len;
        return 0;
    }
    unsigned long long capacity = len / 8 > 1024 ? len / 8 : 1024;
    std::vector<unsigned long long> lines(capacity);
    std::vector<unsigned char> kinds(capacity);
    unsigned int count = 0, overflow = 0;
    for_threads(len - start, [&] {
        ref_text::text_find_lines(buf, len, start, comment, secondary, lines.data(), kinds.data(), &count,
                                  (unsigned)capacity, &overflow);
    });
    if (overflow) return 1;
    std::vector<std::pair<unsigned long long, unsigned char>> pairs;
    for (unsigned i = 0; i < count; ++i) pairs.emplace_back(lines[i], kinds[i]);
    std::sort(pairs.begin(), pairs.end());
    std::vector<unsigned long long> recs, hdrs;
    for (auto &pr : pairs) (pr.second == 1 ? hdrs : recs).push_back(pr.first);
    if (recs.size() > cap_lines || hdrs.size() > cap_lines) return 2;
    for (size_t i = 0; i < hdrs.size(); ++i) hdr_off[i] = hdrs[i];
    *n_hdr = hdrs.size();
    *tail = len;
    const unsigned n = (unsigned)recs.size();
    if (n == 0) return 0;
    std::vector<unsigned int> counts(n);
    std::vector<unsigned long long> ends(n);
    for_threads(n, [&] { ref_text::text_count_fields(buf, len, recs.data(), n, counts.data(), ends.data()); });
    std::vector<unsigned long long> st(n + 1, 0);
    for (unsigned i = 0; i < n; ++i) st[i + 1] = st[i] + counts[i];
    if (st[n] > cap_tabs) return 2;
    for_threads(n, [&] { ref_text::text_write_fields(buf, recs.data(), ends.data(), n, st.data(), tabs); });
    for (unsigned i = 0; i < n; ++i) {
        rec_off[i] = recs[i];
        rec_end[i] = ends[i];
    }
    for (unsigned i = 0; i <= n; ++i) starts[i] = st[i];
    *n_rec = n;
    *n_tabs = st[n];
    *tail = ends[n - 1] >= len ? recs[n - 1] : len;
    return 0;
}

} // extern "C"
