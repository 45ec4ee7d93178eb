/*
 * TEST INFRASTRUCTURE ONLY.  Drives the reference's kernels, compiled as host
 * C++ from their own sources (crates/fritillaria-cuda/kernels/*.cu), one
 * "thread" at a time, in the launch order of the reference's launchers
 * (crates/fritillaria-cuda/src/backend.rs:635-720, src/bam.rs:368-573).
 * Built by oracle/build.py into oracle/_ref/ only where the reference tree is
 * present; never shipped.
 */
#include <cstdint>
#include <cstring>
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

} // extern "C"
