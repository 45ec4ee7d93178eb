// BAM record scan / decode kernels: constants and the column pointer block.
#pragma once

#include "common.cuh"

// Record offsets stored per member during the scan.  A record occupies at
// least 36 bytes, so a member of at most 65,536 inflated bytes holds at most
// 1,821 record starts.
#define FRT_SCAN_CAP 1824

struct FrtBamColumnsDev {
    int *ref_id;
    int *pos;
    u16 *flags;
    u8 *mapq;
    u32 *seq_len;
    int *mate_ref_id;
    int *mate_pos;
    int *tlen;
    u64 *record_offsets;
    u32 *cigar_start;
    u32 *sequence_start;
    u32 *quality_start;
    u32 *aux_start;
    u32 *record_end;
    u16 *bin;
    u16 *n_cigar;
    u8 *name_len;
    u64 *virtual_offset;
    u32 *aux_count;
    u8 *aux_status;
};


cudaError_t frt_launch_bam_spec(const u8 *buf, u64 len, const u64 *starts, u32 n, u64 start, int n_ref, u64 *entry,
                                u32 *count, u64 *land, u8 *flags, u16 *scratch, cudaStream_t s,
                                const u64 *start_dev = nullptr, const int *nref_dev = nullptr);
cudaError_t frt_launch_bam_reconcile(const u8 *buf, u64 len, const u64 *starts, u32 n, u64 start, u64 *entry,
                                     u32 *count, u64 *land, u8 *flags, u16 *scratch, u32 *first_index, u64 *totals,
                                     cudaStream_t s, const u64 *start_dev = nullptr);
cudaError_t frt_launch_bam_decode(const u8 *buf, const u64 *starts, const u64 *coff, u32 n, const u32 *count,
                                  const u32 *first_index, const u16 *scratch, const FrtBamColumnsDev &c,
                                  cudaStream_t s);
size_t frt_scan_partials_len(u64 n);

// One record chain of a region query: members [m0, m0 + n) of a tick's member
// table (their n + 1 starts at starts + m0 + segment index), the chain start
// and the end of its inflated bytes (offsets in the tick's output arena), and
// the filter: records starting before chunk_end (a virtual offset) that
// overlap [beg, end] (1-based inclusive) on reference `ref`.
struct FrtScanSeg {
    u64 start, len;
    u32 m0, n;
    u64 chunk_end;
    u64 beg, end;
    int ref;
    u32 request;  // the request's slot in the tick
    u64 out_base; // where the request's inflated bytes start in the arena
};

struct FrtRegionColumns {
    u64 *virtual_offset;
    u64 *record_offset; // into the request's inflated bytes
    int *ref_id;
    int *pos;
    u16 *flags;
    u8 *mapq;
    u32 *seq_len;
    u32 *request;
};

cudaError_t frt_launch_region_scan(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_segs, u32 n_total,
                                   int n_ref, const u64 *starts, const u64 *coff, u64 *entry, u32 *count, u64 *land,
                                   u8 *flags, u16 *scratch, u32 *first_index, u64 *totals, u32 *kept, cudaStream_t s);
cudaError_t frt_launch_region_emit(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_total,
                                   const u64 *starts, const u64 *coff, const u32 *count, const u16 *scratch,
                                   const u32 *kept_first, const FrtRegionColumns &out, cudaStream_t s);
cudaError_t frt_launch_scan_u32(const u32 *in, u64 n, u32 *partials, u32 *out, u32 *total, cudaStream_t s);
cudaError_t frt_launch_bam_aux_dir(const u8 *buf, const u64 *record_offsets, const u32 *aux_start,
                                   const u32 *record_end, const u32 *aux_count, const u32 *aux_first, u32 *entries,
                                   u64 n, cudaStream_t s);
cudaError_t frt_launch_bam_decode_capped(const u8 *buf, const u64 *starts, const u64 *coff, u32 n, const u32 *count,
                                         const u32 *first_index, const u16 *scratch, const FrtBamColumnsDev &c,
                                         u64 rec_cap, cudaStream_t s);
cudaError_t frt_launch_bam_aux_dir_capped(const u8 *buf, const u64 *record_offsets, const u32 *aux_start,
                                          const u32 *record_end, const u32 *aux_count, const u32 *aux_first,
                                          u32 *entries, const u64 *n_dev, u64 rec_cap, u64 aux_cap, cudaStream_t s);
