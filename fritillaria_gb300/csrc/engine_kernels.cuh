// Kernels of the batched, device-resident form: BGZF member discovery, the
// inflate plan, the size-sorted work queue and the BAM header parse.
#pragma once

#include "common.cuh"

// Device-side state of one engine run; the host reads it once at the end.
struct EngineDevState {
    u64 block_err;      // min over (member << 8 | frt_status) of failing members; ~0 if none
    u64 n_members;      // members discovered
    u64 tiling_failed;  // candidate headers did not tile the buffer
    u64 walk_err;       // offset + 1 of an invalid header met by the fallback walk, 0 if none
    u64 inflated_total; // sum of ISIZE
    u64 records_start;  // after the BAM header
    u64 totals[4];      // records, tail, malformed, fallbacks
    u32 n_aux;
    int n_ref;
    int header_status;  // 0 ok, 1 malformed header
    u32 capacity_err;   // a count exceeded what the buffers were sized for
    u32 queue_head;
    u32 pad;
};

__global__ void k_bgzf_sieve(const u8 *buf, u64 len, u64 tile, u32 *counts, const u32 *tile_base, u64 *cand,
                             u64 cand_cap);
__global__ void k_bgzf_tiling(const u8 *buf, u64 len, const u64 *cand, const u32 *n_cand, EngineDevState *st);
__global__ void k_bgzf_walk(const u8 *buf, u64 len, u64 *cand, u64 cap, EngineDevState *st);
__global__ void k_bgzf_spans(const u8 *buf, u64 len, const u64 *cand, u64 n_cap, EngineDevState *st, u64 *in_off,
                             u32 *in_len, u32 *isize, u32 *crc, u64 *coffset);
__global__ void k_queue_hist(const u32 *in_len, u64 n, u32 *hist);
__global__ void k_queue_scatter(const u32 *in_len, u64 n, u32 *cursor, u32 *order);
__global__ void k_bam_header(const u8 *buf, const u64 *total, EngineDevState *st);
