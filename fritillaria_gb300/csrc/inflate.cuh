// Inflate kernels: variants, tunings and entry points.
#pragma once

#include "common.cuh"
#include "../../include/frt.h"

// Largest warps per CTA and members per queue pop a tuning may ask for.
#define FRT_INFLATE_MAX_WARPS 8
#define FRT_INFLATE_MAX_CHUNK 64

// The compiled variants of the member inflate (table roots, window buffer and
// match queue per warp) and the process-wide default tuning that engines,
// codecs and servers start from.
const frt_inflate_variant *frt_inflate_variant_at(int v);
frt_inflate_tuning frt_inflate_default();
void frt_inflate_set_default(const frt_inflate_tuning &t);

// Dynamic shared memory of one CTA under a tuning; CTAs per SM it runs with
// on the current device (0: the tuning is invalid or does not fit).
size_t frt_inflate_smem_bytes(const frt_inflate_tuning &t);
int frt_inflate_ctas_per_sm(const frt_inflate_tuning &t);
int frt_inflate_persistent_grid(const frt_inflate_tuning &t);

cudaError_t frt_inflate_prepare();
cudaError_t frt_launch_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                       const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                       u32 *crc, u32 n, const frt_inflate_tuning &t, cudaStream_t s);
cudaError_t frt_launch_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                          const u64 *out_off, const u32 *isize, const u32 *crc_expect, u32 *status,
                                          u32 *produced, u32 *crc, const u32 *order, const u64 *n_ptr, u64 n_cap,
                                          u64 out_capacity, u32 *queue_head, u32 grid, unsigned long long *block_err,
                                          const frt_inflate_tuning &t, cudaStream_t s);
cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s);
