// Inflate kernels: launch constants and entry points.
#pragma once

#include "common.cuh"

// Warps per CTA of the inflate kernels; table roots; per warp, the window
// output buffer and the window's match queue.
#ifndef INF_WARPS_PER_CTA
#define INF_WARPS_PER_CTA 3
#endif
#ifndef INF_LIT_BITS
#define INF_LIT_BITS 10
#endif
#ifndef INF_DIST_BITS
#define INF_DIST_BITS 8
#endif
#ifndef INF_WINBUF
#define INF_WINBUF 2048
#endif
#ifndef INF_MAXQ
#define INF_MAXQ 384
#endif

__device__ u32 inflate_member_warp(const u8 *in, u32 in_len, u8 *out, u32 cap, void *smem, u32 *produced_out,
                                   u32 *crc_out);

size_t frt_inflate_warp_smem();


size_t frt_inflate_smem_bytes(int warps);
cudaError_t frt_inflate_prepare();
cudaError_t frt_launch_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                       const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                       u32 *crc, u32 n, cudaStream_t s);
cudaError_t frt_launch_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                          const u64 *out_off, const u32 *isize, const u32 *crc_expect, u32 *status,
                                          u32 *produced, u32 *crc, const u32 *order, const u64 *n_ptr, u64 n_cap,
                                          u64 out_capacity, u32 *queue_head, u32 chunk, u32 grid,
                                          unsigned long long *block_err, cudaStream_t s);
int frt_inflate_persistent_grid();
cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s);
