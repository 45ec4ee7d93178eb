// Inflate kernels: launch constants and entry points.
#pragma once

#include "common.cuh"

// Warps per CTA of the inflate kernels, decoded-output staging chunk and the
// back-reference queue length per chunk.
#ifndef INF_WARPS_PER_CTA
#define INF_WARPS_PER_CTA 8
#endif
#define INF_CHUNK 2048
#define INF_MAXM 192

__device__ u32 inflate_member_warp(const u8 *in, u32 in_len, u8 *out, u32 cap, void *smem, const u32 *crc_tab,
                                   u32 *produced_out, u32 *crc_out);

size_t frt_inflate_warp_smem();


size_t frt_inflate_smem_bytes(int warps);
cudaError_t frt_inflate_prepare();
cudaError_t frt_launch_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                       const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                       u32 *crc, u32 n, cudaStream_t s);
cudaError_t frt_launch_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                          const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                          u32 *crc, const u32 *order, const u32 *n_ptr, u32 *queue_head,
                                          u32 chunk, u32 grid, cudaStream_t s);
cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s);
