// The batched, device-resident form.
//
// Instead of one launch sequence per batch of 256 members with a host sync
// for the statuses and another for the record totals (the reference's launch
// model, crates/fritillaria-cuda/src/backend.rs:547-720 and src/bam.rs:324-573),
// a whole BGZF file resident in HBM goes through one pass of device-only
// stages, with no host round trip until the final stats read:
//
//   discovery   16-byte-vector sieve for gzip/BGZF headers, ordered
//               compaction (count, scan, emit), then a tiling proof that
//               the candidates chain from offset 0 to the end; a serial walk
//               only if the proof fails;
//   plan        member spans from the headers/trailers, exclusive scan of
//               ISIZE into output offsets;
//   queue       counting sort of members by compressed size, longest first;
//   inflate     the persistent warp-per-member kernel pulls from the queue
//               and verifies CRC32/ISIZE in-kernel into one error word;
//   records     BAM header parse, per-member speculative scan, reconcile,
//               column decode, aux-count scan and aux directory.
//
// bind() runs the stages once eagerly to size every buffer, then captures the
// stage sequence as a CUDA graph; run() replays it.

#include <algorithm>
#include <cstring>
#include <vector>

#include "bam.cuh"
#include "engine_kernels.cuh"
#include "fields.h"
#include "inflate.cuh"
#include "runtime.h"

using namespace frt;

namespace {

constexpr u64 SIEVE_TILE = 1ull << 16;

// A BGZF member header at p (block.rs:88-165): returns bsize (0 if none) and
// the header size.  Only complete members inside the buffer count.
__device__ __forceinline__ u32 member_at(const u8 *buf, u64 len, u64 p, u32 *hsize)
{
    if (p + 12 > len) return 0;
    if (buf[p] != 0x1f || buf[p + 1] != 0x8b || buf[p + 2] != 8 || !(buf[p + 3] & 4)) return 0;
    u32 xlen = ld_u16le(buf + p + 10);
    if (p + 12 + xlen > len) return 0;
    u32 off = 0, bsize = 0;
    bool found = false;
    while (off + 4 <= xlen) {
        const u8 *x = buf + p + 12 + off;
        u32 slen = ld_u16le(x + 2);
        if (off + 4 + slen > xlen) break;
        if (x[0] == 'B' && x[1] == 'C') {
            if (slen == 2) {
                bsize = ld_u16le(x + 4) + 1;
                found = true;
            }
            break;
        }
        off += 4 + slen;
    }
    if (!found) return 0;
    if (bsize > 65536u || bsize < 12 + xlen + 8) return 0;
    if (p + bsize > len) return 0;
    *hsize = 12 + xlen;
    return bsize;
}

} // namespace

// One warp per 64 KiB tile, 16 bytes per lane per step.  Count mode
// (tile_base == nullptr) writes the tile's candidate count; emit mode writes
// the candidates in order starting at tile_base[tile].
__global__ void k_bgzf_sieve(const u8 *buf, u64 len, u64 tile, u32 *counts, const u32 *tile_base, u64 *cand,
                             u64 cand_cap)
{
    const u32 lane = lane_id();
    u64 t = (u64)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    u64 t0 = t * tile;
    if (t0 >= len) return;
    u64 t1 = min(len, t0 + tile);
    u32 found = 0;
    u64 out = tile_base ? tile_base[t] : 0;
    for (u64 base = t0; base < t1; base += 512) {
        u64 p0 = base + 16ull * lane;
        u32 mine = 0;
        u64 hits[2];
        if (p0 < t1) {
            u32 w[4];
            if (p0 + 16 <= len && ((u64)(buf + p0) & 15ull) == 0) {
                uint4 v = *(const uint4 *)(buf + p0);
                w[0] = v.x;
                w[1] = v.y;
                w[2] = v.z;
                w[3] = v.w;
            } else {
                for (int k = 0; k < 4; ++k) {
                    u32 x = 0;
                    for (int b = 0; b < 4; ++b) {
                        u64 q = p0 + 4 * k + b;
                        x |= (u32)(q < len ? buf[q] : 0) << (8 * b);
                    }
                    w[k] = x;
                }
            }
            // bytes equal to 0x1f: the zero-byte test on w ^ 0x1f1f1f1f
            for (int k = 0; k < 4; ++k) {
                u32 x = w[k] ^ 0x1f1f1f1fu;
                u32 z = (x - 0x01010101u) & ~x & 0x80808080u;
                while (z) {
                    int b = (__ffs(z) - 1) >> 3;
                    z &= z - 1;
                    u64 p = p0 + 4 * k + b;
                    u32 hs;
                    if (p < t1 && member_at(buf, len, p, &hs)) {
                        if (mine < 2) hits[mine] = p;
                        ++mine;
                    }
                }
            }
        }
        // ordered output within the warp: lanes in address order
        u32 x = mine;
        for (int d = 1; d < 32; d <<= 1) {
            u32 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
            if (lane >= (u32)d) x += y;
        }
        u32 excl = x - mine;
        u32 step_total = __shfl_sync(FRT_FULL_MASK, x, 31);
        if (tile_base && mine) {
            // a lane holds at most 16 bytes, so more than two headers in it is
            // impossible for valid members; extra ones are re-found serially
            u32 k = 0;
            for (u32 j = 0; j < mine && j < 2; ++j, ++k)
                if (out + found + excl + k < cand_cap) cand[out + found + excl + k] = hits[j];
            if (mine > 2) {
                u32 seen = 0;
                for (int b = 0; b < 16; ++b) {
                    u64 p = p0 + b;
                    u32 hs;
                    if (p < t1 && buf[p] == 0x1f && member_at(buf, len, p, &hs)) {
                        if (seen >= 2 && out + found + excl + seen < cand_cap) cand[out + found + excl + seen] = p;
                        ++seen;
                    }
                }
            }
        }
        found += step_total;
    }
    if (!tile_base && lane == 0) counts[t] = found;
}

// The candidates tile the buffer iff the first is at 0, each one's successor
// is the next, and the last ends exactly at the buffer end.
__global__ void k_bgzf_tiling(const u8 *buf, u64 len, const u64 *cand, const u32 *n_cand, u64 n_cap,
                              EngineDevState *st)
{
    u64 n = *n_cand;
    if (n > n_cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            st->capacity_err = 1;
            st->tiling_failed = 1;
        }
        n = n_cap;
    }
    u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) {
        st->n_members = n;
        if (n == 0 ? len != 0 : cand[0] != 0) st->tiling_failed = 1;
    }
    if (k >= n) return;
    u32 hs;
    u32 bs = member_at(buf, len, cand[k], &hs);
    u64 next = cand[k] + bs;
    u64 want = k + 1 < n ? cand[k + 1] : len;
    if (bs == 0 || next != want) st->tiling_failed = 1;
}

// Fallback when the candidates do not tile: walk the headers from 0 (one
// thread).  An invalid header stops the walk and is reported.
__global__ void k_bgzf_walk(const u8 *buf, u64 len, u64 *cand, u64 cap, EngineDevState *st)
{
    if (threadIdx.x != 0 || blockIdx.x != 0 || !st->tiling_failed) return;
    u64 p = 0, n = 0;
    while (p < len) {
        u32 hs;
        u32 bs = member_at(buf, len, p, &hs);
        if (bs == 0) {
            st->walk_err = p + 1;
            break;
        }
        if (n < cap) cand[n] = p;
        ++n;
        p += bs;
    }
    st->n_members = n;
}

// Member spans for the first n members; entries past n (up to n_cap) become
// empty members so every later stage stays in bounds.
__global__ void k_bgzf_spans(const u8 *buf, u64 len, const u64 *cand, u64 n_cap, EngineDevState *st, u64 *in_off,
                             u32 *in_len, u32 *isize, u32 *crc, u64 *coffset)
{
    u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_cap) return;
    u64 n = st->n_members;
    if (n > n_cap) {
        if (k == 0) st->capacity_err = 1;
        n = n_cap;
    }
    if (k >= n) {
        in_off[k] = 0;
        in_len[k] = 0;
        isize[k] = 0;
        crc[k] = 0;
        coffset[k] = len;
        return;
    }
    u64 p = cand[k];
    u32 hs = 0;
    u32 bs = member_at(buf, len, p, &hs);
    if (bs == 0) { // cannot happen for a proven tiling; keep the member empty
        in_off[k] = 0;
        in_len[k] = 0;
        isize[k] = 0;
        crc[k] = 0;
        coffset[k] = p;
        atomicMin((unsigned long long *)&st->block_err, ((unsigned long long)k << 8) | 2ull);
        return;
    }
    u32 isz = ld_u32le(buf + p + bs - 4);
    in_off[k] = p + hs;
    in_len[k] = bs - hs - 8;
    crc[k] = ld_u32le(buf + p + bs - 8);
    coffset[k] = p;
    if (isz > 65536u) { // discover.rs:88-95
        atomicMin((unsigned long long *)&st->block_err, ((unsigned long long)k << 8) | 2ull);
        isz = 0;
    }
    isize[k] = isz;
}

// Work queue: members by compressed size, longest first (1024 buckets of 64 B).
__global__ void k_queue_hist(const u32 *in_len, u64 n, u32 *hist)
{
    u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    u32 b = 1023u - min(1023u, in_len[k] >> 6);
    atomicAdd(&hist[b], 1u);
}

__global__ void k_queue_scatter(const u32 *in_len, u64 n, u32 *cursor, u32 *order)
{
    u64 k = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    u32 b = 1023u - min(1023u, in_len[k] >> 6);
    u32 slot = atomicAdd(&cursor[b], 1u);
    order[slot] = (u32)k;
}

// BAM header (crates/fritillaria-bam/src/columnar/header.rs:43-101): one thread.
__global__ void k_bam_header(const u8 *buf, const u64 *total, EngineDevState *st)
{
    if (threadIdx.x || blockIdx.x) return;
    u64 len = *total;
    st->header_status = 1;
    if (len < 12 || buf[0] != 'B' || buf[1] != 'A' || buf[2] != 'M' || buf[3] != 1) return;
    int l_text = (int)ld_u32le(buf + 4);
    if (l_text < 0) return;
    u64 pos = 8ull + (u64)l_text;
    if (pos + 4 > len) return;
    int n_ref = (int)ld_u32le(buf + pos);
    if (n_ref < 0) return;
    pos += 4;
    for (int i = 0; i < n_ref; ++i) {
        if (pos + 4 > len) return;
        int l_name = (int)ld_u32le(buf + pos);
        if (l_name < 0) return;
        pos += 4 + (u64)l_name;
        if (pos + 4 > len) return;
        pos += 4;
    }
    st->records_start = pos;
    st->n_ref = n_ref;
    st->header_status = 0;
}

namespace {

// exclusive scan of u32 values into u64 offsets (n + 1 entries)
__global__ void __launch_bounds__(1024) k_scan64_partials(const u32 *in, u64 n, u64 *partials)
{
    __shared__ u64 s[32];
    u64 base = (u64)blockIdx.x * 4096;
    u64 acc = 0;
    for (int k = 0; k < 4; ++k) {
        u64 i = base + (u64)k * 1024 + threadIdx.x;
        if (i < n) acc += in[i];
    }
    for (int d = 16; d; d >>= 1) acc += __shfl_down_sync(FRT_FULL_MASK, acc, d);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        u64 v = s[threadIdx.x];
        for (int d = 16; d; d >>= 1) v += __shfl_down_sync(FRT_FULL_MASK, v, d);
        if (threadIdx.x == 0) partials[blockIdx.x] = v;
    }
}

__device__ u64 block_scan64(u64 v, u64 *s_warp, u64 *total)
{
    const u32 lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    u64 x = v;
    for (int d = 1; d < 32; d <<= 1) {
        u64 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
        if (lane >= (u32)d) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        u64 w = s_warp[lane];
        for (int d = 1; d < 32; d <<= 1) {
            u64 y = __shfl_up_sync(FRT_FULL_MASK, w, d);
            if (lane >= (u32)d) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    u64 ex = x - v + (wid ? s_warp[wid - 1] : 0ull);
    *total = s_warp[31];
    __syncthreads();
    return ex;
}

__global__ void __launch_bounds__(1024) k_scan64_partials_scan(u64 *partials, u64 n_parts)
{
    __shared__ u64 s_warp[32];
    u64 carry = 0;
    for (u64 b = 0; b < n_parts; b += 1024) {
        u64 i = b + threadIdx.x;
        u64 v = i < n_parts ? partials[i] : 0ull;
        u64 tot;
        u64 ex = block_scan64(v, s_warp, &tot);
        if (i < n_parts) partials[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(1024) k_scan64_apply(const u32 *in, u64 n, const u64 *partials, u64 *out,
                                                       u64 *total_out)
{
    __shared__ u64 s_warp[32];
    u64 base = (u64)blockIdx.x * 4096;
    u64 carry = partials[blockIdx.x];
    for (int k = 0; k < 4; ++k) {
        u64 i = base + (u64)k * 1024 + threadIdx.x;
        u64 v = i < n ? in[i] : 0ull;
        u64 tot;
        u64 ex = block_scan64(v, s_warp, &tot);
        if (i <= n) out[i] = carry + ex;
        carry += tot;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0 && total_out) *total_out = carry;
}

// Exclusive scan of the 1024 queue buckets into cursors (one CTA).
__global__ void __launch_bounds__(1024) k_queue_cursor(const u32 *hist, u32 *cursor)
{
    __shared__ u64 s_warp[32];
    u64 tot;
    u64 ex = block_scan64(hist[threadIdx.x], s_warp, &tot);
    cursor[threadIdx.x] = (u32)ex;
}

// Decoded-record and aux-field counts must fit what bind sized.
__global__ void k_check_counts(EngineDevState *st, u64 rec_cap, u64 aux_cap)
{
    if (threadIdx.x || blockIdx.x) return;
    // the steady state replays what bind measured: any other count means the
    // bound buffer changed
    if (st->totals[0] != rec_cap || (u64)st->n_aux != aux_cap) st->capacity_err = 1;
}

// The error words of the per-group inflate launches of a pipelined host run:
// member indices there are relative to the group; the first failing member in
// file order wins, as in the single launch.
__global__ void k_merge_group_errors(const u64 *errs, const u64 *first, u32 groups, EngineDevState *st)
{
    if (threadIdx.x != 0) return;
    u64 best = ~0ull;
    for (u32 g = 0; g < groups; ++g) {
        const u64 w = errs[g];
        if (w == ~0ull) continue;
        const u64 v = ((first[g] + (w >> 8)) << 8) | (w & 0xffull);
        if (v < best) best = v;
    }
    st->block_err = best;
}

} // namespace

// ===========================================================================
// host side
// ===========================================================================
struct frt_engine {
    int device = 0;
    SharedStream *shared = nullptr;
    cudaStream_t stream = nullptr;
    frt_engine_config cfg{};
    frt_inflate_tuning tuning{};
    int grid = 0;
    // bound file
    const uint8_t *in = nullptr;
    size_t len = 0;
    u64 n_cap = 0, tiles = 0, out_cap = 0, rec_cap = 0, aux_cap = 0;
    // buffers
    EngineDevState *st = nullptr;
    u32 *tile_counts = nullptr, *tile_base = nullptr;
    u64 *cand = nullptr, *in_off = nullptr, *coffset = nullptr, *out_off = nullptr, *scan_parts = nullptr;
    u32 *in_len = nullptr, *isize = nullptr, *crc_expect = nullptr, *order = nullptr, *hist = nullptr,
        *cursor = nullptr, *status = nullptr, *produced = nullptr, *crc = nullptr;
    u8 *out = nullptr;
    // records
    u64 *entry = nullptr, *land = nullptr;
    u32 *count = nullptr, *first = nullptr, *aux_parts = nullptr, *aux_entries = nullptr;
    u8 *flags = nullptr;
    u16 *scratch = nullptr;
    u8 *cols = nullptr;
    size_t col_off[FRT_COL_COUNT] = {};
    size_t col_bytes[FRT_COL_COUNT] = {};
    std::vector<void *> allocs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    EngineDevState host_state{};
    // several files: one inflate over all members, then each file's decoder
    struct File {
        frt_engine_file desc{};
        u64 m0 = 0, m1 = 0;     // member range
        u64 out0 = 0, out1 = 0; // inflated range
        u64 records_start = 0;
        int32_t n_ref = -1;
        uint32_t samples = 0, contigs = 0;
        frt_inflate_batch *view = nullptr;
        frt_record_batch *bam = nullptr;
        frt_columns *cols = nullptr;
        cudaEvent_t t0 = nullptr, t1 = nullptr; // around the file's decode
    };
    bool multi = false;
    std::vector<File> files;
    std::vector<u64> bound_coff, bound_out_off; // the plan the file views were built on
    frt_bam_decoder *bam_dec = nullptr;
    frt_fastq_scanner *fastq = nullptr;
    frt_bcf_scanner *bcf = nullptr;
    frt_fasta_compactor *fasta = nullptr;
    int decode_rc = FRT_OK;
    frt_error decode_err{};
    // host-buffer runs with the upload overlapped (run_host_pipelined)
    struct HostPipe {
        cudaStream_t copy = nullptr;
        std::vector<cudaStream_t> lanes; // one per inflate group
        cudaEvent_t plan = nullptr;
        std::vector<cudaEvent_t> up, done;
        uint8_t *staging = nullptr; // pinned plan
        size_t staging_bytes = 0;
        u64 *d_count = nullptr;     // members per group
        u64 *d_errs = nullptr;      // per-group error words
        u64 *d_first = nullptr;     // first member of each group
        u32 *d_heads = nullptr;     // per-group queue heads
    } pipe;
};

namespace {

template <typename T> int ealloc(frt_engine *e, T **p, size_t n, frt_error *err)
{
    void *q = nullptr;
    cudaError_t ce = cudaMallocAsync(&q, n * sizeof(T) + 64, e->stream);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "allocating engine buffers");
    e->allocs.push_back(q);
    *p = (T *)q;
    return FRT_OK;
}

void release_results(frt_engine *e)
{
    for (auto &f : e->files) {
        if (f.bam) frt_record_batch_free(f.bam);
        if (f.cols) frt_columns_free(f.cols);
        f.bam = nullptr;
        f.cols = nullptr;
    }
}

void free_all(frt_engine *e)
{
    release_results(e);
    for (auto &f : e->files) {
        if (f.view) batch_release(f.view);
        if (f.t0) cudaEventDestroy(f.t0);
        if (f.t1) cudaEventDestroy(f.t1);
    }
    e->files.clear();
    e->multi = false;
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->exec = nullptr;
    e->graph = nullptr;
    for (void *p : e->allocs) cudaFreeAsync(p, e->stream);
    e->allocs.clear();
    cudaStreamSynchronize(e->stream);
}

template <typename T> T *ecol(frt_engine *e, int c) { return (T *)(e->cols + e->col_off[c]); }

// The discovery, plan and queue stages (everything up to the inflate).
cudaError_t enqueue_front(frt_engine *e)
{
    cudaStream_t s = e->stream;
    cudaMemsetAsync(e->st, 0, sizeof(EngineDevState), s);
    cudaMemsetAsync(&e->st->block_err, 0xff, 8, s);
    u64 tiles = e->tiles;
    unsigned sieve_grid = (unsigned)((tiles + 7) / 8);
    if (tiles) k_bgzf_sieve<<<sieve_grid, 256, 0, s>>>(e->in, e->len, SIEVE_TILE, e->tile_counts, nullptr, nullptr, 0);
    frt_launch_scan_u32(e->tile_counts, tiles, (u32 *)e->scan_parts, e->tile_base, e->tile_base + tiles + 1, s);
    if (tiles)
        k_bgzf_sieve<<<sieve_grid, 256, 0, s>>>(e->in, e->len, SIEVE_TILE, nullptr, e->tile_base, e->cand, e->n_cap);
    k_bgzf_tiling<<<(unsigned)((e->n_cap + 255) / 256 + 1), 256, 0, s>>>(e->in, e->len, e->cand, e->tile_base + tiles,
                                                                         e->n_cap, e->st);
    k_bgzf_walk<<<1, 32, 0, s>>>(e->in, e->len, e->cand, e->n_cap, e->st);
    unsigned mgrid = (unsigned)((e->n_cap + 255) / 256);
    k_bgzf_spans<<<mgrid, 256, 0, s>>>(e->in, e->len, e->cand, e->n_cap, e->st, e->in_off, e->in_len, e->isize,
                                      e->crc_expect, e->coffset);
    u64 parts = e->n_cap / 4096 + 1;
    k_scan64_partials<<<(unsigned)parts, 1024, 0, s>>>(e->isize, e->n_cap, e->scan_parts);
    k_scan64_partials_scan<<<1, 1024, 0, s>>>(e->scan_parts, parts);
    k_scan64_apply<<<(unsigned)parts, 1024, 0, s>>>(e->isize, e->n_cap, e->scan_parts, e->out_off,
                                                    &e->st->inflated_total);
    cudaMemsetAsync(e->hist, 0, 1024 * 4, s);
    if (e->cfg.sort_queue) {
        k_queue_hist<<<mgrid, 256, 0, s>>>(e->in_len, e->n_cap, e->hist);
        k_queue_cursor<<<1, 1024, 0, s>>>(e->hist, e->cursor);
        k_queue_scatter<<<mgrid, 256, 0, s>>>(e->in_len, e->n_cap, e->cursor, e->order);
    }
    return cudaGetLastError();
}

cudaError_t enqueue_inflate(frt_engine *e)
{
    return frt_launch_inflate_persistent(e->in, e->in_off, e->in_len, e->out, e->out_off, e->isize, e->crc_expect,
                                         e->status, e->produced, e->crc, e->cfg.sort_queue ? e->order : nullptr,
                                         &e->st->n_members, e->n_cap, e->out_cap, &e->st->queue_head, (u32)e->grid,
                                         (unsigned long long *)&e->st->block_err, e->tuning, e->stream);
}

void column_ptrs(frt_engine *e, FrtBamColumnsDev &c)
{
    c.ref_id = ecol<int>(e, FRT_COL_REF_ID);
    c.pos = ecol<int>(e, FRT_COL_POS);
    c.flags = ecol<u16>(e, FRT_COL_FLAGS);
    c.mapq = ecol<u8>(e, FRT_COL_MAPQ);
    c.seq_len = ecol<u32>(e, FRT_COL_SEQ_LEN);
    c.mate_ref_id = ecol<int>(e, FRT_COL_MATE_REF_ID);
    c.mate_pos = ecol<int>(e, FRT_COL_MATE_POS);
    c.tlen = ecol<int>(e, FRT_COL_TLEN);
    c.record_offsets = ecol<u64>(e, FRT_COL_RECORD_OFFSETS);
    c.cigar_start = ecol<u32>(e, FRT_COL_CIGAR_START);
    c.sequence_start = ecol<u32>(e, FRT_COL_SEQUENCE_START);
    c.quality_start = ecol<u32>(e, FRT_COL_QUALITY_START);
    c.aux_start = ecol<u32>(e, FRT_COL_AUX_START);
    c.record_end = ecol<u32>(e, FRT_COL_RECORD_END);
    c.bin = ecol<u16>(e, FRT_COL_BIN);
    c.n_cigar = ecol<u16>(e, FRT_COL_N_CIGAR);
    c.name_len = ecol<u8>(e, FRT_COL_NAME_LEN);
    c.virtual_offset = ecol<u64>(e, FRT_COL_VIRTUAL_OFFSET);
    c.aux_count = ecol<u32>(e, FRT_COL_AUX_COUNT);
    c.aux_status = ecol<u8>(e, FRT_COL_AUX_STATUS);
}

// Record stages: header, speculative scan, reconcile, and (once the record
// and aux counts are sized) decode and the aux directory.
cudaError_t enqueue_records(frt_engine *e, bool with_columns)
{
    cudaStream_t s = e->stream;
    k_bam_header<<<1, 32, 0, s>>>(e->out, &e->st->inflated_total, e->st);
    u32 n = (u32)e->n_cap;
    u64 len = e->out_cap; // scans stay inside the planned output
    frt_launch_bam_spec(e->out, len, e->out_off, n, 0, 0, e->entry, e->count, e->land, e->flags, e->scratch, s,
                        &e->st->records_start, &e->st->n_ref);
    frt_launch_bam_reconcile(e->out, len, e->out_off, n, 0, e->entry, e->count, e->land, e->flags, e->scratch,
                             e->first, e->st->totals, s, &e->st->records_start);
    if (!with_columns) return cudaGetLastError();
    FrtBamColumnsDev c;
    column_ptrs(e, c);
    frt_launch_bam_decode_capped(e->out, e->out_off, e->coffset, n, e->count, e->first, e->scratch, c, e->rec_cap, s);
    frt_launch_scan_u32(c.aux_count, e->rec_cap, e->aux_parts, ecol<u32>(e, FRT_COL_AUX_FIRST), &e->st->n_aux, s);
    k_check_counts<<<1, 32, 0, s>>>(e->st, e->rec_cap, e->aux_cap);
    frt_launch_bam_aux_dir_capped(e->out, c.record_offsets, c.aux_start, c.record_end, c.aux_count,
                                  ecol<u32>(e, FRT_COL_AUX_FIRST), e->aux_entries, &e->st->totals[0], e->rec_cap,
                                  e->aux_cap, s);
    return cudaGetLastError();
}

// Captures the steady state as a graph (when the engine uses one): front,
// inflate and, for one BAM, the record stages; several files replay front and
// inflate, their decoders running eagerly.  Drops any earlier graph.
cudaError_t capture_graph(frt_engine *e)
{
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->exec = nullptr;
    e->graph = nullptr;
    if (!e->cfg.use_graph) return cudaSuccess;
    cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
    if (ce != cudaSuccess) return ce;
    enqueue_front(e);
    enqueue_inflate(e);
    if (!e->multi) enqueue_records(e, true);
    ce = cudaStreamEndCapture(e->stream, &e->graph);
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&e->exec, e->graph, 0);
    return ce;
}

int stats_from_state(frt_engine *e, frt_engine_stats *stats, frt_error *err)
{
    EngineDevState &h = e->host_state;
    frt_engine_stats out{};
    out.members = h.n_members;
    out.compressed_bytes = e->len;
    out.inflated_bytes = h.inflated_total;
    out.records = h.totals[0];
    out.tail = h.totals[1];
    out.aux_fields = h.n_aux;
    out.fallbacks = h.totals[3];
    out.status = FRT_OK;
    out.error_member = 0xffffffffu;
    int rc = FRT_OK;
    if (h.walk_err) {
        set_error(err, FRT_ERR_INVALID_BLOCK, h.walk_err - 1, 0, 0, 0, nullptr, "not a BGZF member header");
        rc = FRT_ERR_INVALID_BLOCK;
    } else if (h.block_err != ~0ull) {
        u64 m = h.block_err >> 8;
        int code = (int)(h.block_err & 0xff);
        out.error_member = (uint32_t)m;
        uint32_t vals[3] = {0, 0, 0};
        uint64_t coff = 0;
        uint32_t want[2] = {0, 0};
        cudaMemcpy(&vals[0], e->status + m, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&vals[1], e->produced + m, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&vals[2], e->crc + m, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&coff, e->coffset + m, 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(&want[0], e->isize + m, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(&want[1], e->crc_expect + m, 4, cudaMemcpyDeviceToHost);
        if (code == FRT_ERR_INFLATE)
            set_error(err, code, coff, 0, 0, 0, nullptr, "%s", inflate_status_message(vals[0]));
        else if (code == FRT_ERR_SIZE)
            set_error(err, code, coff, want[0], vals[1], 0, nullptr, "ISIZE says %u bytes, inflated %u", want[0],
                      vals[1]);
        else if (code == FRT_ERR_CHECKSUM)
            set_error(err, code, coff, want[1], vals[2], 0, nullptr, "expected crc32 %#010x, got %#010x", want[1],
                      vals[2]);
        else
            set_error(err, code, coff, 0, 0, 0, nullptr, "invalid BGZF member");
        rc = code;
    } else if (h.tiling_failed && h.n_members == 0 && e->len) {
        set_error(err, FRT_ERR_INVALID_BLOCK, 0, 0, 0, 0, nullptr, "not a BGZF member header");
        rc = FRT_ERR_INVALID_BLOCK;
    } else if (h.capacity_err) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr,
                  "the bound buffer changed since bind: counts exceed the planned capacity");
        rc = FRT_ERR_INVALID_DEVICE_BATCH;
    } else if (h.header_status) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, 0, "bam header", "malformed BAM header");
        rc = FRT_ERR_MALFORMED;
    } else if (h.totals[2]) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, h.totals[1], "bam",
                  "malformed record reached from a confirmed boundary");
        rc = FRT_ERR_MALFORMED;
    }
    out.status = rc;
    if (stats) *stats = out;
    return rc;
}

void layout(frt_engine *e)
{
    size_t off = 0;
    for (int c = 0; c < FRT_COL_COUNT; ++c) {
        size_t bytes = c == FRT_COL_AUX_FIRST ? 4 * (e->rec_cap + 1)
                                              : (c == FRT_COL_AUX_ENTRIES ? 0 : bam_column_width(c) * e->rec_cap);
        e->col_off[c] = off;
        e->col_bytes[c] = bytes;
        off += (bytes + 255) & ~(size_t)255;
    }
}

size_t layout_total(frt_engine *e)
{
    size_t t = 0;
    for (int c = 0; c < FRT_COL_COUNT; ++c) t += (e->col_bytes[c] + 255) & ~(size_t)255;
    return t;
}

} // namespace

extern "C" int frt_engine_create(int device, void *stream, const frt_engine_config *cfg, frt_engine **out,
                                 frt_error *err)
{
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuardLite g(device);
    configure_pool(device);
    cudaError_t ce = frt_inflate_prepare();
    if (ce != cudaSuccess) return cuda_fail(err, ce, "configuring inflate kernels");
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    frt_engine *e = new frt_engine;
    e->device = device;
    e->shared = ss;
    e->stream = ss->s;
    if (cfg) e->cfg = *cfg;
    else e->cfg = frt_engine_config{0, 0, 1, 1};
    e->tuning = frt_inflate_default();
    if (e->cfg.warps_per_cta) e->tuning.warps_per_cta = (int32_t)e->cfg.warps_per_cta;
    if (e->cfg.queue_chunk) e->tuning.queue_chunk = (int32_t)e->cfg.queue_chunk;
    e->grid = frt_inflate_persistent_grid(e->tuning);
    if (e->grid < 1) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "inflate tuning (variant %d, %d warps per CTA, chunk %d) does not fit device %d", e->tuning.variant,
                  e->tuning.warps_per_cta, e->tuning.queue_chunk, device);
        stream_release(ss);
        delete e;
        return FRT_ERR_INVALID_ARGUMENT;
    }
    *out = e;
    return FRT_OK;
}

extern "C" void frt_engine_destroy(frt_engine *e)
{
    if (!e) return;
    DeviceGuardLite g(e->device);
    {
        auto &pp = e->pipe;
        if (pp.copy) cudaStreamSynchronize(pp.copy);
        for (cudaStream_t q : pp.lanes) cudaStreamSynchronize(q);
        for (cudaEvent_t ev : pp.up) cudaEventDestroy(ev);
        for (cudaEvent_t ev : pp.done) cudaEventDestroy(ev);
        if (pp.plan) cudaEventDestroy(pp.plan);
        if (pp.copy) cudaStreamDestroy(pp.copy);
        for (cudaStream_t q : pp.lanes) cudaStreamDestroy(q);
        if (pp.staging) cudaFreeHost(pp.staging);
        for (void *q : {(void *)pp.d_count, (void *)pp.d_errs, (void *)pp.d_first, (void *)pp.d_heads})
            if (q) cudaFree(q);
    }
    free_all(e);
    frt_bam_decoder_destroy(e->bam_dec);
    frt_fastq_scanner_destroy(e->fastq);
    frt_bcf_scanner_destroy(e->bcf);
    frt_fasta_compactor_destroy(e->fasta);
    stream_release(e->shared);
    delete e;
}

// Discovery, plan, queue and one eager inflate of a bound buffer; sizes every
// member-indexed buffer and the output.
static int bind_front(frt_engine *e, const uint8_t *dev_bgzf, size_t len, frt_error *err)
{
    free_all(e);
    e->in = dev_bgzf;
    e->len = len;
    e->tiles = (len + SIEVE_TILE - 1) / SIEVE_TILE;
    // Pass 1: discovery alone, to learn the member count.
    e->n_cap = 0;
    int rc;
    u64 tiles = e->tiles;
    if ((rc = ealloc(e, &e->st, 1, err))) return rc;
    if ((rc = ealloc(e, &e->tile_counts, tiles + 1, err))) return rc;
    if ((rc = ealloc(e, &e->tile_base, tiles + 2, err))) return rc;
    if ((rc = ealloc(e, &e->scan_parts, tiles / 4096 + 2 + 1, err))) return rc;
    cudaStream_t s = e->stream;
    cudaMemsetAsync(e->st, 0, sizeof(EngineDevState), s);
    unsigned sieve_grid = (unsigned)((tiles + 7) / 8);
    if (tiles) {
        k_bgzf_sieve<<<sieve_grid, 256, 0, s>>>(e->in, len, SIEVE_TILE, e->tile_counts, nullptr, nullptr, 0);
        frt_launch_scan_u32(e->tile_counts, tiles, (u32 *)e->scan_parts, e->tile_base, e->tile_base + tiles + 1, s);
    } else {
        cudaMemsetAsync(e->tile_base, 0, 8, s);
    }
    u32 n_cand = 0;
    cudaMemcpyAsync(&n_cand, e->tile_base + tiles, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "discovery");
    // Capacity: the candidates, or (if they do not tile) what a walk can find.
    e->n_cap = n_cand ? n_cand : 1;
    // Pass 2: size the member arrays, run discovery + plan + queue + inflate.
    u64 n = e->n_cap;
    u64 parts64 = n / 4096 + 2;
    if (parts64 > tiles / 4096 + 3) {
        if ((rc = ealloc(e, &e->scan_parts, parts64 + 1, err))) return rc;
    }
    if ((rc = ealloc(e, &e->cand, n, err)) || (rc = ealloc(e, &e->in_off, n, err)) ||
        (rc = ealloc(e, &e->coffset, n + 1, err)) || (rc = ealloc(e, &e->out_off, n + 1, err)) ||
        (rc = ealloc(e, &e->in_len, n, err)) || (rc = ealloc(e, &e->isize, n, err)) ||
        (rc = ealloc(e, &e->crc_expect, n, err)) || (rc = ealloc(e, &e->order, n, err)) ||
        (rc = ealloc(e, &e->hist, 1024, err)) || (rc = ealloc(e, &e->cursor, 1024, err)) ||
        (rc = ealloc(e, &e->status, n, err)) || (rc = ealloc(e, &e->produced, n, err)) ||
        (rc = ealloc(e, &e->crc, n, err)))
        return rc;
    // plan once to learn the inflated size
    e->out_cap = 0;
    e->out = nullptr;
    if ((ce = enqueue_front(e)) != cudaSuccess) return cuda_fail(err, ce, "planning");
    EngineDevState h{};
    cudaMemcpyAsync(&h, e->st, sizeof h, cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(err, ce, "planning");
    if (h.tiling_failed && h.n_members > n) {
        set_error(err, FRT_ERR_INVALID_BLOCK, 0, 0, 0, 0, nullptr, "BGZF members do not tile the buffer");
        return FRT_ERR_INVALID_BLOCK;
    }
    e->out_cap = h.inflated_total;
    if ((rc = ealloc(e, &e->out, e->out_cap + 64, err))) return rc;
    if ((ce = enqueue_inflate(e)) != cudaSuccess) return cuda_fail(err, ce, "inflate");
    return FRT_OK;
}

extern "C" int frt_engine_bind_bam(frt_engine *e, const uint8_t *dev_bgzf, size_t len, frt_error *err)
{
    DeviceGuardLite g(e->device);
    int rc = bind_front(e, dev_bgzf, len, err);
    if (rc) return rc;
    cudaStream_t s = e->stream;
    cudaError_t ce;
    u64 n = e->n_cap;
    EngineDevState h{};
    // Record scan once to learn the record count.
    if ((rc = ealloc(e, &e->entry, n, err)) || (rc = ealloc(e, &e->land, n, err)) ||
        (rc = ealloc(e, &e->count, n, err)) || (rc = ealloc(e, &e->first, n, err)) ||
        (rc = ealloc(e, &e->flags, n, err)) || (rc = ealloc(e, &e->scratch, n * FRT_SCAN_CAP, err)))
        return rc;
    if ((ce = enqueue_records(e, false)) != cudaSuccess) return cuda_fail(err, ce, "record scan");
    cudaMemcpyAsync(&h, e->st, sizeof h, cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(err, ce, "record scan");
    e->host_state = h;
    if ((rc = stats_from_state(e, nullptr, err))) return rc;
    e->rec_cap = h.totals[0];
    layout(e);
    if ((rc = ealloc(e, &e->cols, layout_total(e), err))) return rc;
    if ((rc = ealloc(e, &e->aux_parts, e->rec_cap / 4096 + 2, err))) return rc;
    // aux count: decode once with no directory capacity, then size it
    e->aux_cap = 0;
    e->aux_entries = nullptr;
    if ((ce = enqueue_records(e, true)) != cudaSuccess) return cuda_fail(err, ce, "decode");
    cudaMemcpyAsync(&h, e->st, sizeof h, cudaMemcpyDeviceToHost, s);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(err, ce, "decode");
    e->aux_cap = h.n_aux;
    if ((rc = ealloc(e, &e->aux_entries, 3 * (e->aux_cap + 1), err))) return rc;
    e->col_bytes[FRT_COL_AUX_ENTRIES] = 12 * e->aux_cap;
    // Capture the steady state.
    if ((ce = capture_graph(e)) != cudaSuccess) return cuda_fail(err, ce, "capturing the engine graph");
    return FRT_OK;
}


// ---- several files ---------------------------------------------------------

namespace {

// Parses a header from the start of a file's inflated range, growing the
// host copy until the parse succeeds or the range is exhausted.
template <typename Parse> int parse_prefix(frt_engine *e, const frt_engine::File &f, Parse parse, frt_error *err)
{
    u64 len = f.out1 - f.out0;
    std::vector<uint8_t> host;
    for (u64 take = 1u << 16;; take *= 4) {
        u64 n = take < len ? take : len;
        host.resize(n);
        cudaError_t ce = cudaMemcpyAsync(host.data(), e->out + f.out0, n, cudaMemcpyDeviceToHost, e->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
        if (ce != cudaSuccess) return cuda_fail(err, ce, "reading a header");
        int rc = parse(host.data(), n, err);
        if (rc == FRT_OK || rc != FRT_ERR_MALFORMED || n == len) return rc;
    }
}

// Each file's decoder over its inflated range (the views' events order them
// after the inflate).
int decode_files(frt_engine *e, frt_error *err)
{
    release_results(e);
    for (auto &f : e->files) {
        cudaEventRecord(f.view->ready, e->stream);
        cudaEventRecord(f.t0, e->stream);
        int rc = FRT_OK;
        switch (f.desc.format) {
        case FRT_FORMAT_BAM:
            frt_bam_decoder_set_reference_count(e->bam_dec, f.n_ref);
            rc = frt_bam_decode(e->bam_dec, f.view, f.records_start, &f.bam, err);
            break;
        case FRT_FORMAT_BCF:
            rc = frt_bcf_decode(e->bcf, f.view, f.records_start, f.samples, f.contigs, &f.cols, err);
            break;
        case FRT_FORMAT_FASTQ:
            rc = frt_fastq_decode(e->fastq, f.view, 0, &f.cols, err);
            break;
        default:
            rc = frt_fasta_compact(e->fasta, f.view, &f.cols, err);
            break;
        }
        cudaEventRecord(f.t1, e->stream);
        if (rc) return rc;
    }
    return FRT_OK;
}

// Kernels each decoder launches (counted from their launch sequences in
// decoder.cu and formats.cu; the BCF walk adds two when it runs).
uint64_t decode_launches(const frt_engine::File &f)
{
    switch (f.desc.format) {
    case FRT_FORMAT_BAM: return 7;   // spec, reconcile, decode, 3-kernel scan, aux directory
    case FRT_FORMAT_BCF: return 8;   // sieve, 3-kernel scan, gather, check, finalize, decode
    case FRT_FORMAT_FASTQ: return 13; // newline slots, scan, gather, line count, scan, line emit, check, finalize, decode
    default: return 6;                // sum, chunk scan, top, apply, emit, lengths
    }
}

// Inflate errors first: decoding garbage would only hide them.
int inflate_status(frt_engine *e, frt_error *err)
{
    cudaMemcpyAsync(&e->host_state, e->st, sizeof(EngineDevState), cudaMemcpyDeviceToHost, e->stream);
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "engine run");
    EngineDevState &h = e->host_state;
    if (h.walk_err || h.block_err != ~0ull || (h.tiling_failed && h.n_members == 0 && e->len))
        return stats_from_state(e, nullptr, err);
    return FRT_OK;
}

int run_multi(frt_engine *e, frt_error *err)
{
    cudaError_t ce;
    if (e->exec) {
        ce = cudaGraphLaunch(e->exec, e->stream);
    } else {
        enqueue_front(e);
        ce = enqueue_inflate(e);
    }
    if (ce != cudaSuccess) return cuda_fail(err, ce, "launching the engine");
    int rc = inflate_status(e, err);
    if (rc) return rc;
    return decode_files(e, err);
}

} // namespace

extern "C" int frt_engine_bind_files(frt_engine *e, const uint8_t *dev, size_t len, const frt_engine_file *files,
                                     size_t n_files, frt_error *err)
{
    if (!e || (!files && n_files)) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(e->device);
    // the files must tile the buffer, in order
    uint64_t at = 0;
    for (size_t i = 0; i < n_files; ++i) {
        if (files[i].offset != at || files[i].format < FRT_FORMAT_BAM || files[i].format > FRT_FORMAT_FASTA) {
            set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                      "file %zu: files must lie back to back from offset 0 with a known format", i);
            return FRT_ERR_INVALID_ARGUMENT;
        }
        at += files[i].length;
    }
    if (at != len) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "the files cover %llu of %zu bytes",
                  (unsigned long long)at, len);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    int rc = bind_front(e, dev, len, err);
    if (rc) return rc;
    cudaStream_t s = e->stream;
    EngineDevState h{};
    cudaMemcpyAsync(&h, e->st, sizeof h, cudaMemcpyDeviceToHost, s);
    cudaError_t ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "inflate");
    e->host_state = h;
    if ((rc = stats_from_state(e, nullptr, err))) return rc;
    const u64 n = h.n_members;
    std::vector<uint64_t> coff(n + 1), out_off(n + 1);
    if (n) {
        cudaMemcpyAsync(coff.data(), e->coffset, 8 * n, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(out_off.data(), e->out_off, 8 * (n + 1), cudaMemcpyDeviceToHost, s);
        if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(err, ce, "reading the plan");
    }
    coff[n] = len;
    e->multi = true;
    e->bound_coff.assign(coff.begin(), coff.begin() + n);
    e->bound_out_off = out_off;
    // decoders on the engine's stream
    if (!e->bam_dec && (rc = frt_bam_decoder_create(e->device, s, &e->bam_dec, err))) return rc;
    if (!e->fastq && (rc = frt_fastq_scanner_create(e->device, s, &e->fastq, err))) return rc;
    if (!e->bcf && (rc = frt_bcf_scanner_create(e->device, s, &e->bcf, err))) return rc;
    if (!e->fasta && (rc = frt_fasta_compactor_create(e->device, s, &e->fasta, err))) return rc;
    e->files.resize(n_files);
    for (size_t i = 0; i < n_files; ++i) {
        auto &f = e->files[i];
        f.desc = files[i];
        f.m0 = (u64)(std::lower_bound(coff.begin(), coff.begin() + n, files[i].offset) - coff.begin());
        f.m1 = (u64)(std::lower_bound(coff.begin(), coff.begin() + n, files[i].offset + files[i].length) - coff.begin());
        if (f.m0 < n && coff[f.m0] != files[i].offset) {
            set_error(err, FRT_ERR_INVALID_ARGUMENT, files[i].offset, 0, 0, 0, nullptr,
                      "file %zu does not start on a BGZF member", i);
            return FRT_ERR_INVALID_ARGUMENT;
        }
        f.out0 = out_off[f.m0];
        f.out1 = out_off[f.m1];
        // a non-owning batch over the file's inflated bytes
        frt_inflate_batch *v = new frt_inflate_batch;
        v->device = e->device;
        v->stream = s;
        v->shared = stream_retain(e->shared);
        v->owns_data = false;
        v->data = e->out + f.out0;
        v->len = f.out1 - f.out0;
        u64 k = f.m1 - f.m0;
        v->offsets.resize(k + 1);
        v->coffsets.resize(k);
        for (u64 j = 0; j <= k; ++j) v->offsets[j] = out_off[f.m0 + j] - f.out0;
        for (u64 j = 0; j < k; ++j) v->coffsets[j] = coff[f.m0 + j] - files[i].offset;
        std::vector<uint64_t> dev_off(2 * k + 1);
        std::copy(v->offsets.begin(), v->offsets.end(), dev_off.begin());
        std::copy(v->coffsets.begin(), v->coffsets.end(), dev_off.begin() + k + 1);
        cudaEventCreateWithFlags(&v->ready, cudaEventDisableTiming);
        cudaEventCreate(&f.t0);
        cudaEventCreate(&f.t1);
        f.view = v;
        if ((rc = dev_alloc((void **)&v->d_offsets, 8 * dev_off.size(), s, err))) return rc;
        if ((ce = cudaMemcpyAsync(v->d_offsets, dev_off.data(), 8 * dev_off.size(), cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
            return cuda_fail(err, ce, "uploading a file's member offsets");
        if (f.desc.format == FRT_FORMAT_BAM && v->len) {
            rc = parse_prefix(e, f, [&](const uint8_t *b, u64 m, frt_error *er) {
                return frt_bam_parse_header(b, m, &f.records_start, &f.n_ref, er);
            }, err);
        } else if (f.desc.format == FRT_FORMAT_BCF && v->len) {
            rc = parse_prefix(e, f, [&](const uint8_t *b, u64 m, frt_error *er) {
                return frt_bcf_parse_header(b, m, &f.records_start, &f.samples, &f.contigs, er);
            }, err);
        }
        if (rc) return rc;
    }
    cudaStreamSynchronize(s); // the offsets uploads read from host vectors
    if ((rc = decode_files(e, err))) return rc;
    if ((ce = capture_graph(e)) != cudaSuccess) return cuda_fail(err, ce, "capturing the engine graph");
    return FRT_OK;
}

extern "C" size_t frt_engine_file_count(const frt_engine *e) { return e ? e->files.size() : 0; }

extern "C" int frt_engine_get_file_info(const frt_engine *e, size_t i, frt_engine_file_info *info)
{
    if (!e || i >= e->files.size() || !info) return FRT_ERR_INVALID_ARGUMENT;
    const auto &f = e->files[i];
    frt_engine_file_info o{};
    o.format = f.desc.format;
    o.members = f.m1 - f.m0;
    o.compressed_bytes = f.desc.length;
    o.inflated_offset = f.out0;
    o.inflated_bytes = f.out1 - f.out0;
    if (f.bam) {
        o.records = frt_record_batch_len(f.bam);
        o.tail = frt_record_batch_tail(f.bam);
    } else if (f.cols) {
        o.records = frt_columns_len(f.cols);
        o.tail = f.desc.format == FRT_FORMAT_FASTA ? frt_columns_total_bases(f.cols) : frt_columns_tail(f.cols);
        frt_columns_scan_info(f.cols, &o.proof, nullptr, nullptr);
    }
    float ms = 0;
    if (f.t1 && cudaEventSynchronize(f.t1) == cudaSuccess && cudaEventElapsedTime(&ms, f.t0, f.t1) == cudaSuccess)
        o.decode_ms = ms;
    o.launches = decode_launches(f);
    *info = o;
    return FRT_OK;
}

extern "C" const frt_record_batch *frt_engine_file_bam(const frt_engine *e, size_t i)
{
    return e && i < e->files.size() ? e->files[i].bam : nullptr;
}

extern "C" const frt_columns *frt_engine_file_columns(const frt_engine *e, size_t i)
{
    return e && i < e->files.size() ? e->files[i].cols : nullptr;
}

extern "C" int frt_engine_run(frt_engine *e, frt_error *err)
{
    DeviceGuardLite g(e->device);
    if (!e->in && e->len) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "no file bound");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (e->multi) {
        e->decode_rc = run_multi(e, &e->decode_err);
        if (e->decode_rc && err) *err = e->decode_err;
        return e->decode_rc;
    }
    cudaError_t ce;
    if (e->exec) {
        ce = cudaGraphLaunch(e->exec, e->stream);
    } else {
        enqueue_front(e);
        enqueue_inflate(e);
        ce = enqueue_records(e, true);
    }
    if (ce != cudaSuccess) return cuda_fail(err, ce, "launching the engine");
    return FRT_OK;
}

extern "C" int frt_engine_get_tuning(const frt_engine *e, frt_inflate_tuning *out)
{
    if (!e || !out) return FRT_ERR_INVALID_ARGUMENT;
    *out = e->tuning;
    return FRT_OK;
}

extern "C" int frt_engine_set_tuning(frt_engine *e, const frt_inflate_tuning *t, frt_error *err)
{
    if (!e || !t) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(e->device);
    const int grid = frt_inflate_persistent_grid(*t);
    if (grid < 1) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "inflate tuning (variant %d, %d warps per CTA, %d CTAs per SM, chunk %d) is invalid or does not "
                  "fit device %d",
                  t->variant, t->warps_per_cta, t->ctas_per_sm, t->queue_chunk, e->device);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    e->tuning = *t;
    e->grid = grid;
    if (e->in) {
        cudaError_t ce = capture_graph(e);
        if (ce != cudaSuccess) return cuda_fail(err, ce, "capturing the engine graph");
    }
    return FRT_OK;
}

extern "C" int frt_engine_time_inflate(frt_engine *e, const frt_inflate_tuning *t, uint64_t members, int32_t reps,
                                       double *ms, uint64_t *inflated_bytes, frt_error *err)
{
    if (!e || !t || !ms) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(e->device);
    if (!e->in || e->n_cap == 0) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "no file bound");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    const int grid = frt_inflate_persistent_grid(*t);
    if (grid < 1) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "inflate tuning (variant %d, %d warps per CTA, %d CTAs per SM, chunk %d) is invalid or does not "
                  "fit device %d",
                  t->variant, t->warps_per_cta, t->ctas_per_sm, t->queue_chunk, e->device);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    const u64 k = members && members < e->n_cap ? members : e->n_cap;
    cudaStream_t s = e->stream;
    cudaError_t ce;
    u64 last_off = 0;
    u32 last_size = 0;
    if ((ce = cudaMemcpyAsync(&last_off, e->out_off + (k - 1), 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(&last_size, e->isize + (k - 1), 4, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(err, ce, "reading the plan");
    if (inflated_bytes) *inflated_bytes = last_off + last_size;
    cudaEvent_t ev[2];
    if ((ce = cudaEventCreate(&ev[0])) != cudaSuccess) return cuda_fail(err, ce, "creating events");
    if ((ce = cudaEventCreate(&ev[1])) != cudaSuccess) {
        cudaEventDestroy(ev[0]);
        return cuda_fail(err, ce, "creating events");
    }
    double best = 0;
    unsigned long long block_err = ~0ull;
    for (int r = 0; r <= (reps > 0 ? reps : 1) && ce == cudaSuccess; ++r) { // the first launch warms up
        if ((ce = cudaMemsetAsync(&e->st->queue_head, 0, sizeof(u32), s)) != cudaSuccess) break;
        if ((ce = cudaMemsetAsync(&e->st->block_err, 0xff, sizeof(unsigned long long), s)) != cudaSuccess) break;
        if ((ce = cudaEventRecord(ev[0], s)) != cudaSuccess) break;
        if ((ce = frt_launch_inflate_persistent(e->in, e->in_off, e->in_len, e->out, e->out_off, e->isize,
                                                e->crc_expect, e->status, e->produced, e->crc, nullptr,
                                                &e->st->n_members, k, e->out_cap, &e->st->queue_head, (u32)grid,
                                                (unsigned long long *)&e->st->block_err, *t, s)) != cudaSuccess)
            break;
        if ((ce = cudaEventRecord(ev[1], s)) != cudaSuccess) break;
        if ((ce = cudaMemcpyAsync(&block_err, &e->st->block_err, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((ce = cudaEventSynchronize(ev[1])) != cudaSuccess || (ce = cudaStreamSynchronize(s)) != cudaSuccess) break;
        float t_ms = 0;
        if ((ce = cudaEventElapsedTime(&t_ms, ev[0], ev[1])) != cudaSuccess) break;
        if (block_err != ~0ull) break;
        if (r > 0 && (best == 0 || t_ms < best)) best = t_ms;
    }
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "timing the inflate");
    if (block_err != ~0ull) {
        const u64 m = block_err >> 8;
        set_error(err, FRT_ERR_MALFORMED, m, 0, block_err & 0xff, 0, "bgzf",
                  "member %llu failed its trailer check while timing the inflate", (unsigned long long)m);
        return FRT_ERR_MALFORMED;
    }
    *ms = best;
    return FRT_OK;
}

extern "C" int frt_engine_finish(frt_engine *e, frt_engine_stats *stats, frt_error *err)
{
    DeviceGuardLite g(e->device);
    cudaMemcpyAsync(&e->host_state, e->st, sizeof(EngineDevState), cudaMemcpyDeviceToHost, e->stream);
    cudaError_t ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "engine run");
    if (!e->multi) return stats_from_state(e, stats, err);
    // several files: the inflate's own errors, then the decoders'
    frt_engine_stats out{};
    int rc = stats_from_state(e, &out, err);
    out.records = out.tail = out.aux_fields = out.fallbacks = 0;
    for (auto &f : e->files) {
        if (f.bam) {
            out.records += frt_record_batch_len(f.bam);
            out.aux_fields += frt_record_batch_aux_fields(f.bam);
        } else if (f.cols) {
            out.records += frt_columns_len(f.cols);
        }
    }
    if (!rc && e->decode_rc) {
        rc = e->decode_rc;
        if (err) *err = e->decode_err;
    }
    out.status = rc;
    if (stats) *stats = out;
    return rc;
}

namespace {

constexpr int kPipeSlices = 8; // upload slices, and at most this many inflate groups

// A host-buffer run of one bound BAM with the upload overlapped: the file goes
// to the device in slices on a copy stream while the host walks the member
// headers (the plan the device front would compute: member spans, trailers,
// output offsets); each group of members whose bytes have all arrived is
// inflated by its own launch of the persistent kernel (longest member first
// within the group) on a stream of its own, so each launch's CTAs take the SMs
// as the ones before retire -- a group of a small file may hold fewer members
// than the GPU has warps; the record stages then run on the engine stream.  Returns 1 when
// the host plan does not match the bound file (the caller then runs the
// single-launch path on the uploaded bytes), else an frt_status.
int run_host_pipelined(frt_engine *e, const uint8_t *host, size_t len, frt_error *err)
{
    auto &pp = e->pipe;
    cudaError_t ce;
    if (!pp.copy) {
        if ((ce = cudaStreamCreateWithFlags(&pp.copy, cudaStreamNonBlocking)) != cudaSuccess ||
            (ce = cudaEventCreateWithFlags(&pp.plan, cudaEventDisableTiming)) != cudaSuccess)
            return cuda_fail(err, ce, "creating the upload streams");
        pp.lanes.assign(kPipeSlices, nullptr);
        for (int k = 0; k < kPipeSlices; ++k)
            if ((ce = cudaStreamCreateWithFlags(&pp.lanes[k], cudaStreamNonBlocking)) != cudaSuccess)
                return cuda_fail(err, ce, "creating the inflate streams");
        pp.up.resize(kPipeSlices);
        pp.done.resize(kPipeSlices);
        for (int k = 0; k < kPipeSlices; ++k)
            if ((ce = cudaEventCreateWithFlags(&pp.up[k], cudaEventDisableTiming)) != cudaSuccess ||
                (ce = cudaEventCreateWithFlags(&pp.done[k], cudaEventDisableTiming)) != cudaSuccess)
                return cuda_fail(err, ce, "creating the upload events");
        if ((ce = cudaMalloc(&pp.d_count, 8 * kPipeSlices)) != cudaSuccess ||
            (ce = cudaMalloc(&pp.d_errs, 8 * kPipeSlices)) != cudaSuccess ||
            (ce = cudaMalloc(&pp.d_first, 8 * kPipeSlices)) != cudaSuccess ||
            (ce = cudaMalloc(&pp.d_heads, 4 * kPipeSlices)) != cudaSuccess)
            return cuda_fail(err, ce, "allocating the group state");
    }
    // the previous run's inflate streams are done before its buffers are reused
    if ((ce = cudaStreamWaitEvent(pp.copy, pp.plan, 0)) != cudaSuccess) return cuda_fail(err, ce, "ordering uploads");
    // The copy stream carries slice 0, slice 1, plan 0, slice 2, plan 1, ...:
    // a group's plan follows its own slice with one slice of lookahead, so it
    // never waits behind the whole file on the copy engine.
    constexpr int kLookahead = 2;
    u64 slice_end[kPipeSlices];
    for (int k = 0; k < kPipeSlices; ++k) slice_end[k] = (u64)len * (k + 1) / kPipeSlices;
    int issued = 0; // slices on the copy stream
    auto upload_through = [&](int last) -> cudaError_t {
        for (; issued <= last && issued < kPipeSlices; ++issued) {
            const u64 a = issued ? slice_end[issued - 1] : 0, b = slice_end[issued];
            if (b > a) {
                cudaError_t c = cudaMemcpyAsync((void *)(e->in + a), host + a, b - a, cudaMemcpyHostToDevice, pp.copy);
                if (c != cudaSuccess) return c;
            }
        }
        return cudaSuccess;
    };
    if ((ce = upload_through(kLookahead - 1)) != cudaSuccess) return cuda_fail(err, ce, "uploading the file");
    // The plan, on the host, one slice at a time while the slices travel: a
    // group is the members whose blocks end in its slice, and it launches as
    // soon as its slice is walked and uploaded.
    const u64 cap = e->n_cap;
    const size_t need = cap * (8 + 4 + 4 + 4 + 8 + 4) + 8 * (cap + 1) + sizeof(EngineDevState) + 8 * 4 * kPipeSlices + 64;
    if (need > pp.staging_bytes) {
        if (pp.staging) cudaFreeHost(pp.staging);
        pp.staging = nullptr;
        if ((ce = cudaHostAlloc(&pp.staging, need, cudaHostAllocDefault)) != cudaSuccess)
            return cuda_fail(err, ce, "allocating the plan staging");
        pp.staging_bytes = need;
    }
    uint8_t *at = pp.staging;
    auto take = [&](size_t bytes) {
        uint8_t *q = at;
        at += (bytes + 7) & ~(size_t)7;
        return q;
    };
    u64 *h_in_off = (u64 *)take(8 * cap), *h_coff = (u64 *)take(8 * cap), *h_out_off = (u64 *)take(8 * (cap + 1));
    u32 *h_in_len = (u32 *)take(4 * cap), *h_isize = (u32 *)take(4 * cap), *h_crc = (u32 *)take(4 * cap);
    u32 *h_order = (u32 *)take(4 * cap);
    EngineDevState *h_st = (EngineDevState *)take(sizeof(EngineDevState));
    u64 *h_count = (u64 *)take(8 * kPipeSlices), *h_first = (u64 *)take(8 * kPipeSlices);
    cudaStream_t s = e->stream;
    if ((ce = cudaMemsetAsync(pp.d_errs, 0xff, 8 * kPipeSlices, s)) != cudaSuccess ||
        (ce = cudaMemsetAsync(pp.d_heads, 0, 4 * kPipeSlices, s)) != cudaSuccess ||
        (ce = cudaEventRecord(pp.plan, s)) != cudaSuccess)
        return cuda_fail(err, ce, "resetting the group state");
    int groups = 0;
    // on a plan that differs from the bound file's, the groups already
    // launched finish before the caller's fallback run rewrites their output
    auto bail = [&]() {
        for (int k = 0; k < groups; ++k) cudaStreamWaitEvent(s, pp.done[k], 0);
        return upload_through(kPipeSlices - 1) == cudaSuccess ? 1 : FRT_ERR_CUDA;
    };
    std::vector<frt_span> spans;
    spans.reserve(cap);
    u64 pos = 0, acc = 0, m0 = 0;
    std::vector<u32> idx;
    for (int k = 0; k < kPipeSlices; ++k) {
        size_t consumed = 0;
        frt_error scratch{};
        if (slice_end[k] > pos &&
            discover(host + pos, slice_end[k] - pos, pos, spans, &consumed, &scratch) != FRT_OK)
            return bail();
        const u64 m1 = spans.size();
        if (m1 > cap) return bail();
        for (u64 m = m0; m < m1; ++m) {
            h_in_off[m] = pos + spans[m].payload_start; // discover's payload_start is relative to its buffer
            h_in_len[m] = (u32)spans[m].payload_len;
            h_isize[m] = spans[m].isize;
            h_crc[m] = spans[m].crc32;
            h_coff[m] = spans[m].compressed_offset;
            h_out_off[m] = acc;
            acc += spans[m].isize;
        }
        pos += consumed;
        if (acc > e->out_cap) return bail();
        if (e->multi) // the per-file views hold the bound plan's offsets
            for (u64 m = m0; m < m1; ++m)
                if (h_coff[m] != e->bound_coff[m] || h_out_off[m] != e->bound_out_off[m]) return bail();
        h_first[k] = m0;
        h_count[k] = m1 - m0;
        // longest first within the group, as the single launch's queue
        idx.resize(m1 - m0);
        for (u64 q = 0; q < m1 - m0; ++q) idx[q] = (u32)q;
        std::stable_sort(idx.begin(), idx.end(), [&](u32 a, u32 b) {
            return spans[m0 + a].payload_len > spans[m0 + b].payload_len;
        });
        std::copy(idx.begin(), idx.end(), h_order + m0);
        cudaStream_t sg = pp.lanes[k];
        struct Copy {
            void *dst;
            const void *src;
            size_t bytes;
        } copies[] = {{e->in_off + m0, h_in_off + m0, 8 * (m1 - m0)},    {e->coffset + m0, h_coff + m0, 8 * (m1 - m0)},
                      {e->out_off + m0, h_out_off + m0, 8 * (m1 - m0)},  {e->in_len + m0, h_in_len + m0, 4 * (m1 - m0)},
                      {e->isize + m0, h_isize + m0, 4 * (m1 - m0)},      {e->crc_expect + m0, h_crc + m0, 4 * (m1 - m0)},
                      {e->order + m0, h_order + m0, 4 * (m1 - m0)},      {pp.d_count + k, h_count + k, 8},
                      {pp.d_first + k, h_first + k, 8}};
        for (const Copy &c : copies)
            if (c.bytes && (ce = cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyHostToDevice, pp.copy)) != cudaSuccess)
                return cuda_fail(err, ce, "uploading the plan");
        // slice k and plan k are on the device once up[k] fires
        if ((ce = cudaEventRecord(pp.up[k], pp.copy)) != cudaSuccess ||
            (ce = upload_through(k + kLookahead)) != cudaSuccess)
            return cuda_fail(err, ce, "uploading the file");
        if ((ce = cudaStreamWaitEvent(sg, pp.plan, 0)) != cudaSuccess ||
            (ce = cudaStreamWaitEvent(sg, pp.up[k], 0)) != cudaSuccess)
            return cuda_fail(err, ce, "ordering the inflate");
        if (m1 > m0 &&
            (ce = frt_launch_inflate_persistent(e->in, e->in_off + m0, e->in_len + m0, e->out, e->out_off + m0,
                                                e->isize + m0, e->crc_expect + m0, e->status + m0, e->produced + m0,
                                                e->crc + m0, e->order + m0, pp.d_count + k, m1 - m0, e->out_cap,
                                                pp.d_heads + k, (u32)e->grid, (unsigned long long *)(pp.d_errs + k),
                                                e->tuning, sg)) != cudaSuccess)
            return cuda_fail(err, ce, "launching the inflate");
        if ((ce = cudaEventRecord(pp.done[k], sg)) != cudaSuccess) return cuda_fail(err, ce, "ordering the inflate");
        groups = k + 1;
        m0 = m1;
    }
    if (pos != len || m0 != cap || (e->multi && acc != e->bound_out_off[cap])) return bail();
    const u64 n = m0;
    h_out_off[n] = acc;
    memset(h_st, 0, sizeof(EngineDevState));
    h_st->block_err = ~0ull;
    h_st->n_members = n;
    h_st->inflated_total = acc;
    for (int k = 0; k < groups; ++k)
        if ((ce = cudaStreamWaitEvent(s, pp.done[k], 0)) != cudaSuccess) return cuda_fail(err, ce, "joining the inflate");
    if ((ce = cudaMemcpyAsync(e->out_off + n, h_out_off + n, 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(e->st, h_st, sizeof(EngineDevState), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(err, ce, "uploading the totals");
    // the next run's uploads wait for everything that reads this run's staging
    k_merge_group_errors<<<1, 32, 0, s>>>(pp.d_errs, pp.d_first, (u32)groups, e->st);
    if (!e->multi && (ce = enqueue_records(e, true)) != cudaSuccess)
        return cuda_fail(err, ce, "launching the record stages");
    if ((ce = cudaEventRecord(pp.plan, s)) != cudaSuccess) return cuda_fail(err, ce, "ordering the run");
    return FRT_OK;
}

} // namespace

extern "C" int frt_engine_run_host(frt_engine *e, const uint8_t *host, size_t len, frt_engine_stats *stats,
                                   frt_error *err)
{
    DeviceGuardLite g(e->device);
    if (!e->in || len != e->len) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "bind a device buffer of this length first; run_host refills it from host memory");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    int rc = run_host_pipelined(e, host, len, err);
    if (rc == FRT_OK) {
        if (e->multi) { // the inflate's status, then each file's decoder, as run_multi
            e->decode_rc = inflate_status(e, &e->decode_err);
            if (!e->decode_rc) e->decode_rc = decode_files(e, &e->decode_err);
            if (e->decode_rc) {
                if (err) *err = e->decode_err;
                return e->decode_rc;
            }
        }
        return frt_engine_finish(e, stats, err);
    }
    if (rc != 1) return rc;
    // the host plan differs from the bound file's: the bytes are (being)
    // uploaded on the copy stream; run the single launch after them
    cudaError_t ce = cudaEventRecord(e->pipe.up[kPipeSlices - 1], e->pipe.copy);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e->stream, e->pipe.up[kPipeSlices - 1], 0);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "ordering after the upload");
    rc = frt_engine_run(e, err);
    if (rc) return rc;
    return frt_engine_finish(e, stats, err);
}

extern "C" int frt_engine_column(const frt_engine *e, int column, void **ptr, size_t *bytes, size_t *width)
{
    if (!e || column < 0 || column >= FRT_COL_COUNT) return FRT_ERR_INVALID_ARGUMENT;
    u64 n = e->host_state.totals[0] < e->rec_cap ? e->host_state.totals[0] : e->rec_cap;
    if (ptr) *ptr = column == FRT_COL_AUX_ENTRIES ? (void *)e->aux_entries : (void *)(e->cols + e->col_off[column]);
    if (bytes) {
        if (column == FRT_COL_AUX_ENTRIES) *bytes = 12ull * e->host_state.n_aux;
        else if (column == FRT_COL_AUX_FIRST) *bytes = 4ull * (n + 1);
        else *bytes = bam_column_width(column) * n;
    }
    if (width) *width = bam_column_width(column);
    return FRT_OK;
}

extern "C" int frt_engine_column_to_host(const frt_engine *e, int column, void *dst, size_t cap, frt_error *err)
{
    void *p = nullptr;
    size_t bytes = 0;
    if (frt_engine_column(e, column, &p, &bytes, nullptr)) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "bad column %d", column);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (cap < bytes) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "destination too small");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(e->device);
    cudaError_t ce = cudaMemcpyAsync(dst, p, bytes, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "downloading column");
    return FRT_OK;
}

extern "C" const uint8_t *frt_engine_inflated(const frt_engine *e, size_t *len)
{
    if (len) *len = e ? e->host_state.inflated_total : 0;
    return e ? e->out : nullptr;
}

// ---- record fields over the engine's last run -------------------------------
static int engine_fields(const frt_engine *e, int op, const char *tag, frt_columns **out, frt_error *err)
{
    if (!e || !e->in || e->multi) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "record fields need an engine with one BAM bound (a batch of several files: use its file's records)");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    frt_engine *m = const_cast<frt_engine *>(e);
    RecordView v;
    v.buf = e->out;
    v.n = e->host_state.totals[0] < e->rec_cap ? e->host_state.totals[0] : e->rec_cap;
    v.record_offsets = ecol<uint64_t>(m, FRT_COL_RECORD_OFFSETS);
    v.cigar_start = ecol<uint32_t>(m, FRT_COL_CIGAR_START);
    v.sequence_start = ecol<uint32_t>(m, FRT_COL_SEQUENCE_START);
    v.quality_start = ecol<uint32_t>(m, FRT_COL_QUALITY_START);
    v.aux_start = ecol<uint32_t>(m, FRT_COL_AUX_START);
    v.record_end = ecol<uint32_t>(m, FRT_COL_RECORD_END);
    v.seq_len = ecol<uint32_t>(m, FRT_COL_SEQ_LEN);
    v.aux_count = ecol<uint32_t>(m, FRT_COL_AUX_COUNT);
    v.aux_first = ecol<uint32_t>(m, FRT_COL_AUX_FIRST);
    v.aux_entries = e->aux_entries;
    v.n_cigar = ecol<uint16_t>(m, FRT_COL_N_CIGAR);
    v.name_len = ecol<uint8_t>(m, FRT_COL_NAME_LEN);
    v.aux_status = ecol<uint8_t>(m, FRT_COL_AUX_STATUS);
    DeviceGuardLite g(e->device);
    return fields_run(v, op, tag, e->device, e->stream, e->shared, nullptr, nullptr, out, err);
}

extern "C" int frt_engine_aux_lookup(const frt_engine *e, const char tag[2], frt_columns **out, frt_error *err)
{
    return engine_fields(e, FIELDS_AUX_LOOKUP, tag, out, err);
}

extern "C" int frt_engine_cigar_resolved(const frt_engine *e, frt_columns **out, frt_error *err)
{
    return engine_fields(e, FIELDS_CIGAR_RESOLVED, nullptr, out, err);
}

extern "C" int frt_engine_unpack_sequences(const frt_engine *e, frt_columns **out, frt_error *err)
{
    return engine_fields(e, FIELDS_UNPACK_SEQUENCES, nullptr, out, err);
}

extern "C" int frt_engine_compact(const frt_engine *e, frt_columns **out, frt_error *err)
{
    return engine_fields(e, FIELDS_COMPACT, nullptr, out, err);
}

extern "C" int frt_engine_inflated_to_host(const frt_engine *e, uint8_t *dst, size_t cap, frt_error *err)
{
    size_t len = 0;
    const uint8_t *p = e ? frt_engine_inflated(e, &len) : nullptr;
    if (!e || (len && (!p || !dst))) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (cap < len) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, len, cap, 0, nullptr, "destination too small");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (!len) return FRT_OK;
    DeviceGuardLite g(e->device);
    cudaError_t ce = cudaMemcpyAsync(dst, p, len, cudaMemcpyDeviceToHost, e->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->stream);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "downloading the inflated bytes");
    return FRT_OK;
}

extern "C" void *frt_engine_stream(const frt_engine *e) { return e ? (void *)e->stream : nullptr; }

int frt::engine_device(const frt_engine *e) { return e ? e->device : 0; }

// Per-stage timing of an eager run (front / inflate / records), averaged over
// `repeats` runs, with CUDA events on the engine stream.
extern "C" int frt_engine_time_stages(frt_engine *e, float *ms, int repeats, frt_error *err)
{
    DeviceGuardLite g(e->device);
    if (repeats < 1) repeats = 1;
    cudaEvent_t ev[4];
    for (auto &x : ev) cudaEventCreate(&x);
    float acc[3] = {0, 0, 0};
    cudaError_t ce = cudaSuccess;
    for (int r = 0; r < repeats && ce == cudaSuccess; ++r) {
        cudaEventRecord(ev[0], e->stream);
        enqueue_front(e);
        cudaEventRecord(ev[1], e->stream);
        enqueue_inflate(e);
        cudaEventRecord(ev[2], e->stream);
        if (e->multi) {
            int drc = decode_files(e, err);
            if (drc) {
                for (auto &x : ev) cudaEventDestroy(x);
                return drc;
            }
        } else {
            enqueue_records(e, true);
        }
        cudaEventRecord(ev[3], e->stream);
        ce = cudaStreamSynchronize(e->stream);
        for (int k = 0; k < 3 && ce == cudaSuccess; ++k) {
            float t = 0;
            cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (ce != cudaSuccess) return cuda_fail(err, ce, "timing stages");
    for (int k = 0; k < 3; ++k) ms[k] = acc[k] / repeats;
    return frt_engine_finish(e, nullptr, err);
}

// Kernels this library launches per engine run (the graph's kernel nodes).
extern "C" uint64_t frt_engine_launches(const frt_engine *e)
{
    if (!e) return 0;
    uint64_t dec = 0;
    for (auto &f : e->files) dec += decode_launches(f);
    if (!e->graph) return dec;
    size_t n = 0;
    cudaGraphGetNodes(e->graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(e->graph, nodes.data(), &n);
    uint64_t k = 0;
    for (auto &nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    return k + dec;
}
