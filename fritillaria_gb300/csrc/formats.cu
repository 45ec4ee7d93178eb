// FASTQ, BCF and FASTA on the same container: record boundaries and columns
// of a device-resident inflated batch.
//
//   FASTQ  FastqScanner::scan/decode  (crates/fritillaria-cuda/src/fastq.rs:94-140, 486-560)
//   BCF    BcfScanner::scan/decode    (crates/fritillaria-cuda/src/bcf.rs:94-150, 280-420)
//   FASTA  FastaCompactor::compact    (crates/fritillaria-cuda/src/fasta.rs:60-80, 212-300)
//
// Results are the reference launchers' results; the way there is different.
//
// FASTQ.  A newline index of the batch is built in two streaming passes (count
// per 16 KiB tile, scan, emit in order).  With every line start indexed, the
// four-line test of a record start (fastq record.rs:79-130) is O(1) per line,
// so every line start is validated in parallel and the valid ones compacted in
// order.  The reference proves a tiling of those survivors on the host and
// otherwise walks one record at a time on one thread; here both its tiling
// and its walk are checked for every adjacent pair in parallel (the walk
// differs from the tiling only by blank lines between records), and a serial
// walk over the index runs only when a decoy breaks the chain.
//
// BCF.  The reference's device result always equals its length-prefix walk
// from `start` (the tiling, when it holds, is that chain; when it does not,
// the walk runs).  Here the sieve of every byte offset runs over tiles staged
// in shared memory, survivors are validated inline and emitted in order, the
// tiling and the whole-record probe at its end are checked in parallel, and
// the serial walk runs only when they fail.
//
// FASTA.  Three streaming passes over the batch with a line-state machine
// (before any record / definition line / sequence line) carried across tiles
// by a scan of composed per-tile transfer functions; pass three writes the
// bases of sequence lines, newlines dropped, through a shared-memory staging
// buffer with coalesced stores, plus each contig's record and sequence offset.

#include <cstring>

#include "bam.cuh"
#include "common.cuh"
#include "runtime.h"

using namespace frt;

namespace {

constexpr int TB = 256;          // threads per tile
constexpr int CH = 64;           // bytes per thread
constexpr u64 TILE = TB * CH;    // bytes per tile
constexpr u32 SIEVE_TILE = 8192; // BCF positions per tile
constexpr u32 SIEVE_LIST = 1024; // survivors a BCF tile can order in shared memory

// ---- block helpers (256 threads) -------------------------------------------

template <typename T> __device__ T block_excl_sum(T v, T *s_warp, T *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(FRT_FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        T w = lane < TB / 32 ? s_warp[lane] : (T)0;
#pragma unroll
        for (int o = 1; o < TB / 32; o <<= 1) {
            T y = __shfl_up_sync(FRT_FULL_MASK, w, o);
            if (lane >= o) w += y;
        }
        if (lane < TB / 32) s_warp[lane] = w;
    }
    __syncthreads();
    T excl = x - v + (wid ? s_warp[wid - 1] : (T)0);
    if (total) *total = s_warp[TB / 32 - 1];
    __syncthreads();
    return excl;
}

// Loads bytes [p0, p0 + 64) into 16 little-endian words; bytes outside
// [lo, hi) read as 0.  Vector loads when the whole chunk is in range and
// 16-byte aligned.
__device__ __forceinline__ void load64(const u8 *buf, u64 p0, u64 lo, u64 hi, bool aligned, u32 w[16])
{
    if (aligned && p0 >= lo && p0 + 64 <= hi) {
        const uint4 *q = reinterpret_cast<const uint4 *>(buf + p0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            uint4 x = __ldg(q + k);
            w[4 * k] = x.x;
            w[4 * k + 1] = x.y;
            w[4 * k + 2] = x.z;
            w[4 * k + 3] = x.w;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        u32 v = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            u64 i = p0 + 4 * k + b;
            u32 c = (i >= lo && i < hi) ? (u32)buf[i] : 0u;
            v |= c << (8 * b);
        }
        w[k] = v;
    }
}


// 0x80 in every byte of x that is zero, 0 elsewhere (exact: no borrow runs
// between bytes, as the high bits are handled apart from the low seven).
__device__ __forceinline__ u32 zero_bytes(u32 x) { return ~(((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x | 0x7f7f7f7fu); }
// The four 0x80-or-0 bytes of z as bits 0..3 (byte order).
__device__ __forceinline__ u32 byte_bits(u32 z) { return ((z >> 7) * 0x01020408u) >> 24; }

// =============================================================================
// FASTQ
// =============================================================================

// The newline index, in one read of the bytes.  Pass 1 (k_nl_slots) counts
// each tile's newlines and, when they fit the tile's NL_SLOT slots, stores
// their offsets within the tile and the byte after each; pass 2 (k_nl_gather),
// after a scan of the counts, copies the slots to their places, and only a
// tile with more newlines than slots reads its bytes again.  Both passes take
// `buf` at a 16-byte boundary at or before the scan's start `lo`; positions
// are written as offsets from `lo`.
constexpr u32 NL_SLOT = 1024; // a tile of 16 KiB averaging 16 bytes a line or more fits

// The newlines of one 64-byte chunk in order: nl[at..] gets their offsets from
// `lo`, lf[at..] the byte after each (the first byte of the next line, 0 past
// hi).  `pos` maps a chunk byte to what is stored.
template <typename P, typename F>
__device__ __forceinline__ void chunk_newlines(const u8 *buf, u64 p0, u64 hi, const u32 w[16], u32 at, P *nl,
                                               u8 *lf, F pos)
{
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        u32 mk = zero_bytes(w[k] ^ 0x0a0a0a0au);
        while (mk) {
            const int b = (__ffs(mk) - 1) >> 3; // byte of the word
            const u32 next = b < 3 ? (w[k] >> (8 * (b + 1))) & 0xffu
                                   : (k < 15 ? w[k + 1 < 16 ? k + 1 : 15] & 0xffu
                                             : (p0 + CH < hi ? (u32)buf[p0 + CH] : 0u));
            lf[at] = (u8)next;
            nl[at++] = pos(4 * k + b);
            mk &= mk - 1;
        }
    }
}

__device__ __forceinline__ u32 chunk_count(const u32 w[16])
{
    u32 c = 0;
#pragma unroll
    for (int k = 0; k < 16; ++k) c += __popc(zero_bytes(w[k] ^ 0x0a0a0a0au));
    return c;
}

// Pass 1.  *last_nl (when given) says whether the byte before hi is a newline,
// so that the caller knows the line count with the newline count.
__global__ void __launch_bounds__(TB, 6) k_nl_slots(const u8 *buf, u64 lo, u64 hi, u64 tbase, u32 *tile_count,
                                                  u16 *slot_pos, u8 *slot_lf, u32 *last_nl)
{
    __shared__ u32 s_warp[TB / 32];
    const u32 r0 = threadIdx.x * CH; // the chunk's offset in the tile
    const u64 p0 = tbase + (u64)blockIdx.x * TILE + r0;
    u32 w[16];
    load64(buf, p0, lo, hi, true, w);
    if (last_nl && hi > lo && hi - 1 >= p0 && hi - 1 < p0 + CH) *last_nl = buf[hi - 1] == '\n' ? 1u : 0u;
    u32 tot;
    const u32 at = block_excl_sum<u32>(chunk_count(w), s_warp, &tot);
    if (threadIdx.x == 0) tile_count[blockIdx.x] = tot;
    if (tot > NL_SLOT) return; // the gather reads this tile's bytes again
    chunk_newlines(buf, p0, hi, w, at, slot_pos + (u64)blockIdx.x * NL_SLOT, slot_lf + (u64)blockIdx.x * NL_SLOT,
                   [r0](u32 j) { return (u16)(r0 + j); });
}

// Pass 2, a warp per tile: tile_base is the exclusive scan of tile_count.
__global__ void __launch_bounds__(TB, 6) k_nl_gather(const u8 *buf, u64 lo, u64 hi, u64 tbase, u64 n_tiles,
                                                   const u32 *tile_count, const u32 *tile_base,
                                                   const u16 *slot_pos, const u8 *slot_lf, u32 *nl, u8 *lf)
{
    const u64 tile = (u64)blockIdx.x * (TB / 32) + (threadIdx.x >> 5);
    const u32 lane = threadIdx.x & 31;
    if (tile >= n_tiles) return;
    const u32 n = tile_count[tile], base = tile_base[tile];
    const u64 t0 = tbase + tile * TILE;
    if (n <= NL_SLOT) {
        const u16 *sp = slot_pos + tile * NL_SLOT;
        const u8 *sl = slot_lf + tile * NL_SLOT;
        for (u32 i = lane; i < n; i += 32) {
            nl[base + i] = (u32)(t0 + sp[i] - lo); // every newline is at or past lo
            lf[base + i] = sl[i];
        }
        return;
    }
    // a tile denser than its slots: its bytes again, 32 chunks at a time
    u32 at = base;
    for (u32 r = 0; r < TILE; r += 32 * CH) {
        const u64 p0 = t0 + r + lane * CH;
        u32 w[16];
        load64(buf, p0, lo, hi, true, w);
        const u32 c = chunk_count(w);
        u32 x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(FRT_FULL_MASK, x, o);
            if (lane >= (u32)o) x += y;
        }
        chunk_newlines(buf, p0, hi, w, at + x - c, nl, lf, [p0, lo](u32 j) { return (u32)(p0 + j - lo); });
        at += __shfl_sync(FRT_FULL_MASK, x, 31);
    }
}

struct FqIndex {
    const u8 *buf;
    u64 start, len;
    const u32 *nl; // newline positions less `start` (a batch spans less than 4 GiB from start)
    u32 n_nl, n_lines;
    const u8 *lf; // lf[i]: the byte after newline i
    __device__ __forceinline__ u64 nlp(u32 i) const { return start + nl[i]; } // newline i's position
    __device__ __forceinline__ u64 ls(u32 k) const { return k == 0 ? start : nlp(k - 1) + 1; }
    // the first byte of line k (a line that starts inside the batch)
    __device__ __forceinline__ u32 first(u32 k) const { return k == 0 ? buf[start] : lf[k - 1]; }
    // end of the record whose definition is line k (valid record assumed)
    __device__ __forceinline__ u64 rec_end(u32 k) const { return k + 3 < n_nl ? nlp(k + 3) + 1 : len; }
    __device__ __forceinline__ bool blank(u32 k) const { return first(k) == '\n'; }
    // bounds_at (fastq record.rs:79-130) from the index
    __device__ __forceinline__ bool valid(u32 k) const
    {
        if (first(k) != '@' || k + 2 >= n_nl) return false;
        if (lf[k + 1] != '+') return false;
        u64 seq_len = (u64)nl[k + 1] - nl[k] - 1;
        u64 qs = nlp(k + 2) + 1, qe = k + 3 < n_nl ? nlp(k + 3) : len;
        return qe - qs == seq_len;
    }
};

// =============================================================================
// Tab-delimited text: SAM, VCF, BED, GFF, GTF (kernels/text_scan.cu, src/text.rs)
// =============================================================================
// The reference appends line starts with an atomic, sorts them on the host and
// walks each line with one thread.  Here the line starts come in order from the
// newline index (the FASTQ one), the records and header lines are compacted by
// scans, and a warp per record counts, then writes, its tab offsets in order.

// Per line: record (not blank, not a header), header line, or blank
// (text_find_lines, text_scan.cu:41-72).
__global__ void k_tx_lines(FqIndex ix, u32 comment, u32 secondary, u32 *is_rec, u32 *is_hdr)
{
    u32 k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ix.n_lines) return;
    const u64 s = ix.ls(k);
    u32 r = 0, h = 0;
    if (s < ix.len) {
        const u32 first = ix.first(k);
        if (first != '\n') {
            h = (first == comment || (secondary < 256u && first == secondary)) ? 1u : 0u;
            r = 1u - h;
        }
    }
    is_rec[k] = r;
    is_hdr[k] = h;
}

// A line ends at its newline, or at the end of the batch (text_count_fields).
__global__ void k_tx_place(FqIndex ix, const u32 *is_rec, const u32 *rec_pos, const u32 *is_hdr,
                           const u32 *hdr_pos, u64 *rec_off, u64 *rec_end, u64 *hdr_off)
{
    u32 k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ix.n_lines) return;
    const u64 s = ix.ls(k);
    if (is_rec[k]) {
        rec_off[rec_pos[k]] = s;
        rec_end[rec_pos[k]] = k < ix.n_nl ? ix.nlp(k) : ix.len;
    }
    if (is_hdr[k]) hdr_off[hdr_pos[k]] = s;
}

// A record's tabs, a warp per record.  The bytes before the record's first
// 16-byte boundary and after its last go one a lane; the aligned 16-byte
// blocks between, one a lane with vector loads, 32 blocks a step.  Only
// blocks wholly inside the record are loaded as vectors.
struct TabSplit {
    u64 a, lo, hi, b; // [a, lo) head, [lo, hi) aligned blocks, [hi, b) tail
    __device__ __forceinline__ TabSplit(const u8 *buf, u64 a_, u64 b_) : a(a_), b(b_)
    {
        const u64 base = (u64)(uintptr_t)buf;
        const u64 up = ((base + a + 15ull) & ~15ull) - base, down = ((base + b) & ~15ull) - base;
        lo = up < b ? up : b;
        hi = down > lo ? down : lo;
    }
};

// Bit i set when byte i of the block is a tab: zero_bytes marks a byte 0x80,
// and the multiply gathers the four top bits (7, 15, 23, 31) to bits 28-31
// (its partial products never overlap, so nothing carries).
__device__ __forceinline__ u32 tab_bits(uint4 v)
{
    auto f = [](u32 w) { return (zero_bytes(w ^ 0x09090909u) * 0x00204081u) >> 28; };
    return f(v.x) | (f(v.y) << 4) | (f(v.z) << 8) | (f(v.w) << 12);
}

__global__ void k_tx_count_tabs(const u8 *buf, const u64 *rec_off, const u64 *rec_end, u32 n, u32 *counts)
{
    const u32 r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (r >= n) return;
    const TabSplit sp(buf, rec_off[r], rec_end[r]);
    u32 c = 0;
    if (sp.a + lane < sp.lo) c += buf[sp.a + lane] == '\t' ? 1u : 0u;
    for (u64 q = sp.lo + 16ull * lane; q < sp.hi; q += 512) c += __popc(tab_bits(*(const uint4 *)(buf + q)));
    if (sp.hi + lane < sp.b) c += buf[sp.hi + lane] == '\t' ? 1u : 0u;
#pragma unroll
    for (int d = 16; d; d >>= 1) c += __shfl_down_sync(FRT_FULL_MASK, c, d);
    if (lane == 0) counts[r] = c;
}

// The same split, writing each tab's offset in order: the lanes' counts are
// scanned across the warp to place each lane's tabs.
__global__ void k_tx_emit_tabs(const u8 *buf, const u64 *rec_off, const u64 *rec_end, u32 n, const u32 *tab_base,
                               u64 *tabs)
{
    const u32 r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (r >= n) return;
    const TabSplit sp(buf, rec_off[r], rec_end[r]);
    u32 at = tab_base[r];
    {
        const u64 q = sp.a + lane;
        const bool t = q < sp.lo && buf[q] == '\t';
        const u32 m = __ballot_sync(FRT_FULL_MASK, t);
        if (t) tabs[at + __popc(m & lanemask_lt())] = q;
        at += __popc(m);
    }
    for (u64 q0 = sp.lo; q0 < sp.hi; q0 += 512) {
        const u64 q = q0 + 16ull * lane;
        u32 bits = q < sp.hi ? tab_bits(*(const uint4 *)(buf + q)) : 0u;
        const u32 c = __popc(bits);
        u32 incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 y = __shfl_up_sync(FRT_FULL_MASK, incl, d);
            if ((int)lane >= d) incl += y;
        }
        u32 w = at + incl - c;
        for (; bits; bits &= bits - 1u) tabs[w++] = q + (u32)(__ffs(bits) - 1);
        at += __shfl_sync(FRT_FULL_MASK, incl, 31);
    }
    {
        const u64 q = sp.hi + lane;
        const bool t = q < sp.b && buf[q] == '\t';
        const u32 m = __ballot_sync(FRT_FULL_MASK, t);
        if (t) tabs[at + __popc(m & lanemask_lt())] = q;
    }
}

__global__ void k_tx_starts(const u32 *tab_base, u32 n1, u64 *starts)
{
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n1) starts[i] = tab_base[i];
}

// The valid record starts among each block's TB lines (counted), then, after
// a scan of the counts, the same test again with each valid line written in
// order: no per-line flag array is stored and re-read.
// The validity of lines k0..k0+3 as bits 0..3.  Away from the batch's ends
// the index entries they need come in two 16-byte and two 4-byte loads.
__device__ __forceinline__ u32 valid4(const FqIndex &ix, u32 k0)
{
    u32 v = 0;
    if (k0 == 0 || (u64)k0 + 8 > ix.n_nl || (((uintptr_t)ix.nl | (uintptr_t)ix.lf) & 15)) {
#pragma unroll
        for (u32 j = 0; j < 4; ++j)
            if (k0 + j < ix.n_lines && ix.valid(k0 + j)) v |= 1u << j;
        return v;
    }
    const uint4 a = *reinterpret_cast<const uint4 *>(ix.nl + k0);
    const uint4 b = *reinterpret_cast<const uint4 *>(ix.nl + k0 + 4);
    const u32 n[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    const u32 f = *reinterpret_cast<const u32 *>(ix.lf + k0), g = *reinterpret_cast<const u32 *>(ix.lf + k0 + 4);
    // L[j + 1] = lf[k0 + j]: the first byte of line k0 + j + 1
    const u32 L[6] = {ix.lf[k0 - 1], f & 0xffu, (f >> 8) & 0xffu, (f >> 16) & 0xffu, f >> 24, g & 0xffu};
#pragma unroll
    for (u32 j = 0; j < 4; ++j) {
        // line k: '@' first, '+' first two lines on, and a quality line as long as
        // its sequence line (all four lines end inside the batch, k + 3 < n_nl)
        const bool ok = L[j] == '@' && L[j + 2] == '+' && n[j + 3] - n[j + 2] == n[j + 1] - n[j];
        v |= ok ? 1u << j : 0u;
    }
    return v;
}

// Record starts, four lines a thread: each thread's four validity bits go
// to vmask, and each block's count to block_count.
__global__ void __launch_bounds__(TB) k_fq_lines_count(FqIndex ix, u8 *vmask, u32 *block_count)
{
    __shared__ u32 s_warp[TB / 32];
    const u32 t = blockIdx.x * TB + threadIdx.x;
    const u32 v = (u64)t * 4 < ix.n_lines ? valid4(ix, t * 4) : 0u;
    if ((u64)t * 4 < ix.n_lines) vmask[t] = (u8)v;
    u32 tot;
    block_excl_sum<u32>(__popc(v), s_warp, &tot);
    if (threadIdx.x == 0) block_count[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(TB) k_fq_lines_emit(FqIndex ix, const u8 *vmask, const u32 *block_base, u32 *S)
{
    __shared__ u32 s_warp[TB / 32];
    const u32 t = blockIdx.x * TB + threadIdx.x;
    u32 v = (u64)t * 4 < ix.n_lines ? vmask[t] : 0u;
    u32 at = block_base[blockIdx.x] + block_excl_sum<u32>(__popc(v), s_warp, nullptr);
    while (v) {
        S[at++] = t * 4 + (__ffs(v) - 1);
        v &= v - 1;
    }
}

// bit 0: the survivors do not tile (fastq.rs:585-598); bit 1: they are not the
// walk's chain either (a gap between records holds something besides newlines).
__global__ void k_fq_check(FqIndex ix, const u32 *S, const u32 *n_s_dev, u32 *fails)
{
    const u32 n_s = *n_s_dev;
    u32 j = blockIdx.x * blockDim.x + threadIdx.x;
    u32 f = 0;
    if (j + 1 < n_s) {
        u32 k0 = S[j], k1 = S[j + 1];
        u64 e0 = ix.rec_end(k0), p1 = ix.ls(k1);
        if (p1 != e0) f |= 1u;
        if (k1 < k0 + 4 || e0 > p1 || p1 - e0 != (u64)(k1 - k0 - 4)) f |= 2u;
    }
    u32 any = __reduce_or_sync(FRT_FULL_MASK, f);
    if ((threadIdx.x & 31) == 0 && any) atomicOr(fails, any);
}

// totals: n, tail, proof, survivors, use_walk_list
__global__ void k_fq_finalize(FqIndex ix, const u32 *S, const u32 *n_s_dev, const u32 *fails,
                              u32 *W, u64 *totals)
{
    u32 n_s = *n_s_dev;
    u32 a = 0;
    while (a < ix.n_lines && ix.blank(a)) ++a;
    u64 anchor = a < ix.n_lines ? ix.ls(a) : ix.len;
    u64 n = 0, tail = anchor, proof = 1, use_w = 0;
    if (n_s > 0 && ix.ls(S[0]) == anchor) {
        u64 e = ix.rec_end(S[n_s - 1]);
        if (!(*fails & 1u)) {
            n = n_s;
            tail = e;
            proof = 0;
        } else if (!(*fails & 2u)) {
            n = n_s;
            if (e >= ix.len) {
                tail = ix.len;
            } else {
                u32 c = S[n_s - 1] + 4;
                while (c < ix.n_lines && ix.blank(c)) ++c;
                tail = c < ix.n_lines ? ix.ls(c) : ix.len;
            }
        } else {
            // a decoy among the survivors: the walk of fastq_scan.cu:173-215
            u32 c = a, m = 0;
            tail = ix.len;
            while (c < ix.n_lines) {
                if (!ix.valid(c)) {
                    tail = ix.ls(c);
                    break;
                }
                W[m++] = c;
                if (c + 3 >= ix.n_nl) { // unterminated last record ends the batch
                    tail = ix.len;
                    c = ix.n_lines;
                    break;
                }
                c += 4;
                while (c < ix.n_lines && ix.blank(c)) ++c;
            }
            n = m;
            use_w = 1;
        }
    }
    totals[0] = n;
    totals[1] = tail;
    totals[2] = proof;
    totals[3] = n_s;
    totals[4] = use_w;
}

__global__ void k_fq_decode(FqIndex ix, const u32 *list, u32 n, u64 *rec_off, u32 *seq_start, u32 *plus_start,
                            u32 *qual_start, u32 *seq_len, u32 *rec_end)
{
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u32 k = list[i];
    u64 p = ix.ls(k);
    u64 qe = k + 3 < ix.n_nl ? ix.nlp(k + 3) : ix.len;
    u64 e = qe < ix.len ? qe + 1 : qe;
    rec_off[i] = p;
    seq_start[i] = (u32)(ix.nlp(k) + 1 - p);
    plus_start[i] = (u32)(ix.nlp(k + 1) + 1 - p);
    qual_start[i] = (u32)(ix.nlp(k + 2) + 1 - p);
    seq_len[i] = (u32)(ix.nl[k + 1] - ix.nl[k] - 1);
    rec_end[i] = (u32)(e - p);
}

// =============================================================================
// BCF (typed values: crates/fritillaria-bcf/src/columnar/typed.rs:381-447)
// =============================================================================

__device__ __forceinline__ u32 bcf_type_size(u32 code)
{
    // 0 missing, 1 int8, 2 int16, 3 int32, 5 float, 7 char; others reserved
    switch (code) {
    case 0: return 0;
    case 1: case 7: return 1;
    case 2: return 2;
    case 3: case 5: return 4;
    default: return 0xffffffffu;
    }
}

// Descriptor at pos: header length (0 if malformed); count and kind out.
__device__ u32 bcf_descriptor(const u8 *buf, u64 lim, u64 pos, u32 *count, u32 *kind)
{
    if (pos >= lim) return 0;
    u32 d = buf[pos], code = d & 15u;
    if (bcf_type_size(code) == 0xffffffffu) return 0;
    *kind = code;
    if ((d >> 4) < 15u) {
        *count = d >> 4;
        return 1;
    }
    if (pos + 1 >= lim) return 0;
    u32 inner = buf[pos + 1], ic = inner & 15u;
    if ((inner >> 4) != 1u || (ic != 1u && ic != 2u && ic != 3u)) return 0;
    u32 wdt = bcf_type_size(ic);
    if (pos + 2 + wdt > lim) return 0;
    const u8 *p = buf + pos + 2;
    int v = ic == 1u ? (int)(signed char)p[0] : ic == 2u ? (int)(short)ld_u16le(p) : (int)ld_u32le(p);
    if (v < 15) return 0;
    *count = (u32)v;
    return 2 + wdt;
}

__device__ __forceinline__ u64 bcf_skip(const u8 *buf, u64 lim, u64 pos)
{
    u32 count = 0, kind = 0;
    u32 h = bcf_descriptor(buf, lim, pos, &count, &kind);
    if (!h) return 0;
    u64 e = pos + h + (u64)count * bcf_type_size(kind);
    return e > lim ? 0 : e;
}

// Record::validate (crates/fritillaria-bcf/src/columnar/record.rs:427-489).
__device__ bool bcf_validate(const u8 *buf, u64 len, u64 pos)
{
    if (pos + 32 > len) return false;
    u64 l_shared = ld_u32le(buf + pos), l_indiv = ld_u32le(buf + pos + 4);
    u64 indiv = pos + 8 + l_shared, end = indiv + l_indiv;
    if (l_shared < 24 || end > len) return false;
    u32 n_info = ld_u16le(buf + pos + 24), n_allele = ld_u16le(buf + pos + 26);
    u32 n_sample = ld_u16le(buf + pos + 28) | ((u32)buf[pos + 30] << 16), n_fmt = buf[pos + 31];
    u64 at = bcf_skip(buf, indiv, pos + 32);
    if (!at) return false;
    for (u32 i = 0; i < n_allele; ++i)
        if (!(at = bcf_skip(buf, indiv, at))) return false;
    if (!(at = bcf_skip(buf, indiv, at))) return false;
    for (u32 i = 0; i < n_info; ++i) {
        if (!(at = bcf_skip(buf, indiv, at))) return false;
        if (!(at = bcf_skip(buf, indiv, at))) return false;
    }
    if (at != indiv) return false;
    for (u32 i = 0; i < n_fmt; ++i) {
        if (!(at = bcf_skip(buf, end, at))) return false;
        u32 count = 0, kind = 0;
        u32 h = bcf_descriptor(buf, end, at, &count, &kind);
        if (!h) return false;
        at += h + (u64)count * bcf_type_size(kind) * n_sample;
        if (at > end) return false;
    }
    return at == end;
}

// looks_like_a_record (record.rs:149-206) over a staged copy: `s` holds the
// bytes from position `base`; `pos` is absolute.
__device__ __forceinline__ bool bcf_plausible(const u8 *s, u64 off, u64 pos, u64 len, u32 samples, u32 contigs)
{
    if (pos + 32 > len) return false;
    const u8 *p = s + off;
    u32 n_sample = (u32)p[28] | ((u32)p[29] << 8) | ((u32)p[30] << 16);
    if (n_sample != samples) return false;
    u32 l_shared = (u32)p[0] | ((u32)p[1] << 8) | ((u32)p[2] << 16) | ((u32)p[3] << 24);
    u32 l_indiv = (u32)p[4] | ((u32)p[5] << 8) | ((u32)p[6] << 16) | ((u32)p[7] << 24);
    if (l_shared < 24) return false;
    if (pos + 8 + (u64)l_shared + l_indiv > len) return false;
    int chrom = (int)((u32)p[8] | ((u32)p[9] << 8) | ((u32)p[10] << 16) | ((u32)p[11] << 24));
    int position = (int)((u32)p[12] | ((u32)p[13] << 8) | ((u32)p[14] << 16) | ((u32)p[15] << 24));
    int rlen = (int)((u32)p[16] | ((u32)p[17] << 8) | ((u32)p[18] << 16) | ((u32)p[19] << 24));
    if (chrom < 0 || (u32)chrom >= contigs || position < -1 || rlen < 0) return false;
    u32 n_allele = (u32)p[26] | ((u32)p[27] << 8), n_fmt = p[31];
    if (n_allele == 0) return false;
    if (n_fmt == 0) return l_indiv == 0;
    return (u64)l_indiv >= (u64)n_fmt * 2;
}

// mode 0: survivors per tile.  mode 1: survivors emitted in position order at
// tile_base[tile] (a tile with more than SIEVE_LIST survivors sets *overflow
// and emits nothing; the caller then takes the walk).
__global__ void __launch_bounds__(TB) k_bcf_sieve(const u8 *buf, u64 start, u64 len, u32 samples, u32 contigs,
                                                  int mode, u32 *tile_count, const u32 *tile_base, u64 *out,
                                                  u32 *overflow)
{
    __shared__ __align__(16) u8 s[SIEVE_TILE + 48];
    __shared__ u64 s_list[SIEVE_LIST];
    __shared__ u32 s_n, s_warp[TB / 32];
    const u64 base = start + (u64)blockIdx.x * SIEVE_TILE;
    for (u32 i = threadIdx.x; i < SIEVE_TILE + 32; i += TB) {
        u64 p = base + i;
        s[i] = p < len ? buf[p] : 0;
    }
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    u32 c = 0;
    for (u32 i = threadIdx.x; i < SIEVE_TILE; i += TB) {
        u64 pos = base + i;
        if (pos >= len) break;
        if (!bcf_plausible(s, i, pos, len, samples, contigs)) continue;
        if (!bcf_validate(buf, len, pos)) continue;
        if (mode == 0) {
            ++c;
        } else {
            u32 slot = atomicAdd(&s_n, 1u);
            if (slot < SIEVE_LIST) s_list[slot] = pos;
        }
    }
    if (mode == 0) {
        u32 tot;
        block_excl_sum<u32>(c, s_warp, &tot);
        if (threadIdx.x == 0) tile_count[blockIdx.x] = tot;
        return;
    }
    __syncthreads();
    u32 n = s_n;
    if (n > SIEVE_LIST) {
        // the tile cannot order its survivors: mark its slots out of range
        // so nothing reads through them, and send the batch to the walk
        if (threadIdx.x == 0) atomicOr(overflow, 1u);
        for (u32 i = tile_base[blockIdx.x] + threadIdx.x; i < tile_base[blockIdx.x + 1]; i += TB) out[i] = len;
        return;
    }
    // rank sort: survivors per tile are few (one per record at most)
    u32 at = tile_base[blockIdx.x];
    for (u32 i = threadIdx.x; i < n; i += TB) {
        u64 v = s_list[i];
        u32 r = 0;
        for (u32 j = 0; j < n; ++j) r += s_list[j] < v;
        out[at + r] = v;
    }
}

// The single-pass sieve: the tile, staged with 16-byte loads from the
// 16-byte boundary at or before the batch (`abuf`, `sh` bytes before `buf`),
// is tested at every offset, first by the 24-bit n_sample match four offsets
// at a time (two shared-memory words, two funnel shifts, the three bytes
// compared by XOR and one zero-byte test), then by bcf_plausible.  Candidates go in position order into the
// tile's slot of `lists` (SIEVE_CAP entries) and their number into
// tile_count; a tile with more than SIEVE_CAP sets *overflow and the caller
// runs the two-pass sieve instead.  The full validation of the candidates
// runs afterwards, a thread each (k_bcf_check), so that its chains of
// dependent loads (through a record's typed values, often past the staged
// tile) overlap across all records instead of holding each tile.
constexpr u32 SIEVE_CAP = 96;

__global__ void __launch_bounds__(TB) k_bcf_sieve1(const u8 *abuf, u64 sh, u64 start, u64 len, u32 samples,
                                                   u32 contigs, u32 *tile_count, u64 *lists, u32 *overflow)
{
    __shared__ __align__(16) u8 s[SIEVE_TILE + 48];
    __shared__ u64 s_list[SIEVE_CAP];
    __shared__ u32 s_n;
    const u64 lo = start + sh, hi = len + sh; // candidate positions, in abuf coordinates
    const u64 T0 = (lo & ~15ull) + (u64)blockIdx.x * SIEVE_TILE;
    for (u32 i = threadIdx.x; i < (SIEVE_TILE + 48) / 16; i += TB) {
        const u64 q = T0 + 16ull * i;
        uint4 v;
        if (q >= sh && q + 16 <= hi) {
            v = __ldg(reinterpret_cast<const uint4 *>(abuf + q));
        } else {
            u32 w[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                u32 x = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const u64 a = q + 4 * k + b;
                    x |= (a >= sh && a < hi ? (u32)abuf[a] : 0u) << (8 * b);
                }
                w[k] = x;
            }
            v = make_uint4(w[0], w[1], w[2], w[3]);
        }
        *reinterpret_cast<uint4 *>(s + 16 * i) = v;
    }
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    const u32 *s32 = reinterpret_cast<const u32 *>(s);
    const u32 b0 = (samples & 0xffu) * 0x01010101u, b1 = ((samples >> 8) & 0xffu) * 0x01010101u,
              b2 = ((samples >> 16) & 0xffu) * 0x01010101u;
    // groups of four offsets, consecutive lanes on consecutive groups (their
    // shared-memory words fall in different banks)
#pragma unroll 2
    for (u32 g = threadIdx.x; g < SIEVE_TILE / 4; g += TB) {
        const u32 q = 4u * g; // tile-relative
        const u32 w0 = s32[(q + 28) >> 2], w1 = s32[(q + 32) >> 2];
        // byte k is zero where all three n_sample bytes match at offset q + k
        u32 m = zero_bytes((w0 ^ b0) | (__funnelshift_r(w0, w1, 8) ^ b1) | (__funnelshift_r(w0, w1, 16) ^ b2));
        while (m) {
            const u32 k = (u32)(__ffs(m) - 1) >> 3;
            m &= m - 1;
            const u64 pa = T0 + q + k; // abuf coordinates
            if (pa < lo || pa >= hi) continue;
            const u64 pos = pa - sh;
            if (!bcf_plausible(s, q + k, pos, len, samples, contigs)) continue;
            const u32 slot = atomicAdd(&s_n, 1u);
            if (slot < SIEVE_CAP) s_list[slot] = pos;
        }
    }
    __syncthreads();
    const u32 n = s_n;
    if (n > SIEVE_CAP) {
        if (threadIdx.x == 0) {
            atomicOr(overflow, 1u);
            tile_count[blockIdx.x] = 0;
        }
        return;
    }
    for (u32 i = threadIdx.x; i < n; i += TB) {
        const u64 v = s_list[i];
        u32 r = 0;
        for (u32 j = 0; j < n; ++j) r += s_list[j] < v;
        lists[(u64)blockIdx.x * SIEVE_CAP + r] = v;
    }
    if (threadIdx.x == 0) tile_count[blockIdx.x] = n;
}

// Survivors of the single-pass sieve, tile lists concatenated in order.
__global__ void k_bcf_gather(const u32 *tile_count, const u32 *tile_base, const u64 *lists, u64 n_tiles, u64 *V)
{
    const u64 t = (u64)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (t >= n_tiles) return;
    const u32 c = tile_count[t], at = tile_base[t];
    for (u32 j = threadIdx.x & 31; j < c; j += 32) V[at + j] = lists[t * SIEVE_CAP + j];
}

__device__ __forceinline__ u64 bcf_end(const u8 *buf, u64 pos)
{
    return pos + 8 + (u64)ld_u32le(buf + pos) + (u64)ld_u32le(buf + pos + 4);
}

// bit 0: the survivors do not tile; bit 1 (with `validate`): a candidate
// failed the full validation, so the list is not the sieve's survivor list
// and the caller takes the two-pass sieve.
__global__ void k_bcf_check(const u8 *buf, u64 start, u64 len, const u64 *V, u32 nv, u32 *fails, bool validate)
{
    u32 j = blockIdx.x * blockDim.x + threadIdx.x;
    u32 f = 0;
    if (j < nv) {
        u64 p = V[j];
        if (p + 32 > len) f = 1; // an overflowed tile's sentinel
        else {
            if (j == 0 && p != start) f = 1;
            if (j + 1 < nv && V[j + 1] != bcf_end(buf, p)) f = 1;
            if (validate && !bcf_validate(buf, len, p)) f |= 2;
        }
    }
    u32 any = __reduce_or_sync(FRT_FULL_MASK, f);
    if ((threadIdx.x & 31) == 0 && any) atomicOr(fails, 1u);
}

// totals: n, tail, proof, sieved(validated), need_walk
__global__ void k_bcf_finalize(const u8 *buf, u64 start, u64 len, const u64 *V, const u32 *nv_dev, const u32 *fails,
                               const u32 *overflow, u64 *totals)
{
    u32 nv = *nv_dev;
    bool tiled = !(*fails & 1u) && !*overflow;
    u64 at = start;
    if (tiled && nv) at = bcf_end(buf, V[nv - 1]); // every survivor passed the range checks
    if (tiled && at + 8 <= len && bcf_end(buf, at) <= len) tiled = false; // a whole record the sieve missed
    totals[0] = tiled ? nv : 0;
    totals[1] = at;
    totals[2] = tiled ? 0 : 1;
    totals[3] = nv;
    totals[4] = tiled ? 0 : 1;
    totals[5] = *fails;
}

// The length-prefix walk of bcf_scan.cu:374-410; `out` null counts only.
__global__ void k_bcf_walk(const u8 *buf, u64 start, u64 len, u64 *out, u64 *totals)
{
    u64 pos = start, n = 0;
    for (;;) {
        if (pos + 8 > len) break;
        u64 ls = ld_u32le(buf + pos), li = ld_u32le(buf + pos + 4);
        if (ls < 24) break;
        u64 end = pos + 8 + ls + li;
        if (end > len) break;
        if (out) out[n] = pos;
        ++n;
        pos = end;
    }
    totals[0] = n;
    totals[1] = pos;
}

struct BcfCols {
    int *chrom, *pos, *rlen;
    u32 *qual;
    u16 *n_info, *n_allele;
    u32 *n_sample;
    u8 *n_fmt;
    u64 *rec_off;
    u32 *alleles, *filters, *info, *genotypes, *end;
};

// bcf_decode (bcf_scan.cu:432-510): the site core and the field offsets.
__global__ void k_bcf_decode(const u8 *buf, u64 len, const u64 *offsets, u32 n, BcfCols c, u32 *errors)
{
    u32 i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 pos = offsets[i];
    c.rec_off[i] = pos;
    if (pos + 32 > len) {
        atomicAdd(errors, 1u);
        return;
    }
    u64 ls = ld_u32le(buf + pos), li = ld_u32le(buf + pos + 4);
    u64 end = pos + 8 + ls + li;
    if (ls < 24 || end > len) {
        atomicAdd(errors, 1u);
        return;
    }
    u32 n_allele = ld_u16le(buf + pos + 26);
    c.chrom[i] = (int)ld_u32le(buf + pos + 8);
    c.pos[i] = (int)ld_u32le(buf + pos + 12);
    c.rlen[i] = (int)ld_u32le(buf + pos + 16);
    c.qual[i] = ld_u32le(buf + pos + 20);
    c.n_info[i] = (u16)ld_u16le(buf + pos + 24);
    c.n_allele[i] = (u16)n_allele;
    c.n_sample[i] = ld_u16le(buf + pos + 28) | ((u32)buf[pos + 30] << 16);
    c.n_fmt[i] = buf[pos + 31];
    c.genotypes[i] = (u32)(8 + ls);
    c.end[i] = (u32)(end - pos);
    u64 w = bcf_skip(buf, end, pos + 32);
    if (!w) {
        atomicAdd(errors, 1u);
        return;
    }
    c.alleles[i] = (u32)(w - pos);
    for (u32 a = 0; a < n_allele; ++a) {
        w = bcf_skip(buf, end, w);
        if (!w) {
            atomicAdd(errors, 1u);
            return;
        }
    }
    c.filters[i] = (u32)(w - pos);
    w = bcf_skip(buf, end, w);
    if (!w) {
        atomicAdd(errors, 1u);
        return;
    }
    c.info[i] = (u32)(w - pos);
}

// =============================================================================
// FASTA
// =============================================================================
//
// Line states: 0 before any record, 1 definition line, 2 sequence line.  A
// line start beginning with '>' enters 1; any other line start enters 2
// unless no record has begun.  Over a span of bytes the effect on the state is
// one of four functions: identity (no line start), OTHER (only non-'>' line
// starts: 0 stays 0, else 2), or a constant 1 or 2 (the last '>' line start
// and what follows it decide).

enum : u32 { F_ID = 0, F_OTHER = 1, F_HDR = 2, F_SEQ = 3 };

__device__ __forceinline__ u32 f_apply(u32 f, u32 s)
{
    return f == F_ID ? s : f == F_OTHER ? (s == 0 ? 0u : 2u) : f == F_HDR ? 1u : 2u;
}
// the function "f, then g"
__device__ __forceinline__ u32 f_then(u32 f, u32 g)
{
    if (g == F_HDR || g == F_SEQ) return g;
    if (g == F_ID) return f;
    return f == F_HDR || f == F_SEQ ? F_SEQ : F_OTHER;
}

// Exclusive scan of transfer functions across the block (composition).
__device__ u32 block_excl_compose(u32 f, u32 *s_warp)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    u32 x = f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        u32 y = __shfl_up_sync(FRT_FULL_MASK, x, o);
        if (lane >= o) x = f_then(y, x);
    }
    u32 ex = __shfl_up_sync(FRT_FULL_MASK, x, 1);
    if (lane == 0) ex = F_ID;
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        u32 wv = lane < TB / 32 ? s_warp[lane] : F_ID;
#pragma unroll
        for (int o = 1; o < TB / 32; o <<= 1) {
            u32 y = __shfl_up_sync(FRT_FULL_MASK, wv, o);
            if (lane >= o) wv = f_then(y, wv);
        }
        if (lane < TB / 32) s_warp[lane] = wv;
    }
    __syncthreads();
    u32 pre = wid ? s_warp[wid - 1] : F_ID;
    u32 r = f_then(pre, ex);
    __syncthreads();
    return r;
}

// A chunk of CH = 64 bytes as bit masks.  Its bytes come from aligned 16-byte
// loads of `abuf`, the 16-byte boundary at or before the batch; the batch is
// [lo, hi) of abuf.  nl and gt mark '\n' and '>', ls the line starts (the
// batch start and every byte after a newline), hs/os the line starts that
// open a definition line or another line.  Each byte's line is found by a
// log-step fill: after it, O marks the bytes whose nearest line start at or
// before them opens another (not a definition) line, and K the bytes with a
// line start at or before them in the chunk.
struct FaMasks {
    u64 valid, nl, ls, hs, O, K;
};


__device__ __forceinline__ void fa_masks(const u8 *abuf, u64 lo, u64 hi, u64 p0, FaMasks &f, u32 w[16])
{
    load64(abuf, p0, lo, hi, true, w);
    u64 nl = 0, gt = 0;
    u32 odd = 0; // bit 6 of a byte: clear in '\n' and '>', set in every letter
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const u32 z = zero_bytes(w[k] ^ 0x0a0a0a0au);
        nl |= (u64)byte_bits(z) << (4 * k);
        odd |= (~w[k] & 0x40404040u) ^ (z >> 1); // bit 6 clear, not a newline
    }
    if (odd) { // '>' is rare: its mask is built only where a byte might be one
#pragma unroll
        for (int k = 0; k < 16; ++k) gt |= (u64)byte_bits(zero_bytes(w[k] ^ 0x3e3e3e3eu)) << (4 * k);
    }
    u64 valid = ~0ull;
    if (p0 < lo) valid &= lo - p0 >= 64 ? 0ull : ~0ull << (lo - p0);
    if (p0 + 64 > hi) valid &= hi <= p0 ? 0ull : (~0ull >> (64 - (hi - p0)));
    nl &= valid;
    gt &= valid;
    const bool prev_nl = p0 > lo && abuf[p0 - 1] == '\n';
    const u64 first = lo >= p0 && lo < p0 + 64 ? 1ull << (lo - p0) : 0ull;
    const u64 ls = ((nl << 1) | (prev_nl ? 1ull : 0ull) | first) & valid;
    const u64 hs = ls & gt, os = ls & ~gt;
    u64 O = os, K = ls;
#pragma unroll
    for (int sft = 1; sft < 64; sft <<= 1) {
        O |= (O << sft) & ~K;
        K |= K << sft;
    }
    f.valid = valid;
    f.nl = nl;
    f.ls = ls;
    f.hs = hs;
    f.O = O;
    f.K = K;
}

// The chunk's transfer function: identity with no line start, else decided
// by its last line start (a definition line: constant 1; another line after
// a definition line in the chunk: constant 2; else OTHER).
__device__ __forceinline__ u32 fa_func(const FaMasks &f)
{
    if (!f.ls) return F_ID;
    const int last = 63 - __clzll((long long)f.ls);
    if ((f.hs >> last) & 1ull) return F_HDR;
    return f.hs ? F_SEQ : F_OTHER;
}

// The bytes the chunk keeps when it is entered in state s: bytes of sequence
// lines that are not newlines.  A byte before the chunk's first line start is
// in state s; a byte of a definition line is not kept; a byte of another line
// is kept when a definition line came before it in the chunk or s is not 0.
__device__ __forceinline__ u64 fa_keep(const FaMasks &f, u32 s)
{
    const int fh = f.hs ? __ffsll((long long)f.hs) - 1 : 64;
    const u64 below = fh >= 64 ? ~0ull : (1ull << fh) - 1ull;
    const u64 text = f.valid & ~f.nl;
    const u64 pre = ~f.K & text, other = f.O & text;
    return (s == 2u ? pre : 0ull) | (s != 0u ? (other & below) : 0ull) | (other & ~below);
}

// Pass 1, per tile of TILE bytes (abuf coordinates from 0): the transfer
// function, the record starts, and the bytes kept when the tile is entered in
// each state (3 per tile); the position after the last record start goes to
// *last_contig (batch coordinates, for the unterminated-header check).
__global__ void __launch_bounds__(TB, 8) k_fa_sum(const u8 *abuf, u64 sh, u64 len, u8 *tile_f, u32 *tile_contigs,
                                               u32 *tile_kept3, unsigned long long *last_contig)
{
    __shared__ u32 s_warp[TB / 32];
    __shared__ u64 s_w64[TB / 32];
    const u64 lo = sh, hi = len + sh;
    const u64 p0 = (u64)blockIdx.x * TILE + (u64)threadIdx.x * CH;
    FaMasks m;
    u32 w[16];
    fa_masks(abuf, lo, hi, p0, m, w);
    const u32 f = fa_func(m), k = (u32)__popcll(m.hs);
    if (m.hs) atomicMax(last_contig, (unsigned long long)(p0 + 63 - __clzll((long long)m.hs) - sh + 1));
    u32 kept[3];
#pragma unroll
    for (u32 st = 0; st < 3; ++st) kept[st] = (u32)__popcll(fa_keep(m, st));
    const u32 ex = block_excl_compose(f, s_warp);
    // one sum of four 16-bit fields: the record starts (a tile holds at most
    // 8,193: each but the first follows a newline) and the bytes kept (at
    // most 16,384) for each state the tile can be entered in
    const u64 packed = (u64)k | (u64)kept[f_apply(ex, 0)] << 16 | (u64)kept[f_apply(ex, 1)] << 32 |
                       (u64)kept[f_apply(ex, 2)] << 48;
    u64 tot;
    block_excl_sum<u64>(packed, s_w64, &tot);
    if (threadIdx.x == TB - 1) tile_f[blockIdx.x] = (u8)f_then(ex, f);
    if (threadIdx.x == 0) {
        tile_contigs[blockIdx.x] = (u32)(tot & 0xffffu);
#pragma unroll
        for (u32 st = 0; st < 3; ++st) tile_kept3[3 * blockIdx.x + st] = (u32)(tot >> (16 * (st + 1))) & 0xffffu;
    }
}

// The tiles' layout, in three parallel steps over chunks of 1,024 tiles (a
// chunk a block): each chunk's composed function, record count and kept
// bytes for each entering state; one block scans the chunks from state 0 at
// the batch start; each chunk then gives its tiles their entry state, first
// contig and output offset.

// Exclusive scan across a block of 1,024 threads under an associative `op`
// (earlier element on the left); *total gets the whole block's result.
template <class T, class Op> __device__ __forceinline__ T excl_scan1024(T x, T id, Op op, T *s_w, T *total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(FRT_FULL_MASK, inc, o);
        if (lane >= o) inc = op(y, inc);
    }
    if (lane == 31) s_w[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T wv = s_w[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(FRT_FULL_MASK, wv, o);
            if (lane >= o) wv = op(y, wv);
        }
        s_w[lane] = wv;
    }
    __syncthreads();
    T ex = __shfl_up_sync(FRT_FULL_MASK, inc, 1);
    if (lane == 0) ex = id;
    const T r = wid ? op(s_w[wid - 1], ex) : ex;
    if (total) *total = s_w[31];
    __syncthreads();
    return r;
}

struct FaCompose {
    __device__ __forceinline__ u32 operator()(u32 f, u32 g) const { return f_then(f, g); }
};
struct AddU64 {
    __device__ __forceinline__ u64 operator()(u64 a, u64 b) const { return a + b; }
};

__global__ void __launch_bounds__(1024) k_fa_chunks(const u8 *tile_f, const u32 *tile_contigs, const u32 *tile_kept3,
                                                    u32 n_tiles, u8 *chunk_f, u32 *chunk_contigs, u64 *chunk_kept3)
{
    __shared__ u32 s_f[32];
    __shared__ u64 s_k[32];
    const u32 t = blockIdx.x * 1024 + threadIdx.x;
    const bool in = t < n_tiles;
    const u32 f = in ? tile_f[t] : F_ID;
    u32 all_f;
    const u32 ex = excl_scan1024<u32>(f, F_ID, FaCompose(), s_f, &all_f);
    u64 c_all;
    excl_scan1024<u64>(in ? tile_contigs[t] : 0u, 0ull, AddU64(), s_k, &c_all);
    u64 k_all[3];
#pragma unroll
    for (u32 st = 0; st < 3; ++st)
        excl_scan1024<u64>(in ? tile_kept3[3 * t + f_apply(ex, st)] : 0u, 0ull, AddU64(), s_k, &k_all[st]);
    if (threadIdx.x == 0) {
        chunk_f[blockIdx.x] = (u8)all_f;
        chunk_contigs[blockIdx.x] = (u32)c_all;
        for (u32 st = 0; st < 3; ++st) chunk_kept3[3 * blockIdx.x + st] = k_all[st];
    }
}

// One block over the chunks: entry state, first contig and output offset of
// each chunk; totals = contigs, bases, whether the last record was dropped.  A
// record whose definition line is not terminated is not a record
// (fasta record.rs:101-110): the last record start (*last_contig - 1) is
// checked for a newline after it.
__global__ void __launch_bounds__(1024) k_fa_top(const u8 *buf, u64 len, const u8 *chunk_f, const u32 *chunk_contigs,
                                                 const u64 *chunk_kept3, u32 n_chunks, u8 *chunk_state,
                                                 u64 *chunk_contig_base, u64 *chunk_out_base,
                                                 const unsigned long long *last_contig, u64 *totals)
{
    __shared__ u32 s_f[32];
    __shared__ u64 s_k[32];
    u32 carry_f = F_ID;
    u64 carry_c = 0, carry_o = 0;
    for (u32 b0 = 0; b0 < n_chunks; b0 += 1024) {
        const u32 c = b0 + threadIdx.x;
        const bool in = c < n_chunks;
        u32 all_f;
        const u32 ex = excl_scan1024<u32>(in ? chunk_f[c] : F_ID, F_ID, FaCompose(), s_f, &all_f);
        const u32 state = f_apply(f_then(carry_f, ex), 0u);
        u64 all_c, all_o;
        const u64 cb = excl_scan1024<u64>(in ? chunk_contigs[c] : 0u, 0ull, AddU64(), s_k, &all_c);
        const u64 ob = excl_scan1024<u64>(in ? chunk_kept3[3 * c + state] : 0ull, 0ull, AddU64(), s_k, &all_o);
        if (in) {
            chunk_state[c] = (u8)state;
            chunk_contig_base[c] = carry_c + cb;
            chunk_out_base[c] = carry_o + ob;
        }
        carry_f = f_then(carry_f, all_f);
        carry_c += all_c;
        carry_o += all_o;
    }
    if (threadIdx.x == 0) {
        u64 drop = 0;
        if (carry_c && *last_contig) {
            u64 p = *last_contig - 1;
            while (p < len && buf[p] != '\n') ++p;
            drop = p >= len;
        }
        totals[0] = carry_c - drop;
        totals[1] = carry_o;
        totals[2] = drop;
    }
}

__global__ void __launch_bounds__(1024) k_fa_apply(const u8 *tile_f, const u32 *tile_contigs, const u32 *tile_kept3,
                                                   u32 n_tiles, const u8 *chunk_state, const u64 *chunk_contig_base,
                                                   const u64 *chunk_out_base, u8 *tile_state, u32 *contig_base,
                                                   u64 *out_base)
{
    __shared__ u32 s_f[32];
    __shared__ u64 s_k[32];
    const u32 t = blockIdx.x * 1024 + threadIdx.x;
    const bool in = t < n_tiles;
    const u32 ex = excl_scan1024<u32>(in ? tile_f[t] : F_ID, F_ID, FaCompose(), s_f, nullptr);
    const u32 state = f_apply(ex, chunk_state[blockIdx.x]);
    const u64 cb = excl_scan1024<u64>(in ? tile_contigs[t] : 0u, 0ull, AddU64(), s_k, nullptr);
    const u64 ob = excl_scan1024<u64>(in ? tile_kept3[3 * t + state] : 0u, 0ull, AddU64(), s_k, nullptr);
    if (in) {
        tile_state[t] = (u8)state;
        contig_base[t] = (u32)(chunk_contig_base[blockIdx.x] + cb);
        out_base[t] = chunk_out_base[blockIdx.x] + ob;
    }
}

// Pass 2: each tile's kept bytes, compacted in order through a shared-memory
// staging buffer and written with coalesced stores, and each record's offset
// and the offset of its first base.
__global__ void __launch_bounds__(TB, 6) k_fa_emit(const u8 *abuf, u64 sh, u64 len, const u8 *tile_state,
                                                const u32 *contig_base, const u64 *out_base, u64 n_contigs, u8 *seq,
                                                u64 *seq_off, u64 *rec_off)
{
    __shared__ u32 s_warp[TB / 32];
    __shared__ u64 s_w64[TB / 32];
    __shared__ __align__(16) u8 s_out[TILE + 16];
    const u64 lo = sh, hi = len + sh;
    const u64 p0 = (u64)blockIdx.x * TILE + (u64)threadIdx.x * CH;
    FaMasks m;
    u32 w[16];
    fa_masks(abuf, lo, hi, p0, m, w);
    const u32 f = fa_func(m);
    const u32 ex = block_excl_compose(f, s_warp);
    const u32 st = f_apply(ex, tile_state[blockIdx.x]);
    const u64 keep = fa_keep(m, st);
    // bytes kept (low half) and record starts (high half) in one scan
    u64 tot2;
    const u64 ex2 = block_excl_sum<u64>((u64)__popcll(keep) | (u64)__popcll(m.hs) << 32, s_w64, &tot2);
    const u32 at = (u32)ex2, tile_total = (u32)tot2;
    u32 ci = contig_base[blockIdx.x] + (u32)(ex2 >> 32);
    const u64 obase = out_base[blockIdx.x];
    // record starts (a few per tile at most)
    for (u64 h = m.hs; h; h &= h - 1) {
        const int i = __ffsll((long long)h) - 1;
        if (ci < n_contigs) {
            rec_off[ci] = p0 + (u64)i - sh;
            seq_off[ci] = obase + at + (u32)__popcll(keep & ((1ull << i) - 1ull));
        }
        ++ci;
    }
    u32 o = at;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const u32 kb = (u32)(keep >> (4 * k)) & 15u, wk = w[k];
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if ((kb >> b) & 1u) s_out[o++] = (u8)(wk >> (8 * b));
    }
    __syncthreads();
    // the bytes before the output's first 4-byte boundary, then whole words
    // put together from shared memory with funnel shifts, then the rest
    const u32 h = min((u32)((4u - (u32)(obase & 3u)) & 3u), tile_total);
    if (threadIdx.x < h) seq[obase + threadIdx.x] = s_out[threadIdx.x];
    const u32 nw = (tile_total - h) >> 2;
    u32 *dst = reinterpret_cast<u32 *>(seq + obase + h);
    const u32 *s32 = reinterpret_cast<const u32 *>(s_out);
    for (u32 j = threadIdx.x; j < nw; j += TB) {
        const u32 off = h + 4u * j;
        dst[j] = __funnelshift_r(s32[off >> 2], s32[(off >> 2) + 1], 8u * (off & 3u));
    }
    for (u32 i = h + 4u * nw + threadIdx.x; i < tile_total; i += TB) seq[obase + i] = s_out[i];
}

__global__ void k_fa_lengths(const u64 *seq_off, u64 n, u64 total, u64 *seq_len)
{
    u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) seq_len[i] = (i + 1 < n ? seq_off[i + 1] : total) - seq_off[i];
}

unsigned grid_for(u64 n, unsigned block) { return (unsigned)((n + block - 1) / block); }

} // namespace

// =============================================================================
// host side
// =============================================================================

namespace {

enum { FMT_FASTQ = 1, FMT_BCF = 2, FMT_FASTA = 3, FMT_TEXT = 4 };
const size_t kTextWidths[FRT_TEXT_COL_COUNT] = {8, 8, 8, 8, 8};

const size_t kFastqWidths[FRT_FASTQ_COL_COUNT] = {8, 4, 4, 4, 4, 4};
const size_t kBcfWidths[FRT_BCF_COL_COUNT] = {4, 4, 4, 4, 2, 2, 4, 1, 8, 4, 4, 4, 4, 4};
const size_t kFastaWidths[FRT_FASTA_COL_COUNT] = {1, 8, 8, 8};

struct Scanner {
    int device = 0;
    cudaStream_t stream = nullptr;
    SharedStream *shared = nullptr;
    std::mutex mu;
    // The newline index's tile slots (3 bytes per NL_SLOT per tile), kept
    // from call to call and grown to the largest batch seen: calls on the
    // scanner's stream run in order, so one array serves them all.
    void *slots = nullptr;
    size_t slots_bytes = 0;
};

int scanner_slots(Scanner &s, u64 n_tiles, u16 **pos, u8 **lf, frt_error *err)
{
    const size_t need = (size_t)n_tiles * NL_SLOT * 3 + 16;
    if (need > s.slots_bytes) {
        dev_free(s.slots, s.stream);
        s.slots = nullptr;
        s.slots_bytes = 0;
        int rc = dev_alloc(&s.slots, need, s.stream, err);
        if (rc) return rc;
        s.slots_bytes = need;
    }
    *pos = (u16 *)s.slots;
    *lf = (u8 *)s.slots + (size_t)n_tiles * NL_SLOT * 2;
    return FRT_OK;
}

void scanner_release(Scanner &s)
{
    if (s.slots) {
        DeviceGuardLite g(s.device);
        dev_free(s.slots, s.stream);
    }
    stream_release(s.shared);
}

int scanner_create(int device, void *stream, Scanner *s, frt_error *err)
{
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuardLite g(device);
    configure_pool(device);
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    s->device = device;
    s->shared = ss;
    s->stream = ss->s;
    return FRT_OK;
}

} // namespace

struct frt_fastq_scanner {
    Scanner s;
};
struct frt_bcf_scanner {
    Scanner s;
};
struct frt_fasta_compactor {
    Scanner s;
};
struct frt_text_scanner {
    Scanner s;
};


namespace {

// Work buffers of one call, freed on every return path.
struct Work {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Work(cudaStream_t s) : st(s) {}
    ~Work()
    {
        for (void *p : ptrs) dev_free(p, st);
    }
    template <typename T> int get(T **p, size_t count, frt_error *err)
    {
        void *q = nullptr;
        int rc = dev_alloc(&q, count * sizeof(T) + 16, st, err);
        if (rc) return rc;
        ptrs.push_back(q);
        *p = (T *)q;
        return FRT_OK;
    }
};

frt_columns *columns_new(const Scanner &s, int format, const size_t *widths, int n_cols, uint64_t n)
{
    frt_columns *c = new frt_columns;
    c->device = s.device;
    c->format = format;
    c->stream = s.stream;
    c->shared = stream_retain(s.shared);
    c->widths = widths;
    c->n_cols = n_cols;
    c->n = n;
    size_t off = 0;
    for (int k = 0; k < n_cols; ++k) {
        c->col_off[k] = off;
        c->col_bytes[k] = widths[k] * n;
        off += (c->col_bytes[k] + 255) & ~(size_t)255;
    }
    return c;
}

// The extent of the column layout: the end of its last column, from the
// offsets laid out by columns_new (a column whose bytes are set to 0 after,
// as FASTA's bases in their own allocation, keeps its place in the layout).
size_t columns_bytes(const frt_columns *c)
{
    size_t t = 0;
    for (int k = 0; k < c->n_cols; ++k) {
        const size_t end = c->col_off[k] + ((c->col_bytes[k] + 255) & ~(size_t)255);
        if (end > t) t = end;
    }
    return t;
}

void columns_discard(frt_columns *c)
{
    if (!c) return;
    dev_free(c->cols, c->stream);
    dev_free(c->seq, c->stream);
    stream_release(c->shared);
    delete c;
}

int columns_finish(frt_columns *c, const frt_inflate_batch *src, frt_columns **out)
{
    if (src) {
        const_cast<frt_inflate_batch *>(src)->refs.fetch_add(1);
        c->source = src;
    }
    cudaEventCreateWithFlags(&c->ready, cudaEventDisableTiming);
    cudaEventRecord(c->ready, c->stream);
    *out = c;
    return FRT_OK;
}

int columns_alloc(frt_columns *c, frt_error *err)
{
    return dev_alloc((void **)&c->cols, columns_bytes(c) + 256, c->stream, err);
}

template <typename T> T *colp(frt_columns *c, int k) { return (T *)(c->cols + c->col_off[k]); }

int check_batch(const Scanner &s, const frt_inflate_batch *b, frt_error *err)
{
    if (b->device != s.device) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr, "batch is on device %d but this scanner is on %d",
                  b->device, s.device);
        return FRT_ERR_INVALID_DEVICE_BATCH;
    }
    cudaError_t e = cudaStreamWaitEvent(s.stream, b->ready, 0);
    if (e != cudaSuccess) return cuda_fail(err, e, "ordering after the inflate");
    return FRT_OK;
}

int read_back(cudaStream_t st, const void *src, void *dst, size_t bytes, frt_error *err, const char *what)
{
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(err, e, what);
    return FRT_OK;
}

#define LAUNCH_OK(what)                                                                                                \
    do {                                                                                                               \
        cudaError_t le_ = cudaGetLastError();                                                                          \
        if (le_ != cudaSuccess) return cuda_fail(err, le_, what);                                                      \
    } while (0)

} // namespace

// ---- FASTQ -------------------------------------------------------------------

extern "C" int frt_fastq_scanner_create(int device, void *stream, frt_fastq_scanner **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    frt_fastq_scanner *s = new frt_fastq_scanner;
    int rc = scanner_create(device, stream, &s->s, err);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return FRT_OK;
}

extern "C" void frt_fastq_scanner_destroy(frt_fastq_scanner *s)
{
    if (!s) return;
    scanner_release(s->s);
    delete s;
}

extern "C" int frt_fastq_decode(frt_fastq_scanner *sc, const frt_inflate_batch *b, uint64_t start, frt_columns **out,
                                frt_error *err)
{
    if (!sc || !out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = sc->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    uint64_t len = b && b->data ? b->len : 0;
    if (start >= len) { // empty(start.min(len)), fastq.rs:487-492
        frt_columns *c = columns_new(s, FMT_FASTQ, kFastqWidths, FRT_FASTQ_COL_COUNT, 0);
        c->tail = start < len ? start : len;
        int rc = columns_alloc(c, err);
        if (rc) {
            columns_discard(c);
            return rc;
        }
        return columns_finish(c, b, out);
    }
    int rc = check_batch(s, b, err);
    if (rc) return rc;
    if (len - start >= 0xffffffffull) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "FASTQ batch of %llu bytes exceeds 4 GiB",
                  (unsigned long long)(len - start));
        return FRT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st = s.stream;
    Work w(st);
    // The newline index reads aligned 16-byte blocks, so it works from the
    // 16-byte boundary at or before the batch (the sh bytes before the batch
    // are never read) and writes batch positions.
    const u64 sh = (uintptr_t)b->data & 15u;
    const u8 *abuf = b->data - sh;
    const u64 tbase = (start + sh) & ~15ull;
    const u64 n_tiles = (len + sh - tbase + TILE - 1) / TILE;
    u32 *tile_count, *tile_base, *partials, *d_u32;
    u16 *slot_pos;
    u8 *slot_lf;
    u64 *totals;
    if ((rc = w.get(&tile_count, n_tiles, err)) || (rc = w.get(&tile_base, n_tiles + 1, err)) ||
        (rc = w.get(&partials, frt_scan_partials_len(n_tiles) + frt_scan_partials_len(len) + 8, err)) ||
        (rc = w.get(&d_u32, 8, err)) || (rc = w.get(&totals, 8, err)) ||
        (rc = scanner_slots(s, n_tiles, &slot_pos, &slot_lf, err)))
        return rc;
    k_nl_slots<<<(unsigned)n_tiles, TB, 0, st>>>(abuf, start + sh, len + sh, tbase, tile_count, slot_pos, slot_lf,
                                                 d_u32 + 7);
    LAUNCH_OK("launching the newline count");
    cudaError_t e = frt_launch_scan_u32(tile_count, n_tiles, partials, tile_base, d_u32, st);
    if (e != cudaSuccess) return cuda_fail(err, e, "scanning newline counts");
    uint32_t hd[8] = {};
    if ((rc = read_back(st, d_u32, hd, sizeof hd, err, "newline count"))) return rc;
    const uint32_t n_nl = hd[0];
    u32 *nl;
    u8 *lf;
    if ((rc = w.get(&nl, (size_t)n_nl + 1, err)) || (rc = w.get(&lf, (size_t)n_nl + 1, err))) return rc;
    k_nl_gather<<<(unsigned)((n_tiles + TB / 32 - 1) / (TB / 32)), TB, 0, st>>>(
        abuf, start + sh, len + sh, tbase, n_tiles, tile_count, tile_base, slot_pos, slot_lf, nl, lf);
    LAUNCH_OK("launching the newline index");
    // line starts: start, and one past every newline that is not the last byte
    const uint32_t n_lines = n_nl && hd[7] ? n_nl : n_nl + 1;
    FqIndex ix{b->data, start, len, nl, n_nl, n_lines, lf};
    const u64 n_quads = ((u64)n_lines + 3) / 4; // the validation takes four lines a thread
    const u32 n_blocks = grid_for(n_quads, TB);
    u32 *bcount, *bbase, *S, *W, *fails;
    u8 *vmask;
    if ((rc = w.get(&bcount, n_blocks, err)) || (rc = w.get(&bbase, (size_t)n_blocks + 1, err)) ||
        (rc = w.get(&fails, 4, err)) || (rc = w.get(&vmask, n_quads, err)))
        return rc;
    cudaMemsetAsync(fails, 0, 16, st);
    k_fq_lines_count<<<n_blocks, TB, 0, st>>>(ix, vmask, bcount);
    LAUNCH_OK("launching the line validation");
    if ((e = frt_launch_scan_u32(bcount, n_blocks, partials, bbase, d_u32, st)) != cudaSuccess)
        return cuda_fail(err, e, "scanning record starts");
    // the record starts are at most the lines: no read-back to size them
    if ((rc = w.get(&S, (size_t)n_lines + 1, err)) || (rc = w.get(&W, (size_t)n_lines + 1, err))) return rc;
    k_fq_lines_emit<<<n_blocks, TB, 0, st>>>(ix, vmask, bbase, S);
    k_fq_check<<<grid_for(n_lines + 1, 256), 256, 0, st>>>(ix, S, d_u32, fails);
    k_fq_finalize<<<1, 1, 0, st>>>(ix, S, d_u32, fails, W, totals);
    LAUNCH_OK("launching the tiling checks");
    uint64_t tot[5];
    if ((rc = read_back(st, totals, tot, sizeof tot, err, "FASTQ scan"))) return rc;
    frt_columns *c = columns_new(s, FMT_FASTQ, kFastqWidths, FRT_FASTQ_COL_COUNT, tot[0]);
    c->tail = tot[1];
    c->info[0] = tot[2];
    c->info[1] = tot[3];
    c->info[2] = tot[3];
    if ((rc = columns_alloc(c, err))) {
        columns_discard(c);
        return rc;
    }
    if (c->n) {
        k_fq_decode<<<grid_for(c->n, 256), 256, 0, st>>>(
            ix, tot[4] ? W : S, (u32)c->n, colp<u64>(c, FRT_FASTQ_COL_RECORD_OFFSETS),
            colp<u32>(c, FRT_FASTQ_COL_SEQUENCE_START), colp<u32>(c, FRT_FASTQ_COL_PLUS_START),
            colp<u32>(c, FRT_FASTQ_COL_QUALITY_START), colp<u32>(c, FRT_FASTQ_COL_SEQUENCE_LEN),
            colp<u32>(c, FRT_FASTQ_COL_RECORD_END));
        if ((e = cudaGetLastError()) != cudaSuccess) {
            columns_discard(c);
            return cuda_fail(err, e, "launching the FASTQ decode");
        }
    }
    return columns_finish(c, b, out);
}

// ---- BCF ---------------------------------------------------------------------

extern "C" int frt_bcf_scanner_create(int device, void *stream, frt_bcf_scanner **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    frt_bcf_scanner *s = new frt_bcf_scanner;
    int rc = scanner_create(device, stream, &s->s, err);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return FRT_OK;
}

extern "C" void frt_bcf_scanner_destroy(frt_bcf_scanner *s)
{
    if (!s) return;
    scanner_release(s->s);
    delete s;
}

extern "C" int frt_bcf_decode(frt_bcf_scanner *sc, const frt_inflate_batch *b, uint64_t start, uint32_t samples,
                              uint32_t contigs, frt_columns **out, frt_error *err)
{
    if (!sc || !out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = sc->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    uint64_t len = b && b->data ? b->len : 0;
    if (start >= len) { // empty(start.min(len)), bcf.rs:284-290
        frt_columns *c = columns_new(s, FMT_BCF, kBcfWidths, FRT_BCF_COL_COUNT, 0);
        c->tail = start < len ? start : len;
        int rc = columns_alloc(c, err);
        if (rc) {
            columns_discard(c);
            return rc;
        }
        return columns_finish(c, b, out);
    }
    int rc = check_batch(s, b, err);
    if (rc) return rc;
    if (len - start >= 0xffffffffull) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "BCF batch of %llu bytes exceeds 4 GiB",
                  (unsigned long long)(len - start));
        return FRT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st = s.stream;
    Work w(st);
    const u64 n_tiles = (len - start + SIEVE_TILE - 1) / SIEVE_TILE;
    u32 *tile_count, *tile_base, *partials, *d_u32;
    u64 *totals;
    if ((rc = w.get(&tile_count, n_tiles, err)) || (rc = w.get(&tile_base, n_tiles + 1, err)) ||
        (rc = w.get(&partials, frt_scan_partials_len(n_tiles) + 8, err)) || (rc = w.get(&d_u32, 8, err)) ||
        (rc = w.get(&totals, 8, err)))
        return rc;
    cudaMemsetAsync(d_u32, 0, 32, st);
    // One pass: per-tile survivor lists, their counts scanned, then gathered.
    // A tile with more survivors than its list holds sends the batch to the
    // two-pass sieve (count, scan, emit).
    const u64 sh = (uintptr_t)b->data & 15u;
    const u64 n_tiles1 = (((len + sh) - ((start + sh) & ~15ull)) + SIEVE_TILE - 1) / SIEVE_TILE;
    u32 *count1, *base1;
    u64 *lists;
    if ((rc = w.get(&count1, n_tiles1, err)) || (rc = w.get(&base1, n_tiles1 + 1, err)) ||
        (rc = w.get(&lists, n_tiles1 * SIEVE_CAP, err)))
        return rc;
    if ((rc = w.get(&partials, frt_scan_partials_len(n_tiles1) + 8, err))) return rc;
    k_bcf_sieve1<<<(unsigned)n_tiles1, TB, 0, st>>>(b->data - sh, sh, start, len, samples, contigs, count1, lists,
                                                    d_u32 + 5);
    LAUNCH_OK("launching the BCF sieve");
    cudaError_t e = frt_launch_scan_u32(count1, n_tiles1, partials, base1, d_u32, st);
    if (e != cudaSuccess) return cuda_fail(err, e, "scanning survivors");
    uint32_t head[6] = {};
    if ((rc = read_back(st, d_u32, head, sizeof head, err, "survivor count"))) return rc;
    uint32_t nv = head[0];
    u64 *V = nullptr;
    u32 *fails = d_u32 + 2, *overflow = d_u32 + 3;
    uint64_t tot[6];
    bool exact = head[5] != 0; // the two-pass sieve, which validates in the sieve
    if (!exact) {
        if ((rc = w.get(&V, (size_t)nv + 1, err))) return rc;
        k_bcf_gather<<<(unsigned)((n_tiles1 + 7) / 8), 256, 0, st>>>(count1, base1, lists, n_tiles1, V);
        k_bcf_check<<<grid_for(nv + 1, 256), 256, 0, st>>>(b->data, start, len, V, nv, fails, true);
        k_bcf_finalize<<<1, 1, 0, st>>>(b->data, start, len, V, d_u32, fails, overflow, totals);
        LAUNCH_OK("launching the BCF tiling proof");
        if ((rc = read_back(st, totals, tot, sizeof tot, err, "BCF scan"))) return rc;
        exact = (tot[5] & 2u) != 0; // a candidate is not a record: its list is not the survivors'
    }
    if (exact) {
        cudaMemsetAsync(d_u32, 0, 32, st);
        k_bcf_sieve<<<(unsigned)n_tiles, TB, 0, st>>>(b->data, start, len, samples, contigs, 0, tile_count,
                                                      nullptr, nullptr, nullptr);
        LAUNCH_OK("launching the BCF sieve");
        if ((e = frt_launch_scan_u32(tile_count, n_tiles, partials, tile_base, d_u32, st)) != cudaSuccess)
            return cuda_fail(err, e, "scanning survivors");
        if ((rc = read_back(st, d_u32, &nv, 4, err, "survivor count"))) return rc;
        if ((rc = w.get(&V, (size_t)nv + 1, err))) return rc;
        k_bcf_sieve<<<(unsigned)n_tiles, TB, 0, st>>>(b->data, start, len, samples, contigs, 1, tile_count,
                                                      tile_base, V, overflow);
        k_bcf_check<<<grid_for(nv + 1, 256), 256, 0, st>>>(b->data, start, len, V, nv, fails, false);
        k_bcf_finalize<<<1, 1, 0, st>>>(b->data, start, len, V, d_u32, fails, overflow, totals);
        LAUNCH_OK("launching the BCF tiling proof");
        if ((rc = read_back(st, totals, tot, sizeof tot, err, "BCF scan"))) return rc;
    }
    const u64 *list = V;
    if (tot[4]) { // the walk (bcf.rs:376-410): count, then emit
        k_bcf_walk<<<1, 1, 0, st>>>(b->data, start, len, nullptr, totals);
        LAUNCH_OK("launching the BCF walk");
        uint64_t wt[2];
        if ((rc = read_back(st, totals, wt, sizeof wt, err, "BCF walk"))) return rc;
        u64 *Wl;
        if ((rc = w.get(&Wl, wt[0] + 1, err))) return rc;
        k_bcf_walk<<<1, 1, 0, st>>>(b->data, start, len, Wl, totals);
        LAUNCH_OK("launching the BCF walk");
        tot[0] = wt[0];
        tot[1] = wt[1];
        list = Wl;
    }
    frt_columns *c = columns_new(s, FMT_BCF, kBcfWidths, FRT_BCF_COL_COUNT, tot[0]);
    c->tail = tot[1];
    c->info[0] = tot[2];
    c->info[1] = tot[3];
    c->info[2] = tot[3];
    if ((rc = columns_alloc(c, err))) {
        columns_discard(c);
        return rc;
    }
    if (c->n) {
        BcfCols bc{colp<int>(c, FRT_BCF_COL_CHROMOSOME_ID), colp<int>(c, FRT_BCF_COL_POSITION),
                   colp<int>(c, FRT_BCF_COL_REFERENCE_SPAN), colp<u32>(c, FRT_BCF_COL_QUALITY),
                   colp<u16>(c, FRT_BCF_COL_INFO_COUNT), colp<u16>(c, FRT_BCF_COL_ALLELE_COUNT),
                   colp<u32>(c, FRT_BCF_COL_SAMPLE_COUNT), colp<u8>(c, FRT_BCF_COL_FORMAT_COUNT),
                   colp<u64>(c, FRT_BCF_COL_RECORD_OFFSETS), colp<u32>(c, FRT_BCF_COL_ALLELES_START),
                   colp<u32>(c, FRT_BCF_COL_FILTERS_START), colp<u32>(c, FRT_BCF_COL_INFO_START),
                   colp<u32>(c, FRT_BCF_COL_GENOTYPES_START), colp<u32>(c, FRT_BCF_COL_RECORD_END)};
        u32 *errors = d_u32 + 4;
        k_bcf_decode<<<grid_for(c->n, 256), 256, 0, st>>>(b->data, len, list, (u32)c->n, bc, errors);
        uint32_t n_err = 0;
        if ((e = cudaGetLastError()) != cudaSuccess) {
            columns_discard(c);
            return cuda_fail(err, e, "launching the BCF decode");
        }
        if ((rc = read_back(st, errors, &n_err, 4, err, "BCF decode"))) {
            columns_discard(c);
            return rc;
        }
        if (n_err) { // bcf.rs:343-356
            columns_discard(c);
            set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, 0, "bcf", "%u of %llu records failed to decode", n_err,
                      (unsigned long long)tot[0]);
            return FRT_ERR_MALFORMED;
        }
    }
    return columns_finish(c, b, out);
}

// BCF header (crates/fritillaria-bcf/src/columnar/header.rs:111-310): where
// records start, the sample count and the contig count.
namespace {
bool ws(uint8_t c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

const uint8_t *attr(const uint8_t *b, const uint8_t *be, const char *key, const uint8_t **ve)
{
    size_t kl = strlen(key);
    const uint8_t *p = b;
    while (p < be) {
        const uint8_t *s0 = p, *eq = nullptr;
        bool quoted = false;
        while (p < be) {
            if (*p == '"') quoted = !quoted;
            else if (*p == '=' && !quoted && !eq) eq = p;
            else if (*p == ',' && !quoted) break;
            ++p;
        }
        if (eq) {
            const uint8_t *ns = s0, *ne = eq;
            while (ns < ne && ws(*ns)) ++ns;
            while (ne > ns && ws(ne[-1])) --ne;
            if ((size_t)(ne - ns) == kl && memcmp(ns, key, kl) == 0) {
                const uint8_t *v = eq + 1, *vend = p;
                while (v < vend && ws(*v)) ++v;
                while (vend > v && ws(vend[-1])) --vend;
                if (vend - v >= 2 && *v == '"' && vend[-1] == '"') {
                    ++v;
                    --vend;
                }
                *ve = vend;
                return v;
            }
        }
        ++p;
    }
    return nullptr;
}

bool has_prefix(const uint8_t *s, const uint8_t *e, const char *pfx)
{
    size_t n = strlen(pfx);
    return (size_t)(e - s) >= n && memcmp(s, pfx, n) == 0;
}
} // namespace

extern "C" int frt_bcf_parse_header(const uint8_t *buf, size_t len, uint64_t *records_start, uint32_t *samples,
                                    uint32_t *contigs, frt_error *err)
{
    auto bad = [&](uint64_t pos, const char *why) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, pos, "bcf header", "%s", why);
        return FRT_ERR_MALFORMED;
    };
    if (!buf || len < 9) return bad(0, "truncated header");
    if (memcmp(buf, "BCF", 3) != 0) return bad(0, "bad magic; expected BCF");
    if (buf[3] != 2) return bad(3, "unsupported major version; expected 2");
    uint64_t l_text = (uint64_t)buf[5] | ((uint64_t)buf[6] << 8) | ((uint64_t)buf[7] << 16) | ((uint64_t)buf[8] << 24);
    if (9 + l_text > len) return bad(5, "l_text runs past the end of the buffer");
    const uint8_t *t = buf + 9, *te = buf + 9 + l_text;
    while (te > t && te[-1] == 0) --te;
    uint32_t n_samples = 0, n_contigs = 0;
    std::vector<std::pair<const uint8_t *, size_t>> seen;
    for (const uint8_t *line = t; line < te;) {
        const uint8_t *le = (const uint8_t *)memchr(line, '\n', (size_t)(te - line));
        if (!le) le = te;
        const uint8_t *next = le < te ? le + 1 : te;
        if (le > line && le[-1] == '\r') --le;
        if (le == line) {
            line = next;
            continue;
        }
        if (has_prefix(line, le, "#CHROM")) {
            size_t pieces = 1;
            for (const uint8_t *p = line + 6; p < le; ++p) pieces += *p == '\t';
            n_samples = pieces > 9 ? (uint32_t)(pieces - 9) : 0;
            line = next;
            continue;
        }
        const uint8_t *open = (const uint8_t *)memchr(line, '<', (size_t)(le - line)), *close = nullptr;
        for (const uint8_t *p = le; p > line; --p)
            if (p[-1] == '>') {
                close = p - 1;
                break;
            }
        const uint8_t *ide = nullptr, *id = (open && close && close > open) ? attr(open + 1, close, "ID", &ide) : nullptr;
        if (!id) {
            line = next;
            continue;
        }
        if (has_prefix(line, le, "##contig=")) {
            ++n_contigs;
        } else if (has_prefix(line, le, "##FILTER=") || has_prefix(line, le, "##INFO=") ||
                   has_prefix(line, le, "##FORMAT=")) {
            size_t il = (size_t)(ide - id);
            bool dup = il == 4 && memcmp(id, "PASS", 4) == 0;
            for (auto &p : seen)
                if (!dup && p.second == il && memcmp(p.first, id, il) == 0) dup = true;
            if (!dup) {
                const uint8_t *xe = nullptr, *x = attr(open + 1, close, "IDX", &xe);
                if (x) {
                    bool ok = xe > x;
                    for (const uint8_t *p = x; p < xe && ok; ++p) ok = *p >= '0' && *p <= '9';
                    if (!ok) return bad(0, "unparseable IDX on header line");
                }
                seen.emplace_back(id, il);
            }
        }
        line = next;
    }
    if (records_start) *records_start = 9 + l_text;
    if (samples) *samples = n_samples;
    if (contigs) *contigs = n_contigs;
    return FRT_OK;
}

// ---- FASTA -------------------------------------------------------------------

extern "C" int frt_fasta_compactor_create(int device, void *stream, frt_fasta_compactor **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    frt_fasta_compactor *s = new frt_fasta_compactor;
    int rc = scanner_create(device, stream, &s->s, err);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return FRT_OK;
}

extern "C" void frt_fasta_compactor_destroy(frt_fasta_compactor *s)
{
    if (!s) return;
    scanner_release(s->s);
    delete s;
}

extern "C" int frt_fasta_compact(frt_fasta_compactor *sc, const frt_inflate_batch *b, frt_columns **out,
                                 frt_error *err)
{
    if (!sc || !out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = sc->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    uint64_t len = b && b->data ? b->len : 0;
    auto empty = [&]() {
        frt_columns *c = columns_new(s, FMT_FASTA, kFastaWidths, FRT_FASTA_COL_COUNT, 0);
        c->col_bytes[FRT_FASTA_COL_SEQUENCE] = 0;
        int rc = columns_alloc(c, err);
        if (rc) {
            columns_discard(c);
            return rc;
        }
        return columns_finish(c, b, out);
    };
    if (len == 0) return empty();
    int rc = check_batch(s, b, err);
    if (rc) return rc;
    cudaStream_t st = s.stream;
    Work w(st);
    const u64 n_tiles = (len + TILE - 1) / TILE;
    if (n_tiles >= 0xffffffffull) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "FASTA batch too large");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    // the passes read aligned 16-byte blocks from the 16-byte boundary at or
    // before the batch (the sh bytes before it are never read)
    const u64 sh = (uintptr_t)b->data & 15u;
    const u8 *abuf = b->data - sh;
    const u64 n_tiles2 = (len + sh + TILE - 1) / TILE;
    u8 *tile_f, *tile_state;
    u32 *tile_contigs, *contig_base, *tile_kept3;
    u64 *out_base, *totals;
    unsigned long long *last_contig;
    if ((rc = w.get(&tile_f, n_tiles2, err)) || (rc = w.get(&tile_state, n_tiles2, err)) ||
        (rc = w.get(&tile_contigs, n_tiles2, err)) || (rc = w.get(&contig_base, n_tiles2, err)) ||
        (rc = w.get(&tile_kept3, 3 * n_tiles2, err)) ||
        (rc = w.get(&out_base, n_tiles2 + 1, err)) || (rc = w.get(&totals, 8, err)) ||
        (rc = w.get(&last_contig, 2, err)))
        return rc;
    cudaMemsetAsync(last_contig, 0, 16, st);
    cudaMemsetAsync(totals, 0, 64, st);
    const u32 n_chunks = (u32)((n_tiles2 + 1023) / 1024);
    u8 *chunk_f, *chunk_state;
    u32 *chunk_contigs;
    u64 *chunk_kept3, *chunk_contig_base, *chunk_out_base;
    if ((rc = w.get(&chunk_f, n_chunks, err)) || (rc = w.get(&chunk_state, n_chunks, err)) ||
        (rc = w.get(&chunk_contigs, n_chunks, err)) || (rc = w.get(&chunk_kept3, 3ull * n_chunks, err)) ||
        (rc = w.get(&chunk_contig_base, n_chunks, err)) || (rc = w.get(&chunk_out_base, n_chunks, err)))
        return rc;
    k_fa_sum<<<(unsigned)n_tiles2, TB, 0, st>>>(abuf, sh, len, tile_f, tile_contigs, tile_kept3, last_contig);
    k_fa_chunks<<<n_chunks, 1024, 0, st>>>(tile_f, tile_contigs, tile_kept3, (u32)n_tiles2, chunk_f, chunk_contigs,
                                           chunk_kept3);
    k_fa_top<<<1, 1024, 0, st>>>(b->data, len, chunk_f, chunk_contigs, chunk_kept3, n_chunks, chunk_state,
                                 chunk_contig_base, chunk_out_base, last_contig, totals);
    k_fa_apply<<<n_chunks, 1024, 0, st>>>(tile_f, tile_contigs, tile_kept3, (u32)n_tiles2, chunk_state,
                                          chunk_contig_base, chunk_out_base, tile_state, contig_base, out_base);
    LAUNCH_OK("launching the FASTA scans");
    uint64_t tot[3];
    if ((rc = read_back(st, totals, tot, sizeof tot, err, "FASTA layout"))) return rc;
    const uint64_t n = tot[0], total = tot[1];
    if (n == 0) return empty();
    frt_columns *c = columns_new(s, FMT_FASTA, kFastaWidths, FRT_FASTA_COL_COUNT, n);
    c->total = total;
    c->col_bytes[FRT_FASTA_COL_SEQUENCE] = 0; // the bases have their own allocation
    if ((rc = columns_alloc(c, err)) || (rc = dev_alloc((void **)&c->seq, total + 16, st, err))) {
        columns_discard(c);
        return rc;
    }
    c->col_bytes[FRT_FASTA_COL_SEQUENCE] = total;
    u64 *seq_off = colp<u64>(c, FRT_FASTA_COL_SEQUENCE_OFFSETS), *seq_len = colp<u64>(c, FRT_FASTA_COL_SEQUENCE_LENGTHS),
        *rec_off = colp<u64>(c, FRT_FASTA_COL_RECORD_OFFSETS);
    k_fa_emit<<<(unsigned)n_tiles2, TB, 0, st>>>(abuf, sh, len, tile_state, contig_base, out_base, n, c->seq,
                                                 seq_off, rec_off);
    k_fa_lengths<<<grid_for(n, 256), 256, 0, st>>>(seq_off, n, total, seq_len);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        columns_discard(c);
        return cuda_fail(err, e, "launching the FASTA compaction");
    }
    return columns_finish(c, b, out);
}

// ---- column batches ------------------------------------------------------------

extern "C" uint64_t frt_columns_len(const frt_columns *c) { return c ? c->n : 0; }
extern "C" uint64_t frt_columns_tail(const frt_columns *c) { return c ? c->tail : 0; }
extern "C" uint64_t frt_columns_total_bases(const frt_columns *c) { return c ? c->total : 0; }
extern "C" int frt_columns_count(const frt_columns *c) { return c ? c->n_cols : 0; }
extern "C" int frt_columns_device_ordinal(const frt_columns *c) { return c ? c->device : -1; }
extern "C" void *frt_columns_ready_event(const frt_columns *c) { return c ? (void *)c->ready : nullptr; }

extern "C" void frt_columns_scan_info(const frt_columns *c, uint64_t *proof, uint64_t *survivors, uint64_t *validated)
{
    if (proof) *proof = c ? c->info[0] : 0;
    if (survivors) *survivors = c ? c->info[1] : 0;
    if (validated) *validated = c ? c->info[2] : 0;
}

static const uint8_t *column_base(const frt_columns *c, int k)
{
    if (c->format == FMT_FASTA && k == FRT_FASTA_COL_SEQUENCE) return c->seq;
    return c->cols + c->col_off[k];
}

extern "C" int frt_columns_column(const frt_columns *c, int column, void **ptr, size_t *bytes, size_t *width)
{
    if (!c || column < 0 || column >= c->n_cols) return FRT_ERR_INVALID_ARGUMENT;
    if (ptr) *ptr = (void *)column_base(c, column);
    if (bytes) *bytes = c->col_bytes[column];
    if (width) *width = c->widths[column];
    return FRT_OK;
}

extern "C" int frt_columns_column_to_host(const frt_columns *c, int column, void *dst, size_t cap, frt_error *err)
{
    if (!c || column < 0 || column >= c->n_cols) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "bad column %d", column);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    size_t bytes = c->col_bytes[column];
    if (cap < bytes) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "destination holds %zu bytes, column has %zu",
                  cap, bytes);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (!bytes) return FRT_OK;
    DeviceGuardLite g(c->device);
    cudaError_t e = cudaMemcpyAsync(dst, column_base(c, column), bytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "downloading column");
    return FRT_OK;
}

extern "C" void frt_columns_free(frt_columns *c)
{
    if (!c) return;
    {
        DeviceGuardLite g(c->device);
        if (c->ready) cudaEventDestroy(c->ready);
    }
    const frt_inflate_batch *src = c->source;
    {
        DeviceGuardLite g(c->device);
        columns_discard(c);
    }
    if (src) batch_release(src);
}

// ---- tab-delimited text --------------------------------------------------------

extern "C" int frt_text_scanner_create(int device, void *stream, frt_text_scanner **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    frt_text_scanner *s = new frt_text_scanner;
    int rc = scanner_create(device, stream, &s->s, err);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return FRT_OK;
}

extern "C" void frt_text_scanner_destroy(frt_text_scanner *s)
{
    if (!s) return;
    scanner_release(s->s);
    delete s;
}

// TextScanner::scan (crates/fritillaria-cuda/src/text.rs:233-420): records,
// their ends, header lines and the field table; the tail is the last record's
// start when that record runs to the end of the batch, else the batch end.
extern "C" int frt_text_scan(frt_text_scanner *sc, const frt_inflate_batch *b, uint64_t start, int32_t comment,
                             int32_t secondary, frt_columns **out, frt_error *err)
{
    if (!sc || !out || comment < 0 || comment > 255 || secondary > 255) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "null argument, or a header byte outside 0..255 (secondary -1: none)");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = sc->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    uint64_t len = b && b->data ? b->len : 0;
    auto finish = [&](frt_columns *c, uint64_t n_hdr, uint64_t n_tabs) {
        c->col_bytes[FRT_TEXT_COL_HEADER_OFFSETS] = 8 * n_hdr;
        c->col_bytes[FRT_TEXT_COL_TABS] = 8 * n_tabs;
        c->col_bytes[FRT_TEXT_COL_FIELD_STARTS] = c->n ? 8 * (c->n + 1) : 0;
        size_t off = 0;
        for (int k = 0; k < FRT_TEXT_COL_COUNT; ++k) {
            c->col_off[k] = off;
            off += (c->col_bytes[k] + 255) & ~(size_t)255;
        }
        c->info[0] = n_hdr;
        c->total = n_tabs;
        return columns_alloc(c, err);
    };
    if (start >= len) { // empty(start.min(len))
        frt_columns *c = columns_new(s, FMT_TEXT, kTextWidths, FRT_TEXT_COL_COUNT, 0);
        c->tail = start < len ? start : len;
        int rc = finish(c, 0, 0);
        if (rc) {
            columns_discard(c);
            return rc;
        }
        return columns_finish(c, b, out);
    }
    int rc = check_batch(s, b, err);
    if (rc) return rc;
    if (len - start >= 0xffffffffull) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "text batch of %llu bytes exceeds 4 GiB",
                  (unsigned long long)(len - start));
        return FRT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st = s.stream;
    Work w(st);
    // The newline index reads aligned 16-byte blocks, so it works from the
    // 16-byte boundary at or before the batch (the sh bytes before the batch
    // are never read) and writes batch positions.
    const u64 sh = (uintptr_t)b->data & 15u;
    const u8 *abuf = b->data - sh;
    const u64 tbase = (start + sh) & ~15ull;
    const u64 n_tiles = (len + sh - tbase + TILE - 1) / TILE;
    u32 *tile_count, *tile_base, *partials, *d_u32;
    u16 *slot_pos;
    u8 *slot_lf;
    if ((rc = w.get(&tile_count, n_tiles, err)) || (rc = w.get(&tile_base, n_tiles + 1, err)) ||
        (rc = w.get(&partials, frt_scan_partials_len(n_tiles) + frt_scan_partials_len(len) + 8, err)) ||
        (rc = w.get(&d_u32, 8, err)) || (rc = scanner_slots(s, n_tiles, &slot_pos, &slot_lf, err)))
        return rc;
    k_nl_slots<<<(unsigned)n_tiles, TB, 0, st>>>(abuf, start + sh, len + sh, tbase, tile_count, slot_pos, slot_lf,
                                                 d_u32 + 7);
    LAUNCH_OK("launching the newline count");
    cudaError_t e = frt_launch_scan_u32(tile_count, n_tiles, partials, tile_base, d_u32, st);
    if (e != cudaSuccess) return cuda_fail(err, e, "scanning newline counts");
    uint32_t hd[8] = {};
    if ((rc = read_back(st, d_u32, hd, sizeof hd, err, "newline count"))) return rc;
    const uint32_t n_nl = hd[0];
    u32 *nl;
    u8 *lf;
    if ((rc = w.get(&nl, (size_t)n_nl + 1, err)) || (rc = w.get(&lf, (size_t)n_nl + 1, err))) return rc;
    k_nl_gather<<<(unsigned)((n_tiles + TB / 32 - 1) / (TB / 32)), TB, 0, st>>>(
        abuf, start + sh, len + sh, tbase, n_tiles, tile_count, tile_base, slot_pos, slot_lf, nl, lf);
    LAUNCH_OK("launching the newline index");
    // line starts: start, and one past every newline that is not the last byte
    const uint32_t n_lines = n_nl && hd[7] ? n_nl : n_nl + 1;
    FqIndex ix{b->data, start, len, nl, n_nl, n_lines, lf};
    u32 *is_rec, *is_hdr, *rec_pos, *hdr_pos;
    if ((rc = w.get(&is_rec, n_lines, err)) || (rc = w.get(&is_hdr, n_lines, err)) ||
        (rc = w.get(&rec_pos, (size_t)n_lines + 1, err)) || (rc = w.get(&hdr_pos, (size_t)n_lines + 1, err)))
        return rc;
    k_tx_lines<<<grid_for(n_lines, 256), 256, 0, st>>>(ix, (u32)comment, secondary < 0 ? 0xffffffffu : (u32)secondary,
                                                         is_rec, is_hdr);
    LAUNCH_OK("launching the line kinds");
    uint32_t counts[2] = {0, 0};
    if ((e = frt_launch_scan_u32(is_rec, n_lines, partials, rec_pos, d_u32, st)) != cudaSuccess ||
        (e = frt_launch_scan_u32(is_hdr, n_lines, partials, hdr_pos, d_u32 + 1, st)) != cudaSuccess)
        return cuda_fail(err, e, "scanning line kinds");
    if ((rc = read_back(st, d_u32, counts, 8, err, "line kinds"))) return rc;
    const uint32_t n_rec = counts[0], n_hdr = counts[1];
    u64 *rec_off, *rec_end, *hdr_off;
    if ((rc = w.get(&rec_off, (size_t)n_rec + 1, err)) || (rc = w.get(&rec_end, (size_t)n_rec + 1, err)) ||
        (rc = w.get(&hdr_off, (size_t)n_hdr + 1, err)))
        return rc;
    k_tx_place<<<grid_for(n_lines, 256), 256, 0, st>>>(ix, is_rec, rec_pos, is_hdr, hdr_pos, rec_off, rec_end,
                                                         hdr_off);
    LAUNCH_OK("placing lines");
    u32 *tab_count, *tab_base;
    uint32_t n_tabs = 0;
    uint64_t tail = len;
    if (n_rec) {
        if ((rc = w.get(&tab_count, n_rec, err)) || (rc = w.get(&tab_base, (size_t)n_rec + 1, err))) return rc;
        k_tx_count_tabs<<<grid_for((u64)n_rec * 32, 256), 256, 0, st>>>(b->data, rec_off, rec_end, n_rec, tab_count);
        LAUNCH_OK("counting fields");
        if ((e = frt_launch_scan_u32(tab_count, n_rec, partials, tab_base, d_u32, st)) != cudaSuccess)
            return cuda_fail(err, e, "scanning field counts");
        uint64_t last[2] = {0, 0};
        if ((rc = read_back(st, d_u32, &n_tabs, 4, err, "field count")) ||
            (rc = read_back(st, rec_off + n_rec - 1, &last[0], 8, err, "last record")) ||
            (rc = read_back(st, rec_end + n_rec - 1, &last[1], 8, err, "last record")))
            return rc;
        tail = last[1] >= len ? last[0] : len; // text.rs:393-397
    }
    frt_columns *c = columns_new(s, FMT_TEXT, kTextWidths, FRT_TEXT_COL_COUNT, n_rec);
    c->tail = tail;
    if ((rc = finish(c, n_hdr, n_tabs))) {
        columns_discard(c);
        return rc;
    }
    auto put = [&](int k, const void *src) {
        return c->col_bytes[k] ? cudaMemcpyAsync(colp<u8>(c, k), src, c->col_bytes[k], cudaMemcpyDeviceToDevice, st)
                               : cudaSuccess;
    };
    if ((e = put(FRT_TEXT_COL_RECORD_OFFSETS, rec_off)) != cudaSuccess ||
        (e = put(FRT_TEXT_COL_RECORD_ENDS, rec_end)) != cudaSuccess ||
        (e = put(FRT_TEXT_COL_HEADER_OFFSETS, hdr_off)) != cudaSuccess) {
        columns_discard(c);
        return cuda_fail(err, e, "placing text columns");
    }
    if (n_rec) {
        if (n_tabs)
            k_tx_emit_tabs<<<grid_for((u64)n_rec * 32, 256), 256, 0, st>>>(
                b->data, rec_off, rec_end, n_rec, tab_base, colp<u64>(c, FRT_TEXT_COL_TABS));
        k_tx_starts<<<grid_for((u64)n_rec + 1, 256), 256, 0, st>>>(tab_base, n_rec + 1,
                                                                   colp<u64>(c, FRT_TEXT_COL_FIELD_STARTS));
        if ((e = cudaGetLastError()) != cudaSuccess) {
            columns_discard(c);
            return cuda_fail(err, e, "launching the field table");
        }
    }
    return columns_finish(c, b, out);
}

// ---- columnar VCF over the text framing --------------------------------------
//
// The fixed fields of every VCF record of a text batch, with the semantics of
// the vendored lazy reader: read_record (crates/fritillaria-vcf/src/io/reader/
// record.rs:9-118) takes seven tab-terminated fields, then the INFO field up to
// a tab or the end of the line, and drops a carriage return before the line
// feed; the accessors (record/fields.rs:20-103, record.rs:35-79) read "."
// as missing, "0" as the telomere start, a position with usize::from_str and
// Position::try_from, the quality with f32::from_str, and the alternate bases
// split on ','.  The reference's own device path stops at the text framing
// (its README lists columnar VCF.gz as the next step); this is that step.

namespace {

const size_t kVcfWidths[FRT_VCF_COL_COUNT] = {4, 8, 4 * FRT_VCF_BOUNDS, 4, 4, 2, 1};
const size_t kVcfGtWidths[FRT_VCF_GT_COL_COUNT] = {4, 4};
enum { FMT_VCF = 5, FMT_VCF_GT = 6 };

struct VcfDict {
    const u32 *slots = nullptr; // index + 1 per slot, 0 empty; open addressing
    const u32 *name_off = nullptr; // n + 1 offsets into names
    const u8 *names = nullptr;
    u32 mask = 0, n = 0;
};

__host__ __device__ __forceinline__ u32 fnv1a(const u8 *p, u32 n)
{
    u32 h = 2166136261u;
    for (u32 i = 0; i < n; ++i) h = (h ^ p[i]) * 16777619u;
    return h;
}

__device__ int vcf_contig(const VcfDict &d, const u8 *p, u32 n)
{
    if (!d.n) return -1;
    for (u32 s = fnv1a(p, n) & d.mask;; s = (s + 1) & d.mask) {
        const u32 v = d.slots[s];
        if (!v) return -1;
        const u32 a = d.name_off[v - 1], b = d.name_off[v];
        if (b - a != n) continue;
        u32 i = 0;
        while (i < n && d.names[a + i] == p[i]) ++i;
        if (i == n) return (int)(v - 1);
    }
}

// usize::from_str: an optional '+', then one or more ASCII digits, no overflow.
__device__ bool vcf_usize(const u8 *p, u32 n, u64 *out)
{
    u32 i = n && p[0] == '+' ? 1u : 0u;
    if (i == n) return false;
    u64 v = 0;
    for (; i < n; ++i) {
        const u32 c = (u32)p[i] - '0';
        if (c > 9u) return false;
        if (v > (~0ull - c) / 10ull) return false;
        v = v * 10ull + c;
    }
    *out = v;
    return true;
}

__device__ __forceinline__ bool vcf_is(const u8 *p, u32 n, const char *lit, u32 m)
{
    if (n != m) return false;
    for (u32 i = 0; i < m; ++i)
        if (p[i] != (u8)lit[i]) return false;
    return true;
}

// The quality as f32::from_str would give it, when Clinger's fast path
// ("How to read floating point numbers accurately", 1990) applies: a decimal
// of at most 2^24 with a power of ten of at most 10^10 either way, both exact
// in binary32, so one correctly rounded multiply or divide is the correctly
// rounded value.  Anything else -- more digits, a larger exponent, inf, NaN or
// text f32::from_str rejects -- is left unparsed (returns false).
__device__ bool vcf_qual(const u8 *p, u32 n, float *out)
{
    u32 i = 0;
    bool neg = false;
    if (i < n && (p[i] == '+' || p[i] == '-')) neg = p[i++] == '-';
    u64 m = 0;
    int e10 = 0, digits = 0;
    bool big = false;
    for (; i < n && p[i] >= '0' && p[i] <= '9'; ++i, ++digits) {
        if (m < 100000000000000000ull) m = m * 10ull + (p[i] - '0');
        else { big = true; ++e10; }
    }
    if (i < n && p[i] == '.') {
        for (++i; i < n && p[i] >= '0' && p[i] <= '9'; ++i, ++digits)
            if (m < 100000000000000000ull) { m = m * 10ull + (p[i] - '0'); --e10; }
            else big = true;
    }
    if (!digits) return false;
    if (i < n && (p[i] == 'e' || p[i] == 'E')) {
        ++i;
        bool eneg = false;
        if (i < n && (p[i] == '+' || p[i] == '-')) eneg = p[i++] == '-';
        if (i == n) return false;
        int x = 0;
        for (; i < n && p[i] >= '0' && p[i] <= '9'; ++i)
            if (x < 100000) x = x * 10 + (p[i] - '0');
        e10 += eneg ? -x : x;
    }
    if (i != n || big) return false;
    if (m == 0) {
        *out = neg ? -0.0f : 0.0f;
        return true;
    }
    while (e10 < 0 && m % 10ull == 0) { // trailing zeros of the fraction
        m /= 10ull;
        ++e10;
    }
    while (e10 > 10 && m * 10ull <= (1ull << 24)) { // a small mantissa absorbs the excess exponent
        m *= 10ull;
        --e10;
    }
    if (m > (1ull << 24) || e10 > 10 || e10 < -10) return false;
    const float p10[11] = {1e0f, 1e1f, 1e2f, 1e3f, 1e4f, 1e5f, 1e6f, 1e7f, 1e8f, 1e9f, 1e10f};
    const float v = (float)m;
    const float r = e10 >= 0 ? __fmul_rn(v, p10[e10]) : __fdiv_rn(v, p10[-e10]);
    *out = neg ? -r : r;
    return true;
}

__global__ void k_vcf_fields(const u8 *buf, u64 buf_len, const u64 *rec_off, const u64 *rec_end, const u64 *tabs,
                             const u64 *field_starts, u64 n, VcfDict dict, int *chrom, u64 *pos, u32 *bounds,
                             u32 *n_alt, u32 *qual, u16 *flags, u8 *status)
{
    const u64 r = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const u64 a = rec_off[r];
    const u8 *p = buf + a;
    const u32 len = (u32)(rec_end[r] - a);
    const u64 fs = field_starts[r], nt = field_starts[r + 1] - fs;
    // read_field and read_line drop a carriage return before a line feed; a
    // record ends at its line feed, or at the batch end when it has none
    const bool lf = rec_end[r] < buf_len;
    const u32 content = lf && len && p[len - 1] == '\r' ? len - 1 : len;
    u32 e[FRT_VCF_BOUNDS] = {};
    int cid = -1;
    u64 v = 0;
    u32 na = 0, qv = 0x7fc00000u;
    u16 fl = 0;
    u8 st = 0;
    if (nt < 7) {
        st = FRT_VCF_STATUS_UNEXPECTED_EOL;
    } else {
#pragma unroll
        for (int k = 0; k < 7; ++k) e[k] = (u32)(tabs[fs + k] - a);
        e[7] = nt >= 8 ? (u32)(tabs[fs + 7] - a) : content;
        e[8] = content;
        cid = vcf_contig(dict, p, e[0]);
        const u8 *f = p + e[0] + 1;
        u32 fn = e[1] - e[0] - 1;
        if (vcf_is(f, fn, "0", 1)) {
            fl |= FRT_VCF_FLAG_TELOMERE;
        } else if (!vcf_usize(f, fn, &v) || v == 0) {
            v = 0;
            st = FRT_VCF_STATUS_INVALID_POSITION;
        }
        if (vcf_is(p + e[1] + 1, e[2] - e[1] - 1, ".", 1)) fl |= FRT_VCF_FLAG_ID_MISSING;
        f = p + e[3] + 1;
        fn = e[4] - e[3] - 1;
        if (vcf_is(f, fn, ".", 1)) {
            fl |= FRT_VCF_FLAG_ALT_MISSING;
        } else if (fn) {
            na = 1;
            for (u32 i = 0; i < fn; ++i) na += f[i] == ',' ? 1u : 0u;
        }
        f = p + e[4] + 1;
        fn = e[5] - e[4] - 1;
        float q;
        if (vcf_is(f, fn, ".", 1)) fl |= FRT_VCF_FLAG_QUAL_MISSING;
        else if (vcf_qual(f, fn, &q)) {
            fl |= FRT_VCF_FLAG_QUAL_PARSED;
            qv = __float_as_uint(q);
        }
        f = p + e[5] + 1;
        fn = e[6] - e[5] - 1;
        if (vcf_is(f, fn, ".", 1)) fl |= FRT_VCF_FLAG_FILTER_MISSING;
        else if (vcf_is(f, fn, "PASS", 4)) fl |= FRT_VCF_FLAG_FILTER_PASS;
        if (vcf_is(p + e[6] + 1, e[7] - e[6] - 1, ".", 1)) fl |= FRT_VCF_FLAG_INFO_MISSING;
        // samples: what follows INFO; missing when empty or its first piece is "."
        if (nt < 8) {
            fl |= FRT_VCF_FLAG_SAMPLES_MISSING;
        } else {
            const u32 s0 = e[7] + 1, s1 = nt >= 9 ? (u32)(tabs[fs + 8] - a) : content;
            if (s0 >= content || vcf_is(p + s0, s1 - s0, ".", 1)) fl |= FRT_VCF_FLAG_SAMPLES_MISSING;
        }
    }
    chrom[r] = cid;
    pos[r] = v;
#pragma unroll
    for (int k = 0; k < FRT_VCF_BOUNDS; ++k) bounds[FRT_VCF_BOUNDS * r + k] = e[k];
    n_alt[r] = na;
    qual[r] = qv;
    flags[r] = fl;
    status[r] = st;
}

// One sample's GT value (crates/fritillaria-vcf/src/record/samples/series/
// value.rs:17-30 and value/genotype/iter.rs): "." is missing; otherwise the
// alleles split before each '|' or '/', the first one's phasing explicit when
// it opens with one, else unphased when a '/' follows anywhere and phased
// when none does; each position "." or usize::from_str; an empty value is an
// error.  Packed as FRT_VCF_GT_*.
__device__ u32 vcf_gt_code(const u8 *p, u32 n)
{
    if (n == 1 && p[0] == '.') return (u32)FRT_VCF_GT_MISSING << 28;
    if (n == 0) return (u32)FRT_VCF_GT_INVALID << 28;
    u32 codes[2] = {0, 0}, phased[2] = {0, 0}, ploidy = 0;
    u32 i = 0;
    while (i < n) {
        // the allele: [i, j) with the next separator searched from i + 1
        u32 j = i + 1;
        while (j < n && p[j] != '|' && p[j] != '/') ++j;
        u32 a = i, ph;
        if (p[a] == '|' || p[a] == '/') {
            ph = p[a] == '|';
            ++a;
        } else { // only the first allele can lack a separator
            ph = 1;
            for (u32 k = j; k < n; ++k)
                if (p[k] == '/') ph = 0;
        }
        u32 code;
        if (j - a == 1 && p[a] == '.') {
            code = 0;
        } else {
            u64 v;
            if (!vcf_usize(p + a, j - a, &v)) return (u32)FRT_VCF_GT_INVALID << 28;
            if (v >= 4095ull) code = 0x1000u; // valid but wider than 12 bits
            else code = (u32)v + 1u;
        }
        if (ploidy < 2) {
            codes[ploidy] = code;
            phased[ploidy] = ph;
        }
        ++ploidy;
        i = j;
    }
    // the whole value was walked, so an invalid allele anywhere is reported first
    if (ploidy > 2 || codes[0] == 0x1000u || codes[1] == 0x1000u) return (u32)FRT_VCF_GT_UNREPRESENTED << 28;
    return (ploidy << 26) | (phased[1] << 25) | (phased[0] << 24) | (codes[1] << 12) | codes[0];
}

// Every sample's GT, 2^wl warps per record with their lanes over its
// samples (a population VCF holds thousands a record, so one warp a record
// leaves most of the GPU idle on a few thousand records).  Each warp finds
// the GT key itself.  calls[t] is the call of the sample that tab t opens
// (tabs 8 on of each record); the first eight tabs of a record get 0.
// key[r] = GT's index among the FORMAT keys, -1 when the record has no
// samples or no GT key.
__global__ void k_vcf_gt(const u8 *buf, u64 buf_len, const u64 *rec_off, const u64 *rec_end, const u64 *tabs,
                         const u64 *field_starts, u64 n, u32 wl, u32 *calls, int *key)
{
    const u64 gw = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const u64 r = gw >> wl;
    const u32 sub = (u32)(gw & ((1ull << wl) - 1ull));
    const u32 lane = threadIdx.x & 31u;
    if (r >= n) return;
    const u64 a = rec_off[r];
    const u8 *p = buf + a;
    const u32 len = (u32)(rec_end[r] - a);
    const u64 fs = field_starts[r], nt = field_starts[r + 1] - fs;
    const u32 content = rec_end[r] < buf_len && len && p[len - 1] == '\r' ? len - 1 : len;
    if (sub == 0)
        for (u64 t = lane; t < nt && t < 8ull; t += 32) calls[fs + t] = 0;
    if (nt < 8) {
        if (sub == 0 && lane == 0) key[r] = -1;
        return;
    }
    // FORMAT: [tab 7 + 1, tab 8 or the end); samples are missing when there
    // is nothing after INFO or FORMAT is "."
    const u32 f0 = (u32)(tabs[fs + 7] - a) + 1u, f1 = nt >= 9 ? (u32)(tabs[fs + 8] - a) : content;
    int g = -1;
    if (f0 < content && !(f1 - f0 == 1 && p[f0] == '.')) {
        int k = 0;
        for (u32 q = f0; q <= f1; ++k) {
            u32 e = q;
            while (e < f1 && p[e] != ':') ++e;
            if (e - q == 2 && p[q] == 'G' && p[q + 1] == 'T') {
                g = k;
                break;
            }
            q = e + 1;
        }
    }
    if (sub == 0 && lane == 0) key[r] = g;
    for (u64 j = 32u * sub + lane; j + 8 < nt; j += 32ull << wl) {
        u32 code = (u32)FRT_VCF_GT_NONE << 28;
        if (g >= 0) {
            const u32 s0 = (u32)(tabs[fs + 8 + j] - a) + 1u;
            const u32 s1 = j + 9 < nt ? (u32)(tabs[fs + 9 + j] - a) : content;
            if (s0 < s1) { // an empty sample has no values
                u32 q = s0;
                int k = 0;
                for (; k < g && q <= s1; ++k) {
                    while (q < s1 && p[q] != ':') ++q;
                    ++q;
                }
                if (q <= s1) {
                    u32 e = q;
                    while (e < s1 && p[e] != ':') ++e;
                    code = vcf_gt_code(p + q, e - q);
                }
            }
        }
        calls[fs + 8 + j] = code;
    }
}

} // namespace

struct frt_vcf_decoder {
    Scanner s;
    u32 *slots = nullptr, *name_off = nullptr;
    u8 *names = nullptr;
    u32 mask = 0, n = 0;
};

extern "C" int frt_vcf_decoder_create(int device, void *stream, frt_vcf_decoder **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    frt_vcf_decoder *d = new frt_vcf_decoder;
    int rc = scanner_create(device, stream, &d->s, err);
    if (rc) {
        delete d;
        return rc;
    }
    *out = d;
    return FRT_OK;
}

namespace {
void vcf_free_dict(frt_vcf_decoder *d)
{
    dev_free(d->slots, d->s.stream);
    dev_free(d->name_off, d->s.stream);
    dev_free(d->names, d->s.stream);
    d->slots = d->name_off = nullptr;
    d->names = nullptr;
    d->mask = d->n = 0;
}
} // namespace

extern "C" void frt_vcf_decoder_destroy(frt_vcf_decoder *d)
{
    if (!d) return;
    {
        DeviceGuardLite g(d->s.device);
        vcf_free_dict(d);
        cudaStreamSynchronize(d->s.stream);
    }
    stream_release(d->s.shared);
    delete d;
}

// The contig dictionary CHROM is looked up in: names[i] (lens[i] bytes) is
// contig i.  A name given twice keeps its first index.
extern "C" int frt_vcf_set_contigs(frt_vcf_decoder *d, const char *const *names, const size_t *lens, size_t n,
                                   frt_error *err)
{
    if (!d || (n && (!names || !lens)) || n >= 0x7fffffffu) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument or too many contigs");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(d->s.device);
    std::lock_guard<std::mutex> lk(d->s.mu);
    std::vector<u32> off(n + 1, 0);
    std::vector<u8> blob;
    for (size_t i = 0; i < n; ++i) {
        if (!names[i] && lens[i]) {
            set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "contig %zu has no name", i);
            return FRT_ERR_INVALID_ARGUMENT;
        }
        blob.insert(blob.end(), (const u8 *)names[i], (const u8 *)names[i] + lens[i]);
        if (blob.size() >= 0xffffffffull) {
            set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "contig names exceed 4 GiB");
            return FRT_ERR_INVALID_ARGUMENT;
        }
        off[i + 1] = (u32)blob.size();
    }
    u32 cap = 16;
    while (cap < 2 * n) cap <<= 1;
    std::vector<u32> slots(cap, 0);
    for (size_t i = 0; i < n; ++i) {
        const u8 *p = blob.data() + off[i];
        const u32 len = off[i + 1] - off[i];
        u32 s = fnv1a(p, len) & (cap - 1);
        bool dup = false;
        for (; slots[s]; s = (s + 1) & (cap - 1)) {
            const u32 j = slots[s] - 1;
            if (off[j + 1] - off[j] == len && std::memcmp(blob.data() + off[j], p, len) == 0) {
                dup = true;
                break;
            }
        }
        if (!dup) slots[s] = (u32)i + 1;
    }
    cudaStream_t st = d->s.stream;
    vcf_free_dict(d);
    int rc;
    if ((rc = dev_alloc((void **)&d->slots, 4 * slots.size(), st, err)) ||
        (rc = dev_alloc((void **)&d->name_off, 4 * off.size(), st, err)) ||
        (rc = dev_alloc((void **)&d->names, blob.size() + 1, st, err))) {
        vcf_free_dict(d);
        return rc;
    }
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d->slots, slots.data(), 4 * slots.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d->name_off, off.data(), 4 * off.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (blob.size() &&
         (e = cudaMemcpyAsync(d->names, blob.data(), blob.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        vcf_free_dict(d);
        return cuda_fail(err, e, "uploading the contig dictionary");
    }
    d->mask = cap - 1;
    d->n = (u32)n;
    return FRT_OK;
}

// The contigs of a VCF header: the ID of every "##contig=<...>" line, in
// order (the VCF 4.x meta-information structure; keys are comma-separated
// inside the angle brackets and the ID value runs to the next ',' or '>').
extern "C" int frt_vcf_set_contigs_from_header(frt_vcf_decoder *d, const uint8_t *text, size_t len, size_t *n_out,
                                               frt_error *err)
{
    if (!d || (len && !text)) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    static const char kPrefix[] = "##contig=<";
    const size_t kp = sizeof(kPrefix) - 1;
    std::vector<const char *> names;
    std::vector<size_t> lens;
    size_t i = 0;
    while (i < len) {
        size_t eol = i;
        while (eol < len && text[eol] != '\n') ++eol;
        if (eol - i > kp && std::memcmp(text + i, kPrefix, kp) == 0) {
            size_t k = i + kp;
            while (k < eol) {
                size_t ke = k;
                while (ke < eol && text[ke] != '=' && text[ke] != ',' && text[ke] != '>') ++ke;
                if (ke < eol && text[ke] == '=') {
                    size_t ve = ke + 1;
                    bool quoted = ve < eol && text[ve] == '"';
                    if (quoted) {
                        ++ve;
                        while (ve < eol && text[ve] != '"') ++ve;
                        if (ve < eol) ++ve;
                    }
                    while (ve < eol && text[ve] != ',' && text[ve] != '>') ++ve;
                    if (ke - k == 2 && text[k] == 'I' && text[k + 1] == 'D') {
                        names.push_back((const char *)text + ke + 1);
                        lens.push_back(ve - ke - 1);
                        break;
                    }
                    k = ve + 1;
                } else {
                    k = ke + 1;
                }
            }
        }
        i = eol + 1;
    }
    if (n_out) *n_out = names.size();
    return frt_vcf_set_contigs(d, names.data(), lens.data(), names.size(), err);
}

// Columns of the records of a text scan (frt_text_scan with the VCF dialect);
// the result holds the scan's batch alive.
extern "C" int frt_vcf_decode(frt_vcf_decoder *d, const frt_columns *text, frt_columns **out, frt_error *err)
{
    if (!d || !text || !out || text->format != FMT_TEXT) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument, or not the result of a text scan");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = d->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    if (text->device != s.device) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr, "text columns on device %d, decoder on %d",
                  text->device, s.device);
        return FRT_ERR_INVALID_DEVICE_BATCH;
    }
    cudaError_t e;
    if (text->ready && (e = cudaStreamWaitEvent(s.stream, text->ready, 0)) != cudaSuccess)
        return cuda_fail(err, e, "ordering after the text scan");
    const u64 n = text->n;
    frt_columns *c = columns_new(s, FMT_VCF, kVcfWidths, FRT_VCF_COL_COUNT, n);
    c->tail = text->tail;
    int rc = columns_alloc(c, err);
    if (rc) {
        columns_discard(c);
        return rc;
    }
    if (n) {
        const frt_columns *t = text;
        auto tcol = [&](int k) { return (const u64 *)(t->cols + t->col_off[k]); };
        VcfDict dict;
        dict.slots = d->slots;
        dict.name_off = d->name_off;
        dict.names = d->names;
        dict.mask = d->mask;
        dict.n = d->n;
        k_vcf_fields<<<grid_for(n, 256), 256, 0, s.stream>>>(
            text->source->data, text->source->len, tcol(FRT_TEXT_COL_RECORD_OFFSETS), tcol(FRT_TEXT_COL_RECORD_ENDS),
            tcol(FRT_TEXT_COL_TABS), tcol(FRT_TEXT_COL_FIELD_STARTS), n, dict, colp<int>(c, FRT_VCF_COL_CHROM),
            colp<u64>(c, FRT_VCF_COL_POS), colp<u32>(c, FRT_VCF_COL_BOUNDS), colp<u32>(c, FRT_VCF_COL_N_ALT),
            colp<u32>(c, FRT_VCF_COL_QUAL), colp<u16>(c, FRT_VCF_COL_FLAGS), colp<u8>(c, FRT_VCF_COL_STATUS));
        if ((e = cudaGetLastError()) != cudaSuccess) {
            columns_discard(c);
            return cuda_fail(err, e, "launching the VCF decode");
        }
    }
    return columns_finish(c, text->source, out);
}

// Every sample's GT of the records of `text` (an frt_text_scan result):
// column FRT_VCF_GT_COL_CALLS has one u32 per tab of the scan, the call of
// the sample that tab opens; FRT_VCF_GT_COL_KEY one i32 per record.
extern "C" int frt_vcf_genotypes(frt_vcf_decoder *d, const frt_columns *text, frt_columns **out, frt_error *err)
{
    if (!d || !text || !out || text->format != FMT_TEXT) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument, or not the result of a text scan");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    Scanner &s = d->s;
    DeviceGuardLite g(s.device);
    std::lock_guard<std::mutex> lk(s.mu);
    if (text->device != s.device) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr, "text columns on device %d, decoder on %d",
                  text->device, s.device);
        return FRT_ERR_INVALID_DEVICE_BATCH;
    }
    cudaError_t e;
    if (text->ready && (e = cudaStreamWaitEvent(s.stream, text->ready, 0)) != cudaSuccess)
        return cuda_fail(err, e, "ordering after the text scan");
    const u64 n = text->n, n_tabs = text->total;
    frt_columns *c = columns_new(s, FMT_VCF_GT, kVcfGtWidths, FRT_VCF_GT_COL_COUNT, n);
    c->tail = text->tail;
    c->total = n_tabs;
    c->col_bytes[FRT_VCF_GT_COL_CALLS] = 4 * n_tabs;
    size_t off = 0;
    for (int k = 0; k < FRT_VCF_GT_COL_COUNT; ++k) {
        c->col_off[k] = off;
        off += (c->col_bytes[k] + 255) & ~(size_t)255;
    }
    int rc = columns_alloc(c, err);
    if (rc) {
        columns_discard(c);
        return rc;
    }
    if (n) {
        const frt_columns *t = text;
        auto tcol = [&](int k) { return (const u64 *)(t->cols + t->col_off[k]); };
        // warps per record: a power of two that gives a lane at most eight
        // of the average record's samples, up to 16
        const u64 samples = n_tabs / n > 8 ? n_tabs / n - 8 : 0;
        u32 wl = 0;
        while (wl < 4 && (256ull << wl) < samples) ++wl;
        k_vcf_gt<<<grid_for((n << wl) * 32, 256), 256, 0, s.stream>>>(
            text->source->data, text->source->len, tcol(FRT_TEXT_COL_RECORD_OFFSETS), tcol(FRT_TEXT_COL_RECORD_ENDS),
            tcol(FRT_TEXT_COL_TABS), tcol(FRT_TEXT_COL_FIELD_STARTS), n, wl, colp<u32>(c, FRT_VCF_GT_COL_CALLS),
            colp<int>(c, FRT_VCF_GT_COL_KEY));
        if ((e = cudaGetLastError()) != cudaSuccess) {
            columns_discard(c);
            return cuda_fail(err, e, "launching the genotype decode");
        }
    }
    return columns_finish(c, text->source, out);
}
