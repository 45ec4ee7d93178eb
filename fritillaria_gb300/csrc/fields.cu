// Opt-in record fields on the device, over decoded BAM records.  The
// reference reads each of these on the host, one record at a time:
//
//   aux lookup        Record::aux_get (crates/fritillaria-bam/src/columnar/record.rs:286-294):
//                     the first field with the tag, or an error when the aux
//                     block is malformed before it.  Here every record at once,
//                     through the aux directory the decoder builds (which lists
//                     the fields up to the first malformed one).
//   resolved CIGAR    Record::has_long_cigar_placeholder / cigar_resolved
//                     (record.rs:316-357): two stored ops, a soft clip as long as
//                     the read then N, mean the real ops are CG's B:I array; a
//                     placeholder with no CG, or a CG of another type, is an error.
//   unpack_sequences  seq.rs decode_sequence: "=ACMGRSVTWYHKDBN"[nibble], high
//                     nibble first (docs/device-api.md:261-263: an opt-in kernel).
//   compact           the payload columns sketched in docs/device-api.md:250-256,
//                     filled from the Record accessors name (without its NUL),
//                     cigar_raw, sequence_packed, qualities, aux_raw
//                     (record.rs:222-270), so the inflated batch can be dropped.
//
// The payload copies take three launches: per-CTA byte counts, a scan of
// those counts, and one copy in which each CTA scans its records' lengths,
// writes their offsets into the result and stages every record's bytes in
// shared memory with 16-byte loads before consecutive lanes write them out.

#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.h"

using namespace frt;

namespace {

constexpr u32 kScanBlock = 1024;

// The payload copies.  compact fills five payloads -- the name without its
// NUL, CIGAR, packed sequence, qualities, aux -- from each record's bytes after
// its 36 fixed ones; unpack expands the packed sequence to one byte a base.
enum CopyMode { COPY_COMPACT = 0, COPY_BASES = 1 };
template <int MODE> __host__ __device__ constexpr int kinds() { return MODE == COPY_COMPACT ? 5 : 1; }
constexpr u32 kRoundRecords = 256; // records per round: one a thread, 32 a warp
constexpr u32 kRounds = 4;
constexpr u32 kBlockRecords = kRoundRecords * kRounds;

// A record's copy: its source bytes [src, src + cut[5]) and, relative to src,
// compact's payload bounds -- name [0, cut[0]), CIGAR [cut[1], cut[2]),
// sequence [cut[2], cut[3]), qualities [cut[3], cut[4]), aux [cut[4], cut[5])
// -- or, for unpack, the packed sequence with cut[0] = l_seq bases.
struct Span {
    u64 src;
    u32 cut[6];
    u8 *dst[5];
};

struct CopyOut {
    u64 *off[5];
    u8 *data[5];
};

__device__ __forceinline__ u64 record_span(const RecordView &v, u64 i, int mode, u32 cut[6])
{
    const u8 *p = v.buf + v.record_offsets[i];
    if (mode == COPY_BASES) {
        const u32 l = v.seq_len[i];
        cut[0] = l;
        cut[1] = cut[2] = cut[3] = cut[4] = 0;
        cut[5] = (l + 1u) >> 1;
        return (u64)(p + v.sequence_start[i]);
    }
    const u32 nl = v.name_len[i];
    cut[0] = nl && p[36u + nl - 1u] == 0 ? nl - 1u : nl; // Record::name strips the NUL
    cut[1] = v.cigar_start[i] - 36u;
    cut[2] = v.sequence_start[i] - 36u;
    cut[3] = v.quality_start[i] - 36u;
    cut[4] = v.aux_start[i] - 36u;
    cut[5] = v.record_end[i] - 36u;
    return (u64)(p + 36);
}

template <int MODE> __device__ __forceinline__ u32 payload_len(const u32 cut[6], int k)
{
    if (MODE == COPY_BASES || k == 0) return cut[0];
    return cut[k + 1] - cut[k];
}

// Exclusive scan of each kind's block totals, one CTA a kind, 1024 at a time:
// part[k * stride + b] for b < nb, the kind's total to part[k * stride + nb]
// and to totals[k].
__global__ void __launch_bounds__(kScanBlock) k_scan_parts(u64 *part, u64 nb, u64 stride, u64 *totals)
{
    __shared__ u64 warps[32];
    __shared__ u64 carry;
    part += blockIdx.x * stride;
    const u32 lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (u64 base = 0; base < nb; base += kScanBlock) {
        const u64 i = base + threadIdx.x;
        const u64 x = i < nb ? part[i] : 0ull;
        u64 s = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u64 y = __shfl_up_sync(FRT_FULL_MASK, s, d);
            if ((int)lane >= d) s += y;
        }
        if (lane == 31u) warps[w] = s;
        __syncthreads();
        if (w == 0) {
            u64 t = warps[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const u64 y = __shfl_up_sync(FRT_FULL_MASK, t, d);
                if ((int)lane >= d) t += y;
            }
            warps[lane] = t;
        }
        __syncthreads();
        const u64 before = w ? warps[w - 1] : 0ull;
        const u64 c = carry;
        if (i < nb) part[i] = c + before + s - x;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry = c + before + s;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[nb] = carry;
        totals[blockIdx.x] = carry;
    }
}

// Each CTA's payload bytes per kind, over its kBlockRecords records.
template <int MODE> __global__ void __launch_bounds__(kRoundRecords) k_fields_count(RecordView v, u64 *part, u64 stride)
{
    constexpr int K = kinds<MODE>();
    __shared__ u64 wsum[K][kRoundRecords / 32];
    const u32 lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    u64 s[K] = {};
    const u64 b0 = (u64)blockIdx.x * kBlockRecords;
    for (u32 q = 0; q < kRounds; ++q) {
        const u64 i = b0 + q * kRoundRecords + threadIdx.x;
        if (i < v.n) {
            u32 cut[6];
            record_span(v, i, MODE, cut);
#pragma unroll
            for (int k = 0; k < K; ++k) s[k] += payload_len<MODE>(cut, k);
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int d = 16; d; d >>= 1) s[k] += __shfl_down_sync(FRT_FULL_MASK, s[k], d);
        if (lane == 0) wsum[k][w] = s[k];
    }
    __syncthreads();
    if (threadIdx.x < (u32)K) {
        u64 t = 0;
        for (u32 j = 0; j < kRoundRecords / 32; ++j) t += wsum[threadIdx.x][j];
        part[threadIdx.x * stride + blockIdx.x] = t;
    }
}

// "=ACMGRSVTWYHKDBN"[nib], from two words instead of a table every lane
// indexes differently.
__device__ __forceinline__ u8 base_of(u32 nib)
{
    const u64 lo = 0x565352474D43413Dull; // "=ACMGRSV", byte k = base k
    const u64 hi = 0x4E42444B48595754ull; // "TWYHKDBN"
    const u64 w = nib < 8u ? lo : hi;
    return (u8)(w >> (8u * (nib & 7u)));
}

// Writes the record's bytes [lo, hi) to its payloads; in[r] is its byte r.
// pairs[b] holds the two bases of packed byte b, the high nibble's first.
template <int MODE>
__device__ __forceinline__ void emit(const Span &sp, const u8 *in, u32 lo, u32 hi, u32 lane, const u16 *pairs)
{
    if (MODE == COPY_BASES) {
        const u32 l = sp.cut[0];
        u8 *d = sp.dst[0];
        if (((uintptr_t)d & 1u) == 0) {
            for (u32 r = lo + lane; r < hi; r += 32u) {
                const u32 v = pairs[in[r]];
                if (2u * r + 1u < l)
                    *(u16 *)(d + 2u * r) = (u16)v;
                else
                    d[2u * r] = (u8)v;
            }
        } else {
            for (u32 r = lo + lane; r < hi; r += 32u) {
                const u32 v = pairs[in[r]];
                d[2u * r] = (u8)v;
                if (2u * r + 1u < l) d[2u * r + 1u] = (u8)(v >> 8);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const u32 sk = k ? sp.cut[k] : 0u, ek = k ? sp.cut[k + 1] : sp.cut[0];
            u8 *d = sp.dst[k];
            for (u32 r = max(sk, lo) + lane; r < min(ek, hi); r += 32u) d[r - sk] = in[r];
        }
    }
}

// A warp's 32 records.  Each turn gathers, into the warp's shared-memory
// stage, the aligned 16-byte blocks that hold the bytes of as many of the
// next records as fit in kStageBlocks -- every lane loads up to four blocks,
// all in flight together, each found by a binary search over the warp's
// prefix of per-record block counts -- then writes those records' payloads
// with consecutive lanes on consecutive bytes.  A record larger than a turn
// goes through in turns of its own.  The inflated buffers start 256-byte
// aligned and carry at least 16 bytes of padding past their last byte, so
// every aligned block that holds a record byte lies inside the allocation.
constexpr u32 kStageBlocks = 128;
constexpr u32 kStageLoads = kStageBlocks / 32;
constexpr u32 kBigSpan = 4096;  // records with more bytes go to k_fields_copy_big
constexpr u32 kPiece = 16384;   // a warp's share of such a record at a time (eight turns)

template <int MODE>
__device__ __forceinline__ void copy_spans(const Span *spans, u8 *stage, u32 lane, const u16 *pairs)
{
    const Span &mine = spans[lane];
    const u32 mo = (u32)(mine.src & 15u);
    const u64 mbase = mine.src - mo;
    const u32 mlen = mine.cut[5];
    // blocks of this lane's record, capped past a turn (such a record goes alone)
    const u32 nbk = mlen ? min((mo + mlen + 15u) >> 4, kStageBlocks + 1u) : 0u;
    u32 pre = nbk;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const u32 y = __shfl_up_sync(FRT_FULL_MASK, pre, d);
        if ((int)lane >= d) pre += y;
    }
    const u32 excl = pre - nbk;
    u32 j0 = 0;
    while (j0 < 32u) {
        const u32 base = __shfl_sync(FRT_FULL_MASK, excl, j0);
        const u32 fit = __ballot_sync(FRT_FULL_MASK, lane >= j0 && pre - base <= kStageBlocks);
        if (!((fit >> j0) & 1u)) { // record j0 alone is larger than a turn
            const Span &sp = spans[j0];
            const u32 len = sp.cut[5], o = (u32)(sp.src & 15u);
            const u8 *a0 = (const u8 *)(sp.src - o);
            for (u32 cb = 0; cb < len + o; cb += 16u * kStageBlocks) {
                uint4 v[kStageLoads];
#pragma unroll
                for (u32 h = 0; h < kStageLoads; ++h) {
                    const u32 blk = cb + 16u * (lane + 32u * h);
                    if (blk < len + o) v[h] = __ldg((const uint4 *)(a0 + blk));
                }
#pragma unroll
                for (u32 h = 0; h < kStageLoads; ++h)
                    if (cb + 16u * (lane + 32u * h) < len + o) *(uint4 *)(stage + 16u * (lane + 32u * h)) = v[h];
                __syncwarp();
                emit<MODE>(sp, stage + o - cb, cb > o ? cb - o : 0u, min(len, cb + 16u * kStageBlocks - o), lane, pairs);
                __syncwarp();
            }
            ++j0;
            continue;
        }
        const u32 j1 = 32u - __clz(fit); // one past the last record of this turn
        const u32 nb = __shfl_sync(FRT_FULL_MASK, pre, j1 - 1u) - base;
        uint4 v[kStageLoads];
#pragma unroll
        for (u32 h = 0; h < kStageLoads; ++h) {
            const u32 t = lane + 32u * h;
            // the first record j in [j0, j1) whose blocks end past t
            u32 lo = j0, hi = j1 - 1u;
#pragma unroll
            for (int step = 0; step < 5; ++step) {
                const u32 mid = (lo + hi) >> 1;
                if (__shfl_sync(FRT_FULL_MASK, pre, mid) - base > t)
                    hi = mid;
                else
                    lo = mid + 1u;
            }
            const u32 j = min(lo, 31u);
            const u32 first = __shfl_sync(FRT_FULL_MASK, excl, j) - base;
            const u64 at = __shfl_sync(FRT_FULL_MASK, mbase, j) + 16ull * (t - first);
            if (t < nb) v[h] = __ldg((const uint4 *)at);
        }
#pragma unroll
        for (u32 h = 0; h < kStageLoads; ++h)
            if (lane + 32u * h < nb) *(uint4 *)(stage + 16u * (lane + 32u * h)) = v[h];
        __syncwarp();
        for (u32 j = j0; j < j1; ++j) {
            const Span &sp = spans[j];
            const u32 first = __shfl_sync(FRT_FULL_MASK, excl, j) - base;
            if (sp.cut[5]) emit<MODE>(sp, stage + 16u * first + (u32)(sp.src & 15u), 0u, sp.cut[5], lane, pairs);
        }
        __syncwarp();
        j0 = j1;
    }
}

// Per round a thread reads one record's bounds; a CTA scan of the payload
// lengths, plus the CTA's prefix from k_scan_parts, gives the output offsets,
// written straight into the result; then each warp copies its 32 records.
template <int MODE> __global__ void __launch_bounds__(kRoundRecords, 4) k_fields_copy(RecordView v, const u64 *part,
                                                                                    u64 stride, CopyOut out, u64 *big,
                                                                                    u32 *big_count, u32 big_cap)
{
    constexpr int K = kinds<MODE>();
    __shared__ Span spans[kRoundRecords];
    __shared__ __align__(16) u8 stage[kRoundRecords / 32][16 * kStageBlocks];
    __shared__ u64 wsum[K][kRoundRecords / 32];
    __shared__ u64 carry[K]; // each kind's bytes before this round
    __shared__ u16 pairs[MODE == COPY_BASES ? 256 : 1];
    const u32 lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    if (MODE == COPY_BASES)
        for (u32 b = threadIdx.x; b < 256u; b += blockDim.x) pairs[b] = (u16)(base_of(b >> 4) | ((u32)base_of(b & 15u) << 8));
    const u64 b0 = (u64)blockIdx.x * kBlockRecords;
    if (threadIdx.x < (u32)K) carry[threadIdx.x] = part[threadIdx.x * stride + blockIdx.x];
    for (u32 q = 0; q < kRounds; ++q) {
        const u64 first = b0 + q * kRoundRecords;
        if (first >= v.n) break;
        const u64 i = first + threadIdx.x;
        const bool valid = i < v.n;
        u32 cut[6] = {0, 0, 0, 0, 0, 0};
        const u64 src = valid ? record_span(v, i, MODE, cut) : 0ull;
        u64 len[K], incl[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            len[k] = payload_len<MODE>(cut, k);
            u64 x = len[k];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const u64 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
                if ((int)lane >= d) x += y;
            }
            incl[k] = x;
            if (lane == 31u) wsum[k][w] = x;
        }
        __syncthreads();
        Span &sp = spans[threadIdx.x];
        u64 next_carry = 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            u64 before = 0, total = 0;
#pragma unroll
            for (u32 j = 0; j < kRoundRecords / 32; ++j) {
                const u64 t = wsum[k][j];
                before += j < w ? t : 0ull;
                total += t;
            }
            const u64 off = carry[k] + before + incl[k] - len[k];
            if (valid) {
                out.off[k][i] = off;
                if (i == v.n - 1) out.off[k][v.n] = off + len[k];
            }
            sp.dst[k] = out.data[k] + off;
            if (threadIdx.x == (u32)k) next_carry = carry[k] + total;
        }
        sp.src = src;
#pragma unroll
        for (int c = 0; c < 6; ++c) sp.cut[c] = cut[c];
        if (cut[5] > kBigSpan) { // k_fields_copy_big's, an empty span here
            const u32 np = ((u32)(src & 15u) + cut[5] + kPiece - 1u) / kPiece;
            const u32 slot = atomicAdd(big_count, np);
            for (u32 j = 0; j < np && slot + j < big_cap; ++j) big[slot + j] = ((u64)i << 20) | j;
            sp.cut[5] = 0;
        }
        __syncthreads();
        if (threadIdx.x < (u32)K) carry[threadIdx.x] = next_carry; // read again after the round's last barrier
        copy_spans<MODE>(spans + 32u * w, stage[w], lane, pairs);
        __syncthreads();
    }
}

__global__ void k_aux_lookup(RecordView v, u32 tag, u8 *status, u8 *type, u8 *subtype, u32 *count, long long *value,
                             u64 *offset)
{
    const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const u32 first = v.aux_first[i], nf = v.aux_count[i];
    u8 st = v.aux_status[i] ? 2 : 0, ty = 0, su = 0;
    u32 cn = 0;
    long long val = 0;
    u64 off = 0;
    for (u32 t = 0; t < nf; ++t) {
        const u32 *e = v.aux_entries + 3ull * (first + t);
        const u32 w0 = e[0];
        if ((w0 & 0xffffu) != tag) continue;
        ty = (u8)(w0 >> 16);
        su = (u8)(w0 >> 24);
        cn = e[2];
        const u64 at = v.record_offsets[i] + e[1];
        const u8 *p = v.buf + at;
        switch (ty) {
        case 'A': case 'C': val = p[0]; break;
        case 'c': val = (signed char)p[0]; break;
        case 's': val = (short)ld_u16le(p); break;
        case 'S': val = ld_u16le(p); break;
        case 'i': val = (int)ld_u32le(p); break;
        case 'I': case 'f': val = (long long)ld_u32le(p); break;
        default: break;
        }
        off = ty == 'B' ? at + 5u : at; // B: subtype byte, u32 count, then the elements
        st = 1;
        break;
    }
    status[i] = st;
    type[i] = ty;
    subtype[i] = su;
    count[i] = cn;
    value[i] = val;
    offset[i] = off;
}

__global__ void k_cigar_resolve(RecordView v, u64 *offset, u32 *ops, u8 *status)
{
    const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const u64 r = v.record_offsets[i];
    const u8 *p = v.buf + r;
    const u32 nc = v.n_cigar[i], cs = v.cigar_start[i];
    u64 off = r + cs;
    u32 n = nc;
    u8 st = 0;
    if (nc == 2u) {
        const u32 op0 = ld_u32le(p + cs), op1 = ld_u32le(p + cs + 4u);
        // "MIDNSHP=X": S is 4, N is 3; the clip must cover the whole read
        if ((op0 & 15u) == 4u && (op0 >> 4) == v.seq_len[i] && (op1 & 15u) == 3u) {
            st = 2;
            off = 0;
            n = 0;
            const u32 first = v.aux_first[i], nf = v.aux_count[i];
            for (u32 t = 0; t < nf; ++t) {
                const u32 *e = v.aux_entries + 3ull * (first + t);
                if ((e[0] & 0xffffu) != ('C' | ('G' << 8))) continue;
                if (((e[0] >> 16) & 0xffu) == 'B' && (e[0] >> 24) == 'I') {
                    st = 1;
                    off = r + e[1] + 5u;
                    n = e[2];
                }
                break;
            }
        }
    }
    offset[i] = off;
    ops[i] = n;
    status[i] = st;
}

// Records whose bytes pass kBigSpan, listed by k_fields_copy as pieces of
// kPiece bytes (record index << 20 | piece): each warp takes one piece at a
// time and copies its turns, so the work is shared out by bytes and no warp
// waits on another (a few reads of hundreds of kilobytes would otherwise hold
// one warp each while the rest of the GPU idles).
template <int MODE> __global__ void __launch_bounds__(kRoundRecords, 4)
    k_fields_copy_big(RecordView v, const u64 *big, const u32 *big_count, u32 big_cap, u32 *big_next, CopyOut out)
{
    constexpr int K = kinds<MODE>();
    constexpr u32 kTurn = 16u * kStageBlocks;
    __shared__ __align__(16) u8 stage[kRoundRecords / 32][kTurn];
    __shared__ u16 pairs[MODE == COPY_BASES ? 256 : 1];
    const u32 lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    if (MODE == COPY_BASES) {
        for (u32 b = threadIdx.x; b < 256u; b += blockDim.x) pairs[b] = (u16)(base_of(b >> 4) | ((u32)base_of(b & 15u) << 8));
        __syncthreads();
    }
    const u32 npieces = min(*big_count, big_cap);
    u8 *st = stage[w];
    for (;;) {
        u32 b = 0;
        if (lane == 0) b = atomicAdd(big_next, 1u);
        b = __shfl_sync(FRT_FULL_MASK, b, 0);
        if (b >= npieces) break;
        const u64 item = big[b];
        const u64 i = item >> 20;
        const u32 piece = (u32)(item & 0xfffffu);
        Span sp;
        sp.src = record_span(v, i, MODE, sp.cut);
#pragma unroll
        for (int k = 0; k < K; ++k) sp.dst[k] = out.data[k] + out.off[k][i];
        const u32 len = sp.cut[5], o = (u32)(sp.src & 15u);
        const u8 *a0 = (const u8 *)(sp.src - o);
        const u32 stop = min(len + o, (piece + 1u) * kPiece);
        for (u32 cb = piece * kPiece; cb < stop; cb += kTurn) {
            uint4 x[kStageLoads];
#pragma unroll
            for (u32 h = 0; h < kStageLoads; ++h) {
                const u32 blk = cb + 16u * (lane + 32u * h);
                if (blk < len + o) x[h] = __ldg((const uint4 *)(a0 + blk));
            }
#pragma unroll
            for (u32 h = 0; h < kStageLoads; ++h)
                if (cb + 16u * (lane + 32u * h) < len + o) *(uint4 *)(st + 16u * (lane + 32u * h)) = x[h];
            __syncwarp();
            emit<MODE>(sp, st + o - cb, cb > o ? cb - o : 0u, min(len, cb + kTurn - o), lane, pairs);
            __syncwarp();
        }
    }
}

// Work buffers of one call, freed on every return path.
struct Temp {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Temp(cudaStream_t s) : st(s) {}
    ~Temp()
    {
        for (void *p : ptrs) dev_free(p, st);
    }
    template <typename T> int get(T **p, size_t count, frt_error *err)
    {
        void *q = nullptr;
        int rc = dev_alloc(&q, count * sizeof(T) + 16, st, err);
        if (rc == FRT_OK) {
            ptrs.push_back(q);
            *p = (T *)q;
        }
        return rc;
    }
};

const size_t kAuxWidths[FRT_AUXV_COL_COUNT] = {1, 1, 1, 4, 8, 8};
const size_t kCigarWidths[FRT_CIGAR_COL_COUNT] = {8, 4, 1};
const size_t kBasesWidths[FRT_BASES_COL_COUNT] = {8, 1};
const size_t kCompactWidths[FRT_COMPACT_COL_COUNT] = {8, 1, 8, 4, 8, 1, 8, 1, 8, 1};

// Formats of the frt_columns these produce (after the scanners' 1-3).
enum { FMT_AUX_VALUES = 16, FMT_CIGAR = 17, FMT_BASES = 18, FMT_COMPACT = 19 };

size_t pad(size_t b) { return (b + 255) & ~(size_t)255; }

} // namespace

int frt::fields_run(const RecordView &v, int op, const char *tag, int device, cudaStream_t st, SharedStream *shared,
                    cudaEvent_t after, const frt_inflate_batch *retain, frt_columns **out, frt_error *err)
{
    if (!out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null output handle");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (op == FIELDS_AUX_LOOKUP && (!tag || !tag[0] || !tag[1])) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "an aux tag is two bytes");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e;
    if (after && (e = cudaStreamWaitEvent(st, after, 0)) != cudaSuccess) return cuda_fail(err, e, "ordering after the batch");
    const u64 n = v.n;
    Temp tmp(st);
    int rc;

    // Layout: the fixed columns first, then the payload columns whose sizes
    // come from scans.
    const size_t *widths = nullptr;
    int n_cols = 0, format = 0;
    size_t col_bytes[16] = {};
    int kinds = 0, mode = 0; // payloads copied: (offsets, data) column pairs
    switch (op) {
    case FIELDS_AUX_LOOKUP:
        widths = kAuxWidths, n_cols = FRT_AUXV_COL_COUNT, format = FMT_AUX_VALUES;
        for (int k = 0; k < n_cols; ++k) col_bytes[k] = widths[k] * n;
        break;
    case FIELDS_CIGAR_RESOLVED:
        widths = kCigarWidths, n_cols = FRT_CIGAR_COL_COUNT, format = FMT_CIGAR;
        for (int k = 0; k < n_cols; ++k) col_bytes[k] = widths[k] * n;
        break;
    case FIELDS_UNPACK_SEQUENCES:
        widths = kBasesWidths, n_cols = FRT_BASES_COL_COUNT, format = FMT_BASES;
        kinds = 1, mode = COPY_BASES;
        break;
    case FIELDS_COMPACT:
        widths = kCompactWidths, n_cols = FRT_COMPACT_COL_COUNT, format = FMT_COMPACT;
        kinds = 5, mode = COPY_COMPACT;
        break;
    default:
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "unknown record-field operation %d", op);
        return FRT_ERR_INVALID_ARGUMENT;
    }

    // Payload totals: per-CTA byte counts, their scan, the totals back to the
    // host to size the result.  The scanned counts stay for the copy.
    const u64 nb = (n + kBlockRecords - 1) / kBlockRecords, stride = nb + 1;
    u64 *part = nullptr;
    u64 totals[5] = {};
    if (kinds) {
        u64 *d_tot = nullptr;
        if ((rc = tmp.get(&part, kinds * stride, err)) || (rc = tmp.get(&d_tot, kinds, err))) return rc;
        if (n) {
            if (mode == COPY_BASES)
                k_fields_count<COPY_BASES><<<(unsigned)nb, kRoundRecords, 0, st>>>(v, part, stride);
            else
                k_fields_count<COPY_COMPACT><<<(unsigned)nb, kRoundRecords, 0, st>>>(v, part, stride);
            k_scan_parts<<<kinds, kScanBlock, 0, st>>>(part, nb, stride, d_tot);
            if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(err, e, "counting payload bytes");
            if ((e = cudaMemcpyAsync(totals, d_tot, 8 * kinds, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return cuda_fail(err, e, "reading payload totals");
        }
        for (int k = 0; k < kinds; ++k) {
            col_bytes[2 * k] = 8 * (n + 1);
            col_bytes[2 * k + 1] = totals[k];
        }
    }

    frt_columns *c = new frt_columns;
    c->device = device;
    c->format = format;
    c->stream = st;
    c->shared = stream_retain(shared);
    c->widths = widths;
    c->n_cols = n_cols;
    c->n = n;
    size_t total_bytes = 0;
    for (int k = 0; k < n_cols; ++k) {
        c->col_off[k] = total_bytes;
        c->col_bytes[k] = col_bytes[k];
        total_bytes += pad(col_bytes[k]);
    }
    auto fail = [&](int code) {
        dev_free(c->cols, st);
        stream_release(c->shared);
        delete c;
        return code;
    };
    if (total_bytes && (rc = dev_alloc((void **)&c->cols, total_bytes, st, err))) return fail(rc);
    auto col = [&](int k) { return c->cols + c->col_off[k]; };
    const unsigned tgrid = (unsigned)((n + 255) / 256);
    if (n) {
        switch (op) {
        case FIELDS_AUX_LOOKUP: {
            const u32 t16 = (u32)(u8)tag[0] | ((u32)(u8)tag[1] << 8);
            k_aux_lookup<<<tgrid, 256, 0, st>>>(v, t16, col(0), col(1), col(2), (u32 *)col(3), (long long *)col(4),
                                                (u64 *)col(5));
            break;
        }
        case FIELDS_CIGAR_RESOLVED:
            k_cigar_resolve<<<tgrid, 256, 0, st>>>(v, (u64 *)col(0), (u32 *)col(1), col(2));
            break;
        default: {
            CopyOut o{};
            for (int k = 0; k < kinds; ++k) {
                o.off[k] = (u64 *)col(2 * k);
                o.data[k] = col(2 * k + 1);
            }
            // A record past kBigSpan bytes holds at least kBigSpan payload bytes
            // (compact drops at most the name's NUL, so span <= payload + 1)
            // and splits into at most span / kPiece + 2 pieces: the list holds
            // at most payload / kPiece + 3 * records of them.
            u64 payload = 0;
            for (int k = 0; k < kinds; ++k) payload += totals[k];
            const u64 records = payload / kBigSpan + 1, cap64 = payload / kPiece + 3 * records + 2;
            const u32 cap = (u32)(cap64 < 0xffffffffull ? cap64 : 0xffffffffull);
            u64 *big = nullptr;
            u32 *counters = nullptr;
            int sms = 0;
            if ((rc = tmp.get(&big, cap, err)) || (rc = tmp.get(&counters, 2, err))) return fail(rc);
            if ((e = cudaMemsetAsync(counters, 0, 8, st)) != cudaSuccess ||
                (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
                return fail(cuda_fail(err, e, "preparing the payload copy"));
            if (mode == COPY_BASES) {
                k_fields_copy<COPY_BASES><<<(unsigned)nb, kRoundRecords, 0, st>>>(v, part, stride, o, big, counters, cap);
                k_fields_copy_big<COPY_BASES><<<(unsigned)sms * 4u, kRoundRecords, 0, st>>>(v, big, counters, cap,
                                                                                            counters + 1, o);
            } else {
                k_fields_copy<COPY_COMPACT><<<(unsigned)nb, kRoundRecords, 0, st>>>(v, part, stride, o, big, counters,
                                                                                   cap);
                k_fields_copy_big<COPY_COMPACT><<<(unsigned)sms * 4u, kRoundRecords, 0, st>>>(v, big, counters, cap,
                                                                                              counters + 1, o);
            }
        }
        }
    } else {
        for (int k = 0; k < kinds; ++k) // one offset, 0
            if ((e = cudaMemsetAsync(col(2 * k), 0, 8, st)) != cudaSuccess)
                return fail(cuda_fail(err, e, "placing payload offsets"));
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(cuda_fail(err, e, "launching record-field kernels"));
    if (op == FIELDS_UNPACK_SEQUENCES) c->total = totals[0];
    if ((e = cudaEventCreateWithFlags(&c->ready, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventRecord(c->ready, st)) != cudaSuccess)
        return fail(cuda_fail(err, e, "recording the result event"));
    if (retain && (op == FIELDS_AUX_LOOKUP || op == FIELDS_CIGAR_RESOLVED)) {
        const_cast<frt_inflate_batch *>(retain)->refs.fetch_add(1);
        c->source = retain;
    }
    *out = c;
    return FRT_OK;
}
