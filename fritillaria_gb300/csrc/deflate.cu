// BGZF compression on the device: the write side of the path.
//
// The reference's DeviceBlockCompressor (crates/fritillaria-core/src/device.rs:
// 326-372) compresses device-resident chunks into framed BGZF blocks that come
// back to the host (the small side), one block per chunk, no EOF block; its
// only implementation hands the deflate to nvCOMP and frames the result with
// kernels/bgzf_frame.cu, choosing the framing on the host
// (choose_framing/framed_size, crates/fritillaria-core/src/compress.rs:
// 100-142).  DeviceBgzfWriter (crates/fritillaria-bgzf/src/device_write.rs)
// batches chunks through it and appends the EOF block at the end.  The
// contract is a round trip, not byte identity: inflating the output must give
// back the input, block for block.
//
// Here the deflate is this library's own, a warp per chunk:
//   * CRC-32 of the chunk first, each lane over a slice from zero (lane 0 from
//     the initial register), combined by linearity (crc_shift);
//   * greedy LZ77 over a 32 KiB window with a hash table of the last position
//     of each 3-byte prefix in shared memory: each step the 32 lanes look up
//     the next 32 positions, the first lane whose candidate matches ends a run
//     of literals, the warp extends that match 32 bytes a compare, and every
//     position passed is entered in the table (atomicMax: the latest wins);
//   * the parse runs twice, identically: first counting its symbols, from
//     which lane 0 builds length-limited Huffman codes (RFC 1951 3.2.7) and
//     keeps them when they beat the fixed codes (3.2.6) header included; then
//     emitting one final block with the winner, the lanes' codes packed into
//     a shared-memory ring of words with a warp scan of their bit lengths and
//     flushed to the chunk's slot 64 words at a time.
// A stream longer than a BGZF block can carry stops early; the host then
// stores the chunk, as choose_framing does.

#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "runtime.h"

using namespace frt;

namespace {

constexpr u32 kMaxBlock = 65536;                         // MAX_BLOCK_SIZE
constexpr u32 kHeader = 18, kTrailer = 8, kStoredHeader = 5;
constexpr u32 kMaxDeflate = kMaxBlock - kHeader - kTrailer; // MAX_DEFLATE_STREAM
constexpr u32 kMaxPayload = kMaxDeflate - kStoredHeader;    // MAX_COMPRESSIBLE_PAYLOAD
constexpr u32 kSlot = 65536;                              // a chunk's deflate slot (bytes)
constexpr u32 kTooBig = 0xffffffffu;                      // a stream past kMaxDeflate
constexpr int kHashBits = 11;
constexpr u32 kWindow = 32768;
constexpr u32 kWarpsPerCta = 4;
constexpr u32 kRing = 128;  // words of the bit-packing ring
constexpr u32 kFlush = 64;  // words flushed at a time

enum Framing : u8 { FRAMING_DEFLATED = 0, FRAMING_STORED = 1, FRAMING_EMPTY = 2 };

struct ByteCrc {
    u32 t[256];
};
constexpr ByteCrc make_byte_crc()
{
    ByteCrc c{};
    for (u32 i = 0; i < 256; ++i) {
        u32 v = i;
        for (int k = 0; k < 8; ++k) v = (v >> 1) ^ (0xEDB88320u & (0u - (v & 1u)));
        c.t[i] = v;
    }
    return c;
}
__device__ const ByteCrc g_bcrc = make_byte_crc();

struct WarpState {
    // the hash table: the last position + 1 of each prefix hash (0 none);
    // between the passes, the Huffman builder's scratch
    u32 table[1u << kHashBits];
    u32 ring[kRing];
    u32 lf[286], df[30]; // literal/length and distance symbol counts of the parse
    u16 lcode[286], dcode[30], ccode[19]; // codes, reversed as they are packed
    u8 llen[286], dlen[30], clen[19];
    u16 items[320]; // the code lengths, run-length coded: symbol | extra value << 5
    u32 cf[19];     // counts of the code-length code's symbols
    u32 n_items, hlit, hdist, hclen, dynamic;
};
static_assert(sizeof(u32) * (1u << kHashBits) >= 4u * (512 + 1024) + 2u * 1024, "the builder's scratch fits");

__device__ __forceinline__ u32 prefix_hash(u32 b0, u32 b1, u32 b2)
{
    return (((b0 << 16) | (b1 << 8) | b2) * 2654435761u) >> (32 - kHashBits);
}

// A Huffman code as it is packed: the code reversed (deflate sends Huffman
// codes most significant bit first into a stream filled from the least
// significant bit), in the low bits.
__device__ __forceinline__ u32 rev(u32 code, u32 len) { return len ? __brev(code) >> (32u - len) : 0u; }

// Fixed literal/length code of symbol s (RFC 1951 3.2.6): (packed bits, length).
__device__ __forceinline__ void fixed_lit(u32 s, u32 *v, u32 *n)
{
    if (s < 144) *v = rev(0x30u + s, 8), *n = 8;
    else if (s < 256) *v = rev(0x190u + (s - 144u), 9), *n = 9;
    else if (s < 280) *v = rev(s - 256u, 7), *n = 7;
    else *v = rev(0xC0u + (s - 280u), 8), *n = 8;
}

// The length symbol of a match length (3..258) with its extra bits (RFC 1951 3.2.5).
__device__ __forceinline__ void len_sym(u32 L, u32 *sym, u32 *ex, u32 *nb)
{
    if (L == 258) {
        *sym = 285, *ex = 0, *nb = 0;
    } else if (L <= 10) {
        *sym = 254u + L, *ex = 0, *nb = 0;
    } else {
        const u32 x = L - 3u, k = 31u - __clz(x), hi = (x >> (k - 2u)) & 3u;
        *sym = 257u + 4u * (k - 1u) + hi;
        *nb = k - 2u;
        *ex = L - (3u + ((4u | hi) << (k - 2u)));
    }
}

// The distance symbol of a distance (1..32768) with its extra bits.
__device__ __forceinline__ void dist_sym(u32 d, u32 *sym, u32 *ex, u32 *nb)
{
    const u32 y = d - 1u;
    if (y < 4u) {
        *sym = y, *ex = 0, *nb = 0;
    } else {
        const u32 k = 31u - __clz(y), hi = (y >> (k - 1u)) & 1u;
        *sym = 2u * k + hi;
        *nb = k - 1u;
        *ex = d - (1u + ((2u | hi) << (k - 1u)));
    }
}

// Adds each lane's (v, n), n <= 31, at bit `bitpos` + the bits of the lanes
// below it; returns the new bit position (warp-uniform).
__device__ __forceinline__ u32 pack(WarpState *ws, u32 bitpos, u32 v, u32 n, u32 lane)
{
    u32 x = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const u32 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
        if (lane >= (u32)d) x += y;
    }
    const u32 total = __shfl_sync(FRT_FULL_MASK, x, 31);
    if (n) {
        const u32 o = bitpos + x - n, w = o >> 5, sh = o & 31u;
        atomicOr(&ws->ring[w % kRing], v << sh);
        if (sh + n > 32u) atomicOr(&ws->ring[(w + 1u) % kRing], v >> (32u - sh));
    }
    __syncwarp();
    return bitpos + total;
}

// Writes the ring's words [from, to) to the slot and clears them.
__device__ __forceinline__ void flush(WarpState *ws, u32 *slot, u32 from, u32 to, u32 lane)
{
    for (u32 w = from + lane; w < to; w += 32u) {
        slot[w] = ws->ring[w % kRing];
        ws->ring[w % kRing] = 0;
    }
    __syncwarp();
}

__device__ __forceinline__ u32 byte_at(const u8 *p, u32 i, u32 len) { return i < len ? p[i] : 0u; }

enum PassMode { COUNT = 0, EMIT_FIXED = 1, EMIT_DYNAMIC = 2 };

// One pass of the greedy parse over the chunk (the same parse every time: the
// table starts empty and atomicMax makes its contents order-free).  COUNT
// tallies the symbols; the EMIT modes pack their codes, a match as two groups
// (length, distance) of at most 20 and 28 bits.  Returns false when the
// stream outgrows a BGZF block.
template <int MODE>
__device__ bool lz_pass(WarpState *ws, const u8 *p, u32 len, u32 lane, u32 *slot, u32 &bitpos, u32 &flushed)
{
    for (u32 i = lane; i < (1u << kHashBits); i += 32u) ws->table[i] = 0;
    __syncwarp();
    u32 pos = 0;
    while (pos < len) {
        const u32 q = pos + lane;
        const u32 b0 = byte_at(p, q, len), b1 = byte_at(p, q + 1u, len), b2 = byte_at(p, q + 2u, len);
        const bool has3 = q + 3u <= len;
        const u32 h = prefix_hash(b0, b1, b2);
        const u32 e = has3 ? ws->table[h] : 0u;
        bool ok = false;
        u32 c = 0;
        if (e) {
            c = e - 1u;
            ok = q - c <= kWindow && p[c] == b0 && p[c + 1u] == b1 && p[c + 2u] == b2;
        }
        const u32 hits = __ballot_sync(FRT_FULL_MASK, ok);
        const u32 k = hits ? (u32)__ffs(hits) - 1u : 32u;
        const u32 nlit = min(k, len - pos);
        u32 L = 0, dist = 0;
        if (k < 32u) {
            const u32 m = pos + k, cm = __shfl_sync(FRT_FULL_MASK, c, k);
            const u32 cap = min(258u, len - m);
            L = 3u;
            while (L < cap) {
                const u32 i = L + lane;
                const bool diff = i >= cap || p[cm + i] != p[m + i];
                const u32 db = __ballot_sync(FRT_FULL_MASK, diff);
                if (db) {
                    L += (u32)__ffs(db) - 1u;
                    break;
                }
                L += 32u;
            }
            L = min(L, cap);
            dist = m - cm;
        }
        u32 ls = 0, lex = 0, lnb = 0, ds = 0, dex = 0, dnb = 0;
        if (lane == k && L) {
            len_sym(L, &ls, &lex, &lnb);
            dist_sym(dist, &ds, &dex, &dnb);
        }
        if (MODE == COUNT) {
            if (lane < nlit) atomicAdd(&ws->lf[b0], 1u);
            if (lane == k && L) {
                atomicAdd(&ws->lf[ls], 1u);
                atomicAdd(&ws->df[ds], 1u);
            }
        } else {
            u32 v = 0, nb = 0, v2 = 0, nb2 = 0;
            if (lane < nlit) {
                if (MODE == EMIT_FIXED) fixed_lit(b0, &v, &nb);
                else v = ws->lcode[b0], nb = ws->llen[b0];
            } else if (lane == k && L) {
                if (MODE == EMIT_FIXED) {
                    fixed_lit(ls, &v, &nb);
                    v2 = rev(ds, 5), nb2 = 5;
                } else {
                    v = ws->lcode[ls], nb = ws->llen[ls];
                    v2 = ws->dcode[ds], nb2 = ws->dlen[ds];
                }
                v |= lex << nb;
                nb += lnb;
                v2 |= dex << nb2;
                nb2 += dnb;
            }
            bitpos = pack(ws, bitpos, v, nb, lane);
            if (k < 32u && L) bitpos = pack(ws, bitpos, v2, nb2, lane);
        }
        if (lane < nlit && has3) atomicMax(&ws->table[h], q + 1u);
        const u32 adv = nlit + L;
        for (u32 j = nlit + lane; j < adv; j += 32u) {
            const u32 r = pos + j;
            if (r + 3u <= len) atomicMax(&ws->table[prefix_hash(p[r], p[r + 1u], p[r + 2u])], r + 1u);
        }
        __syncwarp();
        pos += adv;
        if (MODE != COUNT) {
            if ((bitpos >> 3) > kMaxDeflate) return false;
            const u32 done = bitpos >> 5;
            if (done - flushed >= kFlush) {
                flush(ws, slot, flushed, flushed + kFlush, lane);
                flushed += kFlush;
            }
        }
    }
    return true;
}

// Code lengths of a Huffman code for freq[0, n), at most maxlen bits: the
// used symbols (at least two; the lowest unused ones get a count of 1) sorted
// by (count, symbol) with a warp bitonic sort, a two-queue Huffman merge,
// the lengths past maxlen folded in by the Kraft sum (each excess leaf moves
// one shorter code a level down), and the shortest codes to the most frequent
// symbols.  Scratch: keys[512], wt[1024], parent[1024] (u16).
__device__ void huff_lengths(u32 *freq, u32 n, u32 maxlen, u8 *lens, u32 *keys, u32 *wt, u16 *parent, u32 lane)
{
    if (lane == 0) {
        u32 used = 0;
        for (u32 s = 0; s < n; ++s) used += freq[s] ? 1u : 0u;
        for (u32 s = 0; s < n && used < 2u; ++s)
            if (!freq[s]) freq[s] = 1u, ++used;
    }
    __syncwarp();
    for (u32 i = lane; i < 512u; i += 32u) keys[i] = i < n && freq[i] ? (freq[i] << 9) | i : 0xffffffffu;
    for (u32 i = lane; i < n; i += 32u) lens[i] = 0;
    __syncwarp();
    for (u32 size = 2; size <= 512u; size <<= 1)
        for (u32 stride = size >> 1; stride; stride >>= 1) {
            for (u32 t = lane; t < 256u; t += 32u) {
                const u32 i = 2u * t - (t & (stride - 1u)), j = i + stride;
                const bool up = (i & size) == 0;
                const u32 a = keys[i], b = keys[j];
                if ((a > b) == up) keys[i] = b, keys[j] = a;
            }
            __syncwarp();
        }
    if (lane == 0) {
        u32 m = 0;
        while (m < 512u && keys[m] != 0xffffffffu) ++m;
        for (u32 i = 0; i < m; ++i) wt[i] = keys[i] >> 9;
        u32 li = 0, ii = m, nxt = m;
        while (nxt < 2u * m - 1u) {
            u32 pick[2];
            for (int t = 0; t < 2; ++t) {
                if (li < m && (ii >= nxt || wt[li] <= wt[ii])) pick[t] = li++;
                else pick[t] = ii++;
            }
            wt[nxt] = wt[pick[0]] + wt[pick[1]];
            parent[pick[0]] = parent[pick[1]] = (u16)nxt;
            ++nxt;
        }
        // depths, root first; wt[] now holds them
        wt[2u * m - 2u] = 0;
        for (int i = (int)(2u * m) - 3; i >= 0; --i) wt[i] = wt[parent[i]] + 1u;
        u32 cnt[16] = {};
        for (u32 i = 0; i < m; ++i) ++cnt[min(wt[i], maxlen)];
        u32 total = 0;
        for (u32 L = 1; L <= maxlen; ++L) total += cnt[L] << (maxlen - L);
        while (total > (1u << maxlen)) {
            --cnt[maxlen];
            for (u32 L = maxlen - 1u; L > 0; --L)
                if (cnt[L]) {
                    --cnt[L];
                    cnt[L + 1u] += 2u;
                    break;
                }
            --total;
        }
        u32 k = m; // keys[m - 1] is the most frequent
        for (u32 L = 1; L <= maxlen; ++L)
            for (u32 c = 0; c < cnt[L]; ++c) lens[keys[--k] & 511u] = (u8)L;
    }
    __syncwarp();
}

// Canonical codes of lens[0, n) (RFC 1951 3.2.2), reversed for packing.
__device__ void canonical(const u8 *lens, u32 n, u16 *codes)
{
    u32 bl[16] = {}, next[16];
    for (u32 s = 0; s < n; ++s) ++bl[lens[s]];
    bl[0] = 0;
    u32 code = 0;
    for (u32 b = 1; b < 16; ++b) {
        code = (code + bl[b - 1]) << 1;
        next[b] = code;
    }
    for (u32 s = 0; s < n; ++s)
        if (lens[s]) codes[s] = (u16)rev(next[lens[s]]++, lens[s]);
}

__device__ const u8 kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

__device__ __forceinline__ u32 fixed_len(u32 s) { return s < 144 ? 8u : s < 256 ? 9u : s < 280 ? 7u : 8u; }
__device__ __forceinline__ u32 cl_extra(u32 sym) { return sym == 16 ? 2u : sym == 17 ? 3u : sym == 18 ? 7u : 0u; }

// The dynamic trees from the counts (lf[256] counts the end of block), and
// whether they beat the fixed codes, their header included (the extra bits
// of lengths and distances are the same either way).
__device__ void build_trees(WarpState *ws, u32 lane)
{
    u32 *keys = ws->table, *wt = ws->table + 512;
    u16 *parent = (u16 *)(ws->table + 1536);
    huff_lengths(ws->lf, 286, 15, ws->llen, keys, wt, parent, lane);
    huff_lengths(ws->df, 30, 15, ws->dlen, keys, wt, parent, lane);
    if (lane == 0) {
        u32 hlit = 286;
        while (hlit > 257 && !ws->llen[hlit - 1]) --hlit;
        u32 hdist = 30;
        while (hdist > 1 && !ws->dlen[hdist - 1]) --hdist;
        // run-length code the lengths (RFC 1951 3.2.7): 16 repeats the previous
        // length 3-6 times, 17 and 18 are runs of 3-10 and 11-138 zeros
        const u32 total = hlit + hdist;
        u32 n = 0, i = 0;
        while (i < total) {
            const u32 v = i < hlit ? ws->llen[i] : ws->dlen[i - hlit];
            u32 j = i;
            while (j < total && (j < hlit ? ws->llen[j] : ws->dlen[j - hlit]) == v) ++j;
            u32 run = j - i;
            if (v == 0) {
                while (run >= 11) {
                    const u32 r = min(run, 138u);
                    ws->items[n++] = (u16)(18u | ((r - 11u) << 5));
                    run -= r;
                }
                if (run >= 3) {
                    ws->items[n++] = (u16)(17u | ((run - 3u) << 5));
                    run = 0;
                }
                while (run--) ws->items[n++] = 0;
            } else {
                ws->items[n++] = (u16)v;
                --run;
                while (run >= 3) {
                    const u32 r = min(run, 6u);
                    ws->items[n++] = (u16)(16u | ((r - 3u) << 5));
                    run -= r;
                }
                while (run--) ws->items[n++] = (u16)v;
            }
            i = j;
        }
        ws->n_items = n;
        ws->hlit = hlit;
        ws->hdist = hdist;
        for (u32 t = 0; t < 19; ++t) ws->cf[t] = 0;
        for (u32 t = 0; t < n; ++t) ++ws->cf[ws->items[t] & 31u];
    }
    __syncwarp();
    huff_lengths(ws->cf, 19, 7, ws->clen, keys, wt, parent, lane);
    if (lane == 0) {
        u32 hclen = 19;
        while (hclen > 4 && !ws->clen[kClOrder[hclen - 1]]) --hclen;
        ws->hclen = hclen;
        canonical(ws->llen, 286, ws->lcode);
        canonical(ws->dlen, 30, ws->dcode);
        canonical(ws->clen, 19, ws->ccode);
        u64 dyn = 17u + 3u * hclen, fix = 3;
        for (u32 t = 0; t < ws->n_items; ++t) {
            const u32 sym = ws->items[t] & 31u;
            dyn += ws->clen[sym] + cl_extra(sym);
        }
        for (u32 sy = 0; sy < 286; ++sy) {
            dyn += (u64)ws->lf[sy] * ws->llen[sy];
            fix += (u64)ws->lf[sy] * fixed_len(sy);
        }
        for (u32 d = 0; d < 30; ++d) {
            dyn += (u64)ws->df[d] * ws->dlen[d];
            fix += (u64)ws->df[d] * 5u;
        }
        ws->dynamic = dyn < fix ? 1u : 0u;
    }
    __syncwarp();
}

__device__ __forceinline__ void flush_some(WarpState *ws, u32 *slot, u32 bitpos, u32 &flushed, u32 lane)
{
    if ((bitpos >> 5) - flushed >= kFlush) {
        flush(ws, slot, flushed, flushed + kFlush, lane);
        flushed += kFlush;
    }
}

__global__ void __launch_bounds__(32 * kWarpsPerCta) k_deflate_chunks(const u8 *data, const u64 *bounds, u32 n,
                                                                      u8 *slots, u32 *deflate_len, u32 *crcs)
{
    __shared__ WarpState states[kWarpsPerCta];
    const u32 lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    const u32 chunk = blockIdx.x * kWarpsPerCta + wi;
    if (chunk >= n) return;
    WarpState *ws = &states[wi];
    const u8 *p = data + bounds[chunk];
    const u32 len = (u32)(bounds[chunk + 1] - bounds[chunk]);

    // CRC-32: lane slices from zero, shifted past the bytes after them
    {
        const u32 s = (len + 31u) / 32u, b0 = min(len, lane * s), b1 = min(len, b0 + s);
        u32 c = lane == 0 ? 0xffffffffu : 0u;
        for (u32 i = b0; i < b1; ++i) c = g_bcrc.t[(c ^ p[i]) & 0xffu] ^ (c >> 8);
        c = crc_shift(c, len - b1);
#pragma unroll
        for (int d = 16; d; d >>= 1) c ^= __shfl_xor_sync(FRT_FULL_MASK, c, d);
        if (lane == 0) crcs[chunk] = ~c;
    }
    if (len == 0) {
        if (lane == 0) deflate_len[chunk] = 0;
        return;
    }
    for (u32 i = lane; i < kRing; i += 32u) ws->ring[i] = 0;
    for (u32 i = lane; i < 286u; i += 32u) ws->lf[i] = 0;
    if (lane < 30u) ws->df[lane] = 0;
    __syncwarp();
    u32 *slot = (u32 *)(slots + (size_t)chunk * kSlot);
    u32 bitpos = 0, flushed = 0;
    lz_pass<COUNT>(ws, p, len, lane, slot, bitpos, flushed); // the counts only
    if (lane == 0) ws->lf[256] += 1u;                          // the end of block
    __syncwarp();
    build_trees(ws, lane);
    const bool dyn = ws->dynamic != 0;
    bitpos = 0;
    if (!dyn) {
        bitpos = pack(ws, 0, 3u, lane == 0 ? 3u : 0u, lane); // BFINAL 1, BTYPE 01
    } else {
        // BFINAL 1, BTYPE 10, HLIT, HDIST, HCLEN; the code-length code's lengths
        // in their permuted order; the run-length coded lengths
        const u32 h = 1u | (2u << 1) | ((ws->hlit - 257u) << 3) | ((ws->hdist - 1u) << 8) | ((ws->hclen - 4u) << 13);
        bitpos = pack(ws, 0, lane == 0 ? h : 0u, lane == 0 ? 17u : 0u, lane);
        bitpos = pack(ws, bitpos, lane < ws->hclen ? ws->clen[kClOrder[lane]] : 0u, lane < ws->hclen ? 3u : 0u, lane);
        for (u32 base = 0; base < ws->n_items; base += 32u) {
            const u32 i = base + lane;
            u32 v = 0, nb = 0;
            if (i < ws->n_items) {
                const u32 it = ws->items[i], sym = it & 31u;
                v = ws->ccode[sym] | ((it >> 5) << ws->clen[sym]);
                nb = ws->clen[sym] + cl_extra(sym);
            }
            bitpos = pack(ws, bitpos, v, nb, lane);
            flush_some(ws, slot, bitpos, flushed, lane);
        }
    }
    bool ok = dyn ? lz_pass<EMIT_DYNAMIC>(ws, p, len, lane, slot, bitpos, flushed)
                  : lz_pass<EMIT_FIXED>(ws, p, len, lane, slot, bitpos, flushed);
    if (ok) {
        const u32 v = dyn ? ws->lcode[256] : 0u, nb = dyn ? ws->llen[256] : 7u; // the end of block
        bitpos = pack(ws, bitpos, lane == 0 ? v : 0u, lane == 0 ? nb : 0u, lane);
        ok = ((bitpos + 7u) >> 3) <= kMaxDeflate;
    }
    if (!ok) {
        if (lane == 0) deflate_len[chunk] = kTooBig;
        return;
    }
    flush(ws, slot, flushed, (bitpos + 31u) >> 5, lane);
    if (lane == 0) deflate_len[chunk] = (bitpos + 7u) >> 3;
}

// One CTA per block: the gzip header with the BC subfield, the body
// (deflated, stored or the empty stream) and CRC32 + ISIZE, at out_offsets[i].
__global__ void k_frame_blocks(const u8 *slots, const u32 *deflate_len, const u8 *data, const u64 *bounds,
                               const u32 *crcs, const u8 *framing, const u64 *out_offsets, u8 *out, u32 n)
{
    const u32 i = blockIdx.x;
    if (i >= n) return;
    u8 *b = out + out_offsets[i];
    const u32 size = (u32)(out_offsets[i + 1] - out_offsets[i]);
    const u32 raw = (u32)(bounds[i + 1] - bounds[i]);
    const u8 how = framing[i];
    if (threadIdx.x == 0) {
        const u8 h[16] = {0x1f, 0x8b, 8, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, 'B', 'C', 2, 0};
        for (int k = 0; k < 16; ++k) b[k] = h[k];
        b[16] = (u8)((size - 1u) & 0xffu);
        b[17] = (u8)((size - 1u) >> 8);
        u8 *t = b + size - kTrailer;
        const u32 c = crcs[i];
        for (int k = 0; k < 4; ++k) t[k] = (u8)(c >> (8 * k));
        for (int k = 0; k < 4; ++k) t[4 + k] = (u8)(raw >> (8 * k));
        if (how == FRAMING_EMPTY) {
            b[kHeader] = 0x03;
            b[kHeader + 1] = 0x00;
        } else if (how == FRAMING_STORED) {
            u8 *s = b + kHeader;
            s[0] = 0x01; // BFINAL 1, BTYPE 00
            s[1] = (u8)(raw & 0xffu);
            s[2] = (u8)(raw >> 8);
            s[3] = (u8)(~raw & 0xffu);
            s[4] = (u8)((~raw >> 8) & 0xffu);
        }
    }
    if (how == FRAMING_DEFLATED) {
        const u8 *src = slots + (size_t)i * kSlot;
        const u32 dl = deflate_len[i];
        for (u32 k = threadIdx.x; k < dl; k += blockDim.x) b[kHeader + k] = src[k];
    } else if (how == FRAMING_STORED) {
        const u8 *src = data + bounds[i];
        for (u32 k = threadIdx.x; k < raw; k += blockDim.x) b[kHeader + kStoredHeader + k] = src[k];
    }
}

} // namespace

struct frt_compressor {
    int device = 0;
    SharedStream *shared = nullptr;
    cudaStream_t stream = nullptr;
    std::mutex mu;
};

extern "C" int frt_compressor_create(int device, void *stream, frt_compressor **out, frt_error *err)
{
    if (!out) return FRT_ERR_INVALID_ARGUMENT;
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuardLite g(device);
    configure_pool(device);
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    frt_compressor *c = new frt_compressor;
    c->device = device;
    c->shared = ss;
    c->stream = ss->s;
    *out = c;
    return FRT_OK;
}

extern "C" void frt_compressor_destroy(frt_compressor *c)
{
    if (!c) return;
    stream_release(c->shared);
    delete c;
}

extern "C" const char *frt_compressor_name(const frt_compressor *) { return "gb300-deflate"; }

extern "C" int frt_compressor_device_ordinal(const frt_compressor *c) { return c ? c->device : -1; }

// choose_framing (compress.rs:115-128) and framed_size (compress.rs:134-142).
extern "C" int frt_choose_framing(size_t payload_len, size_t deflate_len)
{
    if (payload_len == 0) return FRAMING_EMPTY;
    if (deflate_len > kMaxDeflate || deflate_len > payload_len + kStoredHeader) return FRAMING_STORED;
    return FRAMING_DEFLATED;
}

extern "C" size_t frt_framed_size(size_t payload_len, size_t deflate_len)
{
    const int how = frt_choose_framing(payload_len, deflate_len);
    const size_t body = how == FRAMING_DEFLATED ? deflate_len : how == FRAMING_STORED ? payload_len + kStoredHeader : 2;
    return kHeader + body + kTrailer;
}

extern "C" size_t frt_compress_bound(size_t n_chunks) { return n_chunks * (size_t)kMaxBlock; }

// DeviceBlockCompressor::compress_batch_device (device.rs:357-371): each
// range bounds[i]..bounds[i + 1] of the device bytes becomes one framed block,
// written to the host buffer `out` (out_offsets[i] .. out_offsets[i + 1]); no
// EOF block.  The ranges need not cover the buffer.
extern "C" int frt_compress_batch_device(frt_compressor *cp, const uint8_t *data, size_t data_len,
                                         const uint64_t *bounds, size_t n_bounds, uint8_t *out, size_t out_cap,
                                         uint64_t *out_offsets, size_t *out_len, frt_error *err)
{
    if (!cp || !bounds || n_bounds == 0 || (n_bounds > 1 && (!data || !out || !out_offsets))) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument or no bounds");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    const size_t n = n_bounds - 1;
    for (size_t i = 0; i < n; ++i) {
        if (bounds[i + 1] < bounds[i] || bounds[i + 1] > data_len || bounds[i + 1] - bounds[i] > kMaxPayload) {
            set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, bounds[i], "bgzf",
                      "chunk %zu is [%llu, %llu): bounds must rise, stay within the %zu device bytes and hold at "
                      "most %u bytes",
                      i, (unsigned long long)bounds[i], (unsigned long long)bounds[i + 1], data_len, kMaxPayload);
            return FRT_ERR_MALFORMED;
        }
    }
    if (out_offsets) out_offsets[0] = 0;
    if (out_len) *out_len = 0;
    if (n == 0) return FRT_OK;
    if (n >= 0xffffffffull) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "too many chunks");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(cp->device);
    std::lock_guard<std::mutex> lk(cp->mu);
    cudaStream_t st = cp->stream;
    const size_t work = 8 * (n + 1) + 4 * n + 4 * n + (size_t)kSlot * n;
    u8 *w = nullptr;
    int rc = dev_alloc((void **)&w, work + 64, st, err);
    if (rc) return rc;
    u64 *d_bounds = (u64 *)w;
    u32 *d_len = (u32 *)(w + 8 * (n + 1));
    u32 *d_crc = d_len + n;
    u8 *d_slots = (u8 *)(d_crc + n) + ((64 - ((uintptr_t)(d_crc + n) & 63)) & 63);
    std::vector<u32> lens(n);
    cudaError_t e;
    auto fail = [&](cudaError_t ce, const char *what) {
        dev_free(w, st);
        return cuda_fail(err, ce, what);
    };
    if ((e = cudaMemcpyAsync(d_bounds, bounds, 8 * (n + 1), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail(e, "uploading the chunk bounds");
    k_deflate_chunks<<<(unsigned)((n + kWarpsPerCta - 1) / kWarpsPerCta), 32 * kWarpsPerCta, 0, st>>>(
        data, d_bounds, (u32)n, d_slots, d_len, d_crc);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "launching the deflate");
    if ((e = cudaMemcpyAsync(lens.data(), d_len, 4 * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(e, "reading the deflate sizes");
    // the framing and the dense layout, decided on the host as the reference does
    std::vector<u64> offs(n + 1, 0);
    std::vector<u8> framing(n);
    for (size_t i = 0; i < n; ++i) {
        const size_t raw = bounds[i + 1] - bounds[i];
        const size_t dl = lens[i] == kTooBig ? (size_t)kMaxDeflate + 1 : lens[i];
        framing[i] = (u8)frt_choose_framing(raw, dl);
        offs[i + 1] = offs[i] + frt_framed_size(raw, dl);
    }
    if (offs[n] > out_cap) {
        dev_free(w, st);
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, offs[n], out_cap, 0, nullptr,
                  "the %zu framed blocks take %llu bytes; the output holds %zu", n, (unsigned long long)offs[n],
                  out_cap);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    u8 *d_out = nullptr, *d_meta = nullptr;
    if ((rc = dev_alloc((void **)&d_out, offs[n] + 16, st, err)) ||
        (rc = dev_alloc((void **)&d_meta, 8 * (n + 1) + n + 16, st, err))) {
        dev_free(d_out, st);
        dev_free(w, st);
        return rc;
    }
    u64 *d_offs = (u64 *)d_meta;
    u8 *d_framing = d_meta + 8 * (n + 1);
    auto fail2 = [&](cudaError_t ce, const char *what) {
        dev_free(d_meta, st);
        dev_free(d_out, st);
        return fail(ce, what);
    };
    if ((e = cudaMemcpyAsync(d_offs, offs.data(), 8 * (n + 1), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_framing, framing.data(), n, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail2(e, "uploading the framing");
    k_frame_blocks<<<(unsigned)n, 256, 0, st>>>(d_slots, d_len, data, d_bounds, d_crc, d_framing, d_offs, d_out,
                                                (u32)n);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail2(e, "launching the framing");
    if ((e = cudaMemcpyAsync(out, d_out, offs[n], cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail2(e, "reading the blocks back");
    dev_free(d_meta, st);
    dev_free(d_out, st);
    dev_free(w, st);
    std::memcpy(out_offsets, offs.data(), 8 * (n + 1));
    if (out_len) *out_len = offs[n];
    return FRT_OK;
}

// ---- DeviceBgzfWriter (crates/fritillaria-bgzf/src/device_write.rs) ----------

namespace {
// The 28-byte BGZF end-of-file block (crates/fritillaria-bgzf/src/block.rs:40-43).
const uint8_t kEofBlock[28] = {0x1f, 0x8b, 8, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, 'B', 'C', 2, 0,
                               0x1b, 0, 3, 0, 0, 0, 0, 0, 0, 0, 0, 0};
} // namespace

struct frt_bgzf_writer {
    frt_write_fn write = nullptr;
    void *ctx = nullptr;
    frt_compressor *compressor = nullptr;
    size_t chunks_per_batch = 1024; // DEFAULT_CHUNKS_PER_BATCH
    size_t payload_size = 65280;    // DEFAULT_PAYLOAD_SIZE
    uint64_t blocks = 0, batches = 0, compressed = 0, uncompressed = 0;
    bool finished = false;
    std::vector<uint8_t> buf;
    std::vector<uint64_t> offs;
};

extern "C" int frt_bgzf_writer_open(frt_write_fn write, void *ctx, frt_compressor *c, frt_bgzf_writer **out,
                                    frt_error *err)
{
    if (!write || !c || !out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    frt_bgzf_writer *w = new frt_bgzf_writer;
    w->write = write;
    w->ctx = ctx;
    w->compressor = c;
    *out = w;
    return FRT_OK;
}

extern "C" void frt_bgzf_writer_set_chunks_per_batch(frt_bgzf_writer *w, size_t chunks)
{
    if (w) w->chunks_per_batch = chunks ? chunks : 1;
}

extern "C" void frt_bgzf_writer_set_payload_size(frt_bgzf_writer *w, size_t size)
{
    if (w) w->payload_size = size < 1 ? 1 : (size > kMaxPayload ? kMaxPayload : size);
}

namespace {
int writer_emit(frt_bgzf_writer *w, const uint8_t *p, size_t n, frt_error *err)
{
    while (n) {
        const int64_t k = w->write(w->ctx, p, n);
        if (k <= 0) {
            set_error(err, FRT_ERR_IO, 0, 0, 0, 0, nullptr, "the sink refused %zu bytes", n);
            return FRT_ERR_IO;
        }
        p += k;
        n -= (size_t)k;
    }
    return FRT_OK;
}
} // namespace

// write_batch (device_write.rs:106-141): the chunks bounds[i]..bounds[i + 1]
// of the device bytes, compressed chunks_per_batch at a time and written out.
extern "C" int frt_bgzf_writer_write_batch(frt_bgzf_writer *w, const uint8_t *data, size_t len, const uint64_t *bounds,
                                           size_t n_bounds, frt_error *err)
{
    if (!w || (!bounds && n_bounds) || w->finished) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument, or the writer is finished");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (n_bounds == 0) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, w->compressed, "bgzf", "bounds must have at least one entry");
        return FRT_ERR_MALFORMED;
    }
    if (bounds[n_bounds - 1] > len) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, w->compressed, "bgzf", "bounds reach byte %llu of %zu device bytes",
                  (unsigned long long)bounds[n_bounds - 1], len);
        return FRT_ERR_MALFORMED;
    }
    size_t start = 0;
    while (start + 1 < n_bounds) {
        const size_t end = start + w->chunks_per_batch + 1 < n_bounds ? start + w->chunks_per_batch + 1 : n_bounds;
        const size_t k = end - start - 1;
        w->buf.resize(frt_compress_bound(k));
        w->offs.resize(k + 1);
        size_t got = 0;
        int rc = frt_compress_batch_device(w->compressor, data, len, bounds + start, end - start, w->buf.data(),
                                           w->buf.size(), w->offs.data(), &got, err);
        if (rc) return rc;
        if ((rc = writer_emit(w, w->buf.data(), got, err))) return rc;
        w->uncompressed += bounds[end - 1] - bounds[start];
        w->compressed += got;
        w->blocks += k;
        ++w->batches;
        start = end - 1;
    }
    return FRT_OK;
}

// The device bytes in payload_size chunks (the write path of a caller that
// holds one contiguous buffer).
extern "C" int frt_bgzf_writer_write_device(frt_bgzf_writer *w, const uint8_t *data, size_t len, frt_error *err)
{
    if (!w) return FRT_ERR_INVALID_ARGUMENT;
    std::vector<uint64_t> b(1, 0);
    for (size_t at = 0; at < len;) {
        at = at + w->payload_size < len ? at + w->payload_size : len;
        b.push_back(at);
    }
    return frt_bgzf_writer_write_batch(w, data, len, b.data(), b.size(), err);
}

// finish: the EOF block, once.
extern "C" int frt_bgzf_writer_finish(frt_bgzf_writer *w, frt_error *err)
{
    if (!w) return FRT_ERR_INVALID_ARGUMENT;
    if (w->finished) return FRT_OK;
    int rc = writer_emit(w, kEofBlock, sizeof kEofBlock, err);
    if (rc) return rc;
    w->compressed += sizeof kEofBlock;
    w->finished = true;
    return FRT_OK;
}

extern "C" void frt_bgzf_writer_stats(const frt_bgzf_writer *w, uint64_t *blocks, uint64_t *batches,
                                      uint64_t *compressed, uint64_t *uncompressed)
{
    if (!w) return;
    if (blocks) *blocks = w->blocks;
    if (batches) *batches = w->batches;
    if (compressed) *compressed = w->compressed;
    if (uncompressed) *uncompressed = w->uncompressed;
}

extern "C" void frt_bgzf_writer_destroy(frt_bgzf_writer *w) { delete w; }
