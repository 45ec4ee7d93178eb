// Raw-DEFLATE inflate of BGZF members, one warp per member, with the CRC-32
// of the output folded in.
//
// A DEFLATE stream is a serial chain: a symbol's bit position is known only
// once the previous symbol is decoded.  So one lane (lane 0) walks the chain,
// and the other 31 lanes take everything that is not on it.  What the
// measurements of BGZF'd BAM drove the design to:
//
//   * a 64 KiB member of short reads holds ~20k literals and ~10k matches of
//     4.4 bytes on average, with distances spread over the whole 32 KiB
//     window (62% within 4 KiB, 84% within 16 KiB).  Matches, not literals,
//     dominate if each one is a round trip to L2.
//   * So output goes through a shared-memory ring of the last INF_RING bytes.
//     Lane 0 writes literals into it and copies a match whose source is in
//     the ring immediately (ring to ring).  A match reaching further back
//     ("far") is queued and its destination marked pending in a bitmap; a
//     near match whose source touches a pending byte is queued behind it.
//   * Every INF_FLUSH bytes the warp services the ring: far matches are
//     copied in parallel (one lane each) from the member's output already in
//     HBM, queued near matches in order, then the chunk is written to HBM
//     with coalesced stores and its CRC-32 is computed from shared memory in
//     32 slices merged by the GF(2) shift-and-xor combine.
//   * Decode tables are 16-bit entries in shared memory: a 10-bit
//     literal/length table and an 8-bit distance table, built by the whole
//     warp (counts by shared atomics, symbols sorted by __match_any_sync
//     ranking, entries filled in parallel from canonical-code limits); codes
//     longer than the root take a canonical-limit search.
//   * Stored blocks are copied by the whole warp.
//
// RFC 1951 is the specification; the checks and status codes follow the
// reference kernel (crates/fritillaria-cuda/kernels/inflate.cu:78-458), so a
// stream it rejects is rejected here with the same code.

#include "common.cuh"
#include "inflate.cuh"

namespace {

constexpr int LIT_BITS = 10;
constexpr int DIST_BITS = 8;
constexpr int CL_BITS = 7;
constexpr u32 RING = INF_RING;
constexpr u32 RMASK = RING - 1;
constexpr u32 FLUSH = INF_FLUSH;
constexpr u32 SEG = INF_SEG;   // bits of one lane's segment in a window
constexpr u32 MAXQ = INF_MAXQ; // matches queued per window
static_assert((RING & (RING - 1)) == 0, "ring size must be a power of two");
static_assert(RING >= FLUSH + 6144, "the ring holds the unflushed bytes plus a window's output");
static_assert(SEG % 32 == 0, "a segment is whole mark words");
static_assert(MAXQ <= 32 * 32, "a lane tracks at most 32 queued matches");

struct CodeState {
    u32 count[16];
    u16 first[16]; // first canonical code of each length
    u16 offs[16];  // index in `sorted` of the first symbol of each length
};

// Decode-table entries (32 bits), so the serial chain does one lookup and one
// shift per symbol:
//   [4:0]   bits to consume: the code, plus a length/distance code's extra bits
//   [7:5]   kind: 0 literal (or a valid distance), 1 length, 2 end of block,
//           3 invalid symbol
//   [11:8]  the code's own length (where its extra bits start)
//   [15:12] extra bits
//   [31:16] literal byte, or length/distance base
// An entry of 0 means no code of at most the table's root length matches:
// the long-code path.
struct WarpSmem {
    u32 lit[1 << LIT_BITS];
    u32 dist[1 << DIST_BITS];
    CodeState lcode;
    CodeState dcode;
    u16 lsorted[288];
    u16 dsorted[32];
    u32 run[16];
    u32 pend[RING / 32]; // unresolved match destinations, relative to the last flush
    u32 marks[SEG];      // token starts found by each lane in its own segment
    u32 q_dst[MAXQ];     // matches of the current window: destination
    u32 q_ld[MAXQ];      //   len | dist << 9
    u8 lens[320];
    u8 ring[RING];
};

__device__ __forceinline__ u32 lit_entry(u32 sym, u32 L)
{
    if (sym < 256) return L | (L << 8) | (sym << 16);
    if (sym == 256) return L | (2u << 5) | (L << 8);
    if (sym > 285) return L | (3u << 5) | (L << 8);
    u32 i = sym - 257, extra, base;
    if (i < 8) {
        extra = 0;
        base = 3 + i;
    } else if (i == 28) {
        extra = 0;
        base = 258;
    } else {
        extra = (i - 4) >> 2;
        base = ((4u + (i & 3u)) << extra) + 3u;
    }
    return (L + extra) | (1u << 5) | (L << 8) | (extra << 12) | (base << 16);
}

__device__ __forceinline__ u32 dist_entry(u32 sym, u32 L)
{
    if (sym >= 30) return L | (3u << 5) | (L << 8);
    u32 extra = sym < 4 ? 0u : (sym - 2u) >> 1;
    u32 base = sym < 4 ? sym + 1u : ((2u + (sym & 1u)) << extra) + 1u;
    return (L + extra) | (L << 8) | (extra << 12) | (base << 16);
}

__device__ __forceinline__ u32 cl_entry(u32 sym, u32 L) { return L | (L << 8) | (sym << 16); }

// Builds a decode table for `n` code lengths.  Returns puff's construct()
// result: 0 complete (or all-empty), >0 incomplete, <0 over-subscribed.
// kind: 0 literal/length, 1 distance, 2 code-length code.
__device__ int build_table(const u8 *lens, int n, int root, u32 *table, u16 *sorted, CodeState *cs, u32 *run,
                           int kind)
{
    const u32 lane = lane_id();
    if (lane < 16) cs->count[lane] = 0;
    __syncwarp();
    for (int s = lane; s < n; s += 32) atomicAdd(&cs->count[lens[s]], 1u);
    __syncwarp();
    int left = 1;
    if (lane == 0) {
        u32 code = 0, off = 0;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= (int)cs->count[len];
            if (left < 0) break;
        }
        cs->first[0] = 0;
        cs->offs[0] = 0;
        for (int len = 1; len < 16; ++len) {
            cs->first[len] = (u16)code;
            cs->offs[len] = (u16)off;
            run[len] = off;
            code = (code + cs->count[len]) << 1;
            off += cs->count[len];
        }
        if ((int)cs->count[0] == n) left = 0;
    }
    left = __shfl_sync(FRT_FULL_MASK, left, 0);
    __syncwarp();
    if (left < 0) return left;
    for (int base = 0; base < n; base += 32) {
        int s = base + (int)lane;
        u32 L = s < n ? lens[s] : 0u;
        u32 peers = __match_any_sync(FRT_FULL_MASK, L);
        u32 rank = __popc(peers & lanemask_lt());
        if (s < n && L != 0) sorted[run[L] + rank] = (u16)s;
        __syncwarp();
        if (L != 0 && rank == 0) run[L] += __popc(peers);
        __syncwarp();
    }
    // Entry e holds the root-bit prefix LSB first; reversed it is the
    // MSB-first prefix v, and the code length is the smallest L whose
    // left-aligned limit exceeds v (limits grow with L for canonical codes).
    u32 lim[16];
#pragma unroll
    for (int l = 1; l < 16; ++l) lim[l] = l <= root ? ((u32)cs->first[l] + cs->count[l]) << (root - l) : 0u;
    const int size = 1 << root;
    for (int e = lane; e < size; e += 32) {
        u32 v = __brev((u32)e) >> (32 - root);
        u32 L = 1;
#pragma unroll
        for (int l = 1; l < 16; ++l)
            if (l <= root) L += (v >= lim[l]) ? 1u : 0u;
        u32 entry = 0;
        if ((int)L <= root) {
            u32 sym = sorted[cs->offs[L] + ((v >> (root - L)) - cs->first[L])];
            entry = kind == 0 ? lit_entry(sym, L) : (kind == 1 ? dist_entry(sym, L) : cl_entry(sym, L));
        }
        table[e] = entry;
    }
    __syncwarp();
    return left;
}

// Codes longer than the table root: canonical search over lengths
// root+1..15 on the 15 bits at the head of the buffer.  Returns the length
// (0 when no code matches) and the symbol.
__device__ __forceinline__ u32 decode_long(u64 bitbuf, int root, const CodeState *cs, const u16 *sorted, u32 *sym)
{
    u32 v = __brev((u32)bitbuf & 0x7fffu) >> 17;
    for (int l = root + 1; l < 16; ++l) {
        u32 lim = ((u32)cs->first[l] + cs->count[l]) << (15 - l);
        if (v < lim) {
            *sym = sorted[cs->offs[l] + ((v >> (15 - l)) - cs->first[l])];
            return (u32)l;
        }
    }
    return 0;
}

// A bit reader that can start at any bit of a member's payload (positions
// count bits from the payload start).  Words are read aligned from HBM through
// the L1; words past the payload read as zero.
struct LaneBits {
    const u32 *base; // aligned word at or before the payload start
    u32 nwords;      // words holding payload bytes
    u32 bit0;        // payload start, in bits from base
    u64 buf;
    int cnt; // valid bits in buf
    u32 nw;  // next word to load

    __device__ __forceinline__ void attach(const u8 *in, u32 in_len)
    {
        u64 a = (u64)in;
        base = (const u32 *)(a & ~3ull);
        bit0 = 8u * (u32)(a & 3ull);
        nwords = (bit0 + 8u * in_len + 31u) / 32u;
    }
    __device__ __forceinline__ u32 word(u32 i) const { return i < nwords ? __ldg(base + i) : 0u; }
    __device__ __forceinline__ void seek(u32 p)
    {
        u32 a = p + bit0, w = a >> 5, sh = a & 31u;
        buf = (((u64)word(w + 1) << 32) | word(w)) >> sh;
        cnt = 64 - (int)sh;
        nw = w + 2;
    }
    // After refill, cnt > 32.
    __device__ __forceinline__ void refill()
    {
        if (cnt <= 32) {
            buf |= (u64)word(nw) << cnt;
            cnt += 32;
            ++nw;
        }
    }
    __device__ __forceinline__ u32 tell() const { return nw * 32u - (u32)cnt - bit0; }
    __device__ __forceinline__ u32 peek(int n) const { return (u32)buf & ((1u << n) - 1u); }
    __device__ __forceinline__ void drop(int n)
    {
        buf >>= n;
        cnt -= n;
    }
};

enum : u32 { TK_LIT = 0, TK_MATCH = 1, TK_EOB = 2, TK_BADCODE = 3, TK_BADDIST = 4 };

// One token of a Huffman block: a literal, a length/distance pair or the
// end of block.  Returns the kind; *v is the literal or the length.
__device__ __forceinline__ u32 decode_token(LaneBits &r, const WarpSmem *sm, u32 *v, u32 *dist)
{
    r.refill();
    u32 e = sm->lit[(u32)r.buf & ((1u << LIT_BITS) - 1u)];
    if (e == 0) {
        u32 sym, L = decode_long(r.buf, LIT_BITS, &sm->lcode, sm->lsorted, &sym);
        if (L == 0) {
            r.drop(15); // the reference reads 15 bits before giving up
            return TK_BADCODE;
        }
        e = lit_entry(sym, L);
    }
    u32 kind = (e >> 5) & 7u;
    if (kind == 0) {
        *v = e >> 16;
        r.drop((int)(e & 31u));
        return TK_LIT;
    }
    if (kind != 1) {
        r.drop((int)(e & 31u));
        return kind == 2 ? TK_EOB : TK_BADCODE;
    }
    u32 len = (e >> 16) + ((u32)(r.buf >> ((e >> 8) & 15u)) & ((1u << ((e >> 12) & 15u)) - 1u));
    r.drop((int)(e & 31u));
    r.refill();
    u32 d = sm->dist[(u32)r.buf & ((1u << DIST_BITS) - 1u)];
    if (d == 0) {
        u32 sym, L = decode_long(r.buf, DIST_BITS, &sm->dcode, sm->dsorted, &sym);
        if (L == 0) {
            r.drop(15);
            return TK_BADDIST;
        }
        d = dist_entry(sym, L);
    }
    if ((d >> 5) & 7u) {
        r.drop((int)(d & 31u));
        return TK_BADDIST;
    }
    *dist = (d >> 16) + ((u32)(r.buf >> ((d >> 8) & 15u)) & ((1u << ((d >> 12) & 15u)) - 1u));
    r.drop((int)(d & 31u));
    *v = len;
    return TK_MATCH;
}

// Pending-bit helpers over the ring (offsets relative to the last flush).
// Destinations of different matches can share a word, hence the atomics.
__device__ __forceinline__ void pend_set(u32 *pend, u32 a, u32 b, bool on)
{
    while (a < b) {
        u32 w = a >> 5, bit = a & 31u;
        u32 n = min(32u - bit, b - a);
        u32 m = (n == 32u ? 0xffffffffu : ((1u << n) - 1u)) << bit;
        if (on) atomicOr(&pend[w], m);
        else atomicAnd(&pend[w], ~m);
        a += n;
    }
}

__device__ __forceinline__ bool pend_any(const u32 *pend, u32 a, u32 b)
{
    while (a < b) {
        u32 w = a >> 5, bit = a & 31u;
        u32 n = min(32u - bit, b - a);
        u32 m = (n == 32u ? 0xffffffffu : ((1u << n) - 1u)) << bit;
        if (pend[w] & m) return true;
        a += n;
    }
    return false;
}

// Resolves the window's nq queued matches in parallel rounds: in each round
// every match whose source bytes are final is copied, one lane per match.
// The earliest unresolved match is always ready, so rounds make progress.
// A source byte still in the ring (at or after pos - RING) is read there;
// anything older has been flushed and is read from HBM.
__device__ void resolve(WarpSmem *sm, const u8 *out, u32 flushed, u32 pos, u32 nq)
{
    const u32 lane = lane_id();
    for (u32 k = lane; k < nq; k += 32) {
        u32 d = sm->q_dst[k];
        pend_set(sm->pend, d - flushed, d + (sm->q_ld[k] & 511u) - flushed, true);
    }
    __syncwarp();
    u32 todo = 0;
    for (u32 j = 0; lane + 32 * j < nq; ++j) todo |= 1u << j;
    const u32 ring_lo = pos > RING ? pos - RING : 0u;
    while (__any_sync(FRT_FULL_MASK, todo != 0)) {
        u32 ready = 0;
        for (u32 t = todo; t; t &= t - 1) {
            u32 j = __ffs(t) - 1, k = lane + 32 * j;
            u32 d = sm->q_dst[k], ld = sm->q_ld[k];
            u32 len = ld & 511u, dist = ld >> 9;
            u32 s = d - dist, e = s + min(len, dist);
            if (e <= flushed || !pend_any(sm->pend, max(s, flushed) - flushed, e - flushed)) ready |= 1u << j;
        }
        __syncwarp();
        for (u32 t = ready; t; t &= t - 1) {
            u32 j = __ffs(t) - 1, k = lane + 32 * j;
            u32 d = sm->q_dst[k], ld = sm->q_ld[k];
            u32 len = ld & 511u, s = d - (ld >> 9);
            for (u32 i = 0; i < len; ++i) {
                u32 p = s + i;
                u8 b = p >= ring_lo ? sm->ring[p & RMASK] : out[p];
                sm->ring[(d + i) & RMASK] = b;
            }
        }
        __syncwarp();
        for (u32 t = ready; t; t &= t - 1) {
            u32 j = __ffs(t) - 1, k = lane + 32 * j;
            u32 d = sm->q_dst[k];
            pend_set(sm->pend, d - flushed, d + (sm->q_ld[k] & 511u) - flushed, false);
        }
        todo &= ~ready;
        __syncwarp();
    }
}

// Writes [flushed, pos) to HBM with coalesced stores and folds its CRC into
// *crc: 32 slices from shared memory, merged pairwise by the GF(2) combine.
__device__ void flush_crc(const WarpSmem *sm, u8 *out, u32 flushed, u32 pos, const u32 *crc_tab, u32 *crc)
{
    const u32 lane = lane_id();
    u32 F = pos - flushed;
    for (u32 j = lane; j < F; j += 32) out[flushed + j] = sm->ring[(flushed + j) & RMASK];
    u32 slice = (F + 31) / 32;
    u32 b0 = min(F, lane * slice), b1 = min(F, b0 + slice);
    u32 c = 0xffffffffu;
    for (u32 i = b0; i < b1; ++i) c = crc_tab[(c ^ sm->ring[(flushed + i) & RMASK]) & 0xffu] ^ (c >> 8);
    c = ~c;
    u32 mylen = b1 - b0;
    for (int d = 1; d < 32; d <<= 1) {
        u32 oc = __shfl_down_sync(FRT_FULL_MASK, c, d);
        u32 ol = __shfl_down_sync(FRT_FULL_MASK, mylen, d);
        if ((lane & (2 * d - 1)) == 0 && lane + d < 32) {
            c = crc_combine(c, oc, ol);
            mylen += ol;
        }
    }
    c = __shfl_sync(FRT_FULL_MASK, c, 0);
    *crc = crc_combine(*crc, c, F);
    __syncwarp();
}

// Errors found on the true chain, ranked by bit position so the earliest
// one is reported, as a sequential decoder would.
__device__ __forceinline__ u64 err_key(u32 bitpos, u32 code) { return ((u64)bitpos << 8) | code; }

struct Window {
    u32 next;   // bit position where decoding continues
    u32 status; // INF_OK or the first error
    int eob;    // the block ended in this window
};

// One window of a Huffman block, decoded by all 32 lanes.
//
//   A  lane k decodes the tokens that start in its segment
//      [bitpos + k*SEG, bitpos + (k+1)*SEG) from the segment start -- a
//      guess, except for lane 0 -- and marks each token start.
//   B  lane k continues its chain into segment k+1 until it reaches a start
//      that lane k+1 marked.  From there the two decodings agree (decoding is
//      deterministic from a true boundary), so lane k+1's chain is proven by
//      lane k's, and by induction from lane 0 every lane up to the first one
//      that did not synchronise is on the true chain.
//   C  each proven lane re-decodes its true range, counting output bytes and
//      matches and finding the end of block or an error.
//   D  after a warp scan places every range in the output, each lane decodes
//      its range once more, writing literals into the ring and queueing
//      matches; then the matches are resolved in parallel rounds.
// A lane that did not synchronise within the next segment ends the window at
// its last proven token; the next window starts there.
__device__ Window decode_window(WarpSmem *sm, LaneBits &r, u32 bitpos, u32 total, u8 *out, u32 flushed, u32 *pos_io,
                                u32 cap)
{
    const u32 lane = lane_id();
    const u32 pos = *pos_io;
    for (u32 w = lane; w < SEG; w += 32) sm->marks[w] = 0;
    __syncwarp();
    // ---- A
    const u32 s0 = bitpos + lane * SEG, s1 = s0 + SEG;
    u32 exitp = s0;
    if (s0 < total) {
        u32 p = s0;
        r.seek(p);
        while (p < s1 && p < total) {
            u32 v, dd;
            u32 k = decode_token(r, sm, &v, &dd);
            if (k >= TK_BADCODE) { // not a token start: slide one bit
                ++p;
                r.seek(p);
                continue;
            }
            u32 rel = p - bitpos;
            sm->marks[rel >> 5] |= 1u << (rel & 31u);
            p = r.tell();
        }
        exitp = p;
    }
    __syncwarp();
    // ---- B
    enum { SYNC = 0, FAIL = 1, END = 2, STOP = 3, LAST = 4 };
    u32 outcome = END, q = exitp;
    if (lane < 31) {
        const u32 s2 = s1 + SEG;
        r.seek(q);
        while (true) {
            if (q >= total) {
                outcome = END;
                break;
            }
            if (q >= s2) {
                outcome = FAIL;
                break;
            }
            u32 rel = q - bitpos;
            if ((sm->marks[rel >> 5] >> (rel & 31u)) & 1u) {
                outcome = SYNC;
                break;
            }
            u32 v, dd;
            u32 k = decode_token(r, sm, &v, &dd);
            if (k >= TK_EOB) { // end of block or an error: pass C reports it
                outcome = STOP;
                break;
            }
            q = r.tell();
        }
    } else {
        outcome = LAST; // lane 31's range ends with its segment
        q = exitp;
    }
    u32 notsync = __ballot_sync(FRT_FULL_MASK, outcome != SYNC);
    const u32 V = __ffs(notsync) - 1; // lanes 0..V are on the true chain
    u32 prevq = __shfl_up_sync(FRT_FULL_MASK, q, 1);
    const u32 start = lane == 0 ? bitpos : prevq;
    u32 end = q;
    if (lane == V && (outcome == STOP || outcome == END)) end = 0xffffffffu; // run until the stop itself
    // ---- C
    u32 nbytes = 0, nmatch = 0, cstop = 0, cpos = 0; // cstop: 0 none, 1 eob, else an INF_ error
    if (lane <= V) {
        u32 p = start;
        r.seek(p);
        while (p < end) {
            if (p >= total) {
                cstop = INF_TRUNCATED;
                cpos = p;
                break;
            }
            u32 v, dd;
            u32 k = decode_token(r, sm, &v, &dd);
            u32 np = r.tell();
            if (np > total) {
                cstop = INF_TRUNCATED;
                cpos = p;
                break;
            }
            if (k == TK_EOB) {
                cstop = 1;
                cpos = np;
                break;
            }
            if (k == TK_BADCODE) {
                cstop = INF_BAD_CODE;
                cpos = p;
                break;
            }
            if (k == TK_BADDIST) {
                cstop = INF_BAD_DISTANCE;
                cpos = p;
                break;
            }
            nbytes += k == TK_LIT ? 1u : v;
            nmatch += k == TK_MATCH ? 1u : 0u;
            p = np;
        }
        if (!cstop) cpos = p;
    }
    // the first lane that stopped ends the true chain
    u32 stopped = __ballot_sync(FRT_FULL_MASK, lane <= V && cstop != 0);
    u32 last = stopped ? (u32)(__ffs(stopped) - 1) : V;
    // place the ranges; keep the prefix that fits the ring and the queue
    u32 inc_b = lane <= last ? nbytes : 0u, inc_m = lane <= last ? nmatch : 0u;
    for (int d = 1; d < 32; d <<= 1) {
        u32 yb = __shfl_up_sync(FRT_FULL_MASK, inc_b, d), ym = __shfl_up_sync(FRT_FULL_MASK, inc_m, d);
        if (lane >= (u32)d) {
            inc_b += yb;
            inc_m += ym;
        }
    }
    const u32 budget = RING - 258u - (pos - flushed);
    u32 fits = __ballot_sync(FRT_FULL_MASK, lane <= last && inc_b <= budget && inc_m <= MAXQ);
    u32 cut = fits == 0xffffffffu ? 32u : (u32)(__ffs(~fits) - 1); // lanes [0, cut) kept; fits is a prefix
    if (cut > last + 1) cut = last + 1;
    Window w;
    w.status = INF_OK;
    w.eob = 0;
    if (cut == 0) {
        // lane 0's range alone overflows the ring: only lane 0 proceeds, one
        // token at a time, through the serial path of the caller
        w.next = bitpos;
        w.status = 0xffffffffu;
        return w;
    }
    const u32 base_b = inc_b - (lane <= last ? nbytes : 0u);
    const u32 base_m = inc_m - (lane <= last ? nmatch : 0u);
    const u32 tot_b = __shfl_sync(FRT_FULL_MASK, inc_b, cut - 1);
    const u32 tot_m = __shfl_sync(FRT_FULL_MASK, inc_m, cut - 1);
    // ---- D
    u64 ekey = ~0ull;
    if (lane < cut) {
        u32 p = start, o = pos + base_b, m = base_m;
        u32 lim = lane == last ? cpos : end;
        r.seek(p);
        while (p < lim) {
            u32 v, dd;
            u32 k = decode_token(r, sm, &v, &dd);
            if (k == TK_LIT) {
                if (o >= cap) {
                    ekey = err_key(p, INF_OUTPUT_OVERFLOW);
                    break;
                }
                sm->ring[o & RMASK] = (u8)v;
                ++o;
            } else if (k == TK_MATCH) {
                if (dd > o) {
                    ekey = err_key(p, INF_BAD_DISTANCE);
                    break;
                }
                if (o + v > cap) {
                    ekey = err_key(p, INF_OUTPUT_OVERFLOW);
                    break;
                }
                sm->q_dst[m] = o;
                sm->q_ld[m] = v | (dd << 9);
                ++m;
                o += v;
            } else {
                break; // the end of block (only in the last lane's range)
            }
            p = r.tell();
        }
        if (lane == last && lane < cut && cstop > 1 && ekey == ~0ull) ekey = err_key(cpos, cstop);
    }
    // earliest error on the chain
    for (int d = 16; d; d >>= 1) {
        u64 o = __shfl_xor_sync(FRT_FULL_MASK, ekey, d);
        ekey = o < ekey ? o : ekey;
    }
    __syncwarp();
    if (ekey != ~0ull) {
        w.status = (u32)(ekey & 0xffu);
        w.next = (u32)(ekey >> 8);
        return w;
    }
    resolve(sm, out, flushed, pos + tot_b, tot_m);
    *pos_io = pos + tot_b;
    u32 nextp = __shfl_sync(FRT_FULL_MASK, start, cut < 32 ? cut : 0);
    if (cut <= last) {
        w.next = nextp; // continue at the first range that did not fit
    } else {
        u32 lastp = __shfl_sync(FRT_FULL_MASK, cpos, last);
        u32 lasts = __shfl_sync(FRT_FULL_MASK, cstop, last);
        w.next = lastp;
        w.eob = lasts == 1;
    }
    return w;
}

// The rare path for a range whose output does not fit a window: lane 0
// decodes token by token, the warp flushing the ring between tokens.
__device__ u32 decode_serial_range(WarpSmem *sm, LaneBits &r, u32 *bitpos_io, u32 total, u8 *out, u32 *flushed_io,
                                   u32 *pos_io, u32 cap, u32 tokens, const u32 *crc_tab, u32 *crc, int *eob)
{
    const u32 lane = lane_id();
    u32 bitpos = *bitpos_io, status = INF_OK;
    for (u32 t = 0; t < tokens; ++t) {
        u32 kind = 0, v = 0, dd = 0, np = 0;
        if (lane == 0) {
            r.seek(bitpos);
            kind = decode_token(r, sm, &v, &dd);
            np = r.tell();
        }
        kind = __shfl_sync(FRT_FULL_MASK, kind, 0);
        v = __shfl_sync(FRT_FULL_MASK, v, 0);
        dd = __shfl_sync(FRT_FULL_MASK, dd, 0);
        np = __shfl_sync(FRT_FULL_MASK, np, 0);
        if (np > total) status = INF_TRUNCATED;
        else if (kind == TK_BADCODE) status = INF_BAD_CODE;
        else if (kind == TK_BADDIST) status = INF_BAD_DISTANCE;
        if (status != INF_OK) break;
        if (kind == TK_EOB) {
            *eob = 1;
            bitpos = np;
            break;
        }
        u32 n = kind == TK_LIT ? 1u : v;
        if (*pos_io - *flushed_io + n > RING - 258u) {
            flush_crc(sm, out, *flushed_io, *pos_io, crc_tab, crc);
            *flushed_io = *pos_io;
        }
        u32 o = *pos_io;
        if (kind == TK_LIT) {
            if (o >= cap) {
                status = INF_OUTPUT_OVERFLOW;
                break;
            }
            if (lane == 0) sm->ring[o & RMASK] = (u8)v;
        } else {
            if (dd > o) {
                status = INF_BAD_DISTANCE;
                break;
            }
            if (o + v > cap) {
                status = INF_OUTPUT_OVERFLOW;
                break;
            }
            if (lane == 0) {
                sm->q_dst[0] = o;
                sm->q_ld[0] = v | (dd << 9);
            }
            __syncwarp();
            resolve(sm, out, *flushed_io, o + v, 1);
        }
        __syncwarp();
        *pos_io = o + n;
        bitpos = np;
    }
    *bitpos_io = bitpos;
    return status;
}

} // namespace

// Inflates one member with the calling warp into out[0, cap).  Returns the
// status; *produced_out and *crc_out are valid in every lane.
__device__ u32 inflate_member_warp(const u8 *in, u32 in_len, u8 *out, u32 cap, void *smem_v, const u32 *crc_tab,
                                   u32 *produced_out, u32 *crc_out)
{
    WarpSmem *sm = (WarpSmem *)smem_v;
    const u32 lane = lane_id();
    LaneBits r;
    r.attach(in, in_len);
    for (u32 w = lane; w < RING / 32; w += 32) sm->pend[w] = 0;
    __syncwarp();
    const u32 total = 8u * in_len;
    u32 bitpos = 0;  // next unread bit of the stream (warp-uniform)
    u32 pos = 0;     // bytes decoded
    u32 flushed = 0; // bytes written to HBM
    u32 crc = 0;     // CRC-32 of [0, flushed)
    u32 status = INF_OK;
    int last = 0;

    while (true) {
        int type = 0;
        if (lane == 0) {
            if (bitpos + 3 > total) {
                status = INF_TRUNCATED;
            } else {
                r.seek(bitpos);
                last = (int)r.peek(1);
                type = (int)((r.buf >> 1) & 3u);
            }
        }
        status = __shfl_sync(FRT_FULL_MASK, status, 0);
        if (status != INF_OK) break;
        type = __shfl_sync(FRT_FULL_MASK, type, 0);
        last = __shfl_sync(FRT_FULL_MASK, last, 0);
        bitpos += 3;
        if (type == 3) {
            status = INF_BLOCK_TYPE;
            break;
        }

        if (type == 0) {
            // ---- stored block: copied by the whole warp through the ring ----
            u32 bytepos = (bitpos + 7) / 8, len = 0;
            if (lane == 0) {
                if (bytepos + 4 > in_len) {
                    status = INF_TRUNCATED;
                } else {
                    u32 l = (u32)in[bytepos] | ((u32)in[bytepos + 1] << 8);
                    u32 nl = (u32)in[bytepos + 2] | ((u32)in[bytepos + 3] << 8);
                    if (l != (~nl & 0xffffu)) status = INF_STORED_LEN;
                    else if (bytepos + 4 + l > in_len) status = INF_TRUNCATED;
                    else if (pos + l > cap) status = INF_OUTPUT_OVERFLOW;
                    len = l;
                }
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            len = __shfl_sync(FRT_FULL_MASK, len, 0);
            const u8 *src = in + bytepos + 4;
            bitpos = 8u * (bytepos + 4 + len);
            while (len) {
                if (pos - flushed >= FLUSH) {
                    flush_crc(sm, out, flushed, pos, crc_tab, &crc);
                    flushed = pos;
                }
                u32 n = min(len, FLUSH - (pos - flushed));
                for (u32 j = lane; j < n; j += 32) sm->ring[(pos + j) & RMASK] = src[j];
                __syncwarp();
                pos += n;
                src += n;
                len -= n;
            }
            if (last) break;
            continue;
        }

        // ---- Huffman block: tables ------------------------------------------
        if (type == 1) {
            for (int s = lane; s < 288; s += 32) sm->lens[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
            __syncwarp();
            build_table(sm->lens, 288, LIT_BITS, sm->lit, sm->lsorted, &sm->lcode, sm->run, 0);
            sm->lens[lane] = 5;
            __syncwarp();
            build_table(sm->lens, 32, DIST_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 1);
        } else {
            int nlen = 0, ndist = 0, ncode = 0;
            u32 bp = bitpos;
            if (lane == 0) {
                if (bp + 14 > total) {
                    status = INF_TRUNCATED;
                } else {
                    r.seek(bp);
                    nlen = (int)r.peek(5) + 257;
                    ndist = (int)((r.buf >> 5) & 31u) + 1;
                    ncode = (int)((r.buf >> 10) & 15u) + 4;
                    r.drop(14);
                    if (nlen > 286 || ndist > 30) status = INF_BAD_COUNTS;
                }
                if (status == INF_OK) {
                    // the code-length code lengths arrive in this permuted order
                    const u8 order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
                    for (int i = 0; i < 19; ++i) sm->lens[order[i]] = 0;
                    for (int i = 0; i < ncode; ++i) {
                        r.refill();
                        if (r.tell() + 3 > total) {
                            status = INF_TRUNCATED;
                            break;
                        }
                        sm->lens[order[i]] = (u8)r.peek(3);
                        r.drop(3);
                    }
                }
                bp = r.tell();
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            nlen = __shfl_sync(FRT_FULL_MASK, nlen, 0);
            ndist = __shfl_sync(FRT_FULL_MASK, ndist, 0);
            __syncwarp();
            // the code-length code must be complete (all-zero counts as
            // complete and fails at first use, as in the reference)
            if (build_table(sm->lens, 19, CL_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 2) != 0) {
                status = INF_BAD_TABLE;
                break;
            }
            if (lane == 0) {
                int index = 0;
                r.seek(bp);
                while (index < nlen + ndist) {
                    r.refill();
                    u32 e = sm->dist[r.peek(CL_BITS)];
                    u32 L = e & 31u;
                    u32 left = total - min(total, r.tell());
                    if (L == 0) {
                        status = left < 15 ? INF_TRUNCATED : INF_BAD_CODE;
                        break;
                    }
                    if (L > left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    r.drop((int)L);
                    u32 sym = e >> 16;
                    if (sym < 16) {
                        sm->lens[index++] = (u8)sym;
                        continue;
                    }
                    u32 val = 0;
                    u32 nb = sym == 16 ? 2 : (sym == 17 ? 3 : 7);
                    if (sym == 16) {
                        if (index == 0) {
                            status = INF_BAD_LENGTH_REPEAT;
                            break;
                        }
                        val = sm->lens[index - 1];
                    }
                    if (r.tell() + nb > total) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    u32 rep = (sym == 18 ? 11u : 3u) + r.peek((int)nb);
                    r.drop((int)nb);
                    if (index + (int)rep > nlen + ndist) {
                        status = INF_BAD_LENGTH_REPEAT;
                        break;
                    }
                    while (rep--) sm->lens[index++] = (u8)val;
                }
                if (status == INF_OK && sm->lens[256] == 0) status = INF_BAD_TABLE;
                bp = r.tell();
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            bitpos = __shfl_sync(FRT_FULL_MASK, bp, 0);
            __syncwarp();
            int rl = build_table(sm->lens, nlen, LIT_BITS, sm->lit, sm->lsorted, &sm->lcode, sm->run, 0);
            if (rl != 0 && (rl < 0 || nlen != (int)sm->lcode.count[0] + 1)) { // incomplete only with one code
                status = INF_BAD_TABLE;
                break;
            }
            int rd = build_table(sm->lens + nlen, ndist, DIST_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 1);
            if (rd != 0 && (rd < 0 || ndist != (int)sm->dcode.count[0] + 1)) {
                status = INF_BAD_TABLE;
                break;
            }
        }

        // ---- Huffman block: symbols, a window at a time ----------------------
        while (true) {
            if (pos - flushed >= FLUSH) {
                flush_crc(sm, out, flushed, pos, crc_tab, &crc);
                flushed = pos;
            }
            if (bitpos >= total) { // the stream ended before the end of block
                status = INF_TRUNCATED;
                break;
            }
            Window w = decode_window(sm, r, bitpos, total, out, flushed, &pos, cap);
            if (w.status == 0xffffffffu) {
                int eob = 0;
                status = decode_serial_range(sm, r, &bitpos, total, out, &flushed, &pos, cap, 16, crc_tab, &crc, &eob);
                if (status != INF_OK || eob) break;
                continue;
            }
            if (w.status != INF_OK) {
                status = w.status;
                break;
            }
            bitpos = w.next;
            if (w.eob) break;
        }
        if (status != INF_OK) break;
        if (last) break;
    }
    if (status == INF_OK) flush_crc(sm, out, flushed, pos, crc_tab, &crc);
    // on error nothing more is written: the member's output is discarded
    *produced_out = pos;
    *crc_out = crc;
    return status;
}

size_t frt_inflate_warp_smem() { return sizeof(WarpSmem); }

__device__ __forceinline__ void init_crc_table(u32 *tab)
{
    for (u32 i = threadIdx.x; i < 256; i += blockDim.x) {
        u32 c = i;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
        tab[i] = c;
    }
}

#define WSM_BYTES ((sizeof(WarpSmem) + 15) & ~(size_t)15)

// Plain form: one warp per member of this launch, members in span order.
__global__ void __launch_bounds__(INF_WARPS_PER_CTA * 32, 1)
k_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                  const u32 *out_cap, u32 *status, u32 *produced, u32 *crc, u32 n)
{
    extern __shared__ __align__(16) unsigned char smem[];
    u32 *crc_tab = (u32 *)smem;
    init_crc_table(crc_tab);
    __syncthreads();
    const u32 warp = threadIdx.x / 32;
    void *wsm = smem + 1024 + warp * WSM_BYTES;
    u32 m = blockIdx.x * (blockDim.x / 32) + warp;
    if (m >= n) return;
    u32 p = 0, c = 0;
    u32 st = inflate_member_warp(in + in_off[m], in_len[m], out + out_off[m], out_cap[m], wsm, crc_tab, &p, &c);
    if (lane_id() == 0) {
        status[m] = st;
        produced[m] = p;
        crc[m] = st == INF_OK ? c : 0u;
    }
}

// Batched form: a persistent grid pulls members from a device work queue
// (`order`, longest first) through an atomic head, `chunk` members per pop,
// one warp per member, and verifies each member against its trailer as it
// finishes: the first failing member in file order wins the error word
// (member << 8 | frt_status), as in verify_and_offsets (backend.rs:221-256).
__global__ void __launch_bounds__(INF_WARPS_PER_CTA * 32, 1)
k_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                     const u32 *isize, const u32 *crc_expect, u32 *status, u32 *produced, u32 *crc,
                     const u32 *order, const u64 *n_ptr, u64 n_cap, u64 out_capacity, u32 *queue_head, u32 chunk,
                     unsigned long long *block_err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    u32 *crc_tab = (u32 *)smem;
    init_crc_table(crc_tab);
    __syncthreads();
    const u32 warp = threadIdx.x / 32;
    void *wsm = smem + 1024 + warp * WSM_BYTES;
    u64 n64 = *n_ptr;
    const u32 n = (u32)(n64 < n_cap ? n64 : n_cap);
    if (chunk == 0) chunk = 1;
    while (true) {
        u32 base = 0;
        if (lane_id() == 0) base = atomicAdd(queue_head, chunk);
        base = __shfl_sync(FRT_FULL_MASK, base, 0);
        if (base >= n) break;
        u32 end = min(n, base + chunk);
        for (u32 q = base; q < end; ++q) {
            u32 m = order ? order[q] : q;
            if (m >= n) continue;
            u32 cap = isize[m];
            u32 p = 0, c = 0, st;
            if (out_off[m] + cap > out_capacity) {
                st = INF_OUTPUT_OVERFLOW; // sizes changed since the buffers were planned
            } else {
                st = inflate_member_warp(in + in_off[m], in_len[m], out + out_off[m], cap, wsm, crc_tab, &p, &c);
            }
            if (lane_id() == 0) {
                status[m] = st;
                produced[m] = p;
                crc[m] = st == INF_OK ? c : 0u;
                unsigned long long code = st != INF_OK ? 5ull : (p != cap ? 4ull : (c != crc_expect[m] ? 3ull : 0ull));
                if (code) atomicMin(block_err, ((unsigned long long)m << 8) | code);
            }
        }
    }
}

// Standalone CRC of already-inflated members (the reference's crc32_blocks,
// crates/fritillaria-cuda/kernels/crc32.cu:13-38), one warp per member.
__global__ void k_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n)
{
    __shared__ u32 tab[256];
    init_crc_table(tab);
    __syncthreads();
    u32 m = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (m >= n) return;
    const u8 *p = data + offsets[m];
    u32 len = lengths[m];
    u32 lane = lane_id();
    u32 slice = (len + 31) / 32;
    u32 b0 = min(len, lane * slice), b1 = min(len, b0 + slice);
    u32 c = 0xffffffffu;
    for (u32 i = b0; i < b1; ++i) c = tab[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    c = ~c;
    u32 mylen = b1 - b0;
    for (int d = 1; d < 32; d <<= 1) {
        u32 oc = __shfl_down_sync(FRT_FULL_MASK, c, d);
        u32 ol = __shfl_down_sync(FRT_FULL_MASK, mylen, d);
        if ((lane & (2 * d - 1)) == 0 && lane + d < 32) {
            c = crc_combine(c, oc, ol);
            mylen += ol;
        }
    }
    if (lane == 0) out[m] = c;
}

// ---- host launchers --------------------------------------------------------
size_t frt_inflate_smem_bytes(int warps) { return 1024 + (size_t)warps * WSM_BYTES; }

cudaError_t frt_inflate_prepare()
{
    cudaError_t e = cudaFuncSetAttribute(k_inflate_members, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)frt_inflate_smem_bytes(INF_WARPS_PER_CTA));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_inflate_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)frt_inflate_smem_bytes(INF_WARPS_PER_CTA));
}

cudaError_t frt_launch_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                       const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                       u32 *crc, u32 n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    u32 grid = (n + INF_WARPS_PER_CTA - 1) / INF_WARPS_PER_CTA;
    k_inflate_members<<<grid, INF_WARPS_PER_CTA * 32, frt_inflate_smem_bytes(INF_WARPS_PER_CTA), s>>>(
        in, in_off, in_len, out, out_off, out_cap, status, produced, crc, n);
    return cudaGetLastError();
}

cudaError_t frt_launch_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                          const u64 *out_off, const u32 *isize, const u32 *crc_expect, u32 *status,
                                          u32 *produced, u32 *crc, const u32 *order, const u64 *n_ptr, u64 n_cap,
                                          u64 out_capacity, u32 *queue_head, u32 chunk, u32 grid,
                                          unsigned long long *block_err, cudaStream_t s)
{
    k_inflate_persistent<<<grid, INF_WARPS_PER_CTA * 32, frt_inflate_smem_bytes(INF_WARPS_PER_CTA), s>>>(
        in, in_off, in_len, out, out_off, isize, crc_expect, status, produced, crc, order, n_ptr, n_cap,
        out_capacity, queue_head, chunk, block_err);
    return cudaGetLastError();
}

int frt_inflate_persistent_grid()
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_inflate_persistent, INF_WARPS_PER_CTA * 32,
                                                  frt_inflate_smem_bytes(INF_WARPS_PER_CTA));
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_crc32_members<<<(n + 7) / 8, 256, 0, s>>>(data, offsets, lengths, out, n);
    return cudaGetLastError();
}
