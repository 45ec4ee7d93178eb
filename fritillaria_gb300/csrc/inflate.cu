// Raw-DEFLATE inflate of BGZF members, one warp per member, with the CRC-32
// of the output folded in.
//
// A DEFLATE stream is a serial chain: a symbol's bit position is known only
// once the previous symbol is decoded, and on GB300 one link of that chain --
// a shared-memory table lookup feeding a 64-bit shift feeding the next lookup
// -- costs ~120 cycles.  So lane 0 walks the chain and does nothing else, and
// the other 31 lanes take all the work that is not on it:
//
//   * Decode tables are 32-bit entries in shared memory that carry a symbol
//     with its extra bits (one lookup and one shift per literal, two per
//     match): a 10-bit literal/length root and an 8-bit distance root side by
//     side, codes longer than the root taking a canonical-limit search.  The
//     warp builds them (counts by shared atomics, symbols ranked with
//     __match_any_sync, entries filled in parallel from canonical limits).
//   * Lane 0 writes literals into a shared-memory window buffer and queues
//     matches.  A 64 KiB member of short reads holds ~20k literals and ~10k
//     matches of 4.4 bytes whose sources spread over the whole 32 KiB window,
//     so copying them on the chain would stall it on L2 round trips.
//   * When the buffer or the queue is full, the warp resolves the queued
//     matches in parallel rounds (each copied once its source bytes are
//     final; sources before the window come from the member's output already
//     in HBM, loaded in groups so the loads overlap), writes the window to HBM
//     with coalesced stores and folds its CRC-32 in, computed from shared
//     memory in 32 slices merged by the GF(2) shift-and-xor combine.
//   * Stored blocks are copied by the whole warp.
//
// RFC 1951 is the specification; the checks and status codes follow the
// reference kernel (crates/fritillaria-cuda/kernels/inflate.cu:78-458), so a
// stream it rejects is rejected here with the same code.

#include <atomic>
#include <cstddef>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "inflate.cuh"
#include "runtime.h"

namespace {

constexpr int CL_BITS = 7;
constexpr u32 MAX_WB = 4096; // the largest window buffer of any variant

// One configuration of the member inflate: the literal/length and distance
// table roots, the window output buffer, the window's match queue and a
// register cap (more warps per SM against fewer registers per lane).  The
// library carries a few (kVariants below); a tuning picks one per device and
// workload.
template <int LB, int DB, u32 W, u32 Q, int R = 128, u32 S = 0> struct Cfg {
    static constexpr int REGS = R; // register cap per thread (ptxas), trading per-warp speed for occupancy
    static constexpr u32 STAGE = S; // 0: read the compressed bytes through L1; else staging-ring half (bytes)
    static constexpr int LIT_BITS = LB;
    static constexpr int DIST_BITS = DB;
    static constexpr u32 DIST_BASE = 1u << LB; // distance entries follow the literal/length ones
    static constexpr u32 LIT_MASK = (1u << LB) - 1u;
    static constexpr u32 DIST_MASK = (1u << DB) - 1u;
    static constexpr u32 WB = W;   // window output buffer (bytes)
    static constexpr u32 MAXQ = Q; // matches per window
    // After a refill the buffer holds at least 33 bits: enough for a length
    // whose code and extra bits fit the root plus a distance whose code fits
    // its root (at most 13 extra bits), so a fast match needs no second refill.
    static_assert(LB + DB + 13 <= 33, "a fast match must fit one refill");
    static_assert(LB <= 15 && DB <= 15, "roots are at most the longest code");
    static_assert(Q <= 32 * 32, "a lane tracks at most 32 queued matches");
    static_assert(W % 32 == 0 && W > 2 * 258 && W <= MAX_WB, "pending bits cover whole words");
    static_assert(S == 0 || (S >= 64 && (S & (S - 1)) == 0), "a staging half is a power of two of 64+ bytes");
};

// CRC-32 tables, computed at compile time: slice[k][b] is the register that
// byte b followed by k zero bytes leaves from zero (slicing by 4; slice[0] is
// the byte table), xpow[m] = x^(8m) mod P in the reflected order the
// registers use (bit 31 is x^0), for every window length.
struct CrcTables {
    u32 slice[4][256];
    u32 xpow[MAX_WB + 1];
};

constexpr CrcTables make_crc_tables()
{
    CrcTables t{};
    for (u32 i = 0; i < 256; ++i) {
        u32 c = i;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
        t.slice[0][i] = c;
    }
    for (int k = 1; k < 4; ++k)
        for (u32 i = 0; i < 256; ++i) t.slice[k][i] = (t.slice[k - 1][i] >> 8) ^ t.slice[0][t.slice[k - 1][i] & 0xffu];
    u32 v = 0x80000000u;
    for (u32 m = 0; m <= MAX_WB; ++m) {
        t.xpow[m] = v;
        for (int k = 0; k < 8; ++k) v = (v >> 1) ^ (0xEDB88320u & (0u - (v & 1u)));
    }
    return t;
}

__device__ const CrcTables g_crc = make_crc_tables();

struct CodeState {
    u32 count[16];
    u16 first[16]; // first canonical code of each length
    u16 offs[16];  // index in `sorted` of the first symbol of each length
};

// Decode-table entries (32 bits), so one lookup and one shift take a symbol
// with its extra bits:
//   [4:0]   bits to consume: the code plus its extra bits
//   [7:5]   kind: 0 literal (or a valid distance), 1 length resolved in the
//           table (its extra bits were part of the index), 2 end of block,
//           3 invalid symbol, 4 length whose extra bits are read at decode
//           time, 7 no code of at most the root length matches (the
//           long-code path)
//   [11:8]  the code's own length (where its extra bits start)
//   [15:12] extra bits
//   [31:16] literal byte, resolved length, or length/distance base
// The code-length code's table marks a missing code with 0 instead.
template <class C> struct WarpSmem {
    u32 tab[C::DIST_BASE + (1u << C::DIST_BITS)];
    CodeState lcode;
    CodeState dcode;
    u16 lsorted[288];
    u16 dsorted[32];
    u32 run[16];
    u32 pend[C::WB / 32]; // unresolved match destinations in the window
    u64 q[C::MAXQ];       // matches of the window: destination (member offset) | (len | dist << 9) << 32
    alignas(16) u8 win[C::WB + 264];
    // staging (C::STAGE > 0): two ring halves filled by bulk copies, their
    // barriers, and the barriers' phases and a give-up flag kept between members
    alignas(16) u8 ring[C::STAGE ? 2 * C::STAGE : 16];
    u64 bar[2];
    u32 phase, broken;
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
    return (L + extra) | (4u << 5) | (L << 8) | (extra << 12) | (base << 16);
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
        u32 entry = kind == 2 ? 0u : (7u << 5);
        if ((int)L <= root) {
            u32 sym = sorted[cs->offs[L] + ((v >> (root - L)) - cs->first[L])];
            if (kind == 0) {
                entry = lit_entry(sym, L);
                // a length whose extra bits also fit the root: the index holds
                // them (they follow the code in the stream), so resolve it here
                const u32 x = (entry >> 12) & 15u;
                if (((entry >> 5) & 7u) == 4u && L + x <= (u32)root)
                    entry = (L + x) | (1u << 5) | (((entry >> 16) + (((u32)e >> L) & ((1u << x) - 1u))) << 16);
            } else {
                entry = kind == 1 ? dist_entry(sym, L) : cl_entry(sym, L);
            }
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
    template <class SM> __device__ __forceinline__ void attach(const u8 *in, u32 in_len, SM *) { attach(in, in_len); }
    template <class SM> __device__ __forceinline__ void finish(SM *) {}
    __device__ __forceinline__ u32 word(u32 i) const { return i < nwords ? __ldg(base + i) : 0u; }
    __device__ __forceinline__ void seek(u32 p)
    {
        u32 a = p + bit0, w = a >> 5, sh = a & 31u;
        const u32 lo = word(w), hi = word(w + 1); // in order: the staged reader moves forward
        buf = (((u64)hi << 32) | lo) >> sh;
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

// ---- staging the compressed bytes by bulk copies ------------------------------
__device__ __forceinline__ u32 smem_u32(const void *p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(const u64 *bar, u32 parity)
{
    u32 ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// One lane's reader of a member whose compressed bytes are staged in shared
// memory: the member's 16-byte-aligned words go, HALF bytes at a time, into
// the two halves of a ring by cp.async.bulk copies (1-D, global to shared,
// completing on one mbarrier per half); while the chain reads chunk c, chunk
// c + 1 is already being copied.  The copies start at the 16-byte boundary at
// or before the payload and cover whole 16-byte blocks up to its end; the few
// words after the last whole block, and reads past the payload, take the
// plain path of LaneBits.  A wait that does not complete within its bound
// marks the warp's staging broken (`timeout`): the member fails with
// INF_STAGING_TIMEOUT and the warp reads through L1 from then on.
template <class C> struct RingBits {
    static constexpr u32 HALF = C::STAGE;
    enum : u32 { PEND0 = 1, PEND1 = 2, PHASE0 = 4, PHASE1 = 8, BROKEN = 16, TIMEOUT = 32 };
    const u32 *base; // 16-byte-aligned word at or before the payload start
    u32 nwords, bit0;
    u64 buf;
    int cnt;
    u32 nw;
    u8 *ring;     // two halves, then the two barriers (WarpSmem::ring, ::bar)
    u32 bulk;     // bytes from base covered by bulk copies (a multiple of 16)
    u32 hc0, hc1; // chunk held (or in flight) in each half
    u32 ready;    // chunk resident and waited for
    u32 st;       // PEND*, PHASE* (parity of each half's next completion), BROKEN, TIMEOUT

    __device__ __forceinline__ u64 *bar() const { return reinterpret_cast<u64 *>(ring + 2 * HALF); }
    __device__ __forceinline__ void attach(const u8 *in, u32 in_len, WarpSmem<C> *sm)
    {
        static_assert(offsetof(WarpSmem<C>, bar) == offsetof(WarpSmem<C>, ring) + 2 * C::STAGE,
                      "the barriers follow the ring");
        const u64 a = (u64)in, b = a & ~15ull;
        base = (const u32 *)b;
        bit0 = 8u * (u32)(a - b);
        nwords = (bit0 + 8u * in_len + 31u) / 32u;
        const u64 e = (a + in_len) & ~15ull;
        bulk = e > b ? (u32)(e - b) : 0u;
        ring = sm->ring;
        hc0 = hc1 = ready = 0xffffffffu;
        st = sm->phase * PHASE0 | (sm->broken ? BROKEN : 0u);
    }
    __device__ __forceinline__ bool wait(u32 h)
    {
        const u32 par = (st >> (2 + h)) & 1u;
        for (u32 it = 0; it < (1u << 20); ++it) {
            if (mbar_try_wait(bar() + h, par)) {
                st ^= PHASE0 << h;
                st &= ~(PEND0 << h);
                return true;
            }
        }
        st |= BROKEN | TIMEOUT;
        return false;
    }
    __device__ __forceinline__ void issue(u32 c, u32 h)
    {
        const u32 off = c * HALF, bytes = min(HALF, bulk - off);
        u8 *dst = ring + h * HALF;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); // earlier reads of the half come first
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar() + h)), "r"(bytes)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(dst)),
                     "l"((const u8 *)base + off), "r"(bytes), "r"(smem_u32(bar() + h))
                     : "memory");
        st |= PEND0 << h;
        if (h) hc1 = c;
        else hc0 = c;
    }
    __device__ __forceinline__ void make_ready(u32 c)
    {
        const u32 h = c & 1u, g = h ^ 1u;
        if ((h ? hc1 : hc0) != c) {
            if (((st >> h) & 1u) && !wait(h)) return;
            issue(c, h);
        }
        if (((st >> h) & 1u) && !wait(h)) return;
        ready = c;
        const u32 n = c + 1;
        if (n * HALF < bulk && (g ? hc1 : hc0) != n) {
            if (((st >> g) & 1u) && !wait(g)) return;
            issue(n, g);
        }
    }
    __device__ __forceinline__ u32 word(u32 i)
    {
        const u32 o = 4u * i;
        if (o < bulk && !(st & BROKEN)) {
            const u32 c = o / HALF;
            if (c != ready) make_ready(c);
            if (!(st & BROKEN)) return *(const u32 *)(ring + (c & 1u) * HALF + (o & (HALF - 1u)));
        }
        return i < nwords ? __ldg(base + i) : 0u;
    }
    __device__ __forceinline__ u32 timeout() const { return (st & TIMEOUT) ? 1u : 0u; }
    // every copy in flight completed, and the barrier phases kept for the
    // warp's next member (called by the reading lane)
    __device__ __forceinline__ void finish(WarpSmem<C> *sm)
    {
        for (u32 h = 0; h < 2; ++h)
            if (((st >> h) & 1u) && !(st & BROKEN)) wait(h);
        sm->phase = (st >> 2) & 3u;
        sm->broken = (st & BROKEN) ? 1u : 0u;
    }
    __device__ __forceinline__ void seek(u32 p)
    {
        u32 a = p + bit0, w = a >> 5, sh = a & 31u;
        const u32 lo = word(w), hi = word(w + 1); // in order: the staged reader moves forward
        buf = (((u64)hi << 32) | lo) >> sh;
        cnt = 64 - (int)sh;
        nw = w + 2;
    }
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

// The reader a variant uses.
template <class C> using Reader = typename std::conditional<(C::STAGE > 0), RingBits<C>, LaneBits>::type;

// The staging barriers of a warp, set up once per launch by its lane 0.
template <class C> __device__ __forceinline__ void stage_init(WarpSmem<C> *sm)
{
    if constexpr (C::STAGE > 0) {
        if (lane_id() == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(sm->bar)) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(sm->bar + 1)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            sm->phase = 0;
            sm->broken = 0;
        }
        __syncwarp();
    }
}

// Pending-bit helpers over the window buffer.  Destinations of different
// matches can share a word, hence the atomics.
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

// Copies one queued match into the window.  Source bytes before the window
// (wstart) are read from HBM, where earlier windows were written, in groups
// so the loads overlap; bytes inside it come from the window buffer (with a
// distance shorter than the length, from the match's own first bytes).
template <class C> __device__ __forceinline__ void copy_match(WarpSmem<C> *sm, const u8 *out, u32 wstart, u64 q)
{
    const u32 d = (u32)q, len = (u32)(q >> 32) & 511u, s = d - (u32)(q >> 41);
    u32 i = 0;
    while (i < len && s + i < wstart) {
        u32 n = min(min(8u, len - i), wstart - (s + i));
        u8 b[8];
#pragma unroll
        for (u32 x = 0; x < 8; ++x)
            if (x < n) b[x] = out[s + i + x];
#pragma unroll
        for (u32 x = 0; x < 8; ++x)
            if (x < n) sm->win[d + i + x - wstart] = b[x];
        i += n;
    }
    for (; i < len; ++i) sm->win[d + i - wstart] = sm->win[s + i - wstart];
}

// Resolves the window's nq queued matches.  A match whose source lies before
// the window (its first min(len, dist) bytes: later ones are its own) reads
// only final bytes, so all of those are copied in a first pass, one lane per
// match.  The others read the window, where a source byte is final once it is
// a literal, a byte of a match from the first pass, or a byte of another
// window match already copied: those go in parallel rounds, each copying every
// match whose source bytes carry no pending mark; the earliest unresolved one
// is always ready, so rounds make progress.
template <class C> __device__ void resolve(WarpSmem<C> *sm, const u8 *out, u32 wstart, u32 nq)
{
    const u32 lane = lane_id();
    u32 todo = 0;
    for (u32 j = 0, k = lane; k < nq; ++j, k += 32) {
        const u64 q = sm->q[k];
        const u32 d = (u32)q, len = (u32)(q >> 32) & 511u, dist = (u32)(q >> 41);
        if (d - dist + min(len, dist) <= wstart) {
            copy_match(sm, out, wstart, q);
        } else {
            pend_set(sm->pend, d - wstart, d + len - wstart, true);
            todo |= 1u << j;
        }
    }
    __syncwarp();
    while (__any_sync(FRT_FULL_MASK, todo != 0)) {
        u32 ready = 0;
        for (u32 t = todo; t; t &= t - 1) {
            const u32 j = __ffs(t) - 1;
            const u64 q = sm->q[lane + 32 * j];
            const u32 d = (u32)q, len = (u32)(q >> 32) & 511u, dist = (u32)(q >> 41);
            const u32 s = d - dist, e = s + min(len, dist);
            if (!pend_any(sm->pend, max(s, wstart) - wstart, e - wstart)) ready |= 1u << j;
        }
        __syncwarp();
        for (u32 t = ready; t; t &= t - 1) copy_match(sm, out, wstart, sm->q[lane + 32 * (__ffs(t) - 1)]);
        __syncwarp();
        for (u32 t = ready; t; t &= t - 1) {
            const u64 q = sm->q[lane + 32 * (__ffs(t) - 1)];
            const u32 d = (u32)q;
            pend_set(sm->pend, d - wstart, d + ((u32)(q >> 32) & 511u) - wstart, false);
        }
        todo &= ~ready;
        __syncwarp();
    }
}

// Writes the window's n bytes to out[wstart, wstart + n) with coalesced
// stores and advances the member's CRC-32 over them.  The CRC register is
// linear in (state, data): the register after A||B is the register after A
// shifted by |B| bytes (times x^(8|B|) mod P) XOR the register B alone
// produces from zero.  So lane 0 runs the first slice from the member's
// register, every other lane its slice from zero (slicing by 4), each lane
// shifts its result past the bytes after its slice with one multiply by a
// tabulated power, and an XOR across the warp gives the new register.
template <class C> __device__ void write_window(const WarpSmem<C> *sm, u8 *out, u32 wstart, u32 n, u32 *crc)
{
    const u32 lane = lane_id();
    for (u32 j = lane; j < n; j += 32) out[wstart + j] = sm->win[j];
    u32 s = ((n + 31u) / 32u + 3u) & ~3u; // slice length, whole words,
    if ((s & 4u) == 0u) s += 4u;          // an odd number of them: no bank conflicts
    const u32 b0 = min(n, lane * s), b1 = min(n, b0 + s);
    u32 c = lane == 0 ? ~*crc : 0u;
    u32 i = b0;
    for (; i + 4u <= b1; i += 4u) {
        c ^= *(const u32 *)(sm->win + i);
        c = g_crc.slice[3][c & 0xffu] ^ g_crc.slice[2][(c >> 8) & 0xffu] ^ g_crc.slice[1][(c >> 16) & 0xffu] ^
            g_crc.slice[0][c >> 24];
    }
    for (; i < b1; ++i) c = g_crc.slice[0][(c ^ sm->win[i]) & 0xffu] ^ (c >> 8);
    c = gf2_mulmod(g_crc.xpow[n - b1], c);
#pragma unroll
    for (int d = 16; d; d >>= 1) c ^= __shfl_xor_sync(FRT_FULL_MASK, c, d);
    *crc = ~c;
    __syncwarp();
}

// The common symbols, decoded with as little control flow as possible: on
// GB300 lane 0's chain is bound by dependent instructions (about 5.5 cycles
// each), and the SIMT reconvergence bookkeeping that nested branches and
// breaks cost per symbol made up a third of them.  Takes literals and
// lengths resolved in the table, with distances whose code fits the distance
// root, while every symbol is sure to fit (o < lim, and a match adds at most
// 258 bytes); stops in front of any other symbol, which slow_symbol then
// decodes, and leaves a distance it rejects to slow_symbol as well.  One
// exit test at the bottom of the loop, and the refill takes a word loaded
// one refill earlier, so its load latency is off the chain.  A literal is
// followed by a second lookup without going round the loop (the buffer still
// holds a root's worth of bits), as literals come in runs.  A literal whose
// code is longer than the root (rare byte values: 5% of the symbols of a
// short-read BAM) is decoded in the loop too; any other long code leaves it.
template <class C>
__device__ __forceinline__ void fast_run(WarpSmem<C> *sm, Reader<C> &r, u32 pos, u32 lim, u32 &o_io, u32 &nq_io)
{
    constexpr u32 LIT_MASK = C::LIT_MASK, DIST_MASK = C::DIST_MASK, DIST_BASE = C::DIST_BASE, MAXQ = C::MAXQ;
    u64 buf = r.buf;
    int cnt = r.cnt;
    u32 nw = r.nw, o = o_io, nq = nq_io;
    const u32 *tab = sm->tab;
    u32 nextw = r.word(nw); // loaded one refill ahead
    bool go;
    do {
        if (cnt <= 32) {
            buf |= (u64)nextw << cnt;
            cnt += 32;
            ++nw;
            nextw = r.word(nw);
        }
        const u32 e = tab[(u32)buf & LIT_MASK];
        go = false;
        if ((e & 0xE0u) == 0u) { // literal
            sm->win[o++] = (u8)(e >> 16);
            buf >>= (e & 31u);
            cnt -= (int)(e & 31u);
            // a second literal needs no refill: at least 33 - LIT_BITS bits remain
            const u32 e2 = tab[(u32)buf & LIT_MASK];
            if ((e2 & 0xE0u) == 0u) {
                sm->win[o++] = (u8)(e2 >> 16);
                buf >>= (e2 & 31u);
                cnt -= (int)(e2 & 31u);
            }
            go = true;
        } else if ((e & 0xE0u) == 0x20u) { // resolved length
            const u64 b2 = buf >> (e & 31u);
            const u32 d = tab[DIST_BASE + ((u32)b2 & DIST_MASK)];
            const u32 lo = (u32)b2;
            const u32 dist = (d >> 16) + ((lo >> ((d >> 8) & 15u)) & ((1u << ((d >> 12) & 15u)) - 1u));
            const u32 dst = pos + o;
            if ((d & 0xE0u) == 0u && dist <= dst) {
                buf = b2 >> (d & 31u);
                cnt -= (int)((e & 31u) + (d & 31u));
                const u32 len = e >> 16;
                sm->q[nq] = (u64)dst | ((u64)(len | (dist << 9)) << 32);
                ++nq;
                o += len;
                go = nq < MAXQ;
            }
        } else if ((e & 0xE0u) == 0xE0u) { // a code longer than the root: a literal is taken here
            u32 sym;
            const u32 L = decode_long(buf, C::LIT_BITS, &sm->lcode, sm->lsorted, &sym);
            if (L != 0u && sym < 256u) {
                sm->win[o++] = (u8)sym;
                buf >>= L;
                cnt -= (int)L;
                go = true;
            }
        }
    } while (go && o < lim);
    r.buf = buf;
    r.cnt = cnt;
    r.nw = nw;
    o_io = o;
    nq_io = nq;
}

// One symbol (a literal, or a length with its distance) with every check,
// in the order of the reference kernel.  Returns 0 to go on, 1 at the end of
// the block, 2 on an error (status set).
template <class C>
__device__ __forceinline__ int slow_symbol(WarpSmem<C> *sm, Reader<C> &r, u32 pos, u32 cap, u32 &o, u32 &nq, u32 &status)
{
    constexpr int LIT_BITS = C::LIT_BITS, DIST_BITS = C::DIST_BITS;
    constexpr u32 LIT_MASK = C::LIT_MASK, DIST_MASK = C::DIST_MASK, DIST_BASE = C::DIST_BASE;
    r.refill();
    u32 e = sm->tab[(u32)r.buf & LIT_MASK];
    if (((e >> 5) & 7u) == 7u) {
        u32 sym, L = decode_long(r.buf, LIT_BITS, &sm->lcode, sm->lsorted, &sym);
        if (L == 0) {
            r.drop(15); // the reference reads 15 bits before giving up
            status = INF_BAD_CODE;
            return 2;
        }
        e = lit_entry(sym, L);
    }
    const u32 kind = (e >> 5) & 7u;
    if (kind == 0) {
        if (pos + o >= cap) {
            status = INF_OUTPUT_OVERFLOW;
            return 2;
        }
        sm->win[o++] = (u8)(e >> 16);
        r.drop((int)(e & 31u));
        return 0;
    }
    if (kind == 2 || kind == 3) {
        r.drop((int)(e & 31u));
        if (kind == 2) return 1;
        status = INF_BAD_CODE;
        return 2;
    }
    u32 len = e >> 16;
    if (kind == 4) len += (u32)(r.buf >> ((e >> 8) & 15u)) & ((1u << ((e >> 12) & 15u)) - 1u);
    r.drop((int)(e & 31u));
    r.refill();
    u32 d = sm->tab[DIST_BASE + ((u32)r.buf & DIST_MASK)];
    if (((d >> 5) & 7u) == 7u) {
        u32 sym, L = decode_long(r.buf, DIST_BITS, &sm->dcode, sm->dsorted, &sym);
        if (L == 0) {
            r.drop(15);
            status = INF_BAD_DISTANCE;
            return 2;
        }
        d = dist_entry(sym, L);
    }
    if ((d >> 5) & 7u) {
        r.drop((int)(d & 31u));
        status = INF_BAD_DISTANCE;
        return 2;
    }
    u32 dist = (d >> 16) + ((u32)(r.buf >> ((d >> 8) & 15u)) & ((1u << ((d >> 12) & 15u)) - 1u));
    r.drop((int)(d & 31u));
    const u32 dst = pos + o;
    if (dist > dst) {
        status = INF_BAD_DISTANCE;
        return 2;
    }
    if (dst + len > cap) {
        status = INF_OUTPUT_OVERFLOW;
        return 2;
    }
    sm->q[nq] = (u64)dst | ((u64)(len | (dist << 9)) << 32);
    ++nq;
    o += len;
    return 0;
}

// The serial part of one window of a Huffman block, run by the lane that
// holds the member's reader: one table lookup and one shift per symbol,
// literals into the window buffer, matches into the queue, until the buffer
// or the queue is full or the block ends.  Truncation is checked once per
// burst: bits past the payload read as zero, and a symbol that used one is
// where a sequential decoder reports it.  Sets o (bytes), nq (matches),
// status and eob.
template <class C>
__device__ __forceinline__ void decode_symbols(WarpSmem<C> *sm, Reader<C> &r, u32 total, u32 pos, u32 cap, u32 &o,
                                               u32 &nq, u32 &status, int &eob)
{
    constexpr u32 WB = C::WB, MAXQ = C::MAXQ;
    o = 0;
    nq = 0;
    status = INF_OK;
    eob = 0;
    // below lim every symbol fits the window and the declared size
    const u32 room = cap - pos;
    const u32 lim = room >= WB ? WB - 258u : (room > 258u ? room - 258u : 0u);
    while (o < WB - 258u && nq < MAXQ) {
        if (o < lim) {
            fast_run(sm, r, pos, lim, o, nq);
            if (o >= WB - 258u || nq >= MAXQ) break;
        }
        const int rc = slow_symbol(sm, r, pos, cap, o, nq, status);
        if (rc == 1) eob = 1;
        if (rc != 0) break;
    }
    if (r.tell() > total) status = INF_TRUNCATED; // a symbol needed bits past the payload
}

// One window of a Huffman block.  Lane 0 walks the serial chain
// (decode_symbols); the warp then resolves the queued matches in parallel
// rounds and writes the window to HBM with its CRC.
template <class C>
__device__ u32 decode_burst(WarpSmem<C> *sm, Reader<C> &r, u32 total, u8 *out, u32 *pos_io, u32 cap, u32 *crc,
                            int *eob_out)
{
    const u32 lane = lane_id();
    const u32 pos = *pos_io;
    u32 o = 0, nq = 0, status = INF_OK;
    int eob = 0;
    if (lane == 0) decode_symbols(sm, r, total, pos, cap, o, nq, status, eob);
    status = __shfl_sync(FRT_FULL_MASK, status, 0);
    *eob_out = __shfl_sync(FRT_FULL_MASK, eob, 0);
    o = __shfl_sync(FRT_FULL_MASK, o, 0);
    nq = __shfl_sync(FRT_FULL_MASK, nq, 0);
    __syncwarp();
    if (status != INF_OK) return status;
    resolve(sm, out, pos, nq);
    write_window(sm, out, pos, o, crc);
    *pos_io = pos + o;
    return INF_OK;
}

// The block starting at bit `bitpos` of a member, up to its first symbol, by
// the whole warp; lane `leader` holds the member's reader and does the serial
// parts.  A stored block is copied whole (its bytes written and folded into
// the CRC; pos, crc and bitpos advance past it).  A Huffman block gets its
// tables built in sm, bitpos moves past its header and the leader's reader is
// placed at the first symbol (*huffman set).  *last is the block's BFINAL.
// Returns the status; every output is warp-uniform.
template <class C>
__device__ __forceinline__ u32 block_header(WarpSmem<C> *sm, Reader<C> &r, const u8 *in, u32 in_len, u8 *out, u32 cap, u32 &pos,
                            u32 &crc, u32 &bitpos, int *last_out, bool *huffman, const u32 leader)
{
    constexpr int LIT_BITS = C::LIT_BITS, DIST_BITS = C::DIST_BITS;
    constexpr u32 DIST_BASE = C::DIST_BASE, WB = C::WB;
    static_assert((1u << C::DIST_BITS) >= (1u << CL_BITS), "the code-length table shares the distance region");
    // A block's code lengths are read and turned into tables before its first
    // symbol, while the window buffer holds nothing: they live there.
    static_assert(C::WB >= 320, "the code lengths fit the window buffer");
    u8 *const lens = sm->win;
    const u32 lane = lane_id();
    const u32 total = 8u * in_len;
    u32 status = INF_OK;
    int type = 0, last = 0;
    *huffman = false;
    if (lane == leader) {
        if (bitpos + 3 > total) {
            status = INF_TRUNCATED;
        } else {
            r.seek(bitpos);
            last = (int)r.peek(1);
            type = (int)((r.buf >> 1) & 3u);
        }
    }
    status = __shfl_sync(FRT_FULL_MASK, status, leader);
    type = __shfl_sync(FRT_FULL_MASK, type, leader);
    last = __shfl_sync(FRT_FULL_MASK, last, leader);
    *last_out = last;
    if (status != INF_OK) return status;
    bitpos += 3;
    if (type == 3) return INF_BLOCK_TYPE;

    if (type == 0) {
        // ---- stored block: copied by the whole warp -----------------------
        u32 bytepos = (bitpos + 7) / 8, len = 0;
        if (lane == leader) {
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
        status = __shfl_sync(FRT_FULL_MASK, status, leader);
        if (status != INF_OK) return status;
        len = __shfl_sync(FRT_FULL_MASK, len, leader);
        const u8 *src = in + bytepos + 4;
        bitpos = 8u * (bytepos + 4 + len);
        while (len) {
            u32 n = min(len, WB);
            for (u32 j = lane; j < n; j += 32) sm->win[j] = src[j];
            __syncwarp();
            write_window(sm, out, pos, n, &crc);
            pos += n;
            src += n;
            len -= n;
        }
        return INF_OK;
    }

    // ---- Huffman block: tables ------------------------------------------
    if (type == 1) {
        for (int s = lane; s < 288; s += 32) lens[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
        __syncwarp();
        build_table(lens, 288, LIT_BITS, sm->tab, sm->lsorted, &sm->lcode, sm->run, 0);
        lens[lane] = 5;
        __syncwarp();
        build_table(lens, 32, DIST_BITS, sm->tab + DIST_BASE, sm->dsorted, &sm->dcode, sm->run, 1);
    } else {
        int nlen = 0, ndist = 0, ncode = 0;
        u32 bp = bitpos;
        if (lane == leader) {
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
                for (int i = 0; i < 19; ++i) lens[order[i]] = 0;
                for (int i = 0; i < ncode; ++i) {
                    r.refill();
                    if (r.tell() + 3 > total) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    lens[order[i]] = (u8)r.peek(3);
                    r.drop(3);
                }
            }
            bp = r.tell();
        }
        status = __shfl_sync(FRT_FULL_MASK, status, leader);
        if (status != INF_OK) return status;
        nlen = __shfl_sync(FRT_FULL_MASK, nlen, leader);
        ndist = __shfl_sync(FRT_FULL_MASK, ndist, leader);
        __syncwarp();
        // the code-length code must be complete (all-zero counts as
        // complete and fails at first use, as in the reference)
        if (build_table(lens, 19, CL_BITS, sm->tab + DIST_BASE, sm->dsorted, &sm->dcode, sm->run, 2) != 0)
            return INF_BAD_TABLE;
        if (lane == leader) {
            int index = 0;
            r.seek(bp);
            while (index < nlen + ndist) {
                r.refill();
                u32 e = sm->tab[DIST_BASE + r.peek(CL_BITS)];
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
                    lens[index++] = (u8)sym;
                    continue;
                }
                u32 val = 0;
                u32 nb = sym == 16 ? 2 : (sym == 17 ? 3 : 7);
                if (sym == 16) {
                    if (index == 0) {
                        status = INF_BAD_LENGTH_REPEAT;
                        break;
                    }
                    val = lens[index - 1];
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
                while (rep--) lens[index++] = (u8)val;
            }
            if (status == INF_OK && lens[256] == 0) status = INF_BAD_TABLE;
            bp = r.tell();
        }
        status = __shfl_sync(FRT_FULL_MASK, status, leader);
        if (status != INF_OK) return status;
        bitpos = __shfl_sync(FRT_FULL_MASK, bp, leader);
        __syncwarp();
        int rl = build_table(lens, nlen, LIT_BITS, sm->tab, sm->lsorted, &sm->lcode, sm->run, 0);
        if (rl != 0 && (rl < 0 || nlen != (int)sm->lcode.count[0] + 1)) // incomplete only with one code
            return INF_BAD_TABLE;
        int rd = build_table(lens + nlen, ndist, DIST_BITS, sm->tab + DIST_BASE, sm->dsorted, &sm->dcode, sm->run,
                             1);
        if (rd != 0 && (rd < 0 || ndist != (int)sm->dcode.count[0] + 1)) return INF_BAD_TABLE;
    }
    if (lane == leader) r.seek(bitpos);
    *huffman = true;
    return INF_OK;
}

// Inflates one member with the calling warp into out[0, cap).  Returns the
// status; *produced_out and *crc_out are valid in every lane.
template <class C>
__device__ u32 inflate_member_warp(const u8 *in, u32 in_len, u8 *out, u32 cap, WarpSmem<C> *sm, u32 *produced_out,
                                   u32 *crc_out)
{
    constexpr u32 WB = C::WB;
    const u32 lane = lane_id();
    Reader<C> r;
    r.attach(in, in_len, sm);
    for (u32 w = lane; w < WB / 32; w += 32) sm->pend[w] = 0;
    __syncwarp();
    const u32 total = 8u * in_len;
    u32 bitpos = 0; // next unread bit of the stream (warp-uniform)
    u32 pos = 0;    // bytes produced and written
    u32 crc = 0;    // CRC-32 of [0, pos)
    u32 status = INF_OK;
    while (true) {
        int last = 0;
        bool huffman = false;
        status = block_header(sm, r, in, in_len, out, cap, pos, crc, bitpos, &last, &huffman, 0u);
        if (status != INF_OK) break;
        if (huffman) {
            // ---- Huffman block: symbols, a window at a time -----------------
            while (true) {
                int eob = 0;
                status = decode_burst(sm, r, total, out, &pos, cap, &crc, &eob);
                if (status != INF_OK || eob) break;
            }
            if (status != INF_OK) break;
            if (lane == 0) bitpos = r.tell();
            bitpos = __shfl_sync(FRT_FULL_MASK, bitpos, 0);
        }
        if (last) break;
    }
    if constexpr (C::STAGE > 0) {
        u32 to = 0;
        if (lane == 0) {
            r.finish(sm);
            to = r.timeout();
        }
        if (__shfl_sync(FRT_FULL_MASK, to, 0)) status = INF_STAGING_TIMEOUT;
        __syncwarp();
    }
    *produced_out = pos;
    *crc_out = crc;
    return status;
}

template <class C> __host__ __device__ constexpr size_t warp_smem_bytes() { return (sizeof(WarpSmem<C>) + 15) & ~(size_t)15; }

// Plain form: one warp per member of this launch, members in span order.
template <class C>
__global__ void __maxnreg__(C::REGS)
k_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                  const u32 *out_cap, u32 *status, u32 *produced, u32 *crc, u32 n)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 warp = threadIdx.x / 32;
    WarpSmem<C> *wsm = (WarpSmem<C> *)(smem + warp * warp_smem_bytes<C>());
    u32 m = blockIdx.x * (blockDim.x / 32) + warp;
    if (m >= n) return;
    stage_init<C>(wsm);
    u32 p = 0, c = 0;
    u32 st = inflate_member_warp<C>(in + in_off[m], in_len[m], out + out_off[m], out_cap[m], wsm, &p, &c);
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
template <class C>
__global__ void __maxnreg__(C::REGS)
k_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                     const u32 *isize, const u32 *crc_expect, u32 *status, u32 *produced, u32 *crc,
                     const u32 *order, const u64 *n_ptr, u64 n_cap, u64 out_capacity, u32 *queue_head, u32 chunk,
                     unsigned long long *block_err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 warp = threadIdx.x / 32;
    WarpSmem<C> *wsm = (WarpSmem<C> *)(smem + warp * warp_smem_bytes<C>());
    u64 n64 = *n_ptr;
    const u32 n = (u32)(n64 < n_cap ? n64 : n_cap);
    if (chunk == 0) chunk = 1;
    stage_init<C>(wsm);
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
                st = inflate_member_warp<C>(in + in_off[m], in_len[m], out + out_off[m], cap, wsm, &p, &c);
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

// ---- several chains per warp -------------------------------------------------
// One lane walking one member's chain leaves 31 lanes of every instruction of
// the decode loop idle.  The multi-chain form gives a warp K members: lanes
// 0..K-1 each hold one member's reader and decode a window of symbols side by
// side, so an instruction both (or all) take serves K symbols; a literal and a
// match diverge, and SIMT runs both paths, but the common part is shared.  The
// work that is not on the chain (block headers and tables, match resolution,
// the coalesced window write and its CRC) stays warp-cooperative and goes one
// member at a time.  Each member keeps its own tables, window buffer and
// queue (K times the shared memory of the one-chain form per warp).

enum : u32 { SLOT_EMPTY = 0, SLOT_HEADER = 1, SLOT_DECODE = 2, SLOT_DONE = 3 };

// A member in flight in a multi-chain warp.  In shared memory: the
// cooperative phases read every member's state.
struct Slot {
    const u8 *in;
    u8 *out;
    u32 m, in_len, cap;
    u32 pos;    // bytes produced and written
    u32 crc;    // CRC-32 of [0, pos)
    u32 bitpos; // next unread bit at a block header
    u32 status, phase;
    u32 o, nq; // the last burst: bytes in the window buffer, queued matches
    int last, eob;
};

template <class C, int K> __host__ __device__ constexpr size_t multi_slots_bytes()
{
    return (sizeof(Slot) * K + 15) & ~(size_t)15;
}
template <class C, int K> __host__ __device__ constexpr size_t multi_warp_bytes()
{
    return multi_slots_bytes<C, K>() + K * warp_smem_bytes<C>();
}

// K members per warp until no member is left.  PERSISTENT: members come from
// the device work queue (one per pop) and are verified against their
// trailers as they finish; otherwise slot s takes member first + s once.
template <class C, int K, bool PERSISTENT>
__device__ void inflate_multi(unsigned char *wbase, const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                              const u64 *out_off, const u32 *caps, const u32 *crc_expect, u32 *status, u32 *produced,
                              u32 *crc, const u32 *order, u32 n, u64 out_capacity, u32 *queue_head,
                              unsigned long long *block_err, u32 first)
{
    static_assert(K >= 2 && K <= 32, "chains per warp");
    const u32 lane = lane_id();
    Slot *slots = (Slot *)wbase;
    WarpSmem<C> *sms = (WarpSmem<C> *)(wbase + multi_slots_bytes<C, K>());
    constexpr u32 PW = C::WB / 32;
    for (u32 w = lane; w < K * PW; w += 32) sms[w / PW].pend[w % PW] = 0;
    if (lane < K) slots[lane].phase = SLOT_EMPTY;
    Reader<C> r; // lane s < K: the reader of slot s's member
    bool more = true;
    __syncwarp();
    while (true) {
        // 1. a member for every empty slot
        if (more) {
            bool exhausted = false;
            if (lane < K && slots[lane].phase == SLOT_EMPTY) {
                u32 m = 0xffffffffu;
                if (PERSISTENT) {
                    const u32 q = atomicAdd(queue_head, 1u);
                    if (q < n) m = order ? order[q] : q;
                    else exhausted = true;
                } else {
                    m = first + lane;
                }
                if (m < n) {
                    Slot &S = slots[lane];
                    const u32 cap = caps[m];
                    S.m = m;
                    S.in = in + in_off[m];
                    S.in_len = in_len[m];
                    S.out = out + out_off[m];
                    S.cap = cap;
                    S.pos = 0;
                    S.crc = 0;
                    S.bitpos = 0;
                    S.last = 0;
                    S.status = INF_OK;
                    if (PERSISTENT && out_off[m] + cap > out_capacity) {
                        S.status = INF_OUTPUT_OVERFLOW; // sizes changed since the buffers were planned
                        S.phase = SLOT_DONE;
                    } else {
                        S.phase = SLOT_HEADER;
                        r.attach(S.in, S.in_len);
                    }
                }
            }
            if (!PERSISTENT) more = false;
            else if (__any_sync(FRT_FULL_MASK, exhausted)) more = false;
        }
        __syncwarp();
        const u32 busy = __ballot_sync(FRT_FULL_MASK, lane < K && slots[lane].phase != SLOT_EMPTY);
        if (!busy) {
            if (!more) break;
            continue;
        }
        // 2. block headers (and whole stored blocks), one member at a time
        for (u32 t = __ballot_sync(FRT_FULL_MASK, lane < K && slots[lane].phase == SLOT_HEADER); t; t &= t - 1) {
            const u32 s = __ffs(t) - 1;
            Slot &S = slots[s];
            u32 pos = S.pos, c = S.crc, bp = S.bitpos;
            int last = 0;
            bool huffman = false;
            const u32 st = block_header(&sms[s], r, S.in, S.in_len, S.out, S.cap, pos, c, bp, &last, &huffman, s);
            __syncwarp();
            if (lane == 0) {
                S.pos = pos;
                S.crc = c;
                S.bitpos = bp;
                S.last = last;
                S.status = st;
                S.phase = st != INF_OK ? SLOT_DONE : (huffman ? SLOT_DECODE : (last ? SLOT_DONE : SLOT_HEADER));
            }
            __syncwarp();
        }
        // 3. a window of symbols for every decoding member, side by side
        const u32 dec = __ballot_sync(FRT_FULL_MASK, lane < K && slots[lane].phase == SLOT_DECODE);
        if ((dec >> lane) & 1u) {
            Slot &S = slots[lane];
            u32 o, nq, st;
            int eob;
            decode_symbols(&sms[lane], r, 8u * S.in_len, S.pos, S.cap, o, nq, st, eob);
            S.o = o;
            S.nq = nq;
            S.status = st;
            S.eob = eob;
        }
        __syncwarp();
        // 4. each window's matches resolved and its bytes written, one member at a time
        for (u32 t = dec; t; t &= t - 1) {
            const u32 s = __ffs(t) - 1;
            Slot &S = slots[s];
            if (S.status == INF_OK) {
                const u32 pos = S.pos, o = S.o;
                u32 c = S.crc;
                resolve(&sms[s], S.out, pos, S.nq);
                write_window(&sms[s], S.out, pos, o, &c);
                u32 bp = 0;
                if (lane == s) bp = r.tell();
                bp = __shfl_sync(FRT_FULL_MASK, bp, s);
                const int eob = S.eob, last = S.last;
                __syncwarp();
                if (lane == 0) {
                    S.pos = pos + o;
                    S.crc = c;
                    if (eob) {
                        S.bitpos = bp;
                        S.phase = last ? SLOT_DONE : SLOT_HEADER;
                    }
                }
            } else {
                __syncwarp();
                if (lane == 0) S.phase = SLOT_DONE;
            }
            __syncwarp();
        }
        // 5. finished members: results and, in the batched form, the trailer check
        if (lane < K && slots[lane].phase == SLOT_DONE) {
            Slot &S = slots[lane];
            const u32 m = S.m, st = S.status, p = S.pos, c = S.crc;
            status[m] = st;
            produced[m] = p;
            crc[m] = st == INF_OK ? c : 0u;
            if (PERSISTENT) {
                const u32 cap = S.cap;
                unsigned long long code = st != INF_OK ? 5ull : (p != cap ? 4ull : (c != crc_expect[m] ? 3ull : 0ull));
                if (code) atomicMin(block_err, ((unsigned long long)m << 8) | code);
            }
            S.phase = SLOT_EMPTY;
        }
        __syncwarp();
    }
}

// Plain form with K members per warp, members in span order.
template <class C, int K>
__global__ void __maxnreg__(C::REGS)
k_inflate_members_multi(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                        const u32 *out_cap, u32 *status, u32 *produced, u32 *crc, u32 n)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const u32 warp = threadIdx.x / 32;
    const u32 first = (blockIdx.x * (blockDim.x / 32) + warp) * K;
    if (first >= n) return;
    inflate_multi<C, K, false>(smem + warp * multi_warp_bytes<C, K>(), in, in_off, in_len, out, out_off, out_cap,
                               nullptr, status, produced, crc, nullptr, n, ~0ull, nullptr, nullptr, first);
}

// Batched form with K members per warp: the persistent grid of
// k_inflate_persistent, each slot popping its own members (the chunk is one).
template <class C, int K>
__global__ void __maxnreg__(C::REGS)
k_inflate_persistent_multi(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                           const u32 *isize, const u32 *crc_expect, u32 *status, u32 *produced, u32 *crc,
                           const u32 *order, const u64 *n_ptr, u64 n_cap, u64 out_capacity, u32 *queue_head,
                           u32 chunk, unsigned long long *block_err)
{
    extern __shared__ __align__(16) unsigned char smem[];
    (void)chunk;
    const u32 warp = threadIdx.x / 32;
    u64 n64 = *n_ptr;
    const u32 n = (u32)(n64 < n_cap ? n64 : n_cap);
    inflate_multi<C, K, true>(smem + warp * multi_warp_bytes<C, K>(), in, in_off, in_len, out, out_off, isize,
                              crc_expect, status, produced, crc, order, n, out_capacity, queue_head, block_err, 0u);
}

} // namespace

// Standalone CRC of already-inflated members (the reference's crc32_blocks,
// crates/fritillaria-cuda/kernels/crc32.cu:13-38), one warp per member.
__global__ void k_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n)
{
    const u32 *tab = g_crc.slice[0];
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

// ---- variants, tunings, launchers -----------------------------------------
namespace {

using MembersKernel = void (*)(const u8 *, const u64 *, const u32 *, u8 *, const u64 *, const u32 *, u32 *, u32 *,
                               u32 *, u32);
using PersistentKernel = void (*)(const u8 *, const u64 *, const u32 *, u8 *, const u64 *, const u32 *, const u32 *,
                                  u32 *, u32 *, u32 *, const u32 *, const u64 *, u64, u64, u32 *, u32,
                                  unsigned long long *);

struct Variant {
    frt_inflate_variant info;
    MembersKernel members;
    PersistentKernel persistent;
};

template <class C> Variant make_variant()
{
    return {{C::LIT_BITS, C::DIST_BITS, (int32_t)C::WB, (int32_t)C::MAXQ, C::REGS, 1, (int32_t)C::STAGE,
             (uint64_t)warp_smem_bytes<C>()},
            k_inflate_members<C>, k_inflate_persistent<C>};
}

template <class C, int K> Variant make_multi_variant()
{
    return {{C::LIT_BITS, C::DIST_BITS, (int32_t)C::WB, (int32_t)C::MAXQ, C::REGS, K, (int32_t)C::STAGE,
             (uint64_t)multi_warp_bytes<C, K>()},
            k_inflate_members_multi<C, K>, k_inflate_persistent_multi<C, K>};
}

// The compiled variants: the table roots trade shared memory (members in
// flight) against codes that take the long path; the window buffer and its
// queue trade shared memory against bursts per member; a register cap (80:
// no spills; 72, 64 and 56: up to ~120 spilled bytes) lets more CTAs fit an SM.
// Variant 0 is the default before any tuning.
const Variant kVariants[] = {
    make_variant<Cfg<10, 8, 2048, 384>>(),     make_variant<Cfg<9, 8, 2048, 384>>(),
    make_variant<Cfg<11, 8, 2048, 384>>(),     make_variant<Cfg<10, 8, 1024, 256>>(),
    make_variant<Cfg<9, 7, 1024, 256>>(),      make_variant<Cfg<10, 8, 4096, 768>>(),
    make_variant<Cfg<9, 8, 2048, 384, 80>>(),  make_variant<Cfg<9, 7, 1024, 256, 80>>(),
    make_variant<Cfg<10, 8, 2048, 384, 80>>(), make_variant<Cfg<9, 7, 1024, 256, 72>>(),
    make_variant<Cfg<9, 7, 1024, 192, 64>>(), make_variant<Cfg<9, 7, 1024, 160, 56>>(),
    // several chains per warp (the shared memory per warp is K members')
    make_multi_variant<Cfg<9, 7, 1024, 192, 128>, 2>(), make_multi_variant<Cfg<9, 7, 1024, 192, 128>, 4>(),
    // compressed bytes staged in shared memory by bulk copies (ring halves of 256 bytes)
    make_variant<Cfg<9, 7, 1024, 192, 64, 256>>(),
};
constexpr int kNumVariants = (int)(sizeof(kVariants) / sizeof(kVariants[0]));

std::mutex g_tuning_mu;
frt_inflate_tuning g_tuning = {0, 3, 0, 1, -1};

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

} // namespace

extern "C" int frt_inflate_variant_count(void) { return kNumVariants; }

const frt_inflate_variant *frt_inflate_variant_at(int v) { return v >= 0 && v < kNumVariants ? &kVariants[v].info : nullptr; }

extern "C" int frt_inflate_variant_info(int32_t variant, frt_inflate_variant *out, frt_error *err)
{
    if (!out || variant < 0 || variant >= kNumVariants) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, kNumVariants, (uint64_t)variant, 0, nullptr,
                       "no inflate variant %d (%d compiled)", variant, kNumVariants);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    *out = kVariants[variant].info;
    return FRT_OK;
}

frt_inflate_tuning frt_inflate_default()
{
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    return g_tuning;
}

void frt_inflate_set_default(const frt_inflate_tuning &t)
{
    std::lock_guard<std::mutex> lk(g_tuning_mu);
    g_tuning = t;
}

size_t frt_inflate_smem_bytes(const frt_inflate_tuning &t)
{
    return (size_t)t.warps_per_cta * kVariants[t.variant].info.smem_per_warp;
}

cudaError_t frt_inflate_prepare()
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    for (const Variant &v : kVariants) {
        if ((e = cudaFuncSetAttribute(v.members, cudaFuncAttributeMaxDynamicSharedMemorySize, optin)) != cudaSuccess)
            return e;
        if ((e = cudaFuncSetAttribute(v.persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, optin)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

int frt_inflate_ctas_per_sm(const frt_inflate_tuning &t)
{
    if (t.variant < 0 || t.variant >= kNumVariants || t.warps_per_cta < 1 || t.warps_per_cta > FRT_INFLATE_MAX_WARPS ||
        t.ctas_per_sm < 0 || t.queue_chunk < 1 || t.queue_chunk > FRT_INFLATE_MAX_CHUNK || t.spread_variant < -1 ||
        t.spread_variant >= kNumVariants || (t.spread_variant >= 0 && kVariants[t.spread_variant].info.chains != 1))
        return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kVariants[t.variant].persistent, t.warps_per_cta * 32,
                                                      frt_inflate_smem_bytes(t)) != cudaSuccess)
        return 0;
    if (t.ctas_per_sm > 0 && t.ctas_per_sm < per_sm) per_sm = t.ctas_per_sm;
    return per_sm;
}

int frt_inflate_persistent_grid(const frt_inflate_tuning &t) { return sm_count() * frt_inflate_ctas_per_sm(t); }

extern "C" void frt_inflate_get_default_tuning(frt_inflate_tuning *out)
{
    if (out) *out = frt_inflate_default();
}

extern "C" int frt_inflate_tuning_ctas_per_sm(int device, const frt_inflate_tuning *t)
{
    if (!t || frt::check_device(device, nullptr) != FRT_OK) return 0;
    frt::DeviceGuardLite g(device);
    if (frt_inflate_prepare() != cudaSuccess) return 0;
    return frt_inflate_ctas_per_sm(*t);
}

extern "C" int frt_inflate_set_default_tuning(int device, const frt_inflate_tuning *t, frt_error *err)
{
    if (!t) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null tuning");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    int rc = frt::check_device(device, err);
    if (rc != FRT_OK) return rc;
    if (frt_inflate_tuning_ctas_per_sm(device, t) < 1) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                       "inflate tuning (variant %d, %d warps per CTA, %d CTAs per SM, chunk %d) is invalid or does "
                       "not fit device %d",
                       t->variant, t->warps_per_cta, t->ctas_per_sm, t->queue_chunk, device);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    frt_inflate_set_default(*t);
    return FRT_OK;
}

namespace {
// One-warp CTAs of each variant an SM holds (0: not yet asked), for spread launches.
std::atomic<int> g_spread_ctas[kNumVariants];

// A launch of n members that one wave of one-warp CTAs holds is made one warp
// per CTA, one CTA per member at most: the block scheduler deals CTAs out to
// the SMs evenly, while CTAs of w warps put w members on one SM and leave
// other SMs idle.  A member's decode is a serial chain, so a small launch
// ends with its slowest member: fewer members per SM shorten it.  Returns
// false (t unchanged) where the launch fills the GPU anyway.
bool spread_launch(frt_inflate_tuning &t, u64 n, u32 *grid)
{
    const int v = t.spread_variant >= 0 ? t.spread_variant : t.variant;
    if (kVariants[v].info.chains != 1 || n == 0) return false;
    if (t.warps_per_cta <= 1 && v == t.variant) return false;
    int per_sm = g_spread_ctas[v].load(std::memory_order_relaxed);
    if (per_sm == 0) {
        frt_inflate_tuning one{v, 1, 0, 1, -1};
        per_sm = frt_inflate_ctas_per_sm(one);
        g_spread_ctas[v].store(per_sm > 0 ? per_sm : -1, std::memory_order_relaxed);
    }
    if (per_sm <= 0 || n > (u64)per_sm * (u64)sm_count()) return false;
    t.variant = v;
    t.warps_per_cta = 1;
    t.ctas_per_sm = 0;
    t.queue_chunk = 1;
    *grid = (u32)n;
    return true;
}
} // namespace

cudaError_t frt_launch_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                       const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                       u32 *crc, u32 n, const frt_inflate_tuning &tuned, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    frt_inflate_tuning t = tuned;
    u32 unused = 0;
    spread_launch(t, n, &unused);
    const u32 w = (u32)t.warps_per_cta * (u32)kVariants[t.variant].info.chains; // members per CTA
    kVariants[t.variant].members<<<(n + w - 1) / w, t.warps_per_cta * 32, frt_inflate_smem_bytes(t), s>>>(
        in, in_off, in_len, out, out_off, out_cap, status, produced, crc, n);
    return cudaGetLastError();
}

cudaError_t frt_launch_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out,
                                          const u64 *out_off, const u32 *isize, const u32 *crc_expect, u32 *status,
                                          u32 *produced, u32 *crc, const u32 *order, const u64 *n_ptr, u64 n_cap,
                                          u64 out_capacity, u32 *queue_head, u32 grid, unsigned long long *block_err,
                                          const frt_inflate_tuning &tuned, cudaStream_t s)
{
    // n_cap bounds the members (the device count may be lower): fewer than
    // the tuned grid's warps gives a spread launch of n_cap one-warp CTAs
    frt_inflate_tuning t = tuned;
    if (n_cap < (u64)grid * (u64)tuned.warps_per_cta) spread_launch(t, n_cap, &grid);
    kVariants[t.variant].persistent<<<grid, t.warps_per_cta * 32, frt_inflate_smem_bytes(t), s>>>(
        in, in_off, in_len, out, out_off, isize, crc_expect, status, produced, crc, order, n_ptr, n_cap,
        out_capacity, queue_head, (u32)t.queue_chunk, block_err);
    return cudaGetLastError();
}

cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_crc32_members<<<(n + 7) / 8, 256, 0, s>>>(data, offsets, lengths, out, n);
    return cudaGetLastError();
}
