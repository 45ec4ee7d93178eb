// Raw-DEFLATE inflate of BGZF members, one warp per member, with the CRC-32
// of the output folded in.
//
// Decoding a DEFLATE stream is a serial chain: a symbol's bit position is only
// known once the previous symbol is decoded.  So a member is decoded by one
// lane, and the other 31 lanes are put to work on everything that is not that
// chain:
//   * Huffman decode tables are built by the whole warp in shared memory
//     (counts by shared atomics, symbol sort by __match_any_sync ranking, the
//     table filled entry-parallel from the canonical-code limits);
//   * lane 0 decodes symbols through a 10-bit literal/length table and an
//     8-bit distance table (longer codes take a canonical-limit search), writes
//     literals into a shared-memory output chunk and queues back-references;
//   * the warp then materialises the queued back-references in order, each as
//     a 32-lane copy, and flushes the chunk to HBM with coalesced stores;
//   * stored blocks are copied global->global by the warp;
//   * the CRC-32 of the member is computed in 32 slices and merged by the GF(2)
//     shift-and-xor combine.
// RFC 1951 is the specification; the checks and status codes follow the
// reference kernel (crates/fritillaria-cuda/kernels/inflate.cu:78-458) so a
// stream it rejects is rejected here with the same code.

#include "common.cuh"
#include "inflate.cuh"

namespace {

constexpr int LIT_BITS = 10;
constexpr int DIST_BITS = 8;
constexpr int CL_BITS = 7;

// Length code 257+i: base and extra bits follow the RFC 1951 table, which is
// regular enough to compute.
__device__ __forceinline__ u32 lit_entry(u32 sym, u32 L)
{
    if (sym < 256) return L | (0u << 4) | (sym << 16);
    if (sym == 256) return L | (2u << 4);
    if (sym > 285) return L | (3u << 4); // 286, 287: invalid in the fixed code
    u32 i = sym - 257;
    u32 extra, base;
    if (i == 28) {
        extra = 0;
        base = 258;
    } else if (i < 8) {
        extra = 0;
        base = 3 + i;
    } else {
        extra = (i - 4) >> 2;
        base = ((4u + (i & 3u)) << extra) + 3u;
    }
    return L | (1u << 4) | (extra << 8) | (base << 16);
}

__device__ __forceinline__ u32 dist_entry(u32 sym, u32 L)
{
    if (sym >= 30) return L | (1u << 8); // 30, 31: invalid
    u32 extra = sym < 4 ? 0u : (sym - 2u) >> 1;
    u32 base = sym < 4 ? sym + 1u : ((2u + (sym & 1u)) << extra) + 1u;
    return L | (extra << 4) | (base << 16);
}

__device__ __forceinline__ u32 cl_entry(u32 sym, u32 L) { return L | (sym << 16); }

// One canonical Huffman code as decode state.
struct CodeState {
    u32 count[16];
    u32 first[16]; // first canonical code of each length
    u32 offs[16];  // index in `sorted` of the first symbol of each length
};

struct WarpSmem {
    u32 lit[1 << LIT_BITS];
    u32 dist[1 << DIST_BITS];
    CodeState lcode;
    CodeState dcode;
    u16 lsorted[288];
    u16 dsorted[32];
    u32 run[16];
    u8 lens[320];
    u8 chunk[INF_CHUNK + 264];
    u32 mpos[INF_MAXM];
    u32 mlen[INF_MAXM];
    u32 mdist[INF_MAXM];
};

// Builds a decode table for `n` code lengths in `lens`.  Returns puff's
// construct() result: 0 complete (or all-empty), >0 incomplete, <0
// over-subscribed.  kind: 0 literal/length, 1 distance, 2 code-length code.
__device__ int build_table(const u8 *lens, int n, int root, u32 *table, u16 *sorted, CodeState *cs,
                           u32 *run, int kind)
{
    const u32 lane = lane_id();
    if (lane < 16) cs->count[lane] = 0;
    __syncwarp();
    for (int s = lane; s < n; s += 32) atomicAdd(&cs->count[lens[s]], 1u);
    __syncwarp();
    int left = 1;
    if (lane == 0) {
        u32 code = 0, off = 0;
        cs->first[0] = 0;
        cs->offs[0] = 0;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= (int)cs->count[len];
            if (left < 0) break;
        }
        for (int len = 1; len < 16; ++len) {
            cs->first[len] = code;
            cs->offs[len] = off;
            run[len] = off;
            code = (code + cs->count[len]) << 1;
            off += cs->count[len];
        }
        if ((int)cs->count[0] == n) left = 0;
    }
    left = __shfl_sync(FRT_FULL_MASK, left, 0);
    __syncwarp();
    if (left < 0) return left;
    // Sort symbols by (length, symbol): rank within a 32-symbol group by match.
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
    // Fill: entry e holds the root-bit prefix in LSB-first order; reversed it
    // is the MSB-first code prefix v, and the code length is the smallest L
    // whose left-aligned limit exceeds v.
    u32 lim[16];
#pragma unroll
    for (int l = 1; l < 16; ++l) lim[l] = l <= root ? (cs->first[l] + cs->count[l]) << (root - l) : 0u;
    const int size = 1 << root;
    for (int e = lane; e < size; e += 32) {
        u32 v = __brev((u32)e) >> (32 - root);
        u32 L = 1;
#pragma unroll
        for (int l = 1; l < 16; ++l)
            if (l <= root) L += (v >= lim[l]) ? 1u : 0u;
        u32 entry = 0; // 0: take the long-code path
        if ((int)L <= root) {
            u32 idx = cs->offs[L] + ((v >> (root - L)) - cs->first[L]);
            u32 sym = sorted[idx];
            entry = kind == 0 ? lit_entry(sym, L) : (kind == 1 ? dist_entry(sym, L) : cl_entry(sym, L));
        }
        table[e] = entry;
    }
    __syncwarp();
    return left;
}

// Long-code path: canonical search over lengths root+1..15 using the 15 bits
// at the head of the buffer.  Returns the length (0 if no code matches) and
// the symbol.
__device__ __forceinline__ u32 decode_long(u64 bitbuf, int root, const CodeState *cs, const u16 *sorted,
                                           u32 *sym)
{
    u32 v = __brev((u32)bitbuf & 0x7fffu) >> 17; // 15 MSB-first bits
    for (int l = root + 1; l < 16; ++l) {
        u32 lim = (cs->first[l] + cs->count[l]) << (15 - l);
        if (v < lim) {
            u32 idx = cs->offs[l] + ((v >> (15 - l)) - cs->first[l]);
            *sym = sorted[idx];
            return (u32)l;
        }
    }
    return 0;
}

// Lane-0 bit reader over one member's payload in global memory.
struct BitReader {
    const u32 *wp;   // next aligned word to load
    const u8 *end;   // one past the payload
    u64 buf;
    int cnt;         // valid bits in buf
    long long left;  // payload bits not yet consumed

    __device__ __forceinline__ void init(const u8 *p, u32 len)
    {
        u64 a = (u64)p;
        wp = (const u32 *)(a & ~3ull);
        end = p + len;
        int skip = (int)(a & 3ull);
        u32 w = len ? __ldg(wp) : 0u;
        ++wp;
        buf = (u64)(w >> (8 * skip));
        cnt = 32 - 8 * skip;
        left = 8ll * len;
    }
    __device__ __forceinline__ void refill()
    {
        // A word is loaded only while it still holds payload bytes; past the
        // end the buffer fills with zeros, which `left` rejects if consumed.
        while (cnt <= 32) {
            u32 w = ((const u8 *)wp < end) ? __ldg(wp) : 0u;
            ++wp;
            buf |= (u64)w << cnt;
            cnt += 32;
        }
    }
    __device__ __forceinline__ u32 peek(int n) const { return (u32)buf & ((1u << n) - 1u); }
    __device__ __forceinline__ void drop(int n)
    {
        buf >>= n;
        cnt -= n;
        left -= n;
    }
    // Byte position of the next unconsumed whole byte (after discarding the
    // partial byte), relative to the payload start.
};

__device__ __forceinline__ void warp_copy_global(u8 *dst, const u8 *src, u32 n)
{
    for (u32 j = lane_id(); j < n; j += 32) dst[j] = src[j];
}

} // namespace

// Inflates one member with the calling warp.  Output goes to out[0, cap).
// Returns status; *produced_out and *crc_out are valid in every lane.
__device__ u32 inflate_member_warp(const u8 *in, u32 in_len, u8 *out, u32 cap, void *smem_v,
                                   const u32 *crc_tab, u32 *produced_out, u32 *crc_out)
{
    WarpSmem *sm = (WarpSmem *)smem_v;
    const u32 lane = lane_id();
    BitReader br;
    if (lane == 0) br.init(in, in_len);
    u32 produced = 0; // bytes flushed to `out` (warp-uniform)
    u32 status = INF_OK;
    int last = 0;

    while (true) {
        // ---- block header -------------------------------------------------
        int type = 0;
        if (lane == 0) {
            br.refill();
            if (br.left < 3) {
                status = INF_TRUNCATED;
            } else {
                last = (int)br.peek(1);
                type = (int)((br.buf >> 1) & 3u);
                br.drop(3);
            }
        }
        status = __shfl_sync(FRT_FULL_MASK, status, 0);
        if (status != INF_OK) break;
        type = __shfl_sync(FRT_FULL_MASK, type, 0);
        last = __shfl_sync(FRT_FULL_MASK, last, 0);

        if (type == 3) {
            status = INF_BLOCK_TYPE;
            break;
        }

        if (type == 0) {
            // ---- stored block --------------------------------------------
            u32 pos = 0, len = 0;
            if (lane == 0) {
                // discard the partial byte; the next byte is at (consumed bits)/8
                long long consumed = 8ll * in_len - br.left;
                long long bytepos = (consumed + 7) / 8;
                if (bytepos + 4 > (long long)in_len) {
                    status = INF_TRUNCATED;
                } else {
                    u32 l = (u32)in[bytepos] | ((u32)in[bytepos + 1] << 8);
                    u32 nl = (u32)in[bytepos + 2] | ((u32)in[bytepos + 3] << 8);
                    if (l != (~nl & 0xffffu)) status = INF_STORED_LEN;
                    else if ((u64)bytepos + 4 + l > in_len) status = INF_TRUNCATED;
                    else if ((u64)produced + l > cap) status = INF_OUTPUT_OVERFLOW;
                    pos = (u32)bytepos + 4;
                    len = l;
                    if (status == INF_OK) br.init(in + pos + len, in_len - pos - len);
                    // re-anchor the reader after the stored bytes; `left` then
                    // counts only what follows, and consumed positions are kept
                    // relative to the new anchor through `in`/`in_len` below.
                }
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            pos = __shfl_sync(FRT_FULL_MASK, pos, 0);
            len = __shfl_sync(FRT_FULL_MASK, len, 0);
            warp_copy_global(out + produced, in + pos, len);
            __syncwarp();
            produced += len;
            in += pos + len;
            in_len -= pos + len;
            if (last) break;
            continue;
        }

        // ---- Huffman block: tables -----------------------------------------
        int nlen = 0, ndist = 0;
        if (type == 1) {
            for (int s = lane; s < 288; s += 32) sm->lens[s] = s < 144 ? 8 : (s < 256 ? 9 : (s < 280 ? 7 : 8));
            __syncwarp();
            build_table(sm->lens, 288, LIT_BITS, sm->lit, sm->lsorted, &sm->lcode, sm->run, 0);
            for (int s = lane; s < 32; s += 32) sm->lens[s] = 5;
            __syncwarp();
            build_table(sm->lens, 32, DIST_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 1);
        } else {
            int ncode = 0;
            if (lane == 0) {
                br.refill();
                if (br.left < 14) {
                    status = INF_TRUNCATED;
                } else {
                    nlen = (int)br.peek(5) + 257;
                    ndist = (int)((br.buf >> 5) & 31u) + 1;
                    ncode = (int)((br.buf >> 10) & 15u) + 4;
                    br.drop(14);
                    if (nlen > 286 || ndist > 30) status = INF_BAD_COUNTS;
                }
                if (status == INF_OK) {
                    const u8 order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
                    for (int i = 0; i < 19; ++i) sm->lens[order[i]] = 0;
                    for (int i = 0; i < ncode; ++i) {
                        br.refill();
                        if (br.left < 3) {
                            status = INF_TRUNCATED;
                            break;
                        }
                        sm->lens[order[i]] = (u8)br.peek(3);
                        br.drop(3);
                    }
                }
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            nlen = __shfl_sync(FRT_FULL_MASK, nlen, 0);
            ndist = __shfl_sync(FRT_FULL_MASK, ndist, 0);
            __syncwarp();
            // The code-length code must be complete (an all-zero one counts as
            // complete and fails at its first use, as in the reference).
            int r = build_table(sm->lens, 19, CL_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 2);
            if (r != 0) {
                status = INF_BAD_TABLE;
                break;
            }
            if (lane == 0) {
                int index = 0;
                while (index < nlen + ndist) {
                    br.refill();
                    u32 e = sm->dist[br.peek(CL_BITS)];
                    u32 L = e & 15u;
                    if (L == 0) {
                        // no code: puff reads up to 15 bits before giving up
                        status = br.left < 15 ? INF_TRUNCATED : INF_BAD_CODE;
                        break;
                    }
                    if ((long long)L > br.left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    br.drop((int)L);
                    u32 sym = e >> 16;
                    if (sym < 16) {
                        sm->lens[index++] = (u8)sym;
                        continue;
                    }
                    u32 rep, val = 0;
                    int nb = sym == 16 ? 2 : (sym == 17 ? 3 : 7);
                    if (sym == 16) {
                        if (index == 0) {
                            status = INF_BAD_LENGTH_REPEAT;
                            break;
                        }
                        val = sm->lens[index - 1];
                    }
                    if (br.left < nb) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    rep = (sym == 18 ? 11u : 3u) + br.peek(nb);
                    br.drop(nb);
                    if (index + (int)rep > nlen + ndist) {
                        status = INF_BAD_LENGTH_REPEAT;
                        break;
                    }
                    while (rep--) sm->lens[index++] = (u8)val;
                }
                if (status == INF_OK && sm->lens[256] == 0) status = INF_BAD_TABLE;
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            if (status != INF_OK) break;
            __syncwarp();
            int rl = build_table(sm->lens, nlen, LIT_BITS, sm->lit, sm->lsorted, &sm->lcode, sm->run, 0);
            // incomplete codes are legal only when exactly one symbol is used
            if (rl != 0 && (rl < 0 || nlen != (int)sm->lcode.count[0] + 1)) {
                status = INF_BAD_TABLE;
                break;
            }
            int rd = build_table(sm->lens + nlen, ndist, DIST_BITS, sm->dist, sm->dsorted, &sm->dcode, sm->run, 1);
            if (rd != 0 && (rd < 0 || ndist != (int)sm->dcode.count[0] + 1)) {
                status = INF_BAD_TABLE;
                break;
            }
        }

        // ---- Huffman block: symbols, one output chunk at a time ----------------
        int eob = 0;
        while (true) {
            u32 o = 0, nm = 0;
            if (lane == 0) {
                while (o < INF_CHUNK && nm < INF_MAXM) {
                    br.refill();
                    u32 e = sm->lit[br.peek(LIT_BITS)];
                    u32 L = e & 15u;
                    if (L == 0) {
                        u32 sym;
                        L = decode_long(br.buf, LIT_BITS, &sm->lcode, sm->lsorted, &sym);
                        if (L == 0) {
                            status = br.left < 15 ? INF_TRUNCATED : INF_BAD_CODE;
                            break;
                        }
                        e = lit_entry(sym, L);
                    }
                    if ((long long)L > br.left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    br.drop((int)L);
                    u32 kind = (e >> 4) & 3u;
                    if (kind == 0) {
                        if (produced + o >= cap) {
                            status = INF_OUTPUT_OVERFLOW;
                            break;
                        }
                        sm->chunk[o++] = (u8)(e >> 16);
                        continue;
                    }
                    if (kind == 2) {
                        eob = 1;
                        break;
                    }
                    if (kind == 3) {
                        status = INF_BAD_CODE;
                        break;
                    }
                    u32 ex = (e >> 8) & 15u;
                    if ((long long)ex > br.left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    u32 len = (e >> 16) + br.peek((int)ex);
                    br.drop((int)ex);
                    br.refill();
                    u32 d = sm->dist[br.peek(DIST_BITS)];
                    u32 dl = d & 15u;
                    if (dl == 0) {
                        u32 sym;
                        dl = decode_long(br.buf, DIST_BITS, &sm->dcode, sm->dsorted, &sym);
                        if (dl == 0) {
                            status = br.left < 15 ? INF_TRUNCATED : INF_BAD_DISTANCE;
                            break;
                        }
                        d = dist_entry(sym, dl);
                    }
                    if ((long long)dl > br.left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    br.drop((int)dl);
                    if (d & (1u << 8)) {
                        status = INF_BAD_DISTANCE;
                        break;
                    }
                    u32 dex = (d >> 4) & 15u;
                    if ((long long)dex > br.left) {
                        status = INF_TRUNCATED;
                        break;
                    }
                    u32 dist = (d >> 16) + br.peek((int)dex);
                    br.drop((int)dex);
                    if (dist > produced + o) {
                        status = INF_BAD_DISTANCE;
                        break;
                    }
                    if (produced + o + len > cap) {
                        status = INF_OUTPUT_OVERFLOW;
                        break;
                    }
                    sm->mpos[nm] = o;
                    sm->mlen[nm] = len;
                    sm->mdist[nm] = dist;
                    ++nm;
                    o += len;
                }
            }
            status = __shfl_sync(FRT_FULL_MASK, status, 0);
            eob = __shfl_sync(FRT_FULL_MASK, eob, 0);
            o = __shfl_sync(FRT_FULL_MASK, o, 0);
            nm = __shfl_sync(FRT_FULL_MASK, nm, 0);
            __syncwarp();
            // Back-references in order; each one a warp copy.  A source byte
            // before this chunk is read from HBM/L2, one inside it from smem.
            // The period trick covers overlapping copies (dist < len).
            for (u32 m = 0; m < nm; ++m) {
                u32 p = sm->mpos[m], len = sm->mlen[m], dist = sm->mdist[m];
                for (u32 j = lane; j < len; j += 32) {
                    u32 jj = dist < len ? j % dist : j;
                    long long src = (long long)p - (long long)dist + (long long)jj; // chunk-relative
                    u8 b = src >= 0 ? sm->chunk[src] : out[(long long)produced + src];
                    sm->chunk[p + j] = b;
                }
                __syncwarp();
            }
            // flush the chunk (only bytes that were decoded before an error)
            for (u32 j = lane; j < o; j += 32) out[produced + j] = sm->chunk[j];
            __syncwarp();
            produced += o;
            if (status != INF_OK || eob) break;
        }
        if (status != INF_OK) break;
        if (last) break;
    }

    // ---- CRC-32 over the produced bytes, 32 slices merged in GF(2) -----------
    u32 crc = 0;
    if (status == INF_OK) {
        u32 slice = (produced + 31) / 32;
        u32 b0 = lane * slice;
        u32 b1 = min(produced, b0 + slice);
        u32 c = 0xffffffffu;
        for (u32 i = b0; i < b1; ++i) c = crc_tab[(c ^ out[i]) & 0xffu] ^ (c >> 8);
        c = ~c;
        u32 mylen = b1 > b0 ? b1 - b0 : 0u;
        // tree merge: lane l absorbs lane l+d
        for (int d = 1; d < 32; d <<= 1) {
            u32 oc = __shfl_down_sync(FRT_FULL_MASK, c, d);
            u32 ol = __shfl_down_sync(FRT_FULL_MASK, mylen, d);
            if ((lane & (2 * d - 1)) == 0 && lane + d < 32) {
                c = crc_combine(c, oc, ol);
                mylen += ol;
            }
        }
        crc = __shfl_sync(FRT_FULL_MASK, c, 0);
    }
    *produced_out = produced;
    *crc_out = crc;
    return status;
}

// Shared-memory bytes per warp for the inflate state.
size_t frt_inflate_warp_smem() { return sizeof(WarpSmem); }

__device__ __forceinline__ void init_crc_table(u32 *tab)
{
    for (u32 i = threadIdx.x; i < 256; i += blockDim.x) {
        u32 c = i;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
        tab[i] = c;
    }
}

// Plain form: one warp per member of this launch, members in span order.
__global__ void __launch_bounds__(INF_WARPS_PER_CTA * 32)
k_inflate_members(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                    const u32 *out_cap, u32 *status, u32 *produced, u32 *crc, u32 n)
{
    extern __shared__ __align__(16) unsigned char smem[];
    u32 *crc_tab = (u32 *)smem;
    init_crc_table(crc_tab);
    __syncthreads();
    const u32 warp = threadIdx.x / 32;
    const size_t per_warp = (sizeof(WarpSmem) + 15) & ~(size_t)15;
    void *wsm = smem + 1024 + warp * per_warp;
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
// (`order`, longest first) through an atomic head.  One warp per member.
__global__ void __launch_bounds__(INF_WARPS_PER_CTA * 32)
k_inflate_persistent(const u8 *in, const u64 *in_off, const u32 *in_len, u8 *out, const u64 *out_off,
                       const u32 *out_cap, u32 *status, u32 *produced, u32 *crc, const u32 *order,
                       const u32 *n_ptr, u32 *queue_head, u32 chunk)
{
    extern __shared__ __align__(16) unsigned char smem[];
    u32 *crc_tab = (u32 *)smem;
    init_crc_table(crc_tab);
    __syncthreads();
    const u32 warp = threadIdx.x / 32;
    const size_t per_warp = (sizeof(WarpSmem) + 15) & ~(size_t)15;
    void *wsm = smem + 1024 + warp * per_warp;
    const u32 n = *n_ptr;
    if (chunk == 0) chunk = 1;
    while (true) {
        u32 base = 0;
        if (lane_id() == 0) base = atomicAdd(queue_head, chunk);
        base = __shfl_sync(FRT_FULL_MASK, base, 0);
        if (base >= n) break;
        u32 end = min(n, base + chunk);
        for (u32 q = base; q < end; ++q) {
            u32 m = order ? order[q] : q;
            u32 p = 0, c = 0;
            u32 st = inflate_member_warp(in + in_off[m], in_len[m], out + out_off[m], out_cap[m], wsm, crc_tab, &p, &c);
            if (lane_id() == 0) {
                status[m] = st;
                produced[m] = p;
                crc[m] = st == INF_OK ? c : 0u;
            }
        }
    }
}

// Standalone CRC of already-inflated members (the reference's crc32_blocks,
// crates/fritillaria-cuda/kernels/crc32.cu:13-38), one warp per member.
__global__ void k_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out,
                                             u32 n)
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
    u32 b0 = lane * slice, b1 = min(len, b0 + slice);
    u32 c = 0xffffffffu;
    for (u32 i = b0; i < b1; ++i) c = tab[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    c = ~c;
    u32 mylen = b1 > b0 ? b1 - b0 : 0u;
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
size_t frt_inflate_smem_bytes(int warps) { return 1024 + (size_t)warps * ((sizeof(WarpSmem) + 15) & ~(size_t)15); }

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
                                          const u64 *out_off, const u32 *out_cap, u32 *status, u32 *produced,
                                          u32 *crc, const u32 *order, const u32 *n_ptr, u32 *queue_head,
                                          u32 chunk, u32 grid, cudaStream_t s)
{
    k_inflate_persistent<<<grid, INF_WARPS_PER_CTA * 32, frt_inflate_smem_bytes(INF_WARPS_PER_CTA), s>>>(
        in, in_off, in_len, out, out_off, out_cap, status, produced, crc, order, n_ptr, queue_head, chunk);
    return cudaGetLastError();
}

cudaError_t frt_launch_crc32_members(const u8 *data, const u64 *offsets, const u32 *lengths, u32 *out, u32 n,
                                     cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_crc32_members<<<(n + 7) / 8, 256, 0, s>>>(data, offsets, lengths, out, n);
    return cudaGetLastError();
}
