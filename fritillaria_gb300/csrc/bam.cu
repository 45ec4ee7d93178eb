// BAM record boundaries and columnar decode on device.
//
// The record chain is serial (record n+1 starts where record n ends), and on
// BAMs whose BGZF members start mid-record (writers that pack members full)
// the reference's speculation from member starts fails for almost every
// member and its single-thread reconcile walks the whole batch
// (crates/fritillaria-cuda/kernels/bam_decode.cu:154-216).  This file removes
// that serial walk:
//
//   1. spec: one warp per member searches the member for its first plausible
//      record start (a 32-offset sieve with a strict validator: block_size,
//      refID/next_refID range, positions, NUL-terminated name, declared fields
//      fit, and the following record validates too) and walks the chain from
//      there to the member end, recording record offsets in scratch;
//   2. reconcile: one CTA proves the chain.  The true arrival into member m is
//      max(start, lands of earlier members that hold a record start) -- a
//      prefix max, computed block-wide.  Member m is proven when its
//      speculative entry equals its arrival (or it is covered by an earlier
//      record); the first member that is not proven is walked from its true
//      arrival by one thread, and the proof resumes after it.  Correctness
//      never depends on the speculation: a speculative walk is only adopted
//      from a proven boundary, as in the reference (blocked.rs:10-37).
//   3. decode: one warp per member writes its records' columns, lanes over
//      records, including the aux-tag count; a second pass writes the aux-tag
//      directory after an exclusive scan of the counts.
//
// Semantics (record validity, tail, Malformed position) follow
// crates/fritillaria-bam/src/columnar/blocked.rs:106-282.

#include "bam.cuh"
#include "common.cuh"

namespace {

constexpr u64 INF64 = 0xffffffffffffffffull;

// fields_fit (blocked.rs:106-131; kernels/bam_decode.cu:63-73)
__device__ __forceinline__ bool fields_fit(const u8 *buf, u64 start, u64 end)
{
    u32 name_len = buf[start + 12];
    if (name_len == 0u) return false;
    u64 n_cigar = ld_u16le(buf + start + 16);
    u64 l_seq = ld_u32le(buf + start + 20);
    u64 need = 36ull + name_len + 4ull * n_cigar + (l_seq + 1ull) / 2ull + l_seq;
    return start + need <= end;
}

// A strict plausibility test for a record starting at p.  Every condition
// holds for a well-formed record, so a true boundary is never rejected; it is
// only a hint, the proof is the reconcile.
__device__ __forceinline__ bool plausible(const u8 *buf, u64 len, u64 p, int n_ref)
{
    if (p + 36 > len) return false;
    u32 bs = ld_u32le(buf + p);
    if (bs < 32u) return false;
    int ref = (int)ld_u32le(buf + p + 4);
    int pos = (int)ld_u32le(buf + p + 8);
    int nref = (int)ld_u32le(buf + p + 24);
    int npos = (int)ld_u32le(buf + p + 28);
    if (ref < -1 || ref >= n_ref || nref < -1 || nref >= n_ref) return false;
    if (pos < -1 || npos < -1) return false;
    u32 name_len = buf[p + 12];
    if (name_len == 0) return false;
    if (!fields_fit(buf, p, p + 4ull + bs)) return false;
    u64 nul = p + 36 + name_len - 1;
    if (nul < len && buf[nul] != 0) return false;
    // QNAME is printable ([!-~]); the first 16 characters are checked
    u32 nchk = min(name_len - 1, 16u);
    for (u32 k = 0; k < nchk && p + 36 + k < len; ++k) {
        u32 c = buf[p + 36 + k];
        if (c < 0x21u || c > 0x7eu) return false;
    }
    return true;
}

struct Seg {
    u64 land;
    u32 count;
    int complete;
    int valid;
};

// walk_segment (blocked.rs:139-179), recording in-member offsets.
__device__ Seg walk_record(const u8 *buf, u64 len, u64 from, u64 until, u64 mstart, u16 *rec, u32 cap)
{
    Seg s{from, 0u, 1, 1};
    u64 cur = from;
    for (;;) {
        if (cur >= until) {
            s.land = cur;
            s.complete = 1;
            return s;
        }
        if (cur + 4 > len) {
            s.land = cur;
            s.complete = 0;
            return s;
        }
        u32 bs = ld_u32le(buf + cur);
        if (bs < 32u) {
            s.land = cur;
            s.valid = 0;
            return s;
        }
        u64 end = cur + 4ull + bs;
        if (end > len) {
            s.land = cur;
            s.complete = 0;
            return s;
        }
        if (!fields_fit(buf, cur, end)) {
            s.land = cur;
            s.valid = 0;
            return s;
        }
        if (s.count < cap) rec[s.count] = (u16)(cur - mstart);
        s.count++;
        cur = end;
    }
}

} // namespace

// Phase 1 for member m: the first plausible record start, then the walk to
// the member end.  Called by one whole warp.
__device__ void spec_member(const u8 *buf, u64 len, const u64 *starts, u32 m, u64 start, int n_ref, u64 *entry,
                            u32 *count, u64 *land, u8 *flags, u16 *scratch)
{
    const u32 lane = lane_id();
    u64 ms = starts[m], me = starts[m + 1];
    u64 e = INF64;
    if (me <= start) {
        // entirely before the first record: nothing starts here
    } else if (ms <= start) {
        e = start;
    } else {
        // 128 offsets a turn, four a lane.  plausible() needs ref_id in
        // [-1, n_ref), which random bytes almost never hold, so each lane first
        // builds its four ref_id words from two aligned word loads and runs the
        // full test only where that passes.  A word outside [0, len) reads as 0
        // (the full test then rejects the offset: its header would pass len);
        // the ref_id words of any offset with a whole header lie inside.
        const long long A = (long long)(((uintptr_t)(buf + ms) & ~(uintptr_t)3) - (uintptr_t)buf);
        for (long long base = A; base < (long long)me; base += 128) {
            const long long wo = base + 4ll * lane + 4ll;
            const u32 w0 = wo >= 0 && wo + 4 <= (long long)len ? *(const u32 *)(buf + wo) : 0u;
            const u32 w1 = wo + 4 >= 0 && wo + 8 <= (long long)len ? *(const u32 *)(buf + wo + 4) : 0u;
            u32 first = 4;
#pragma unroll
            for (u32 k = 0; k < 4u; ++k) {
                const u32 ref = k ? __funnelshift_r(w0, w1, 8u * k) : w0;
                const long long ps = base + 4ll * lane + k;
                if (first == 4 && ps >= (long long)ms && ps < (long long)me && ref + 1u <= (u32)n_ref) {
                    const u64 p = (u64)ps;
                    bool ok = plausible(buf, len, p, n_ref);
                    if (ok) {
                        // the next two records must validate as well, wherever they
                        // fall in the batch (a decoy's length usually lands far away)
                        u64 q = p + 4ull + ld_u32le(buf + p);
                        for (int j = 0; j < 2 && ok && q + 36 <= len; ++j) {
                            ok = plausible(buf, len, q, n_ref);
                            q += 4ull + ld_u32le(buf + q);
                        }
                    }
                    if (ok) first = k;
                }
            }
            const u32 hit = __ballot_sync(FRT_FULL_MASK, first < 4u);
            if (hit) {
                const u32 src = (u32)(__ffs(hit) - 1);
                e = (u64)(base + 4ll * src + __shfl_sync(FRT_FULL_MASK, first, src));
                break;
            }
        }
    }
    Seg s{e, 0u, 1, 1};
    if (lane == 0 && e != INF64) s = walk_record(buf, len, e, me, ms, scratch + (size_t)m * FRT_SCAN_CAP, FRT_SCAN_CAP);
    if (lane == 0) {
        entry[m] = e;
        count[m] = s.count;
        land[m] = e == INF64 ? 0ull : s.land;
        flags[m] = (u8)((s.complete ? 1 : 0) | (s.valid ? 2 : 0));
    }
}

// Phase 1.  One warp per member.
__global__ void k_bam_spec(const u8 *buf, u64 len, const u64 *starts, u32 n_members, u64 start,
                                        int n_ref, u64 *entry, u32 *count, u64 *land, u8 *flags, u16 *scratch,
                                        const u64 *start_dev, const int *nref_dev)
{
    u32 m = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (m >= n_members) return;
    if (start_dev) start = *start_dev;
    if (nref_dev) n_ref = *nref_dev < 0 ? (1 << 24) : *nref_dev;
    spec_member(buf, len, starts, m, start, n_ref, entry, count, land, flags, scratch);
}

// Phase 1 over many segments (independent record chains, each over its own
// members): segment s owns members [seg[s].m0, seg[s].m0 + seg[s].n) of the
// per-member arrays and the n + 1 starts at starts + seg[s].m0 + s.
__global__ void k_bam_spec_seg(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_total, int n_ref,
                               const u64 *starts, u64 *entry, u32 *count, u64 *land, u8 *flags, u16 *scratch)
{
    u32 g = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (g >= n_total) return;
    u32 si = seg_of[g];
    FrtScanSeg sg = seg[si];
    u32 j = g - sg.m0;
    spec_member(buf, sg.len, starts + sg.m0 + si, j, sg.start, n_ref, entry + sg.m0, count + sg.m0, land + sg.m0,
                flags + sg.m0, scratch + (size_t)sg.m0 * FRT_SCAN_CAP);
}

// Phase 2 for one record chain, by one CTA of 1024 threads.  totals =
// {n_records, tail, status, fallbacks}.
__device__ void reconcile_chain(const u8 *buf, u64 len, const u64 *starts, u32 n_members, u64 start, u64 *entry,
                                u32 *count, u64 *land, u8 *flags, u16 *scratch, u32 *first_index, u64 *totals)
{
    __shared__ u64 s_warp[32];
    __shared__ u64 s_carry;
    __shared__ u32 s_bad;
    __shared__ u32 s_stop;   // 0 running, 1 truncated (tail), 2 malformed
    __shared__ u64 s_tail;
    __shared__ u32 s_fallbacks;
    __shared__ u32 s_cnt_warp[32];
    __shared__ u64 s_total;
    const u32 tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
        s_carry = start;
        s_stop = 0;
        s_tail = 0;
        s_fallbacks = 0;
    }
    __syncthreads();
    u32 base = 0;
    u32 stop_at = n_members; // members >= stop_at hold no records
    while (base < n_members) {
        u32 m = base + tid;
        u64 ms = 0, me = 0, L = 0, e = INF64;
        u8 f = 3;
        if (m < n_members) {
            ms = starts[m];
            me = starts[m + 1];
            e = entry[m];
            f = flags[m];
            if (e != INF64) L = (f & 1) ? land[m] : INF64;
        }
        // block-wide inclusive prefix max of L
        u64 x = L;
        for (int d = 1; d < 32; d <<= 1) {
            u64 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
            if (lane >= (u32)d) x = max(x, y);
        }
        if (lane == 31) s_warp[wid] = x;
        if (tid == 0) s_bad = 0xffffffffu;
        __syncthreads();
        if (wid == 0) {
            u64 w = s_warp[lane];
            for (int d = 1; d < 32; d <<= 1) {
                u64 y = __shfl_up_sync(FRT_FULL_MASK, w, d);
                if (lane >= (u32)d) w = max(w, y);
            }
            s_warp[lane] = w;
        }
        __syncthreads();
        u64 excl_in_warp = __shfl_up_sync(FRT_FULL_MASK, x, 1);
        u64 excl = lane ? excl_in_warp : 0ull;
        if (wid) excl = max(excl, s_warp[wid - 1]);
        u64 arrival = max(s_carry, excl);
        bool bad = false;
        if (m < n_members) {
            bool covered = arrival >= me;
            if (covered) bad = (e != INF64) && (L > arrival);
            else bad = (e != arrival) || !(f & 2) || !(f & 1);
        }
        if (bad) atomicMin(&s_bad, m);
        __syncthreads();
        u32 b = s_bad;
        // Members before the first unproven one are final.  A covered member
        // whose speculative entry was a decoy inside an earlier record holds
        // no records.
        if (m < n_members && m < b && arrival >= me && e != INF64) {
            entry[m] = INF64;
            count[m] = 0;
        }
        if (b == 0xffffffffu) {
            u64 chunk_max = s_warp[31];
            __syncthreads();
            if (tid == 0) s_carry = max(s_carry, chunk_max);
            __syncthreads();
            base += blockDim.x;
            continue;
        }
        // Member b is the first that is not proven: fix it serially.
        if (m == b) {
            u64 ms_b = ms, me_b = me;
            if (arrival >= me_b) {
                // covered by an earlier record: the speculative entry was a decoy
                entry[b] = INF64;
                count[b] = 0;
                land[b] = 0;
                flags[b] = 3;
            } else if (e == arrival && (f & 2) && !(f & 1)) {
                // proven walk that runs into the buffer end: the tail
                s_stop = 1;
                s_tail = land[b];
            } else if (e == arrival && !(f & 2)) {
                // proven walk that meets a malformed record
                s_stop = 2;
                s_tail = arrival;
            } else {
                Seg s = walk_record(buf, len, arrival, me_b, ms_b, scratch + (size_t)b * FRT_SCAN_CAP, FRT_SCAN_CAP);
                entry[b] = arrival;
                count[b] = s.count;
                land[b] = s.land;
                flags[b] = (u8)((s.complete ? 1 : 0) | (s.valid ? 2 : 0));
                s_fallbacks++;
                if (!s.valid) {
                    s_stop = 2;
                    s_tail = arrival;
                } else if (!s.complete) {
                    s_stop = 1;
                    s_tail = s.land;
                }
            }
            s_carry = arrival;
        }
        __syncthreads();
        if (s_stop) {
            stop_at = s_stop == 1 ? b + 1 : b;
            break;
        }
        base = b; // resume the proof at the fixed member, carry = its arrival
        __syncthreads();
    }
    __syncthreads();
    // Counts of proven members, exclusive prefix into first_index.
    if (tid == 0) s_total = 0;
    __syncthreads();
    for (u32 cb = 0; cb < n_members; cb += blockDim.x) {
        u32 m = cb + tid;
        u32 c = 0;
        if (m < n_members) {
            u64 e = entry[m];
            // a member holds records if it was proven with an entry; covered
            // decoys were cleared above; members after a stop hold none
            bool proven = m < stop_at && e != INF64;
            if (proven) c = count[m];
            if (!proven && m < n_members) count[m] = 0;
        }
        u32 x = c;
        for (int d = 1; d < 32; d <<= 1) {
            u32 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
            if (lane >= (u32)d) x += y;
        }
        if (lane == 31) s_cnt_warp[wid] = x;
        __syncthreads();
        if (wid == 0) {
            u32 w = s_cnt_warp[lane];
            for (int d = 1; d < 32; d <<= 1) {
                u32 y = __shfl_up_sync(FRT_FULL_MASK, w, d);
                if (lane >= (u32)d) w += y;
            }
            s_cnt_warp[lane] = w;
        }
        __syncthreads();
        u32 excl = x - c + (wid ? s_cnt_warp[wid - 1] : 0u);
        if (m < n_members) first_index[m] = (u32)(s_total + excl);
        __syncthreads();
        if (tid == 0) s_total += s_cnt_warp[31];
        __syncthreads();
    }
    if (tid == 0) {
        totals[0] = s_total;
        totals[1] = s_stop ? s_tail : s_carry;
        totals[2] = s_stop == 2 ? 1ull : 0ull;
        totals[3] = s_fallbacks;
    }
}

// Phase 2.  One CTA of 1024 threads.
__global__ void __launch_bounds__(1024)
k_bam_reconcile(const u8 *buf, u64 len, const u64 *starts, u32 n_members, u64 start, u64 *entry, u32 *count,
                  u64 *land, u8 *flags, u16 *scratch, u32 *first_index, u64 *totals, const u64 *start_dev)
{
    if (start_dev) start = *start_dev;
    reconcile_chain(buf, len, starts, n_members, start, entry, count, land, flags, scratch, first_index, totals);
}

// Phase 2 over many segments: one CTA per segment, totals at totals + 4 * s.
__global__ void __launch_bounds__(1024)
k_bam_reconcile_seg(const u8 *buf, const FrtScanSeg *seg, const u64 *starts, u64 *entry, u32 *count, u64 *land,
                    u8 *flags, u16 *scratch, u32 *first_index, u64 *totals)
{
    u32 si = blockIdx.x;
    FrtScanSeg sg = seg[si];
    reconcile_chain(buf, sg.len, starts + sg.m0 + si, sg.n, sg.start, entry + sg.m0, count + sg.m0, land + sg.m0,
                    flags + sg.m0, scratch + (size_t)sg.m0 * FRT_SCAN_CAP, first_index + sg.m0, totals + 4ull * si);
}

// Region filter (crates/fritillaria-bam/src/io/reader/query.rs:97-122 with the
// chunk bound of the csi query reader): a record is kept when its start
// virtual offset is below its segment's chunk end, its reference is `ref`
// and [pos + 1, pos + span] meets [beg, end] (span from the CIGAR's
// M/D/N/=/X, at least 1).  One warp per member, lanes over its records.
__device__ __forceinline__ bool region_keep(const u8 *buf, u64 rec, u64 voff, const FrtScanSeg &sg)
{
    if (voff >= sg.chunk_end) return false;
    int ref = (int)ld_u32le(buf + rec + 4), pos = (int)ld_u32le(buf + rec + 8);
    if (ref != sg.ref || pos < 0) return false;
    u32 name_len = buf[rec + 12], n_cigar = ld_u16le(buf + rec + 16);
    u64 span = 0;
    for (u32 k = 0; k < n_cigar; ++k) {
        u32 op = ld_u32le(buf + rec + 36 + name_len + 4 * k), kind = op & 15u;
        if (kind == 0 || kind == 2 || kind == 3 || kind == 7 || kind == 8) span += op >> 4;
    }
    if (span == 0) span = 1;
    u64 a0 = (u64)pos + 1, a1 = a0 + span - 1;
    return a0 <= sg.end && sg.beg <= a1;
}

__device__ __forceinline__ u64 member_voff(const u64 *coff, u32 m, u64 in_member) { return (coff[m] << 16) | in_member; }

__global__ void k_region_count(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_total, const u64 *starts,
                               const u64 *coff, const u32 *count, const u16 *scratch, u32 *kept)
{
    u32 g = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (g >= n_total) return;
    u32 si = seg_of[g];
    FrtScanSeg sg = seg[si];
    const u64 ms = starts[g + si];
    u32 n = count[g], c = 0;
    const u16 *r = scratch + (size_t)g * FRT_SCAN_CAP;
    for (u32 k = lane_id(); k < n; k += 32) {
        u64 rec = ms + r[k];
        c += region_keep(buf, rec, member_voff(coff, g, r[k]), sg);
    }
    for (int o = 16; o; o >>= 1) c += __shfl_down_sync(FRT_FULL_MASK, c, o);
    if (lane_id() == 0) kept[g] = c;
}

__global__ void k_region_emit(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_total,
                              const u64 *starts, const u64 *coff, const u32 *count, const u16 *scratch,
                              const u32 *kept_first, FrtRegionColumns out)
{
    u32 g = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (g >= n_total) return;
    u32 si = seg_of[g];
    FrtScanSeg sg = seg[si];
    const u64 ms = starts[g + si];
    u32 n = count[g], at = kept_first[g];
    const u16 *r = scratch + (size_t)g * FRT_SCAN_CAP;
    const u32 lane = lane_id();
    for (u32 b = 0; b < n; b += 32) {
        u32 k = b + lane;
        bool keep = false;
        u64 rec = 0, voff = 0;
        if (k < n) {
            rec = ms + r[k];
            voff = member_voff(coff, g, r[k]);
            keep = region_keep(buf, rec, voff, sg);
        }
        u32 mask = __ballot_sync(FRT_FULL_MASK, keep);
        if (keep) {
            u32 i = at + __popc(mask & lanemask_lt());
            out.virtual_offset[i] = voff;
            out.record_offset[i] = rec - sg.out_base;
            out.ref_id[i] = (int)ld_u32le(buf + rec + 4);
            out.pos[i] = (int)ld_u32le(buf + rec + 8);
            out.flags[i] = (u16)ld_u16le(buf + rec + 18);
            out.mapq[i] = buf[rec + 13];
            out.seq_len[i] = ld_u32le(buf + rec + 20);
            out.request[i] = sg.request;
        }
        at += __popc(mask);
    }
}

namespace {

// One aux field at `pos` (aux.rs:301-405): returns the offset just past it,
// or 0 when malformed.  Fills type/subtype/value offset/count.
// The first zero byte of rec[q, end), or end.  Long Z strings (MM:Z of an
// ultra-long read runs to 100 KB) go 32 bytes a step through aligned 16-byte
// loads; no load reaches past end.
__device__ __forceinline__ u32 find_nul(const u8 *rec, u32 q, u32 end)
{
    for (; q < end && ((uintptr_t)(rec + q) & 15u); ++q)
        if (rec[q] == 0) return q;
    for (; q + 32u <= end; q += 32u) {
        const uint4 a = *(const uint4 *)(rec + q), b = *(const uint4 *)(rec + q + 16u);
        const u32 m[8] = {__vcmpeq4(a.x, 0u), __vcmpeq4(a.y, 0u), __vcmpeq4(a.z, 0u), __vcmpeq4(a.w, 0u),
                          __vcmpeq4(b.x, 0u), __vcmpeq4(b.y, 0u), __vcmpeq4(b.z, 0u), __vcmpeq4(b.w, 0u)};
        if (m[0] | m[1] | m[2] | m[3] | m[4] | m[5] | m[6] | m[7]) {
#pragma unroll
            for (u32 k = 0; k < 8u; ++k)
                if (m[k]) return q + 4u * k + ((u32)(__ffs(m[k]) - 1) >> 3);
        }
    }
    for (; q < end; ++q)
        if (rec[q] == 0) return q;
    return end;
}

__device__ __forceinline__ u32 aux_field(const u8 *rec, u32 pos, u32 end, u32 *w0, u32 *voff, u32 *cnt)
{
    if (pos + 3 > end) return 0;
    u32 ty = rec[pos + 2];
    u32 v = pos + 3;
    u32 sub = 0, count = 1, next;
    switch (ty) {
    case 'A': case 'c': case 'C': next = v + 1; break;
    case 's': case 'S': next = v + 2; break;
    case 'i': case 'I': case 'f': next = v + 4; break;
    case 'Z': case 'H': {
        const u32 q = find_nul(rec, v, end);
        if (q >= end) return 0;
        count = q - v;
        if (ty == 'H') {
            if (count & 1u) return 0;
            for (u32 h = v; h < q; ++h) {
                u32 c = rec[h];
                bool hex = (c >= '0' && c <= '9') || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F');
                if (!hex) return 0;
            }
        }
        next = q + 1;
        break;
    }
    case 'B': {
        if (v + 5 > end) return 0;
        sub = rec[v];
        count = ld_u32le(rec + v + 1);
        u64 w;
        switch (sub) {
        case 'c': case 'C': w = 1; break;
        case 's': case 'S': w = 2; break;
        case 'i': case 'I': case 'f': w = 4; break;
        default: return 0;
        }
        u64 stop = (u64)v + 5ull + (u64)count * w;
        if (stop > end) return 0;
        next = (u32)stop;
        break;
    }
    default: return 0;
    }
    if (next > end) return 0;
    *w0 = (u32)rec[pos] | ((u32)rec[pos + 1] << 8) | (ty << 16) | (sub << 24);
    *voff = v;
    *cnt = count;
    return next;
}

} // namespace

// Phase 3: columns.  One warp per member, lanes over its records.
__global__ void k_bam_decode(const u8 *buf, const u64 *starts, const u64 *member_coffset, u32 n_members,
                                          const u32 *count, const u32 *first_index, const u16 *scratch,
                                          FrtBamColumnsDev c, u64 rec_cap)
{
    u32 m = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (m >= n_members) return;
    u32 n = count[m];
    if (n == 0) return;
    u64 ms = starts[m];
    u64 vbase = member_coffset ? (member_coffset[m] << 16) : 0ull;
    u32 first = first_index[m];
    const u16 *rec = scratch + (size_t)m * FRT_SCAN_CAP;
    for (u32 k = lane_id(); k < n; k += 32) {
        u32 rel = rec[k];
        u64 r = ms + rel;
        const u8 *p = buf + r;
        u64 i = (u64)first + k;
        if (i >= rec_cap) break;
        u32 bs = ld_u32le(p);
        u32 name_len = p[12];
        u32 n_cigar = ld_u16le(p + 16);
        u32 l_seq = ld_u32le(p + 20);
        c.ref_id[i] = (int)ld_u32le(p + 4);
        c.pos[i] = (int)ld_u32le(p + 8);
        c.name_len[i] = (u8)name_len;
        c.mapq[i] = p[13];
        c.bin[i] = (u16)ld_u16le(p + 14);
        c.n_cigar[i] = (u16)n_cigar;
        c.flags[i] = (u16)ld_u16le(p + 18);
        c.seq_len[i] = l_seq;
        c.mate_ref_id[i] = (int)ld_u32le(p + 24);
        c.mate_pos[i] = (int)ld_u32le(p + 28);
        c.tlen[i] = (int)ld_u32le(p + 32);
        c.record_offsets[i] = r;
        c.virtual_offset[i] = vbase | rel;
        u32 cs = 36u + name_len;
        u32 ss = cs + 4u * n_cigar;
        u32 qs = ss + (l_seq + 1u) / 2u;
        u32 as = qs + l_seq;
        u32 re = 4u + bs;
        c.cigar_start[i] = cs;
        c.sequence_start[i] = ss;
        c.quality_start[i] = qs;
        c.aux_start[i] = as;
        c.record_end[i] = re;
        u32 nt = 0, st = 0, pos = as;
        while (pos < re) {
            u32 w0, vo, cn;
            u32 nx = aux_field(p, pos, re, &w0, &vo, &cn);
            if (!nx) {
                st = 1;
                break;
            }
            ++nt;
            pos = nx;
        }
        c.aux_count[i] = nt;
        c.aux_status[i] = (u8)st;
    }
}

// Phase 4: aux-tag directory, one thread per record, entries at aux_first[i].
__global__ void k_bam_aux_dir(const u8 *buf, const u64 *record_offsets, const u32 *aux_start,
                                           const u32 *record_end, const u32 *aux_count, const u32 *aux_first,
                                           u32 *entries, u64 n, const u64 *n_dev, u64 aux_cap)
{
    u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev && *n_dev < n) n = *n_dev;
    if (i >= n) return;
    if ((u64)aux_first[i] + aux_count[i] > aux_cap) return;
    const u8 *p = buf + record_offsets[i];
    u32 pos = aux_start[i], re = record_end[i], nt = aux_count[i];
    u32 *out = entries + 3ull * aux_first[i];
    for (u32 t = 0; t < nt; ++t) {
        u32 w0, vo, cn;
        u32 nx = aux_field(p, pos, re, &w0, &vo, &cn);
        out[3 * t] = w0;
        out[3 * t + 1] = vo;
        out[3 * t + 2] = cn;
        pos = nx;
    }
}

// Exclusive scan of u32 counts into out[0..n], out[n] = total (three passes).
__global__ void __launch_bounds__(1024) k_scan_partials(const u32 *in, u64 n, u32 *partials)
{
    __shared__ u32 s[32];
    u64 base = (u64)blockIdx.x * 4096;
    u32 acc = 0;
    for (int k = 0; k < 4; ++k) {
        u64 i = base + (u64)k * 1024 + threadIdx.x;
        if (i < n) acc += in[i];
    }
    for (int d = 16; d; d >>= 1) acc += __shfl_down_sync(FRT_FULL_MASK, acc, d);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        u32 v = s[threadIdx.x];
        for (int d = 16; d; d >>= 1) v += __shfl_down_sync(FRT_FULL_MASK, v, d);
        if (threadIdx.x == 0) partials[blockIdx.x] = v;
    }
}

__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32 *s_warp, u32 *total)
{
    const u32 lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    u32 x = v;
    for (int d = 1; d < 32; d <<= 1) {
        u32 y = __shfl_up_sync(FRT_FULL_MASK, x, d);
        if (lane >= (u32)d) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        u32 w = s_warp[lane];
        for (int d = 1; d < 32; d <<= 1) {
            u32 y = __shfl_up_sync(FRT_FULL_MASK, w, d);
            if (lane >= (u32)d) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    u32 excl = x - v + (wid ? s_warp[wid - 1] : 0u);
    *total = s_warp[31];
    __syncthreads();
    return excl;
}

__global__ void __launch_bounds__(1024) k_scan_partials_scan(u32 *partials, u64 n_parts)
{
    __shared__ u32 s_warp[32];
    u32 carry = 0;
    for (u64 b = 0; b < n_parts; b += 1024) {
        u64 i = b + threadIdx.x;
        u32 v = i < n_parts ? partials[i] : 0u;
        u32 tot;
        u32 ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < n_parts) partials[i] = carry + ex;
        carry += tot;
    }
}

__global__ void __launch_bounds__(1024) k_scan_apply(const u32 *in, u64 n, const u32 *partials, u32 *out,
                                                                 u32 *total_out)
{
    __shared__ u32 s_warp[32];
    u64 base = (u64)blockIdx.x * 4096;
    u32 carry = partials[blockIdx.x];
    for (int k = 0; k < 4; ++k) {
        u64 i = base + (u64)k * 1024 + threadIdx.x;
        u32 v = i < n ? in[i] : 0u;
        u32 tot;
        u32 ex = block_exclusive_scan(v, s_warp, &tot);
        if (i < n) out[i] = carry + ex;
        if (i == n) out[i] = carry + ex;
        carry += tot;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0 && total_out) *total_out = carry;
}

// ---- host launchers --------------------------------------------------------
cudaError_t frt_launch_bam_spec(const u8 *buf, u64 len, const u64 *starts, u32 n, u64 start, int n_ref, u64 *entry,
                                u32 *count, u64 *land, u8 *flags, u16 *scratch, cudaStream_t s, const u64 *start_dev,
                                const int *nref_dev)
{
    if (n == 0) return cudaSuccess;
    k_bam_spec<<<(n + 7) / 8, 256, 0, s>>>(buf, len, starts, n, start, n_ref, entry, count, land, flags, scratch,
                                           start_dev, nref_dev);
    return cudaGetLastError();
}

cudaError_t frt_launch_bam_reconcile(const u8 *buf, u64 len, const u64 *starts, u32 n, u64 start, u64 *entry,
                                     u32 *count, u64 *land, u8 *flags, u16 *scratch, u32 *first_index, u64 *totals,
                                     cudaStream_t s, const u64 *start_dev)
{
    k_bam_reconcile<<<1, 1024, 0, s>>>(buf, len, starts, n, start, entry, count, land, flags, scratch, first_index,
                                         totals, start_dev);
    return cudaGetLastError();
}

cudaError_t frt_launch_bam_decode(const u8 *buf, const u64 *starts, const u64 *coff, u32 n, const u32 *count,
                                  const u32 *first_index, const u16 *scratch, const FrtBamColumnsDev &c,
                                  cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_bam_decode<<<(n + 7) / 8, 256, 0, s>>>(buf, starts, coff, n, count, first_index, scratch, c, ~0ull);
    return cudaGetLastError();
}

size_t frt_scan_partials_len(u64 n) { return (size_t)(n / 4096 + 1); }

cudaError_t frt_launch_region_scan(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_segs, u32 n_total,
                                   int n_ref, const u64 *starts, const u64 *coff, u64 *entry, u32 *count, u64 *land,
                                   u8 *flags, u16 *scratch, u32 *first_index, u64 *totals, u32 *kept, cudaStream_t s)
{
    if (n_total == 0 || n_segs == 0) return cudaSuccess;
    unsigned g = (n_total + 7) / 8;
    k_bam_spec_seg<<<g, 256, 0, s>>>(buf, seg, seg_of, n_total, n_ref, starts, entry, count, land, flags, scratch);
    k_bam_reconcile_seg<<<n_segs, 1024, 0, s>>>(buf, seg, starts, entry, count, land, flags, scratch, first_index,
                                                totals);
    k_region_count<<<g, 256, 0, s>>>(buf, seg, seg_of, n_total, starts, coff, count, scratch, kept);
    return cudaGetLastError();
}

cudaError_t frt_launch_region_emit(const u8 *buf, const FrtScanSeg *seg, const u32 *seg_of, u32 n_total,
                                   const u64 *starts, const u64 *coff, const u32 *count, const u16 *scratch,
                                   const u32 *kept_first, const FrtRegionColumns &out, cudaStream_t s)
{
    if (n_total == 0) return cudaSuccess;
    k_region_emit<<<(n_total + 7) / 8, 256, 0, s>>>(buf, seg, seg_of, n_total, starts, coff, count, scratch,
                                                    kept_first, out);
    return cudaGetLastError();
}

// out has n + 1 entries; partials has frt_scan_partials_len(n) entries.
cudaError_t frt_launch_scan_u32(const u32 *in, u64 n, u32 *partials, u32 *out, u32 *total, cudaStream_t s)
{
    u64 parts = frt_scan_partials_len(n);
    k_scan_partials<<<(unsigned)parts, 1024, 0, s>>>(in, n, partials);
    k_scan_partials_scan<<<1, 1024, 0, s>>>(partials, parts);
    k_scan_apply<<<(unsigned)parts, 1024, 0, s>>>(in, n, partials, out, total);
    return cudaGetLastError();
}

cudaError_t frt_launch_bam_aux_dir(const u8 *buf, const u64 *record_offsets, const u32 *aux_start,
                                   const u32 *record_end, const u32 *aux_count, const u32 *aux_first, u32 *entries,
                                   u64 n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_bam_aux_dir<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(buf, record_offsets, aux_start, record_end, aux_count,
                                                                aux_first, entries, n, nullptr, ~0ull);
    return cudaGetLastError();
}

cudaError_t frt_launch_bam_decode_capped(const u8 *buf, const u64 *starts, const u64 *coff, u32 n, const u32 *count,
                                         const u32 *first_index, const u16 *scratch, const FrtBamColumnsDev &c,
                                         u64 rec_cap, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    k_bam_decode<<<(n + 7) / 8, 256, 0, s>>>(buf, starts, coff, n, count, first_index, scratch, c, rec_cap);
    return cudaGetLastError();
}

cudaError_t frt_launch_bam_aux_dir_capped(const u8 *buf, const u64 *record_offsets, const u32 *aux_start,
                                          const u32 *record_end, const u32 *aux_count, const u32 *aux_first,
                                          u32 *entries, const u64 *n_dev, u64 rec_cap, u64 aux_cap, cudaStream_t s)
{
    if (rec_cap == 0) return cudaSuccess;
    k_bam_aux_dir<<<(unsigned)((rec_cap + 255) / 256), 256, 0, s>>>(buf, record_offsets, aux_start, record_end,
                                                                    aux_count, aux_first, entries, rec_cap, n_dev,
                                                                    aux_cap);
    return cudaGetLastError();
}
