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
// Lengths are turned into offsets by a device exclusive scan; the copies are a
// warp per record with consecutive lanes on consecutive bytes.

#include <cstring>
#include <vector>

#include "common.cuh"
#include "fields.h"

using namespace frt;

namespace {

constexpr u32 kScanBlock = 1024;

// In-place exclusive scan of a[0, n) per 1024-element block; block totals to part.
__global__ void __launch_bounds__(kScanBlock) k_scan_block(u64 *a, u64 n, u64 *part)
{
    __shared__ u64 warps[32];
    const u64 i = (u64)blockIdx.x * kScanBlock + threadIdx.x;
    const u32 lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const u64 x = i < n ? a[i] : 0ull;
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
    if (i < n) a[i] = before + s - x;
    if (threadIdx.x == kScanBlock - 1) part[blockIdx.x] = before + s;
}

// Exclusive scan of the nb block totals by one block, 1024 at a time.
__global__ void __launch_bounds__(kScanBlock) k_scan_parts(u64 *part, u64 nb)
{
    __shared__ u64 warps[32];
    __shared__ u64 carry;
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
}

__global__ void k_scan_add(u64 *a, u64 n, const u64 *part)
{
    const u64 i = (u64)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) a[i] += part[blockIdx.x];
}

// What each payload of a record spans, relative to the record start.
enum Payload { P_NAME = 0, P_CIGAR = 1, P_SEQ = 2, P_QUAL = 3, P_AUX = 4, P_BASES = 5 };

__device__ __forceinline__ void payload_range(const RecordView &v, u64 i, int which, u32 *from, u32 *len)
{
    const u8 *p = v.buf + v.record_offsets[i];
    switch (which) {
    case P_NAME: {
        const u32 nl = v.name_len[i];
        *from = 36u;
        *len = nl && p[36u + nl - 1u] == 0 ? nl - 1u : nl; // Record::name strips the NUL
        break;
    }
    case P_CIGAR: *from = v.cigar_start[i]; *len = v.sequence_start[i] - v.cigar_start[i]; break;
    case P_SEQ: *from = v.sequence_start[i]; *len = v.quality_start[i] - v.sequence_start[i]; break;
    case P_QUAL: *from = v.quality_start[i]; *len = v.aux_start[i] - v.quality_start[i]; break;
    case P_AUX: *from = v.aux_start[i]; *len = v.record_end[i] - v.aux_start[i]; break;
    default: *from = v.sequence_start[i]; *len = v.seq_len[i]; break; // bases: one byte each
    }
}

// lens[i] = the payload's length for i < n, lens[n] = 0 (the scan makes it the total).
__global__ void k_payload_lengths(RecordView v, int which, u64 *lens)
{
    const u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > v.n) return;
    if (i == v.n) {
        lens[i] = 0;
        return;
    }
    u32 from, len;
    payload_range(v, i, which, &from, &len);
    lens[i] = len;
}

__global__ void k_copy_payload(RecordView v, int which, const u64 *offs, u8 *out)
{
    const u64 r = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= v.n) return;
    const u32 lane = threadIdx.x & 31u;
    u32 from, len;
    payload_range(v, r, which, &from, &len);
    const u8 *src = v.buf + v.record_offsets[r] + from;
    u8 *dst = out + offs[r];
    for (u32 j = lane; j < len; j += 32) dst[j] = src[j];
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

__global__ void k_unpack_bases(RecordView v, const u64 *offs, u8 *out)
{
    const u64 r = ((u64)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= v.n) return;
    const u32 lane = threadIdx.x & 31u, l = v.seq_len[r];
    const u8 *packed = v.buf + v.record_offsets[r] + v.sequence_start[r];
    u8 *dst = out + offs[r];
    for (u32 j = lane; 2u * j < l; j += 32) {
        const u32 b = packed[j];
        dst[2u * j] = base_of(b >> 4);
        if (2u * j + 1u < l) dst[2u * j + 1u] = base_of(b & 15u);
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

// Exclusive scan of lens[0, n] in place (lens[n] becomes the total).
int scan_u64(u64 *lens, u64 n1, cudaStream_t st, Temp &tmp, frt_error *err)
{
    const u64 nb = (n1 + kScanBlock - 1) / kScanBlock;
    u64 *part = nullptr;
    int rc = tmp.get(&part, nb, err);
    if (rc) return rc;
    k_scan_block<<<(unsigned)nb, kScanBlock, 0, st>>>(lens, n1, part);
    k_scan_parts<<<1, kScanBlock, 0, st>>>(part, nb);
    k_scan_add<<<(unsigned)nb, kScanBlock, 0, st>>>(lens, n1, part);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FRT_OK : cuda_fail(err, e, "scanning payload lengths");
}

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
    std::vector<int> payloads; // which payload each (offsets, data) pair holds
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
        payloads = {P_BASES};
        break;
    case FIELDS_COMPACT:
        widths = kCompactWidths, n_cols = FRT_COMPACT_COL_COUNT, format = FMT_COMPACT;
        payloads = {P_NAME, P_CIGAR, P_SEQ, P_QUAL, P_AUX};
        break;
    default:
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "unknown record-field operation %d", op);
        return FRT_ERR_INVALID_ARGUMENT;
    }

    // Payload offsets: lengths, scan, totals back to the host to size the result.
    std::vector<u64 *> offs(payloads.size(), nullptr);
    std::vector<u64> totals(payloads.size(), 0);
    if (!payloads.empty()) {
        const unsigned grid = (unsigned)((n + 1 + 255) / 256);
        u64 *d_tot = nullptr;
        if ((rc = tmp.get(&d_tot, payloads.size(), err))) return rc;
        for (size_t k = 0; k < payloads.size(); ++k) {
            if ((rc = tmp.get(&offs[k], n + 1, err))) return rc;
            k_payload_lengths<<<grid, 256, 0, st>>>(v, payloads[k], offs[k]);
            if ((rc = scan_u64(offs[k], n + 1, st, tmp, err))) return rc;
            if ((e = cudaMemcpyAsync(d_tot + k, offs[k] + n, 8, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
                return cuda_fail(err, e, "collecting payload totals");
        }
        if ((e = cudaMemcpyAsync(totals.data(), d_tot, 8 * payloads.size(), cudaMemcpyDeviceToHost, st)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(err, e, "reading payload totals");
        for (size_t k = 0; k < payloads.size(); ++k) {
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
    const unsigned tgrid = (unsigned)((n + 255) / 256), wgrid = (unsigned)((n * 32 + 255) / 256);
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
        default:
            for (size_t k = 0; k < payloads.size(); ++k) {
                if ((e = cudaMemcpyAsync(col((int)(2 * k)), offs[k], 8 * (n + 1), cudaMemcpyDeviceToDevice, st)) !=
                    cudaSuccess)
                    return fail(cuda_fail(err, e, "placing payload offsets"));
                if (payloads[k] == P_BASES)
                    k_unpack_bases<<<wgrid, 256, 0, st>>>(v, offs[k], col((int)(2 * k + 1)));
                else
                    k_copy_payload<<<wgrid, 256, 0, st>>>(v, payloads[k], offs[k], col((int)(2 * k + 1)));
            }
        }
    } else {
        for (size_t k = 0; k < payloads.size(); ++k) // one offset, 0
            if ((e = cudaMemsetAsync(col((int)(2 * k)), 0, 8, st)) != cudaSuccess)
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
