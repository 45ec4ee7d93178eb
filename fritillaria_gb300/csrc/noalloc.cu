// Record boundaries of an inflated BAM batch, without allocating.
//
// frt_bam_decode allocates its per-member scratch and its columns with
// stream-ordered cudaMallocAsync.  Some callers cannot do that: a host that
// owns every byte of device memory through its own arena or pool (and must
// not have a library allocating behind its back), code running where
// allocation is forbidden or would break a capture or a memory budget, or a
// pipeline that preallocated its buffers once at start-up.  This entry point
// serves them: the caller passes the inflated bytes, the member offsets and
// the output array, and the scan's scratch lives in one file-scope device
// array of fixed size below.
//
// Limits and sharing:
//   * at most FRT_NOALLOC_MAX_MEMBERS members per call (4 MiB of scratch,
//     held by every GPU that loads the library until the process exits);
//   * each member holds at most 65,536 inflated bytes (BGZF's limit, which
//     sizes the per-member slots of the scratch), the offsets ascend and the
//     last is at most len; a call that breaks this is rejected with
//     FRT_ERR_INVALID_ARGUMENT after the scan, which never writes outside
//     the scratch or the caller's arrays in the meantime;
//   * every call shares that one array, which keeps the last call's
//     contents; calls that overlap on the GPU (two streams, two threads)
//     race on it and must be serialised by the caller;
//   * the first call on a device looks up the array's device address with
//     that device current; make that first call before any stream capture.

#include <cstring>
#include <mutex>

#include "../../include/frt.h"
#include "bam.cuh"
#include "runtime.h"

using namespace frt;

namespace {

constexpr u32 MAX_MEMBERS = FRT_NOALLOC_MAX_MEMBERS;
// per member: entry u64, land u64, count u32, first u32, flags u8; then the
// in-member record offsets (u16 x FRT_SCAN_CAP)
constexpr size_t OFF_ENTRY = 0;
constexpr size_t OFF_LAND = OFF_ENTRY + 8ull * MAX_MEMBERS;
constexpr size_t OFF_TOTALS = OFF_LAND + 8ull * MAX_MEMBERS;
constexpr size_t OFF_COUNT = OFF_TOTALS + 64;
constexpr size_t OFF_FIRST = OFF_COUNT + 4ull * MAX_MEMBERS;
constexpr size_t OFF_FLAGS = OFF_FIRST + 4ull * MAX_MEMBERS;
constexpr size_t OFF_RECS = (OFF_FLAGS + MAX_MEMBERS + 255) & ~(size_t)255;
constexpr size_t SCRATCH_BYTES = OFF_RECS + 2ull * FRT_SCAN_CAP * MAX_MEMBERS;

static __device__ __align__(256) unsigned char g_scan_scratch[SCRATCH_BYTES];

// Device address of g_scan_scratch per device, looked up once with that
// device current (the symbol's name in host code is only a stand-in).
constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
unsigned char *g_addr[MAX_DEVICES] = {};

int scratch_for(int device, unsigned char **out, frt_error *err)
{
    if (device < 0 || device >= MAX_DEVICES) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "device %d out of range", device);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
        if (e != cudaSuccess) return cuda_fail(err, e, "looking up the scan scratch");
        g_addr[device] = (unsigned char *)p;
    }
    *out = g_addr[device];
    return FRT_OK;
}

// Flags (bad[0] = 1) a member table the scratch cannot hold: a member of
// more than 65,536 inflated bytes, offsets that descend, or an end past len.
__global__ void k_check_members(const u64 *starts, u32 n, u64 len, u64 *bad)
{
    for (u32 m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
        u64 ms = starts[m], me = starts[m + 1];
        if (me < ms || me - ms > 65536ull || me > len) *bad = 1ull;
    }
}

// Record offsets from the per-member scratch: one warp per member.
__global__ void k_emit_offsets(const u64 *starts, u32 n, const u32 *count, const u32 *first, const u16 *recs,
                               u64 *out, u64 cap)
{
    u32 m = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    if (m >= n) return;
    u32 c = min(count[m], (u32)FRT_SCAN_CAP);
    u64 ms = starts[m];
    const u16 *r = recs + (size_t)m * FRT_SCAN_CAP;
    for (u32 k = lane_id(); k < c; k += 32) {
        u64 i = (u64)first[m] + k;
        if (i < cap) out[i] = ms + r[k];
    }
}

} // namespace

extern "C" int frt_bam_scan_noalloc(const uint8_t *data, uint64_t len, const uint64_t *member_offsets,
                                    uint32_t n_members, uint64_t start, int32_t n_ref, uint64_t *record_offsets,
                                    uint64_t record_cap, uint64_t *n_records, uint64_t *tail, void *stream,
                                    frt_error *err)
{
    if (n_members > MAX_MEMBERS) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "%u members exceed the %u-member scratch of frt_bam_scan_noalloc; split the batch or use "
                  "frt_bam_decode",
                  n_members, MAX_MEMBERS);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if ((!data && len) || (!member_offsets && n_members) || !n_records || !tail) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (!record_offsets && record_cap) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "record_offsets is null but record_cap is %llu (a null array counts records only with "
                  "record_cap 0)",
                  (unsigned long long)record_cap);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_fail(err, e, "querying the current device");
    unsigned char *s = nullptr;
    int rc = scratch_for(device, &s, err);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_members == 0 || len == 0) {
        *n_records = 0;
        *tail = start;
        return FRT_OK;
    }
    u64 *entry = (u64 *)(s + OFF_ENTRY), *land = (u64 *)(s + OFF_LAND), *totals = (u64 *)(s + OFF_TOTALS);
    u32 *count = (u32 *)(s + OFF_COUNT), *first = (u32 *)(s + OFF_FIRST);
    u8 *flags = s + OFF_FLAGS;
    u16 *recs = (u16 *)(s + OFF_RECS);
    int bound = n_ref >= 0 ? n_ref : (1 << 24);
    // the previous call's totals must not leak into this one
    if ((e = cudaMemsetAsync(totals, 0, 64, st)) != cudaSuccess) return cuda_fail(err, e, "clearing the totals");
    k_check_members<<<(n_members + 255) / 256, 256, 0, st>>>(member_offsets, n_members, len, totals + 4);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(err, e, "launching the member check");
    if ((e = frt_launch_bam_spec(data, len, member_offsets, n_members, start, bound, entry, count, land, flags, recs,
                                 st)) != cudaSuccess)
        return cuda_fail(err, e, "launching the record scan");
    if ((e = frt_launch_bam_reconcile(data, len, member_offsets, n_members, start, entry, count, land, flags, recs,
                                      first, totals, st)) != cudaSuccess)
        return cuda_fail(err, e, "launching the reconcile");
    if (record_offsets && record_cap) {
        k_emit_offsets<<<(n_members + 7) / 8, 256, 0, st>>>(member_offsets, n_members, count, first, recs,
                                                            (u64 *)record_offsets, record_cap);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(err, e, "launching the offset emit");
    }
    uint64_t tot[5] = {0, 0, 0, 0, 0};
    if ((e = cudaMemcpyAsync(tot, totals, sizeof tot, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(err, e, "reading the totals");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(err, e, "record scan");
    if (tot[4]) {
        *n_records = 0;
        *tail = start;
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "a member holds more than 65,536 inflated bytes, or the member offsets descend or run past "
                  "len: the scan's per-member scratch holds BGZF members only");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    *n_records = tot[0];
    *tail = tot[1];
    if (tot[2]) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, tot[1], "bam", "malformed record reached from a confirmed boundary");
        return FRT_ERR_MALFORMED;
    }
    // a null array with record_cap 0 asks for the count alone
    if (record_offsets && tot[0] > record_cap) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, tot[0], record_cap, 0, nullptr,
                  "the batch holds %llu records but record_offsets has room for %llu",
                  (unsigned long long)tot[0], (unsigned long long)record_cap);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    return FRT_OK;
}
