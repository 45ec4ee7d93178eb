// Host runtime and C ABI: the codec, the device batch reader with its carry,
// the BAM decoder and the record batches.  The behaviour mirrors the
// reference's Rust surface for this path; each function names the item it
// stands in for.

#include <fcntl.h>
#include <unistd.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/frt.h"
#include "bam.cuh"
#include "inflate.cuh"
#include "runtime.h"

namespace frt {

void set_error(frt_error *err, int code, uint64_t offset, uint64_t expected, uint64_t actual, uint64_t position,
               const char *format, const char *fmt, ...)
{
    if (!err) return;
    memset(err, 0, sizeof *err);
    err->code = code;
    err->offset = offset;
    err->expected = expected;
    err->actual = actual;
    err->position = position;
    if (format) snprintf(err->format, sizeof err->format, "%s", format);
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err->reason, sizeof err->reason, fmt, ap);
    va_end(ap);
}

int cuda_fail(frt_error *err, cudaError_t e, const char *what)
{
    set_error(err, FRT_ERR_CUDA, 0, 0, 0, 0, nullptr, "%s: %s", what, cudaGetErrorString(e));
    return FRT_ERR_CUDA;
}

// Maps an inflate status to a message (the reference's inflate_status_message,
// crates/fritillaria-cuda/src/backend.rs:66-79).
const char *inflate_status_message(uint32_t s)
{
    switch (s) {
    case 1: return "truncated deflate stream";
    case 2: return "reserved deflate block type";
    case 3: return "stored block LEN/NLEN mismatch";
    case 4: return "output overran the size declared by ISIZE";
    case 5: return "invalid Huffman code";
    case 6: return "invalid or out-of-range back-reference distance";
    case 7: return "malformed Huffman table";
    case 8: return "invalid code-length repeat";
    case 9: return "code counts exceed the DEFLATE maximum";
    case 10: return "a staging copy of the compressed member did not complete";
    default: return "unknown device error";
    }
}

int check_device(int device, frt_error *err)
{
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error(err, FRT_ERR_CUDA_UNAVAILABLE, 0, 0, 0, 0, nullptr, "no CUDA device: %s",
                  e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
        return FRT_ERR_CUDA_UNAVAILABLE;
    }
    if (device < 0 || device >= count) {
        set_error(err, FRT_ERR_CUDA_UNAVAILABLE, 0, 0, 0, 0, nullptr, "device %d out of range (%d devices)", device,
                  count);
        return FRT_ERR_CUDA_UNAVAILABLE;
    }
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return cuda_fail(err, e, "querying device");
    if (!(prop.major == 10 && prop.minor == 3)) {
        set_error(err, FRT_ERR_CUDA_UNAVAILABLE, 0, 0, 0, 0, nullptr,
                  "device %d is sm_%d%d; this library is built for sm_103a (GB300)", device, prop.major, prop.minor);
        return FRT_ERR_CUDA_UNAVAILABLE;
    }
    return FRT_OK;
}

// Pool-backed, stream-ordered allocations.
int dev_alloc(void **p, size_t bytes, cudaStream_t s, frt_error *err)
{
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 1, s);
    if (e != cudaSuccess) return cuda_fail(err, e, "allocating device memory");
    return FRT_OK;
}

void dev_free(void *p, cudaStream_t s)
{
    if (p) cudaFreeAsync(p, s);
}

void configure_pool(int device)
{
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t threshold = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
    }
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int d)
    {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Host bytes in page-locked memory, so H2D copies run at full link speed.
struct PinnedBytes {
    uint8_t *p = nullptr;
    size_t n = 0, cap = 0;
    ~PinnedBytes()
    {
        if (p) cudaFreeHost(p);
    }
    bool reserve(size_t want)
    {
        if (want <= cap) return true;
        size_t nc = cap ? cap : 1 << 20;
        while (nc < want) nc *= 2;
        uint8_t *q = nullptr;
        if (cudaMallocHost((void **)&q, nc) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (n) memcpy(q, p, n);
        if (p) cudaFreeHost(p);
        p = q;
        cap = nc;
        return true;
    }
    bool resize(size_t m)
    {
        if (!reserve(m)) return false;
        n = m;
        return true;
    }
};

} // namespace frt

using namespace frt;

// ===========================================================================
// Codec
// ===========================================================================
frt::SharedStream *frt::stream_create(int device, void *user_stream, frt_error *err)
{
    SharedStream *s = new SharedStream;
    s->device = device;
    if (user_stream) {
        s->s = (cudaStream_t)user_stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->s, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete s;
            cuda_fail(err, e, "creating stream");
            return nullptr;
        }
        s->own = true;
    }
    return s;
}

frt::SharedStream *frt::stream_retain(SharedStream *s)
{
    if (s) s->refs.fetch_add(1);
    return s;
}

void frt::stream_release(SharedStream *s)
{
    if (!s || s->refs.fetch_sub(1) != 1) return;
    if (s->own) {
        DeviceGuard g(s->device);
        cudaStreamSynchronize(s->s);
        cudaStreamDestroy(s->s);
    }
    delete s;
}

void frt::batch_release(const frt_inflate_batch *cb)
{
    frt_inflate_batch *b = const_cast<frt_inflate_batch *>(cb);
    if (!b) return;
    if (b->refs.fetch_sub(1) != 1) return;
    {
        DeviceGuard g(b->device);
        if (b->owns_data) dev_free(b->data, b->stream);
        dev_free(b->d_offsets, b->stream);
        if (b->ready) cudaEventDestroy(b->ready);
    }
    stream_release(b->shared);
    delete b;
}

extern "C" int frt_cuda_is_usable(void)
{
    frt_error e;
    return check_device(0, &e) == FRT_OK;
}

extern "C" int frt_codec_create(int device, void *stream, frt_codec **out, frt_error *err)
{
    if (!out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null output handle");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuard g(device);
    configure_pool(device);
    cudaError_t e = frt_inflate_prepare();
    if (e != cudaSuccess) return cuda_fail(err, e, "configuring inflate kernels");
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    frt_codec *c = new frt_codec;
    c->device = device;
    c->tuning = frt_inflate_default();
    c->shared = ss;
    c->stream = ss->s;
    *out = c;
    return FRT_OK;
}

extern "C" int frt_select_codec(int backend, frt_codec **out, int *resolved, frt_error *err)
{
    switch (backend) {
    case FRT_BACKEND_AUTO:
    case FRT_BACKEND_CUDA: {
        int rc = frt_codec_create(0, nullptr, out, err);
        if (rc == FRT_OK && resolved) *resolved = FRT_BACKEND_CUDA;
        return rc;
    }
    case FRT_BACKEND_NVCOMP:
        set_error(err, FRT_ERR_CUDA_UNAVAILABLE, 0, 0, 0, 0, nullptr,
                  "nvCOMP is not a backend of this library; use Cuda");
        return FRT_ERR_CUDA_UNAVAILABLE;
    case FRT_BACKEND_CPU:
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr,
                  "the CPU codec is not part of this library; it has no CPU fallback");
        return FRT_ERR_INVALID_ARGUMENT;
    default:
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "unknown backend %d", backend);
        return FRT_ERR_INVALID_ARGUMENT;
    }
}

extern "C" void frt_codec_destroy(frt_codec *c)
{
    if (!c) return;
    stream_release(c->shared);
    delete c;
}

extern "C" const char *frt_codec_name(const frt_codec *) { return "cuda-device"; }
extern "C" int frt_codec_device_ordinal(const frt_codec *c) { return c ? c->device : -1; }
extern "C" void *frt_codec_stream(const frt_codec *c) { return c ? (void *)c->stream : nullptr; }

namespace frt {

// The plain per-batch inflate: plan on the host (BatchPlan::new,
// backend.rs:95-133), one launch over the batch's members, a 12-byte status
// per member back, verification in span order (verify_and_offsets,
// backend.rs:221-256).
int inflate_batch(frt_codec *c, const uint8_t *batch, size_t batch_len, const frt_span *spans, size_t n,
                  frt_inflate_batch **out, frt_error *err)
{
    std::vector<uint64_t> plan64(2 * n + 1);
    std::vector<uint32_t> plan32(2 * n);
    uint64_t *in_off = plan64.data(), *out_off = plan64.data() + n;
    uint32_t *in_len = plan32.data(), *cap = plan32.data() + n;
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        const frt_span &s = spans[i];
        if (s.isize > 65536u) {
            set_error(err, FRT_ERR_INVALID_BLOCK, s.compressed_offset, 0, 0, 0, nullptr, "ISIZE exceeds 64 KiB");
            return FRT_ERR_INVALID_BLOCK;
        }
        uint64_t end = s.payload_start + s.payload_len;
        if (end < s.payload_start || end > batch_len || s.payload_len > 0xffffffffull) {
            set_error(err, FRT_ERR_INVALID_BLOCK, s.compressed_offset, 0, 0, 0, nullptr,
                      "payload extends past the end of the batch");
            return FRT_ERR_INVALID_BLOCK;
        }
        in_off[i] = s.payload_start;
        in_len[i] = (uint32_t)s.payload_len;
        out_off[i] = total;
        cap[i] = s.isize;
        total += s.isize;
    }
    out_off[n] = total;
    DeviceGuard g(c->device);
    std::lock_guard<std::mutex> lk(c->mu);
    cudaStream_t st = c->stream;
    // one work buffer: in_off | out_off(n+1) | in_len | cap | status | produced | crc
    size_t work_bytes = 8 * (2 * n + 1) + 4 * 5 * n;
    uint8_t *work = nullptr, *input = nullptr, *output = nullptr;
    uint64_t *d_offsets = nullptr;
    int rc;
    if ((rc = dev_alloc((void **)&work, work_bytes, st, err))) return rc;
    if ((rc = dev_alloc((void **)&input, batch_len + 64, st, err))) {
        dev_free(work, st);
        return rc;
    }
    if ((rc = dev_alloc((void **)&output, total + 16, st, err))) {
        dev_free(work, st);
        dev_free(input, st);
        return rc;
    }
    if ((rc = dev_alloc((void **)&d_offsets, 8 * (2 * n + 1), st, err))) {
        dev_free(work, st);
        dev_free(input, st);
        dev_free(output, st);
        return rc;
    }
    auto fail = [&](cudaError_t e, const char *what) {
        dev_free(work, st);
        dev_free(input, st);
        dev_free(output, st);
        dev_free(d_offsets, st);
        return cuda_fail(err, e, what);
    };
    uint64_t *d_in_off = (uint64_t *)work;
    uint64_t *d_out_off = d_in_off + n;
    uint32_t *d_in_len = (uint32_t *)(d_out_off + n + 1);
    uint32_t *d_cap = d_in_len + n;
    uint32_t *d_status = d_cap + n;
    uint32_t *d_produced = d_status + n;
    uint32_t *d_crc = d_produced + n;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(input, batch, batch_len, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e, "uploading batch");
    if ((e = cudaMemsetAsync(input + batch_len, 0, 64, st)) != cudaSuccess) return fail(e, "padding batch");
    if ((e = cudaMemcpyAsync(work, plan64.data(), 8 * (2 * n + 1), cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e, "uploading plan");
    if ((e = cudaMemcpyAsync(d_in_len, plan32.data(), 8 * n, cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail(e, "uploading plan");
    if ((e = frt_launch_inflate_members(input, d_in_off, d_in_len, output, d_out_off, d_cap, d_status, d_produced,
                                        d_crc, (u32)n, c->tuning, st)) != cudaSuccess)
        return fail(e, "launching inflate");
    std::vector<uint32_t> res(3 * n);
    if (n && (e = cudaMemcpyAsync(res.data(), d_status, 12 * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return fail(e, "downloading status");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "inflate");
    for (size_t i = 0; i < n; ++i) {
        uint32_t status = res[i], produced = res[n + i], crc = res[2 * n + i];
        int code = 0;
        if (status != 0) {
            set_error(err, FRT_ERR_INFLATE, spans[i].compressed_offset, 0, 0, 0, nullptr, "%s",
                      inflate_status_message(status));
            code = FRT_ERR_INFLATE;
        } else if (produced != spans[i].isize) {
            set_error(err, FRT_ERR_SIZE, spans[i].compressed_offset, spans[i].isize, produced, 0, nullptr,
                      "ISIZE says %u bytes, inflated %u", spans[i].isize, produced);
            code = FRT_ERR_SIZE;
        } else if (crc != spans[i].crc32) {
            set_error(err, FRT_ERR_CHECKSUM, spans[i].compressed_offset, spans[i].crc32, crc, 0, nullptr,
                      "expected crc32 %#010x, got %#010x", spans[i].crc32, crc);
            code = FRT_ERR_CHECKSUM;
        }
        if (code) {
            dev_free(work, st);
            dev_free(input, st);
            dev_free(output, st);
            dev_free(d_offsets, st);
            return code;
        }
    }
    frt_inflate_batch *b = new frt_inflate_batch;
    b->device = c->device;
    b->stream = st;
    b->shared = stream_retain(c->shared);
    b->data = output;
    b->len = total;
    b->offsets.assign(out_off, out_off + n + 1);
    b->coffsets.resize(n);
    for (size_t i = 0; i < n; ++i) b->coffsets[i] = spans[i].compressed_offset;
    std::vector<uint64_t> both(2 * n + 1);
    memcpy(both.data(), out_off, 8 * (n + 1));
    memcpy(both.data() + n + 1, b->coffsets.data(), 8 * n);
    cudaMemcpyAsync(d_offsets, both.data(), 8 * (2 * n + 1), cudaMemcpyHostToDevice, st);
    b->d_offsets = d_offsets;
    cudaEventCreateWithFlags(&b->ready, cudaEventDisableTiming);
    cudaEventRecord(b->ready, st);
    dev_free(work, st);
    dev_free(input, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
        batch_release(b);
        return cuda_fail(err, e, "finishing inflate");
    }
    *out = b;
    return FRT_OK;
}

} // namespace frt

extern "C" int frt_codec_inflate_batch_device(frt_codec *c, const uint8_t *batch, size_t batch_len,
                                              const frt_span *spans, size_t n, frt_inflate_batch **out,
                                              frt_error *err)
{
    if (!c || !out || (!batch && batch_len) || (!spans && n)) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    return inflate_batch(c, batch, batch_len, spans, n, out, err);
}

extern "C" int frt_codec_inflate_batch_host(frt_codec *c, const uint8_t *batch, size_t batch_len,
                                            const frt_span *spans, size_t n, uint8_t *out, size_t out_cap,
                                            uint64_t *out_offsets, frt_error *err)
{
    frt_inflate_batch *b = nullptr;
    int rc = frt_codec_inflate_batch_device(c, batch, batch_len, spans, n, &b, err);
    if (rc) return rc;
    rc = frt_inflate_batch_to_host(b, out, out_cap, err);
    if (!rc && out_offsets) memcpy(out_offsets, b->offsets.data(), 8 * b->offsets.size());
    batch_release(b);
    return rc;
}

extern "C" int frt_codec_crc32_device(frt_codec *c, const uint8_t *data, const uint64_t *offsets,
                                      const uint32_t *lengths, size_t n, uint32_t *crcs, frt_error *err)
{
    DeviceGuard g(c->device);
    std::lock_guard<std::mutex> lk(c->mu);
    cudaStream_t st = c->stream;
    uint8_t *work = nullptr;
    int rc = dev_alloc((void **)&work, 16 * n + 16, st, err);
    if (rc) return rc;
    uint64_t *d_off = (uint64_t *)work;
    uint32_t *d_len = (uint32_t *)(d_off + n);
    uint32_t *d_out = d_len + n;
    cudaMemcpyAsync(d_off, offsets, 8 * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_len, lengths, 4 * n, cudaMemcpyHostToDevice, st);
    cudaError_t e = frt_launch_crc32_members(data, d_off, d_len, d_out, (u32)n, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(crcs, d_out, 4 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(work, st);
    if (e != cudaSuccess) return cuda_fail(err, e, "crc32");
    return FRT_OK;
}

// ---- inflate batch accessors ----------------------------------------------
extern "C" size_t frt_inflate_batch_len(const frt_inflate_batch *b) { return b ? b->offsets.size() - 1 : 0; }
extern "C" size_t frt_inflate_batch_byte_len(const frt_inflate_batch *b) { return b ? b->len : 0; }
extern "C" const uint8_t *frt_inflate_batch_data(const frt_inflate_batch *b) { return b ? b->data : nullptr; }
extern "C" const uint64_t *frt_inflate_batch_offsets(const frt_inflate_batch *b) { return b ? b->offsets.data() : nullptr; }
extern "C" const uint64_t *frt_inflate_batch_compressed_offsets(const frt_inflate_batch *b)
{
    return b ? b->coffsets.data() : nullptr;
}
extern "C" int frt_inflate_batch_device_ordinal(const frt_inflate_batch *b) { return b ? b->device : -1; }
extern "C" void *frt_inflate_batch_ready_event(const frt_inflate_batch *b) { return b ? (void *)b->ready : nullptr; }
extern "C" int frt_inflate_batch_to_host(const frt_inflate_batch *b, uint8_t *dst, size_t cap, frt_error *err)
{
    if (!b) return FRT_OK;
    if (cap < b->len) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "destination holds %zu bytes, batch has %zu",
                  cap, b->len);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuard g(b->device);
    cudaError_t e = cudaMemcpyAsync(dst, b->data, b->len, cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "downloading batch");
    return FRT_OK;
}
extern "C" void frt_inflate_batch_free(frt_inflate_batch *b) { batch_release(b); }

// ===========================================================================
// Host BGZF framing (crates/fritillaria-bgzf/src/block.rs:88-165,
// discover.rs:51-109)
// ===========================================================================
namespace frt {

static inline uint32_t rd16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
static inline uint32_t rd32(const uint8_t *p)
{
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

int parse_bgzf_header(const uint8_t *buf, size_t len, uint64_t offset, uint32_t *block_size, uint32_t *header_size,
                      frt_error *err)
{
    auto invalid = [&](const char *why) {
        set_error(err, FRT_ERR_INVALID_BLOCK, offset, 0, 0, 0, nullptr, "%s", why);
        return FRT_ERR_INVALID_BLOCK;
    };
    if (len < 12) return invalid("truncated header");
    if (buf[0] != 0x1f || buf[1] != 0x8b) return invalid("not a gzip member (bad magic)");
    if (buf[2] != 8) return invalid("unsupported compression method");
    if ((buf[3] & 0x04) == 0) return invalid("missing FEXTRA; not BGZF (plain gzip?)");
    size_t xlen = rd16(buf + 10), hsize = 12 + xlen;
    if (len < hsize) return invalid("truncated extra field");
    const uint8_t *x = buf + 12;
    size_t left = xlen;
    bool found = false;
    uint32_t bsize = 0;
    while (left >= 4) {
        size_t slen = rd16(x + 2);
        if (4 + slen > left) break;
        if (x[0] == 'B' && x[1] == 'C') {
            if (slen == 2) {
                bsize = rd16(x + 4);
                found = true;
            }
            break;
        }
        x += 4 + slen;
        left -= 4 + slen;
    }
    if (!found) return invalid("missing BC subfield; not BGZF");
    uint32_t bs = bsize + 1;
    if (bs > 65536u) return invalid("block size exceeds 64 KiB");
    if (bs < hsize + 8) return invalid("block size smaller than its own framing");
    *block_size = bs;
    *header_size = (uint32_t)hsize;
    return FRT_OK;
}

int discover(const uint8_t *buf, size_t len, uint64_t base, std::vector<frt_span> &spans, size_t *consumed,
             frt_error *err)
{
    size_t pos = 0;
    while (pos < len) {
        const uint8_t *rest = buf + pos;
        size_t rlen = len - pos;
        if (rlen < 12) break;
        size_t hl = 12 + rd16(rest + 10);
        if (hl > rlen) break;
        uint32_t bs, hs;
        int rc = parse_bgzf_header(rest, rlen, base + pos, &bs, &hs, err);
        if (rc) {
            *consumed = pos;
            return rc;
        }
        if (bs > rlen) break;
        uint32_t isz = rd32(rest + bs - 4);
        if (isz > 65536u) {
            set_error(err, FRT_ERR_INVALID_BLOCK, base + pos, 0, 0, 0, nullptr, "ISIZE exceeds 64 KiB");
            *consumed = pos;
            return FRT_ERR_INVALID_BLOCK;
        }
        frt_span s;
        s.compressed_offset = base + pos;
        s.payload_start = pos + hs;
        s.payload_len = bs - hs - 8;
        s.isize = isz;
        s.crc32 = rd32(rest + bs - 8);
        spans.push_back(s);
        pos += bs;
    }
    *consumed = pos;
    return FRT_OK;
}

} // namespace frt

extern "C" int frt_bgzf_discover(const uint8_t *buf, size_t len, uint64_t base_offset, frt_span *spans, size_t cap,
                                 size_t *n_spans, size_t *consumed, frt_error *err)
{
    std::vector<frt_span> v;
    size_t used = 0;
    int rc = discover(buf, len, base_offset, v, &used, err);
    size_t k = v.size() < cap ? v.size() : cap;
    if (spans && k) memcpy(spans, v.data(), k * sizeof(frt_span));
    if (n_spans) *n_spans = v.size();
    if (consumed) *consumed = used;
    return rc;
}

// ===========================================================================
// DeviceBgzfReader (crates/fritillaria-bgzf/src/device_read.rs:57-280)
// ===========================================================================
struct frt_reader {
    frt_read_fn read = nullptr;
    void *ctx = nullptr;
    frt_codec *codec = nullptr;
    int fd = -1;
    const uint8_t *mem = nullptr;
    size_t mem_len = 0, mem_pos = 0;
    size_t blocks_per_batch = 256; // DEFAULT_BLOCKS_PER_BATCH, read.rs:37
    PinnedBytes compressed;
    uint64_t batch_offset = 0;
    std::vector<uint8_t> carry;
    size_t carry_start = 0;
    std::vector<frt_span> spans;
    bool exhausted = false;

    int64_t pull(uint8_t *buf, size_t cap)
    {
        if (mem) {
            size_t k = mem_len - mem_pos < cap ? mem_len - mem_pos : cap;
            memcpy(buf, mem + mem_pos, k);
            mem_pos += k;
            return (int64_t)k;
        }
        if (fd >= 0) {
            for (;;) {
                ssize_t r = ::read(fd, buf, cap);
                if (r < 0 && errno == EINTR) continue;
                return (int64_t)r;
            }
        }
        return read(ctx, buf, cap);
    }
};

static int reader_new(frt_codec *codec, frt_reader **out, frt_error *err, frt_reader *r)
{
    if (!codec || !out) {
        delete r;
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    r->codec = codec;
    *out = r;
    return FRT_OK;
}

extern "C" int frt_reader_open(frt_read_fn read, void *ctx, frt_codec *codec, frt_reader **out, frt_error *err)
{
    frt_reader *r = new frt_reader;
    r->read = read;
    r->ctx = ctx;
    if (!read) {
        delete r;
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null read callback");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    return reader_new(codec, out, err, r);
}

extern "C" int frt_reader_open_memory(const uint8_t *data, size_t len, frt_codec *codec, frt_reader **out,
                                      frt_error *err)
{
    frt_reader *r = new frt_reader;
    static const uint8_t empty = 0;
    r->mem = data ? data : &empty;
    r->mem_len = data ? len : 0;
    return reader_new(codec, out, err, r);
}

extern "C" int frt_reader_open_path(const char *path, frt_codec *codec, frt_reader **out, frt_error *err)
{
    int fd = open(path, O_RDONLY);
    if (fd < 0) {
        set_error(err, FRT_ERR_IO, 0, 0, 0, 0, nullptr, "cannot open %s: %s", path, strerror(errno));
        return FRT_ERR_IO;
    }
    frt_reader *r = new frt_reader;
    r->fd = fd;
    return reader_new(codec, out, err, r);
}

extern "C" void frt_reader_set_blocks_per_batch(frt_reader *r, size_t blocks)
{
    if (r) r->blocks_per_batch = blocks < 1 ? 1 : blocks;
}

extern "C" int frt_reader_carry_from(frt_reader *r, uint64_t tail, frt_error *err)
{
    // block_offsets: uncompressed offset of each block of the last batch
    std::vector<uint64_t> offsets(r->spans.size() + 1, 0);
    for (size_t i = 0; i < r->spans.size(); ++i) offsets[i + 1] = offsets[i] + r->spans[i].isize;
    uint64_t total = offsets.back();
    if (tail > total) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr,
                  "carry offset %llu is past the batch's %llu bytes", (unsigned long long)tail,
                  (unsigned long long)total);
        return FRT_ERR_INVALID_DEVICE_BATCH;
    }
    if (tail == total) {
        r->carry_start = 0;
        return FRT_OK;
    }
    // the block containing tail: last block starting at or before it
    size_t block = (size_t)(std::upper_bound(offsets.begin(), offsets.end(), tail) - offsets.begin()) - 1;
    size_t block_start = (size_t)(r->spans[block].compressed_offset - r->batch_offset);
    r->carry.assign(r->compressed.p + block_start, r->compressed.p + r->compressed.n);
    r->carry_start = (size_t)(tail - offsets[block]);
    return FRT_OK;
}

extern "C" int frt_reader_next_batch(frt_reader *r, frt_inflate_batch **out, uint64_t *start, int *has_batch,
                                     frt_error *err)
{
    *has_batch = 0;
    for (;;) {
        if (r->exhausted && r->carry.empty()) return FRT_OK;
        if (r->exhausted && r->compressed.n != 0 && r->carry.size() == r->compressed.n) {
            set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, r->batch_offset, "bgzf",
                      "stream ends inside a record: the trailing bytes are not a complete record");
            return FRT_ERR_MALFORMED;
        }
        r->batch_offset += r->compressed.n;
        r->batch_offset -= r->carry.size();
        size_t lead = r->carry.size();
        size_t want = r->blocks_per_batch * 65536;
        if (!r->compressed.resize(lead + want)) {
            set_error(err, FRT_ERR_CUDA, 0, 0, 0, 0, nullptr, "allocating pinned host memory");
            return FRT_ERR_CUDA;
        }
        if (lead) memcpy(r->compressed.p, r->carry.data(), lead);
        r->carry.clear();
        size_t filled = lead;
        while (filled < r->compressed.n) {
            int64_t k = r->pull(r->compressed.p + filled, r->compressed.n - filled);
            if (k == 0) {
                r->exhausted = true;
                break;
            }
            if (k < 0) {
                set_error(err, FRT_ERR_IO, 0, 0, 0, 0, nullptr, "read failed");
                return FRT_ERR_IO;
            }
            filled += (size_t)k;
        }
        r->compressed.n = filled;
        r->spans.clear();
        size_t consumed = 0;
        int rc = discover(r->compressed.p, r->compressed.n, r->batch_offset, r->spans, &consumed, err);
        if (rc) return rc;
        r->carry.assign(r->compressed.p + consumed, r->compressed.p + r->compressed.n);
        if (r->exhausted && !r->carry.empty()) {
            set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, r->batch_offset + consumed, "bgzf",
                      "truncated BGZF: %zu trailing bytes are not a complete block", r->carry.size());
            return FRT_ERR_MALFORMED;
        }
        if (r->spans.empty()) {
            if (r->exhausted) return FRT_OK;
            continue;
        }
        frt_inflate_batch *b = nullptr;
        rc = inflate_batch(r->codec, r->compressed.p, r->compressed.n, r->spans.data(), r->spans.size(), &b, err);
        if (rc) return rc;
        if (b->len == 0) {
            batch_release(b);
            if (r->exhausted) return FRT_OK;
            continue;
        }
        *start = r->carry_start;
        r->carry_start = 0;
        *out = b;
        *has_batch = 1;
        return FRT_OK;
    }
}

extern "C" const char *frt_reader_codec_name(const frt_reader *r) { return r ? frt_codec_name(r->codec) : ""; }
extern "C" int frt_reader_device_ordinal(const frt_reader *r) { return r ? r->codec->device : -1; }
extern "C" void frt_reader_close(frt_reader *r)
{
    if (!r) return;
    if (r->fd >= 0) close(r->fd);
    delete r;
}

// ===========================================================================
// BAM header (crates/fritillaria-bam/src/columnar/header.rs:43-101)
// ===========================================================================
extern "C" int frt_bam_parse_header(const uint8_t *buf, size_t len, uint64_t *records_start, int32_t *n_ref,
                                    frt_error *err)
{
    auto bad = [&](uint64_t pos, const char *why) {
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, pos, "bam header", "%s", why);
        return FRT_ERR_MALFORMED;
    };
    if (len < 12) return bad(0, "truncated header");
    if (memcmp(buf, "BAM\1", 4) != 0) return bad(0, "bad magic; expected BAM\\1");
    int32_t l_text = (int32_t)rd32(buf + 4);
    if (l_text < 0) return bad(4, "negative l_text");
    uint64_t text_end = 8 + (uint64_t)l_text;
    if (text_end > len) return bad(4, "l_text runs past the end of the buffer");
    if (text_end + 4 > len) return bad(text_end, "truncated n_ref");
    int32_t nr = (int32_t)rd32(buf + text_end);
    if (nr < 0) return bad(text_end, "negative n_ref");
    uint64_t pos = text_end + 4;
    for (int32_t i = 0; i < nr; ++i) {
        if (pos + 4 > len) return bad(pos, "truncated l_name");
        int32_t l_name = (int32_t)rd32(buf + pos);
        if (l_name < 0) return bad(pos, "negative l_name");
        pos += 4;
        if (pos + (uint64_t)l_name > len) return bad(pos, "truncated name");
        pos += (uint64_t)l_name;
        if (pos + 4 > len) return bad(pos, "truncated l_ref");
        pos += 4;
    }
    if (records_start) *records_start = pos;
    if (n_ref) *n_ref = nr;
    return FRT_OK;
}
