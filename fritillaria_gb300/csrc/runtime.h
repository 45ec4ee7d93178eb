// Internal helpers shared by the host runtime translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/frt.h"

namespace frt {

void set_error(frt_error *err, int code, uint64_t offset, uint64_t expected, uint64_t actual, uint64_t position,
               const char *format, const char *fmt, ...);
int cuda_fail(frt_error *err, cudaError_t e, const char *what);
const char *inflate_status_message(uint32_t s);
int check_device(int device, frt_error *err);
int engine_device(const frt_engine *e);
int dev_alloc(void **p, size_t bytes, cudaStream_t s, frt_error *err);
void dev_free(void *p, cudaStream_t s);
void configure_pool(int device);
int parse_bgzf_header(const uint8_t *buf, size_t len, uint64_t offset, uint32_t *block_size, uint32_t *header_size,
                      frt_error *err);
int discover(const uint8_t *buf, size_t len, uint64_t base, std::vector<frt_span> &spans, size_t *consumed,
             frt_error *err);

// Element width of each BAM column (frt_bam_column order).
inline size_t bam_column_width(int c)
{
    static const size_t w[FRT_COL_COUNT] = {4, 4, 2, 1, 4, 4, 4, 4, 8, 4, 4, 4, 4, 4, 2, 2, 1, 8, 4, 1, 4, 12};
    return (c >= 0 && c < FRT_COL_COUNT) ? w[c] : 0;
}

struct DeviceGuardLite {
    int prev = -1;
    explicit DeviceGuardLite(int d)
    {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~DeviceGuardLite()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

} // namespace frt

namespace frt {
// A stream shared by a codec or decoder and every buffer it hands out, so a
// buffer can be freed after its producer is gone (the reference's buffers hold
// an Arc<CudaStream>, crates/fritillaria-cuda/src/backend.rs:266-300).
struct SharedStream {
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t s = nullptr;
    bool own = false;
};
SharedStream *stream_create(int device, void *user_stream, frt_error *err);
SharedStream *stream_retain(SharedStream *s);
void stream_release(SharedStream *s);
} // namespace frt

struct frt_codec {
    int device = 0;
    frt_inflate_tuning tuning{}; // the process default when the codec was made
    cudaStream_t stream = nullptr;
    frt::SharedStream *shared = nullptr;
    std::mutex mu;
};

// An owned inflated batch: the device bytes, the member layout (host and
// device copies) and a completion event.  Reference-counted so the record
// batches decoded from it keep it alive.
struct frt_inflate_batch {
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t stream = nullptr;
    uint8_t *data = nullptr;
    size_t len = 0;
    std::vector<uint64_t> offsets{0};
    std::vector<uint64_t> coffsets;
    uint64_t *d_offsets = nullptr; // n + 1 member starts, then n compressed offsets
    cudaEvent_t ready = nullptr;
    frt::SharedStream *shared = nullptr;
    bool owns_data = true; // false for a view into memory owned elsewhere (an engine's output)
};

// A set of device columns (FASTQ/BCF/FASTA scans, record fields): column k is
// col_bytes[k] bytes at cols + col_off[k] (FASTA's bases in `seq`), elements of
// widths[k] bytes.  Holds its source batch when its columns point into it.
struct frt_columns {
    int device = 0;
    int format = 0;
    cudaStream_t stream = nullptr;
    frt::SharedStream *shared = nullptr;
    uint64_t n = 0, tail = 0, total = 0;
    uint64_t info[3] = {0, 0, 0}; // proof, survivors, validated
    int n_cols = 0;
    const size_t *widths = nullptr;
    uint8_t *cols = nullptr;
    uint8_t *seq = nullptr; // FASTA bases
    size_t col_off[16] = {}, col_bytes[16] = {};
    const frt_inflate_batch *source = nullptr;
    cudaEvent_t ready = nullptr;
};

namespace frt {
void batch_release(const frt_inflate_batch *b);
int inflate_batch(frt_codec *c, const uint8_t *batch, size_t batch_len, const frt_span *spans, size_t n,
                  frt_inflate_batch **out, frt_error *err);
} // namespace frt
