// BamDecoder and DeviceRecordBatch (crates/fritillaria-cuda/src/bam.rs:113-573,
// crates/fritillaria-bam/src/columnar/device.rs:135-297).
//
// decode(batch, start): speculate per member, reconcile the chain on device,
// one host read of {records, tail, status} (the count sizes the columns, as in
// the reference), then the column and aux-directory passes.

#include <cstring>

#include "bam.cuh"
#include "fields.h"
#include "runtime.h"

using namespace frt;

struct frt_bam_decoder {
    int device = 0;
    cudaStream_t stream = nullptr;
    SharedStream *shared = nullptr;
    int32_t n_ref = -1;
    uint64_t last_fallbacks = 0;
    std::mutex mu;
};

struct frt_record_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t n = 0, tail = 0, n_aux = 0;
    const frt_inflate_batch *source = nullptr; // retained
    uint8_t *cols = nullptr;                   // one allocation for the per-record columns
    uint8_t *aux = nullptr;                    // the aux-field directory (its own allocation)
    size_t col_off[FRT_COL_COUNT] = {};
    size_t col_bytes[FRT_COL_COUNT] = {};
    cudaEvent_t ready = nullptr;
    SharedStream *shared = nullptr;
};

static void rb_discard(frt_record_batch *rb)
{
    stream_release(rb->shared);
    delete rb;
}

extern "C" int frt_bam_decoder_create(int device, void *stream, frt_bam_decoder **out, frt_error *err)
{
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuardLite g(device);
    configure_pool(device);
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    frt_bam_decoder *d = new frt_bam_decoder;
    d->device = device;
    d->shared = ss;
    d->stream = ss->s;
    *out = d;
    return FRT_OK;
}

extern "C" void frt_bam_decoder_set_reference_count(frt_bam_decoder *d, int32_t n_ref)
{
    if (d) d->n_ref = n_ref;
}

extern "C" void frt_bam_decoder_destroy(frt_bam_decoder *d)
{
    if (!d) return;
    stream_release(d->shared);
    delete d;
}

extern "C" uint64_t frt_bam_decoder_last_fallbacks(const frt_bam_decoder *d) { return d ? d->last_fallbacks : 0; }

static void layout_columns(frt_record_batch *rb)
{
    size_t off = 0;
    for (int c = 0; c < FRT_COL_COUNT; ++c) {
        size_t bytes;
        if (c == FRT_COL_AUX_FIRST) bytes = 4 * (rb->n + 1);
        else if (c == FRT_COL_AUX_ENTRIES) bytes = 12 * rb->n_aux;
        else bytes = bam_column_width(c) * rb->n;
        rb->col_off[c] = off;
        rb->col_bytes[c] = bytes;
        off += (bytes + 255) & ~(size_t)255;
    }
}

static size_t columns_total(const frt_record_batch *rb)
{
    size_t t = 0;
    for (int c = 0; c < FRT_COL_COUNT; ++c) t += (rb->col_bytes[c] + 255) & ~(size_t)255;
    return t;
}

template <typename T> static T *col(frt_record_batch *rb, int c) { return (T *)(rb->cols + rb->col_off[c]); }

// DeviceRecordBatch for no records: the tail is where decoding started
// (bam.rs:575-597).
static int empty_batch(frt_bam_decoder *d, const frt_inflate_batch *src, uint64_t start, frt_record_batch **out,
                       frt_error *err)
{
    frt_record_batch *rb = new frt_record_batch;
    rb->device = d->device;
    rb->stream = d->stream;
    rb->shared = stream_retain(d->shared);
    rb->tail = start;
    layout_columns(rb);
    int rc = dev_alloc((void **)&rb->cols, columns_total(rb) + 256, d->stream, err);
    if (rc) {
        rb_discard(rb);
        return rc;
    }
    cudaMemsetAsync(rb->cols, 0, 256, d->stream); // aux_first[0] = 0
    if (src) {
        const_cast<frt_inflate_batch *>(src)->refs.fetch_add(1);
        rb->source = src;
    }
    cudaEventCreateWithFlags(&rb->ready, cudaEventDisableTiming);
    cudaEventRecord(rb->ready, d->stream);
    *out = rb;
    return FRT_OK;
}

extern "C" int frt_bam_decode(frt_bam_decoder *d, const frt_inflate_batch *b, uint64_t start, frt_record_batch **out,
                              frt_error *err)
{
    if (!d || !out) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(d->device);
    std::lock_guard<std::mutex> lk(d->mu);
    if (!b || !b->data || b->len == 0) return empty_batch(d, b, start, out, err);
    if (b->device != d->device) {
        set_error(err, FRT_ERR_INVALID_DEVICE_BATCH, 0, 0, 0, 0, nullptr, "batch is on device %d but this decoder is on %d",
                  b->device, d->device);
        return FRT_ERR_INVALID_DEVICE_BATCH;
    }
    cudaStream_t st = d->stream;
    cudaError_t e = cudaStreamWaitEvent(st, b->ready, 0);
    if (e != cudaSuccess) return cuda_fail(err, e, "ordering after the inflate");
    const uint32_t n = (uint32_t)(b->offsets.size() - 1);
    const uint64_t len = b->len;
    // work: entry u64[n] | land u64[n] | totals u64[4] | count u32[n] | first u32[n] | flags u8[n] | scratch
    size_t o_entry = 0, o_land = 8ull * n, o_tot = 16ull * n, o_count = o_tot + 32, o_first = o_count + 4ull * n,
           o_flags = o_first + 4ull * n, o_scr = (o_flags + n + 255) & ~(size_t)255;
    size_t work_bytes = o_scr + (size_t)n * FRT_SCAN_CAP * 2;
    uint8_t *work = nullptr;
    int rc = dev_alloc((void **)&work, work_bytes, st, err);
    if (rc) return rc;
    u64 *entry = (u64 *)(work + o_entry), *land = (u64 *)(work + o_land), *totals = (u64 *)(work + o_tot);
    u32 *count = (u32 *)(work + o_count), *first = (u32 *)(work + o_first);
    u8 *flags = work + o_flags;
    u16 *scratch = (u16 *)(work + o_scr);
    const u64 *starts = b->d_offsets;
    const u64 *coff = b->d_offsets + n + 1;
    int nref_bound = d->n_ref >= 0 ? d->n_ref : (1 << 24);
    auto fail = [&](cudaError_t ee, const char *what) {
        dev_free(work, st);
        return cuda_fail(err, ee, what);
    };
    if ((e = frt_launch_bam_spec(b->data, len, starts, n, start, nref_bound, entry, count, land, flags, scratch, st)) !=
        cudaSuccess)
        return fail(e, "launching record scan");
    if ((e = frt_launch_bam_reconcile(b->data, len, starts, n, start, entry, count, land, flags, scratch, first, totals,
                                      st)) != cudaSuccess)
        return fail(e, "launching reconcile");
    uint64_t tot[4] = {0, 0, 0, 0};
    if ((e = cudaMemcpyAsync(tot, totals, sizeof tot, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return fail(e, "totals");
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "record scan");
    d->last_fallbacks = tot[3];
    if (tot[2] != 0) {
        dev_free(work, st);
        set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, tot[1], "bam", "malformed record reached from a confirmed boundary");
        return FRT_ERR_MALFORMED;
    }
    frt_record_batch *rb = new frt_record_batch;
    rb->device = d->device;
    rb->stream = st;
    rb->shared = stream_retain(d->shared);
    rb->n = tot[0];
    rb->tail = tot[1];
    rb->n_aux = 0;
    layout_columns(rb);
    // columns without the aux entries first; the entries are sized after the scan
    size_t base_bytes = columns_total(rb);
    if ((rc = dev_alloc((void **)&rb->cols, base_bytes + 256, st, err))) {
        rb_discard(rb);
        dev_free(work, st);
        return rc;
    }
    FrtBamColumnsDev c;
    c.ref_id = col<int>(rb, FRT_COL_REF_ID);
    c.pos = col<int>(rb, FRT_COL_POS);
    c.flags = col<u16>(rb, FRT_COL_FLAGS);
    c.mapq = col<u8>(rb, FRT_COL_MAPQ);
    c.seq_len = col<u32>(rb, FRT_COL_SEQ_LEN);
    c.mate_ref_id = col<int>(rb, FRT_COL_MATE_REF_ID);
    c.mate_pos = col<int>(rb, FRT_COL_MATE_POS);
    c.tlen = col<int>(rb, FRT_COL_TLEN);
    c.record_offsets = col<u64>(rb, FRT_COL_RECORD_OFFSETS);
    c.cigar_start = col<u32>(rb, FRT_COL_CIGAR_START);
    c.sequence_start = col<u32>(rb, FRT_COL_SEQUENCE_START);
    c.quality_start = col<u32>(rb, FRT_COL_QUALITY_START);
    c.aux_start = col<u32>(rb, FRT_COL_AUX_START);
    c.record_end = col<u32>(rb, FRT_COL_RECORD_END);
    c.bin = col<u16>(rb, FRT_COL_BIN);
    c.n_cigar = col<u16>(rb, FRT_COL_N_CIGAR);
    c.name_len = col<u8>(rb, FRT_COL_NAME_LEN);
    c.virtual_offset = col<u64>(rb, FRT_COL_VIRTUAL_OFFSET);
    c.aux_count = col<u32>(rb, FRT_COL_AUX_COUNT);
    c.aux_status = col<u8>(rb, FRT_COL_AUX_STATUS);
    u32 *aux_first = col<u32>(rb, FRT_COL_AUX_FIRST);
    if ((e = frt_launch_bam_decode(b->data, starts, coff, n, count, first, scratch, c, st)) != cudaSuccess) {
        dev_free(rb->cols, st);
        rb_discard(rb);
        return fail(e, "launching decode");
    }
    // exclusive scan of the aux counts (scratch reused for the partials)
    u32 *partials = (u32 *)work; // entry/land are no longer needed
    size_t parts = frt_scan_partials_len(rb->n);
    u32 *d_total = nullptr;
    uint8_t *extra = nullptr;
    if (parts * 4 + 8 > o_count) {
        if ((rc = dev_alloc((void **)&extra, parts * 4 + 16, st, err))) {
            dev_free(rb->cols, st);
            rb_discard(rb);
            dev_free(work, st);
            return rc;
        }
        partials = (u32 *)extra;
    }
    d_total = (u32 *)(work + o_tot);
    if ((e = frt_launch_scan_u32(c.aux_count, rb->n, partials, aux_first, d_total, st)) != cudaSuccess) {
        dev_free(extra, st);
        dev_free(rb->cols, st);
        rb_discard(rb);
        return fail(e, "scanning aux counts");
    }
    uint32_t n_aux = 0;
    if ((e = cudaMemcpyAsync(&n_aux, d_total, 4, cudaMemcpyDeviceToHost, st)) == cudaSuccess) e = cudaStreamSynchronize(st);
    dev_free(extra, st);
    if (e != cudaSuccess) {
        dev_free(rb->cols, st);
        rb_discard(rb);
        return fail(e, "decode");
    }
    rb->n_aux = n_aux;
    // move into a final allocation that also holds the aux entries
    size_t aux_bytes = 12ull * n_aux;
    uint8_t *aux = nullptr;
    if ((rc = dev_alloc((void **)&aux, aux_bytes + 16, st, err))) {
        dev_free(rb->cols, st);
        rb_discard(rb);
        dev_free(work, st);
        return rc;
    }
    if ((e = frt_launch_bam_aux_dir(b->data, c.record_offsets, c.aux_start, c.record_end, c.aux_count, aux_first,
                                    (u32 *)aux, rb->n, st)) != cudaSuccess) {
        dev_free(aux, st);
        dev_free(rb->cols, st);
        rb_discard(rb);
        return fail(e, "launching aux directory");
    }
    rb->aux = aux;
    rb->col_bytes[FRT_COL_AUX_ENTRIES] = aux_bytes;
    dev_free(work, st);
    const_cast<frt_inflate_batch *>(b)->refs.fetch_add(1);
    rb->source = b;
    cudaEventCreateWithFlags(&rb->ready, cudaEventDisableTiming);
    cudaEventRecord(rb->ready, st);
    *out = rb;
    return FRT_OK;
}

extern "C" uint64_t frt_record_batch_len(const frt_record_batch *rb) { return rb ? rb->n : 0; }
extern "C" uint64_t frt_record_batch_tail(const frt_record_batch *rb) { return rb ? rb->tail : 0; }
extern "C" uint64_t frt_record_batch_aux_fields(const frt_record_batch *rb) { return rb ? rb->n_aux : 0; }
extern "C" int frt_record_batch_device_ordinal(const frt_record_batch *rb) { return rb ? rb->device : -1; }
extern "C" void *frt_record_batch_ready_event(const frt_record_batch *rb) { return rb ? (void *)rb->ready : nullptr; }

extern "C" int frt_record_batch_column(const frt_record_batch *rb, int column, void **ptr, size_t *bytes, size_t *width)
{
    if (!rb || column < 0 || column >= FRT_COL_COUNT) return FRT_ERR_INVALID_ARGUMENT;
    if (ptr) *ptr = column == FRT_COL_AUX_ENTRIES ? (void *)rb->aux : (void *)(rb->cols + rb->col_off[column]);
    if (bytes) *bytes = rb->col_bytes[column];
    if (width) *width = bam_column_width(column);
    return FRT_OK;
}

extern "C" int frt_record_batch_column_to_host(const frt_record_batch *rb, int column, void *dst, size_t cap,
                                               frt_error *err)
{
    if (!rb || column < 0 || column >= FRT_COL_COUNT) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "bad column %d", column);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    size_t bytes = rb->col_bytes[column];
    if (cap < bytes) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "destination holds %zu bytes, column has %zu",
                  cap, bytes);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (!bytes) return FRT_OK;
    DeviceGuardLite g(rb->device);
    const uint8_t *src = column == FRT_COL_AUX_ENTRIES ? rb->aux : rb->cols + rb->col_off[column];
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, rb->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(rb->stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "downloading column");
    return FRT_OK;
}

// ---- record fields over a record batch ----------------------------------------
static RecordView view_of(const frt_record_batch *rb)
{
    auto col = [rb](int k) { return (const void *)(rb->cols + rb->col_off[k]); };
    RecordView v;
    v.buf = rb->source ? rb->source->data : nullptr;
    v.n = rb->n;
    v.record_offsets = (const uint64_t *)col(FRT_COL_RECORD_OFFSETS);
    v.cigar_start = (const uint32_t *)col(FRT_COL_CIGAR_START);
    v.sequence_start = (const uint32_t *)col(FRT_COL_SEQUENCE_START);
    v.quality_start = (const uint32_t *)col(FRT_COL_QUALITY_START);
    v.aux_start = (const uint32_t *)col(FRT_COL_AUX_START);
    v.record_end = (const uint32_t *)col(FRT_COL_RECORD_END);
    v.seq_len = (const uint32_t *)col(FRT_COL_SEQ_LEN);
    v.aux_count = (const uint32_t *)col(FRT_COL_AUX_COUNT);
    v.aux_first = (const uint32_t *)col(FRT_COL_AUX_FIRST);
    v.aux_entries = (const uint32_t *)rb->aux;
    v.n_cigar = (const uint16_t *)col(FRT_COL_N_CIGAR);
    v.name_len = (const uint8_t *)col(FRT_COL_NAME_LEN);
    v.aux_status = (const uint8_t *)col(FRT_COL_AUX_STATUS);
    return v;
}

static int rb_fields(const frt_record_batch *rb, int op, const char *tag, frt_columns **out, frt_error *err)
{
    if (!rb) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null record batch");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(rb->device);
    return fields_run(view_of(rb), op, tag, rb->device, rb->stream, rb->shared, rb->ready, rb->source, out, err);
}

extern "C" int frt_record_batch_aux_lookup(const frt_record_batch *rb, const char tag[2], frt_columns **out,
                                           frt_error *err)
{
    return rb_fields(rb, FIELDS_AUX_LOOKUP, tag, out, err);
}

extern "C" int frt_record_batch_cigar_resolved(const frt_record_batch *rb, frt_columns **out, frt_error *err)
{
    return rb_fields(rb, FIELDS_CIGAR_RESOLVED, nullptr, out, err);
}

extern "C" int frt_record_batch_unpack_sequences(const frt_record_batch *rb, frt_columns **out, frt_error *err)
{
    return rb_fields(rb, FIELDS_UNPACK_SEQUENCES, nullptr, out, err);
}

extern "C" int frt_record_batch_compact(const frt_record_batch *rb, frt_columns **out, frt_error *err)
{
    return rb_fields(rb, FIELDS_COMPACT, nullptr, out, err);
}

extern "C" void frt_record_batch_free(frt_record_batch *rb)
{
    if (!rb) return;
    {
        DeviceGuardLite g(rb->device);
        dev_free(rb->aux, rb->stream);
        dev_free(rb->cols, rb->stream);
        if (rb->ready) cudaEventDestroy(rb->ready);
    }
    if (rb->source) batch_release(rb->source);
    rb_discard(rb);
}
