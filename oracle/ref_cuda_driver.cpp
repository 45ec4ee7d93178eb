/*
 * TEST INFRASTRUCTURE ONLY.  Runs the reference's own CUDA kernels on the GPU
 * in the reference's launch order, to time its CUDA path beside this
 * library's and to check its results against the oracle.
 *
 * The kernels come from oracle/_ref/ref_kernels_sm103a.cubin, which
 * oracle/build.py compiles from the reference's kernels/inflate.cu and
 * kernels/bam_decode.cu (ref_cuda_kernels.cu).  This file restates the host
 * side that drives them:
 *   - the reader, DeviceBgzfReader::next_batch / carry_from
 *     (crates/fritillaria-bgzf/src/device_read.rs:155-280): a window of the
 *     carried bytes plus blocks_per_batch x 64 KiB read fresh, the complete
 *     members in it form the batch, a partial trailing member and, after the
 *     decode, every member from the one holding the record tail lead the next
 *     window;
 *   - the codec, CudaContext::launch_inflate and verify_and_offsets
 *     (crates/fritillaria-cuda/src/backend.rs:221-256, 635-720): upload the
 *     window and the plan, synchronise, inflate_blocks<<<ceil(n/256), 256>>>,
 *     synchronise, download status/produced/crc and verify on the host in
 *     span order (status, then ISIZE, then CRC);
 *   - the decoder, BamDecoder::decode (crates/fritillaria-cuda/src/bam.rs:
 *     324-573): upload the block starts, bam_scan_blocks (a thread per
 *     block), bam_reconcile<<<1, 1>>>, download the three totals,
 *     bam_emit_offsets, bam_decode_fields (a thread per record).
 * Allocation is stream-ordered (cudaMallocAsync), as cudarc's stream
 * allocations are.  The BAM header is parsed on the host from the first
 * batch, as the reference's consumer loop does (examples/bench_decode.rs:
 * 105-113).
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "frt_oracle.h"

namespace {

struct Module {
    CUmodule mod = nullptr;
    CUfunction inflate = nullptr, scan = nullptr, reconcile = nullptr, emit = nullptr, decode = nullptr;
    int device = -1;
};
Module g_mod;
std::string g_err;

bool cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

bool drv_ok(CUresult r, const char *what)
{
    if (r == CUDA_SUCCESS) return true;
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "driver error");
    return false;
}

bool launch(CUfunction f, unsigned grid, unsigned block, cudaStream_t st, void **args, const char *what)
{
    if (grid == 0) return true;
    return drv_ok(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, (CUstream)st, args, nullptr), what);
}

template <class T> T *dalloc(size_t n, cudaStream_t st)
{
    void *p = nullptr;
    if (cudaMallocAsync(&p, n ? n * sizeof(T) : 1, st) != cudaSuccess) return nullptr;
    return (T *)p;
}

} // namespace

extern "C" {

typedef struct {
    uint64_t records;
    uint64_t inflated_bytes;
    uint64_t members;    /* members inflated, counting re-inflated carries */
    uint64_t consumed_bytes; /* inflated bytes consumed once (the carried member's bytes count in the next batch) */
    uint64_t batches;
    double seconds;      /* wall time of the whole loop */
    double inflate_ms;   /* inflate_blocks kernel time, summed over batches (CUDA events) */
    double reconcile_ms; /* bam_reconcile<<<1,1>>> kernel time, summed */
    double kernels_ms;   /* every kernel of the path, summed */
    int32_t status;      /* 0, or the frt_status of the first failure */
} refcu_result;

/* Optional host outputs for parity: record offsets in whole-file inflated
 * coordinates and four columns, `cap` records. */
typedef struct {
    uint64_t *record_offsets;
    int32_t *ref_id;
    int32_t *pos;
    uint16_t *flags;
    uint32_t *seq_len;
    uint64_t cap;
} refcu_columns;

const char *refcu_last_error(void) { return g_err.c_str(); }

int refcu_open(const char *cubin_path, int device)
{
    if (g_mod.mod && g_mod.device == device) return 0;
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice") || !cuda_ok(cudaFree(nullptr), "context")) return -1;
    if (!drv_ok(cuModuleLoad(&g_mod.mod, cubin_path), "loading the reference cubin")) return -1;
    if (!drv_ok(cuModuleGetFunction(&g_mod.inflate, g_mod.mod, "inflate_blocks"), "inflate_blocks") ||
        !drv_ok(cuModuleGetFunction(&g_mod.scan, g_mod.mod, "bam_scan_blocks"), "bam_scan_blocks") ||
        !drv_ok(cuModuleGetFunction(&g_mod.reconcile, g_mod.mod, "bam_reconcile"), "bam_reconcile") ||
        !drv_ok(cuModuleGetFunction(&g_mod.emit, g_mod.mod, "bam_emit_offsets"), "bam_emit_offsets") ||
        !drv_ok(cuModuleGetFunction(&g_mod.decode, g_mod.mod, "bam_decode_fields"), "bam_decode_fields"))
        return -1;
    g_mod.device = device;
    return 0;
}

/* Runs the loop over the file; with stop_after > 0 the consumer stops once
 * the next batch would start at or past that compressed offset (a bounded
 * sample of the file). */
int refcu_run_bam(const uint8_t *file, uint64_t len, uint32_t blocks_per_batch, uint64_t stop_after,
                  refcu_result *res, const refcu_columns *cols)
{
    memset(res, 0, sizeof *res);
    if (!g_mod.mod) {
        g_err = "refcu_open was not called";
        return res->status = -1;
    }
    const uint32_t BLOCK = 256; /* backend.rs:27, bam.rs:203 */
    const uint64_t want = (uint64_t)blocks_per_batch * 65536u;
    cudaStream_t st = nullptr;
    if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) return res->status = -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // whole-file inflated coordinates of each member, for the parity outputs
    std::vector<orc_span> all;
    std::vector<uint64_t> all_out;
    if (cols) {
        all.resize(len / 28 + 1);
        size_t n = 0, used = 0;
        orc_error oe;
        orc_bgzf_discover(file, len, 0, all.data(), all.size(), &n, &used, &oe);
        all.resize(n);
        all_out.resize(n + 1);
        uint64_t t = 0;
        for (size_t i = 0; i < n; ++i) { all_out[i] = t; t += all[i].isize; }
        all_out[n] = t;
    }

    auto t0 = std::chrono::steady_clock::now();
    uint64_t batch_offset = 0; // compressed offset of the window's first byte
    uint64_t read_pos = 0;     // next byte not yet read into any window
    uint64_t carry_start = 0;  // record start in the window's first member
    bool header_done = false;
    int32_t n_ref = 0;
    int status = 0;
    std::vector<orc_span> spans(want / 28 + 1024);
    auto kernel_ms = [&](double *acc) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *acc += ms;
        res->kernels_ms += ms;
    };
    uint64_t prev_start = UINT64_MAX, prev_end = 0; // the last window inflated
    while (!status) {
        if (batch_offset >= len) break;
        if (stop_after && batch_offset >= stop_after) break;
        // nothing new can be read and the window would be rebuilt identically:
        // the stream ends inside a record (device_read.rs:190-203)
        if (read_pos >= len && batch_offset == prev_start && prev_end == len) {
            status = 6;
            break;
        }
        uint64_t end = read_pos + want < len ? read_pos + want : len;
        read_pos = end;
        const uint8_t *win = file + batch_offset;
        uint64_t wlen = end - batch_offset;
        if (wlen == 0) break;
        size_t n = 0, consumed = 0;
        if (spans.size() < wlen / 28 + 1024) spans.resize(wlen / 28 + 1024);
        orc_error oe;
        if (orc_bgzf_discover(win, wlen, batch_offset, spans.data(), spans.size(), &n, &consumed, &oe)) {
            status = oe.code;
            break;
        }
        if (n == 0) {
            if (end == len) {
                if (wlen) status = 6; /* truncated BGZF / ends inside a record */
                break;
            }
            continue;
        }
        // the plan (BatchPlan::new): output offsets at the ISIZE prefix sum
        std::vector<uint64_t> in_off(n), out_off(n + 1);
        std::vector<uint32_t> in_len(n), caps(n);
        uint64_t total = 0;
        for (size_t i = 0; i < n; ++i) {
            in_off[i] = spans[i].payload_start;
            in_len[i] = (uint32_t)spans[i].payload_len;
            caps[i] = spans[i].isize;
            out_off[i] = total;
            total += spans[i].isize;
        }
        out_off[n] = total;
        const uint64_t after_members = batch_offset + consumed; // partial trailing member, if any, is carried
        if (total == 0) {
            // only empty members (an EOF marker): read on
            batch_offset = after_members;
            if (end == len) break;
            continue;
        }
        res->batches++;
        res->members += n;
        prev_start = batch_offset;
        prev_end = end;
        // upload (backend.rs upload) and synchronise
        uint8_t *d_in = dalloc<uint8_t>(consumed, st);
        uint64_t *d_in_off = dalloc<uint64_t>(n, st), *d_out_off = dalloc<uint64_t>(n, st);
        uint32_t *d_in_len = dalloc<uint32_t>(n, st), *d_caps = dalloc<uint32_t>(n, st);
        uint8_t *d_out = dalloc<uint8_t>(total, st);
        uint32_t *d_status = dalloc<uint32_t>(n, st), *d_prod = dalloc<uint32_t>(n, st), *d_crc = dalloc<uint32_t>(n, st);
        if (!d_in || !d_in_off || !d_out_off || !d_in_len || !d_caps || !d_out || !d_status || !d_prod || !d_crc) {
            g_err = "device allocation failed";
            status = -1;
            break;
        }
        cudaMemcpyAsync(d_in, win, consumed, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_in_off, in_off.data(), 8 * n, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_in_len, in_len.data(), 4 * n, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_out_off, out_off.data(), 8 * n, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d_caps, caps.data(), 4 * n, cudaMemcpyHostToDevice, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "upload")) { status = -1; break; }
        int count = (int)n;
        void *ia[] = {&d_in, &d_in_off, &d_in_len, &d_out, &d_out_off, &d_caps, &d_status, &d_prod, &d_crc, &count};
        cudaEventRecord(e0, st);
        if (!launch(g_mod.inflate, (unsigned)((n + BLOCK - 1) / BLOCK), BLOCK, st, ia, "inflate_blocks")) { status = -1; break; }
        cudaEventRecord(e1, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "inflate_blocks")) { status = -1; break; }
        kernel_ms(&res->inflate_ms);
        std::vector<uint32_t> h_status(n), h_prod(n), h_crc(n);
        cudaMemcpyAsync(h_status.data(), d_status, 4 * n, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(h_prod.data(), d_prod, 4 * n, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(h_crc.data(), d_crc, 4 * n, cudaMemcpyDeviceToHost, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "status download")) { status = -1; break; }
        for (size_t i = 0; i < n && !status; ++i) {
            if (h_status[i]) status = 5;                    /* Inflate */
            else if (h_prod[i] != caps[i]) status = 4;      /* SizeMismatch */
            else if (h_crc[i] != spans[i].crc32) status = 3; /* ChecksumMismatch */
        }
        cudaFreeAsync(d_in, st);
        cudaFreeAsync(d_in_off, st);
        cudaFreeAsync(d_in_len, st);
        cudaFreeAsync(d_out_off, st);
        cudaFreeAsync(d_caps, st);
        cudaFreeAsync(d_status, st);
        cudaFreeAsync(d_prod, st);
        cudaFreeAsync(d_crc, st);
        if (status) {
            cudaFreeAsync(d_out, st);
            break;
        }
        res->inflated_bytes += total;
        uint64_t start = carry_start;
        carry_start = 0;
        if (!header_done) {
            // the consumer loop parses the header on the host from batch 0
            std::vector<uint8_t> head(total);
            cudaMemcpyAsync(head.data(), d_out, total, cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            uint64_t rs = 0;
            if (orc_bam_header(head.data(), total, &rs, &n_ref, &oe)) {
                // the header runs past this batch: carry everything
                cudaFreeAsync(d_out, st);
                res->inflated_bytes -= total;
                res->batches--;
                prev_start = batch_offset;
                prev_end = end;
                continue; // batch_offset unchanged: the window grows
            }
            header_done = true;
            start = rs;
        }
        // BamDecoder::decode: boundaries, then fields
        uint64_t *d_starts = dalloc<uint64_t>(n + 1, st);
        uint32_t *d_spec_counts = dalloc<uint32_t>(n, st);
        uint64_t *d_spec_lands = dalloc<uint64_t>(n, st);
        uint8_t *d_spec_complete = dalloc<uint8_t>(n, st), *d_spec_valid = dalloc<uint8_t>(n, st);
        uint64_t *d_entries = dalloc<uint64_t>(n, st), *d_totals = dalloc<uint64_t>(3, st);
        uint32_t *d_counts = dalloc<uint32_t>(n, st), *d_first = dalloc<uint32_t>(n, st);
        cudaMemcpyAsync(d_starts, out_off.data(), 8 * (n + 1), cudaMemcpyHostToDevice, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "block starts")) { status = -1; break; }
        uint64_t blen = total;
        void *sa[] = {&d_out, &blen, &d_starts, &count, &d_spec_counts, &d_spec_lands, &d_spec_complete, &d_spec_valid};
        cudaEventRecord(e0, st);
        if (!launch(g_mod.scan, (unsigned)((n + BLOCK - 1) / BLOCK), BLOCK, st, sa, "bam_scan_blocks")) { status = -1; break; }
        cudaEventRecord(e1, st);
        cudaStreamSynchronize(st);
        {
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            res->kernels_ms += ms;
        }
        void *ra[] = {&d_out, &blen, &d_starts, &count, &start, &d_spec_counts, &d_spec_lands, &d_spec_complete,
                      &d_spec_valid, &d_entries, &d_counts, &d_first, &d_totals};
        cudaEventRecord(e0, st);
        if (!launch(g_mod.reconcile, 1, 1, st, ra, "bam_reconcile")) { status = -1; break; }
        cudaEventRecord(e1, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "bam_reconcile")) { status = -1; break; }
        kernel_ms(&res->reconcile_ms);
        uint64_t tot[3] = {0, 0, 0};
        cudaMemcpyAsync(tot, d_totals, sizeof tot, cudaMemcpyDeviceToHost, st);
        if (!cuda_ok(cudaStreamSynchronize(st), "totals")) { status = -1; break; }
        if (tot[2]) {
            status = 6; /* Malformed */
            break;
        }
        uint64_t nrec = tot[0], tail = tot[1];
        uint64_t *d_rec = dalloc<uint64_t>(nrec, st);
        int32_t *c_ref = dalloc<int32_t>(nrec, st), *c_pos = dalloc<int32_t>(nrec, st), *c_mref = dalloc<int32_t>(nrec, st),
                *c_mpos = dalloc<int32_t>(nrec, st), *c_tlen = dalloc<int32_t>(nrec, st);
        uint16_t *c_flags = dalloc<uint16_t>(nrec, st);
        uint8_t *c_mapq = dalloc<uint8_t>(nrec, st);
        uint32_t *c_len = dalloc<uint32_t>(nrec, st), *c_cs = dalloc<uint32_t>(nrec, st), *c_ss = dalloc<uint32_t>(nrec, st),
                 *c_qs = dalloc<uint32_t>(nrec, st), *c_as = dalloc<uint32_t>(nrec, st), *c_end = dalloc<uint32_t>(nrec, st);
        if (nrec) {
            void *ea[] = {&d_out, &d_entries, &d_counts, &d_first, &count, &d_rec};
            cudaEventRecord(e0, st);
            if (!launch(g_mod.emit, (unsigned)((n + BLOCK - 1) / BLOCK), BLOCK, st, ea, "bam_emit_offsets")) { status = -1; break; }
            uint32_t nr32 = (uint32_t)nrec;
            void *da[] = {&d_out, &d_rec, &nr32, &c_ref, &c_pos, &c_flags, &c_mapq, &c_len, &c_mref, &c_mpos, &c_tlen,
                          &c_cs, &c_ss, &c_qs, &c_as, &c_end};
            if (!launch(g_mod.decode, (unsigned)((nrec + BLOCK - 1) / BLOCK), BLOCK, st, da, "bam_decode_fields")) { status = -1; break; }
            cudaEventRecord(e1, st);
            if (!cuda_ok(cudaStreamSynchronize(st), "decode")) { status = -1; break; }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            res->kernels_ms += ms;
            if (cols && res->records + nrec <= cols->cap) {
                // whole-file coordinates: the batch's first member's place in the file
                size_t k = 0;
                while (k < all.size() && all[k].compressed_offset < spans[0].compressed_offset) ++k;
                const uint64_t base = all_out[k];
                std::vector<uint64_t> ro(nrec);
                cudaMemcpyAsync(ro.data(), d_rec, 8 * nrec, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(cols->ref_id + res->records, c_ref, 4 * nrec, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(cols->pos + res->records, c_pos, 4 * nrec, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(cols->flags + res->records, c_flags, 2 * nrec, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(cols->seq_len + res->records, c_len, 4 * nrec, cudaMemcpyDeviceToHost, st);
                cudaStreamSynchronize(st);
                for (uint64_t i = 0; i < nrec; ++i) cols->record_offsets[res->records + i] = base + ro[i];
            }
        }
        res->records += nrec;
        // the columns are the batch's result: released when the consumer drops it
        void *frees[] = {d_starts, d_spec_counts, d_spec_lands, d_spec_complete, d_spec_valid, d_entries, d_totals,
                         d_counts, d_first, d_rec, c_ref, c_pos, c_mref, c_mpos, c_tlen, c_flags, c_mapq, c_len,
                         c_cs, c_ss, c_qs, c_as, c_end, d_out};
        for (void *p : frees) cudaFreeAsync(p, st);
        // carry_from(tail): every member from the one holding the tail
        if (tail < total) {
            size_t b = 0;
            while (b + 1 < n && out_off[b + 1] <= tail) ++b;
            batch_offset = spans[b].compressed_offset;
            carry_start = tail - out_off[b];
            res->consumed_bytes += out_off[b];
        } else {
            batch_offset = after_members;
            res->consumed_bytes += total;
        }
    }
    cudaStreamSynchronize(st);
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    res->status = status;
    return status;
}

} // extern "C"
