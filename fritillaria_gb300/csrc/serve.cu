// Region serving: BAI-resolved region queries over BAMs resident in device
// memory, batched continuously into one persistent inflate per tick.
//
// A request (file, reference, [start, end]) resolves through the file's BAI
// (frt_bai_query: BinningIndex::query, crates/fritillaria-csi/src/binning_index/index.rs:93-119)
// to chunks of virtual offsets; each chunk names the members that hold the
// records starting inside it (crates/fritillaria-csi/src/io/query.rs reads a
// chunk from its start until the reader's virtual position reaches its end),
// plus `extra` members after it so a record starting in the last member is
// whole.  Each chunk becomes one record chain ("segment").
//
// A tick takes every queued request that fits the HBM budget and runs, on the
// server's stream with no host round trip in between:
//   upload     one copy of the tick's member and segment tables;
//   inflate    the persistent warp-per-member kernel over all the members of
//              all the requests, longest first, CRC32/ISIZE verified;
//   scan       per-member speculation and a per-segment reconcile (one CTA per
//              segment), then the region filter (query.rs:97-122) counting the
//              records each member keeps;
//   emit       an exclusive scan of the kept counts and the ordered write of
//              the kept records' columns;
//   status     one copy back of the per-member statuses, kept offsets and
//              per-segment totals, then an event.
// progress() polls the events: a finished tick's requests complete (or, if a
// chunk's last record was cut by the member budget, go back to the queue
// with more trailing members), and new ticks launch while earlier ones run.
// Each request's results are a slice of its tick's columns and inflated
// bytes, freed when the last request of the tick is released.

#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "bam.cuh"
#include "common.cuh"
#include "inflate.cuh"
#include "runtime.h"

using namespace frt;

namespace {

double host_ms(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

struct SrvFile {
    uint64_t arena_off = 0, len = 0;
    std::vector<uint64_t> coff;     // member compressed offsets, plus len
    std::vector<uint64_t> pay_off;  // payload offsets
    std::vector<uint32_t> pay_len, isize, crc;
    frt_bai *bai = nullptr;
    int32_t n_ref = -1;
};

struct Tick;

struct SrvReq {
    uint64_t id = 0;
    int32_t file = 0, ref = 0;
    uint64_t beg = 0, end = 0;
    std::vector<frt_chunk> chunks;
    uint32_t extra = 1; // members read past each chunk's last member
    uint32_t retries = 0;
    int state = 0;      // 0 queued, 1 running, 2 done
    int status = FRT_OK;
    frt_error err{};
    double arrival_ms = 0, done_ms = 0;
    uint64_t inflated = 0, members = 0;
    // result: a slice of the tick's columns
    std::shared_ptr<Tick> tick;
    uint64_t first = 0, n = 0;
    uint64_t out_base = 0, out_len = 0; // the request's inflated bytes in the tick arena
};

struct Tick {
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    uint8_t *arena = nullptr;
    FrtRegionColumns cols{};
    cudaEvent_t done = nullptr;
    cudaEvent_t ev_start = nullptr, ev_inflate = nullptr, ev_inflated = nullptr; // the tick's stages on the device
    double host_ms = 0;          // host time building and launching the tick
    void *host_status = nullptr; // pinned
    size_t host_bytes = 0;
    uint64_t budget_bytes = 0;
    std::vector<SrvReq *> reqs;
    // host copies of the plan
    struct SegPlan {
        uint32_t req;
        uint64_t chunk_end_pos; // arena offset of the chunk end (records must start before it)
    };
    std::vector<SegPlan> segs;
    std::vector<uint32_t> req_m0, req_m1; // member range of each request
    uint32_t n_members = 0, n_segs = 0;
    void *staging = nullptr;     // pinned copy of the uploaded tables
    uint64_t *in_use = nullptr;  // the server's budget counter
    ~Tick()
    {
        for (void *p : allocs) cudaFreeAsync(p, stream);
        if (done) cudaEventDestroy(done);
        for (cudaEvent_t ev : {ev_start, ev_inflate, ev_inflated})
            if (ev) cudaEventDestroy(ev);
        if (host_status) cudaFreeHost(host_status);
        if (staging) cudaFreeHost(staging);
        if (in_use) *in_use -= budget_bytes;
    }
};

} // namespace

struct frt_server {
    int device = 0;
    SharedStream *shared = nullptr;
    cudaStream_t stream = nullptr;
    uint64_t budget = 0, in_use = 0;
    // four ticks in flight, each on its own stream: a request that arrives
    // while ticks run starts in a tick of its own at once, on SMs the running
    // ticks leave idle (a small tick puts one member on each of few SMs)
    uint32_t max_batch = 0xffffffffu, max_ticks = 4;
    uint8_t *files_arena = nullptr;
    uint64_t files_bytes = 0, files_cap = 0;
    std::vector<SrvFile> files;
    std::map<uint64_t, std::unique_ptr<SrvReq>> reqs;
    std::deque<SrvReq *> queue;
    std::deque<std::shared_ptr<Tick>> running;
    uint64_t next_id = 1;
    std::chrono::steady_clock::time_point t0;
    cudaEvent_t origin = nullptr; // server clock zero on the device
    frt_codec *codec = nullptr;   // for reading BAM headers at add time
    frt_inflate_tuning tuning{};
    int inflate_grid = 0;
    // With more than one tick in flight each runs on a stream of its own
    // (created on first use, as many as ticks in flight), so a new tick's
    // kernels start on the SMs the running one leaves idle.
    std::vector<cudaStream_t> tick_streams;
    uint64_t tick_seq = 0;
    uint64_t pending = 0;         // submitted, not yet completed
    frt_server_stats stats{};     // per-stage totals over finished ticks
};

namespace {

// Member index holding compressed offset `c` (exact member start), or the
// member containing it.
uint64_t member_of(const SrvFile &f, uint64_t c)
{
    return (uint64_t)(std::upper_bound(f.coff.begin(), f.coff.end() - 1, c) - f.coff.begin()) - 1;
}

struct Plan {
    // per member (global index g)
    std::vector<uint64_t> in_off, out_off, coff;
    std::vector<uint32_t> in_len, isize, crc, seg_of, order;
    std::vector<uint64_t> starts; // per segment n + 1
    std::vector<FrtScanSeg> segs;
    uint64_t arena_bytes = 0, rec_bound = 0;
};

// Chunks -> segments -> members; appends to `pl`.  Returns the request's bytes.
void plan_request(frt_server *sv, SrvReq &r, uint32_t slot, Plan &pl, Tick &t)
{
    const SrvFile &f = sv->files[r.file];
    const uint64_t n_mem = f.isize.size();
    const uint64_t req_base = pl.arena_bytes;
    t.req_m0.push_back((uint32_t)pl.in_off.size());
    uint64_t members = 0;
    for (const frt_chunk &c : r.chunks) {
        uint64_t ma = member_of(f, c.start >> 16);
        uint64_t me = member_of(f, c.end >> 16);
        uint64_t last = ((c.end & 0xffff) == 0 && me > ma) ? me - 1 : me;
        uint64_t mz = std::min<uint64_t>(n_mem - 1, last + r.extra);
        FrtScanSeg sg{};
        sg.m0 = (uint32_t)pl.in_off.size();
        sg.n = (uint32_t)(mz - ma + 1);
        uint64_t seg_base = pl.arena_bytes, at = seg_base, end_pos = ~0ull;
        for (uint64_t m = ma; m <= mz; ++m) {
            if (m == me) end_pos = at + (c.end & 0xffff);
            pl.in_off.push_back(f.arena_off + f.pay_off[m]);
            pl.in_len.push_back(f.pay_len[m]);
            pl.isize.push_back(f.isize[m]);
            pl.crc.push_back(f.crc[m]);
            pl.out_off.push_back(at);
            pl.coff.push_back(f.coff[m]);
            pl.seg_of.push_back((uint32_t)pl.segs.size());
            pl.starts.push_back(at);
            at += f.isize[m];
        }
        pl.starts.push_back(at);
        if (end_pos == ~0ull) end_pos = at; // the chunk ends past the last member read
        sg.start = seg_base + (c.start & 0xffff);
        sg.len = at;
        sg.chunk_end = c.end;
        sg.beg = r.beg;
        sg.end = r.end;
        sg.ref = r.ref;
        sg.request = slot;
        sg.out_base = req_base;
        pl.segs.push_back(sg);
        t.segs.push_back({slot, end_pos});
        pl.arena_bytes = at;
        pl.rec_bound += (at - seg_base) / 36 + sg.n;
        members += sg.n;
    }
    t.req_m1.push_back((uint32_t)pl.in_off.size());
    r.members = members;
    r.out_base = req_base;
    r.out_len = pl.arena_bytes - req_base;
    r.inflated = r.out_len;
}

// Device bytes a tick of this plan takes.
uint64_t plan_bytes(const Plan &pl)
{
    uint64_t n = pl.in_off.size(), s = pl.segs.size();
    return pl.arena_bytes + 64 + n * (8 * 5 + 4 * 8 + 1 + 2ull * FRT_SCAN_CAP + 16) + s * (sizeof(FrtScanSeg) + 40) +
           pl.rec_bound * 35 + 4096;
}

template <typename T> int talloc(Tick &t, T **p, size_t n, frt_error *err)
{
    void *q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, n * sizeof(T) + 64, t.stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "allocating a tick");
    t.allocs.push_back(q);
    *p = (T *)q;
    return FRT_OK;
}

// Launches one tick over `batch`.
int launch_tick(frt_server *sv, std::vector<SrvReq *> &batch, frt_error *err)
{
    const double h0 = host_ms(sv->t0);
    auto t = std::make_shared<Tick>();
    t->stream = sv->stream;
    if (sv->max_ticks > 1) {
        while (sv->tick_streams.size() < sv->max_ticks) {
            cudaStream_t q = nullptr;
            cudaError_t ce = cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking);
            if (ce != cudaSuccess) return cuda_fail(err, ce, "creating a tick stream");
            sv->tick_streams.push_back(q);
        }
        t->stream = sv->tick_streams[sv->tick_seq++ % sv->max_ticks];
        // after everything already on the server's stream (file uploads, releases)
        cudaEvent_t ready = nullptr;
        cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
        cudaEventRecord(ready, sv->stream);
        cudaStreamWaitEvent(t->stream, ready, 0);
        cudaEventDestroy(ready);
    }
    for (cudaEvent_t *ev : {&t->ev_start, &t->ev_inflate, &t->ev_inflated}) cudaEventCreate(ev);
    cudaEventRecord(t->ev_start, t->stream);
    Plan pl;
    for (uint32_t i = 0; i < batch.size(); ++i) plan_request(sv, *batch[i], i, pl, *t);
    const uint32_t n = (uint32_t)pl.in_off.size(), ns = (uint32_t)pl.segs.size();
    t->n_members = n;
    t->n_segs = ns;
    t->reqs = batch;
    t->budget_bytes = plan_bytes(pl);
    // longest member first
    pl.order.resize(n);
    for (uint32_t i = 0; i < n; ++i) pl.order[i] = i;
    std::stable_sort(pl.order.begin(), pl.order.end(), [&](uint32_t a, uint32_t b) { return pl.in_len[a] > pl.in_len[b]; });
    // device tables: one packed upload
    uint64_t *in_off, *out_off, *coff, *starts, *entry, *land, *totals;
    uint32_t *in_len, *isize, *crc, *seg_of, *order, *status, *produced, *crc_out, *count, *first, *kept, *kept_first,
        *parts, *tot32;
    uint8_t *flags;
    uint16_t *scratch;
    FrtScanSeg *segs;
    unsigned long long *block_err;
    uint64_t *n_dev, *queue_head;
    int rc;
    const uint64_t rb = pl.rec_bound + 1;
    if ((rc = talloc(*t, &t->arena, pl.arena_bytes + 64, err)) || (rc = talloc(*t, &in_off, n + 1, err)) ||
        (rc = talloc(*t, &out_off, n + 1, err)) || (rc = talloc(*t, &coff, n + 1, err)) ||
        (rc = talloc(*t, &starts, n + ns + 1, err)) || (rc = talloc(*t, &in_len, n + 1, err)) ||
        (rc = talloc(*t, &isize, n + 1, err)) || (rc = talloc(*t, &crc, n + 1, err)) ||
        (rc = talloc(*t, &seg_of, n + 1, err)) || (rc = talloc(*t, &order, n + 1, err)) ||
        (rc = talloc(*t, &status, n + 1, err)) || (rc = talloc(*t, &produced, n + 1, err)) ||
        (rc = talloc(*t, &crc_out, n + 1, err)) || (rc = talloc(*t, &entry, n + 1, err)) ||
        (rc = talloc(*t, &land, n + 1, err)) || (rc = talloc(*t, &count, n + 1, err)) ||
        (rc = talloc(*t, &first, n + 1, err)) || (rc = talloc(*t, &kept, n + 1, err)) ||
        (rc = talloc(*t, &kept_first, n + 2, err)) || (rc = talloc(*t, &parts, frt_scan_partials_len(n) + 2, err)) ||
        (rc = talloc(*t, &flags, n + 1, err)) || (rc = talloc(*t, &scratch, (size_t)n * FRT_SCAN_CAP + 1, err)) ||
        (rc = talloc(*t, &segs, ns + 1, err)) || (rc = talloc(*t, &totals, 4ull * ns + 4, err)) ||
        (rc = talloc(*t, &block_err, 2, err)) || (rc = talloc(*t, &n_dev, 2, err)) ||
        (rc = talloc(*t, &queue_head, 2, err)) || (rc = talloc(*t, &tot32, 2, err)) ||
        (rc = talloc(*t, &t->cols.virtual_offset, rb, err)) || (rc = talloc(*t, &t->cols.record_offset, rb, err)) ||
        (rc = talloc(*t, &t->cols.ref_id, rb, err)) || (rc = talloc(*t, &t->cols.pos, rb, err)) ||
        (rc = talloc(*t, &t->cols.flags, rb, err)) || (rc = talloc(*t, &t->cols.mapq, rb, err)) ||
        (rc = talloc(*t, &t->cols.seq_len, rb, err)) || (rc = talloc(*t, &t->cols.request, rb, err)))
        return rc;
    cudaStream_t st = t->stream;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
    };
    // one pinned staging buffer, kept with the tick until it completes
    size_t stage_bytes = 8 * (3 * (size_t)n + n + ns + 1) + 4 * (5 * (size_t)n) + sizeof(FrtScanSeg) * ns + 128;
    std::vector<uint8_t> stage(stage_bytes);
    uint8_t *sp = stage.data();
    auto put = [&](const void *src, size_t bytes) {
        uint8_t *at = sp;
        if (bytes) memcpy(sp, src, bytes);
        sp += (bytes + 7) & ~(size_t)7;
        return at;
    };
    uint8_t *h_in_off = put(pl.in_off.data(), 8 * n), *h_out_off = put(pl.out_off.data(), 8 * n),
            *h_coff = put(pl.coff.data(), 8 * n), *h_starts = put(pl.starts.data(), 8 * (n + ns)),
            *h_in_len = put(pl.in_len.data(), 4 * n), *h_isize = put(pl.isize.data(), 4 * n),
            *h_crc = put(pl.crc.data(), 4 * n), *h_seg_of = put(pl.seg_of.data(), 4 * n),
            *h_order = put(pl.order.data(), 4 * n), *h_segs = put(pl.segs.data(), sizeof(FrtScanSeg) * ns);
    uint64_t nn = n;
    uint8_t *h_n = put(&nn, 8);
    cudaError_t e = cudaSuccess;
    void *pinned = nullptr;
    if ((e = cudaMallocHost(&pinned, stage_bytes)) != cudaSuccess) return cuda_fail(err, e, "staging a tick");
    t->staging = pinned;
    memcpy(pinned, stage.data(), stage_bytes);
    auto P = [&](uint8_t *h) { return (uint8_t *)pinned + (h - stage.data()); };
    if ((e = up(in_off, P(h_in_off), 8 * n)) || (e = up(out_off, P(h_out_off), 8 * n)) || (e = up(coff, P(h_coff), 8 * n)) ||
        (e = up(starts, P(h_starts), 8 * (n + ns))) || (e = up(in_len, P(h_in_len), 4 * n)) ||
        (e = up(isize, P(h_isize), 4 * n)) || (e = up(crc, P(h_crc), 4 * n)) || (e = up(seg_of, P(h_seg_of), 4 * n)) ||
        (e = up(order, P(h_order), 4 * n)) || (e = up(segs, P(h_segs), sizeof(FrtScanSeg) * ns)) ||
        (e = up(n_dev, P(h_n), 8)) ||
        (e = cudaMemsetAsync(queue_head, 0, 16, st)) || (e = cudaMemsetAsync(block_err, 0xff, 8, st)) ||
        (e = cudaMemsetAsync(totals, 0, 32ull * ns + 32, st)))
        return cuda_fail(err, e, "uploading a tick");
    // inflate every member of the tick
    cudaEventRecord(t->ev_inflate, st);
    // (a tick of fewer members than the tuned grid has warps is spread one
    // warp per CTA over the SMs by the launcher)
    if ((e = frt_launch_inflate_persistent(sv->files_arena, in_off, in_len, t->arena, out_off, isize, crc, status,
                                           produced, crc_out, order, n_dev, n, pl.arena_bytes, (u32 *)queue_head,
                                           (u32)sv->inflate_grid, block_err, sv->tuning, st)) != cudaSuccess)
        return cuda_fail(err, e, "launching the inflate");
    cudaEventRecord(t->ev_inflated, st);
    int32_t n_ref = 0; // bounds refID in the record-start test
    for (SrvReq *r : batch) n_ref = std::max(n_ref, sv->files[r->file].n_ref < 0 ? (1 << 24) : sv->files[r->file].n_ref);
    if ((e = frt_launch_region_scan(t->arena, segs, seg_of, ns, n, n_ref, starts, coff, entry, count, land, flags,
                                    scratch, first, totals, kept, st)) != cudaSuccess)
        return cuda_fail(err, e, "launching the region scan");
    if ((e = frt_launch_scan_u32(kept, n, parts, kept_first, tot32, st)) != cudaSuccess)
        return cuda_fail(err, e, "scanning kept records");
    if ((e = frt_launch_region_emit(t->arena, segs, seg_of, n, starts, coff, count, scratch, kept_first, t->cols, st)) !=
        cudaSuccess)
        return cuda_fail(err, e, "launching the region emit");
    // status back: statuses (n u32), kept_first (n + 1 u32), totals (4 x ns u64, 8-aligned)
    const uint64_t tot_off = (8ull * n + 4 + 7) & ~7ull;
    t->host_bytes = tot_off + 32ull * ns + 64;
    if ((e = cudaMallocHost(&t->host_status, t->host_bytes)) != cudaSuccess) return cuda_fail(err, e, "tick status");
    uint8_t *hs = (uint8_t *)t->host_status;
    if ((e = cudaMemcpyAsync(hs, status, 4ull * n, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(hs + 4ull * n, kept_first, 4ull * (n + 1), cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(hs + tot_off, totals, 32ull * ns, cudaMemcpyDeviceToHost, st)))
        return cuda_fail(err, e, "reading tick status");
    cudaEventCreate(&t->done);
    cudaEventRecord(t->done, st);
    for (SrvReq *r : batch) r->state = 1;
    sv->in_use += t->budget_bytes;
    t->in_use = &sv->in_use; // released when the tick's memory is
    sv->running.push_back(t);
    t->host_ms = host_ms(sv->t0) - h0;
    return FRT_OK;
}

// A finished tick: statuses, results, or back to the queue for more members.
void finish_tick(frt_server *sv, std::shared_ptr<Tick> t, uint32_t *completed)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, sv->origin, t->done);
    const uint32_t n = t->n_members, ns = t->n_segs;
    {
        float up = 0, inf = 0, rest = 0;
        cudaEventElapsedTime(&up, t->ev_start, t->ev_inflate);
        cudaEventElapsedTime(&inf, t->ev_inflate, t->ev_inflated);
        cudaEventElapsedTime(&rest, t->ev_inflated, t->done);
        frt_server_stats &st = sv->stats;
        st.ticks++;
        st.requests += t->reqs.size();
        st.members += n;
        st.host_ms += t->host_ms;
        st.upload_ms += up;
        st.inflate_ms += inf;
        st.scan_ms += rest;
        if (inf > st.max_inflate_ms) st.max_inflate_ms = inf;
    }
    const uint8_t *hs = (const uint8_t *)t->host_status;
    const uint32_t *status = (const uint32_t *)hs;
    const uint32_t *kept_first = (const uint32_t *)(hs + 4ull * n);
    const uint64_t *totals = (const uint64_t *)(hs + ((8ull * n + 4 + 7) & ~7ull));
    std::vector<uint8_t> cut(t->reqs.size(), 0), bad(t->reqs.size(), 0);
    for (uint32_t s = 0; s < ns; ++s) {
        uint32_t q = t->segs[s].req;
        if (totals[4ull * s + 2]) bad[q] = 1; // malformed record in the chain
        else if (totals[4ull * s + 1] < t->segs[s].chunk_end_pos) cut[q] = 1;
    }
    for (uint32_t q = 0; q < t->reqs.size(); ++q) {
        SrvReq *r = t->reqs[q];
        uint32_t m0 = t->req_m0[q], m1 = t->req_m1[q];
        for (uint32_t m = m0; m < m1 && r->status == FRT_OK; ++m) {
            if (status[m] != INF_OK) {
                r->status = FRT_ERR_INFLATE;
                set_error(&r->err, FRT_ERR_INFLATE, 0, 0, 0, 0, nullptr, "%s", inflate_status_message(status[m]));
            }
        }
        if (r->status == FRT_OK && bad[q]) {
            r->status = FRT_ERR_MALFORMED;
            set_error(&r->err, FRT_ERR_MALFORMED, 0, 0, 0, 0, "bam", "malformed record in a region chunk");
        }
        if (r->status == FRT_OK && cut[q] && r->extra < 1u << 20) {
            // a record starting inside a chunk runs past the members read
            r->extra = r->extra * 4 + 4;
            r->retries++;
            r->state = 0;
            sv->queue.push_front(r);
            continue;
        }
        r->first = kept_first[m0];
        r->n = kept_first[m1] - kept_first[m0];
        r->tick = t;
        r->state = 2;
        r->done_ms = ms;
        sv->pending--;
        if (completed) (*completed)++;
    }
    // the budget stays charged while any request holds the tick's results
    cudaFreeHost(t->host_status);
    t->host_status = nullptr;
    cudaFreeHost(t->staging);
    t->staging = nullptr;
}

} // namespace

extern "C" int frt_server_create(int device, void *stream, uint64_t budget_bytes, frt_server **out, frt_error *err)
{
    int rc = check_device(device, err);
    if (rc) return rc;
    DeviceGuardLite g(device);
    configure_pool(device);
    cudaError_t ce = frt_inflate_prepare();
    if (ce != cudaSuccess) return cuda_fail(err, ce, "configuring inflate kernels");
    SharedStream *ss = stream_create(device, stream, err);
    if (!ss) return FRT_ERR_CUDA;
    frt_server *s = new frt_server;
    s->device = device;
    s->shared = ss;
    s->stream = ss->s;
    s->budget = budget_bytes;
    s->tuning = frt_inflate_default();
    s->inflate_grid = frt_inflate_persistent_grid(s->tuning);
    s->t0 = std::chrono::steady_clock::now();
    cudaEventCreate(&s->origin);
    cudaEventRecord(s->origin, s->stream);
    cudaEventSynchronize(s->origin);
    if ((rc = frt_codec_create(device, s->stream, &s->codec, err))) {
        stream_release(ss);
        delete s;
        return rc;
    }
    *out = s;
    return FRT_OK;
}

extern "C" void frt_server_destroy(frt_server *s)
{
    if (!s) return;
    DeviceGuardLite g(s->device);
    cudaStreamSynchronize(s->stream);
    for (cudaStream_t q : s->tick_streams) cudaStreamSynchronize(q);
    s->running.clear();
    s->reqs.clear();
    for (cudaStream_t q : s->tick_streams) {
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
    }
    for (auto &f : s->files) frt_bai_free(f.bai);
    if (s->files_arena) cudaFree(s->files_arena);
    frt_codec_destroy(s->codec);
    cudaEventDestroy(s->origin);
    stream_release(s->shared);
    delete s;
}

extern "C" void frt_server_set_limits(frt_server *s, uint32_t max_requests_per_tick, uint32_t max_ticks_in_flight)
{
    if (!s) return;
    s->max_batch = max_requests_per_tick ? max_requests_per_tick : 0xffffffffu;
    s->max_ticks = max_ticks_in_flight ? max_ticks_in_flight : 1;
}

extern "C" double frt_server_clock_ms(const frt_server *s) { return s ? host_ms(s->t0) : 0.0; }

extern "C" int frt_server_get_stats(const frt_server *s, frt_server_stats *out, int32_t reset)
{
    if (!s || !out) return FRT_ERR_INVALID_ARGUMENT;
    *out = s->stats;
    if (reset) const_cast<frt_server *>(s)->stats = frt_server_stats{};
    return FRT_OK;
}

extern "C" int frt_server_add_bam(frt_server *s, const uint8_t *bgzf, size_t len, const uint8_t *bai, size_t bai_len,
                                  int32_t *file_id, frt_error *err)
{
    if (!s || !bgzf || !bai || !file_id) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    DeviceGuardLite g(s->device);
    if (!s->running.empty()) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "add files before serving requests");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    SrvFile f;
    int rc = frt_bai_parse(bai, bai_len, &f.bai, err);
    if (rc) return rc;
    std::vector<frt_span> spans;
    size_t used = 0;
    if ((rc = discover(bgzf, len, 0, spans, &used, err))) {
        frt_bai_free(f.bai);
        return rc;
    }
    for (auto &sp : spans) {
        f.coff.push_back(sp.compressed_offset);
        f.pay_off.push_back(sp.payload_start);
        f.pay_len.push_back((uint32_t)sp.payload_len);
        f.isize.push_back(sp.isize);
        f.crc.push_back(sp.crc32);
    }
    f.coff.push_back(len);
    f.len = len;
    // the BAM header, inflated on the device from the leading members
    for (size_t k = 1; k <= spans.size(); k *= 2) {
        size_t take = std::min(k, spans.size());
        uint64_t bytes = 0;
        for (size_t i = 0; i < take; ++i) bytes += spans[i].isize;
        std::vector<uint8_t> host(bytes + 1);
        std::vector<uint64_t> offs(take + 1);
        if ((rc = frt_codec_inflate_batch_host(s->codec, bgzf, len, spans.data(), take, host.data(), host.size(),
                                               offs.data(), err))) {
            frt_bai_free(f.bai);
            return rc;
        }
        uint64_t rs = 0;
        rc = frt_bam_parse_header(host.data(), bytes, &rs, &f.n_ref, err);
        if (rc == FRT_OK) break;
        if (rc != FRT_ERR_MALFORMED || take == spans.size()) {
            frt_bai_free(f.bai);
            return rc;
        }
    }
    // into the file arena
    uint64_t need = s->files_bytes + ((len + 255) & ~255ull);
    if (need > s->files_cap) {
        uint64_t cap = std::max<uint64_t>(need, s->files_cap * 2);
        uint8_t *a = nullptr;
        cudaError_t e = cudaMalloc(&a, cap);
        if (e != cudaSuccess) {
            frt_bai_free(f.bai);
            return cuda_fail(err, e, "allocating the file arena");
        }
        if (s->files_bytes) cudaMemcpy(a, s->files_arena, s->files_bytes, cudaMemcpyDeviceToDevice);
        if (s->files_arena) cudaFree(s->files_arena);
        s->files_arena = a;
        s->files_cap = cap;
    }
    f.arena_off = s->files_bytes;
    cudaError_t e = cudaMemcpy(s->files_arena + f.arena_off, bgzf, len, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        frt_bai_free(f.bai);
        return cuda_fail(err, e, "uploading a file");
    }
    s->files_bytes = need;
    *file_id = (int32_t)s->files.size();
    s->files.push_back(std::move(f));
    return FRT_OK;
}

extern "C" int frt_server_submit(frt_server *s, int32_t file, int32_t ref, uint64_t start, uint64_t end,
                                 double arrival_ms, uint64_t *request, frt_error *err)
{
    if (!s || !request || file < 0 || (size_t)file >= s->files.size()) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "no file %d", file);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    auto r = std::make_unique<SrvReq>();
    r->file = file;
    r->ref = ref;
    r->beg = start ? start : 1;
    r->end = end;
    size_t n = 0;
    const frt_bai *bai = s->files[file].bai;
    int rc = frt_bai_query(bai, ref, start, end, nullptr, 0, &n, err);
    if (rc && n == 0) return rc;
    r->chunks.resize(n);
    if (n && (rc = frt_bai_query(bai, ref, start, end, r->chunks.data(), n, &n, err))) return rc;
    if (!r->end) r->end = (1ull << 29) - 1;
    r->arrival_ms = arrival_ms >= 0 ? arrival_ms : host_ms(s->t0);
    r->id = s->next_id++;
    *request = r->id;
    SrvReq *p = r.get();
    s->reqs[r->id] = std::move(r);
    if (p->chunks.empty()) {
        p->state = 2;
        p->done_ms = host_ms(s->t0);
        return FRT_OK;
    }
    s->queue.push_back(p);
    s->pending++;
    return FRT_OK;
}

extern "C" int frt_server_progress(frt_server *s, uint32_t *completed, frt_error *err)
{
    if (completed) *completed = 0;
    if (!s) return FRT_ERR_INVALID_ARGUMENT;
    DeviceGuardLite g(s->device);
    // completions, as they happen: ticks on streams of their own may finish
    // out of launch order, and a finished tick frees its slot at once
    for (auto it = s->running.begin(); it != s->running.end();) {
        cudaError_t q = cudaEventQuery((*it)->done);
        if (q == cudaErrorNotReady) {
            ++it;
            continue;
        }
        if (q != cudaSuccess) return cuda_fail(err, q, "serving tick");
        auto t = *it;
        it = s->running.erase(it);
        finish_tick(s, t, completed);
    }
    // admit and launch
    while (!s->queue.empty() && s->running.size() < s->max_ticks) {
        std::vector<SrvReq *> batch;
        uint64_t bytes = 0;
        while (!s->queue.empty() && batch.size() < s->max_batch) {
            SrvReq *r = s->queue.front();
            Plan one;
            Tick tt;
            plan_request(s, *r, 0, one, tt);
            uint64_t b = plan_bytes(one);
            if (s->in_use + bytes + b > s->budget) {
                if (batch.empty() && s->running.empty()) {
                    // larger than the whole budget: it can never run
                    s->queue.pop_front();
                    r->status = FRT_ERR_INVALID_ARGUMENT;
                    set_error(&r->err, FRT_ERR_INVALID_ARGUMENT, 0, b, s->budget, 0, nullptr,
                              "the region needs %llu bytes of a %llu-byte budget", (unsigned long long)b,
                              (unsigned long long)s->budget);
                    r->state = 2;
                    r->done_ms = host_ms(s->t0);
                    s->pending--;
                    if (completed) (*completed)++;
                    continue;
                }
                break;
            }
            bytes += b;
            batch.push_back(r);
            s->queue.pop_front();
        }
        if (batch.empty()) break;
        int rc = launch_tick(s, batch, err);
        if (rc) return rc;
    }
    return FRT_OK;
}

extern "C" int frt_server_drain(frt_server *s, frt_error *err)
{
    if (!s) return FRT_ERR_INVALID_ARGUMENT;
    while (s->pending) {
        uint32_t c = 0;
        int rc = frt_server_progress(s, &c, err);
        if (rc) return rc;
        if (!s->running.empty()) cudaEventSynchronize(s->running.front()->done);
        else if (s->pending && s->queue.empty()) break;
    }
    return FRT_OK;
}

extern "C" int frt_server_request_info(const frt_server *s, uint64_t request, frt_region_info *info)
{
    if (!s || !info) return FRT_ERR_INVALID_ARGUMENT;
    auto it = s->reqs.find(request);
    if (it == s->reqs.end()) return FRT_ERR_INVALID_ARGUMENT;
    const SrvReq &r = *it->second;
    frt_region_info o{};
    o.state = r.state;
    o.status = r.status;
    o.records = r.n;
    o.arrival_ms = r.arrival_ms;
    o.done_ms = r.done_ms;
    o.inflated_bytes = r.inflated;
    o.chunks = (uint32_t)r.chunks.size();
    o.members = r.members;
    o.retries = r.retries;
    *info = o;
    return FRT_OK;
}

extern "C" int frt_server_request_error(const frt_server *s, uint64_t request, frt_error *err)
{
    if (!s || !err) return FRT_ERR_INVALID_ARGUMENT;
    auto it = s->reqs.find(request);
    if (it == s->reqs.end()) return FRT_ERR_INVALID_ARGUMENT;
    *err = it->second->err;
    return it->second->status;
}

static const size_t kRegionWidths[FRT_REGION_COL_COUNT] = {8, 8, 4, 4, 2, 1, 4};

extern "C" int frt_server_request_column(const frt_server *s, uint64_t request, int column, void **ptr, size_t *bytes,
                                         size_t *width)
{
    if (!s || column < 0 || column >= FRT_REGION_COL_COUNT) return FRT_ERR_INVALID_ARGUMENT;
    auto it = s->reqs.find(request);
    if (it == s->reqs.end() || it->second->state != 2) return FRT_ERR_INVALID_ARGUMENT;
    const SrvReq &r = *it->second;
    void *base = nullptr;
    if (r.tick) {
        const FrtRegionColumns &c = r.tick->cols;
        void *cols[FRT_REGION_COL_COUNT] = {c.virtual_offset, c.record_offset, c.ref_id, c.pos, c.flags, c.mapq, c.seq_len};
        base = (uint8_t *)cols[column] + kRegionWidths[column] * r.first;
    }
    if (ptr) *ptr = base;
    if (bytes) *bytes = kRegionWidths[column] * r.n;
    if (width) *width = kRegionWidths[column];
    return FRT_OK;
}

extern "C" int frt_server_request_column_to_host(const frt_server *s, uint64_t request, int column, void *dst,
                                                 size_t cap, frt_error *err)
{
    void *p = nullptr;
    size_t bytes = 0;
    if (frt_server_request_column(s, request, column, &p, &bytes, nullptr)) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "request %llu has no completed column %d",
                  (unsigned long long)request, column);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (cap < bytes) {
        set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "destination too small");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (!bytes) return FRT_OK;
    DeviceGuardLite g(s->device);
    cudaError_t e = cudaMemcpyAsync(dst, p, bytes, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "downloading a region column");
    return FRT_OK;
}

extern "C" const uint8_t *frt_server_request_inflated(const frt_server *s, uint64_t request, size_t *len)
{
    if (len) *len = 0;
    if (!s) return nullptr;
    auto it = s->reqs.find(request);
    if (it == s->reqs.end() || !it->second->tick) return nullptr;
    if (len) *len = it->second->out_len;
    return it->second->tick->arena + it->second->out_base;
}

extern "C" void frt_server_release(frt_server *s, uint64_t request)
{
    if (!s) return;
    auto it = s->reqs.find(request);
    if (it == s->reqs.end() || it->second->state == 1) return;
    if (it->second->state == 0) {
        for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
            if (*q == it->second.get()) {
                s->queue.erase(q);
                s->pending--;
                break;
            }
    }
    DeviceGuardLite g(s->device);
    s->reqs.erase(it); // the tick frees its memory with its last request
}
