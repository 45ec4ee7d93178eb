// BAI region resolution (host): the index a region query consults before any
// member is read.
//
//   parse   the BAI layout (SAM specification 5.2; crates/fritillaria-bam/src/bai.rs:13-21):
//           per reference the bins and their chunks, the metadata pseudo-bin
//           37450 kept apart, the 16 kb linear index, the unplaced count;
//   query   BinningIndex::query (crates/fritillaria-csi/src/binning_index/index.rs:93-119):
//           the bins reg2bins names for the 1-based inclusive interval
//           (reference_sequence.rs:376-398), their chunks, the linear index's
//           minimum offset at the interval start (linear_index.rs:11-15), then
//           optimize_chunks (binning_index.rs:33-62).

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "../../include/frt.h"

namespace frt {
void set_error(frt_error *err, int code, uint64_t offset, uint64_t expected, uint64_t actual, uint64_t position,
               const char *format, const char *fmt, ...);
}

namespace {
constexpr int MIN_SHIFT = 14, DEPTH = 5;
constexpr uint32_t META_BIN = 37450;
constexpr uint64_t MAX_POSITION = (1ull << (MIN_SHIFT + DEPTH * 3)) - 1;

struct BaiRef {
    std::unordered_map<uint32_t, std::vector<frt_chunk>> bins;
    std::vector<uint64_t> lidx;
    bool has_meta = false;
    frt_chunk meta_span{0, 0};
    uint64_t mapped = 0, unmapped = 0;
};
} // namespace

struct frt_bai {
    std::vector<BaiRef> refs;
    uint64_t n_no_coor = 0;
    bool has_no_coor = false;
};

namespace {

struct Cursor {
    const uint8_t *p, *end;
    bool ok = true;
    uint32_t u32()
    {
        if (end - p < 4) {
            ok = false;
            return 0;
        }
        uint32_t v = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
        p += 4;
        return v;
    }
    uint64_t u64()
    {
        uint64_t lo = u32();
        return lo | ((uint64_t)u32() << 32);
    }
};

void reg2bins(uint64_t start, uint64_t end, std::vector<uint32_t> &out)
{
    uint64_t beg = start - 1, last = end - 1;
    uint64_t t = 0;
    int s = MIN_SHIFT + DEPTH * 3;
    for (int l = 0; l <= DEPTH; ++l) {
        for (uint64_t i = t + (beg >> s); i <= t + (last >> s); ++i) out.push_back((uint32_t)i);
        s -= 3;
        t += 1ull << (l * 3);
    }
}

} // namespace

extern "C" int frt_bai_parse(const uint8_t *buf, size_t len, frt_bai **out, frt_error *err)
{
    auto bad = [&](const char *why) {
        frt::set_error(err, FRT_ERR_MALFORMED, 0, 0, 0, 0, "bai", "%s", why);
        return FRT_ERR_MALFORMED;
    };
    if (!buf || !out) return bad("null argument");
    if (len < 8 || memcmp(buf, "BAI\x01", 4) != 0) return bad("bad magic; expected BAI\\1");
    Cursor c{buf + 4, buf + len};
    int32_t n_ref = (int32_t)c.u32();
    if (n_ref < 0) return bad("negative reference count");
    frt_bai *b = new frt_bai;
    b->refs.resize((size_t)n_ref);
    for (auto &r : b->refs) {
        int32_t n_bin = (int32_t)c.u32();
        if (!c.ok || n_bin < 0) break;
        for (int32_t i = 0; i < n_bin && c.ok; ++i) {
            uint32_t id = c.u32();
            int32_t n_chunk = (int32_t)c.u32();
            if (!c.ok || n_chunk < 0 || (size_t)(c.end - c.p) / 16 < (size_t)n_chunk) {
                c.ok = false;
                break;
            }
            std::vector<frt_chunk> chunks((size_t)n_chunk);
            for (auto &ch : chunks) {
                ch.start = c.u64();
                ch.end = c.u64();
            }
            if (id == META_BIN && n_chunk == 2) {
                r.has_meta = true;
                r.meta_span = chunks[0];
                r.mapped = chunks[1].start;
                r.unmapped = chunks[1].end;
            } else {
                auto &v = r.bins[id];
                v.insert(v.end(), chunks.begin(), chunks.end());
            }
        }
        int32_t n_intv = (int32_t)c.u32();
        if (!c.ok || n_intv < 0 || (size_t)(c.end - c.p) / 8 < (size_t)n_intv) {
            c.ok = false;
            break;
        }
        r.lidx.resize((size_t)n_intv);
        for (auto &v : r.lidx) v = c.u64();
    }
    if (!c.ok) {
        delete b;
        return bad("truncated BAI");
    }
    if (c.end - c.p >= 8) {
        b->n_no_coor = c.u64();
        b->has_no_coor = true;
    }
    *out = b;
    return FRT_OK;
}

extern "C" void frt_bai_free(frt_bai *b) { delete b; }

extern "C" int32_t frt_bai_reference_count(const frt_bai *b) { return b ? (int32_t)b->refs.size() : 0; }

extern "C" int frt_bai_query(const frt_bai *b, int32_t ref, uint64_t start, uint64_t end, frt_chunk *out, size_t cap,
                             size_t *n, frt_error *err)
{
    if (!b || !n) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (ref < 0 || (size_t)ref >= b->refs.size()) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "invalid reference sequence ID: %d", ref);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (start == 0) start = 1;
    if (end == 0) end = MAX_POSITION;
    if (start > MAX_POSITION || end > MAX_POSITION || end < start) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "invalid interval [%llu, %llu]",
                       (unsigned long long)start, (unsigned long long)end);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    const BaiRef &r = b->refs[(size_t)ref];
    std::vector<uint32_t> bins;
    reg2bins(start, end, bins);
    std::vector<frt_chunk> chunks;
    for (uint32_t id : bins) {
        auto it = r.bins.find(id);
        if (it != r.bins.end()) chunks.insert(chunks.end(), it->second.begin(), it->second.end());
    }
    uint64_t w = (start - 1) >> MIN_SHIFT;
    uint64_t min_offset = w < r.lidx.size() ? r.lidx[w] : 0;
    // optimize_chunks
    chunks.erase(std::remove_if(chunks.begin(), chunks.end(), [&](const frt_chunk &c) { return c.end <= min_offset; }),
                 chunks.end());
    std::stable_sort(chunks.begin(), chunks.end(), [](const frt_chunk &a, const frt_chunk &b2) { return a.start < b2.start; });
    std::vector<frt_chunk> merged;
    for (const frt_chunk &c : chunks) {
        if (merged.empty() || c.start > merged.back().end) merged.push_back(c);
        else if (merged.back().end < c.end) merged.back().end = c.end;
    }
    *n = merged.size();
    if (merged.size() > cap) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, merged.size(), cap, 0, nullptr,
                       "%zu chunks, room for %zu", merged.size(), cap);
        return FRT_ERR_INVALID_ARGUMENT;
    }
    if (out) std::copy(merged.begin(), merged.end(), out);
    return FRT_OK;
}
