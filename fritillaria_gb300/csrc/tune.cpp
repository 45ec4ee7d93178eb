// The inflate autotuner: picks the member-inflate variant (table roots,
// window buffer, match queue), warps per CTA and queue chunk for a device and
// a workload class by timing candidates on an engine's bound input, and
// caches the winner in a JSON file.  No reference counterpart: the reference
// launches one fixed kernel shape (crates/fritillaria-cuda/src/backend.rs:178-219).

#include <cuda_runtime.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/frt.h"
#include "runtime.h"

namespace {

// ---- a minimal JSON value, parser and writer --------------------------------
struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj; // insertion order kept

    const Json *get(const std::string &k) const
    {
        for (const auto &kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
    Json *get_mut(const std::string &k)
    {
        for (auto &kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
    void set(const std::string &k, Json v)
    {
        if (Json *p = get_mut(k)) *p = std::move(v);
        else obj.emplace_back(k, std::move(v));
    }
    static Json number(double v)
    {
        Json j;
        j.kind = Number;
        j.num = v;
        return j;
    }
    static Json string(const std::string &v)
    {
        Json j;
        j.kind = String;
        j.str = v;
        return j;
    }
    static Json object()
    {
        Json j;
        j.kind = Object;
        return j;
    }
};

struct Parser {
    const char *p, *end;
    bool ok = true;

    void ws()
    {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool lit(const char *w)
    {
        size_t n = strlen(w);
        if ((size_t)(end - p) >= n && memcmp(p, w, n) == 0) {
            p += n;
            return true;
        }
        return false;
    }
    std::string parse_string()
    {
        std::string out;
        if (p >= end || *p != '"') {
            ok = false;
            return out;
        }
        ++p;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c != '\\') {
                out.push_back(c);
                continue;
            }
            if (p >= end) break;
            char e = *p++;
            switch (e) {
            case 'n': out.push_back('\n'); break;
            case 't': out.push_back('\t'); break;
            case 'r': out.push_back('\r'); break;
            case 'b': out.push_back('\b'); break;
            case 'f': out.push_back('\f'); break;
            case 'u': {
                if (end - p < 4) {
                    ok = false;
                    return out;
                }
                unsigned v = (unsigned)strtoul(std::string(p, 4).c_str(), nullptr, 16);
                p += 4;
                out.push_back(v < 0x80 ? (char)v : '?'); // keys and values here are ASCII
                break;
            }
            default: out.push_back(e);
            }
        }
        if (p >= end) {
            ok = false;
            return out;
        }
        ++p;
        return out;
    }
    Json parse_value(int depth)
    {
        Json j;
        ws();
        if (p >= end || depth > 32) {
            ok = false;
            return j;
        }
        if (*p == '{') {
            ++p;
            j.kind = Json::Object;
            ws();
            if (p < end && *p == '}') {
                ++p;
                return j;
            }
            while (ok) {
                ws();
                std::string k = parse_string();
                ws();
                if (p >= end || *p != ':') {
                    ok = false;
                    break;
                }
                ++p;
                Json v = parse_value(depth + 1);
                j.obj.emplace_back(std::move(k), std::move(v));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}') {
                    ++p;
                    break;
                }
                ok = false;
            }
            return j;
        }
        if (*p == '[') {
            ++p;
            j.kind = Json::Array;
            ws();
            if (p < end && *p == ']') {
                ++p;
                return j;
            }
            while (ok) {
                j.arr.push_back(parse_value(depth + 1));
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == ']') {
                    ++p;
                    break;
                }
                ok = false;
            }
            return j;
        }
        if (*p == '"') {
            j.kind = Json::String;
            j.str = parse_string();
            return j;
        }
        if (lit("true")) {
            j.kind = Json::Bool;
            j.b = true;
            return j;
        }
        if (lit("false")) {
            j.kind = Json::Bool;
            return j;
        }
        if (lit("null")) return j;
        char *q = nullptr;
        std::string tok;
        while (p < end && (isdigit((unsigned char)*p) || *p == '-' || *p == '+' || *p == '.' || *p == 'e' || *p == 'E'))
            tok.push_back(*p++);
        j.kind = Json::Number;
        j.num = strtod(tok.c_str(), &q);
        if (tok.empty() || !q || *q) ok = false;
        return j;
    }
};

void write_json(const Json &j, std::string &out, int indent)
{
    auto pad = [&](int n) { out.append((size_t)n * 2, ' '); };
    switch (j.kind) {
    case Json::Null: out += "null"; break;
    case Json::Bool: out += j.b ? "true" : "false"; break;
    case Json::Number: {
        char buf[64];
        if (std::isfinite(j.num) && j.num == std::floor(j.num) && std::fabs(j.num) < 1e15)
            snprintf(buf, sizeof buf, "%.0f", j.num);
        else snprintf(buf, sizeof buf, "%.6g", std::isfinite(j.num) ? j.num : 0.0);
        out += buf;
        break;
    }
    case Json::String:
        out.push_back('"');
        for (char c : j.str) {
            if (c == '"' || c == '\\') {
                out.push_back('\\');
                out.push_back(c);
            } else if ((unsigned char)c < 0x20) {
                char buf[8];
                snprintf(buf, sizeof buf, "\\u%04x", (unsigned)(unsigned char)c);
                out += buf;
            } else {
                out.push_back(c);
            }
        }
        out.push_back('"');
        break;
    case Json::Array:
        out += "[";
        for (size_t i = 0; i < j.arr.size(); ++i) {
            if (i) out += ", ";
            write_json(j.arr[i], out, indent + 1);
        }
        out += "]";
        break;
    case Json::Object:
        out += "{\n";
        for (size_t i = 0; i < j.obj.size(); ++i) {
            pad(indent + 1);
            write_json(Json::string(j.obj[i].first), out, 0);
            out += ": ";
            write_json(j.obj[i].second, out, indent + 1);
            out += i + 1 < j.obj.size() ? ",\n" : "\n";
        }
        pad(indent);
        out += "}";
        break;
    }
}

bool read_file(const std::string &path, std::string &out)
{
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

void make_parents(const std::string &path)
{
    for (size_t i = 1; i < path.size(); ++i)
        if (path[i] == '/') {
            std::string d = path.substr(0, i);
            mkdir(d.c_str(), 0755); // an existing directory is fine
        }
}

std::string default_cache_path()
{
    if (const char *e = getenv("FRT_TUNING_CACHE"); e && *e) return e;
    const char *home = getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/fritillaria_gb300/inflate_tuning.json";
}

// ---- workload class and cache key --------------------------------------------
uint32_t variant_set_hash()
{
    uint32_t h = 2166136261u;
    auto mix = [&](int64_t v) {
        for (int i = 0; i < 8; ++i) {
            h ^= (uint32_t)((v >> (8 * i)) & 0xff);
            h *= 16777619u;
        }
    };
    const int n = frt_inflate_variant_count();
    mix(n);
    for (int v = 0; v < n; ++v) {
        frt_inflate_variant info{};
        if (frt_inflate_variant_info(v, &info, nullptr) != FRT_OK) continue;
        mix(info.lit_bits);
        mix(info.dist_bits);
        mix(info.window);
        mix(info.queue);
        mix(info.max_registers);
        mix(info.chains);
        mix(info.stage_half);
        mix((int64_t)info.smem_per_warp);
    }
    return h;
}

std::string workload_key(int device, const frt_engine *e, const frt_engine_stats &st)
{
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, device);
    std::string fmt;
    const size_t nf = frt_engine_file_count(e);
    if (nf == 0) {
        fmt = "bam";
    } else {
        static const char *names[4] = {"bam", "bcf", "fastq", "fasta"};
        bool seen[4] = {};
        for (size_t i = 0; i < nf; ++i) {
            frt_engine_file_info fi{};
            if (frt_engine_get_file_info(e, i, &fi) == FRT_OK && fi.format >= 0 && fi.format < 4) seen[fi.format] = true;
        }
        for (int k = 0; k < 4; ++k)
            if (seen[k]) fmt += (fmt.empty() ? "" : "+") + std::string(names[k]);
    }
    const double members = (double)(st.members ? st.members : 1);
    const int mlog = (int)std::floor(std::log2(members));
    const int ckib = 4 * (int)std::lround(st.compressed_bytes / members / 1024.0 / 4.0);
    const double ratio = st.compressed_bytes ? std::round(4.0 * st.inflated_bytes / st.compressed_bytes) / 4.0 : 0.0;
    char buf[192];
    snprintf(buf, sizeof buf, "%s|sm%d|cc%d.%d|v%08x|%s|m%d|c%d|r%.2f", prop.name, prop.multiProcessorCount, prop.major,
             prop.minor, variant_set_hash(), fmt.c_str(), mlog, ckib, ratio);
    return buf;
}

Json tuning_json(const frt_inflate_tuning &t, double ms, double gbs, uint64_t members, int candidates)
{
    frt_inflate_variant info{};
    frt_inflate_variant_info(t.variant, &info, nullptr);
    Json j = Json::object();
    j.set("variant", Json::number(t.variant));
    j.set("lit_bits", Json::number(info.lit_bits));
    j.set("dist_bits", Json::number(info.dist_bits));
    j.set("window", Json::number(info.window));
    j.set("queue", Json::number(info.queue));
    j.set("max_registers", Json::number(info.max_registers));
    j.set("warps_per_cta", Json::number(t.warps_per_cta));
    j.set("ctas_per_sm", Json::number(t.ctas_per_sm));
    j.set("queue_chunk", Json::number(t.queue_chunk));
    j.set("spread_variant", Json::number(t.spread_variant));
    j.set("chains", Json::number(info.chains));
    j.set("stage_half", Json::number(info.stage_half));
    j.set("sample_members", Json::number((double)members));
    j.set("sample_ms", Json::number(ms));
    j.set("sample_gbs", Json::number(gbs));
    j.set("candidates", Json::number(candidates));
    char when[32];
    time_t now = time(nullptr);
    struct tm tmv;
    gmtime_r(&now, &tmv);
    strftime(when, sizeof when, "%Y-%m-%dT%H:%M:%SZ", &tmv);
    j.set("tuned_at", Json::string(when));
    return j;
}

bool tuning_from_json(const Json &j, frt_inflate_tuning *t)
{
    auto num = [&](const char *k, double *v) {
        const Json *x = j.get(k);
        if (!x || x->kind != Json::Number) return false;
        *v = x->num;
        return true;
    };
    double v, w, c, q, lb, db, win, qu, mr, ch = 1;
    if (!num("variant", &v) || !num("warps_per_cta", &w) || !num("ctas_per_sm", &c) || !num("queue_chunk", &q) ||
        !num("lit_bits", &lb) || !num("dist_bits", &db) || !num("window", &win) || !num("queue", &qu) ||
        !num("max_registers", &mr))
        return false;
    double sh = 0;
    num("chains", &ch); // entries written before multi-chain variants have one chain
    num("stage_half", &sh);
    frt_inflate_variant info{};
    if (frt_inflate_variant_info((int32_t)v, &info, nullptr) != FRT_OK) return false;
    // the variant index must still name the same shape
    if (info.lit_bits != (int)lb || info.dist_bits != (int)db || info.window != (int)win || info.queue != (int)qu ||
        info.max_registers != (int)mr || info.chains != (int)ch || info.stage_half != (int)sh)
        return false;
    // the small-launch variant: absent in entries written before it was
    // tuned (-1, and the caller times it), else a one-chain variant
    double sv = -1;
    num("spread_variant", &sv);
    if (sv >= 0) {
        frt_inflate_variant si{};
        if (frt_inflate_variant_info((int32_t)sv, &si, nullptr) != FRT_OK || si.chains != 1) return false;
    }
    *t = frt_inflate_tuning{(int32_t)v, (int32_t)w, (int32_t)c, (int32_t)q, (int32_t)sv};
    return true;
}

// The variant for small launches (spread one warp per CTA): every one-chain
// variant timed on a launch of one member per SM, the first members of the
// bound input, where each member's serial chain bounds the launch.
int pick_spread_variant(frt_engine *e, int device, uint64_t members, frt_inflate_tuning &t, frt_error *err)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const uint64_t few = members < (uint64_t)sms ? members : (uint64_t)sms;
    t.spread_variant = -1;
    if (few == 0) return FRT_OK;
    double best = 0;
    int best_v = -1;
    for (int v = 0; v < frt_inflate_variant_count(); ++v) {
        frt_inflate_variant vi{};
        if (frt_inflate_variant_info(v, &vi, nullptr) != FRT_OK || vi.chains != 1) continue;
        frt_inflate_tuning c = t;
        c.spread_variant = v;
        if (frt_inflate_tuning_ctas_per_sm(device, &c) < 1) continue;
        double ms = 0;
        uint64_t b = 0;
        int r = frt_engine_time_inflate(e, &c, few, 3, &ms, &b, err);
        if (r != FRT_OK) return r;
        if (ms > 0 && (best == 0 || ms < best)) {
            best = ms;
            best_v = v;
        }
    }
    t.spread_variant = best_v;
    return FRT_OK;
}

// Writes the cache back (a temporary file renamed over the old one).
int write_cache(Json &doc, const std::string &path, frt_error *err)
{
    doc.set("format", Json::string("fritillaria_gb300 inflate tuning"));
    doc.set("version", Json::number(1));
    std::string text;
    write_json(doc, text, 0);
    text.push_back('\n');
    make_parents(path);
    const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
    FILE *f = fopen(tmp.c_str(), "wb");
    bool wrote = f && fwrite(text.data(), 1, text.size(), f) == text.size();
    if (f) wrote = (fclose(f) == 0) && wrote;
    if (!wrote || rename(tmp.c_str(), path.c_str()) != 0) {
        unlink(tmp.c_str());
        frt::set_error(err, FRT_ERR_IO, 0, 0, 0, 0, nullptr, "writing the tuning cache %s: %s", path.c_str(),
                       strerror(errno));
        return FRT_ERR_IO;
    }
    return FRT_OK;
}

} // namespace

extern "C" int frt_autotune(frt_engine *e, const char *cache_path, int32_t force, frt_autotune_result *out,
                            frt_error *err)
{
    if (!e || !out) {
        frt::set_error(err, FRT_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, nullptr, "null argument");
        return FRT_ERR_INVALID_ARGUMENT;
    }
    *out = frt_autotune_result{};
    const int device = frt::engine_device(e);
    frt::DeviceGuardLite g(device);
    // One run with the current tuning: validates the bound input and gives the
    // workload class.
    int rc = frt_engine_run(e, err);
    frt_engine_stats st{};
    if (rc == FRT_OK) rc = frt_engine_finish(e, &st, err);
    if (rc != FRT_OK) return rc;
    const std::string key = workload_key(device, e, st);
    const size_t klen = key.size() < sizeof out->key - 1 ? key.size() : sizeof out->key - 1;
    memcpy(out->key, key.data(), klen);
    out->key[klen] = 0;
    const std::string path = cache_path && *cache_path ? cache_path : default_cache_path();

    Json doc = Json::object();
    {
        std::string text;
        if (read_file(path, text)) {
            Parser ps{text.data(), text.data() + text.size()};
            Json parsed = ps.parse_value(0);
            if (ps.ok && parsed.kind == Json::Object) doc = std::move(parsed);
        }
    }
    if (!doc.get("entries") || doc.get("entries")->kind != Json::Object) doc.set("entries", Json::object());
    Json *entries = doc.get_mut("entries");

    frt_inflate_tuning best{};
    if (!force) {
        const Json *hit = entries->get(key);
        if (hit && hit->kind == Json::Object && tuning_from_json(*hit, &best) &&
            frt_inflate_tuning_ctas_per_sm(device, &best) > 0) {
            if (best.spread_variant < 0) {
                // an entry from before the small-launch variant was tuned: time that alone
                if ((rc = pick_spread_variant(e, device, st.members, best, err)) != FRT_OK) return rc;
                Json *h = entries->get_mut(key);
                h->set("spread_variant", Json::number(best.spread_variant));
                if ((rc = write_cache(doc, path, err)) != FRT_OK) return rc;
                entries = doc.get_mut("entries"); // the write may have grown the document
                hit = entries->get(key);
            }
            if ((rc = frt_engine_set_tuning(e, &best, err)) != FRT_OK) return rc;
            if ((rc = frt_inflate_set_default_tuning(device, &best, err)) != FRT_OK) return rc;
            out->tuning = best;
            out->from_cache = 1;
            const Json *ms = hit->get("sample_ms"), *gbs = hit->get("sample_gbs"), *mem = hit->get("sample_members");
            out->ms = ms && ms->kind == Json::Number ? ms->num : 0;
            out->gbs = gbs && gbs->kind == Json::Number ? gbs->num : 0;
            out->members = mem && mem->kind == Json::Number ? (uint64_t)mem->num : 0;
            return FRT_OK;
        }
    }

    // Search: every variant at each CTA width (and the current tuning), then
    // the queue chunk for the best.
    const uint64_t sample = st.members < 32768 ? st.members : 32768;
    double best_ms = 0;
    uint64_t bytes = 0;
    int timed = 0;
    auto try_one = [&](const frt_inflate_tuning &t) -> int {
        if (frt_inflate_tuning_ctas_per_sm(device, &t) < 1) return FRT_OK;
        double ms = 0;
        uint64_t b = 0;
        int r = frt_engine_time_inflate(e, &t, sample, 3, &ms, &b, err);
        if (r != FRT_OK) return r;
        ++timed;
        if (ms > 0 && (best_ms == 0 || ms < best_ms)) {
            best_ms = ms;
            best = t;
            bytes = b;
        }
        return FRT_OK;
    };
    frt_inflate_tuning cur{};
    frt_engine_get_tuning(e, &cur);
    if ((rc = try_one(cur)) != FRT_OK) return rc;
    static const int widths[] = {2, 3, 4, 6, 8};
    for (int v = 0; v < frt_inflate_variant_count(); ++v)
        for (int w : widths) {
            frt_inflate_tuning t{v, w, 0, 1, -1};
            if (t.variant == cur.variant && t.warps_per_cta == cur.warps_per_cta && cur.ctas_per_sm == 0 &&
                cur.queue_chunk == 1)
                continue;
            if ((rc = try_one(t)) != FRT_OK) return rc;
        }
    const frt_inflate_tuning base = best;
    for (int chunk : {2, 4, 8}) {
        frt_inflate_tuning t = base;
        t.queue_chunk = chunk;
        if ((rc = try_one(t)) != FRT_OK) return rc;
    }
    if (best_ms <= 0) {
        frt::set_error(err, FRT_ERR_CUDA, 0, 0, 0, 0, nullptr, "no inflate tuning could be timed on device %d", device);
        return FRT_ERR_CUDA;
    }
    if ((rc = pick_spread_variant(e, device, st.members, best, err)) != FRT_OK) return rc;
    if ((rc = frt_engine_set_tuning(e, &best, err)) != FRT_OK) return rc;
    if ((rc = frt_inflate_set_default_tuning(device, &best, err)) != FRT_OK) return rc;
    out->tuning = best;
    out->ms = best_ms;
    out->gbs = bytes / (best_ms * 1e6);
    out->members = sample;
    out->candidates = timed;

    entries = doc.get_mut("entries");
    entries->set(key, tuning_json(best, best_ms, out->gbs, sample, timed));
    return write_cache(doc, path, err);
}
