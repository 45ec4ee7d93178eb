// Seeded synthetic BAM generators and a BGZF writer.
//
// Produces the workloads the benchmark and the tests run on:
//   * short paired-end reads (100k records on one 50 Mb contig, or 20M records
//     over 24 contigs proportional to the human chromosomes), CIGAR 150M for
//     90% of reads else one insertion, one deletion or a leading soft clip,
//     uniform ACGT with 0.1% N, Phred ~ N(35, 5) clipped to 2..41, NM/MD/RG;
//   * ultra-long unaligned reads (flag 4, refID -1) with log-normal lengths and
//     MM:Z / ML:B:C / qs:f / ch:i tags.
// The BAM byte layout follows the SAM specification as read by the reference
// (crates/fritillaria-bam/src/columnar/record.rs:1-22, header.rs:1-12).
//
// BGZF packing follows one of two writers:
//   * "full" packs a 65,495-byte staging buffer and flushes only when it is
//     full, so records straddle members (the noodles writer's
//     MAX_BUF_SIZE = 65536 - 18 - 8 - 15, crates/fritillaria-bgzf/src/io/writer.rs:24);
//   * "record" starts a new member before a record that would not fit in
//     65,280 bytes (htslib's bgzf_flush_try), so members start on records
//     unless a record is larger than a member.
// Compression is zlib raw deflate at a per-member level (even/odd members may
// alternate levels).  Everything is deterministic in the seed and independent
// of the thread count.

#include <zlib.h>

#include <algorithm>
#include <functional>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

// xoshiro256** seeded through splitmix64 (Blackman & Vigna, public domain
// algorithms restated here).
struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x)
    {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed, uint64_t stream = 0)
    {
        uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull);
        for (auto &v : s) v = splitmix(x);
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next()
    {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return (uint32_t)(((next() >> 32) * (uint64_t)n) >> 32); }
    double normal()
    {
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

void put32(std::vector<uint8_t> &b, uint32_t v)
{
    uint8_t x[4] = {(uint8_t)v, (uint8_t)(v >> 8), (uint8_t)(v >> 16), (uint8_t)(v >> 24)};
    b.insert(b.end(), x, x + 4);
}
void put16(std::vector<uint8_t> &b, uint16_t v)
{
    b.push_back((uint8_t)v);
    b.push_back((uint8_t)(v >> 8));
}
void patch32(std::vector<uint8_t> &b, size_t at, uint32_t v)
{
    b[at] = (uint8_t)v;
    b[at + 1] = (uint8_t)(v >> 8);
    b[at + 2] = (uint8_t)(v >> 16);
    b[at + 3] = (uint8_t)(v >> 24);
}

// SAM specification, section 5.3: the smallest bin containing [beg, end).
int reg2bin(int64_t beg, int64_t end)
{
    --end;
    if (beg >> 14 == end >> 14) return (int)(((1 << 15) - 1) / 7 + (beg >> 14));
    if (beg >> 17 == end >> 17) return (int)(((1 << 12) - 1) / 7 + (beg >> 17));
    if (beg >> 20 == end >> 20) return (int)(((1 << 9) - 1) / 7 + (beg >> 20));
    if (beg >> 23 == end >> 23) return (int)(((1 << 6) - 1) / 7 + (beg >> 23));
    if (beg >> 26 == end >> 26) return (int)(((1 << 3) - 1) / 7 + (beg >> 26));
    return 0;
}

// Human chromosome lengths (GRCh38, chr1..22, X, Y), used as relative weights.
const double kHumanLengths[24] = {
    248956422, 242193529, 198295559, 190214555, 181538259, 170805979, 159345973, 145138636,
    138394717, 133797422, 135086622, 133275309, 114364328, 107043718, 101991189, 90338345,
    83257441,  80373285,  58617616,  64444167,  46709983,  50818468,  156040895, 57227415};

struct Contig {
    std::string name;
    uint32_t length;
};

std::vector<Contig> make_contigs(int n_contigs, uint64_t genome_len)
{
    std::vector<Contig> c;
    if (n_contigs <= 1) {
        c.push_back({"chr1", (uint32_t)genome_len});
        return c;
    }
    double sum = 0;
    for (int i = 0; i < 24; ++i) sum += kHumanLengths[i];
    for (int i = 0; i < n_contigs && i < 24; ++i) {
        std::string nm = i < 22 ? "chr" + std::to_string(i + 1) : (i == 22 ? "chrX" : "chrY");
        c.push_back({nm, (uint32_t)(genome_len * (kHumanLengths[i] / sum))});
    }
    return c;
}

std::vector<uint8_t> bam_header(const std::vector<Contig> &contigs, bool sorted)
{
    std::string text = sorted ? "@HD\tVN:1.6\tSO:coordinate\n" : "@HD\tVN:1.6\tSO:unsorted\n";
    for (auto &c : contigs) text += "@SQ\tSN:" + c.name + "\tLN:" + std::to_string(c.length) + "\n";
    text += "@RG\tID:rg1\tSM:sample1\n";
    std::vector<uint8_t> b = {'B', 'A', 'M', 1};
    put32(b, (uint32_t)text.size());
    b.insert(b.end(), text.begin(), text.end());
    put32(b, (uint32_t)contigs.size());
    for (auto &c : contigs) {
        put32(b, (uint32_t)c.name.size() + 1);
        b.insert(b.end(), c.name.begin(), c.name.end());
        b.push_back(0);
        put32(b, c.length);
    }
    return b;
}

const uint8_t kNibble[4] = {1, 2, 4, 8}; // A C G T in =ACMGRSVTWYHKDBN
const char kBase[4] = {'A', 'C', 'G', 'T'};

// One short paired-end record (150 bp) at global index `i`.
void short_record(std::vector<uint8_t> &out, uint64_t i, uint64_t n_records,
                  const std::vector<Contig> &contigs, const std::vector<uint64_t> &cum, uint64_t seed)
{
    Rng r(seed, i + 1);
    const int L = 150;
    // Stratified uniform positions: sorted by construction.
    uint64_t genome = cum.back();
    uint64_t g = (uint64_t)(((double)i + r.uniform()) * (double)genome / (double)n_records);
    if (g >= genome) g = genome - 1;
    size_t ci = std::upper_bound(cum.begin(), cum.end(), g) - cum.begin() - 1;
    int64_t pos = (int64_t)(g - cum[ci]);
    int64_t clen = contigs[ci].length;
    if (pos > clen - L) pos = std::max<int64_t>(0, clen - L);

    static const uint16_t kFlags[4] = {99, 147, 83, 163};
    uint16_t flag = kFlags[r.below(4)];
    uint8_t mapq = (uint8_t)r.below(61);

    // CIGAR
    uint32_t cig[3];
    int ncig = 0;
    int kind = 0, k = 0, a = 0;
    int64_t ref_len = L;
    if (r.uniform() >= 0.9) {
        kind = 1 + (int)r.below(3);
        if (kind == 1) { // aM kI bM
            k = 1 + (int)r.below(5);
            a = 10 + (int)r.below(L - 20 - k);
            cig[ncig++] = ((uint32_t)a << 4) | 0;
            cig[ncig++] = ((uint32_t)k << 4) | 1;
            cig[ncig++] = ((uint32_t)(L - a - k) << 4) | 0;
            ref_len = L - k;
        } else if (kind == 2) { // aM kD bM
            k = 1 + (int)r.below(5);
            a = 10 + (int)r.below(L - 20);
            cig[ncig++] = ((uint32_t)a << 4) | 0;
            cig[ncig++] = ((uint32_t)k << 4) | 2;
            cig[ncig++] = ((uint32_t)(L - a) << 4) | 0;
            ref_len = L + k;
        } else { // sS bM
            k = 1 + (int)r.below(30);
            cig[ncig++] = ((uint32_t)k << 4) | 4;
            cig[ncig++] = ((uint32_t)(L - k) << 4) | 0;
            ref_len = L - k;
        }
    } else {
        cig[ncig++] = ((uint32_t)L << 4) | 0;
    }
    int bin = reg2bin(pos, pos + ref_len);
    int insert = (int)std::lround(300 + 50 * r.normal());
    if (insert < L) insert = L;
    bool reverse = (flag & 16) != 0;
    int64_t mpos = reverse ? std::max<int64_t>(0, pos - insert + L) : pos + insert - L;
    int32_t tlen = reverse ? -insert : insert;

    char name[24];
    snprintf(name, sizeof name, "r%09llu", (unsigned long long)(i / 2));
    size_t name_len = strlen(name) + 1;

    // MD/NM over the aligned reference bases
    int aligned = (int)(ref_len - (kind == 2 ? k : 0)); // M bases
    int mism = 0;
    double u = r.uniform();
    mism = u < 0.6 ? 0 : (u < 0.85 ? 1 : (u < 0.95 ? 2 : 3));
    std::vector<int> mpos_list;
    for (int m = 0; m < mism; ++m) mpos_list.push_back((int)r.below((uint32_t)aligned));
    std::sort(mpos_list.begin(), mpos_list.end());
    mpos_list.erase(std::unique(mpos_list.begin(), mpos_list.end()), mpos_list.end());
    std::string md;
    {
        int run = 0, m_idx = 0;
        int del_at = (kind == 2) ? a : -1;
        for (int p = 0; p < aligned; ++p) {
            if (p == del_at) {
                md += std::to_string(run);
                md += '^';
                for (int d = 0; d < k; ++d) md += kBase[r.below(4)];
                run = 0;
            }
            if (m_idx < (int)mpos_list.size() && mpos_list[m_idx] == p) {
                md += std::to_string(run);
                md += kBase[r.below(4)];
                run = 0;
                ++m_idx;
            } else {
                ++run;
            }
        }
        md += std::to_string(run);
    }
    int nm = (int)mpos_list.size() + ((kind == 1 || kind == 2) ? k : 0);

    size_t start = out.size();
    put32(out, 0); // block_size placeholder
    put32(out, (uint32_t)ci);
    put32(out, (uint32_t)pos);
    out.push_back((uint8_t)name_len);
    out.push_back(mapq);
    put16(out, (uint16_t)bin);
    put16(out, (uint16_t)ncig);
    put16(out, flag);
    put32(out, (uint32_t)L);
    put32(out, (uint32_t)ci);
    put32(out, (uint32_t)mpos);
    put32(out, (uint32_t)tlen);
    out.insert(out.end(), name, name + name_len - 1);
    out.push_back(0);
    for (int c = 0; c < ncig; ++c) put32(out, cig[c]);
    uint8_t packed[75];
    for (int b = 0; b < L; b += 2) {
        uint8_t hi = r.uniform() < 0.001 ? 15 : kNibble[r.below(4)];
        uint8_t lo = r.uniform() < 0.001 ? 15 : kNibble[r.below(4)];
        packed[b / 2] = (uint8_t)((hi << 4) | lo);
    }
    out.insert(out.end(), packed, packed + 75);
    for (int b = 0; b < L; ++b) {
        long q = std::lround(35.0 + 5.0 * r.normal());
        q = std::min(41L, std::max(2L, q));
        out.push_back((uint8_t)q);
    }
    // NM:C (htslib writes the narrowest integer type), MD:Z, RG:Z
    out.push_back('N'); out.push_back('M'); out.push_back('C'); out.push_back((uint8_t)nm);
    out.push_back('M'); out.push_back('D'); out.push_back('Z');
    out.insert(out.end(), md.begin(), md.end());
    out.push_back(0);
    const char rg[] = "RGZrg1";
    out.insert(out.end(), rg, rg + 6);
    out.push_back(0);
    patch32(out, start, (uint32_t)(out.size() - start - 4));
}

// One ultra-long unaligned read with base-modification tags.
void long_record(std::vector<uint8_t> &out, uint64_t i, uint32_t l_seq, uint64_t seed)
{
    Rng r(seed ^ 0x5555, i + 1);
    char name[40];
    snprintf(name, sizeof name, "%08x-%04x-%04x-%04x-%012llx", (unsigned)r.next(), (unsigned)(r.next() & 0xffff),
             (unsigned)(r.next() & 0xffff), (unsigned)(r.next() & 0xffff), (unsigned long long)(r.next() & 0xffffffffffffull));
    size_t name_len = strlen(name) + 1;
    size_t start = out.size();
    put32(out, 0);
    put32(out, 0xffffffffu); // refID -1
    put32(out, 0xffffffffu); // pos -1
    out.push_back((uint8_t)name_len);
    out.push_back(0);        // mapq
    put16(out, 4680);        // bin of an unplaced read
    put16(out, 0);           // n_cigar
    put16(out, 4);           // flag: unmapped
    put32(out, l_seq);
    put32(out, 0xffffffffu);
    put32(out, 0xffffffffu);
    put32(out, 0);
    out.insert(out.end(), name, name + name_len - 1);
    out.push_back(0);
    // sequence
    std::vector<uint8_t> bases(l_seq);
    for (uint32_t b = 0; b < l_seq; ++b) bases[b] = (uint8_t)r.below(4);
    size_t p0 = out.size();
    out.resize(p0 + (l_seq + 1) / 2);
    for (uint32_t b = 0; b < l_seq; b += 2) {
        uint8_t hi = kNibble[bases[b]];
        uint8_t lo = (b + 1 < l_seq) ? kNibble[bases[b + 1]] : 0;
        out[p0 + b / 2] = (uint8_t)((hi << 4) | lo);
    }
    // qualities: 5 + geometric(mean ~10), clipped to 5..40
    double qsum = 0;
    size_t q0 = out.size();
    out.resize(q0 + l_seq);
    const double lg = std::log(1.0 - 1.0 / 11.0);
    for (uint32_t b = 0; b < l_seq; ++b) {
        double u = r.uniform();
        if (u < 1e-300) u = 1e-300;
        int q = 5 + (int)std::floor(std::log(u) / lg);
        q = std::min(40, std::max(5, q));
        out[q0 + b] = (uint8_t)q;
        qsum += q;
    }
    // MM:Z C+m? with skip counts over C sites, ML:B:C one byte per listed site
    std::string mm = "C+m?";
    std::vector<uint8_t> ml;
    uint32_t skip = 0;
    for (uint32_t b = 0; b < l_seq; ++b) {
        if (bases[b] != 1) continue;
        if (r.uniform() < 0.2) {
            mm += ',';
            mm += std::to_string(skip);
            ml.push_back((uint8_t)r.below(256));
            skip = 0;
        } else {
            ++skip;
        }
    }
    mm += ';';
    out.push_back('M'); out.push_back('M'); out.push_back('Z');
    out.insert(out.end(), mm.begin(), mm.end());
    out.push_back(0);
    out.push_back('M'); out.push_back('L'); out.push_back('B'); out.push_back('C');
    put32(out, (uint32_t)ml.size());
    out.insert(out.end(), ml.begin(), ml.end());
    float qs = l_seq ? (float)(qsum / l_seq) : 0.0f;
    uint32_t qbits;
    memcpy(&qbits, &qs, 4);
    out.push_back('q'); out.push_back('s'); out.push_back('f');
    put32(out, qbits);
    uint32_t ch = 1 + r.below(512);
    out.push_back('c'); out.push_back('h');
    if (ch <= 255) { out.push_back('C'); out.push_back((uint8_t)ch); }
    else { out.push_back('S'); put16(out, (uint16_t)ch); }
    patch32(out, start, (uint32_t)(out.size() - start - 4));
}


// ---- FASTQ ---------------------------------------------------------------
// Illumina-like (kind 0): 40-60 character names, 150 bases (0.1% N), Phred+33
// qualities ~ N(35, 5) clipped to 2..41, so '@' (Q31) starts about one quality
// line in twenty -- the decoys a record-start scan must reject.  Ultra-long
// (kind 1): log-normal lengths (median 15 kb), qualities ~ N(15, 5) in 1..50.
void fastq_record(std::vector<uint8_t> &out, uint64_t i, int kind, uint64_t seed)
{
    Rng r(seed, 0x20000000ull + i);
    char name[160];
    int nl;
    uint32_t len;
    if (kind == 0) {
        nl = snprintf(name, sizeof name, "@A%05u:%u:H%07uDSXX:%u:%u:%u:%u %u:N:0:%s", 100 + r.below(900),
                      1 + r.below(99), r.below(9999999), 1 + r.below(4), 1101 + r.below(2600),
                      1000 + r.below(30000), 1000 + r.below(30000), 1 + (uint32_t)(i & 1),
                      (i % 3) ? "ACGTACGT+TTGACCAA" : "GGCCTTAA");
        len = 150;
    } else {
        nl = snprintf(name, sizeof name, "@%08x-%04x-%04x-%04x-%012llx runid=%08x read=%llu ch=%u", (uint32_t)r.next(),
                      r.below(65536), r.below(65536), r.below(65536), (unsigned long long)(r.next() >> 16),
                      (uint32_t)r.next(), (unsigned long long)i, 1 + r.below(512));
        double l = std::exp(std::log(15000.0) + 0.8 * r.normal());
        len = (uint32_t)std::min(400000.0, std::max(1.0, std::floor(l)));
    }
    out.insert(out.end(), name, name + nl);
    out.push_back('\n');
    static const char bases[4] = {'A', 'C', 'G', 'T'};
    for (uint32_t k = 0; k < len; ++k) out.push_back(r.below(1000) == 0 ? 'N' : bases[r.next() >> 62]);
    out.push_back('\n');
    out.push_back('+');
    out.push_back('\n');
    for (uint32_t k = 0; k < len; ++k) {
        double q = kind == 0 ? 35.0 + 5.0 * r.normal() : 15.0 + 5.0 * r.normal();
        int qi = (int)std::lround(q);
        qi = kind == 0 ? std::min(41, std::max(2, qi)) : std::min(50, std::max(1, qi));
        out.push_back((uint8_t)(33 + qi));
    }
    out.push_back('\n');
}

// ---- BCF -----------------------------------------------------------------
// Sites over human-proportioned contigs; REF/ALT 90% SNV, else an indel of
// 1-20 bases; QUAL float (1% missing); INFO DP (int8/int16/int32 by value)
// and AF (float), plus every tenth site an ANN string of 16-80 characters so
// the typed-value length escape fires; FORMAT GT (int8 x 2, phased diploid,
// alt allele frequency ~ Beta(0.5, 2)) and DP (int16 ~ N(30, 5.5)) per sample.
const uint8_t T_INT8 = 1, T_INT16 = 2, T_INT32 = 3, T_FLOAT = 5, T_CHAR = 7;

void typed_len(std::vector<uint8_t> &b, uint32_t n, uint8_t type)
{
    if (n < 15) {
        b.push_back((uint8_t)(n << 4 | type));
        return;
    }
    b.push_back((uint8_t)(15 << 4 | type));
    if (n < 128) {
        b.push_back(0x10 | T_INT8);
        b.push_back((uint8_t)n);
    } else if (n < 32768) {
        b.push_back(0x10 | T_INT16);
        put16(b, (uint16_t)n);
    } else {
        b.push_back(0x10 | T_INT32);
        put32(b, n);
    }
}

void typed_string(std::vector<uint8_t> &b, const std::string &s)
{
    typed_len(b, (uint32_t)s.size(), T_CHAR);
    b.insert(b.end(), s.begin(), s.end());
}

void typed_int(std::vector<uint8_t> &b, int32_t v)
{
    if (v > -120 && v < 128) {
        b.push_back(0x10 | T_INT8);
        b.push_back((uint8_t)(int8_t)v);
    } else if (v > -32760 && v < 32768) {
        b.push_back(0x10 | T_INT16);
        put16(b, (uint16_t)(int16_t)v);
    } else {
        b.push_back(0x10 | T_INT32);
        put32(b, (uint32_t)v);
    }
}

std::vector<uint8_t> bcf_header(const std::vector<Contig> &contigs, uint32_t n_samples)
{
    std::string t = "##fileformat=VCFv4.2\n##FILTER=<ID=PASS,Description=\"All filters passed\">\n";
    for (auto &c : contigs) t += "##contig=<ID=" + c.name + ",length=" + std::to_string(c.length) + ">\n";
    t += "##INFO=<ID=DP,Number=1,Type=Integer,Description=\"Total depth\">\n"
         "##INFO=<ID=AF,Number=A,Type=Float,Description=\"Allele frequency\">\n"
         "##INFO=<ID=ANN,Number=.,Type=String,Description=\"Annotation\">\n"
         "##FORMAT=<ID=GT,Number=1,Type=String,Description=\"Genotype\">\n"
         "##FORMAT=<ID=DP,Number=1,Type=Integer,Description=\"Read depth\">\n"
         "#CHROM\tPOS\tID\tREF\tALT\tQUAL\tFILTER\tINFO";
    if (n_samples) t += "\tFORMAT";
    for (uint32_t s = 0; s < n_samples; ++s) t += "\tS" + std::to_string(s);
    t += "\n";
    std::vector<uint8_t> h = {'B', 'C', 'F', 2, 2};
    put32(h, (uint32_t)t.size() + 1);
    h.insert(h.end(), t.begin(), t.end());
    h.push_back(0);
    return h;
}

// Dictionary numbering of the header above: PASS 0, DP 1, AF 2, ANN 3, GT 4.
void bcf_record(std::vector<uint8_t> &out, uint64_t i, int32_t chrom, int32_t pos, uint32_t n_samples,
                uint64_t seed)
{
    Rng r(seed, 0x30000000ull + i);
    static const char bases[4] = {'A', 'C', 'G', 'T'};
    std::string ref(1, bases[r.next() >> 62]), alt(1, bases[r.next() >> 62]);
    if (alt == ref) alt = ref == "A" ? "G" : "A";
    if (r.below(10) == 0) {
        uint32_t l = 1 + r.below(20);
        std::string ins;
        for (uint32_t k = 0; k < l; ++k) ins.push_back(bases[r.next() >> 62]);
        if (r.below(2)) alt = ref + ins;
        else ref = ref + ins;
    }
    size_t base = out.size();
    put32(out, 0); // l_shared
    put32(out, 0); // l_indiv
    put32(out, (uint32_t)chrom);
    put32(out, (uint32_t)pos);
    put32(out, (uint32_t)ref.size());
    float q = (float)(10.0 + 990.0 * r.uniform());
    uint32_t qb;
    memcpy(&qb, &q, 4);
    if (r.below(100) == 0) qb = 0x7F800001u;
    put32(out, qb);
    bool ann = i % 10 == 0;
    put16(out, ann ? 3 : 2);
    put16(out, 2);
    put32(out, n_samples | ((n_samples ? 2u : 0u) << 24));
    if (r.below(10) < 3) typed_string(out, "rs" + std::to_string(1000 + r.below(90000000)));
    else out.push_back(T_CHAR); // '.'
    typed_string(out, ref);
    typed_string(out, alt);
    out.push_back(0x10 | T_INT8); // FILTER: PASS
    out.push_back(0);
    double af = std::pow(r.uniform(), 2.0); // Beta(0.5, 1)-like skew toward rare alleles
    uint32_t dp = 20 * n_samples + r.below(1 + 10 * n_samples);
    typed_int(out, 1);
    typed_int(out, (int32_t)std::min<uint32_t>(dp, 2000000000u));
    typed_int(out, 2);
    out.push_back(0x10 | T_FLOAT);
    float aff = (float)af;
    uint32_t afb;
    memcpy(&afb, &aff, 4);
    put32(out, afb);
    if (ann) {
        typed_int(out, 3);
        std::string a = "T|missense_variant|MODERATE|GENE" + std::to_string(r.below(20000));
        uint32_t extra = r.below(48);
        for (uint32_t k = 0; k < extra; ++k) a.push_back((char)('a' + r.below(26)));
        typed_string(out, a);
    }
    uint32_t l_shared = (uint32_t)(out.size() - base - 8);
    size_t indiv = out.size();
    if (n_samples) {
        typed_int(out, 4); // GT
        out.push_back(0x20 | T_INT8);
        for (uint32_t s = 0; s < n_samples; ++s) {
            for (int h = 0; h < 2; ++h) {
                uint32_t allele = r.uniform() < af ? 1 : 0;
                out.push_back((uint8_t)(((allele + 1) << 1) | (h ? 1 : 0)));
            }
        }
        typed_int(out, 1); // DP
        out.push_back(0x10 | T_INT16);
        for (uint32_t s = 0; s < n_samples; ++s) {
            int d = (int)std::lround(30.0 + 5.5 * r.normal());
            put16(out, (uint16_t)std::max(0, d));
        }
    }
    patch32(out, base, l_shared);
    patch32(out, base + 4, (uint32_t)(out.size() - indiv));
}

// ---- FASTA ---------------------------------------------------------------
// Contigs with lengths proportional to the human chromosomes, `line_width`
// bases per line, soft-masked (lowercase) runs covering about half the bases,
// runs of N of 1 kb - 1 Mb covering about 5%, an NCBI-style definition line
// and, when asked, a blank line between records.  Bases are drawn in
// fixed-size chunks, each from its own stream, so generation is parallel.
void fasta_chunk(uint8_t *dst, uint64_t contig, uint64_t chunk_index, uint64_t n, uint64_t seed)
{
    Rng r(seed, 0x40000000ull + (contig << 24) + chunk_index);
    static const char upper[4] = {'A', 'C', 'G', 'T'}, lower[4] = {'a', 'c', 'g', 't'};
    uint64_t k = 0;
    bool masked = r.below(2);
    while (k < n) {
        uint64_t run;
        if (r.below(1000) == 0) { // an N run
            run = 1000 + (uint64_t)(std::exp(r.uniform() * std::log(1000.0)) * 1000.0) - 1000;
            run = std::min(run, n - k);
            memset(dst + k, 'N', run);
            k += run;
            continue;
        }
        run = 50 + r.below(4000);
        run = std::min(run, n - k);
        const char *tab = masked ? lower : upper;
        for (uint64_t j = 0; j < run; ++j) dst[k + j] = (uint8_t)tab[r.next() >> 62];
        k += run;
        masked = !masked;
    }
}

void run_parallel(int threads, size_t n, const std::function<void(size_t)> &fn)
{
    if (threads < 1) threads = 1;
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            for (;;) {
                size_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i);
            }
        });
    for (auto &th : pool) th.join();
}
} // namespace

extern "C" {

typedef struct {
    int32_t kind;           // 0 short paired reads, 1 ultra-long unaligned
    int32_t n_contigs;      // short reads: 1 or 24
    uint64_t n_records;
    uint64_t genome_len;
    uint64_t seed;
    int32_t threads;
    int32_t n_long_extra;   // ultra-long: extra reads of 250-800 kb
} frt_synth_bam_params;

// Generates an uncompressed BAM stream (header + records).  `record_ends`
// receives, when non-null, a malloc'd array of the end offset of the header
// and of every record (n_records + 1 entries) for record-aligned packing.
int frt_synth_bam(const frt_synth_bam_params *p, uint8_t **raw, size_t *raw_len, uint64_t **record_ends,
                  size_t *n_ends)
{
    std::vector<Contig> contigs;
    if (p->kind == 0) contigs = make_contigs(p->n_contigs, p->genome_len);
    else contigs = make_contigs(1, 248956422);
    std::vector<uint8_t> hdr = bam_header(contigs, p->kind == 0);
    std::vector<uint64_t> cum(1, 0);
    for (auto &c : contigs) cum.push_back(cum.back() + c.length);

    // ultra-long lengths are drawn up front so chunks are independent
    std::vector<uint32_t> lens;
    uint64_t n = p->n_records;
    if (p->kind == 1) {
        Rng r(p->seed, 0x10000);
        uint64_t total = n + (uint64_t)std::max(0, p->n_long_extra);
        lens.resize(total);
        for (uint64_t i = 0; i < n; ++i) {
            double l = std::exp(std::log(15000.0) + 1.0 * r.normal());
            lens[i] = (uint32_t)std::min(1000000.0, std::max(1.0, std::floor(l)));
        }
        for (uint64_t i = n; i < total; ++i) lens[i] = 250000 + r.below(550001);
        // scatter the extra long reads
        for (uint64_t i = total - 1; i > 0; --i) std::swap(lens[i], lens[r.below((uint32_t)std::min<uint64_t>(i + 1, 0xffffffffull))]);
        n = total;
    }
    const uint64_t chunk = p->kind == 0 ? 65536 : 256;
    size_t n_chunks = (size_t)((n + chunk - 1) / chunk);
    std::vector<std::vector<uint8_t>> parts(n_chunks);
    std::vector<std::vector<uint64_t>> ends(n_chunks);
    run_parallel(p->threads, n_chunks, [&](size_t c) {
        uint64_t b = c * chunk, e = std::min(n, b + chunk);
        auto &out = parts[c];
        for (uint64_t i = b; i < e; ++i) {
            if (p->kind == 0) short_record(out, i, n, contigs, cum, p->seed);
            else long_record(out, i, lens[i], p->seed);
            if (record_ends) ends[c].push_back(out.size());
        }
    });
    std::vector<size_t> base(n_chunks + 1, hdr.size());
    for (size_t c = 0; c < n_chunks; ++c) base[c + 1] = base[c] + parts[c].size();
    size_t total = base[n_chunks];
    uint8_t *buf = (uint8_t *)malloc(total ? total : 1);
    if (!buf) return -1;
    memcpy(buf, hdr.data(), hdr.size());
    run_parallel(p->threads, n_chunks, [&](size_t c) {
        memcpy(buf + base[c], parts[c].data(), parts[c].size());
        std::vector<uint8_t>().swap(parts[c]);
    });
    if (record_ends) {
        uint64_t *re = (uint64_t *)malloc(sizeof(uint64_t) * (n + 1));
        re[0] = hdr.size();
        size_t k = 1;
        for (size_t c = 0; c < n_chunks; ++c)
            for (uint64_t v : ends[c]) re[k++] = base[c] + v;
        *record_ends = re;
        *n_ends = k;
    }
    *raw = buf;
    *raw_len = total;
    return 0;
}

// Splits `raw` into BGZF members.  mode 0: fixed payloads of `member_payload`
// bytes (records straddle members).  mode 1: record-aligned, using
// `record_ends` (ascending end offsets; the first is the header's end).
// Members at even index are compressed at level_even, odd at level_odd.
int frt_synth_bgzf(const uint8_t *raw, size_t raw_len, int mode, uint32_t member_payload,
                   const uint64_t *record_ends, size_t n_ends, int level_even, int level_odd,
                   int threads, uint8_t **out, size_t *out_len, uint64_t *n_members_out)
{
    std::vector<uint64_t> cuts; // member start offsets into raw, plus raw_len
    cuts.push_back(0);
    if (member_payload == 0 || member_payload > 65280) member_payload = 65280;
    if (mode == 0) {
        for (uint64_t o = member_payload; o < raw_len; o += member_payload) cuts.push_back(o);
    } else {
        // htslib: flush before a record that does not fit; split larger ones
        uint64_t block_start = 0;
        for (size_t k = 0; k < n_ends; ++k) {
            uint64_t rec_beg = k == 0 ? 0 : record_ends[k - 1];
            uint64_t rec_end = record_ends[k];
            if (k == 0) { // header: its own member(s)
                for (uint64_t o = member_payload; o < rec_end; o += member_payload) cuts.push_back(o);
                if (rec_end < raw_len) cuts.push_back(rec_end);
                block_start = rec_end;
                continue;
            }
            if (rec_end - block_start > member_payload && rec_beg > block_start) {
                cuts.push_back(rec_beg);
                block_start = rec_beg;
            }
            while (rec_end - block_start > member_payload) {
                block_start += member_payload;
                cuts.push_back(block_start);
            }
        }
    }
    if (cuts.back() != raw_len || raw_len == 0) cuts.push_back(raw_len);
    if (raw_len == 0) cuts.assign({0, 0});
    size_t nm = cuts.size() - 1;
    std::vector<std::vector<uint8_t>> mem(nm);
    run_parallel(threads, nm, [&](size_t m) {
        const uint8_t *src = raw + cuts[m];
        uInt len = (uInt)(cuts[m + 1] - cuts[m]);
        int level = (m % 2 == 0) ? level_even : level_odd;
        std::vector<uint8_t> buf(65536 + 64);
        uint32_t clen = 0;
        for (int attempt = 0; attempt < 2; ++attempt) {
            z_stream zs;
            memset(&zs, 0, sizeof zs);
            deflateInit2(&zs, attempt == 0 ? level : 0, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY);
            zs.next_in = (Bytef *)src;
            zs.avail_in = len;
            zs.next_out = buf.data() + 18;
            zs.avail_out = 65536 - 26;
            int rc = deflate(&zs, Z_FINISH);
            clen = (uint32_t)(65536 - 26 - zs.avail_out);
            deflateEnd(&zs);
            if (rc == Z_STREAM_END) break;
        }
        uint32_t bsize = 18 + clen + 8;
        const uint8_t h[18] = {0x1f, 0x8b, 8, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, 'B', 'C', 2, 0,
                               (uint8_t)((bsize - 1) & 0xff), (uint8_t)((bsize - 1) >> 8)};
        memcpy(buf.data(), h, 18);
        uint32_t crc = (uint32_t)crc32(0, src, len);
        uint8_t *t = buf.data() + 18 + clen;
        for (int b = 0; b < 4; ++b) t[b] = (uint8_t)(crc >> (8 * b));
        for (int b = 0; b < 4; ++b) t[4 + b] = (uint8_t)(len >> (8 * b));
        buf.resize(bsize);
        mem[m] = std::move(buf);
    });
    static const uint8_t eof[28] = {0x1f, 0x8b, 0x08, 0x04, 0x00, 0x00, 0x00, 0x00, 0x00, 0xff, 0x06, 0x00, 0x42, 0x43,
                                    0x02, 0x00, 0x1b, 0x00, 0x03, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00, 0x00};
    std::vector<size_t> base(nm + 1, 0);
    for (size_t m = 0; m < nm; ++m) base[m + 1] = base[m] + mem[m].size();
    size_t total = base[nm] + 28;
    uint8_t *o = (uint8_t *)malloc(total);
    if (!o) return -1;
    run_parallel(threads, nm, [&](size_t m) { memcpy(o + base[m], mem[m].data(), mem[m].size()); });
    memcpy(o + base[nm], eof, 28);
    *out = o;
    *out_len = total;
    if (n_members_out) *n_members_out = nm + 1;
    return 0;
}


// Joins per-chunk parts after `head`; optional record end offsets.
static int join_parts(const std::vector<uint8_t> &head, std::vector<std::vector<uint8_t>> &parts,
                      std::vector<std::vector<uint64_t>> &ends, int threads, uint8_t **raw, size_t *raw_len,
                      uint64_t **record_ends, size_t *n_ends)
{
    size_t n_chunks = parts.size();
    std::vector<size_t> base(n_chunks + 1, head.size());
    for (size_t c = 0; c < n_chunks; ++c) base[c + 1] = base[c] + parts[c].size();
    size_t total = base[n_chunks];
    uint8_t *buf = (uint8_t *)malloc(total ? total : 1);
    if (!buf) return -1;
    if (!head.empty()) memcpy(buf, head.data(), head.size());
    run_parallel(threads, n_chunks, [&](size_t c) {
        memcpy(buf + base[c], parts[c].data(), parts[c].size());
        std::vector<uint8_t>().swap(parts[c]);
    });
    if (record_ends) {
        size_t n = 1;
        for (auto &e : ends) n += e.size();
        uint64_t *re = (uint64_t *)malloc(sizeof(uint64_t) * n);
        re[0] = head.size();
        size_t k = 1;
        for (size_t c = 0; c < n_chunks; ++c)
            for (uint64_t v : ends[c]) re[k++] = base[c] + v;
        *record_ends = re;
        *n_ends = k;
    }
    *raw = buf;
    *raw_len = total;
    return 0;
}

// FASTQ stream of `n_records` (kind 0 Illumina-like, 1 ultra-long).
int frt_synth_fastq(int kind, uint64_t n_records, uint64_t seed, int threads, uint8_t **raw, size_t *raw_len,
                    uint64_t **record_ends, size_t *n_ends)
{
    const uint64_t chunk = kind == 0 ? 65536 : 64;
    size_t n_chunks = (size_t)((n_records + chunk - 1) / chunk);
    std::vector<std::vector<uint8_t>> parts(n_chunks);
    std::vector<std::vector<uint64_t>> ends(n_chunks);
    run_parallel(threads, n_chunks, [&](size_t c) {
        for (uint64_t i = c * chunk, e = std::min(n_records, (c + 1) * chunk); i < e; ++i) {
            fastq_record(parts[c], i, kind, seed);
            if (record_ends) ends[c].push_back(parts[c].size());
        }
    });
    return join_parts({}, parts, ends, threads, raw, raw_len, record_ends, n_ends);
}

// BCF stream (header + records) of `n_sites` over `n_contigs` contigs of a
// 3.1 Gb genome with `n_samples` samples.
int frt_synth_bcf(uint64_t n_sites, uint32_t n_samples, int n_contigs, uint64_t seed, int threads, uint8_t **raw,
                  size_t *raw_len, uint64_t **record_ends, size_t *n_ends)
{
    std::vector<Contig> contigs = make_contigs(n_contigs, 3100000000ull);
    std::vector<uint8_t> head = bcf_header(contigs, n_samples);
    // sites per contig in proportion to length, evenly spaced with jitter
    std::vector<uint64_t> first(contigs.size() + 1, 0);
    uint64_t glen = 0;
    for (auto &c : contigs) glen += c.length;
    for (size_t k = 0; k < contigs.size(); ++k)
        first[k + 1] = k + 1 == contigs.size() ? n_sites
                                               : first[k] + (uint64_t)((double)n_sites * contigs[k].length / glen);
    const uint64_t chunk = n_samples > 64 ? 1024 : 16384;
    size_t n_chunks = (size_t)((n_sites + chunk - 1) / chunk);
    std::vector<std::vector<uint8_t>> parts(n_chunks);
    std::vector<std::vector<uint64_t>> ends(n_chunks);
    run_parallel(threads, n_chunks, [&](size_t c) {
        for (uint64_t i = c * chunk, e = std::min(n_sites, (c + 1) * chunk); i < e; ++i) {
            size_t k = (size_t)(std::upper_bound(first.begin(), first.end(), i) - first.begin() - 1);
            uint64_t n_here = std::max<uint64_t>(1, first[k + 1] - first[k]);
            double step = (double)contigs[k].length / (double)n_here;
            Rng j(seed, 0x50000000ull + i);
            int32_t pos = (int32_t)std::min<double>(contigs[k].length - 1.0,
                                                    (double)(i - first[k]) * step + j.uniform() * step * 0.5);
            bcf_record(parts[c], i, (int32_t)k, pos, n_samples, seed);
            if (record_ends) ends[c].push_back(parts[c].size());
        }
    });
    return join_parts(head, parts, ends, threads, raw, raw_len, record_ends, n_ends);
}

// FASTA text of `n_contigs` contigs totalling about `total_bases`, wrapped at
// `line_width`; `blank_lines` puts an empty line between records.
int frt_synth_fasta(int n_contigs, uint64_t total_bases, uint32_t line_width, int blank_lines, uint64_t seed,
                    int threads, uint8_t **raw, size_t *raw_len)
{
    if (line_width == 0) return -1;
    std::vector<Contig> contigs = make_contigs(n_contigs, total_bases);
    uint64_t sum = 0;
    for (auto &c : contigs) sum += c.length;
    for (auto &c : contigs) c.length = (uint32_t)std::max<uint64_t>(1, (uint64_t)((double)c.length * total_bases / sum));
    // chunks of whole lines, about 1 Mb each
    const uint64_t chunk = (uint64_t)line_width * std::max<uint64_t>(1, (1u << 20) / line_width);
    // each contig: definition line, wrapped bases, optional blank line
    struct Piece { uint64_t contig, first, n, dst, index; };
    std::vector<std::string> defs;
    std::vector<uint64_t> contig_at;
    uint64_t at = 0;
    std::vector<Piece> pieces;
    for (size_t k = 0; k < contigs.size(); ++k) {
        Rng r(seed, 0x60000000ull + k);
        std::string d = ">" + contigs[k].name + " AC:CM" + std::to_string(100000 + r.below(900000)) +
                        ".2 LN:" + std::to_string(contigs[k].length) + " rl:Chromosome AS:synthetic\n";
        defs.push_back(d);
        contig_at.push_back(at);
        uint64_t L = contigs[k].length, lines = (L + line_width - 1) / line_width;
        uint64_t seq_at = at + d.size();
        for (uint64_t f = 0; f < L; f += chunk)
            pieces.push_back({k, f, std::min<uint64_t>(chunk, L - f), seq_at + f + f / line_width, f / chunk});
        at = seq_at + L + lines + (blank_lines && k + 1 < contigs.size() ? 1 : 0);
    }
    uint8_t *buf = (uint8_t *)malloc(at ? at : 1);
    if (!buf) return -1;
    for (size_t k = 0; k < contigs.size(); ++k) {
        memcpy(buf + contig_at[k], defs[k].data(), defs[k].size());
        uint64_t L = contigs[k].length, lines = (L + line_width - 1) / line_width;
        uint64_t end = contig_at[k] + defs[k].size() + L + lines;
        if (blank_lines && k + 1 < contigs.size()) buf[end] = '\n';
    }
    run_parallel(threads, pieces.size(), [&](size_t i) {
        const Piece &p = pieces[i];
        std::vector<uint8_t> tmp(p.n);
        fasta_chunk(tmp.data(), p.contig, p.index, p.n, seed);
        uint8_t *d = buf + p.dst;
        uint64_t L = contigs[p.contig].length;
        for (uint64_t j = 0; j < p.n;) {
            uint64_t g = p.first + j, in_line = g % line_width, take = std::min<uint64_t>(line_width - in_line, p.n - j);
            memcpy(d, tmp.data() + j, take);
            d += take;
            j += take;
            if ((g + take) % line_width == 0 || g + take == L) *d++ = '\n';
        }
    });
    *raw = buf;
    *raw_len = at;
    return 0;
}

// BAI (SAM specification 5.2) for a coordinate-sorted BAM already written as
// BGZF: for each reference the bins (reg2bin with min_shift 14, depth 5) with
// their chunks -- a chunk per run of consecutive records in the same bin, as
// htslib's indexer forms them -- the metadata pseudo-bin 37450 (first/last
// virtual offsets, mapped/unmapped counts), and the 16 kb linear index (the
// start of the first record overlapping each window, gaps filled from the
// next window).  Virtual offsets at a member boundary name the next member.
int frt_synth_bai(const uint8_t *raw, size_t raw_len, const uint8_t *bgzf, size_t bgzf_len, uint8_t **out,
                  size_t *out_len)
{
    // member layout: raw start and compressed offset of each member
    std::vector<uint64_t> rstart, coff;
    uint64_t r = 0;
    for (size_t p = 0; p + 18 <= bgzf_len;) {
        uint32_t xlen = bgzf[p + 10] | (bgzf[p + 11] << 8);
        uint32_t bsize = 0;
        for (uint32_t o = 0; o + 4 <= xlen;) {
            const uint8_t *x = bgzf + p + 12 + o;
            uint32_t sl = x[2] | (x[3] << 8);
            if (x[0] == 'B' && x[1] == 'C' && sl == 2) bsize = (x[4] | (x[5] << 8)) + 1;
            o += 4 + sl;
        }
        if (!bsize || p + bsize > bgzf_len) return -1;
        const uint8_t *t = bgzf + p + bsize - 4;
        uint32_t isize = t[0] | (t[1] << 8) | (t[2] << 16) | ((uint32_t)t[3] << 24);
        rstart.push_back(r);
        coff.push_back(p);
        r += isize;
        p += bsize;
    }
    rstart.push_back(r);
    coff.push_back(bgzf_len);
    if (r != raw_len) return -2;
    auto voff = [&](uint64_t x) -> uint64_t {
        size_t m = (size_t)(std::upper_bound(rstart.begin(), rstart.end(), x) - rstart.begin()) - 1;
        while (m + 1 < rstart.size() && rstart[m + 1] == x) ++m; // a boundary names the next member
        if (m + 1 >= rstart.size()) return coff.back() << 16;
        return (coff[m] << 16) | (x - rstart[m]);
    };
    auto rd32 = [&](uint64_t at) { return (uint32_t)raw[at] | (raw[at + 1] << 8) | (raw[at + 2] << 16) | ((uint32_t)raw[at + 3] << 24); };
    // header
    uint64_t at = 4;
    uint32_t l_text = rd32(at);
    at += 4 + l_text;
    int32_t n_ref = (int32_t)rd32(at);
    at += 4;
    for (int32_t i = 0; i < n_ref; ++i) at += 4 + rd32(at) + 4;
    struct Ref {
        std::vector<std::pair<uint32_t, std::vector<std::pair<uint64_t, uint64_t>>>> bins; // in first-seen order
        std::vector<int64_t> lidx;
        uint64_t beg = ~0ull, end = 0, mapped = 0, unmapped = 0;
        bool any = false;
    };
    std::vector<Ref> refs(n_ref > 0 ? n_ref : 0);
    std::vector<std::vector<int>> slot(refs.size()); // bin id -> index into bins (37450 + 1 entries)
    int32_t cur_tid = -1;
    uint32_t save_bin = 0xffffffffu;
    uint64_t save_off = 0, last_off = 0;
    auto flush = [&](int32_t tid) {
        if (tid < 0 || save_bin == 0xffffffffu) return;
        auto &rf = refs[tid];
        auto &sl = slot[tid];
        if (sl.empty()) sl.assign(37451, -1);
        if (sl[save_bin] < 0) {
            sl[save_bin] = (int)rf.bins.size();
            rf.bins.push_back({save_bin, {}});
        }
        rf.bins[sl[save_bin]].second.push_back({save_off, last_off});
    };
    uint64_t n_no_coor = 0;
    while (at + 4 <= raw_len) {
        uint32_t bs = rd32(at);
        uint64_t rec = at, end_at = at + 4 + bs;
        int32_t tid = (int32_t)rd32(rec + 4), pos = (int32_t)rd32(rec + 8);
        uint32_t name_len = raw[rec + 12], n_cigar = raw[rec + 16] | (raw[rec + 17] << 8);
        uint16_t flag = (uint16_t)(raw[rec + 18] | (raw[rec + 19] << 8));
        uint64_t v0 = voff(rec), v1 = voff(end_at);
        if (tid < 0 || tid >= n_ref) {
            ++n_no_coor;
            at = end_at;
            continue;
        }
        int64_t span = 0;
        for (uint32_t k = 0; k < n_cigar; ++k) {
            uint32_t op = rd32(rec + 36 + name_len + 4 * k), kind = op & 15;
            if (kind == 0 || kind == 2 || kind == 3 || kind == 7 || kind == 8) span += op >> 4;
        }
        int64_t beg = pos, end = pos + (span > 0 ? span : 1);
        uint32_t bin = (uint32_t)reg2bin(beg, end);
        if (tid != cur_tid) {
            flush(cur_tid);
            cur_tid = tid;
            save_bin = 0xffffffffu;
        }
        if (bin != save_bin) {
            flush(tid);
            save_bin = bin;
            save_off = v0;
        }
        last_off = v1;
        auto &rf = refs[tid];
        for (int64_t w = beg >> 14; w <= (end - 1) >> 14; ++w) {
            if ((int64_t)rf.lidx.size() <= w) rf.lidx.resize(w + 1, -1);
            if (rf.lidx[w] < 0) rf.lidx[w] = (int64_t)v0;
        }
        rf.any = true;
        rf.beg = std::min(rf.beg, v0);
        rf.end = std::max(rf.end, v1);
        if (flag & 4) ++rf.unmapped;
        else ++rf.mapped;
        at = end_at;
    }
    flush(cur_tid);
    std::vector<uint8_t> o = {'B', 'A', 'I', 1};
    put32(o, (uint32_t)n_ref);
    auto put64 = [&](uint64_t v) {
        put32(o, (uint32_t)v);
        put32(o, (uint32_t)(v >> 32));
    };
    for (auto &rf : refs) {
        put32(o, (uint32_t)(rf.bins.size() + (rf.any ? 1 : 0)));
        for (auto &b : rf.bins) {
            put32(o, b.first);
            put32(o, (uint32_t)b.second.size());
            for (auto &c : b.second) {
                put64(c.first);
                put64(c.second);
            }
        }
        if (rf.any) {
            put32(o, 37450);
            put32(o, 2);
            put64(rf.beg);
            put64(rf.end);
            put64(rf.mapped);
            put64(rf.unmapped);
        }
        // gaps take the next window's offset
        int64_t next = rf.lidx.empty() ? 0 : rf.lidx.back();
        for (size_t w = rf.lidx.size(); w-- > 0;) {
            if (rf.lidx[w] < 0) rf.lidx[w] = next;
            else next = rf.lidx[w];
        }
        put32(o, (uint32_t)rf.lidx.size());
        for (int64_t v : rf.lidx) put64((uint64_t)v);
    }
    put64(n_no_coor);
    uint8_t *buf = (uint8_t *)malloc(o.size());
    if (!buf) return -3;
    memcpy(buf, o.data(), o.size());
    *out = buf;
    *out_len = o.size();
    return 0;
}

void frt_synth_free(void *p) { free(p); }

} // extern "C"
