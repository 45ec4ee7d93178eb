/*
 * TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference's device path for the three other
 * formats that ride on the same BGZF container: bgzipped FASTQ (record scan and
 * line-bound columns), BCF (site-core scan and columns) and FASTA (newline
 * compaction of a whole reference).  The oracle for the CUDA implementation in
 * fritillaria_gb300; the product never calls into it.
 *
 * Where the reference's CPU functions and its device launchers differ on
 * malformed input, this follows the device launchers, which is the path the
 * CUDA implementation replaces; each function says which lines it restates.
 */
#include <stdlib.h>
#include <string.h>

#include "frt_oracle.h"

static void set_err(orc_error *err, int code, uint64_t position, const char *reason)
{
    if (!err) return;
    memset(err, 0, sizeof *err);
    err->code = code;
    err->position = position;
    strncpy(err->reason, reason, sizeof err->reason - 1);
}

static uint32_t ld16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
static uint32_t ld24(const uint8_t *p) { return ld16(p) | ((uint32_t)p[2] << 16); }
static uint32_t ld32(const uint8_t *p) { return ld24(p) | ((uint32_t)p[3] << 24); }

/* Offset of the next '\n' at or after pos, or len. */
static uint64_t next_nl(const uint8_t *buf, uint64_t len, uint64_t pos)
{
    if (pos >= len) return len;
    const void *q = memchr(buf + pos, '\n', (size_t)(len - pos));
    return q ? (uint64_t)((const uint8_t *)q - buf) : len;
}

/* ---------------------------------------------------------------- FASTQ --
 * bounds_at: crates/fritillaria-fastq/src/columnar/record.rs:79-130 and
 * crates/fritillaria-cuda/kernels/fastq_scan.cu:43-95 (identical rules). */
int orc_fastq_bounds_at(const uint8_t *buf, uint64_t len, uint64_t pos, orc_fastq_bounds *b)
{
    if (pos >= len || buf[pos] != '@') return 0;
    uint64_t def_end = next_nl(buf, len, pos);
    if (def_end >= len) return 0;
    uint64_t seq_start = def_end + 1;
    uint64_t seq_end = next_nl(buf, len, seq_start);
    if (seq_end >= len) return 0;
    uint64_t plus = seq_end + 1;
    if (plus >= len || buf[plus] != '+') return 0;
    uint64_t plus_end = next_nl(buf, len, plus);
    if (plus_end >= len) return 0;
    uint64_t qual = plus_end + 1;
    uint64_t seq_len = seq_end - seq_start;
    uint64_t qual_end = next_nl(buf, len, qual);
    if (qual_end - qual != seq_len) return 0;
    uint64_t end = qual_end < len ? qual_end + 1 : qual_end;
    if (b) {
        b->sequence_start = (uint32_t)(seq_start - pos);
        b->plus_start = (uint32_t)(plus - pos);
        b->quality_start = (uint32_t)(qual - pos);
        b->sequence_len = (uint32_t)seq_len;
        b->record_end = (uint32_t)(end - pos);
    }
    return 1;
}

/* FastqScanner::run, crates/fritillaria-cuda/src/fastq.rs:486-540: the sieve
 * (every line start at or after `start` that bounds_at accepts, sorted), the
 * tiling from the anchor (start advanced past newlines) using the decoded
 * record ends (fastq.rs:585-598), else the device walk of fastq_scan.cu:173-215
 * (skips newlines, stops at the first position that is not a whole record). */
int orc_fastq_scan(const uint8_t *buf, uint64_t len, uint64_t start, uint64_t *offsets, size_t cap,
                   size_t *n_out, uint64_t *tail_out, uint64_t *survivors_out, int *proof_out)
{
    *n_out = 0;
    *survivors_out = 0;
    *proof_out = ORC_PROOF_TILED;
    if (start >= len) {
        *tail_out = len < start ? len : start;
        return ORC_OK;
    }
    uint64_t anchor = start;
    while (anchor < len && buf[anchor] == '\n') ++anchor;

    size_t ns = 0;
    uint64_t at = anchor;
    int tiled = 1;
    orc_fastq_bounds b;
    for (uint64_t i = start; i < len; ++i) {
        if (i != start && buf[i - 1] != '\n') continue;
        if (!orc_fastq_bounds_at(buf, len, i, &b)) continue;
        if (ns < cap) offsets[ns] = i;
        ++ns;
        if (tiled) {
            if (i != at) tiled = 0;
            else at = i + b.record_end;
        }
    }
    *survivors_out = ns;
    if (ns > 0 && tiled && ns <= cap) {
        *n_out = ns;
        *tail_out = at;
        return ORC_OK;
    }
    *proof_out = ORC_PROOF_WALKED;
    size_t n = 0;
    uint64_t pos = start;
    while (pos < len) {
        if (buf[pos] == '\n') {
            ++pos;
            continue;
        }
        if (!orc_fastq_bounds_at(buf, len, pos, &b)) break;
        if (n >= cap) return ORC_ERR_INVALID_ARGUMENT;
        offsets[n++] = pos;
        pos += b.record_end;
    }
    *n_out = n;
    *tail_out = pos;
    return ORC_OK;
}

/* fastq_decode, crates/fritillaria-cuda/kernels/fastq_scan.cu:139-166. */
int orc_fastq_decode(const uint8_t *buf, uint64_t len, const uint64_t *offsets, size_t n, uint32_t *sequence_start,
                     uint32_t *plus_start, uint32_t *quality_start, uint32_t *sequence_len, uint32_t *record_end)
{
    int errors = 0;
    for (size_t i = 0; i < n; ++i) {
        orc_fastq_bounds b;
        if (!orc_fastq_bounds_at(buf, len, offsets[i], &b)) {
            ++errors;
            continue;
        }
        sequence_start[i] = b.sequence_start;
        plus_start[i] = b.plus_start;
        quality_start[i] = b.quality_start;
        sequence_len[i] = b.sequence_len;
        record_end[i] = b.record_end;
    }
    return errors;
}

/* ------------------------------------------------------------------ BCF --
 * Typed values: crates/fritillaria-bcf/src/columnar/typed.rs:381-447 and
 * crates/fritillaria-cuda/kernels/bcf_scan.cu:71-196. */
static uint32_t bcf_type_size(uint32_t code)
{
    switch (code) {
    case 0: return 0;
    case 1: case 7: return 1;
    case 2: return 2;
    case 3: case 5: return 4;
    default: return 0xFFFFFFFFu;
    }
}

static uint32_t bcf_descriptor(const uint8_t *buf, uint64_t len, uint64_t pos, uint32_t *count, uint32_t *kind)
{
    if (pos >= len) return 0;
    uint32_t d = buf[pos], code = d & 15u;
    if (bcf_type_size(code) == 0xFFFFFFFFu) return 0;
    *kind = code;
    if ((d >> 4) < 15u) {
        *count = d >> 4;
        return 1;
    }
    if (pos + 1 >= len) return 0;
    uint32_t inner = buf[pos + 1], ic = inner & 15u;
    if ((inner >> 4) != 1u || (ic != 1 && ic != 2 && ic != 3)) return 0;
    uint32_t w = bcf_type_size(ic);
    if (pos + 2 + w > len) return 0;
    const uint8_t *p = buf + pos + 2;
    int32_t v = ic == 1 ? (int32_t)(int8_t)p[0] : ic == 2 ? (int32_t)(int16_t)ld16(p) : (int32_t)ld32(p);
    if (v < 15) return 0;
    *count = (uint32_t)v;
    return 2 + w;
}

static uint64_t bcf_skip(const uint8_t *buf, uint64_t len, uint64_t pos)
{
    uint32_t count = 0, kind = 0;
    uint32_t h = bcf_descriptor(buf, len, pos, &count, &kind);
    if (!h) return 0;
    uint64_t end = pos + h + (uint64_t)count * bcf_type_size(kind);
    return end > len ? 0 : end;
}

/* looks_like_a_record: crates/fritillaria-bcf/src/columnar/record.rs:149-206,
 * bcf_scan.cu:106-144. */
int orc_bcf_looks_like_a_record(const uint8_t *buf, uint64_t len, uint64_t pos, uint32_t samples, uint32_t contigs)
{
    if (pos + 32 > len) return 0;
    uint32_t ls = ld32(buf + pos), li = ld32(buf + pos + 4);
    if (ls < 24) return 0;
    if (pos + 8 + (uint64_t)ls + li > len) return 0;
    int32_t chrom = (int32_t)ld32(buf + pos + 8), p = (int32_t)ld32(buf + pos + 12), rlen = (int32_t)ld32(buf + pos + 16);
    if (chrom < 0 || (uint32_t)chrom >= contigs) return 0;
    if (p < -1 || rlen < 0) return 0;
    uint32_t n_allele = ld16(buf + pos + 26), n_sample = ld24(buf + pos + 28), n_fmt = buf[pos + 31];
    if (n_sample != samples || n_allele == 0) return 0;
    if (n_fmt == 0) return li == 0;
    return (uint64_t)li >= (uint64_t)n_fmt * 2;
}

/* Record::validate: record.rs:427-489, bcf_scan.cu:207-298. */
int orc_bcf_validate(const uint8_t *buf, uint64_t len, uint64_t pos)
{
    if (pos + 32 > len) return 0;
    uint64_t ls = ld32(buf + pos), li = ld32(buf + pos + 4);
    uint64_t indiv = pos + 8 + ls, end = indiv + li;
    if (ls < 24 || end > len) return 0;
    uint32_t n_info = ld16(buf + pos + 24), n_allele = ld16(buf + pos + 26), n_sample = ld24(buf + pos + 28);
    uint32_t n_fmt = buf[pos + 31];
    uint64_t at = bcf_skip(buf, indiv, pos + 32);
    if (!at) return 0;
    for (uint32_t i = 0; i < n_allele; ++i)
        if (!(at = bcf_skip(buf, indiv, at))) return 0;
    if (!(at = bcf_skip(buf, indiv, at))) return 0;
    for (uint32_t i = 0; i < n_info; ++i) {
        if (!(at = bcf_skip(buf, indiv, at))) return 0;
        if (!(at = bcf_skip(buf, indiv, at))) return 0;
    }
    if (at != indiv) return 0;
    for (uint32_t i = 0; i < n_fmt; ++i) {
        if (!(at = bcf_skip(buf, end, at))) return 0;
        uint32_t count = 0, kind = 0;
        uint32_t h = bcf_descriptor(buf, end, at, &count, &kind);
        if (!h) return 0;
        at += h + (uint64_t)count * bcf_type_size(kind) * n_sample;
        if (at > end) return 0;
    }
    return at == end;
}

/* BcfScanner::scan, crates/fritillaria-cuda/src/bcf.rs:280-372: sieve,
 * validate, tiling from `start` (bcf.rs:621-635), the whole-record probe at the
 * tiling's end (bcf_scan.cu:340-347), else the length-prefix walk of
 * bcf_scan.cu:374-410.  The tiled result always equals the walk's; the proof
 * only says which route produced it. */
int orc_bcf_scan(const uint8_t *buf, uint64_t len, uint64_t start, uint32_t samples, uint32_t contigs,
                 uint64_t *offsets, size_t cap, size_t *n_out, uint64_t *tail_out, uint64_t *sieved_out,
                 uint64_t *validated_out, int *proof_out)
{
    *n_out = 0;
    *sieved_out = *validated_out = 0;
    *proof_out = ORC_PROOF_TILED;
    if (start >= len) {
        *tail_out = len < start ? len : start;
        return ORC_OK;
    }
    size_t nv = 0, nsv = 0;
    uint64_t at = start;
    int tiled = 1;
    for (uint64_t pos = start; pos < len; ++pos) {
        if (!orc_bcf_looks_like_a_record(buf, len, pos, samples, contigs)) continue;
        ++nsv;
        if (!orc_bcf_validate(buf, len, pos)) continue;
        uint64_t end = pos + 8 + (uint64_t)ld32(buf + pos) + ld32(buf + pos + 4);
        if (nv < cap) offsets[nv] = pos;
        ++nv;
        if (tiled) {
            if (pos != at || end > len || end <= pos) tiled = 0;
            else at = end;
        }
    }
    *sieved_out = nsv;
    *validated_out = nv;
    if (tiled && nv <= cap) {
        int whole = at + 8 <= len && at + 8 + (uint64_t)ld32(buf + at) + ld32(buf + at + 4) <= len;
        if (!whole) {
            *n_out = nv;
            *tail_out = at;
            return ORC_OK;
        }
    }
    *proof_out = ORC_PROOF_WALKED;
    size_t n = 0;
    uint64_t pos = start;
    for (;;) {
        if (pos + 8 > len) break;
        uint64_t ls = ld32(buf + pos), li = ld32(buf + pos + 4);
        if (ls < 24) break;
        uint64_t end = pos + 8 + ls + li;
        if (end > len) break;
        if (n >= cap) return ORC_ERR_INVALID_ARGUMENT;
        offsets[n++] = pos;
        pos = end;
    }
    *n_out = n;
    *tail_out = pos;
    return ORC_OK;
}

/* bcf_decode, bcf_scan.cu:432-510 (RecordBatch::decode + Record::bounds,
 * crates/fritillaria-bcf/src/columnar/batch.rs:222-241). Returns the number of
 * records whose walk failed. */
int orc_bcf_decode(const uint8_t *buf, uint64_t len, const uint64_t *offsets, size_t n, const orc_bcf_columns *c)
{
    int errors = 0;
    for (size_t i = 0; i < n; ++i) {
        uint64_t pos = offsets[i];
        if (pos + 32 > len) { ++errors; continue; }
        uint64_t ls = ld32(buf + pos), li = ld32(buf + pos + 4);
        if (ls < 24) { ++errors; continue; }
        uint64_t end = pos + 8 + ls + li;
        if (end > len) { ++errors; continue; }
        uint32_t n_allele = ld16(buf + pos + 26);
        c->chromosome_id[i] = (int32_t)ld32(buf + pos + 8);
        c->position[i] = (int32_t)ld32(buf + pos + 12);
        c->reference_span[i] = (int32_t)ld32(buf + pos + 16);
        c->quality[i] = ld32(buf + pos + 20);
        c->info_count[i] = (uint16_t)ld16(buf + pos + 24);
        c->allele_count[i] = (uint16_t)n_allele;
        c->sample_count[i] = ld24(buf + pos + 28);
        c->format_count[i] = buf[pos + 31];
        c->genotypes_start[i] = (uint32_t)(8 + ls);
        c->record_end[i] = (uint32_t)(end - pos);
        uint64_t w = bcf_skip(buf, end, pos + 32);
        if (!w) { ++errors; continue; }
        c->alleles_start[i] = (uint32_t)(w - pos);
        int bad = 0;
        for (uint32_t a = 0; a < n_allele && !bad; ++a)
            if (!(w = bcf_skip(buf, end, w))) bad = 1;
        if (bad) { ++errors; continue; }
        c->filters_start[i] = (uint32_t)(w - pos);
        if (!(w = bcf_skip(buf, end, w))) { ++errors; continue; }
        c->info_start[i] = (uint32_t)(w - pos);
    }
    return errors;
}

/* parse_header: crates/fritillaria-bcf/src/columnar/header.rs:111-310. Only
 * what the scan needs: where records start, the sample count (#CHROM columns
 * after the eight fixed ones) and the contig count (##contig lines with an
 * ID); an unparseable IDX on a FILTER/INFO/FORMAT line is Malformed as there. */
static const uint8_t *trim(const uint8_t *s, const uint8_t *e, const uint8_t **te)
{
    while (s < e && (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r' || *s == '\f' || *s == '\v')) ++s;
    while (e > s && (e[-1] == ' ' || e[-1] == '\t' || e[-1] == '\n' || e[-1] == '\r' || e[-1] == '\f' || e[-1] == '\v')) --e;
    *te = e;
    return s;
}

/* attribute(body, key): value span or NULL (header.rs:280-308). */
static const uint8_t *attribute(const uint8_t *b, const uint8_t *be, const char *key, const uint8_t **ve)
{
    size_t kl = strlen(key);
    const uint8_t *p = b;
    while (p < be) {
        const uint8_t *s = p, *eq = NULL;
        int quoted = 0;
        while (p < be) {
            if (*p == '"') quoted = !quoted;
            else if (*p == '=' && !quoted && !eq) eq = p;
            else if (*p == ',' && !quoted) break;
            ++p;
        }
        if (eq) {
            const uint8_t *ne, *ns = trim(s, eq, &ne);
            if ((size_t)(ne - ns) == kl && memcmp(ns, key, kl) == 0) {
                const uint8_t *vend, *v = trim(eq + 1, p, &vend);
                if (vend - v >= 2 && *v == '"' && vend[-1] == '"') {
                    ++v;
                    --vend;
                }
                *ve = vend;
                return v;
            }
        }
        ++p;
    }
    return NULL;
}

static int starts_with(const uint8_t *s, const uint8_t *e, const char *pfx)
{
    size_t n = strlen(pfx);
    return (size_t)(e - s) >= n && memcmp(s, pfx, n) == 0;
}

int orc_bcf_header(const uint8_t *buf, uint64_t len, uint64_t *records_start, uint32_t *samples, uint32_t *contigs,
                   orc_error *err)
{
    if (len < 9) { set_err(err, ORC_ERR_MALFORMED, 0, "truncated header"); return ORC_ERR_MALFORMED; }
    if (memcmp(buf, "BCF", 3) != 0) { set_err(err, ORC_ERR_MALFORMED, 0, "bad magic; expected BCF"); return ORC_ERR_MALFORMED; }
    if (buf[3] != 2) { set_err(err, ORC_ERR_MALFORMED, 3, "unsupported major version"); return ORC_ERR_MALFORMED; }
    uint64_t l_text = ld32(buf + 5);
    if (9 + l_text > len) {
        set_err(err, ORC_ERR_MALFORMED, 5, "l_text runs past the end of the buffer");
        return ORC_ERR_MALFORMED;
    }
    const uint8_t *t = buf + 9, *te = buf + 9 + l_text;
    while (te > t && te[-1] == 0) --te;
    uint32_t n_samples = 0, n_contigs = 0;
    /* the ids seen among FILTER/INFO/FORMAT lines, for the one-entry rule */
    const uint8_t **seen = NULL;
    size_t *seen_len = NULL, n_seen = 0, cap_seen = 0;
    int rc = ORC_OK;
    for (const uint8_t *line = t; line < te;) {
        const uint8_t *le = memchr(line, '\n', (size_t)(te - line));
        if (!le) le = te;
        const uint8_t *next = le < te ? le + 1 : te;
        if (le > line && le[-1] == '\r') --le;
        if (le == line) { line = next; continue; }
        if (starts_with(line, le, "#CHROM")) {
            /* split the rest on tabs, skip the empty piece and 8 fixed columns */
            size_t pieces = 1;
            for (const uint8_t *p = line + 6; p < le; ++p) pieces += *p == '\t';
            n_samples = pieces > 9 ? (uint32_t)(pieces - 9) : 0;
            line = next;
            continue;
        }
        const uint8_t *open = memchr(line, '<', (size_t)(le - line)), *close = NULL;
        for (const uint8_t *p = le; p > line; --p)
            if (p[-1] == '>') { close = p - 1; break; }
        if (!open || !close || close <= open) { line = next; continue; }
        const uint8_t *ide, *id = attribute(open + 1, close, "ID", &ide);
        if (!id) { line = next; continue; }
        if (starts_with(line, le, "##contig=")) {
            ++n_contigs;
            line = next;
            continue;
        }
        if (!(starts_with(line, le, "##FILTER=") || starts_with(line, le, "##INFO=") ||
              starts_with(line, le, "##FORMAT="))) {
            line = next;
            continue;
        }
        int dup = (ide - id == 4 && memcmp(id, "PASS", 4) == 0);
        for (size_t k = 0; k < n_seen && !dup; ++k)
            dup = seen_len[k] == (size_t)(ide - id) && memcmp(seen[k], id, seen_len[k]) == 0;
        if (dup) { line = next; continue; }
        const uint8_t *xe, *x = attribute(open + 1, close, "IDX", &xe);
        if (x) {
            int ok = xe > x;
            for (const uint8_t *p = x; p < xe && ok; ++p) ok = *p >= '0' && *p <= '9';
            if (!ok) {
                set_err(err, ORC_ERR_MALFORMED, 0, "unparseable IDX on header line");
                rc = ORC_ERR_MALFORMED;
                break;
            }
        }
        if (n_seen == cap_seen) {
            cap_seen = cap_seen ? 2 * cap_seen : 64;
            seen = realloc(seen, cap_seen * sizeof *seen);
            seen_len = realloc(seen_len, cap_seen * sizeof *seen_len);
        }
        seen[n_seen] = id;
        seen_len[n_seen++] = (size_t)(ide - id);
        line = next;
    }
    free(seen);
    free(seen_len);
    if (rc) return rc;
    *records_start = 9 + l_text;
    *samples = n_samples;
    *contigs = n_contigs;
    return ORC_OK;
}

/* ---------------------------------------------------------------- FASTA --
 * bounds_at: crates/fritillaria-fasta/src/columnar/record.rs:101-160. */
int orc_fasta_bounds_at(const uint8_t *buf, uint64_t len, uint64_t pos, orc_fasta_bounds *b)
{
    if (pos >= len || buf[pos] != '>') return 0;
    uint64_t def_end = next_nl(buf, len, pos);
    if (def_end >= len) return 0;
    uint64_t seq_start = def_end + 1, at = seq_start, seq_len = 0;
    uint64_t first = 0, nonblank = 0, last = 0;
    int uniform = 1;
    while (at < len) {
        if (buf[at] == '>') break;
        uint64_t e = next_nl(buf, len, at), l = e - at;
        seq_len += l;
        if (l > 0) {
            /* every non-blank line but the last must equal the first */
            if (nonblank >= 2 && last != first) uniform = 0;
            if (nonblank == 0) first = l;
            last = l;
            ++nonblank;
        }
        at = e < len ? e + 1 : e;
    }
    if (b) {
        b->sequence_start = (uint32_t)(seq_start - pos);
        b->sequence_len = seq_len;
        b->line_bases = (uint32_t)first;
        b->line_width = (uint32_t)(first + 1);
        b->record_end = at - pos;
        b->uniform = (uint8_t)uniform;
    }
    return 1;
}

/* FastaCompactor::compact, crates/fritillaria-cuda/src/fasta.rs:212-300: the
 * records from the first '>' at a line start (fasta_compact.cu:86-111) walked
 * as scan_records(buf, first, at_eof = true) (record.rs:180-214); each
 * contig's bases are its sequence span without newlines (compact_into,
 * record.rs:300-330).  Returns the number of contigs; seq may be NULL to size. */
int orc_fasta_compact(const uint8_t *buf, uint64_t len, uint8_t *seq, uint64_t seq_cap, uint64_t *seq_offsets,
                      uint64_t *seq_lengths, uint64_t *record_offsets, orc_fasta_bounds *bounds, size_t cap,
                      size_t *n_out, uint64_t *total_out)
{
    *n_out = 0;
    *total_out = 0;
    uint64_t first = len;
    for (uint64_t i = 0; i < len; ++i)
        if (buf[i] == '>' && (i == 0 || buf[i - 1] == '\n')) { first = i; break; }
    size_t n = 0;
    uint64_t total = 0, pos = first;
    while (pos < len) {
        if (buf[pos] == '\n') { ++pos; continue; }
        orc_fasta_bounds b;
        if (!orc_fasta_bounds_at(buf, len, pos, &b)) break;
        if (n >= cap) return ORC_ERR_INVALID_ARGUMENT;
        record_offsets[n] = pos;
        seq_offsets[n] = total;
        seq_lengths[n] = b.sequence_len;
        if (bounds) bounds[n] = b;
        if (seq) {
            uint64_t o = total;
            for (uint64_t i = pos + b.sequence_start; i < pos + b.record_end; ++i)
                if (buf[i] != '\n') {
                    if (o >= seq_cap) return ORC_ERR_INVALID_ARGUMENT;
                    seq[o++] = buf[i];
                }
        }
        total += b.sequence_len;
        ++n;
        pos += b.record_end;
    }
    *n_out = n;
    *total_out = total;
    return ORC_OK;
}
