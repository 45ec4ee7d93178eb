/*
 * TEST INFRASTRUCTURE ONLY -- the oracle for fritillaria_gb300.
 *
 * A CPU restatement of the reference's algorithm for the BGZF -> device
 * columns path.  Each function names the reference file:line it follows.
 * Nothing in the product path calls this file; it is the oracle the tests compare against.
 */
#define _GNU_SOURCE
#include "frt_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <zlib.h>

#define MAX_BLOCK_SIZE 65536u /* crates/fritillaria-core/src/lib.rs:41 */

static void set_err(orc_error *err, int code, uint64_t offset, uint64_t expected, uint64_t actual,
                    uint64_t position, const char *reason)
{
    if (!err) return;
    err->code = code;
    err->offset = offset;
    err->expected = expected;
    err->actual = actual;
    err->position = position;
    snprintf(err->reason, sizeof err->reason, "%s", reason ? reason : "");
}

static uint32_t rd32(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24); }
static uint32_t rd16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }

/* ------------------------------------------------------------------------
 * CRC-32/ISO-HDLC, reflected polynomial 0xEDB88320, init/xorout 0xFFFFFFFF.
 * The table is derived from the polynomial (Sarwate's method); the reference
 * computes it bitwise (kernels/crc32.cu:13-38) and through crc32fast
 * (crates/fritillaria-bgzf/src/cpu.rs:59).
 * ---------------------------------------------------------------------- */
static uint32_t crc_table[256];
static pthread_once_t crc_once = PTHREAD_ONCE_INIT;

static void crc_init(void)
{
    for (uint32_t i = 0; i < 256; ++i) {
        uint32_t c = i;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
        crc_table[i] = c;
    }
}

uint32_t orc_crc32(uint32_t crc, const uint8_t *p, size_t n)
{
    pthread_once(&crc_once, crc_init);
    uint32_t c = ~crc;
    for (size_t i = 0; i < n; ++i) c = crc_table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return ~c;
}

/* Multiplication modulo the CRC polynomial in the reflected bit order. */
static uint32_t gf2_mul(uint32_t a, uint32_t b)
{
    uint32_t r = 0;
    for (int i = 0; i < 32; ++i) {
        if (a & 0x80000000u) r ^= b;
        a <<= 1;
        b = (b >> 1) ^ (0xEDB88320u & (0u - (b & 1u)));
    }
    return r;
}

/* x^(8n) mod P, by square-and-multiply from x^8. */
static uint32_t x8n(uint64_t n)
{
    uint32_t result = 0x80000000u; /* x^0 */
    uint32_t sq = 0x00800000u;     /* x^8 */
    while (n) {
        if (n & 1u) result = gf2_mul(result, sq);
        sq = gf2_mul(sq, sq);
        n >>= 1;
    }
    return result;
}

/* crc(A || B) from crc(A), crc(B) and |B|: the GF(2) linearity of CRC. */
uint32_t orc_crc32_combine(uint32_t crc_a, uint32_t crc_b, uint64_t len_b)
{
    return gf2_mul(x8n(len_b), crc_a) ^ crc_b;
}

/* ------------------------------------------------------------------------
 * BGZF framing: crates/fritillaria-bgzf/src/block.rs:88-165 (header_len,
 * parse_header, find_bc_subfield) and discovery discover.rs:51-109.
 * ---------------------------------------------------------------------- */
int orc_bgzf_parse_header(const uint8_t *buf, size_t len, uint64_t offset, uint32_t *block_size,
                          uint32_t *header_size, orc_error *err)
{
    if (len < 12) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "truncated header"); return ORC_ERR_INVALID_BLOCK; }
    if (buf[0] != 0x1f || buf[1] != 0x8b) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "not a gzip member (bad magic)"); return ORC_ERR_INVALID_BLOCK; }
    if (buf[2] != 8) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "unsupported compression method"); return ORC_ERR_INVALID_BLOCK; }
    if ((buf[3] & 0x04) == 0) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "missing FEXTRA; not BGZF (plain gzip?)"); return ORC_ERR_INVALID_BLOCK; }
    size_t xlen = rd16(buf + 10);
    size_t hsize = 12 + xlen;
    if (len < hsize) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "truncated extra field"); return ORC_ERR_INVALID_BLOCK; }
    /* find_bc_subfield: BC need not be first; foreign subfields are skipped. */
    const uint8_t *x = buf + 12;
    size_t left = xlen;
    int found = 0;
    uint32_t bsize = 0;
    while (left >= 4) {
        size_t slen = rd16(x + 2);
        if (4 + slen > left) break;
        if (x[0] == 'B' && x[1] == 'C') {
            if (slen != 2) break;
            bsize = rd16(x + 4);
            found = 1;
            break;
        }
        x += 4 + slen;
        left -= 4 + slen;
    }
    if (!found) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "missing BC subfield; not BGZF"); return ORC_ERR_INVALID_BLOCK; }
    uint32_t bs = bsize + 1;
    if (bs > MAX_BLOCK_SIZE) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "block size exceeds 64 KiB"); return ORC_ERR_INVALID_BLOCK; }
    if (bs < hsize + 8) { set_err(err, ORC_ERR_INVALID_BLOCK, offset, 0, 0, 0, "block size smaller than its own framing"); return ORC_ERR_INVALID_BLOCK; }
    *block_size = bs;
    *header_size = (uint32_t)hsize;
    return ORC_OK;
}

int orc_bgzf_discover(const uint8_t *buf, size_t len, uint64_t base_offset, orc_span *spans,
                      size_t cap, size_t *n_spans, size_t *consumed, orc_error *err)
{
    size_t pos = 0, n = 0;
    while (pos < len) {
        const uint8_t *rest = buf + pos;
        size_t rlen = len - pos;
        /* header_len: too few bytes to measure the header is a resume point */
        if (rlen < 12) break;
        size_t hl = 12 + rd16(rest + 10);
        if (hl > rlen) break;
        uint32_t bs, hs;
        int rc = orc_bgzf_parse_header(rest, rlen, base_offset + pos, &bs, &hs, err);
        if (rc) { *n_spans = n; *consumed = pos; return rc; }
        if (bs > rlen) break; /* partial trailing block: resume point */
        uint32_t crc = rd32(rest + bs - 8);
        uint32_t isz = rd32(rest + bs - 4);
        if (isz > MAX_BLOCK_SIZE) {
            set_err(err, ORC_ERR_INVALID_BLOCK, base_offset + pos, 0, 0, 0, "ISIZE exceeds 64 KiB");
            *n_spans = n; *consumed = pos;
            return ORC_ERR_INVALID_BLOCK;
        }
        if (n < cap) {
            spans[n].compressed_offset = base_offset + pos;
            spans[n].payload_start = pos + hs;
            spans[n].payload_len = bs - hs - 8;
            spans[n].isize = isz;
            spans[n].crc32 = crc;
        }
        ++n;
        pos += bs;
    }
    *n_spans = n;
    *consumed = pos;
    return ORC_OK;
}

/* ------------------------------------------------------------------------
 * Raw inflate through zlib, with the output capped at the declared size: a
 * stream that would write past ISIZE cannot reach its end and fails, which
 * is how the noodles reader treats it (crates/fritillaria-bgzf/src/io/reader/frame.rs:103-156,
 * deflate.rs:22-33).
 * ---------------------------------------------------------------------- */
int orc_inflate_raw(const uint8_t *in, size_t in_len, uint8_t *out, size_t out_cap, size_t *produced)
{
    z_stream zs;
    memset(&zs, 0, sizeof zs);
    if (inflateInit2(&zs, -15) != Z_OK) return -1;
    uint8_t dummy = 0;
    zs.next_in = (Bytef *)in;
    zs.avail_in = (uInt)in_len;
    zs.next_out = out_cap ? out : &dummy;
    zs.avail_out = (uInt)out_cap;
    int rc = inflate(&zs, Z_FINISH);
    *produced = out_cap - zs.avail_out;
    inflateEnd(&zs);
    return rc == Z_STREAM_END ? 0 : -1;
}

/* CpuCodec::inflate_batch (crates/fritillaria-bgzf/src/cpu.rs:39-96) with the
 * plan checks of BatchPlan::new (crates/fritillaria-cuda/src/backend.rs:95-133)
 * and the verification order of verify_and_offsets (backend.rs:221-256):
 * inflate status, then ISIZE, then CRC32, spans in order. */
int orc_inflate_batch(const uint8_t *batch, size_t batch_len, const orc_span *spans, size_t n,
                      uint8_t *out, size_t out_cap, uint64_t *out_offsets, orc_error *err)
{
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) {
        if (spans[i].isize > MAX_BLOCK_SIZE) { set_err(err, ORC_ERR_INVALID_BLOCK, spans[i].compressed_offset, 0, 0, 0, "ISIZE exceeds 64 KiB"); return ORC_ERR_INVALID_BLOCK; }
        if (spans[i].payload_start + spans[i].payload_len > batch_len || spans[i].payload_start + spans[i].payload_len < spans[i].payload_start) {
            set_err(err, ORC_ERR_INVALID_BLOCK, spans[i].compressed_offset, 0, 0, 0, "payload extends past the end of the batch");
            return ORC_ERR_INVALID_BLOCK;
        }
        out_offsets[i] = total;
        total += spans[i].isize;
    }
    out_offsets[n] = total;
    if (total > out_cap) { set_err(err, ORC_ERR_INVALID_ARGUMENT, 0, 0, 0, 0, "output buffer too small"); return ORC_ERR_INVALID_ARGUMENT; }
    for (size_t i = 0; i < n; ++i) {
        size_t produced = 0;
        int rc = orc_inflate_raw(batch + spans[i].payload_start, spans[i].payload_len, out + out_offsets[i], spans[i].isize, &produced);
        if (rc) { set_err(err, ORC_ERR_INFLATE, spans[i].compressed_offset, 0, 0, 0, "inflate failed"); return ORC_ERR_INFLATE; }
        if (produced != spans[i].isize) { set_err(err, ORC_ERR_SIZE, spans[i].compressed_offset, spans[i].isize, produced, 0, "size mismatch"); return ORC_ERR_SIZE; }
        uint32_t c = orc_crc32(0, out + out_offsets[i], produced);
        if (c != spans[i].crc32) { set_err(err, ORC_ERR_CHECKSUM, spans[i].compressed_offset, spans[i].crc32, c, 0, "checksum mismatch"); return ORC_ERR_CHECKSUM; }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------------
 * BAM: header (crates/fritillaria-bam/src/columnar/header.rs:43-101)
 * ---------------------------------------------------------------------- */
int orc_bam_header(const uint8_t *buf, size_t len, uint64_t *records_start, int32_t *n_ref, orc_error *err)
{
    if (len < 12) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, 0, "truncated header"); return ORC_ERR_MALFORMED; }
    if (memcmp(buf, "BAM\1", 4) != 0) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, 0, "bad magic; expected BAM\\1"); return ORC_ERR_MALFORMED; }
    int32_t l_text = (int32_t)rd32(buf + 4);
    if (l_text < 0) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, 4, "negative l_text"); return ORC_ERR_MALFORMED; }
    uint64_t text_end = 8 + (uint64_t)l_text;
    if (text_end > len) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, 4, "l_text runs past the end of the buffer"); return ORC_ERR_MALFORMED; }
    if (text_end + 4 > len) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, text_end, "truncated n_ref"); return ORC_ERR_MALFORMED; }
    int32_t nr = (int32_t)rd32(buf + text_end);
    if (nr < 0) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, text_end, "negative n_ref"); return ORC_ERR_MALFORMED; }
    uint64_t pos = text_end + 4;
    for (int32_t i = 0; i < nr; ++i) {
        if (pos + 4 > len) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, pos, "truncated l_name"); return ORC_ERR_MALFORMED; }
        int32_t l_name = (int32_t)rd32(buf + pos);
        if (l_name < 0) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, pos, "negative l_name"); return ORC_ERR_MALFORMED; }
        pos += 4;
        if (pos + (uint64_t)l_name > len) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, pos, "truncated name"); return ORC_ERR_MALFORMED; }
        pos += (uint64_t)l_name;
        if (pos + 4 > len) { set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, pos, "truncated l_ref"); return ORC_ERR_MALFORMED; }
        pos += 4;
    }
    *records_start = pos;
    *n_ref = nr;
    return ORC_OK;
}

/* scan_records (crates/fritillaria-bam/src/columnar/record.rs:58-95) */
int orc_bam_scan(const uint8_t *buf, size_t len, uint64_t start, uint64_t *offsets, size_t cap,
                 size_t *n, uint64_t *tail, orc_error *err)
{
    uint64_t pos = start;
    size_t k = 0;
    for (;;) {
        if (pos + 4 > len || pos + 4 < pos) break;
        uint32_t bs = rd32(buf + pos);
        if (bs < 32) {
            set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, pos, "block_size smaller than the 32-byte core");
            *n = k; *tail = pos;
            return ORC_ERR_MALFORMED;
        }
        uint64_t end = pos + 4 + (uint64_t)bs;
        if (end > len) break;
        if (k < cap) offsets[k] = pos;
        ++k;
        pos = end;
    }
    *n = k;
    *tail = pos;
    return ORC_OK;
}

/* fields_fit (crates/fritillaria-bam/src/columnar/blocked.rs:106-131) */
static int fields_fit(const uint8_t *buf, size_t len, uint64_t start, uint64_t end)
{
    if (start + 24 > len) return 0;
    uint32_t name_len = buf[start + 12];
    if (name_len == 0) return 0;
    uint64_t n_cigar = rd16(buf + start + 16);
    uint64_t l_seq = rd32(buf + start + 20);
    uint64_t need = 36 + (uint64_t)name_len + 4 * n_cigar + (l_seq + 1) / 2 + l_seq;
    return start + need <= end;
}

typedef struct { uint64_t count, land; int complete, valid; } seg_t;

/* walk_segment (blocked.rs:139-179) */
static seg_t walk_segment(const uint8_t *buf, size_t len, uint64_t from, uint64_t until)
{
    seg_t s = {0, from, 1, 1};
    uint64_t cur = from;
    for (;;) {
        if (cur >= until) { s.land = cur; s.complete = 1; return s; }
        if (cur + 4 > len) { s.land = cur; s.complete = 0; return s; }
        uint32_t bs = rd32(buf + cur);
        if (bs < 32) { s.land = cur; s.valid = 0; return s; }
        uint64_t end = cur + 4 + (uint64_t)bs;
        if (end > len) { s.land = cur; s.complete = 0; return s; }
        if (!fields_fit(buf, len, cur, end)) { s.land = cur; s.valid = 0; return s; }
        s.count++;
        cur = end;
    }
}

/* scan_records_blocked (blocked.rs:193-282): speculate per block, reconcile
 * the true chain over blocks, emit.  This is the device path's semantics
 * (kernels/bam_decode.cu:132-245), including the fields_fit check. */
int orc_bam_scan_blocked(const uint8_t *buf, size_t len, const uint64_t *block_starts,
                         size_t n_blocks, uint64_t start, uint64_t *offsets, size_t cap,
                         size_t *n, uint64_t *tail_out, size_t *fallbacks_out, orc_error *err)
{
    if (n_blocks == 0 || block_starts[0] != 0 || block_starts[n_blocks] != len) {
        set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, 0, "block starts must span the buffer from 0 to its length");
        return ORC_ERR_MALFORMED;
    }
    uint64_t cur = start, tail = len;
    size_t emitted = 0, fallbacks = 0;
    int truncated = 0;
    for (size_t b = 0; b < n_blocks; ++b) {
        if (truncated || cur >= block_starts[b + 1]) continue;
        seg_t s;
        if (cur == block_starts[b]) {
            s = walk_segment(buf, len, block_starts[b], block_starts[b + 1]);
        } else {
            fallbacks++;
            s = walk_segment(buf, len, cur, block_starts[b + 1]);
        }
        if (!s.valid) {
            /* walk from a proven boundary: the record at s.land is corrupt */
            uint64_t p = cur;
            /* emit the valid prefix so callers can see what was proven */
            *n = emitted;
            *tail_out = cur;
            if (fallbacks_out) *fallbacks_out = fallbacks;
            (void)p;
            set_err(err, ORC_ERR_MALFORMED, 0, 0, 0, cur, "malformed record during boundary scan");
            return ORC_ERR_MALFORMED;
        }
        uint64_t r = cur;
        for (uint64_t i = 0; i < s.count; ++i) {
            if (emitted < cap) offsets[emitted] = r;
            emitted++;
            r += 4 + (uint64_t)rd32(buf + r);
        }
        cur = s.land;
        if (!s.complete) { tail = s.land; truncated = 1; }
    }
    if (!truncated) tail = cur;
    *n = emitted;
    *tail_out = tail;
    if (fallbacks_out) *fallbacks_out = fallbacks;
    return ORC_OK;
}

/* ------------------------------------------------------------------------
 * Aux tag walk: Fields / read_value / read_array
 * (crates/fritillaria-bam/src/columnar/aux.rs:301-479).  Returns 0 when the
 * block parses to its end, 1 when a field is malformed (the iterator fuses:
 * n_tags counts the fields before it).
 * ---------------------------------------------------------------------- */
int orc_bam_aux(const uint8_t *rec, uint32_t aux_start, uint32_t record_end, orc_aux_entry *out,
                uint32_t cap, uint32_t *n_tags)
{
    uint64_t pos = aux_start;
    uint64_t end = record_end;
    uint32_t k = 0;
    while (pos < end) {
        if (pos + 3 > end) { *n_tags = k; return 1; }
        uint8_t t0 = rec[pos], t1 = rec[pos + 1], ty = rec[pos + 2];
        uint64_t v = pos + 3;
        uint64_t next;
        uint8_t sub = 0;
        uint32_t count = 1;
        switch (ty) {
        case 'A': case 'c': case 'C':
            if (v + 1 > end) { *n_tags = k; return 1; }
            next = v + 1; break;
        case 's': case 'S':
            if (v + 2 > end) { *n_tags = k; return 1; }
            next = v + 2; break;
        case 'i': case 'I': case 'f':
            if (v + 4 > end) { *n_tags = k; return 1; }
            next = v + 4; break;
        case 'Z': case 'H': {
            uint64_t q = v;
            while (q < end && rec[q] != 0) ++q;
            if (q >= end) { *n_tags = k; return 1; }
            count = (uint32_t)(q - v);
            if (ty == 'H') {
                if (count % 2 != 0) { *n_tags = k; return 1; }
                for (uint64_t h = v; h < q; ++h) {
                    uint8_t c = rec[h];
                    int hex = (c >= '0' && c <= '9') || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F');
                    if (!hex) { *n_tags = k; return 1; }
                }
            }
            next = q + 1;
            break;
        }
        case 'B': {
            if (v + 1 > end) { *n_tags = k; return 1; }
            sub = rec[v];
            if (v + 5 > end) { *n_tags = k; return 1; }
            count = rd32(rec + v + 1);
            uint64_t w;
            switch (sub) {
            case 'c': case 'C': w = 1; break;
            case 's': case 'S': w = 2; break;
            case 'i': case 'I': case 'f': w = 4; break;
            default: *n_tags = k; return 1;
            }
            uint64_t bytes = (uint64_t)count * w;
            if (v + 5 + bytes > end) { *n_tags = k; return 1; }
            next = v + 5 + bytes;
            break;
        }
        default:
            *n_tags = k;
            return 1;
        }
        if (k < cap && out) {
            out[k].tag[0] = t0;
            out[k].tag[1] = t1;
            out[k].type = ty;
            out[k].subtype = sub;
            out[k].value_offset = (uint32_t)v;
            out[k].count = count;
        }
        ++k;
        pos = next;
    }
    *n_tags = k;
    return 0;
}

/* RecordBatch::decode field extraction (crates/fritillaria-bam/src/columnar/batch.rs:165-177,
 * record.rs:121-231) and the field bounds of kernels/bam_decode.cu:254-291. */
void orc_bam_decode(const uint8_t *buf, const uint64_t *offsets, size_t n, const orc_bam_columns *c)
{
    for (size_t i = 0; i < n; ++i) {
        const uint8_t *r = buf + offsets[i];
        uint32_t bs = rd32(r);
        uint32_t name_len = r[12];
        uint32_t n_cigar = rd16(r + 16);
        uint32_t l_seq = rd32(r + 20);
        if (c->ref_id) c->ref_id[i] = (int32_t)rd32(r + 4);
        if (c->pos) c->pos[i] = (int32_t)rd32(r + 8);
        if (c->name_len) c->name_len[i] = (uint8_t)name_len;
        if (c->mapq) c->mapq[i] = r[13];
        if (c->bin) c->bin[i] = (uint16_t)rd16(r + 14);
        if (c->n_cigar) c->n_cigar[i] = (uint16_t)n_cigar;
        if (c->flags) c->flags[i] = (uint16_t)rd16(r + 18);
        if (c->seq_len) c->seq_len[i] = l_seq;
        if (c->mate_ref_id) c->mate_ref_id[i] = (int32_t)rd32(r + 24);
        if (c->mate_pos) c->mate_pos[i] = (int32_t)rd32(r + 28);
        if (c->tlen) c->tlen[i] = (int32_t)rd32(r + 32);
        uint32_t cs = 36 + name_len;
        uint32_t ss = cs + 4 * n_cigar;
        uint32_t qs = ss + (l_seq + 1) / 2;
        uint32_t as = qs + l_seq;
        if (c->cigar_start) c->cigar_start[i] = cs;
        if (c->sequence_start) c->sequence_start[i] = ss;
        if (c->quality_start) c->quality_start[i] = qs;
        if (c->aux_start) c->aux_start[i] = as;
        if (c->record_end) c->record_end[i] = 4 + bs;
        if (c->aux_count || c->aux_status) {
            uint32_t nt = 0;
            int st = orc_bam_aux(r, as, 4 + bs, NULL, 0, &nt);
            if (as > 4 + bs) { nt = 0; st = 1; }
            if (c->aux_count) c->aux_count[i] = nt;
            if (c->aux_status) c->aux_status[i] = (uint8_t)st;
        }
    }
}

/* ------------------------------------------------------------------------
 * CPU baseline.  A restatement of the noodles multithreaded BGZF reader
 * (crates/fritillaria-bgzf/src/io/multithreaded_reader.rs:141-200: blocks
 * inflated by a pool of workers, each frame parsed, inflated and CRC-checked
 * as in io/reader/frame.rs:103-156) feeding the serial record scan and
 * column decode (columnar/record.rs:58, batch.rs:165) plus the aux walk.
 * Workers and the consumer are pipelined: the consumer walks records as the
 * members covering them complete.
 * ---------------------------------------------------------------------- */
typedef struct {
    const uint8_t *file;
    const orc_span *spans;
    const uint64_t *out_off;
    uint8_t *out;
    size_t n;
    atomic_size_t next;
    atomic_uchar *done;
    atomic_int failed;
} bl_ctx;

static void *bl_worker(void *arg)
{
    bl_ctx *c = (bl_ctx *)arg;
    for (;;) {
        size_t i = atomic_fetch_add(&c->next, 1);
        if (i >= c->n) break;
        size_t produced = 0;
        const orc_span *s = &c->spans[i];
        int rc = orc_inflate_raw(c->file + s->payload_start, s->payload_len, c->out + c->out_off[i], s->isize, &produced);
        if (rc || produced != s->isize || crc32(0, c->out + c->out_off[i], (uInt)produced) != s->crc32)
            atomic_store(&c->failed, 1);
        atomic_store_explicit(&c->done[i], 1, memory_order_release);
    }
    return NULL;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

int orc_baseline_bam(const uint8_t *file, size_t len, int threads, uint64_t max_members, orc_baseline_result *res)
{
    memset(res, 0, sizeof *res);
    double t0 = now_s();
    size_t cap = len / 28 + 1;
    orc_span *spans = (orc_span *)malloc(cap * sizeof *spans);
    size_t n = 0, consumed = 0;
    orc_error err;
    if (orc_bgzf_discover(file, len, 0, spans, cap, &n, &consumed, &err)) { free(spans); res->status = err.code; return err.code; }
    if (max_members && n > max_members) n = (size_t)max_members;
    uint64_t *out_off = (uint64_t *)malloc((n + 1) * sizeof *out_off);
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) { out_off[i] = total; total += spans[i].isize; }
    out_off[n] = total;
    uint8_t *out = (uint8_t *)malloc(total + 1);
    bl_ctx ctx;
    ctx.file = file; ctx.spans = spans; ctx.out_off = out_off; ctx.out = out; ctx.n = n;
    atomic_init(&ctx.next, 0);
    atomic_init(&ctx.failed, 0);
    ctx.done = (atomic_uchar *)calloc(n + 1, 1);
    if (threads < 1) threads = 1;
    pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (int t = 0; t < threads; ++t) pthread_create(&tids[t], NULL, bl_worker, &ctx);

    /* consumer: header, then records in order as their members complete */
    size_t ready = 0; /* members [0, ready) are complete */
    uint64_t ready_bytes = 0;
#define WAIT_UNTIL(bytes)                                                                         \
    while (ready_bytes < (bytes) && ready < n) {                                                  \
        while (!atomic_load_explicit(&ctx.done[ready], memory_order_acquire)) sched_yield();      \
        ready_bytes = out_off[ready + 1];                                                         \
        ready++;                                                                                  \
    }
    WAIT_UNTIL(total < 65536 ? total : 65536);
    uint64_t pos = 0;
    int32_t nref = 0;
    uint64_t records = 0, tags = 0, checksum = 0;
    int status = 0;
    /* the header can exceed one member: grow the wait until it parses */
    for (;;) {
        if (orc_bam_header(out, ready_bytes, &pos, &nref, &err) == ORC_OK) break;
        if (ready >= n) { status = ORC_ERR_MALFORMED; break; }
        WAIT_UNTIL(ready_bytes + 1);
    }
    while (!status) {
        WAIT_UNTIL(pos + 4);
        if (pos + 4 > ready_bytes) break;
        uint32_t bs = rd32(out + pos);
        if (bs < 32) { status = ORC_ERR_MALFORMED; break; }
        uint64_t end = pos + 4 + (uint64_t)bs;
        WAIT_UNTIL(end);
        if (end > ready_bytes) break;
        const uint8_t *r = out + pos;
        uint32_t name_len = r[12], n_cigar = rd16(r + 16), l_seq = rd32(r + 20);
        int32_t refid = (int32_t)rd32(r + 4), p = (int32_t)rd32(r + 8);
        uint16_t flag = (uint16_t)rd16(r + 18);
        uint32_t as = 36 + name_len + 4 * n_cigar + (l_seq + 1) / 2 + l_seq;
        uint32_t nt = 0;
        orc_bam_aux(r, as, 4 + bs, NULL, 0, &nt);
        tags += nt;
        checksum += (uint64_t)(uint32_t)refid * 31u + (uint64_t)(uint32_t)p * 7u + flag + l_seq + r[13];
        records++;
        pos = end;
    }
#undef WAIT_UNTIL
    for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
    res->seconds = now_s() - t0;
    if (atomic_load(&ctx.failed)) status = ORC_ERR_CHECKSUM;
    res->members = n;
    res->inflated_bytes = total;
    res->records = records;
    res->aux_tags = tags;
    res->checksum = checksum;
    res->status = status;
    free(tids);
    free((void *)ctx.done);
    free(out);
    free(out_off);
    free(spans);
    return status;
}


/* CPU baseline for the other formats on the container: the same
 * multithreaded inflate (every member inflated and CRC-checked by the worker
 * pool), then the reference's serial CPU scan and decode of the whole file:
 *   FASTQ  scan_records + bounds (fastq record.rs:158-200, batch.rs);
 *   BCF    the length-prefix chain + Record::bounds (bcf batch.rs:222-241);
 *   FASTA  scan_records(at_eof) + compact_into (fasta record.rs:180-330).
 * format: 1 BCF, 2 FASTQ, 3 FASTA (frt_format numbering). */
int orc_baseline_file(const uint8_t *file, size_t len, int format, int threads, orc_baseline_result *res)
{
    memset(res, 0, sizeof *res);
    double t0 = now_s();
    size_t cap = len / 28 + 1;
    orc_span *spans = (orc_span *)malloc(cap * sizeof *spans);
    size_t n = 0, consumed = 0;
    orc_error err;
    if (orc_bgzf_discover(file, len, 0, spans, cap, &n, &consumed, &err)) { free(spans); res->status = err.code; return err.code; }
    uint64_t *out_off = (uint64_t *)malloc((n + 1) * sizeof *out_off);
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) { out_off[i] = total; total += spans[i].isize; }
    out_off[n] = total;
    uint8_t *out = (uint8_t *)malloc(total + 1);
    bl_ctx ctx;
    ctx.file = file; ctx.spans = spans; ctx.out_off = out_off; ctx.out = out; ctx.n = n;
    atomic_init(&ctx.next, 0);
    atomic_init(&ctx.failed, 0);
    ctx.done = (atomic_uchar *)calloc(n + 1, 1);
    if (threads < 1) threads = 1;
    pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (int t = 0; t < threads; ++t) pthread_create(&tids[t], NULL, bl_worker, &ctx);
    for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
    int status = atomic_load(&ctx.failed) ? ORC_ERR_CHECKSUM : ORC_OK;
    uint64_t records = 0, checksum = 0;
    if (!status && format == 2) {
        uint64_t pos = 0;
        orc_fastq_bounds b;
        while (pos < total) {
            if (out[pos] == '\n') { ++pos; continue; }
            if (!orc_fastq_bounds_at(out, total, pos, &b)) break;
            checksum += b.sequence_len * 7u + b.quality_start;
            ++records;
            pos += b.record_end;
        }
    } else if (!status && format == 1) {
        uint64_t start;
        uint32_t samples, contigs;
        if (orc_bcf_header(out, total, &start, &samples, &contigs, &err)) {
            status = err.code;
        } else {
            uint64_t pos = start;
            int32_t chrom, posv, rlen;
            uint32_t qual, ns, a, f, inf, g, e;
            uint16_t ni, na;
            uint8_t nf;
            orc_bcf_columns c = {&chrom, &posv, &rlen, &qual, &ni, &na, &ns, &nf, &a, &f, &inf, &g, &e};
            while (pos + 8 <= total) {
                uint64_t ls = rd32(out + pos), li = rd32(out + pos + 4);
                if (ls < 24 || pos + 8 + ls + li > total) break;
                if (orc_bcf_decode(out, total, &pos, 1, &c)) { status = ORC_ERR_MALFORMED; break; }
                checksum += (uint64_t)(uint32_t)posv * 3u + a + f + inf;
                ++records;
                pos += 8 + ls + li;
            }
        }
    } else if (!status && format == 3) {
        size_t cap2 = total / 2 + 1, nc = 0;
        uint64_t *so = (uint64_t *)malloc(3 * cap2 * sizeof(uint64_t));
        uint64_t bases = 0;
        uint8_t *seq = (uint8_t *)malloc(total + 1);
        if (orc_fasta_compact(out, total, seq, total + 1, so, so + cap2, so + 2 * cap2, NULL, cap2, &nc, &bases))
            status = ORC_ERR_MALFORMED;
        records = nc;
        checksum = bases;
        free(seq);
        free(so);
    }
    res->seconds = now_s() - t0;
    res->members = n;
    res->inflated_bytes = total;
    res->records = records;
    res->checksum = checksum;
    res->status = status;
    free(tids);
    free((void *)ctx.done);
    free(out);
    free(out_off);
    free(spans);
    return status;
}


/* Every member of a BGZF file inflated and CRC/ISIZE-checked by the worker
 * pool of orc_baseline_bam, into `out` at the ISIZE prefix sum.  Returns
 * ORC_ERR_INVALID_ARGUMENT (with *total set) when out_cap is short. */
int orc_inflate_file(const uint8_t *file, size_t len, int threads, uint8_t *out, uint64_t out_cap, uint64_t *members,
                     uint64_t *total_out)
{
    size_t cap = len / 28 + 1;
    orc_span *spans = (orc_span *)malloc(cap * sizeof *spans);
    size_t n = 0, consumed = 0;
    orc_error err;
    *members = 0;
    *total_out = 0;
    if (orc_bgzf_discover(file, len, 0, spans, cap, &n, &consumed, &err)) { free(spans); return err.code; }
    uint64_t *out_off = (uint64_t *)malloc((n + 1) * sizeof *out_off);
    uint64_t total = 0;
    for (size_t i = 0; i < n; ++i) { out_off[i] = total; total += spans[i].isize; }
    out_off[n] = total;
    *members = n;
    *total_out = total;
    int status = total > out_cap ? ORC_ERR_INVALID_ARGUMENT : ORC_OK;
    if (!status) {
        bl_ctx ctx;
        ctx.file = file; ctx.spans = spans; ctx.out_off = out_off; ctx.out = out; ctx.n = n;
        atomic_init(&ctx.next, 0);
        atomic_init(&ctx.failed, 0);
        ctx.done = (atomic_uchar *)calloc(n + 1, 1);
        if (threads < 1) threads = 1;
        pthread_t *tids = (pthread_t *)malloc(sizeof(pthread_t) * threads);
        for (int t = 0; t < threads; ++t) pthread_create(&tids[t], NULL, bl_worker, &ctx);
        for (int t = 0; t < threads; ++t) pthread_join(tids[t], NULL);
        if (atomic_load(&ctx.failed)) status = ORC_ERR_CHECKSUM;
        free(tids);
        free((void *)ctx.done);
    }
    free(out_off);
    free(spans);
    return status;
}

/* Parity at scale: the whole BAM file as the oracle decodes it, so that a
 * device run over the same file can be compared column for column.  Members
 * are inflated and CRC/ISIZE-checked by the worker pool of orc_baseline_bam;
 * then the header (header.rs:43-101), the serial scan (record.rs:58-95), the
 * columns (batch.rs:165-177), each record's virtual offset (member compressed
 * offset << 16 | in-member offset, virtual_offset.rs:24-70) and its aux
 * directory (aux.rs:301-479, entries up to the first malformed field;
 * aux_first holds records + 1 prefix entries).  A capacity that is too small
 * returns ORC_ERR_INVALID_ARGUMENT with the sizes needed in res. */
int orc_bam_file_decode(const uint8_t *file, size_t len, int threads, uint8_t *inflated, uint64_t inflated_cap,
                        uint64_t *record_offsets, uint64_t *virtual_offsets, const orc_bam_columns *cols,
                        uint32_t *aux_first, orc_aux_entry *aux, uint64_t rec_cap, uint64_t aux_cap,
                        orc_file_decode *res)
{
    memset(res, 0, sizeof *res);
    uint64_t total = 0, n_members = 0;
    int status = orc_inflate_file(file, len, threads, inflated, inflated_cap, &n_members, &total);
    res->members = n_members;
    res->inflated_bytes = total;
    /* the spans again, for the virtual offsets (discovery succeeded above) */
    size_t cap = len / 28 + 1;
    orc_span *spans = (orc_span *)malloc(cap * sizeof *spans);
    size_t n = 0, consumed = 0;
    orc_error err;
    if (!status) orc_bgzf_discover(file, len, 0, spans, cap, &n, &consumed, &err);
    uint64_t *out_off = (uint64_t *)malloc((n + 1) * sizeof *out_off);
    uint64_t at = 0;
    for (size_t i = 0; i < n; ++i) { out_off[i] = at; at += spans[i].isize; }
    out_off[n] = at;
    uint64_t start = 0;
    int32_t nref = 0;
    if (!status) status = orc_bam_header(inflated, total, &start, &nref, &err);
    size_t nrec = 0;
    uint64_t tail = 0;
    if (!status) status = orc_bam_scan(inflated, total, start, record_offsets, rec_cap, &nrec, &tail, &err);
    res->records_start = start;
    res->n_ref = nref;
    res->records = nrec;
    res->tail = tail;
    if (!status && nrec > rec_cap) status = ORC_ERR_INVALID_ARGUMENT;
    if (!status) {
        orc_bam_decode(inflated, record_offsets, nrec, cols);
        size_t m = 0;
        uint64_t k = 0;
        for (size_t i = 0; i < nrec; ++i) {
            uint64_t ro = record_offsets[i];
            while (m + 1 < n && out_off[m + 1] <= ro) ++m;
            virtual_offsets[i] = (spans[m].compressed_offset << 16) | (ro - out_off[m]);
            const uint8_t *r = inflated + ro;
            uint32_t bs = rd32(r);
            uint32_t as = cols->aux_start[i];
            uint32_t nt = 0;
            aux_first[i] = (uint32_t)k;
            if (as <= 4 + bs) {
                orc_bam_aux(r, as, 4 + bs, k < aux_cap ? aux + k : NULL, k < aux_cap ? (uint32_t)(aux_cap - k) : 0, &nt);
            }
            k += nt;
        }
        aux_first[nrec] = (uint32_t)k;
        res->aux_entries = k;
        if (k > aux_cap) status = ORC_ERR_INVALID_ARGUMENT;
    }
    res->status = status;
    free(out_off);
    free(spans);
    return status;
}


/* The reference's indexed query over one chunk, on the host: records of the
 * chain from `start` that begin before `chunk_end` (offsets in the inflated
 * chunk), kept when on reference `ref` their [pos + 1, pos + span] meets
 * [beg, end] (crates/fritillaria-bam/src/io/reader/query.rs:97-122; span from
 * the CIGAR's M/D/N/=/X, at least 1).  Writes kept record offsets; returns
 * their count. */
uint64_t orc_region_records(const uint8_t *buf, uint64_t len, uint64_t start, uint64_t chunk_end, int32_t ref,
                            uint64_t beg, uint64_t end, uint64_t *out, uint64_t cap)
{
    uint64_t pos = start, n = 0;
    while (pos < chunk_end && pos + 4 <= len) {
        uint32_t bs = rd32(buf + pos);
        if (bs < 32 || pos + 4 + (uint64_t)bs > len) break;
        const uint8_t *r = buf + pos;
        int32_t rid = (int32_t)rd32(r + 4), p = (int32_t)rd32(r + 8);
        if (rid == ref && p >= 0) {
            uint32_t name_len = r[12], n_cigar = rd16(r + 16);
            uint64_t span = 0;
            for (uint32_t k = 0; k < n_cigar; ++k) {
                uint32_t op = rd32(r + 36 + name_len + 4 * k), kind = op & 15u;
                if (kind == 0 || kind == 2 || kind == 3 || kind == 7 || kind == 8) span += op >> 4;
            }
            if (!span) span = 1;
            uint64_t a0 = (uint64_t)p + 1, a1 = a0 + span - 1;
            if (a0 <= end && beg <= a1) {
                if (n < cap) out[n] = pos;
                ++n;
            }
        }
        pos += 4 + (uint64_t)bs;
    }
    return n;
}
