/*
 * TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU path for BGZF -> inflate ->
 * CRC/ISIZE verify -> BAM record scan -> columns, used as the oracle for the
 * CUDA implementation in fritillaria_gb300.  Only tests, the smoke entry point
 * and the CPU-baseline leg of the benchmark may load it; the product never
 * calls into it.
 *
 * Raw DEFLATE is delegated to zlib 1.3 (raw, windowBits -15): DEFLATE output is
 * uniquely determined by the bitstream, so zlib is an independent oracle for
 * miniz_oxide 0.9.1 / zlib-rs 0.6.7, which the reference links
 * (crates/fritillaria-bgzf/src/cpu.rs:39-69, crates/fritillaria-bgzf/src/deflate.rs:15-33).
 */
#ifndef FRT_ORACLE_H
#define FRT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same numbering as frt_status in include/frt.h (the Error variants of
 * crates/fritillaria-core/src/error.rs:14-67). */
enum {
    ORC_OK = 0,
    ORC_ERR_IO = 1,
    ORC_ERR_INVALID_BLOCK = 2,
    ORC_ERR_CHECKSUM = 3,
    ORC_ERR_SIZE = 4,
    ORC_ERR_INFLATE = 5,
    ORC_ERR_MALFORMED = 6,
    ORC_ERR_INVALID_DEVICE_BATCH = 7,
    ORC_ERR_INVALID_ARGUMENT = 10,
};

typedef struct {
    int32_t code;
    uint64_t offset;   /* member compressed offset (block errors) */
    uint64_t expected; /* crc or isize */
    uint64_t actual;
    uint64_t position; /* Malformed position */
    char reason[128];
} orc_error;

/* crates/fritillaria-core/src/codec.rs:17-41 */
typedef struct {
    uint64_t compressed_offset;
    uint64_t payload_start;
    uint64_t payload_len;
    uint32_t isize;
    uint32_t crc32;
} orc_span;

/* One aux-directory entry (12 bytes); offsets relative to the record start. */
typedef struct {
    uint8_t tag[2];
    uint8_t type;
    uint8_t subtype;
    uint32_t value_offset;
    uint32_t count;
} orc_aux_entry;

uint32_t orc_crc32(uint32_t crc, const uint8_t *p, size_t n);
uint32_t orc_crc32_combine(uint32_t crc_a, uint32_t crc_b, uint64_t len_b);

int orc_bgzf_parse_header(const uint8_t *buf, size_t len, uint64_t offset, uint32_t *block_size,
                          uint32_t *header_size, orc_error *err);
int orc_bgzf_discover(const uint8_t *buf, size_t len, uint64_t base_offset, orc_span *spans,
                      size_t cap, size_t *n_spans, size_t *consumed, orc_error *err);

int orc_inflate_raw(const uint8_t *in, size_t in_len, uint8_t *out, size_t out_cap,
                    size_t *produced);
int orc_inflate_batch(const uint8_t *batch, size_t batch_len, const orc_span *spans, size_t n,
                      uint8_t *out, size_t out_cap, uint64_t *out_offsets, orc_error *err);

int orc_bam_header(const uint8_t *buf, size_t len, uint64_t *records_start, int32_t *n_ref,
                   orc_error *err);
int orc_bam_scan(const uint8_t *buf, size_t len, uint64_t start, uint64_t *offsets, size_t cap,
                 size_t *n, uint64_t *tail, orc_error *err);
int orc_bam_scan_blocked(const uint8_t *buf, size_t len, const uint64_t *block_starts,
                         size_t n_blocks, uint64_t start, uint64_t *offsets, size_t cap,
                         size_t *n, uint64_t *tail, size_t *fallbacks, orc_error *err);

typedef struct {
    int32_t *ref_id;
    int32_t *pos;
    uint16_t *flags;
    uint8_t *mapq;
    uint32_t *seq_len;
    int32_t *mate_ref_id;
    int32_t *mate_pos;
    int32_t *tlen;
    uint32_t *cigar_start;
    uint32_t *sequence_start;
    uint32_t *quality_start;
    uint32_t *aux_start;
    uint32_t *record_end;
    uint16_t *bin;
    uint16_t *n_cigar;
    uint8_t *name_len;
    uint32_t *aux_count;
    uint8_t *aux_status;
} orc_bam_columns;

void orc_bam_decode(const uint8_t *buf, const uint64_t *offsets, size_t n,
                    const orc_bam_columns *cols);
int orc_bam_aux(const uint8_t *rec, uint32_t aux_start, uint32_t record_end, orc_aux_entry *out,
                uint32_t cap, uint32_t *n_tags);

/* Multithreaded CPU baseline: reader + N inflate workers (zlib + crc check),
 * then the serial record scan, column decode and aux walk. */
typedef struct {
    uint64_t members;
    uint64_t inflated_bytes;
    uint64_t records;
    uint64_t aux_tags;
    uint64_t checksum;
    double seconds;
    int32_t status;
} orc_baseline_result;

int orc_baseline_bam(const uint8_t *file, size_t len, int threads, uint64_t max_members,
                     orc_baseline_result *res);
/* Every member of a BGZF file inflated and checked on `threads` host threads. */
int orc_inflate_file(const uint8_t *file, size_t len, int threads, uint8_t *out, uint64_t out_cap, uint64_t *members,
                     uint64_t *total);
/* The whole BAM file decoded by the oracle, for parity against a device run
 * at full size (see frt_oracle.c). */
typedef struct {
    uint64_t members;
    uint64_t inflated_bytes;
    uint64_t records;
    uint64_t aux_entries;
    uint64_t tail;
    uint64_t records_start;
    int32_t n_ref;
    int32_t status;
} orc_file_decode;

int orc_bam_file_decode(const uint8_t *file, size_t len, int threads, uint8_t *inflated, uint64_t inflated_cap,
                        uint64_t *record_offsets, uint64_t *virtual_offsets, const orc_bam_columns *cols,
                        uint32_t *aux_first, orc_aux_entry *aux, uint64_t rec_cap, uint64_t aux_cap,
                        orc_file_decode *res);
/* Records of one BAI chunk that a region query keeps (see frt_oracle.c). */
uint64_t orc_region_records(const uint8_t *buf, uint64_t len, uint64_t start, uint64_t chunk_end, int32_t ref,
                            uint64_t beg, uint64_t end, uint64_t *out, uint64_t cap);
/* The same for a bgzipped BCF (1), FASTQ (2) or FASTA (3) file. */
int orc_baseline_file(const uint8_t *file, size_t len, int format, int threads, orc_baseline_result *res);

/* ---- FASTQ, BCF, FASTA (frt_oracle_formats.c) ---------------------------- */

enum { ORC_PROOF_TILED = 0, ORC_PROOF_WALKED = 1 };

typedef struct {
    uint32_t sequence_start, plus_start, quality_start, sequence_len, record_end;
} orc_fastq_bounds;

int orc_fastq_bounds_at(const uint8_t *buf, uint64_t len, uint64_t pos, orc_fastq_bounds *b);
int orc_fastq_scan(const uint8_t *buf, uint64_t len, uint64_t start, uint64_t *offsets, size_t cap,
                   size_t *n, uint64_t *tail, uint64_t *survivors, int *proof);
int orc_fastq_decode(const uint8_t *buf, uint64_t len, const uint64_t *offsets, size_t n,
                     uint32_t *sequence_start, uint32_t *plus_start, uint32_t *quality_start,
                     uint32_t *sequence_len, uint32_t *record_end);

typedef struct {
    int32_t *chromosome_id;
    int32_t *position;
    int32_t *reference_span;
    uint32_t *quality;
    uint16_t *info_count;
    uint16_t *allele_count;
    uint32_t *sample_count;
    uint8_t *format_count;
    uint32_t *alleles_start;
    uint32_t *filters_start;
    uint32_t *info_start;
    uint32_t *genotypes_start;
    uint32_t *record_end;
} orc_bcf_columns;

int orc_bcf_header(const uint8_t *buf, uint64_t len, uint64_t *records_start, uint32_t *samples,
                   uint32_t *contigs, orc_error *err);
int orc_bcf_looks_like_a_record(const uint8_t *buf, uint64_t len, uint64_t pos, uint32_t samples,
                                uint32_t contigs);
int orc_bcf_validate(const uint8_t *buf, uint64_t len, uint64_t pos);
int orc_bcf_scan(const uint8_t *buf, uint64_t len, uint64_t start, uint32_t samples, uint32_t contigs,
                 uint64_t *offsets, size_t cap, size_t *n, uint64_t *tail, uint64_t *sieved,
                 uint64_t *validated, int *proof);
int orc_bcf_decode(const uint8_t *buf, uint64_t len, const uint64_t *offsets, size_t n,
                   const orc_bcf_columns *cols);

typedef struct {
    uint32_t sequence_start;
    uint32_t line_bases;
    uint32_t line_width;
    uint8_t uniform;
    uint64_t sequence_len;
    uint64_t record_end;
} orc_fasta_bounds;

int orc_fasta_bounds_at(const uint8_t *buf, uint64_t len, uint64_t pos, orc_fasta_bounds *b);
int orc_fasta_compact(const uint8_t *buf, uint64_t len, uint8_t *seq, uint64_t seq_cap,
                      uint64_t *seq_offsets, uint64_t *seq_lengths, uint64_t *record_offsets,
                      orc_fasta_bounds *bounds, size_t cap, size_t *n, uint64_t *total);

#ifdef __cplusplus
}
#endif
#endif
