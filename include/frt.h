/*
 * frt.h -- C ABI of the GB300 BGZF -> device-columns library.
 *
 * The entry points mirror the reference's Rust surface for this path so that a
 * Rust host (through build.rs + an `extern "C"` block) or any other FFI caller
 * can use it as a drop-in.  Each declaration names the reference item it
 * replaces (paths relative to the fritillaria workspace).
 *
 * Conventions
 *   - Every fallible call returns an frt_status and, when `err` is non-null,
 *     fills it; FRT_OK is 0.  Error codes mirror the variants of
 *     crates/fritillaria-core/src/error.rs:14-67; `offset` is the member's
 *     absolute compressed offset, as there.
 *   - Handles are opaque and caller-freed.  A record batch holds a reference
 *     to the inflate batch its columns point into, so freeing the inflate batch
 *     first cannot free the bytes under the columns
 *     (crates/fritillaria-bam/src/columnar/device.rs:39-42).
 *   - Device pointers are plain `void *`/`uint8_t *` in the current CUDA
 *     context; streams and events are passed as `void *` (cudaStream_t /
 *     cudaEvent_t).
 *   - There is no CPU fallback: without a usable GB300 every codec constructor
 *     returns FRT_ERR_CUDA_UNAVAILABLE.
 */
#ifndef FRT_H
#define FRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FRT_OK = 0,
    FRT_ERR_IO = 1,                   /* Error::Io */
    FRT_ERR_INVALID_BLOCK = 2,        /* Error::InvalidBlock{offset, reason} */
    FRT_ERR_CHECKSUM = 3,             /* Error::ChecksumMismatch{offset, expected, actual} */
    FRT_ERR_SIZE = 4,                 /* Error::SizeMismatch{offset, expected, actual} */
    FRT_ERR_INFLATE = 5,              /* Error::Inflate{offset, reason} */
    FRT_ERR_MALFORMED = 6,            /* Error::Malformed{format, position, reason} */
    FRT_ERR_INVALID_DEVICE_BATCH = 7, /* Error::InvalidDeviceBatch{reason} */
    FRT_ERR_CUDA_UNAVAILABLE = 8,     /* Error::CudaUnavailable */
    FRT_ERR_CUDA = 9,                 /* Error::Cuda */
    FRT_ERR_INVALID_ARGUMENT = 10
} frt_status;

typedef struct {
    int32_t code;      /* frt_status */
    uint64_t offset;   /* member compressed offset (block errors) */
    uint64_t expected; /* CRC32 or ISIZE */
    uint64_t actual;
    uint64_t position; /* Malformed: byte position in the inflated batch */
    char format[16];   /* Malformed: "bam", "bgzf", "bcf", "fastq" ... */
    char reason[200];
} frt_error;

/* BlockSpan, crates/fritillaria-core/src/codec.rs:17-41. */
typedef struct {
    uint64_t compressed_offset;
    uint64_t payload_start;
    uint64_t payload_len;
    uint32_t isize;
    uint32_t crc32;
} frt_span;

typedef struct frt_codec frt_codec;
typedef struct frt_inflate_batch frt_inflate_batch;
typedef struct frt_reader frt_reader;
typedef struct frt_bam_decoder frt_bam_decoder;
typedef struct frt_record_batch frt_record_batch;

/* Backend, crates/fritillaria/src/lib.rs:151-176. */
typedef enum { FRT_BACKEND_AUTO = 0, FRT_BACKEND_CPU = 1, FRT_BACKEND_CUDA = 2, FRT_BACKEND_NVCOMP = 3 } frt_backend;

/* ---- device and selection ---------------------------------------------- */

/* cuda_is_usable, crates/fritillaria/src/lib.rs:183-186. */
int frt_cuda_is_usable(void);

/* select_codec, crates/fritillaria/src/lib.rs:242-260.  Auto and Cuda resolve
 * to this library's GB300 codec or fail with FRT_ERR_CUDA_UNAVAILABLE; Nvcomp
 * fails with FRT_ERR_CUDA_UNAVAILABLE (no nvCOMP path); Cpu fails with
 * FRT_ERR_INVALID_ARGUMENT (the CPU codec is not part of this library). */
int frt_select_codec(int backend, frt_codec **out, int *resolved, frt_error *err);

/* ---- codec: CudaCodec as BlockCodec / DeviceBlockCodec ------------------ */

/* CudaCodec::new / with_context(ctx, stream), crates/fritillaria-cuda/src/lib.rs:170-213.
 * `stream` may be NULL (the codec creates its own) or a cudaStream_t on
 * `device` owned by the caller.  Allocations and launches happen in the
 * device's primary context (the one cudarc's CudaContext::new retains); a
 * caller's stream must belong to that context. */
int frt_codec_create(int device, void *stream, frt_codec **out, frt_error *err);
void frt_codec_destroy(frt_codec *codec);
/* DeviceBlockCodec::name / device_ordinal, crates/fritillaria-core/src/device.rs:306-324. */
const char *frt_codec_name(const frt_codec *codec);
int frt_codec_device_ordinal(const frt_codec *codec);
void *frt_codec_stream(const frt_codec *codec);

/* DeviceBlockCodec::inflate_batch_device, crates/fritillaria-core/src/device.rs:316-324,
 * implemented by CudaCodec (crates/fritillaria-cuda/src/lib.rs:276-293).
 * `batch` is host memory holding the compressed window; spans index it.
 * CRC32 and ISIZE are verified; on failure *out is left untouched. */
int frt_codec_inflate_batch_device(frt_codec *codec, const uint8_t *batch, size_t batch_len,
                                   const frt_span *spans, size_t n_spans, frt_inflate_batch **out,
                                   frt_error *err);

/* BlockCodec::inflate_batch, crates/fritillaria-core/src/codec.rs:159-173: the
 * same inflate with the bytes copied back.  `out` receives sum(ISIZE) bytes,
 * `out_offsets` n_spans + 1 entries. */
int frt_codec_inflate_batch_host(frt_codec *codec, const uint8_t *batch, size_t batch_len,
                                 const frt_span *spans, size_t n_spans, uint8_t *out, size_t out_cap,
                                 uint64_t *out_offsets, frt_error *err);

/* crc32_blocks, crates/fritillaria-cuda/kernels/crc32.cu:13-38: CRC32 of
 * device-resident members (`data` device pointer). */
int frt_codec_crc32_device(frt_codec *codec, const uint8_t *data, const uint64_t *offsets,
                           const uint32_t *lengths, size_t n, uint32_t *crcs_host, frt_error *err);

/* ---- DeviceInflateBatch, crates/fritillaria-core/src/device.rs:145-287 --- */

size_t frt_inflate_batch_len(const frt_inflate_batch *b);          /* members */
size_t frt_inflate_batch_byte_len(const frt_inflate_batch *b);     /* inflated bytes */
const uint8_t *frt_inflate_batch_data(const frt_inflate_batch *b); /* device pointer */
const uint64_t *frt_inflate_batch_offsets(const frt_inflate_batch *b); /* host, len + 1 */
const uint64_t *frt_inflate_batch_compressed_offsets(const frt_inflate_batch *b); /* host, len */
int frt_inflate_batch_device_ordinal(const frt_inflate_batch *b);
/* CudaCodec::ready_event, crates/fritillaria-cuda/src/lib.rs:215-225. */
void *frt_inflate_batch_ready_event(const frt_inflate_batch *b);
/* DeviceInflateBatch::to_host, device.rs:276-287. */
int frt_inflate_batch_to_host(const frt_inflate_batch *b, uint8_t *dst, size_t cap, frt_error *err);
void frt_inflate_batch_free(frt_inflate_batch *b);

/* ---- DeviceBgzfReader, crates/fritillaria-bgzf/src/device_read.rs:57-280 -- */

/* A byte source: returns bytes read (0 at end of stream) or -1 on error. */
typedef int64_t (*frt_read_fn)(void *ctx, uint8_t *buf, size_t cap);

/* DeviceBgzfReader::new(inner, codec).  The codec must outlive the reader. */
int frt_reader_open(frt_read_fn read, void *ctx, frt_codec *codec, frt_reader **out, frt_error *err);
/* Convenience sources: a caller-owned memory range, or a file path. */
int frt_reader_open_memory(const uint8_t *data, size_t len, frt_codec *codec, frt_reader **out, frt_error *err);
int frt_reader_open_path(const char *path, frt_codec *codec, frt_reader **out, frt_error *err);
/* with_blocks_per_batch (device_read.rs:113-116): a floor on the compressed
 * budget, blocks x 64 KiB; values below 1 become 1. */
void frt_reader_set_blocks_per_batch(frt_reader *r, size_t blocks);
/* next_batch (device_read.rs:188-280).  *has_batch = 0 at end of stream.
 * *start is DeviceBatch::start. */
int frt_reader_next_batch(frt_reader *r, frt_inflate_batch **out, uint64_t *start, int *has_batch,
                          frt_error *err);
/* carry_from (device_read.rs:155-182). */
int frt_reader_carry_from(frt_reader *r, uint64_t tail, frt_error *err);
const char *frt_reader_codec_name(const frt_reader *r);
int frt_reader_device_ordinal(const frt_reader *r);
void frt_reader_close(frt_reader *r);

/* ---- host BGZF framing, crates/fritillaria-bgzf/src/discover.rs:51-109 ---- */
int frt_bgzf_discover(const uint8_t *buf, size_t len, uint64_t base_offset, frt_span *spans, size_t cap,
                      size_t *n_spans, size_t *consumed, frt_error *err);

/* ---- BAM header, crates/fritillaria-bam/src/columnar/header.rs:43-101 ------
 * Host parse of the header at the start of the first batch: where records
 * begin and how many references there are. */
int frt_bam_parse_header(const uint8_t *buf, size_t len, uint64_t *records_start, int32_t *n_ref, frt_error *err);

/* ---- BamDecoder, crates/fritillaria-cuda/src/bam.rs:113-187 --------------- */

int frt_bam_decoder_create(int device, void *stream, frt_bam_decoder **out, frt_error *err);
/* Bounds refID/next_refID in the boundary validator; -1 (default) means
 * unknown.  Only a hint: results never depend on it. */
void frt_bam_decoder_set_reference_count(frt_bam_decoder *d, int32_t n_ref);
void frt_bam_decoder_destroy(frt_bam_decoder *d);
/* BamDecoder::decode(batch, start) -> DeviceRecordBatch. */
int frt_bam_decode(frt_bam_decoder *d, const frt_inflate_batch *batch, uint64_t start, frt_record_batch **out,
                   frt_error *err);
/* Speculation fallbacks of the last decode (BlockedScan::fallbacks, blocked.rs:80-88). */
uint64_t frt_bam_decoder_last_fallbacks(const frt_bam_decoder *d);

/* Record boundaries without allocating.  No counterpart in the reference: it
 * exists for callers that cannot let a library allocate device memory (a host
 * that owns all device memory through its own arena, code that must not
 * allocate inside a capture or under a fixed budget, pipelines that
 * preallocate once).  The caller passes the inflated bytes (`data`, `len`),
 * the n_members + 1 member start offsets (device), and `record_offsets`
 * (device, room for `record_cap` entries; null only with record_cap 0, which
 * counts the records); the scan's scratch is a fixed device array of the
 * library, so at most FRT_NOALLOC_MAX_MEMBERS members per call (larger
 * batches are rejected with FRT_ERR_INVALID_ARGUMENT), each of at most
 * 65,536 inflated bytes with ascending offsets ending at or before len (else
 * FRT_ERR_INVALID_ARGUMENT).  Results equal frt_bam_decode's record offsets
 * and tail.  All calls share the one scratch array: calls that overlap on the
 * GPU race and must be serialised.  The first call on a device looks up the
 * array's address with that device current; make it before any stream
 * capture.  The address is looked up once per device per process, so after a
 * cudaDeviceReset reload the library before calling again.  Synchronises
 * `stream` to return n_records and tail. */
#define FRT_NOALLOC_MAX_MEMBERS 1024
int frt_bam_scan_noalloc(const uint8_t *data, uint64_t len, const uint64_t *member_offsets, uint32_t n_members,
                         uint64_t start, int32_t n_ref, uint64_t *record_offsets, uint64_t record_cap,
                         uint64_t *n_records, uint64_t *tail, void *stream, frt_error *err);

/* ---- DeviceRecordBatch, crates/fritillaria-bam/src/columnar/device.rs:135-297 */

/* Columns.  0-13 are the reference's DeviceColumns (device.rs:63-110) in its
 * order; 14+ are the additions of this library. */
typedef enum {
    FRT_COL_REF_ID = 0,          /* i32 */
    FRT_COL_POS = 1,             /* i32 */
    FRT_COL_FLAGS = 2,           /* u16 */
    FRT_COL_MAPQ = 3,            /* u8 */
    FRT_COL_SEQ_LEN = 4,         /* u32 */
    FRT_COL_MATE_REF_ID = 5,     /* i32 */
    FRT_COL_MATE_POS = 6,        /* i32 */
    FRT_COL_TLEN = 7,            /* i32 */
    FRT_COL_RECORD_OFFSETS = 8,  /* u64, into the inflate batch */
    FRT_COL_CIGAR_START = 9,     /* u32, record-relative */
    FRT_COL_SEQUENCE_START = 10, /* u32 */
    FRT_COL_QUALITY_START = 11,  /* u32 */
    FRT_COL_AUX_START = 12,      /* u32 */
    FRT_COL_RECORD_END = 13,     /* u32 */
    FRT_COL_BIN = 14,            /* u16 */
    FRT_COL_N_CIGAR = 15,        /* u16 */
    FRT_COL_NAME_LEN = 16,       /* u8, l_read_name including the NUL */
    FRT_COL_VIRTUAL_OFFSET = 17, /* u64: member compressed offset << 16 | in-member offset */
    FRT_COL_AUX_COUNT = 18,      /* u32: aux fields parsed */
    FRT_COL_AUX_STATUS = 19,     /* u8: 0 aux block parses to its end, 1 malformed field */
    FRT_COL_AUX_FIRST = 20,      /* u32, n + 1 entries: exclusive prefix of AUX_COUNT */
    FRT_COL_AUX_ENTRIES = 21,    /* 12 bytes per field: tag[2], type, subtype, u32 value offset, u32 count */
    FRT_COL_COUNT = 22
} frt_bam_column;

uint64_t frt_record_batch_len(const frt_record_batch *rb);
/* DeviceRecordBatch::tail (device.rs:211-215). */
uint64_t frt_record_batch_tail(const frt_record_batch *rb);
uint64_t frt_record_batch_aux_fields(const frt_record_batch *rb);
int frt_record_batch_device_ordinal(const frt_record_batch *rb);
/* Device pointer, byte length and element width of a column. */
int frt_record_batch_column(const frt_record_batch *rb, int column, void **ptr, size_t *bytes, size_t *width);
/* Copies a column to host memory (to_host / field_bounds_to_host, device.rs:223-282). */
int frt_record_batch_column_to_host(const frt_record_batch *rb, int column, void *dst, size_t cap, frt_error *err);
void *frt_record_batch_ready_event(const frt_record_batch *rb);
void frt_record_batch_free(frt_record_batch *rb);

/* ---- FASTQ, BCF and FASTA on the same container ---------------------------
 * Each scanner takes a device-resident inflate batch (from the codec or the
 * reader) and returns an frt_columns handle: device columns in the reference's
 * order, the tail to carry into the next batch, and how the boundaries were
 * established.  The handle keeps its inflate batch alive. */
typedef struct frt_fastq_scanner frt_fastq_scanner;
typedef struct frt_text_scanner frt_text_scanner;
typedef struct frt_bcf_scanner frt_bcf_scanner;
typedef struct frt_fasta_compactor frt_fasta_compactor;
typedef struct frt_columns frt_columns;

/* FASTQ DeviceColumns, crates/fritillaria-fastq/src/columnar/device.rs:44-72. */
typedef enum {
    FRT_FASTQ_COL_RECORD_OFFSETS = 0, /* u64, into the inflate batch */
    FRT_FASTQ_COL_SEQUENCE_START = 1, /* u32, record-relative */
    FRT_FASTQ_COL_PLUS_START = 2,     /* u32 */
    FRT_FASTQ_COL_QUALITY_START = 3,  /* u32 */
    FRT_FASTQ_COL_SEQUENCE_LEN = 4,   /* u32 */
    FRT_FASTQ_COL_RECORD_END = 5,     /* u32 */
    FRT_FASTQ_COL_COUNT = 6
} frt_fastq_column;

/* BCF DeviceColumns, crates/fritillaria-bcf/src/columnar/device.rs:68-110. */
typedef enum {
    FRT_BCF_COL_CHROMOSOME_ID = 0,   /* i32 */
    FRT_BCF_COL_POSITION = 1,        /* i32, 0-based */
    FRT_BCF_COL_REFERENCE_SPAN = 2,  /* i32 */
    FRT_BCF_COL_QUALITY = 3,         /* u32, raw float bits */
    FRT_BCF_COL_INFO_COUNT = 4,      /* u16 */
    FRT_BCF_COL_ALLELE_COUNT = 5,    /* u16 */
    FRT_BCF_COL_SAMPLE_COUNT = 6,    /* u32 */
    FRT_BCF_COL_FORMAT_COUNT = 7,    /* u8 */
    FRT_BCF_COL_RECORD_OFFSETS = 8,  /* u64 */
    FRT_BCF_COL_ALLELES_START = 9,   /* u32, record-relative */
    FRT_BCF_COL_FILTERS_START = 10,  /* u32 */
    FRT_BCF_COL_INFO_START = 11,     /* u32 */
    FRT_BCF_COL_GENOTYPES_START = 12, /* u32 */
    FRT_BCF_COL_RECORD_END = 13,     /* u32 */
    FRT_BCF_COL_COUNT = 14
} frt_bcf_column;

/* FASTA DeviceColumns, crates/fritillaria-fasta/src/columnar/device.rs. */
typedef enum {
    FRT_FASTA_COL_SEQUENCE = 0,         /* u8, every contig's bases, newlines removed */
    FRT_FASTA_COL_SEQUENCE_OFFSETS = 1, /* u64, where each contig starts in SEQUENCE */
    FRT_FASTA_COL_SEQUENCE_LENGTHS = 2, /* u64 */
    FRT_FASTA_COL_RECORD_OFFSETS = 3,   /* u64, the '>' of each contig in the batch */
    FRT_FASTA_COL_COUNT = 4
} frt_fasta_column;

/* FastqScanner::new / with_context, crates/fritillaria-cuda/src/fastq.rs:53-84.
 * The scanner keeps one device array from call to call: the newline index's
 * tile slots, 3/16 of the largest batch it has scanned (3 bytes for each of
 * 1,024 newlines per 16 KiB tile), freed by frt_fastq_scanner_destroy.  The
 * text scanner keeps the same array. */
int frt_fastq_scanner_create(int device, void *stream, frt_fastq_scanner **out, frt_error *err);
void frt_fastq_scanner_destroy(frt_fastq_scanner *s);
/* FastqScanner::decode(batch, start) (fastq.rs:117-140; scan, fastq.rs:94-110,
 * is the same call with the scan info read from the handle). */
int frt_fastq_decode(frt_fastq_scanner *s, const frt_inflate_batch *batch, uint64_t start, frt_columns **out,
                     frt_error *err);

/* parse_header, crates/fritillaria-bcf/src/columnar/header.rs:111-160: where
 * records start, the sample count and the contig count the scan needs. */
int frt_bcf_parse_header(const uint8_t *buf, size_t len, uint64_t *records_start, uint32_t *samples,
                         uint32_t *contigs, frt_error *err);
/* BcfScanner::new / with_context, crates/fritillaria-cuda/src/bcf.rs:46-80. */
int frt_bcf_scanner_create(int device, void *stream, frt_bcf_scanner **out, frt_error *err);
void frt_bcf_scanner_destroy(frt_bcf_scanner *s);
/* BcfScanner::decode(batch, start, samples, contigs) (bcf.rs:125-150). */
int frt_bcf_decode(frt_bcf_scanner *s, const frt_inflate_batch *batch, uint64_t start, uint32_t samples,
                   uint32_t contigs, frt_columns **out, frt_error *err);

/* FastaCompactor::new / with_context and compact(batch),
 * crates/fritillaria-cuda/src/fasta.rs:40-80.  The batch holds a whole FASTA. */
int frt_fasta_compactor_create(int device, void *stream, frt_fasta_compactor **out, frt_error *err);
void frt_fasta_compactor_destroy(frt_fasta_compactor *s);
int frt_fasta_compact(frt_fasta_compactor *s, const frt_inflate_batch *batch, frt_columns **out, frt_error *err);

/* DeviceRecordBatch / DeviceReference accessors. */
uint64_t frt_columns_len(const frt_columns *c);         /* records (contigs for FASTA) */
uint64_t frt_columns_tail(const frt_columns *c);        /* FASTQ/BCF: carry point */
uint64_t frt_columns_total_bases(const frt_columns *c); /* FASTA: bases in SEQUENCE */
int frt_columns_count(const frt_columns *c);            /* columns of this format */
int frt_columns_device_ordinal(const frt_columns *c);
/* SpeculativeScan's proof (0 tiled, 1 walked), survivors and validated
 * (crates/fritillaria-fastq/src/columnar/speculative.rs:62-90,
 * crates/fritillaria-bcf/src/columnar/speculative.rs). */
void frt_columns_scan_info(const frt_columns *c, uint64_t *proof, uint64_t *survivors, uint64_t *validated);
int frt_columns_column(const frt_columns *c, int column, void **ptr, size_t *bytes, size_t *width);
int frt_columns_column_to_host(const frt_columns *c, int column, void *dst, size_t cap, frt_error *err);
void *frt_columns_ready_event(const frt_columns *c);
void frt_columns_free(frt_columns *c);

/* ---- tab-delimited text (SAM, VCF, BED, GFF, GTF) ---------------------------
 * TextScanner::scan (crates/fritillaria-cuda/src/text.rs:79-96, 233-420) over
 * kernels/text_scan.cu: the lines of a device batch from `start`, split into
 * records and header lines by their first byte (Dialect, crates/fritillaria-text/
 * src/columnar/batch.rs:23-76: `comment`, and `secondary` or -1), blank lines
 * skipped, each record's tab offsets in a flat table.  As the reference's
 * device path: a last line without a newline is a record ending at the batch
 * end, and the tail is then its start (else the batch end; an empty batch or
 * start at/after its end: min(start, len)).  Tables are sized from exact
 * counts, so there is no line-capacity error.  frt_columns_len = records;
 * frt_columns_tail = tail; scan_info's first value = header lines. */
typedef enum {
    FRT_TEXT_COL_RECORD_OFFSETS = 0, /* u64, records */
    FRT_TEXT_COL_RECORD_ENDS = 1,    /* u64, records: one past the last byte, newline excluded */
    FRT_TEXT_COL_HEADER_OFFSETS = 2, /* u64, header lines */
    FRT_TEXT_COL_TABS = 3,           /* u64: every tab offset, grouped by record */
    FRT_TEXT_COL_FIELD_STARTS = 4,   /* u64, records + 1 (none for no records): record i's tabs are
                                        TABS[FIELD_STARTS[i], FIELD_STARTS[i + 1]) */
    FRT_TEXT_COL_COUNT = 5
} frt_text_column;

int frt_text_scanner_create(int device, void *stream, frt_text_scanner **out, frt_error *err);
void frt_text_scanner_destroy(frt_text_scanner *s);
int frt_text_scan(frt_text_scanner *s, const frt_inflate_batch *batch, uint64_t start, int32_t comment,
                  int32_t secondary, frt_columns **out, frt_error *err);

/* ---- columnar VCF: the fixed fields of a text scan's records ---------------
 * The records of frt_text_scan with the VCF dialect (comment '#'), each read
 * as the vendored lazy reader reads it: read_record
 * (crates/fritillaria-vcf/src/io/reader/record.rs:9-118: seven tab-terminated
 * fields, then INFO up to a tab or the end of the line, a carriage return
 * before the line feed dropped; fewer fields is "unexpected EOL") and the
 * accessors of src/record/fields.rs:20-103 and src/record.rs:35-79 ("." is
 * missing, POS "0" the telomere, else usize::from_str then a non-zero
 * Position; QUAL f32::from_str; ALT split on ','; samples missing when empty
 * or their first field is "."). The reference's device path ends at the text
 * framing and its README names columnar VCF.gz as the next step: there is no
 * reference interface to replace, so these entry points are additions. */
typedef struct frt_vcf_decoder frt_vcf_decoder;
enum { FRT_VCF_BOUNDS = 9 };
typedef enum {
    FRT_VCF_COL_CHROM = 0,  /* i32: CHROM's index in the contig dictionary, -1 when absent */
    FRT_VCF_COL_POS = 1,    /* u64: the 1-based start; 0 for the telomere and for an invalid POS */
    FRT_VCF_COL_BOUNDS = 2, /* u32 x FRT_VCF_BOUNDS a record, from the record's first byte: the ends of
                               CHROM, POS, ID, REF, ALT, QUAL, FILTER and INFO, then of the line
                               (carriage return dropped); field k > 0 starts one past the end of
                               field k - 1, the samples one past INFO's end when a tab follows it */
    FRT_VCF_COL_N_ALT = 3,  /* u32: alternate alleles (0 when ALT is "." or empty) */
    FRT_VCF_COL_QUAL = 4,   /* u32: the f32 bits of QUAL when FRT_VCF_FLAG_QUAL_PARSED, else a NaN */
    FRT_VCF_COL_FLAGS = 5,  /* u16: FRT_VCF_FLAG_* */
    FRT_VCF_COL_STATUS = 6, /* u8: FRT_VCF_STATUS_* */
    FRT_VCF_COL_COUNT = 7
} frt_vcf_column;
enum {
    FRT_VCF_FLAG_ID_MISSING = 1,
    FRT_VCF_FLAG_ALT_MISSING = 2,
    FRT_VCF_FLAG_QUAL_MISSING = 4,
    FRT_VCF_FLAG_FILTER_MISSING = 8,
    FRT_VCF_FLAG_INFO_MISSING = 16,
    FRT_VCF_FLAG_SAMPLES_MISSING = 32,
    FRT_VCF_FLAG_FILTER_PASS = 64,
    /* QUAL parsed on the device: decimals of at most 2^24 with a power of ten
       of at most 10^10 either way (Clinger's fast path, exact).  A QUAL that
       is neither missing nor parsed (longer decimals, inf, NaN, or text that
       f32::from_str rejects) is left to the caller, by its bounds. */
    FRT_VCF_FLAG_QUAL_PARSED = 128,
    FRT_VCF_FLAG_TELOMERE = 256
};
enum {
    FRT_VCF_STATUS_OK = 0,
    FRT_VCF_STATUS_UNEXPECTED_EOL = 1,    /* fewer than eight fields: the record's other columns are 0 */
    FRT_VCF_STATUS_INVALID_POSITION = 2   /* POS is not a usize, or is 0 written other than "0" */
};

int frt_vcf_decoder_create(int device, void *stream, frt_vcf_decoder **out, frt_error *err);
void frt_vcf_decoder_destroy(frt_vcf_decoder *d);
/* The contig dictionary: names[i] (lens[i] bytes) is contig i; a repeated
 * name keeps its first index.  Replaces any earlier dictionary. */
int frt_vcf_set_contigs(frt_vcf_decoder *d, const char *const *names, const size_t *lens, size_t n,
                        frt_error *err);
/* The dictionary from a VCF header's text: the ID of each "##contig=<...>"
 * line, in order; *n_contigs = how many. */
int frt_vcf_set_contigs_from_header(frt_vcf_decoder *d, const uint8_t *text, size_t len, size_t *n_contigs,
                                    frt_error *err);
/* Columns FRT_VCF_COL_* of the records of `text` (an frt_text_scan result);
 * frt_columns_len and frt_columns_tail are the scan's; the result holds the
 * scan's batch alive. */
int frt_vcf_decode(frt_vcf_decoder *d, const frt_columns *text, frt_columns **out, frt_error *err);

/* Genotypes: every sample's GT value (crates/fritillaria-vcf/src/record/
 * samples/series/value.rs:17-30, value/genotype/iter.rs), found at GT's
 * position among the FORMAT keys (src/record/samples/sample.rs: keys zipped
 * with the sample's ':'-separated values).  One u32 per tab of the text scan:
 * the call of the sample that tab opens (from each record's ninth tab on; the
 * first eight tabs of a record get 0), so sample j of record i is at
 * TABS index FIELD_STARTS[i] + 8 + j.  A call packs FRT_VCF_GT_STATUS in bits
 * 28-31 and, when that is FRT_VCF_GT_CALLED, the ploidy (1 or 2) in bits
 * 26-27, the second and first alleles' phasing (1 phased) in bits 25 and 24,
 * and the second and first alleles' index + 1 (0 for ".") in bits 12-23 and
 * 0-11. */
typedef enum {
    FRT_VCF_GT_COL_CALLS = 0, /* u32 per tab of the scan */
    FRT_VCF_GT_COL_KEY = 1,   /* i32 per record: GT's index among the FORMAT keys; -1 none or no samples */
    FRT_VCF_GT_COL_COUNT = 2
} frt_vcf_gt_column;
enum {
    FRT_VCF_GT_CALLED = 0,        /* the alleles below */
    FRT_VCF_GT_MISSING = 1,       /* the value is "." */
    FRT_VCF_GT_NONE = 2,          /* no value: no GT key, a shorter or empty sample, or no samples */
    FRT_VCF_GT_INVALID = 3,       /* the reader's error: an empty value or an allele neither "." nor a usize */
    FRT_VCF_GT_UNREPRESENTED = 4  /* valid, but more than two alleles or an index above 4093: read its text */
};
int frt_vcf_genotypes(frt_vcf_decoder *d, const frt_columns *text, frt_columns **out, frt_error *err);

/* ---- record fields: opt-in device kernels over decoded BAM records ---------
 * The reference reads these on the host, record by record: Record::aux_get
 * (crates/fritillaria-bam/src/columnar/record.rs:286-294, over the Fields
 * iterator of aux.rs:301-479), Record::cigar_resolved and
 * has_long_cigar_placeholder (record.rs:316-357), decode_sequence (seq.rs), and
 * the payload accessors name/cigar_raw/sequence_packed/qualities/aux_raw
 * (record.rs:222-270).  Here each runs for every record of a decoded batch at
 * once and returns an frt_columns; `unpack_sequences` and `compact` are the
 * opt-ins of docs/device-api.md:261-263 and :443-444.  The record-batch forms
 * keep the batch's inflated bytes alive as long as the result (offsets point
 * into them); the engine forms read the engine's last run (one BAM bound) and
 * their offsets are valid until its next run.  Results are ready when
 * frt_columns_ready_event completes on the source's stream. */
typedef enum {
    FRT_AUXV_STATUS = 0,  /* u8: 0 absent, 1 present, 2 aux block malformed before the tag (aux_get's Err) */
    FRT_AUXV_TYPE = 1,    /* u8: 'A' 'c' 'C' 's' 'S' 'i' 'I' 'f' 'Z' 'H' 'B' */
    FRT_AUXV_SUBTYPE = 2, /* u8: the B array's element type */
    FRT_AUXV_COUNT = 3,   /* u32: 1 for a scalar, string length for Z/H, elements for B */
    FRT_AUXV_VALUE = 4,   /* i64: an integer scalar (sign- or zero-extended), the byte of A, the IEEE bits of f */
    FRT_AUXV_OFFSET = 5,  /* u64: the value's bytes in the inflated batch (B: its first element) */
    FRT_AUXV_COL_COUNT = 6
} frt_aux_value_column;

typedef enum {
    FRT_CIGAR_COL_OFFSET = 0, /* u64: first op (u32 each) in the inflated batch */
    FRT_CIGAR_COL_OPS = 1,    /* u32: ops */
    FRT_CIGAR_COL_STATUS = 2, /* u8: 0 stored CIGAR, 1 long CIGAR from CG, 2 placeholder without a B:I CG */
    FRT_CIGAR_COL_COUNT = 3
} frt_cigar_column;

typedef enum {
    FRT_BASES_COL_OFFSETS = 0, /* u64, n + 1: record i's bases are DATA[OFFSETS[i], OFFSETS[i + 1]) */
    FRT_BASES_COL_DATA = 1,    /* u8: "=ACMGRSVTWYHKDBN"[nibble], high nibble first */
    FRT_BASES_COL_COUNT = 2
} frt_bases_column;

typedef enum {
    FRT_COMPACT_COL_NAME_OFFSETS = 0, FRT_COMPACT_COL_NAME_DATA = 1,         /* name without its NUL */
    FRT_COMPACT_COL_CIGAR_OFFSETS = 2, FRT_COMPACT_COL_CIGAR_DATA = 3,       /* stored ops, u32 each */
    FRT_COMPACT_COL_SEQUENCE_OFFSETS = 4, FRT_COMPACT_COL_SEQUENCE_DATA = 5, /* 4-bit packed */
    FRT_COMPACT_COL_QUALITY_OFFSETS = 6, FRT_COMPACT_COL_QUALITY_DATA = 7,
    FRT_COMPACT_COL_AUX_OFFSETS = 8, FRT_COMPACT_COL_AUX_DATA = 9,           /* raw aux block */
    FRT_COMPACT_COL_COUNT = 10 /* offsets: u64, n + 1 entries, in bytes of the data column */
} frt_compact_column;

int frt_record_batch_aux_lookup(const frt_record_batch *rb, const char tag[2], frt_columns **out, frt_error *err);
int frt_record_batch_cigar_resolved(const frt_record_batch *rb, frt_columns **out, frt_error *err);
int frt_record_batch_unpack_sequences(const frt_record_batch *rb, frt_columns **out, frt_error *err);
int frt_record_batch_compact(const frt_record_batch *rb, frt_columns **out, frt_error *err);

/* ---- BAI region resolution -------------------------------------------------
 * The index (crates/fritillaria-bam/src/bai.rs, the csi BinningIndex) turns a
 * region into chunks of virtual offsets: a record is in the query when its
 * start virtual offset lies in a chunk and it overlaps the region. */
typedef struct frt_bai frt_bai;
typedef struct {
    uint64_t start; /* virtual offset: compressed member offset << 16 | in-member offset */
    uint64_t end;
} frt_chunk;

/* Reads a BAI (SAM specification 5.2). */
int frt_bai_parse(const uint8_t *buf, size_t len, frt_bai **out, frt_error *err);
void frt_bai_free(frt_bai *bai);
int32_t frt_bai_reference_count(const frt_bai *bai);
/* BinningIndex::query (crates/fritillaria-csi/src/binning_index/index.rs:93-119)
 * for [start, end], 1-based inclusive (0 start/end: unbounded).  *n receives
 * the chunk count; FRT_ERR_INVALID_ARGUMENT when it exceeds cap. */
int frt_bai_query(const frt_bai *bai, int32_t ref, uint64_t start, uint64_t end, frt_chunk *out, size_t cap,
                  size_t *n, frt_error *err);

/* ---- region serving ----------------------------------------------------------
 * No reference counterpart as a server: the reference answers one region at a
 * time through its indexed reader (crates/fritillaria-bam/src/io/reader/query.rs).
 * Here BAMs with their BAIs are resident in device memory; region queries are
 * resolved to chunks on the host, and every request admitted within the HBM
 * budget since the last tick is served by one persistent inflate over all their
 * members plus one segmented record scan and region filter, without blocking the
 * caller.  A request's results are the records the reference's query yields
 * (start virtual offset inside a chunk, reference and interval overlap), in file
 * order, as device columns that stay resident until released. */
typedef struct frt_server frt_server;

typedef enum {
    FRT_REGION_COL_VIRTUAL_OFFSET = 0, /* u64 */
    FRT_REGION_COL_RECORD_OFFSET = 1,  /* u64, into the request's inflated bytes */
    FRT_REGION_COL_REF_ID = 2,         /* i32 */
    FRT_REGION_COL_POS = 3,            /* i32, 0-based */
    FRT_REGION_COL_FLAGS = 4,          /* u16 */
    FRT_REGION_COL_MAPQ = 5,           /* u8 */
    FRT_REGION_COL_SEQ_LEN = 6,        /* u32 */
    FRT_REGION_COL_COUNT = 7
} frt_region_column;

typedef struct {
    int32_t state;  /* 0 queued, 1 running, 2 done */
    int32_t status; /* frt_status once done */
    uint64_t records;
    double arrival_ms, done_ms; /* server clock: frt_server_clock_ms; done from the device's completion event */
    uint64_t inflated_bytes;
    uint32_t chunks;
    uint64_t members;
    uint32_t retries; /* re-reads with more trailing members for a record cut at the chunk end */
} frt_region_info;

/* `budget_bytes` bounds the device memory of admitted requests (their inflated
 * bytes, scan scratch and results, held until released). */
int frt_server_create(int device, void *stream, uint64_t budget_bytes, frt_server **out, frt_error *err);
void frt_server_destroy(frt_server *s);
/* Requests per tick and ticks in flight (by default: no limit, and four).
 * 0 for either limit: no limit on requests per tick; 1 tick in flight.
 * With more than one tick in flight each tick runs on a stream the server
 * creates, so ticks overlap on the device. */
void frt_server_set_limits(frt_server *s, uint32_t max_requests_per_tick, uint32_t max_ticks_in_flight);
/* Milliseconds since the server was created (the clock of arrival_ms/done_ms). */
double frt_server_clock_ms(const frt_server *s);
/* Where the time of finished ticks went, summed over ticks: host time to plan,
 * allocate and launch them; device time from a tick's start to its inflate
 * (the table uploads, and any wait behind the tick before it on the stream),
 * in the persistent inflate, and from there to completion (region scan,
 * filter, emit, status copy).  No reference counterpart.  `reset` zeroes
 * the totals after reading them. */
typedef struct {
    uint64_t ticks, requests, members;
    double host_ms, upload_ms, inflate_ms, scan_ms, max_inflate_ms;
} frt_server_stats;
int frt_server_get_stats(const frt_server *s, frt_server_stats *out, int32_t reset);
/* Makes a BGZF BAM and its BAI resident (before the first request). */
int frt_server_add_bam(frt_server *s, const uint8_t *bgzf, size_t len, const uint8_t *bai, size_t bai_len,
                       int32_t *file_id, frt_error *err);
/* Queues [start, end] (1-based inclusive; 0 = unbounded) on reference `ref`.
 * arrival_ms < 0 stamps the request now. */
int frt_server_submit(frt_server *s, int32_t file, int32_t ref, uint64_t start, uint64_t end, double arrival_ms,
                      uint64_t *request, frt_error *err);
/* Completes finished ticks and launches new ones; never waits on the device. */
int frt_server_progress(frt_server *s, uint32_t *completed, frt_error *err);
/* Waits until every submitted request has completed. */
int frt_server_drain(frt_server *s, frt_error *err);
int frt_server_request_info(const frt_server *s, uint64_t request, frt_region_info *info);
int frt_server_request_error(const frt_server *s, uint64_t request, frt_error *err);
int frt_server_request_column(const frt_server *s, uint64_t request, int column, void **ptr, size_t *bytes,
                              size_t *width);
int frt_server_request_column_to_host(const frt_server *s, uint64_t request, int column, void *dst, size_t cap,
                                      frt_error *err);
/* The request's inflated bytes (device), which FRT_REGION_COL_RECORD_OFFSET indexes. */
const uint8_t *frt_server_request_inflated(const frt_server *s, uint64_t request, size_t *len);
void frt_server_release(frt_server *s, uint64_t request);

/* ---- inflate tuning ----------------------------------------------------------
 * No reference counterpart: the reference launches one fixed kernel shape
 * (crates/fritillaria-cuda/src/backend.rs:178-219).  The member inflate here
 * is compiled in several variants -- literal/length and distance table roots,
 * window buffer and match queue per warp -- and a tuning picks a variant, the
 * warps per CTA (one member per warp), the CTAs per SM and the members a warp
 * takes per pop of the device work queue.  Codecs, engines and servers start
 * from the process-wide default; frt_autotune times candidates on an engine's
 * bound input and caches the winner in a JSON file keyed by device, variant
 * set and workload class. */
typedef struct {
    int32_t variant;        /* index of a compiled variant */
    int32_t warps_per_cta;  /* 1..8; each warp takes the variant's chains of members */
    int32_t ctas_per_sm;    /* 0: as many as fit */
    int32_t queue_chunk;    /* members per queue pop, 1..64 */
    int32_t spread_variant; /* -1, or a one-chain variant for small launches: a launch of fewer members
                               than one wave of one-warp CTAs holds is made one warp per CTA, and then
                               each member's serial chain bounds it, so a variant with more registers
                               and wider tables does better than the one tuned for throughput */
} frt_inflate_tuning;

typedef struct {
    int32_t lit_bits;       /* literal/length table root */
    int32_t dist_bits;      /* distance table root */
    int32_t window;         /* window buffer per warp, bytes */
    int32_t queue;          /* matches queued per window */
    int32_t max_registers;  /* register cap per thread */
    int32_t chains;         /* members a warp decodes side by side, one lane each */
    int32_t stage_half;     /* 0: compressed bytes read through L1; else the bytes of each half of a
                               shared-memory ring they are staged in by bulk copies */
    uint64_t smem_per_warp; /* shared memory per warp, bytes */
} frt_inflate_variant;

int frt_inflate_variant_count(void);
int frt_inflate_variant_info(int32_t variant, frt_inflate_variant *out, frt_error *err);
void frt_inflate_get_default_tuning(frt_inflate_tuning *out);
/* Checks that the tuning fits `device` (at least one CTA per SM) and makes it
 * the default of codecs, engines and servers created afterwards. */
int frt_inflate_set_default_tuning(int device, const frt_inflate_tuning *t, frt_error *err);
/* CTAs per SM the tuning runs with on `device`; 0 when it is invalid or does
 * not fit. */
int frt_inflate_tuning_ctas_per_sm(int device, const frt_inflate_tuning *t);

/* ---- batched, device-resident form ---------------------------------------
 * No reference counterpart: the batched launch model.  Members of a whole
 * BGZF file resident in device memory are discovered, inflated, verified,
 * scanned and decoded by one persistent kernel per stage, fed by a device work
 * queue sorted by compressed size; the steady state replays as a CUDA graph. */
typedef struct frt_engine frt_engine;

typedef struct {
    uint32_t warps_per_cta;   /* 0: from the default inflate tuning */
    uint32_t queue_chunk;     /* members taken per queue pop; 0: from the default inflate tuning */
    uint32_t use_graph;       /* replay the steady state as a CUDA graph */
    uint32_t sort_queue;      /* longest member first */
} frt_engine_config;

typedef struct {
    uint64_t members;
    uint64_t compressed_bytes;
    uint64_t inflated_bytes;
    uint64_t records;
    uint64_t tail;
    uint64_t aux_fields;
    uint64_t fallbacks;
    int32_t status;        /* frt_status of the last run */
    uint32_t error_member; /* first failing member, when status is a block error */
} frt_engine_stats;

int frt_engine_create(int device, void *stream, const frt_engine_config *cfg, frt_engine **out, frt_error *err);
void frt_engine_destroy(frt_engine *e);
/* Binds a device-resident BGZF file (a BAM) and sizes every buffer for it. */
int frt_engine_bind_bam(frt_engine *e, const uint8_t *dev_bgzf, size_t len, frt_error *err);
/* Runs the bound file to columns on the engine's stream (asynchronous);
 * frt_engine_finish waits and reports. */
int frt_engine_run(frt_engine *e, frt_error *err);
int frt_engine_finish(frt_engine *e, frt_engine_stats *stats, frt_error *err);
/* Host-buffer convenience: H2D copy, run, and read the stats back. */
int frt_engine_run_host(frt_engine *e, const uint8_t *host_bgzf, size_t len, frt_engine_stats *stats,
                        frt_error *err);
/* The engine's inflate tuning; a new one takes effect at the next run (the
 * graph is captured again). */
int frt_engine_get_tuning(const frt_engine *e, frt_inflate_tuning *out);
int frt_engine_set_tuning(frt_engine *e, const frt_inflate_tuning *t, frt_error *err);
/* Times the persistent inflate alone under a tuning, after a completed run:
 * the first `members` members of the bound input in file order (0: all), best
 * of `reps` launches on the engine's stream.  *inflated_bytes is what the
 * timed members inflate to.  Leaves the columns of the last run invalid until
 * the next run. */
int frt_engine_time_inflate(frt_engine *e, const frt_inflate_tuning *t, uint64_t members, int32_t reps, double *ms,
                            uint64_t *inflated_bytes, frt_error *err);

typedef struct {
    frt_inflate_tuning tuning;
    double ms;          /* best launch time of the winner on the sample */
    double gbs;         /* inflated GB/s of the winner on the sample */
    uint64_t members;   /* sample size, members */
    int32_t from_cache; /* 1: taken from the cache, nothing timed */
    int32_t candidates; /* tunings timed */
    char key[192];      /* cache key: device, variant set, workload class */
} frt_autotune_result;

/* The autotuner.  After a completed run of the engine, looks its workload up
 * in the JSON cache at `cache_path` (NULL: $FRT_TUNING_CACHE, else
 * ~/.cache/fritillaria_gb300/inflate_tuning.json); on a miss, or with
 * `force`, times the candidates (every variant at 2, 3, 4, 6 and 8 warps per
 * CTA, then queue chunks 1..8 for the best) on a sample of the bound input,
 * and writes the winner back.  The winner becomes the engine's tuning and the
 * process default. */
int frt_autotune(frt_engine *e, const char *cache_path, int32_t force, frt_autotune_result *out, frt_error *err);
int frt_engine_column(const frt_engine *e, int column, void **ptr, size_t *bytes, size_t *width);
int frt_engine_column_to_host(const frt_engine *e, int column, void *dst, size_t cap, frt_error *err);
const uint8_t *frt_engine_inflated(const frt_engine *e, size_t *len);
/* Record fields (see "record fields" above) over the engine's last run of one bound BAM. */
int frt_engine_aux_lookup(const frt_engine *e, const char tag[2], frt_columns **out, frt_error *err);
int frt_engine_cigar_resolved(const frt_engine *e, frt_columns **out, frt_error *err);
int frt_engine_unpack_sequences(const frt_engine *e, frt_columns **out, frt_error *err);
int frt_engine_compact(const frt_engine *e, frt_columns **out, frt_error *err);
/* Copies the inflated bytes of the last run to host memory (cap >= len). */
int frt_engine_inflated_to_host(const frt_engine *e, uint8_t *dst, size_t cap, frt_error *err);
void *frt_engine_stream(const frt_engine *e);
/* Several files, several formats, one inflate.  No reference counterpart:
 * BGZF files laid out back to back in one device buffer (each a whole BGZF
 * stream, together covering the buffer) are discovered, queued and inflated
 * as one population of members by the persistent kernel; each file's inflated
 * range then goes through its format's decoder (BamDecoder, BcfScanner,
 * FastqScanner, FastaCompactor).  BAM and BCF headers are parsed at bind.
 * frt_engine_run runs the inflate and the decoders; the per-file results stay
 * valid until the next run. */
typedef enum { FRT_FORMAT_BAM = 0, FRT_FORMAT_BCF = 1, FRT_FORMAT_FASTQ = 2, FRT_FORMAT_FASTA = 3 } frt_format;

typedef struct {
    uint64_t offset; /* in the bound buffer */
    uint64_t length;
    int32_t format;  /* frt_format */
} frt_engine_file;

typedef struct {
    int32_t format;
    uint64_t members;
    uint64_t compressed_bytes;
    uint64_t inflated_offset; /* where the file's bytes start in frt_engine_inflated */
    uint64_t inflated_bytes;
    uint64_t records;         /* contigs for FASTA */
    uint64_t tail;            /* BAM/BCF/FASTQ: carry point; FASTA: total bases */
    uint64_t proof;           /* BCF/FASTQ: 0 tiled, 1 walked */
    double decode_ms;         /* the last run's decode of this file (CUDA events on the engine stream) */
    uint64_t launches;        /* kernels that decode launched */
} frt_engine_file_info;

int frt_engine_bind_files(frt_engine *e, const uint8_t *dev, size_t len, const frt_engine_file *files, size_t n_files,
                          frt_error *err);
size_t frt_engine_file_count(const frt_engine *e);
int frt_engine_get_file_info(const frt_engine *e, size_t file, frt_engine_file_info *info);
/* The last run's result for a file: a BAM file's record batch, or the column
 * batch of a BCF/FASTQ/FASTA file; owned by the engine (do not free). */
const frt_record_batch *frt_engine_file_bam(const frt_engine *e, size_t file);
const frt_columns *frt_engine_file_columns(const frt_engine *e, size_t file);

/* Per-stage milliseconds (front, inflate, records) of eager runs. */
int frt_engine_time_stages(frt_engine *e, float *ms, int repeats, frt_error *err);
/* Kernel launches per run (kernel nodes of the captured graph). */
uint64_t frt_engine_launches(const frt_engine *e);

/* ---- the write side: BGZF compression of device bytes ----------------------
 * DeviceBlockCompressor (crates/fritillaria-core/src/device.rs:326-372) and
 * DeviceBgzfWriter (crates/fritillaria-bgzf/src/device_write.rs).  The
 * reference compresses with nvCOMP; this library uses its own device deflate
 * (greedy LZ77 over a 32 KiB window, fixed Huffman codes).  Contract, as
 * there: one framed block per chunk, chunks of at most 65,505 bytes
 * (MAX_COMPRESSIBLE_PAYLOAD), no EOF block in a batch, and inflating the output
 * gives back the input block for block -- not byte identity with any other
 * compressor.  The framing of each block is chosen by choose_framing
 * (crates/fritillaria-core/src/compress.rs:115-128). */
typedef struct frt_compressor frt_compressor;
typedef struct frt_bgzf_writer frt_bgzf_writer;
/* A byte sink: returns the bytes it took (> 0), or <= 0 on error. */
typedef int64_t (*frt_write_fn)(void *ctx, const uint8_t *buf, size_t len);

int frt_compressor_create(int device, void *stream, frt_compressor **out, frt_error *err);
void frt_compressor_destroy(frt_compressor *c);
const char *frt_compressor_name(const frt_compressor *c);
int frt_compressor_device_ordinal(const frt_compressor *c);
/* choose_framing: 0 deflated, 1 stored, 2 the empty block; framed_size
 * (compress.rs:134-142): header + body + trailer bytes of that choice. */
int frt_choose_framing(size_t payload_len, size_t deflate_len);
size_t frt_framed_size(size_t payload_len, size_t deflate_len);
/* Bytes that always hold the framed blocks of n chunks (64 KiB each). */
size_t frt_compress_bound(size_t n_chunks);
/* compress_batch_device: each range bounds[i]..bounds[i + 1] (n_bounds - 1
 * ranges, rising, within data_len, at most 65,505 bytes) of the device bytes
 * becomes one block; the blocks go to host `out` back to back, block i at
 * out_offsets[i]..out_offsets[i + 1]; *out_len = their total.  The ranges
 * need not cover the buffer.  A bad range is FRT_ERR_MALFORMED. */
int frt_compress_batch_device(frt_compressor *c, const uint8_t *data, size_t data_len, const uint64_t *bounds,
                              size_t n_bounds, uint8_t *out, size_t out_cap, uint64_t *out_offsets, size_t *out_len,
                              frt_error *err);

/* DeviceBgzfWriter::new(inner, compressor): blocks go to `write`.  The
 * compressor must outlive the writer. */
int frt_bgzf_writer_open(frt_write_fn write, void *ctx, frt_compressor *c, frt_bgzf_writer **out, frt_error *err);
/* with_chunks_per_batch (at least 1; 1024 by default) and with_payload_size
 * (clamped to 1..65,505; 65,280 by default, DEFAULT_PAYLOAD_SIZE). */
void frt_bgzf_writer_set_chunks_per_batch(frt_bgzf_writer *w, size_t chunks);
void frt_bgzf_writer_set_payload_size(frt_bgzf_writer *w, size_t size);
/* write_batch (device_write.rs:106-141): the chunks bounds[i]..bounds[i + 1]
 * of the device bytes; bounds must hold at least one entry and end within
 * `len` (else FRT_ERR_MALFORMED). */
int frt_bgzf_writer_write_batch(frt_bgzf_writer *w, const uint8_t *data, size_t len, const uint64_t *bounds,
                                size_t n_bounds, frt_error *err);
/* The device bytes cut into payload-size chunks. */
int frt_bgzf_writer_write_device(frt_bgzf_writer *w, const uint8_t *data, size_t len, frt_error *err);
/* Appends the 28-byte EOF block (crates/fritillaria-bgzf/src/block.rs:40-43), once. */
int frt_bgzf_writer_finish(frt_bgzf_writer *w, frt_error *err);
void frt_bgzf_writer_stats(const frt_bgzf_writer *w, uint64_t *blocks, uint64_t *batches, uint64_t *compressed,
                           uint64_t *uncompressed);
void frt_bgzf_writer_destroy(frt_bgzf_writer *w);

#ifdef __cplusplus
}
#endif
#endif
