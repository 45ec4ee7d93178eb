// Opt-in record fields on the device, over decoded BAM records: one aux tag
// for every record, CIGARs resolved through CG, bases unpacked to ASCII, and
// the variable-length payloads compacted out of the inflated batch.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/frt.h"
#include "runtime.h"

namespace frt {

// Device pointers to the decoded columns of n records and the inflated bytes
// they point into (the frt_bam_column layout).
struct RecordView {
    const uint8_t *buf = nullptr;
    uint64_t n = 0;
    const uint64_t *record_offsets = nullptr;
    const uint32_t *cigar_start = nullptr, *sequence_start = nullptr, *quality_start = nullptr,
                   *aux_start = nullptr, *record_end = nullptr, *seq_len = nullptr, *aux_count = nullptr,
                   *aux_first = nullptr, *aux_entries = nullptr;
    const uint16_t *n_cigar = nullptr;
    const uint8_t *name_len = nullptr, *aux_status = nullptr;
};

enum FieldsOp { FIELDS_AUX_LOOKUP = 0, FIELDS_CIGAR_RESOLVED = 1, FIELDS_UNPACK_SEQUENCES = 2, FIELDS_COMPACT = 3 };

// Runs `op` on the view on stream `st` (after `after`, when given) and returns
// its columns.  `retain` is the batch the results point into (aux lookup and
// resolved CIGAR give offsets into the inflated bytes), held by the result.
int fields_run(const RecordView &v, int op, const char *tag, int device, cudaStream_t st, SharedStream *shared,
               cudaEvent_t after, const frt_inflate_batch *retain, frt_columns **out, frt_error *err);

} // namespace frt
