// Result formats written on the device (formats.cu): shot-major bit-packed rows in device memory turned into the
// bytes of a result file.  Host code sees plain pointers only.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "formats.h"

namespace gfs {

struct FormatArgs {
    const uint8_t *rows;  // shot-major bit-packed rows (device)
    uint64_t stride;      // bytes between rows
    uint64_t shots;
    uint64_t nbits;
    uint32_t fmt;         // Format
    uint8_t c1, c2;       // dets prefixes: bits [0, transition) and the rest (numbered from the transition)
    uint64_t transition;
    uint32_t *lens;       // hits / dets / r8: record bytes per shot (shots entries)
    uint64_t *offs;       // hits / dets / r8: record offsets, exclusive scan (shots + 1 entries)
    uint8_t *out;         // the file's bytes for these shots
};

// Output bytes of a fixed-size format (01, b8, ptb64); 0 for the others.
uint64_t fixed_format_bytes(Format f, uint64_t shots, uint64_t nbits);
// hits / dets / r8: record lengths and offsets; *total (device) receives the bytes of all records.
// block_sums needs (shots + 1024) / 1024 entries.
cudaError_t launch_format_lengths(const FormatArgs &a, uint64_t *block_sums, uint64_t *total, cudaStream_t stream);
// ptb64 file bytes of `shots` shots (a multiple of 64) from detector-major rows: `first` holds n1 rows and
// `second` n2 rows per 128-shot block ([block][row] uint4); the file's bits are first's rows, then second's.
cudaError_t launch_ptb64_detmajor(const uint4 *first, uint64_t n1, const uint4 *second, uint64_t n2, uint64_t shots,
                                  uint8_t *out, cudaStream_t stream);
// Writes the file bytes (01, ptb64, or hits / dets / r8 after launch_format_lengths).
cudaError_t launch_format_write(const FormatArgs &a, cudaStream_t stream);

}  // namespace gfs
