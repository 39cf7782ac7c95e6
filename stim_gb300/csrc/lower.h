// Lowering of a parsed circuit into the device program (program.h).
#pragma once

#include <cstdint>
#include <vector>

#include "circuit.h"
#include "program.h"

namespace gfs {

enum class SampleMode { DETECTIONS, MEASUREMENTS };

struct Program {
    std::vector<DevOp> ops;
    std::vector<uint32_t> pool;
    std::vector<uint32_t> tables;  // gap tables, GFS_TABLE_LEN entries each
    std::vector<DevChan> chans;
    std::vector<uint32_t> qubit_orig;  // compacted row -> circuit qubit index (keys the reset stream)
    uint32_t num_rows = 0;             // compacted qubits
    uint32_t ring = 1;                 // measurement ring rows per 128-shot block
    uint64_t num_detectors = 0;
    uint64_t num_observables = 0;
    uint64_t num_measurements = 0;
    uint32_t max_loop_depth = 0;
    double work = 0;  // estimated cost of one 128-shot block (orders circuits in a batched launch)
    CircuitStats stats;
};

// Throws std::invalid_argument (bad circuit) or std::out_of_range (lookback before the beginning of
// time), mirroring the reference's errors for the same circuits.
Program lower(const Circuit &circuit, SampleMode mode);

}  // namespace gfs
