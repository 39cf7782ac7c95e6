// Circuit IR and .stim parser of the host library.
//
// Mirrors the reference's stim::Circuit (src/stim/circuit/circuit.h:42-290): a list of instructions
// plus nested blocks for REPEAT, with adjacent identical instructions fused exactly as the reference's
// parser does (circuit.cc:237-300), because the flat instruction index keys the random stream.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

#include "gfs_gates.h"

namespace gfs {

struct Instruction {
    gfs_gate gate = GFS_NOT_A_GATE;
    std::vector<uint32_t> targets;
    std::vector<double> args;
    std::string tag;
    uint32_t block = 0;  // REPEAT: index into Circuit::blocks
    uint64_t reps = 0;   // REPEAT: repetition count

    uint64_t count_results() const;
};

struct CircuitStats {
    uint64_t num_qubits = 0;
    uint64_t num_measurements = 0;
    uint64_t num_detectors = 0;
    uint64_t num_observables = 0;
    uint64_t max_lookback = 0;
    uint64_t num_instances = 0;  // instructions with every REPEAT unrolled
};

struct Circuit {
    std::vector<Instruction> ops;
    std::vector<Circuit> blocks;

    static Circuit parse(std::string_view text);
    CircuitStats stats() const;
};

const gfs_gate_info &gate_info(gfs_gate g);

}  // namespace gfs
