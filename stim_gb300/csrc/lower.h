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
    uint64_t num_sweep_bits = 0;  // columns of the sweep table read by sweep feedback (LowerOptions::sweep)
    uint32_t max_loop_depth = 0;
    double work = 0;  // estimated cost of one 128-shot block (orders circuits in a batched launch)
    // Detection sampling: the start-of-shot Z randomization never reaches an output (the kernel may start
    // every frame at zero); ops with the same property carry kNoRandomize.
    bool reset_norand = false;
    std::vector<double> chan_p;  // hit probability of each channel

    // Noise occurrences (a noise instruction instance, or the noise fused before/after a gate) met by one
    // pass over the program, loops unrolled, and the expected number of hits per 128-shot block.
    uint64_t noise_occurrences = 0;
    double hits_per_block = 0;
    // The occurrences in order with their expected hits per 128-shot block (empty when there are more
    // than kMaxNoiseOccurrences).
    std::vector<NoiseOcc> occs;
    std::vector<double> occ_hits_per_block;
    CircuitStats stats;
    // The lean kernel's phase list (program.h LeanPhase) and each phase's instance offset; lean_ok when
    // every op has a lean form (no correlated errors or heralds, compact unit lists, at most two loop levels
    // of fewer than 2^32 repetitions).
    std::vector<LeanPhase> lean;
    std::vector<uint64_t> lean_inst;
    std::vector<OccXform> occ_xform;  // transforms of the hit occurrences the lean plan moved (NoiseOcc.xform)
    bool lean_ok = false;
};

struct LowerOptions {
    // Frames start at zero and measurements / resets draw no randomization (the reference's
    // guarantee_anticommutation_via_frame_randomization = false, frame_simulator.h:65).
    bool no_randomization = false;
    // Sweep-controlled Paulis become OP_FEEDBACK entries reading KernelArgs.sweep (the samplers leave them out:
    // their sweep bits are all zero).
    bool sweep = false;
};

// Throws std::invalid_argument (bad circuit) or std::out_of_range (lookback before the beginning of
// time), mirroring the reference's errors for the same circuits.
Program lower(const Circuit &circuit, SampleMode mode, const LowerOptions &opts = LowerOptions());

// The reference's Circuit::aliased_noiseless_circuit (src/stim/circuit/circuit.cc:775-807): noise instructions
// dropped, heralded errors replaced by MPAD of zeros (same number of results), result-flip probabilities removed.
Circuit noiseless_copy(const Circuit &c);

constexpr uint64_t kMaxNoiseOccurrences = 1u << 16;

// Fills each occurrence's region (off, cap) for slices of `blocks` 128-shot blocks: the expected hits
// plus a margin of eight standard deviations and 32 records (an overflow is detected by the noise kernel
// and the chunk redone inline).  cap_override > 0 caps every region (used to exercise that path).
// Returns the records per slice region.
uint64_t plan_hit_regions(std::vector<NoiseOcc> &occs, const std::vector<double> &hits_per_block, uint32_t blocks,
                          uint64_t cap_override);

}  // namespace gfs
