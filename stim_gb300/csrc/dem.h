// Detector error models: parsing, flattening and lowering for the GPU sampler (gfs_dem_*).
//
// Mirrors the reference's stim::DetectorErrorModel text format (src/stim/dem/detector_error_model.cc:195-360,
// dem_instruction.cc validate) and DemSampler (src/stim/simulators/dem_sampler.inl): the error mechanisms are
// the `error` instructions with REPEAT blocks unrolled and `shift_detectors` offsets applied, in model order.
#pragma once

#include <cstdint>
#include <string_view>
#include <vector>

#include "kernels.h"

namespace gfs {

struct DemModel {
    uint64_t num_detectors = 0;
    uint64_t num_observables = 0;
    std::vector<double> p;          // per mechanism
    std::vector<uint32_t> sym_off;  // per mechanism: symptoms sym[sym_off[m] .. sym_off[m + 1])
    std::vector<uint32_t> sym;      // detector d -> d, observable k -> num_detectors + k (repeats XOR away)
    uint64_t num_errors() const {
        return p.size();
    }
};

// Throws std::invalid_argument / std::out_of_range with the reference's messages for malformed models.
DemModel parse_dem(std::string_view text);

// The sampling layout: mechanisms grouped by probability (groups in order of first appearance, each group's
// mechanisms in model order), and work chunks of up to kDemChunkUnits mechanisms of one group.
constexpr uint32_t kDemChunkUnits = 1024;

struct DemLayout {
    std::vector<DemGroup> groups;
    std::vector<uint32_t> units;   // mechanism ids, grouped
    std::vector<uint32_t> tables;  // gap tables (GFS_TABLE_LEN words each) of the groups with 0 < p < 1
    std::vector<uint32_t> chunk_group, chunk_unit0, chunk_units;
    // For replayed errors: output o (detector, then observable) = XOR of the mechanisms in
    // out_mech[out_off[o] .. out_off[o + 1]).
    std::vector<uint32_t> out_off, out_mech;
};

DemLayout layout_dem(const DemModel &m);

}  // namespace gfs
