// Host reference sample for measurement sampling.
//
// The reference computes it as TableauSimulator<W>::reference_sample_circuit (tableau_simulator.inl:
// 1435-1438): one run of the circuit's noiseless version (circuit.cc:775-807: noise channels dropped,
// measurement flip probabilities dropped, heralded channels replaced by MPAD 0) on a stabilizer tableau
// whose random measurement outcomes are all forced to 0 (sign bias +1, tableau_simulator.inl:1370).  The
// frame sampler's measurement results are this sample XOR the sampled flips.
#pragma once

#include <cstdint>
#include <vector>

#include "circuit.h"

namespace gfs {

// num_measurements bits, little-endian bit-packed ((num_measurements + 7) / 8 bytes).  Throws
// std::invalid_argument for circuits the frame sampler also rejects (anti-Hermitian products, lookbacks
// before the beginning of time).
std::vector<uint8_t> reference_sample(const Circuit &circuit);

}  // namespace gfs
