// The host half of the C++ binding that the integration notes show for the reference's CompiledDetectorSampler /
// CompiledMeasurementSampler, compiled against include/stim_gb300.h and linked to the library: parse the circuit,
// read its counts and reference sample, and create a sampler (on a machine without a GPU that step must fail with
// GFS_ERR_CUDA and a message, which the binding turns into an exception).
//
// Usage: binding_example  ->  prints "measurements <n> reference <bits> sampler <status>".
// Test infrastructure (tests/test_capi_cpu.py compiles and runs it); the product never uses it.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "stim_gb300.h"

int main() {
    const std::string text = "X 0\nH 1\nCX 1 2\nM 0 1 2\nMX 1\nDETECTOR rec[-4]\n";
    gfs_circuit *circuit = nullptr;
    if (gfs_circuit_parse(text.data(), text.size(), &circuit) != GFS_OK) {
        std::printf("parse failed: %s\n", gfs_last_error());
        return 1;
    }
    uint64_t stats[6] = {};
    if (gfs_circuit_stats(circuit, stats) != GFS_OK) {
        std::printf("stats failed: %s\n", gfs_last_error());
        return 1;
    }
    const uint64_t measurements = stats[1];
    std::vector<uint8_t> ref((measurements + 7) / 8);
    if (gfs_circuit_reference_sample(circuit, ref.data(), ref.size()) != GFS_OK) {
        std::printf("reference sample failed: %s\n", gfs_last_error());
        return 1;
    }
    std::string bits;
    for (uint64_t k = 0; k < measurements; k++) {
        bits.push_back((ref[k / 8] >> (k % 8)) & 1 ? '1' : '0');
    }
    gfs_sampler *sampler = nullptr;
    const gfs_status st = gfs_sampler_create(circuit, GFS_MODE_DETECTIONS, 7, 0, &sampler);
    std::printf("measurements %llu reference %s sampler %d%s\n", (unsigned long long)measurements, bits.c_str(), (int)st,
                st == GFS_OK ? "" : (std::strlen(gfs_last_error()) ? " message" : " no-message"));
    if (sampler) {
        gfs_sampler_free(sampler);
    }
    gfs_circuit_free(circuit);
    return 0;
}
