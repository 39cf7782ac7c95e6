/*
 * stim_oracle.h -- CPU oracle for the bulk detection-event / measurement sampler.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library; the product path never does.
 *
 * It is a plain-C restatement of the reference's frame sampler: the .stim grammar of
 * src/stim/circuit/circuit.cc:149-310 and gate_target.h:75-195, and the per-gate frame rules of
 * src/stim/simulators/frame_simulator.inl:152-912, with the random stream replaced by the
 * counter-based contract of stim_gb300/csrc/gfs_contract.h.  Its outputs are pinned against the
 * reference itself (oracle/ref_inject.cc, which runs the reference's FrameSimulator on the same
 * injected bits) through the golden fixtures in tests/golden/.
 */
#ifndef STIM_ORACLE_H
#define STIM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_circuit oracle_circuit;

/* Parses .stim text.  Returns NULL and fills err on failure. */
oracle_circuit *oracle_parse(const char *text, char *err, size_t err_len);
void oracle_free(oracle_circuit *c);

/* out[0..5] = num_qubits, num_measurements, num_detectors, num_observables, max_lookback, num_instances. */
void oracle_stats(const oracle_circuit *c, uint64_t *out);

/*
 * Samples shots [first_shot, first_shot + num_shots) (first_shot a multiple of 128) under seed.
 * Each output that is non-NULL is written shot-major, bit-packed little-endian, ceil(n/8) bytes per
 * shot: dets (detection events), obs (observable flips), meas (measurement flips, before any
 * reference-sample XOR).  Returns 0, or -1 with err filled.
 */
int oracle_sample(const oracle_circuit *c, uint64_t seed, uint64_t first_shot, uint64_t num_shots, int num_threads,
                  uint8_t *dets, uint8_t *obs, uint8_t *meas, char *err, size_t err_len);

/*
 * Measurements to detection events for circuits without sweep data: meas = `shots` rows of
 * ceil(measurements / 8) bit-packed bytes, ref = the reference sample (NULL = zeros); dets / obs receive
 * ceil(n / 8)-byte rows.  Returns 0, or -1 with err filled.
 */
int oracle_m2d(const oracle_circuit *c, uint64_t shots, const uint8_t *meas, const uint8_t *ref, uint8_t *dets,
               uint8_t *obs, char *err, size_t err_len);

/* Detector error models: parse (NULL + err on failure), stats (detectors, observables, errors), and sample
 * shots [first_shot, first_shot + shots) (first_shot a multiple of 128) under the DEM purpose of the
 * contract, or replay recorded errors (replay != NULL: ceil(errors / 8)-byte rows).  Outputs are bit-packed
 * shot-major rows; errs may be NULL. */
typedef struct oracle_dem oracle_dem;
oracle_dem *oracle_dem_parse(const char *text, char *err, size_t err_len);
void oracle_dem_free(oracle_dem *d);
void oracle_dem_stats(const oracle_dem *d, uint64_t *out3);
int oracle_dem_sample(const oracle_dem *d, uint64_t seed, uint64_t first_shot, uint64_t shots, uint8_t *dets,
                      uint8_t *obs, uint8_t *errs, const uint8_t *replay);

#ifdef __cplusplus
}
#endif

#endif
