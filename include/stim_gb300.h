/*
 * stim_gb300.h -- C ABI of the GB300 frame sampler (libstim_gb300.so).
 *
 * Plain pointers and sizes only.  Every entry point returns a gfs_status; on failure
 * gfs_last_error() returns a thread-local message whose text matches the reference's exception
 * message for the same condition.  No C++ exception crosses this boundary.
 *
 * The boundary replaces stim::FrameSimulator<W> as held by the reference's compiled samplers:
 *   - CompiledDetectorSampler  (src/stim/py/compiled_detector_sampler.pybind.h:28-54,
 *                               compiled_detector_sampler.pybind.cc:28-86)
 *   - CompiledMeasurementSampler (src/stim/py/compiled_measurement_sampler.pybind.cc:31-83)
 * and the batch drivers they call (src/stim/simulators/frame_simulator_util.inl:21-35, 290-315).
 */
#ifndef STIM_GB300_H
#define STIM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gfs_status {
    GFS_OK = 0,
    GFS_ERR_INVALID_ARGUMENT = 1, /* reference: std::invalid_argument -> ValueError */
    GFS_ERR_OUT_OF_RANGE = 2,     /* reference: std::out_of_range -> IndexError (e.g. measure_record_batch.inl:84-92) */
    GFS_ERR_CUDA = 3,             /* a CUDA runtime call failed or no device is present */
    GFS_ERR_OUT_OF_MEMORY = 4,
    GFS_ERR_INTERNAL = 5
} gfs_status;

typedef struct gfs_circuit gfs_circuit; /* parsed circuit (host) */
typedef struct gfs_sampler gfs_sampler; /* lowered program + device state + random stream position */

/* Sampling modes. */
#define GFS_MODE_DETECTIONS 0u   /* CompiledDetectorSampler */
#define GFS_MODE_MEASUREMENTS 1u /* CompiledMeasurementSampler */

/* Layout flags of gfs_sample_detections (compiled_detector_sampler.pybind.cc:216-322). */
#define GFS_PREPEND_OBSERVABLES 1u
#define GFS_APPEND_OBSERVABLES 2u
#define GFS_BIT_PACKED 4u

/* Thread-local message of the last failed call on this thread. */
const char *gfs_last_error(void);

/* Library / device information.  out[0] = device count. */
gfs_status gfs_device_count(int *out);

/*
 * Device facts used by the runtime: info[0] = SMs, [1] = opt-in shared memory per CTA (bytes),
 * [2] = shared memory per SM, [3] = pageable host memory access (1 when kernels may write ordinary host
 * memory, as on Grace-based systems), [4] = that access uses host page tables, [5] = SM clock (kHz),
 * [6] = compute capability x 10, [7] = L2 bytes.
 */
gfs_status gfs_device_info(int device, int64_t *info8);

/*
 * Parses .stim text (replaces stim::Circuit(text), src/stim/circuit/circuit.cc:302-310).
 * stats[0..5] = num_qubits, num_measurements, num_detectors, num_observables, max_lookback,
 * number of instructions with REPEAT unrolled.
 */
gfs_status gfs_circuit_parse(const char *text, size_t len, gfs_circuit **out);
gfs_status gfs_circuit_stats(const gfs_circuit *c, uint64_t *stats6);
void gfs_circuit_free(gfs_circuit *c);

/*
 * Lowers the circuit for `mode` on the host only (no device needed) and reports the program:
 * info[0] = device ops, [1] = pool words, [2] = compacted qubit rows, [3] = measurement ring rows,
 * [4] = noise channels, [5] = deepest REPEAT nesting, [6] = shared-memory bytes per 128-shot block,
 * [7] = detectors.  Fails with the same errors as gfs_sampler_create's lowering step.
 */
gfs_status gfs_program_info(const gfs_circuit *c, uint32_t mode, uint64_t *info8);
/*
 * sample_write: samples `shots` shots and writes them to `path` in a result format ("01", "b8", "r8",
 * "hits", "dets", "ptb64"; null = "01").  Detections: flags may prepend or append observables, or
 * obs_path (with obs_format) writes them to a file of their own; at most one of the three.  dets names
 * detectors D<k>, observables L<k>, measurements M<k>.  ptb64 needs a multiple of 64 shots.
 * Replaces CompiledDetectorSampler.sample_write (src/stim/py/compiled_detector_sampler.pybind.cc:88-141,
 * 357-415) and CompiledMeasurementSampler.sample_write (src/stim/py/compiled_measurement_sampler.pybind.cc:
 * 37-45, 245-290); the byte layouts are src/stim/io/measure_record_writer.cc:61-211.
 */
gfs_status gfs_sample_write_detections(gfs_sampler *s, uint64_t shots, const char *path, const char *format,
                                       uint32_t flags, const char *obs_path, const char *obs_format);
gfs_status gfs_sample_write_measurements(gfs_sampler *s, uint64_t shots, const char *path, const char *format,
                                         const uint8_t *ref_sample);

/*
 * The circuit's reference sample: its noiseless version run once on a host stabilizer tableau with every
 * random measurement outcome forced to 0, bit-packed little-endian into out[0 .. (measurements+7)/8).
 * Replaces TableauSimulator<W>::reference_sample_circuit (src/stim/simulators/tableau_simulator.inl:
 * 1435-1438) behind Circuit.reference_sample() and compile_sampler() (src/stim/circuit/circuit.pybind.cc,
 * src/stim/py/compiled_measurement_sampler.pybind.cc:63-83).  Host only, no GPU needed.
 */
gfs_status gfs_circuit_reference_sample(const gfs_circuit *c, uint8_t *out, uint64_t nbytes);
/* Noise occurrences met by one pass over the lowered program (loops unrolled) and the expected number of
 * noise hits per 128-shot block: the sizes of the hit lists (host only, no GPU needed). */
gfs_status gfs_program_noise(const gfs_circuit *c, uint32_t mode, uint64_t *occurrences, double *hits_per_block);

/*
 * Lowers the circuit for `mode` and uploads it to CUDA device `device`; the random stream starts at
 * shot 0 of `seed` (replaces the sampler constructors, compiled_detector_sampler.pybind.cc:28-32,151-154
 * and compiled_measurement_sampler.pybind.cc:63-83).  Successive sample calls continue the stream.
 * Circuits whose frames do not fit in shared memory (about 7,000 qubits and up) are sampled with the frames
 * in device memory (slower, same bits); the batched engine, the server and
 * gfs_sample_detections_device_noalloc reject them.
 */
gfs_status gfs_sampler_create(const gfs_circuit *c, uint32_t mode, uint64_t seed, int device, gfs_sampler **out);
void gfs_sampler_free(gfs_sampler *s);

/*
 * Detection events of `shots` shots into caller-owned HOST memory (mirrors sample(shots,
 * prepend_observables, append_observables, bit_packed, dets_out, obs_out), compiled_detector_sampler.pybind.cc:34-86).
 * dets: shots rows of `dets_stride` bytes holding the detectors (with observables prepended/appended per
 * flags), bit-packed little-endian when GFS_BIT_PACKED, else one 0/1 byte per bit.  obs (may be NULL):
 * the observables alone, same packing, `obs_stride` bytes per shot.
 */
gfs_status gfs_sample_detections(gfs_sampler *s, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dets_stride,
                                 uint8_t *obs, uint64_t obs_stride);

/*
 * Measurement results into caller-owned HOST memory (mirrors CompiledMeasurementSampler.sample,
 * compiled_measurement_sampler.pybind.cc:31-35 -> frame_simulator_util.inl:290-315).  ref_sample: the
 * reference sample, ceil(num_measurements/8) bytes bit-packed, XORed into every shot; NULL = all zero
 * (skip_reference_sample=True).
 */
gfs_status gfs_sample_measurements(gfs_sampler *s, uint64_t shots, uint32_t flags, const uint8_t *ref_sample,
                                   uint8_t *out, uint64_t out_stride);

/*
 * Same as gfs_sample_detections but the outputs are DEVICE pointers on the sampler's device (for callers
 * that keep results in HBM, e.g. a decoder on the same GPU).  The call returns when the results are
 * written.
 */
gfs_status gfs_sample_detections_device(gfs_sampler *s, uint64_t shots, uint32_t flags, void *dets,
                                        uint64_t dets_stride, void *obs, uint64_t obs_stride);

/*
 * Allocation-free variant of gfs_sample_detections_device.  No counterpart in the reference.
 *
 * For callers that must not allocate or free device memory while they sample: for example a real-time
 * decoding loop whose HBM is reserved up front by its own pool allocator, or a loop that cannot afford
 * cudaMalloc/cudaFree's implicit device synchronization and latency.  Each call allocates nothing:
 * the frame kernel's scratch (16 bytes per 128-shot block per detector or observable) lives in a
 * fixed 64 MiB file-scope __device__ array (stim_gb300/csrc/noalloc.cu) that every GPU loading the
 * library holds until the process exits, and the outputs are the caller's device buffers, as in
 * gfs_sample_detections_device.  Creating the sampler (gfs_sampler_create) still allocates the lowered
 * program once, at set-up.
 *
 * The first call on a device looks up the array's device address (cudaGetSymbolAddress, with that
 * device current); make that first call before any stream capture.  CUDA loads modules lazily by
 * default, so that first call is also when the array is placed in the device's memory: make it before
 * reserving the rest of HBM for your own pool.  Circuits whose measurement ring or frames need global
 * memory (beyond the array) are rejected with GFS_ERR_INVALID_ARGUMENT.  Circuits needing more than 64 MiB
 * of scratch for one CTA's slice of shots are rejected with GFS_ERR_INVALID_ARGUMENT.  Larger shot
 * counts are processed in chunks that fit.  All calls share the array and it keeps the last call's
 * contents (nothing in it needs to start at zero: every scratch row is written before it is read).
 * Calls from this process to one device are serialized by a lock; calls that overlap on the GPU by
 * other means (e.g. another copy of the library in the same process) race on the array.
 */
gfs_status gfs_sample_detections_device_noalloc(gfs_sampler *s, uint64_t shots, uint32_t flags, void *dets,
                                                uint64_t dets_stride, void *obs, uint64_t obs_stride);

/*
 * Sampling for a decoder, as sinter's StimThenDecodeSampler does it
 * (glue/sample/src/sinter/_decoding/_stim_then_decode_sampler.py:170-190): `shots` shots of detection
 * events, bit-packed, observables separate.  Shots whose detector row has a set bit under
 * `postselection_mask` (ceil(D / 8) bytes, little-endian bits like the rows; NULL keeps every shot) are
 * dropped on the device, and the kept shots' rows go, in shot order, to the first rows of the host buffers
 * `dets` / `obs` (room for `shots` rows each; either may be NULL).  out3[0] = shots kept, out3[1] = shots
 * dropped, out3[2] = detection events (set detector bits) over all `shots` shots before dropping, sinter's
 * 'detection_events' count.  The stream position advances by `shots` as in gfs_sample_detections.
 */
gfs_status gfs_sample_for_decoder(gfs_sampler *s, uint64_t shots, const uint8_t *postselection_mask, uint8_t *dets,
                                  uint64_t dets_stride, uint8_t *obs, uint64_t obs_stride, uint64_t *out3);

/*
 * Device timings (milliseconds, CUDA events on the sampler's stream) of the last sample call:
 * out[0] = frame kernel, out[1] = transpose kernel(s), out[2] = device->host copies, out[3] = whole call.
 * counts[0] = frame-kernel launches, counts[1] = transpose launches.
 */
gfs_status gfs_sampler_last_timings(const gfs_sampler *s, double *out4, uint64_t *counts2);

/*
 * Launch shape: blocks_per_cta in {1, 2, 4} (128-shot blocks held in one CTA's shared memory),
 * threads per CTA (multiple of 32, <= 256), grid CTAs (0 = one full wave of resident CTAs).
 * Fails when the circuit's state does not fit shared memory with that many blocks.
 */
gfs_status gfs_sampler_set_shape(gfs_sampler *s, int blocks_per_cta, int threads, int grid);
gfs_status gfs_sampler_get_shape(const gfs_sampler *s, int *blocks_per_cta, int *threads, int *grid,
                                 uint64_t *smem_bytes);

/*
 * Where the measurement record window lives: 0 = shared memory, 1 = a per-CTA region of a global
 * (L2-resident) buffer, which frees shared memory for more resident CTAs; -1 = choose automatically (the
 * default).  Results do not depend on it.
 */
gfs_status gfs_sampler_set_ring_placement(gfs_sampler *s, int placement);

/*
 * Measures the shared-memory load+store throughput of `device` with a project-written probe kernel
 * (bytes per second summed over all SMs).  The frame kernel's roofline denominator.  No counterpart in
 * the reference (it has no GPU code).
 */
gfs_status gfs_measure_smem_peak(int device, double *bytes_per_s);

/*
 * Measures the integer-issue peaks of `device` with project-written probe kernels: 32-bit three-input logic
 * operations per second (lop3, the frame kernel's arithmetic) and Philox4x32-10 generator calls per second
 * (the noise kernel's random-draw work), each summed over all SMs.  Roofline denominators for the
 * instruction-bound kernels.  No counterpart in the reference (it has no GPU code).
 */
gfs_status gfs_measure_int_peaks(int device, double *lop3_per_s, double *philox_per_s);

/* Maximum shots per device chunk (bounds HBM use); 0 restores the default. */
gfs_status gfs_sampler_set_chunk_shots(gfs_sampler *s, uint64_t shots);
/*
 * Stream position (the global index of the next shot; a multiple of 128).  Every shot's bits depend only on
 * (circuit, seed, global shot index), so ranks that set disjoint positions sample disjoint parts of one stream
 * (sharding by shot range).  No counterpart in the reference, whose sampler always continues one mt19937_64.
 */
gfs_status gfs_sampler_set_stream_position(gfs_sampler *s, uint64_t shot);
gfs_status gfs_sampler_get_stream_position(const gfs_sampler *s, uint64_t *shot);

/*
 * Noise generation: 1 (default, -1 = automatic) draws every noise hit of a chunk in a separate kernel
 * into a list that the frame kernel then applies; 0 draws noise inside the frame kernel.  Results are
 * identical either way.  No counterpart in the reference.
 */
gfs_status gfs_sampler_set_noise_mode(gfs_sampler *s, int mode);
/*
 * Frame kernel for hit-list launches: 1 (default, -1 = automatic) the lean kernel when the program has a lean
 * phase list (no correlated errors, heralds or sweep feedback; compact unit lists; at most two loop levels),
 * 0 the generic kernel.  Results are identical either way.  gfs_sampler_get_frame_kernel reports which one the
 * next hit-list launch uses (1 lean, 0 generic).  No counterpart in the reference.
 */
gfs_status gfs_sampler_set_frame_kernel(gfs_sampler *s, int kind);
gfs_status gfs_sampler_get_frame_kernel(const gfs_sampler *s, int *kind);
/* Noise-kernel time (ms) of the last sample call; gfs_sampler_last_timings' frame time excludes it. */
gfs_status gfs_sampler_last_noise_ms(const gfs_sampler *s, double *ms);
/* Hit-list region capacity in records per noise occurrence and slice (0 = automatic: expected hits plus a
 * wide margin).  A chunk whose hits do not fit is redone with inline noise, with identical results; a
 * small capacity exercises that. */
gfs_status gfs_sampler_set_hit_capacity(gfs_sampler *s, uint64_t records);
/* Kernel launches of the last sample call: frame, transpose, noise; plus hit-list overflows (chunks redone
 * with inline noise) over the sampler's life. */
gfs_status gfs_sampler_last_counts(const gfs_sampler *s, uint64_t *counts4);

/*
 * Launch-shape autotuner: times the frame kernel on `trial_shots` shots (0 = 2^18) for each candidate
 * shape (blocks per CTA x threads x ring placement) that fits and keeps the fastest; *best_ms (may be
 * null) receives its time.  The sampler's stream position does not move and results never depend on the
 * shape.  No counterpart in the reference (its CPU sampler has no launch shape).
 */
gfs_status gfs_sampler_autotune(gfs_sampler *s, uint64_t trial_shots, double *best_ms);

/*
 * Batched sampling: the next shots of many detection samplers in ONE persistent frame-kernel launch
 * (work items = (circuit, 128-shot slice), claimed dynamically by the CTAs, most expensive circuits
 * first), followed by each circuit's transpose; the launch sequence is captured as a CUDA graph and
 * replayed while shot counts, destinations and launch shape stay the same.  Entry j returns exactly what
 * gfs_sample_detections(samplers[j], shots[j], ...) would have returned at that point, and advances that
 * sampler the same way (a sampler listed twice continues its stream from the first entry to the second).
 * The samplers must stay alive, on one device, and unused elsewhere while the batch is in use.
 * No counterpart in the reference, whose nearest equivalent is one CompiledDetectorSampler per circuit
 * (src/stim/py/compiled_detector_sampler.pybind.cc:216-322).
 */
typedef struct gfs_batch gfs_batch;
gfs_status gfs_batch_create(gfs_sampler *const *samplers, size_t n, gfs_batch **out);
void gfs_batch_free(gfs_batch *b);
/* dets[j] / obs[j]: device pointers (null skips that output); strides in bytes per shot. */
gfs_status gfs_batch_sample_detections_device(gfs_batch *b, const uint64_t *shots, uint32_t flags, void *const *dets,
                                              const uint64_t *dets_stride, void *const *obs,
                                              const uint64_t *obs_stride);
/* Same with host destinations (copied out of a device staging arena). */
gfs_status gfs_batch_sample_detections(gfs_batch *b, const uint64_t *shots, uint32_t flags, uint8_t *const *dets,
                                       const uint64_t *dets_stride, uint8_t *const *obs, const uint64_t *obs_stride);
/* Launch shape of the batched kernel (ring_placement as in gfs_sampler_set_ring_placement). */
gfs_status gfs_batch_set_shape(gfs_batch *b, int blocks_per_cta, int threads, int ring_placement);
gfs_status gfs_batch_get_shape(const gfs_batch *b, int *blocks_per_cta, int *threads, int *grid, uint64_t *smem_bytes,
                               int *ring_global);
/* Times each candidate shape on these shot counts (samplers do not advance) and keeps the fastest. */
gfs_status gfs_batch_autotune(gfs_batch *b, const uint64_t *shots, double *best_ms);
/* out4: frame, transposes, host copies, whole call (ms); counts4: frame launches, transpose launches,
 * graph launches, graph builds (cumulative). */
gfs_status gfs_batch_last_timings(const gfs_batch *b, double *out4, uint64_t *counts4);

/*
 * Request server with continuous batching on one device.  A worker thread keeps lowered circuits in a
 * device-resident cache keyed by circuit text, cuts requests into chunks of at most max_chunk_shots
 * (0 = 2^18) shots, and admits chunks first come first served into the next batched launch while the
 * batch's device-memory footprint stays within half of hbm_budget_bytes (0 = 8 GiB; two batches are in
 * flight at a time).  Request `ticket` returns exactly
 * Circuit(text).compile_detector_sampler(seed=seed).sample(shots, flags...), whatever it was batched
 * with.  Destinations are host memory (device_out = 0; copied out of device staging) or device memory
 * (device_out = 1) and must stay valid until gfs_server_wait reports the request done.
 * No counterpart in the reference (src/stim/py/compiled_detector_sampler.pybind.cc:216-322 is the
 * per-request call this replaces).
 */
typedef struct gfs_server gfs_server;
gfs_status gfs_server_create(int device, uint64_t hbm_budget_bytes, uint64_t max_chunk_shots, gfs_server **out);
/* Drains the queue, then stops the worker. */
void gfs_server_free(gfs_server *s);
gfs_status gfs_server_submit(gfs_server *s, const char *text, size_t len, uint64_t shots, uint64_t seed,
                             uint32_t flags, int device_out, void *dets, uint64_t dets_stride, void *obs,
                             uint64_t obs_stride, uint64_t *ticket);
/* Waits up to timeout_s seconds (< 0: forever).  *done = 1 once the request finished; its status is the
 * request's own (an error message when it failed).  A finished ticket is collected and cannot be waited
 * on again.  *latency_ms (may be null) = submit to completion. */
gfs_status gfs_server_wait(gfs_server *s, uint64_t ticket, double timeout_s, int *done, double *latency_ms);
/* out12: completed, failed, p50 latency ms, p99 latency ms, aggregate Gbit/s (detection + observable bits
 * of completed requests / first submit to last completion), batches, mean chunks per batch, cache hits,
 * cache misses, longest queue, bits completed, seconds spanned. */
gfs_status gfs_server_stats(gfs_server *s, double *out12);
/* Admission counters, out8: requests submitted (accepted into the queue), rejected at submission (invalid
 * circuit or arguments, or a circuit too large for the server), completed, failed after admission, queued now
 * (shots not yet handed to a batch), not yet finished, longest queue seen, chunks admitted into batches. */
gfs_status gfs_server_counters(gfs_server *s, uint64_t *out8);

/*
 * Measurements to detection events (replaces CompiledMeasurementsToDetectionEventsConverter,
 * src/stim/simulators/measurements_to_detection_events.pybind.cc:80-150, behind
 * Circuit.compile_m2d_converter(*, skip_reference_sample), and measurements_to_detection_events_helper,
 * measurements_to_detection_events.inl:29-131).  ref_sample = the circuit's reference sample bit-packed
 * (gfs_circuit_reference_sample), or null for all zeros (skip_reference_sample = True).
 * stats4 = measurements, detectors, observables, sweep bits.
 * gfs_m2d_convert: meas = `shots` host rows of ceil(measurements / 8) bit-packed bytes, meas_stride bytes
 * apart; flags = GFS_BIT_PACKED and at most one of GFS_PREPEND_OBSERVABLES / GFS_APPEND_OBSERVABLES; dets and
 * obs (either may be null) as in gfs_sample_detections.  Detector k fires when the parity of its measurements
 * differs from their parity in the reference sample; observables likewise.  sweep (may be null) = host rows
 * of ceil(sweep bits / 8) bit-packed bytes, sweep_stride bytes apart: the sweep-controlled Paulis they switch
 * on flip measurement results (and observables' Pauli terms) as in the reference, through a noiseless,
 * randomization-free run of the frame kernel over the sweep table (skipped when every bit is zero or no
 * operation is sweep-controlled).
 */
typedef struct gfs_m2d gfs_m2d;
gfs_status gfs_m2d_create(const gfs_circuit *c, const uint8_t *ref_sample, int device, gfs_m2d **out);
void gfs_m2d_free(gfs_m2d *m);
gfs_status gfs_m2d_stats(const gfs_m2d *m, uint64_t *stats4);
gfs_status gfs_m2d_convert(gfs_m2d *m, uint64_t shots, const uint8_t *meas, uint64_t meas_stride,
                           const uint8_t *sweep, uint64_t sweep_stride, uint32_t flags, uint8_t *dets,
                           uint64_t dets_stride, uint8_t *obs, uint64_t obs_stride);
/*
 * File to file (replaces CompiledMeasurementsToDetectionEventsConverter.convert_file,
 * measurements_to_detection_events.pybind.cc:45-77, and the CLI's `stim m2d`): measurement records (and, when
 * sweep_path is non-null, as many sweep records) in one of the result formats "01", "b8", "r8", "hits", "dets",
 * "ptb64" (null format = "01"); detection events written to dets_path (observables appended when
 * append_observables != 0) and observables to obs_path when non-null.  The reference's reader and writer error
 * messages.
 */
/*
 * Host only (replaces stim.read_shot_data_file, src/stim/io/read_write.pybind.cc:97-145): the records of a result
 * file, each num_measurements + num_detectors + num_observables bits (dets tokens M / D / L in that order),
 * bit-packed into `out` (ceil(bits / 8) bytes per record, room for capacity_shots records); *shots = records read.
 */
gfs_status gfs_read_shot_data_file(const char *path, const char *format, uint64_t num_measurements,
                                   uint64_t num_detectors, uint64_t num_observables, uint8_t *out,
                                   uint64_t capacity_shots, uint64_t *shots);
/*
 * Host only (replaces stim.write_shot_data_file, src/stim/io/read_write.pybind.cc:147-183): `shots` bit-packed
 * records (`stride` bytes apart) of num_measurements, or num_detectors + num_observables, bits written to `path`
 * in a result format (dets tokens M<k>, or D<k> then L<k>).
 */
gfs_status gfs_write_shot_data_file(const uint8_t *rows, uint64_t stride, uint64_t shots, const char *path,
                                    const char *format, uint64_t num_measurements, uint64_t num_detectors,
                                    uint64_t num_observables);
gfs_status gfs_m2d_convert_file(gfs_m2d *m, const char *meas_path, const char *meas_format, const char *sweep_path,
                                const char *sweep_format, const char *dets_path, const char *dets_format,
                                int append_observables, const char *obs_path, const char *obs_format);

/*
 * Detector-error-model sampling (replaces DemSampler<W>, src/stim/simulators/dem_sampler.inl:27-77, behind
 * DetectorErrorModel.compile_sampler(seed=...).sample(shots, bit_packed, return_errors,
 * recorded_errors_to_replay), src/stim/simulators/dem_sampler.pybind.cc:40-80; the text format is
 * src/stim/dem/detector_error_model.cc:195-360).
 * gfs_dem_parse_stats: host only; stats3 = detectors, observables, error mechanisms.
 * gfs_dem_sample: `shots` rows of detector / observable / error bits (GFS_BIT_PACKED or one byte per bit;
 * each pointer may be null).  replay = null samples the next shots of the sampler's stream (the position
 * moves on, as after gfs_sample_detections); otherwise replay holds `shots` bit-packed rows of recorded
 * errors (ceil(errors / 8) bytes, replay_stride apart) whose symptoms are XORed instead, the stream does not
 * move, and errs receives the replayed errors.
 */
typedef struct gfs_dem gfs_dem;
gfs_status gfs_dem_parse_stats(const char *text, size_t len, uint64_t *stats3);
gfs_status gfs_dem_create(const char *text, size_t len, uint64_t seed, int device, gfs_dem **out);
void gfs_dem_free(gfs_dem *d);
gfs_status gfs_dem_sample(gfs_dem *d, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dets_stride,
                          uint8_t *obs, uint64_t obs_stride, uint8_t *errs, uint64_t errs_stride,
                          const uint8_t *replay, uint64_t replay_stride);

#ifdef __cplusplus
}
#endif

#endif /* STIM_GB300_H */
