// Launch interface of the frame-sampling kernels (kernels.cu).  Host code only sees plain pointers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "program.h"

namespace gfs {

struct KernelArgs {
    const DevOp *ops;
    const uint32_t *pool;
    const uint32_t *tables;
    const DevChan *chans;
    const uint32_t *qubit_orig;
    uint32_t nrows;
    uint32_t ring;
    uint32_t nobs;
    uint32_t nslices;  // slices of `blocks_per_cta` 128-shot blocks in this launch
    uint64_t ndet;
    uint64_t nmeas;
    uint64_t seed;
    uint64_t block0;   // stream position (global 128-shot block index) of local block 0
    uint4 *det_out;    // [local block][ndet] (may be null when ndet == 0)
    uint4 *obs_out;    // [local block][nobs]
    uint4 *meas_out;   // [local block][nmeas] (measurement mode only)
    uint32_t *status;  // device error word, 0 = ok
    uint32_t smem_table_words;  // > 0: copy the first smem_table_words of `tables` into shared memory
    uint32_t smem_ops;          // > 0: copy the op stream (this many ops) into shared memory
    uint4 *ring_global;         // non-null: measurement ring in global memory, [CTA][ring row][block]
    uint64_t ring_cta_stride;   // uint4 entries between consecutive CTAs' regions of ring_global
    // Precomputed noise (noise_kernel, then frame_kernel in hit-list mode); hits == null: the frame kernel
    // draws its noise inline.
    uint64_t *hits;          // hit records (see hit_record() in kernels.cu): slice s's region starts at
                             // s * slice_cap, occurrence k's records at occs[k].off within it
    uint32_t *hit_count;     // [slice][occurrence] records written
    const NoiseOcc *occs;    // the program's noise occurrences in order
    uint32_t n_occ;
    uint64_t slice_cap;      // records per slice region
    uint32_t smem_occ;       // n_occ when the occurrence offsets and the slice's counts are cached in shared
                             // memory, else 0
    uint32_t reset_zero;     // 1: start every shot's Z frame at zero instead of random (Program::reset_norand)
    const uint4 *sweep;      // [local block][nsweep] sweep bits read by sweep feedback; null: all zero
    uint32_t nsweep;
    // Non-null (LaunchShape::frames_global): the X and Z frames live in this CTA's region of a global buffer
    // (frames_cta_stride uint4 entries per CTA) instead of shared memory, for circuits whose frames do not fit.
    uint4 *frames_global;
    uint64_t frames_cta_stride;
    // Lean kernel (frame_lean.cu): the phase list and each phase's instance offset (Program::lean).
    const LeanPhase *lean;
    const uint64_t *lean_inst;
    uint32_t n_lean;
    // Non-null when the lean kernel consumes the hit records: noise_kernel transforms the Paulis of the occurrences
    // the lean plan moved (NoiseOcc.xform, program.h OccXform).
    const OccXform *occ_xform;
};

// Several circuits in one launch (batch_frame_kernel): circuit j owns work items
// slice_prefix[j] .. slice_prefix[j+1]-1, one per slice of its shots.
struct BatchArgs {
    const KernelArgs *circuits;
    const uint32_t *slice_prefix;  // ncircuits + 1 entries
    uint32_t ncircuits;
    uint32_t total_slices;
    uint32_t *counter;             // next unclaimed work item; zero before the launch
    // Hit-list mode (LaunchShape::hits): batch_noise_kernel runs first, one warp per (circuit, slice,
    // occurrence); circuit j owns noise warps warp_prefix[j] .. warp_prefix[j+1]-1.
    const uint64_t *warp_prefix;   // ncircuits + 1 entries
    uint64_t total_noise_warps;
};

struct LaunchShape {
    int blocks_per_cta;  // 1, 2 or 4 blocks of 128 shots per CTA
    int threads;         // threads per CTA
    int grid;            // CTAs (persistent: each walks slices grid-stride)
    size_t smem;         // dynamic shared memory bytes
    bool ring_global;    // measurement ring in global memory (per-CTA region) instead of shared memory
    bool hits = false;   // hit-list mode (noise precomputed by noise_kernel)
    bool frames_global = false;  // X / Z frames in global memory (one block per CTA only)
};

// `nrows` = frame rows held in shared memory (0 when the frames are in global memory).
size_t frame_smem_bytes(uint32_t nrows, uint32_t ring, uint32_t nobs, int blocks_per_cta, uint32_t table_words,
                        uint32_t smem_ops, uint32_t smem_occ = 0);
// Frame kernel; in hit-list mode (args.hits != null) noise_kernel must have run on the same arguments.
cudaError_t launch_frame_kernel(const KernelArgs &args, const LaunchShape &shape, cudaStream_t stream);
// Draws every noise hit of every slice into args.hits / args.hit_count: one warp per (slice, occurrence).
// Sets status bit 4 when an occurrence's records do not fit its region (the chunk must then be redone
// with inline noise).
cudaError_t launch_noise_kernel(const KernelArgs &args, int blocks_per_cta, cudaStream_t stream);

// Slices (of blocks_per_cta 128-shot blocks) that one noise-kernel warp draws for an occurrence: several per warp
// keep its screening rounds full and spread one setup over them (d=25, one block per CTA: 4 slices 2.43 ms,
// 8: 2.31, 16: 2.13, 32: 2.18 per 2^20 shots; four-block slices, d=11: 4 slices 0.225 ms, 8: 0.206).
#if defined(__CUDACC__)
__host__ __device__
#endif
constexpr int noise_slices_per_warp_for(int blocks_per_cta) {
    return blocks_per_cta == 1 ? 16 : blocks_per_cta == 2 ? 16 : 8;
}
cudaError_t frame_kernel_max_ctas_per_sm(const LaunchShape &shape, int *out);
// The lean frame kernel (hit-list mode, programs with Program::lean_ok): same results as launch_frame_kernel.
size_t lean_smem_bytes(uint32_t nrows, uint32_t ring, uint32_t nobs, int blocks_per_cta, uint32_t n_lean,
                       uint32_t n_occ, int threads);
cudaError_t launch_frame_kernel_lean(const KernelArgs &args, const LaunchShape &shape, cudaStream_t stream);
cudaError_t frame_kernel_lean_max_ctas_per_sm(const LaunchShape &shape, int *out);
// In hit-list mode (shape.hits) this launches batch_noise_kernel and then the frame kernel.
cudaError_t launch_batch_frame_kernel(const BatchArgs &args, const LaunchShape &shape, cudaStream_t stream);
cudaError_t batch_frame_kernel_max_ctas_per_sm(const LaunchShape &shape, int *out);
// The noise kernel of a batch alone (hit-list mode), and the lean batched frame kernel: batch_noise_kernel, then
// the lean kernel over the work items (every circuit with a lean phase list; shape.smem covers the largest).
cudaError_t launch_batch_noise_kernel(const BatchArgs &args, int blocks_per_cta, cudaStream_t stream);
cudaError_t launch_batch_frame_kernel_lean(const BatchArgs &args, const LaunchShape &shape, cudaStream_t stream);
cudaError_t batch_frame_kernel_lean_max_ctas_per_sm(const LaunchShape &shape, int *out);

// Transposes [local block][rows] bit-rows (128 shots per entry) of up to three sources, concatenated
// (src0 rows, then src1, then src2), into shot-major output rows.  `xor_rows` (optional) is a bit vector over the
// concatenated rows that is XORed into every shot (the reference sample of measurement sampling).
struct TransposeArgs {
    const uint4 *src0;
    uint64_t n0;
    const uint4 *src1;
    uint64_t n1;
    const uint4 *src2;
    uint64_t n2;
    const uint8_t *xor_rows;
    uint64_t nshots;
    uint8_t *out;
    uint64_t out_stride;  // bytes between consecutive shots in `out`
    int bit_packed;       // 1: little-endian bit-packed bytes; 0: one byte (0/1) per bit
};
cudaError_t launch_transpose(const TransposeArgs &args, cudaStream_t stream);

// Measurements to detection events (CompiledMeasurementsToDetectionEventsConverter).
// Shot-major bit-packed rows (in_stride bytes apart, nbits bits each) into [local block][nbits] uint4 rows
// (128 shots per uint4); bits of shots past nshots are zero.
struct RowsInArgs {
    const uint8_t *in;
    uint64_t in_stride;
    uint64_t nshots;
    uint64_t nbits;
    uint4 *out;
};
cudaError_t launch_rows_from_shots(const RowsInArgs &args, cudaStream_t stream);

// out row o of block b = XOR of rows[b][idx[j]] for j in [off[o], off[o+1]), inverted when bit o of `expect`
// is set, XORed with the base rows when given; outputs [0, D) go to dets[b][.], [D, D + O) to obs[b][.].
struct FoldArgs {
    const uint4 *rows;
    uint64_t nrows;
    const uint32_t *off;
    const uint32_t *idx;
    const uint8_t *expect;
    uint64_t D, O;
    uint64_t nblk;
    uint4 *dets;
    uint4 *obs;
    const uint4 *base_dets;  // non-null: XORed into the outputs ([block][D] and [block][O], e.g. the frame
    const uint4 *base_obs;   // kernel's detectors and observables of the sweep-driven flips)
};
cudaError_t launch_fold(const FoldArgs &args, cudaStream_t stream);

// Detector-error-model sampling (gfs_dem_*).  A probability group of error mechanisms: its mechanisms are
// units[first .. first + n); gap table at tables[table] (when 0 < p < 1).
struct DemGroup {
    uint32_t first;
    uint32_t n;
    uint32_t table;
    uint32_t flags;  // bit 0: p > 0, bit 1: p >= 1
    float inv_c;
    uint32_t pad[3];
};

// One warp per (128-shot block, chunk of up to 1024 mechanisms of one group): the chunk's segments are walked
// under the contract (purpose GFS_P_DEM, instance = group, segment index within the group) and each error
// XORs its symptoms into dets[block][.] / obs[block][.] (which the caller zeroes) and, when errs != null,
// sets its bit in errs[block][mechanism].
struct DemArgs {
    const DemGroup *groups;
    const uint32_t *units;
    const uint32_t *sym_off;
    const uint32_t *sym;
    const uint32_t *tables;
    const uint32_t *chunk_group;
    const uint32_t *chunk_unit0;
    const uint32_t *chunk_units;
    uint32_t nchunks;
    uint64_t seed;
    uint64_t block0;  // stream position of local block 0
    uint64_t nblk;
    uint64_t D, O, E;
    uint4 *dets, *obs, *errs;
};
cudaError_t launch_dem_sample(const DemArgs &args, cudaStream_t stream);

// Decoder feed (gfs_sample_for_decoder): dense shot-major bit-packed detector rows (drow bytes each) and
// observable rows (orow bytes each) on the device.  A shot is dropped when its detector row has a set bit
// under the postselection mask, given as nmask (byte index, byte bits) pairs.  Shots are handled in groups
// of kFeedGroup: group_kept[g] first counts group g's kept shots, then (after launch_feed_scan) holds the
// output row of its first kept shot.
constexpr uint32_t kFeedGroup = 1024;
struct FeedArgs {
    const uint8_t *dets;
    const uint8_t *obs;
    uint64_t drow, orow, nshots;
    const uint32_t *mask_idx;
    const uint8_t *mask_bits;
    uint32_t nmask;
    uint32_t *group_kept;
    uint8_t *keep;                // per shot: 1 kept, 0 dropped
    unsigned long long *counts;   // [0] += set bits over the detector rows, [1] += dropped shots
    uint8_t *cdets, *cobs;        // kept rows, in shot order
    uint32_t *dst;                // per shot: its kept row's index, or 0xFFFFFFFF when dropped
};
// Copies n words of device memory to `dst`, a mapped page-locked host buffer, with a kernel: small results reach
// the host without a device-to-host copy, which could queue behind a large copy on the copy engine.
cudaError_t launch_publish_words(const uint32_t *src, uint32_t *dst, uint32_t n, cudaStream_t stream);
cudaError_t launch_feed_popcount(const FeedArgs &args, cudaStream_t stream);
cudaError_t launch_feed_flags(const FeedArgs &args, cudaStream_t stream);
cudaError_t launch_feed_scan(const FeedArgs &args, cudaStream_t stream);
cudaError_t launch_feed_compact(const FeedArgs &args, cudaStream_t stream);

// Shared-memory load+store throughput of the current device (bytes per second over all SMs).
cudaError_t measure_smem_peak(double *bytes_per_s);
// 32-bit three-input logic ops per second and Philox4x32-10 calls per second over the whole GPU.
cudaError_t measure_int_peaks(double *lop3_per_s, double *philox_per_s);

}  // namespace gfs
