// Host runtime shared by the C ABI entry points: CUDA error mapping, device buffers, and the sampler
// object (lowered program on the device, stream, launch shape, chunked kernel launches).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/stim_gb300.h"
#include "circuit.h"
#include "gfs_contract.h"
#include "kernels.h"
#include "lower.h"

namespace gfs_rt {

extern thread_local std::string g_err;

struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t c, const char *what) : std::runtime_error(std::string(what) + ": " + cudaGetErrorString(c)), code(c) {
    }
};

inline void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        throw CudaError(e, what);
    }
}

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    int device = -1;
    void ensure(size_t bytes, int dev) {
        if (bytes <= n && p) {
            return;
        }
        release();
        if (bytes == 0) {
            return;
        }
        ck(cudaMalloc(&p, bytes), "cudaMalloc");
        n = bytes;
        device = dev;
    }
    void release() {
        if (p) {
            cudaFree(p);
        }
        p = nullptr;
        n = 0;
    }
    ~DevBuf() {
        release();
    }
};

template <typename T>
void upload(DevBuf &b, const std::vector<T> &v, int dev, cudaStream_t s) {
    size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    b.ensure(bytes, dev);
    if (!v.empty()) {
        ck(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    }
}

inline uint64_t pad32(uint64_t n) {
    return (n + 31) & ~(uint64_t)31;
}

inline gfs_status fail(gfs_status st, const std::string &msg) {
    g_err = msg;
    return st;
}

template <typename F>
gfs_status guarded(F f) {
    try {
        f();
        return GFS_OK;
    } catch (const std::out_of_range &e) {
        return fail(GFS_ERR_OUT_OF_RANGE, e.what());
    } catch (const std::invalid_argument &e) {
        return fail(GFS_ERR_INVALID_ARGUMENT, e.what());
    } catch (const CudaError &e) {
        return fail(e.code == cudaErrorMemoryAllocation ? GFS_ERR_OUT_OF_MEMORY : GFS_ERR_CUDA, e.what());
    } catch (const std::bad_alloc &) {
        return fail(GFS_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(GFS_ERR_INTERNAL, e.what());
    }
}

}  // namespace gfs_rt

// Internal header: the runtime's own translation units use these helpers unqualified.
using namespace gfs_rt;

struct gfs_circuit {
    gfs::Circuit circuit;
    gfs::CircuitStats stats;
};

struct gfs_sampler {
    using DevBuf = gfs_rt::DevBuf;
    int device = 0;
    uint32_t mode = 0;
    uint64_t seed = 0;
    uint64_t next_block = 0;
    gfs::Program prog;
    DevBuf d_ops, d_pool, d_tables, d_chans, d_orig, d_status;
    DevBuf det_tmp, obs_tmp, meas_tmp, out_tmp, ref_bits, ring_buf, frames_buf;
    DevBuf feed_rows[2], feed_compact[2], feed_aux[2];  // gfs_sample_for_decoder (feed.cc), per pipeline slot
    // sample_write (capi.cc), two pipeline slots: a chunk's device rows (detectors or measurements, and observables
    // for their own file), the file bytes the device formatter makes of them (one buffer per output file), page-locked
    // host copies of those bytes, and events for the formatter's end and the copies' end.
    struct WriteSlot {
        DevBuf rows, obs, out[2];
        uint8_t *host[2] = {nullptr, nullptr};
        size_t host_cap[2] = {0, 0};
        uint64_t bytes[2] = {0, 0};
        FILE *file[2] = {nullptr, nullptr};
        cudaEvent_t formatted = nullptr, copied = nullptr;
        bool pending = false;  // copies queued whose bytes are not written yet
    };
    WriteSlot wslot[2];
    DevBuf fmt_lens, fmt_offs, fmt_sums, fmt_total;  // the variable-length formatter's scratch (shared by the slots)
    const uint4 *sweep_rows = nullptr;  // [local block][nsweep] sweep bits for the next run_frame (m2d.cc)
    // 16 words of mapped page-locked host memory: the status word (word 0) and the decoder feed's counts
    // (words 4-7) are published here by a kernel instead of copied (launch_publish_words).
    uint32_t *h_words = nullptr, *h_words_dev = nullptr;
    uint32_t nsweep = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // device->host copies of host-destination chunks
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t pev[2][4] = {};  // per pipeline slot: chunk start, frame done, transpose done, copy done
    cudaEvent_t ev_noise[3][2] = {};  // around a noise kernel launch: device path, pipeline slots 0 and 1
    int cur_slot = -1;                // pipeline slot of the chunk being enqueued (-1: device path)
    bool noise_pending[3] = {false, false, false};
    double t_noise = 0;
    gfs::LaunchShape shape{};
    int num_sms = 0;
    int ring_pref = -1;  // -1 automatic, 0 shared memory, 1 global memory
    int hits_pref = -1;  // noise drawn by noise_kernel into hit lists: -1 automatic, 0 never, 1 when possible
    bool force_inline = false;  // set while a chunk is redone after its hit list overflowed
    gfs::LaunchShape shape_inline{};  // the same shape for the inline-noise frame kernel
    DevBuf hit_buf, hit_count, d_occs;
    // Lean frame kernel (frame_lean.cu): used for hit-list launches of programs with a phase list, unless
    // lean_pref = 0.  shape_lean mirrors `shape` with the lean kernel's shared memory and occupancy.
    DevBuf d_lean, d_lean_inst, d_occ_xform;
    int lean_pref = -1;  // -1 automatic (lean when possible), 0 never, 1 when possible
    bool lean_ready = false;
    gfs::LaunchShape shape_lean{};
    int occs_blocks = 0;          // blocks per slice the uploaded occurrence regions were planned for
    uint64_t slice_cap = 0;       // records per slice region
    uint64_t n_hit_overflows = 0;
    uint64_t hit_capacity_override = 0;  // records per occurrence region (0 = from the expected hits)
    uint64_t chunk_shots = 0;
    double t_frame = 0, t_transpose = 0, t_copy = 0, t_total = 0;
    uint64_t n_frame = 0, n_transpose = 0, n_noise = 0;

    ~gfs_sampler() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
            if (copy_stream) {
                cudaStreamSynchronize(copy_stream);
                cudaStreamDestroy(copy_stream);
            }
            for (auto &e : ev) {
                if (e) {
                    cudaEventDestroy(e);
                }
            }
            for (auto &slot : pev) {
                for (auto &e : slot) {
                    if (e) {
                        cudaEventDestroy(e);
                    }
                }
            }
            for (auto &pair : ev_noise) {
                for (auto &e : pair) {
                    if (e) {
                        cudaEventDestroy(e);
                    }
                }
            }
            cudaStreamDestroy(stream);
        }
        if (h_words) {
            cudaFreeHost(h_words);
        }
        for (WriteSlot &w : wslot) {
            for (uint8_t *h : w.host) {
                if (h) {
                    cudaFreeHost(h);
                }
            }
            if (w.formatted) {
                cudaEventDestroy(w.formatted);
            }
            if (w.copied) {
                cudaEventDestroy(w.copied);
            }
        }
    }

    // Gap tables go to shared memory for the inline-noise kernel when they are small (up to 16 KiB, two
    // distinct probabilities); hit-list mode draws no noise in the frame kernel and keeps none.
    uint32_t smem_table_words(bool hits = false) const {
        return (!hits && prog.tables.size() * sizeof(uint32_t) <= 16384) ? (uint32_t)prog.tables.size() : 0;
    }

    // Small op streams go to shared memory too (every thread reads every op).
    uint32_t smem_ops() const {
        return prog.ops.size() <= 256 ? (uint32_t)prog.ops.size() : 0;
    }

    // Hit-list mode needs the program's noise occurrences listed (at least one, not too many).
    bool hits_possible() const {
        return hits_pref != 0 && !prog.occs.empty();
    }

    // Occurrence offsets and per-slice counts cached in shared memory in hit-list mode (small lists only).
    uint32_t smem_occ(bool hits) const {
        return (hits && prog.occs.size() <= 1024) ? (uint32_t)prog.occs.size() : 0;
    }

    // tables = false: no gap tables in shared memory whatever the mode (the batched engine, whose inline
    // fallback runs with the hit-list shape's shared-memory size).
    // frames_global: the X / Z frames are in global memory (not counted).
    size_t smem_for(int bpc, bool ring_global, bool hits = false, bool tables = true, bool frames_global = false) const {
        return gfs::frame_smem_bytes(frames_global ? 0 : prog.num_rows, ring_global ? 0 : prog.ring,
                                     (uint32_t)prog.num_observables, bpc, tables ? smem_table_words(hits) : 0,
                                     smem_ops(), smem_occ(hits));
    }

    // ring: 0 = shared memory, 1 = global memory, -1 = whichever keeps more 128-shot blocks resident per SM.
    void choose_shape(int bpc, int threads, int grid, int ring = -1) {
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        num_sms = prop.multiProcessorCount;
        if (ring < 0) {
            auto resident = [&](bool g) {
                gfs::LaunchShape t{bpc, threads, 1, smem_for(bpc, g, hits_possible()), g};
                t.hits = hits_possible();
                if (t.smem > (size_t)prop.sharedMemPerBlockOptin) {
                    return 0;
                }
                int per = 0;
                if (gfs::frame_kernel_max_ctas_per_sm(t, &per) != cudaSuccess) {
                    cudaGetLastError();
                    return 0;
                }
                return per * bpc;
            };
            int in_smem = resident(false), in_global = resident(true);
            ring = (in_smem == 0 || in_global * 2 >= in_smem * 3) ? 1 : 0;
        }
        bool ring_global = ring == 1;
        size_t smem = smem_for(bpc, ring_global);
        // Frames too large for shared memory even with the ring in global memory: one block per CTA with the
        // frames in a per-CTA global region (slower, but no size limit short of device memory).
        const bool frames_global = smem > (size_t)prop.sharedMemPerBlockOptin && bpc == 1 &&
                                   smem_for(1, true, false, true, true) <= (size_t)prop.sharedMemPerBlockOptin;
        if (frames_global) {
            ring_global = true;
            smem = smem_for(1, true, false, true, true);
        }
        if (smem > (size_t)prop.sharedMemPerBlockOptin) {
            throw std::invalid_argument("circuit state (" + std::to_string(smem) +
                                        " bytes) does not fit in shared memory with " + std::to_string(bpc) +
                                        " blocks per CTA");
        }
        if (threads <= 0 || threads > 256 || threads % 32) {
            throw std::invalid_argument("threads per CTA must be a multiple of 32 in [32, 256]");
        }
        gfs::LaunchShape s{bpc, threads, 1, smem, ring_global};
        s.frames_global = frames_global;
        gfs::LaunchShape si = s;
        s.hits = hits_possible();
        s.smem = smem_for(bpc, ring_global, s.hits, true, frames_global);
        if (s.smem > (size_t)prop.sharedMemPerBlockOptin) {
            s.hits = false;  // no room for the occurrence cache: draw noise inline
            s.smem = smem;
        }
        int per_sm = 0, per_sm_inline = 0;
        ck(gfs::frame_kernel_max_ctas_per_sm(s, &per_sm), "occupancy");
        ck(gfs::frame_kernel_max_ctas_per_sm(si, &per_sm_inline), "occupancy");
        if (per_sm < 1 || per_sm_inline < 1) {
            throw std::invalid_argument("frame kernel cannot be resident with this launch shape");
        }
        if (frames_global) {  // bound the global frame buffer: at most eight CTAs per SM
            per_sm = std::min(per_sm, 8);
            per_sm_inline = std::min(per_sm_inline, 8);
        }
        s.grid = grid > 0 ? grid : per_sm * num_sms;
        si.grid = grid > 0 ? grid : per_sm_inline * num_sms;
        shape = s;
        shape_inline = si;
        // The lean kernel's shape: same blocks, threads and ring placement, its own shared memory and occupancy.
        lean_ready = false;
        if (prog.lean_ok && s.hits && !frames_global && !prog.occs.empty()) {
            gfs::LaunchShape l = s;
            l.smem = gfs::lean_smem_bytes(prog.num_rows, ring_global ? 0 : prog.ring, (uint32_t)prog.num_observables,
                                          bpc, (uint32_t)prog.lean.size(), (uint32_t)prog.occs.size(), threads);
            int per_sm_lean = 0;
            if (l.smem <= (size_t)prop.sharedMemPerBlockOptin &&
                gfs::frame_kernel_lean_max_ctas_per_sm(l, &per_sm_lean) != cudaSuccess) {
                cudaGetLastError();
                per_sm_lean = 0;
            }
            if (per_sm_lean >= 1) {
                l.grid = grid > 0 ? grid : per_sm_lean * num_sms;
                shape_lean = l;
                lean_ready = true;
            }
        }
    }

    // Transforms of the occurrences the lean phase list moved (null when it moved none).
    const gfs::OccXform *occ_xform() const {
        return prog.occ_xform.empty() ? nullptr : (const gfs::OccXform *)d_occ_xform.p;
    }

    // Whether a hit-list launch of the current shape runs the lean kernel.
    bool lean_active() const {
        return lean_ready && lean_pref != 0 && shape.hits && !force_inline && sweep_rows == nullptr;
    }

    // Shape without timing: four 128-shot blocks per CTA when two such CTAs fit per SM (small and medium
    // circuits), else one block per CTA of 128 threads, the ring wherever more blocks stay resident.
    // (gfs_sampler_autotune picks by measurement instead.)
    void default_shape() {
        try {
            choose_shape(4, 256, 0, ring_pref);
            if (shape.grid >= 2 * num_sms) {
                return;
            }
        } catch (const std::invalid_argument &) {
        }
        choose_shape(1, 128, 0, ring_pref);
    }

    void init(const gfs_circuit *c, uint32_t m, uint64_t sd, int dev) {
        init_program(gfs::lower(c->circuit, m == GFS_MODE_MEASUREMENTS ? gfs::SampleMode::MEASUREMENTS
                                                                     : gfs::SampleMode::DETECTIONS),
                     m, sd, dev);
    }

    // A sampler over an already lowered program (e.g. the converter's noiseless, sweep-reading one).
    void init_program(gfs::Program &&p, uint32_t m, uint64_t sd, int dev) {
        device = dev;
        mode = m;
        seed = sd;
        prog = std::move(p);
        int count = 0;
        ck(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if (dev < 0 || dev >= count) {
            throw std::invalid_argument("no CUDA device " + std::to_string(dev));
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &e : ev) {
            ck(cudaEventCreate(&e), "cudaEventCreate");
        }
        for (auto &slot : pev) {
            for (auto &e : slot) {
                ck(cudaEventCreate(&e), "cudaEventCreate");
            }
        }
        for (auto &pair : ev_noise) {
            for (auto &e : pair) {
                ck(cudaEventCreate(&e), "cudaEventCreate");
            }
        }
        upload(d_ops, prog.ops, device, stream);
        upload(d_pool, prog.pool, device, stream);
        upload(d_tables, prog.tables, device, stream);
        upload(d_chans, prog.chans, device, stream);
        upload(d_orig, prog.qubit_orig, device, stream);
        if (prog.lean_ok) {
            upload(d_lean, prog.lean, device, stream);
            upload(d_lean_inst, prog.lean_inst, device, stream);
            if (!prog.occ_xform.empty()) {
                upload(d_occ_xform, prog.occ_xform, device, stream);
            }
        }
        d_status.ensure(16, device);
        ck(cudaHostAlloc((void **)&h_words, 64, cudaHostAllocMapped), "cudaHostAlloc");
        ck(cudaHostGetDevicePointer((void **)&h_words_dev, h_words, 0), "cudaHostGetDevicePointer");
        ck(cudaMemsetAsync(d_status.p, 0, 16, stream), "memset");
        default_shape();
        ck(cudaStreamSynchronize(stream), "upload sync");
    }

    uint64_t per_block_bytes(uint64_t out_row_bytes) const {
        uint64_t rows = prog.num_detectors + prog.num_observables + (mode == GFS_MODE_MEASUREMENTS ? prog.num_measurements : 0);
        uint64_t b = rows * 16 + 128 * out_row_bytes;
        if (shape.hits) {
            // Region capacity runs above the expected hits; estimate it generously.
            b += (uint64_t)(prog.hits_per_block * 8 * 2.5) + 64 * 8 * prog.noise_occurrences + prog.noise_occurrences * 4;
        }
        return b;
    }

    uint64_t chunk_blocks(uint64_t out_row_bytes) const {
        uint64_t bpc = (uint64_t)shape.blocks_per_cta;
        if (chunk_shots) {
            uint64_t b = std::max<uint64_t>(1, chunk_shots / 128);
            return ((b + bpc - 1) / bpc) * bpc;
        }
        // Up to 12 GiB (a quarter of the free memory at most) per chunk: a 2^20-shot d=25 call then runs as one
        // chunk, one partly filled last wave instead of three (8.27 -> 8.02 ms for noise + frame + transpose).
        uint64_t budget = (uint64_t)12 << 30;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
            budget = std::min<uint64_t>(budget, free_b / 4);
        }
        uint64_t b = std::max<uint64_t>(1, budget / std::max<uint64_t>(1, per_block_bytes(out_row_bytes)));
        uint64_t wave = (uint64_t)shape.grid * bpc;
        if (b > wave) {
            b = (b / wave) * wave;
        }
        return std::max<uint64_t>(bpc, (b / bpc) * bpc);
    }

    void reset_timings() {
        t_frame = t_transpose = t_copy = t_total = t_noise = 0;
        n_frame = n_transpose = n_noise = 0;
        noise_pending[0] = noise_pending[1] = noise_pending[2] = false;
    }

    // Adds the noise kernel time of the chunk last enqueued in `slot` (-1: device path) once the stream has
    // passed it, and returns it.
    double account_noise(int slot) {
        const int i = slot + 1;
        float ms = 0;
        if (noise_pending[i]) {
            if (cudaEventElapsedTime(&ms, ev_noise[i][0], ev_noise[i][1]) != cudaSuccess) {
                cudaGetLastError();
                ms = 0;
            }
            noise_pending[i] = false;
            t_noise += ms;
        }
        return ms;
    }

    float elapsed(int a, int b) {
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, ev[a], ev[b]), "cudaEventElapsedTime");
        return ms;
    }

    // Runs the frame kernel for nblk blocks starting at stream block `block0`; results land in the tmp buffers.
    // Runs the frame kernel for nblk blocks starting at stream block `block0`; results land in the tmp buffers.
    // In hit-list mode noise_kernel runs first and draws the chunk's noise into hit_buf.
    void run_frame(uint64_t nblk, uint64_t block0) {
        const bool lean = lean_active();
        const gfs::LaunchShape &sh = lean ? shape_lean : (shape.hits && !force_inline) ? shape : shape_inline;
        uint64_t bpc = (uint64_t)sh.blocks_per_cta;
        uint64_t nslices = (nblk + bpc - 1) / bpc;
        uint64_t alloc_blocks = nslices * bpc;
        det_tmp.ensure(std::max<uint64_t>(16, alloc_blocks * prog.num_detectors * 16), device);
        obs_tmp.ensure(std::max<uint64_t>(16, alloc_blocks * prog.num_observables * 16), device);
        if (mode == GFS_MODE_MEASUREMENTS) {
            meas_tmp.ensure(std::max<uint64_t>(16, alloc_blocks * prog.num_measurements * 16), device);
        }
        gfs::KernelArgs a{};
        a.ops = (const gfs::DevOp *)d_ops.p;
        a.pool = (const uint32_t *)d_pool.p;
        a.tables = (const uint32_t *)d_tables.p;
        a.chans = (const gfs::DevChan *)d_chans.p;
        a.qubit_orig = (const uint32_t *)d_orig.p;
        a.reset_zero = prog.reset_norand ? 1u : 0u;
        a.sweep = sweep_rows;
        a.nsweep = nsweep;
        a.nrows = prog.num_rows;
        a.ring = prog.ring;
        a.nobs = (uint32_t)prog.num_observables;
        a.nslices = (uint32_t)nslices;
        a.ndet = prog.num_detectors;
        a.nmeas = prog.num_measurements;
        a.seed = seed;
        a.block0 = block0;
        a.det_out = (uint4 *)det_tmp.p;
        a.obs_out = (uint4 *)obs_tmp.p;
        a.meas_out = (uint4 *)meas_tmp.p;
        a.status = (uint32_t *)d_status.p;
        a.smem_table_words = smem_table_words(sh.hits);
        a.smem_ops = smem_ops();
        a.ring_global = nullptr;
        if (sh.frames_global) {
            const uint64_t stride = (uint64_t)2 * prog.num_rows;  // X then Z rows of one block
            frames_buf.ensure((uint64_t)sh.grid * stride * sizeof(uint4), device);
            a.frames_global = (uint4 *)frames_buf.p;
            a.frames_cta_stride = stride;
        }
        if (sh.ring_global) {
            ring_buf.ensure((uint64_t)sh.grid * (uint64_t)sh.blocks_per_cta * prog.ring * sizeof(uint4), device);
            a.ring_global = (uint4 *)ring_buf.p;
            a.ring_cta_stride = (uint64_t)sh.blocks_per_cta * prog.ring;
        }
        if (sh.hits) {
            // Regions per slice and occurrence: the expected hits plus a wide margin (an overflow is detected
            // and the chunk redone with inline noise, so the margin only affects speed).
            if (occs_blocks != sh.blocks_per_cta || !d_occs.p) {
                std::vector<gfs::NoiseOcc> occs = prog.occs;
                slice_cap = gfs::plan_hit_regions(occs, prog.occ_hits_per_block, (uint32_t)sh.blocks_per_cta,
                                                  hit_capacity_override);
                upload(d_occs, occs, device, stream);
                occs_blocks = sh.blocks_per_cta;
            }
            hit_buf.ensure(std::max<uint64_t>(16, nslices * slice_cap * 8), device);
            hit_count.ensure(std::max<uint64_t>(16, nslices * prog.occs.size() * 4), device);
            a.hits = (uint64_t *)hit_buf.p;
            a.hit_count = (uint32_t *)hit_count.p;
            a.occs = (const gfs::NoiseOcc *)d_occs.p;
            a.n_occ = (uint32_t)prog.occs.size();
            a.slice_cap = slice_cap;
            a.smem_occ = smem_occ(true);
            a.occ_xform = lean ? occ_xform() : nullptr;  // records for the lean plan's moved hit phases
            ck(cudaEventRecord(ev_noise[cur_slot + 1][0], stream), "event");
            ck(gfs::launch_noise_kernel(a, sh.blocks_per_cta, stream), "noise kernel launch");
            ck(cudaEventRecord(ev_noise[cur_slot + 1][1], stream), "event");
            noise_pending[cur_slot + 1] = true;
            n_noise++;
        }
        gfs::LaunchShape s = sh;
        s.grid = (int)std::min<uint64_t>((uint64_t)sh.grid, nslices);
        if (lean) {
            a.lean = (const gfs::LeanPhase *)d_lean.p;
            a.lean_inst = (const uint64_t *)d_lean_inst.p;
            a.n_lean = (uint32_t)prog.lean.size();
            ck(gfs::launch_frame_kernel_lean(a, s, stream), "lean frame kernel launch");
        } else {
            ck(gfs::launch_frame_kernel(a, s, stream), "frame kernel launch");
        }
        n_frame++;
    }

    void transpose(const uint4 *s0, uint64_t n0, const uint4 *s1, uint64_t n1, const uint4 *s2, uint64_t n2,
                   const uint8_t *xr, uint64_t nshots, uint8_t *out, uint64_t stride, bool packed) {
        gfs::TransposeArgs t{};
        t.src0 = s0;
        t.n0 = n0;
        t.src1 = s1;
        t.n1 = n1;
        t.src2 = s2;
        t.n2 = n2;
        t.xor_rows = xr;
        t.nshots = nshots;
        t.out = out;
        t.out_stride = stride;
        t.bit_packed = packed ? 1 : 0;
        ck(gfs::launch_transpose(t, stream), "transpose launch");
        n_transpose++;
    }

    // Reads and clears the kernels' status word (after the stream has drained).  Bits 1 and 2 are errors;
    // bit 4 (a hit list overflowed) is returned as true: the caller redoes the affected shots inline.
    bool check_status() {
        ck(gfs::launch_publish_words((const uint32_t *)d_status.p, h_words_dev, 1, stream), "status publish");
        ck(cudaStreamSynchronize(stream), "status read");
        const uint32_t st = *(volatile uint32_t *)h_words;
        if (st) {
            ck(cudaMemsetAsync(d_status.p, 0, 4, stream), "status clear");
            ck(cudaStreamSynchronize(stream), "status clear");
        }
        if (st & 3u) {
            throw std::runtime_error("frame kernel reported error status " + std::to_string(st));
        }
        if (st & 4u) {
            n_hit_overflows++;
            return true;
        }
        return false;
    }

    // Times the frame kernel for each candidate launch shape on whole waves of at least `trial_shots` shots and
    // keeps the fastest per shot.  The stream position does not move (the trial's results are discarded).
    double autotune(uint64_t trial_shots) {
        struct Cand {
            int bpc, threads, ring;
        };
        const Cand cands[] = {{1, 256, 0}, {1, 256, 1}, {1, 128, 0}, {1, 128, 1}, {2, 256, 0},
                              {2, 256, 1}, {2, 128, 0}, {2, 128, 1}, {4, 256, 0}, {4, 256, 1}};
        const gfs::LaunchShape before = shape, before_inline = shape_inline;
        const uint64_t want_blk = std::max<uint64_t>(1, (trial_shots + 127) / 128);
        double best = -1;  // ms per 128-shot block
        gfs::LaunchShape best_shape = shape, best_inline = shape_inline, best_lean = shape_lean;
        bool best_lean_ready = lean_ready;
        const gfs::LaunchShape before_lean = shape_lean;
        const bool before_lean_ready = lean_ready;
        for (const Cand &c : cands) {
            try {
                choose_shape(c.bpc, c.threads, 0, c.ring);
            } catch (const std::invalid_argument &) {
                continue;
            }
            // Whole waves of the candidate's persistent grid (at least two), so that no candidate is timed on a
            // partly filled last wave that a full-size chunk would not have.
            const gfs::LaunchShape &run = lean_active() ? shape_lean : shape;
            const uint64_t wave = (uint64_t)run.grid * (uint64_t)run.blocks_per_cta;
            const uint64_t nblk = std::max<uint64_t>(2, (want_blk + wave - 1) / wave) * wave;
            float total = 0;
            for (int rep = 0; rep < 2; rep++) {
                ck(cudaEventRecord(ev[1], stream), "event");
                run_frame(nblk, next_block);
                ck(cudaEventRecord(ev[2], stream), "event");
                ck(cudaStreamSynchronize(stream), "autotune");
                total = (float)elapsed(1, 2);  // noise kernel + frame kernel
                account_noise(-1);
            }
            check_status();
            const double per_block = total / (double)nblk;
            if (best < 0 || per_block < best) {
                best = per_block;
                best_shape = shape;
                best_inline = shape_inline;
                best_lean = shape_lean;
                best_lean_ready = lean_ready;
            }
        }
        shape = best < 0 ? before : best_shape;
        shape_inline = best < 0 ? before_inline : best_inline;
        shape_lean = best < 0 ? before_lean : best_lean;
        lean_ready = best < 0 ? before_lean_ready : best_lean_ready;
        return best < 0 ? best : best * (double)want_blk;  // ms for the requested trial size
    }

    // Chunk size (in 128-shot blocks) for host destinations: one resident wave of the frame kernel (every
    // CTA one slice, no tail), so that the pipeline's fill (the first chunk's kernels) and drain (the last
    // chunk's copy) are short next to the overlapped middle (d=25 at 2^20 shots: 12.25 ms per request against
    // 12.99 with six chunks; half a wave leaves the frame kernel underfilled), within the device memory budget.
    uint64_t host_chunk_blocks(uint64_t nblk_total, uint64_t slot_row_bytes) const {
        (void)nblk_total;
        uint64_t cb = chunk_blocks(2 * slot_row_bytes);
        if (chunk_shots) {
            return cb;
        }
        uint64_t wave = (uint64_t)shape.grid * (uint64_t)shape.blocks_per_cta;
        return std::min<uint64_t>(cb, std::max<uint64_t>(1, wave));
    }

    // Device->host copy of `rows` rows of `width` bytes on copy_stream: one linear copy when both sides are
    // contiguous (a strided copy of narrow rows moves them one by one).
    void copy_rows(uint8_t *dst, uint64_t dpitch, const uint8_t *src, uint64_t spitch, uint64_t width, uint64_t rows,
                   const char *what) {
        if (dpitch == width && spitch == width) {
            ck(cudaMemcpyAsync(dst, src, width * rows, cudaMemcpyDeviceToHost, copy_stream), what);
        } else {
            ck(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, cudaMemcpyDeviceToHost, copy_stream), what);
        }
    }

    // Host destinations.  Chunk k is sampled and transposed on `stream` into slot k % 2 of a device
    // staging buffer; its device->host copy runs on `copy_stream` while chunk k + 1's kernels run.  The
    // copy of chunk k is issued only after chunk k + 1's kernels are queued, because a copy into pageable
    // memory may hold the calling thread until it completes.
    // Whether every non-null host destination is page-locked: then a chunk's copy can be queued as soon as its
    // kernels are, because cudaMemcpyAsync into page-locked memory returns at once.
    static bool page_locked(std::initializer_list<const void *> ptrs) {
        for (const void *p : ptrs) {
            if (!p) {
                continue;
            }
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
                cudaGetLastError();
                return false;
            }
            if (at.type != cudaMemoryTypeHost) {
                return false;
            }
        }
        return true;
    }

    template <typename Produce, typename Copy>
    void host_pipeline(uint64_t shots, uint64_t slot_row_bytes, Produce produce, Copy copy, bool eager = false) {
        const uint64_t first_block = next_block;
        uint64_t nblk_total = (shots + 127) / 128;
        uint64_t cb = host_chunk_blocks(nblk_total, slot_row_bytes);
        uint64_t slot_bytes = cb * 128 * slot_row_bytes;
        out_tmp.ensure(std::max<uint64_t>(16, 2 * slot_bytes), device);
        uint8_t *slots[2] = {(uint8_t *)out_tmp.p, (uint8_t *)out_tmp.p + slot_bytes};
        struct Chunk {
            uint64_t done, cs;
        };
        Chunk inflight[2] = {};
        bool used[2] = {false, false};
        auto account = [&](int slot) {
            // The copy of this slot's chunk has completed, so its kernel events have too.
            ck(cudaEventSynchronize(pev[slot][3]), "chunk copy");
            float ms = 0;
            ck(cudaEventElapsedTime(&ms, pev[slot][0], pev[slot][1]), "cudaEventElapsedTime");
            t_frame += ms - account_noise(slot);
            ck(cudaEventElapsedTime(&ms, pev[slot][1], pev[slot][2]), "cudaEventElapsedTime");
            t_transpose += ms;
            used[slot] = false;
        };
        auto issue_copy = [&](int slot) {
            ck(cudaStreamWaitEvent(copy_stream, pev[slot][2], 0), "cudaStreamWaitEvent");
            copy(inflight[slot].done, inflight[slot].cs, slots[slot]);
            ck(cudaEventRecord(pev[slot][3], copy_stream), "event");
        };
        ck(cudaEventRecord(ev[0], stream), "event");
        uint64_t done = 0;
        int k = 0, prev = -1;
        while (done < shots) {
            const int slot = k & 1;
            if (used[slot]) {
                account(slot);
            }
            uint64_t cs = std::min<uint64_t>(shots - done, cb * 128);
            uint64_t nblk = (cs + 127) / 128;
            ck(cudaEventRecord(pev[slot][0], stream), "event");
            cur_slot = slot;
            try {
                run_frame(nblk, next_block);
            } catch (...) {
                cur_slot = -1;
                throw;
            }
            cur_slot = -1;
            ck(cudaEventRecord(pev[slot][1], stream), "event");
            produce(done, cs, slots[slot]);
            ck(cudaEventRecord(pev[slot][2], stream), "event");
            inflight[slot] = Chunk{done, cs};
            used[slot] = true;
            if (eager) {
                // Page-locked destinations: queue this chunk's copy now, so the copy engine already holds it when the
                // previous copy ends (the thread's wait for a free slot would otherwise leave a gap between copies).
                issue_copy(slot);
            } else {
                if (prev >= 0) {
                    issue_copy(prev);
                }
                prev = slot;
            }
            next_block += nblk;
            done += cs;
            k++;
        }
        if (prev >= 0) {
            issue_copy(prev);
        }
        ck(cudaEventRecord(ev[1], copy_stream), "event");
        for (int slot = 0; slot < 2; slot++) {
            if (used[slot]) {
                account(slot);
            }
        }
        ck(cudaStreamSynchronize(stream), "sample");
        ck(cudaEventSynchronize(ev[1]), "sample");
        t_total = elapsed(0, 1);
        t_copy = std::max(0.0, t_total - t_frame - t_noise - t_transpose);
        if (check_status()) {
            // A hit list overflowed somewhere: redo the whole request with inline noise (same results).
            next_block = first_block;
            force_inline = true;
            try {
                host_pipeline(shots, slot_row_bytes, produce, copy, eager);
            } catch (...) {
                force_inline = false;
                throw;
            }
            force_inline = false;
        }
    }

    // Enqueues the transposes of one chunk's detection events (and observables) into dd / od.
    void transpose_detections(uint32_t flags, uint64_t cs, uint8_t *dd, uint64_t ds, uint8_t *od, uint64_t os,
                              bool want_dets, bool want_obs) {
        bool packed = flags & GFS_BIT_PACKED;
        uint64_t D = prog.num_detectors, O = prog.num_observables;
        const uint4 *dt = (const uint4 *)det_tmp.p, *ot = (const uint4 *)obs_tmp.p;
        if (want_dets) {
            if ((flags & GFS_PREPEND_OBSERVABLES) && (flags & GFS_APPEND_OBSERVABLES)) {
                transpose(ot, O, dt, D, ot, O, nullptr, cs, dd, ds, packed);
            } else if (flags & GFS_PREPEND_OBSERVABLES) {
                transpose(ot, O, dt, D, nullptr, 0, nullptr, cs, dd, ds, packed);
            } else if (flags & GFS_APPEND_OBSERVABLES) {
                transpose(dt, D, ot, O, nullptr, 0, nullptr, cs, dd, ds, packed);
            } else {
                transpose(dt, D, nullptr, 0, nullptr, 0, nullptr, cs, dd, ds, packed);
            }
        }
        if (want_obs) {
            transpose(ot, O, nullptr, 0, nullptr, 0, nullptr, cs, od, os, packed);
        }
    }

    // Samples `shots` detection-event shots (at most one chunk) and leaves them detector-major in det_tmp / obs_tmp
    // ([128-shot block][detector] and [block][observable] uint4 rows), without the shot-major transpose, for
    // consumers that read that layout (ptb64 files).  An overflowed hit list redoes the chunk with inline noise.
    void detections_detmajor(uint64_t shots) {
        if (mode != GFS_MODE_DETECTIONS) {
            throw std::invalid_argument("sampler was not created in detection mode");
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        reset_timings();
        const uint64_t nblk = (shots + 127) / 128;
        ck(cudaEventRecord(ev[0], stream), "event");
        run_frame(nblk, next_block);
        ck(cudaEventRecord(ev[1], stream), "event");
        ck(cudaStreamSynchronize(stream), "sample");
        t_frame = elapsed(0, 1) - account_noise(-1);
        if (check_status()) {
            force_inline = true;
            try {
                run_frame(nblk, next_block);
                ck(cudaStreamSynchronize(stream), "sample");
            } catch (...) {
                force_inline = false;
                throw;
            }
            force_inline = false;
            check_status();
        }
        next_block += nblk;
        t_total = t_frame + t_noise;
    }

    // Shared driver for detections (host or device destinations).
    void detections(uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dstride, uint8_t *obs, uint64_t ostride,
                    bool device_out) {
        bool packed = flags & GFS_BIT_PACKED;
        uint64_t D = prog.num_detectors, O = prog.num_observables;
        uint64_t nd = D + ((flags & GFS_PREPEND_OBSERVABLES) ? O : 0) + ((flags & GFS_APPEND_OBSERVABLES) ? O : 0);
        uint64_t drow = packed ? (nd + 7) / 8 : nd;
        uint64_t orow = packed ? (O + 7) / 8 : O;
        if (dets && dstride < drow) {
            throw std::invalid_argument("dets row stride too small");
        }
        if (obs && ostride < orow) {
            throw std::invalid_argument("obs row stride too small");
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        reset_timings();
        if (!device_out) {
            // Staging rows use the caller's stride when its rows are contiguous, so that each chunk leaves in
            // one linear copy; otherwise they are padded to 32 bytes and copied row by row.
            const uint64_t ds = dstride == drow ? drow : pad32(drow), os = ostride == orow ? orow : pad32(orow);
            host_pipeline(
                shots, ds + os,
                [&](uint64_t, uint64_t cs, uint8_t *buf) {
                    transpose_detections(flags, cs, buf, ds, buf + cs * ds, os, dets != nullptr, obs != nullptr);
                },
                [&](uint64_t done, uint64_t cs, uint8_t *buf) {
                    if (dets && drow) {
                        copy_rows(dets + done * dstride, dstride, buf, ds, drow, cs, "copy dets");
                    }
                    if (obs && orow) {
                        copy_rows(obs + done * ostride, ostride, buf + cs * ds, os, orow, cs, "copy obs");
                    }
                },
                page_locked({dets, obs}));
            return;
        }
        ck(cudaEventRecord(ev[0], stream), "event");
        uint64_t cb = chunk_blocks(drow + orow);
        uint64_t done = 0;
        while (done < shots) {
            uint64_t cs = std::min<uint64_t>(shots - done, cb * 128);
            uint64_t nblk = (cs + 127) / 128;
            ck(cudaEventRecord(ev[1], stream), "event");
            run_frame(nblk, next_block);
            ck(cudaEventRecord(ev[2], stream), "event");
            transpose_detections(flags, cs, dets ? dets + done * dstride : nullptr, dstride,
                                 obs ? obs + done * ostride : nullptr, ostride, dets != nullptr, obs != nullptr);
            ck(cudaEventRecord(ev[3], stream), "event");
            ck(cudaStreamSynchronize(stream), "sample");
            t_frame += elapsed(1, 2) - account_noise(-1);
            t_transpose += elapsed(2, 3);
            if (check_status()) {
                // The chunk's hit list overflowed: redo it with inline noise (same results).
                force_inline = true;
                try {
                    run_frame(nblk, next_block);
                    transpose_detections(flags, cs, dets ? dets + done * dstride : nullptr, dstride,
                                         obs ? obs + done * ostride : nullptr, ostride, dets != nullptr,
                                         obs != nullptr);
                    ck(cudaStreamSynchronize(stream), "sample");
                } catch (...) {
                    force_inline = false;
                    throw;
                }
                force_inline = false;
                check_status();
            }
            next_block += nblk;
            done += cs;
        }
        ck(cudaEventRecord(ev[1], stream), "event");
        ck(cudaStreamSynchronize(stream), "sample");
        t_total = elapsed(0, 1);
        t_copy = std::max(0.0, t_total - t_frame - t_noise - t_transpose);
    }

    // Measurement records into device memory (shot-major, `stride` bytes apart), the reference sample XORed in.
    void measurements_device(uint64_t shots, uint32_t flags, const uint8_t *ref, uint8_t *out, uint64_t stride) {
        if (mode != GFS_MODE_MEASUREMENTS) {
            throw std::invalid_argument("sampler was not created in measurement mode");
        }
        const bool packed = flags & GFS_BIT_PACKED;
        const uint64_t M = prog.num_measurements;
        const uint64_t row = packed ? (M + 7) / 8 : M;
        if (stride < row) {
            throw std::invalid_argument("output row stride too small");
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        reset_timings();
        const uint8_t *dref = nullptr;
        if (ref && M) {
            ref_bits.ensure((M + 7) / 8, device);
            ck(cudaMemcpyAsync(ref_bits.p, ref, (M + 7) / 8, cudaMemcpyHostToDevice, stream), "ref upload");
            dref = (const uint8_t *)ref_bits.p;
        }
        ck(cudaEventRecord(ev[0], stream), "event");
        const uint64_t cb = chunk_blocks(row);
        for (uint64_t done = 0; done < shots;) {
            const uint64_t cs = std::min<uint64_t>(shots - done, cb * 128);
            const uint64_t nblk = (cs + 127) / 128;
            for (int attempt = 0; attempt < 2; attempt++) {
                run_frame(nblk, next_block);
                transpose((const uint4 *)meas_tmp.p, M, nullptr, 0, nullptr, 0, dref, cs, out + done * stride, stride,
                          packed);
                ck(cudaStreamSynchronize(stream), "sample");
                account_noise(-1);
                const bool overflow = check_status();
                force_inline = false;
                if (!overflow) {
                    break;
                }
                force_inline = true;  // redo the chunk with inline noise (same results)
            }
            next_block += nblk;
            done += cs;
        }
        ck(cudaEventRecord(ev[1], stream), "event");
        ck(cudaStreamSynchronize(stream), "sample");
        t_total = elapsed(0, 1);
    }

    void measurements(uint64_t shots, uint32_t flags, const uint8_t *ref, uint8_t *out, uint64_t stride) {
        if (mode != GFS_MODE_MEASUREMENTS) {
            throw std::invalid_argument("sampler was not created in measurement mode");
        }
        bool packed = flags & GFS_BIT_PACKED;
        uint64_t M = prog.num_measurements;
        uint64_t row = packed ? (M + 7) / 8 : M;
        if (stride < row) {
            throw std::invalid_argument("output row stride too small");
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        reset_timings();
        const uint8_t *dref = nullptr;
        if (ref && M) {
            ref_bits.ensure((M + 7) / 8, device);
            ck(cudaMemcpyAsync(ref_bits.p, ref, (M + 7) / 8, cudaMemcpyHostToDevice, stream), "ref upload");
            dref = (const uint8_t *)ref_bits.p;
        }
        const uint64_t rs = stride == row ? row : pad32(row);
        host_pipeline(
            shots, rs,
            [&](uint64_t, uint64_t cs, uint8_t *buf) {
                transpose((const uint4 *)meas_tmp.p, M, nullptr, 0, nullptr, 0, dref, cs, buf, rs, packed);
            },
            [&](uint64_t done, uint64_t cs, uint8_t *buf) {
                if (row) {
                    copy_rows(out + done * stride, stride, buf, rs, row, cs, "copy meas");
                }
            },
            page_locked({out}));
    }
};

