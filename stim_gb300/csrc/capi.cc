// C ABI (include/stim_gb300.h) and the host runtime behind it: device copies of the lowered program,
// chunked launches of the frame and transpose kernels on a per-sampler stream, and error mapping.
#include "sampler.h"

#include <mutex>

#include "formats.h"
#include "formats_device.h"
#include "noalloc.h"
#include "tableau.h"

namespace gfs_rt {
thread_local std::string g_err;
}  // namespace gfs_rt

namespace {

// Allocation-free detection sampling into caller-owned device buffers: the frame kernel's scratch is the
// fixed array of noalloc.cu instead of cudaMalloc'd buffers; everything else is as in
// gfs_sample_detections_device.  Calls on one device are serialized by a process-wide lock.
void detections_noalloc(gfs_sampler *s, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dstride, uint8_t *obs,
                        uint64_t ostride) {
    if (s->mode != GFS_MODE_DETECTIONS) {
        throw std::invalid_argument("sampler was not created in detection mode");
    }
    bool packed = flags & GFS_BIT_PACKED;
    uint64_t D = s->prog.num_detectors, O = s->prog.num_observables;
    uint64_t nd = D + ((flags & GFS_PREPEND_OBSERVABLES) ? O : 0) + ((flags & GFS_APPEND_OBSERVABLES) ? O : 0);
    uint64_t drow = packed ? (nd + 7) / 8 : nd;
    uint64_t orow = packed ? (O + 7) / 8 : O;
    if (dets && dstride < drow) {
        throw std::invalid_argument("dets row stride too small");
    }
    if (obs && ostride < orow) {
        throw std::invalid_argument("obs row stride too small");
    }
    uint64_t bpc = (uint64_t)s->shape.blocks_per_cta;
    uint64_t per_block = (D + O) * sizeof(uint4);
    uint64_t cap_blocks = per_block ? (uint64_t)(gfs::kNoAllocScratchBytes / per_block) : ((uint64_t)1 << 40);
    cap_blocks = (cap_blocks / bpc) * bpc;
    if (cap_blocks == 0) {
        throw std::invalid_argument(
            "the circuit needs " + std::to_string(per_block * bpc) + " bytes of scratch per " +
            std::to_string(128 * bpc) + "-shot slice (" + std::to_string(D) + " detectors + " + std::to_string(O) +
            " observables), more than the " + std::to_string(gfs::kNoAllocScratchBytes) +
            " bytes the allocation-free entry point holds; use gfs_sample_detections_device instead");
    }
    ck(cudaSetDevice(s->device), "cudaSetDevice");
    std::lock_guard<std::mutex> lock(gfs::noalloc_device_lock(s->device));
    void *scratch = nullptr;
    ck(gfs::noalloc_scratch_address(s->device, &scratch), "scratch address");
    uint4 *det_s = (uint4 *)scratch;
    uint4 *obs_s = det_s + cap_blocks * D;
    s->reset_timings();
    ck(cudaEventRecord(s->ev[0], s->stream), "event");
    uint64_t done = 0;
    while (done < shots) {
        uint64_t cs = std::min<uint64_t>(shots - done, cap_blocks * 128);
        uint64_t nblk = (cs + 127) / 128;
        uint64_t nslices = (nblk + bpc - 1) / bpc;
        gfs::KernelArgs a{};
        a.ops = (const gfs::DevOp *)s->d_ops.p;
        a.pool = (const uint32_t *)s->d_pool.p;
        a.tables = (const uint32_t *)s->d_tables.p;
        a.chans = (const gfs::DevChan *)s->d_chans.p;
        a.qubit_orig = (const uint32_t *)s->d_orig.p;
        a.reset_zero = s->prog.reset_norand ? 1u : 0u;
        a.nrows = s->prog.num_rows;
        a.ring = s->prog.ring;
        a.nobs = (uint32_t)O;
        a.nslices = (uint32_t)nslices;
        a.ndet = D;
        a.nmeas = 0;
        a.seed = s->seed;
        a.block0 = s->next_block;
        a.det_out = det_s;
        a.obs_out = obs_s;
        a.meas_out = nullptr;
        a.status = (uint32_t *)s->d_status.p;
        a.smem_table_words = s->smem_table_words();
        a.smem_ops = s->smem_ops();
        a.ring_global = nullptr;  // this path allocates nothing: the ring stays in shared memory
        gfs::LaunchShape shape = s->shape_inline;  // no hit lists: they would need allocations
        if (shape.frames_global) {
            throw std::invalid_argument("the circuit's frames do not fit in shared memory, which the allocation-free "
                                        "entry point requires");
        }
        if (shape.ring_global) {
            shape.ring_global = false;
            shape.smem = s->smem_for(shape.blocks_per_cta, false);
            int optin = 0;
            ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device), "device attribute");
            int per_sm = 0;
            if (shape.smem <= (size_t)optin &&
                gfs::frame_kernel_max_ctas_per_sm(shape, &per_sm) != cudaSuccess) {
                cudaGetLastError();  // a failed query must not surface as the error of a later launch
                per_sm = 0;
            }
            if (per_sm < 1) {
                throw std::invalid_argument("the circuit's measurement ring does not fit in shared memory, which the "
                                            "allocation-free entry point requires");
            }
            shape.grid = per_sm * s->num_sms;
        }
        shape.grid = (int)std::min<uint64_t>((uint64_t)shape.grid, nslices);
        ck(cudaEventRecord(s->ev[1], s->stream), "event");
        ck(gfs::launch_frame_kernel(a, shape, s->stream), "frame kernel launch");
        s->n_frame++;
        ck(cudaEventRecord(s->ev[2], s->stream), "event");
        uint8_t *dd = dets ? dets + done * dstride : nullptr;
        uint8_t *od = obs ? obs + done * ostride : nullptr;
        if (dets) {
            if ((flags & GFS_PREPEND_OBSERVABLES) && (flags & GFS_APPEND_OBSERVABLES)) {
                s->transpose(obs_s, O, det_s, D, obs_s, O, nullptr, cs, dd, dstride, packed);
            } else if (flags & GFS_PREPEND_OBSERVABLES) {
                s->transpose(obs_s, O, det_s, D, nullptr, 0, nullptr, cs, dd, dstride, packed);
            } else if (flags & GFS_APPEND_OBSERVABLES) {
                s->transpose(det_s, D, obs_s, O, nullptr, 0, nullptr, cs, dd, dstride, packed);
            } else {
                s->transpose(det_s, D, nullptr, 0, nullptr, 0, nullptr, cs, dd, dstride, packed);
            }
        }
        if (obs) {
            s->transpose(obs_s, O, nullptr, 0, nullptr, 0, nullptr, cs, od, ostride, packed);
        }
        ck(cudaEventRecord(s->ev[3], s->stream), "event");
        ck(cudaStreamSynchronize(s->stream), "sample");
        s->t_frame += s->elapsed(1, 2);
        s->t_transpose += s->elapsed(2, 3);
        s->check_status();
        s->next_block += nblk;
        done += cs;
    }
    ck(cudaEventRecord(s->ev[1], s->stream), "event");
    ck(cudaStreamSynchronize(s->stream), "sample");
    s->t_total = s->elapsed(0, 1);
    s->t_copy = 0;
}

struct File {
    FILE *f = nullptr;
    File(const char *path) {
        if (path) {
            f = fopen(path, "wb");
            if (!f) {
                throw std::invalid_argument("Failed to open '" + std::string(path) + "' to write.");
            }
        }
    }
    ~File() {
        if (f) {
            fclose(f);
        }
    }
};

// Shots per sampled chunk when writing files: about 256 MiB of rows or of file bytes (01 is eight times the rows),
// and at most one resident wave of the frame kernel (or the sampler's chunk size, when one is set), so that
// consecutive chunks overlap well; a multiple of 128 shots (so of 64, as ptb64 needs).
uint64_t write_chunk(const gfs_sampler *s, uint64_t row_bytes, gfs::Format f, uint64_t nbits) {
    const uint64_t per_shot = std::max<uint64_t>(1, f == gfs::Format::F01 ? std::max(row_bytes, nbits + 1) : row_bytes);
    uint64_t c = ((uint64_t)256 << 20) / per_shot;
    const gfs::LaunchShape &sh = s->lean_active() ? s->shape_lean : s->shape;
    c = std::min<uint64_t>(c, s->chunk_shots ? s->chunk_shots
                                             : (uint64_t)std::max(1, sh.grid) * (uint64_t)std::max(1, sh.blocks_per_cta) * 128);
    return std::max<uint64_t>(128, c & ~(uint64_t)127);
}

// Makes the file bytes of `shots` device rows (bit-packed, `stride` bytes apart, `nbits` bits) in format f on
// s->stream (formats.cu), into `out` unless the rows already are the file (contiguous b8).  Returns where the
// bytes are and how many.  The prefix rules for dets follow the host writer (formats.cc write_rows).
std::pair<const uint8_t *, uint64_t> format_rows(gfs_sampler *s, DevBuf &out, gfs::Format f, const uint8_t *rows,
                                                 uint64_t stride, uint64_t shots, uint64_t nbits, char c1, char c2,
                                                 uint64_t transition) {
    if (transition == 0) {
        transition = nbits;
        c1 = c2;
    } else if (c1 == c2 || transition >= nbits) {
        transition = nbits;
    }
    gfs::FormatArgs a{};
    a.rows = rows;
    a.stride = stride;
    a.shots = shots;
    a.nbits = nbits;
    a.fmt = (uint32_t)f;
    a.c1 = (uint8_t)c1;
    a.c2 = (uint8_t)c2;
    a.transition = transition;
    if (f == gfs::Format::B8) {
        if (nbits == 0) {  // empty records take no bytes
            return {rows, 0};
        }
        if (stride != (nbits + 7) / 8) {
            throw std::logic_error("b8 rows must be contiguous");
        }
        return {rows, shots * stride};
    }
    uint64_t bytes = 0;
    if (f == gfs::Format::F01 || f == gfs::Format::PTB64) {
        bytes = gfs::fixed_format_bytes(f, shots, nbits);
    } else {
        s->fmt_lens.ensure(std::max<uint64_t>(16, shots * 4), s->device);
        s->fmt_offs.ensure((shots + 1) * 8, s->device);
        s->fmt_sums.ensure(((shots + 1024) / 1024) * 8, s->device);
        s->fmt_total.ensure(16, s->device);
        a.lens = (uint32_t *)s->fmt_lens.p;
        a.offs = (uint64_t *)s->fmt_offs.p;
        ck(gfs::launch_format_lengths(a, (uint64_t *)s->fmt_sums.p, (uint64_t *)s->fmt_total.p, s->stream),
           "format lengths");
        ck(cudaMemcpyAsync(&bytes, s->fmt_total.p, 8, cudaMemcpyDeviceToHost, s->stream), "format size");
        ck(cudaStreamSynchronize(s->stream), "format size");
    }
    out.ensure(std::max<uint64_t>(16, bytes), s->device);
    a.out = (uint8_t *)out.p;
    ck(gfs::launch_format_write(a, s->stream), "format kernel");
    return {a.out, bytes};
}

// File output of sample_write as a two-slot pipeline: chunk k is sampled and formatted on the sampler's stream
// into slot k % 2, its bytes are copied to that slot's page-locked buffers on copy_stream, and written to the files
// once chunk k + 1 has been sampled, so a chunk's copy overlaps the next chunk's kernels and its fwrite the next
// chunk's copy.  Files receive the chunks in order.
class FileWriter {
   public:
    explicit FileWriter(gfs_sampler *s) : s_(s) {
        for (gfs_sampler::WriteSlot &w : s_->wslot) {
            if (!w.formatted) {
                ck(cudaEventCreateWithFlags(&w.formatted, cudaEventDisableTiming), "cudaEventCreate");
            }
            if (!w.copied) {
                ck(cudaEventCreateWithFlags(&w.copied, cudaEventDisableTiming), "cudaEventCreate");
            }
            w.pending = false;
        }
    }
    ~FileWriter() {
        // Normal exit has flushed every slot; after an error, no copy may still be writing into a slot's buffer.
        cudaStreamSynchronize(s_->copy_stream);
        for (gfs_sampler::WriteSlot &w : s_->wslot) {
            w.pending = false;
        }
    }

    // The slot for chunk k (written out two chunks ago, so free).
    gfs_sampler::WriteSlot &slot(uint64_t k) {
        return s_->wslot[k & 1];
    }

    // Queues the copies of the slot's formatted bytes (part 0: the main file, part 1: the observables' file).
    void queue(gfs_sampler::WriteSlot &w, const std::pair<const uint8_t *, uint64_t> part[2], FILE *files[2]) {
        ck(cudaEventRecord(w.formatted, s_->stream), "event");
        ck(cudaStreamWaitEvent(s_->copy_stream, w.formatted, 0), "cudaStreamWaitEvent");
        for (int j = 0; j < 2; j++) {
            w.file[j] = files[j];
            w.bytes[j] = files[j] ? part[j].second : 0;
            if (!w.bytes[j]) {
                continue;
            }
            if (w.bytes[j] > w.host_cap[j]) {
                if (w.host[j]) {
                    cudaFreeHost(w.host[j]);
                    w.host[j] = nullptr;
                    w.host_cap[j] = 0;
                }
                ck(cudaHostAlloc((void **)&w.host[j], w.bytes[j], cudaHostAllocDefault), "cudaHostAlloc");
                w.host_cap[j] = w.bytes[j];
            }
            ck(cudaMemcpyAsync(w.host[j], part[j].first, w.bytes[j], cudaMemcpyDeviceToHost, s_->copy_stream),
               "copy file bytes");
        }
        ck(cudaEventRecord(w.copied, s_->copy_stream), "event");
        w.pending = true;
    }

    // Writes the slot's bytes once their copies are done.
    void flush(gfs_sampler::WriteSlot &w) {
        if (!w.pending) {
            return;
        }
        ck(cudaEventSynchronize(w.copied), "copy file bytes");
        w.pending = false;
        for (int j = 0; j < 2; j++) {
            if (w.bytes[j] && fwrite(w.host[j], 1, w.bytes[j], w.file[j]) != w.bytes[j]) {
                throw std::runtime_error("failed to write the result file");
            }
        }
    }

   private:
    gfs_sampler *s_;
};

// CompiledDetectorSampler.sample_write (compiled_detector_sampler.pybind.cc:88-141 and
// frame_simulator_util.inl:120-200): detection events (observables prepended, appended, or to a file of
// their own) in one of the result formats.
void write_detections(gfs_sampler *s, uint64_t shots, const char *path, const char *format, uint32_t flags,
                      const char *obs_path, const char *obs_format) {
    if (s->mode != GFS_MODE_DETECTIONS) {
        throw std::invalid_argument("sampler was not created in detection mode");
    }
    const bool prepend = flags & GFS_PREPEND_OBSERVABLES, append = flags & GFS_APPEND_OBSERVABLES;
    if ((int)prepend + (int)append + (obs_path != nullptr) > 1) {
        throw std::out_of_range("Can't combine --prepend_observables, --append_observables, or --obs_out");
    }
    const gfs::Format f = gfs::parse_format(format ? format : "01");
    const gfs::Format of = gfs::parse_format(obs_format ? obs_format : "01");
    const uint64_t D = s->prog.num_detectors, O = s->prog.num_observables;
    if ((f == gfs::Format::PTB64 || (obs_path && of == gfs::Format::PTB64)) && shots % 64 != 0) {
        throw std::invalid_argument("shots must be a multiple of 64 to use ptb64 format.");
    }
    File out(path), obs_out(obs_path);
    const uint64_t nd = D + (prepend || append ? O : 0);
    const uint64_t drow = std::max<uint64_t>(1, (nd + 7) / 8), orow = std::max<uint64_t>(1, (O + 7) / 8);
    const uint64_t chunk = std::min(write_chunk(s, drow + orow, f, nd), write_chunk(s, drow + orow, of, O));
    FileWriter fw(s);
    uint64_t k = 0;
    for (uint64_t done = 0; done < shots; k++) {
        const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
        gfs_sampler::WriteSlot &w = fw.slot(k);
        std::pair<const uint8_t *, uint64_t> part[2] = {{nullptr, 0}, {nullptr, 0}};
        if (f == gfs::Format::PTB64 && (!obs_path || of == gfs::Format::PTB64)) {
            // ptb64's words are halves of the frame kernel's detector-major rows: no shot-major rows needed.
            s->detections_detmajor(cs);
            const uint4 *dt = (const uint4 *)s->det_tmp.p, *ot = (const uint4 *)s->obs_tmp.p;
            const uint64_t bytes = gfs::fixed_format_bytes(gfs::Format::PTB64, cs, nd);
            w.out[0].ensure(std::max<uint64_t>(16, bytes), s->device);
            ck(prepend  ? gfs::launch_ptb64_detmajor(ot, O, dt, D, cs, (uint8_t *)w.out[0].p, s->stream)
               : append ? gfs::launch_ptb64_detmajor(dt, D, ot, O, cs, (uint8_t *)w.out[0].p, s->stream)
                        : gfs::launch_ptb64_detmajor(dt, D, nullptr, 0, cs, (uint8_t *)w.out[0].p, s->stream),
               "ptb64 kernel");
            part[0] = {(const uint8_t *)w.out[0].p, bytes};
            if (obs_path) {
                const uint64_t obytes = gfs::fixed_format_bytes(gfs::Format::PTB64, cs, O);
                w.out[1].ensure(std::max<uint64_t>(16, obytes), s->device);
                ck(gfs::launch_ptb64_detmajor(ot, O, nullptr, 0, cs, (uint8_t *)w.out[1].p, s->stream), "ptb64 kernel");
                part[1] = {(const uint8_t *)w.out[1].p, obytes};
            }
        } else {
            w.rows.ensure(cs * drow, s->device);
            if (obs_path) {
                w.obs.ensure(cs * orow, s->device);
            }
            s->detections(cs, (flags & (GFS_PREPEND_OBSERVABLES | GFS_APPEND_OBSERVABLES)) | GFS_BIT_PACKED,
                          (uint8_t *)w.rows.p, drow, obs_path ? (uint8_t *)w.obs.p : nullptr, orow, true);
            // Prefixes as the reference names them: D then L when appended, L then D when prepended.
            part[0] = prepend ? format_rows(s, w.out[0], f, (const uint8_t *)w.rows.p, drow, cs, nd, 'L', 'D', O)
                              : format_rows(s, w.out[0], f, (const uint8_t *)w.rows.p, drow, cs, nd, 'D', 'L', D);
            if (obs_path) {
                part[1] = format_rows(s, w.out[1], of, (const uint8_t *)w.obs.p, orow, cs, O, 'L', 'L', O);
            }
        }
        FILE *files[2] = {out.f, obs_out.f};
        fw.queue(w, part, files);
        fw.flush(fw.slot(k + 1));  // the previous chunk, whose copy ran beside this chunk's kernels
        done += cs;
    }
    fw.flush(fw.slot(k + 1));
    fw.flush(fw.slot(k));
}

// CompiledMeasurementSampler.sample_write (compiled_measurement_sampler.pybind.cc:37-45).
void write_measurements(gfs_sampler *s, uint64_t shots, const char *path, const char *format, const uint8_t *ref) {
    const gfs::Format f = gfs::parse_format(format ? format : "01");
    if (f == gfs::Format::PTB64 && shots % 64 != 0) {
        throw std::invalid_argument("shots must be a multiple of 64 to use ptb64 format.");
    }
    File out(path);
    const uint64_t M = s->prog.num_measurements;
    const uint64_t row = std::max<uint64_t>(1, (M + 7) / 8);
    const uint64_t chunk = write_chunk(s, row, f, M);
    FileWriter fw(s);
    uint64_t k = 0;
    for (uint64_t done = 0; done < shots; k++) {
        const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
        gfs_sampler::WriteSlot &w = fw.slot(k);
        w.rows.ensure(cs * row, s->device);
        s->measurements_device(cs, GFS_BIT_PACKED, ref, (uint8_t *)w.rows.p, row);
        std::pair<const uint8_t *, uint64_t> part[2] = {
            format_rows(s, w.out[0], f, (const uint8_t *)w.rows.p, row, cs, M, 'M', 'M', 0), {nullptr, 0}};
        FILE *files[2] = {out.f, nullptr};
        fw.queue(w, part, files);
        fw.flush(fw.slot(k + 1));
        done += cs;
    }
    fw.flush(fw.slot(k + 1));
    fw.flush(fw.slot(k));
}

}  // namespace

extern "C" {

gfs_status gfs_sample_write_detections(gfs_sampler *s, uint64_t shots, const char *path, const char *format,
                                       uint32_t flags, const char *obs_path, const char *obs_format) {
    return guarded([&] { write_detections(s, shots, path, format, flags, obs_path, obs_format); });
}

gfs_status gfs_sample_write_measurements(gfs_sampler *s, uint64_t shots, const char *path, const char *format,
                                         const uint8_t *ref_sample) {
    return guarded([&] { write_measurements(s, shots, path, format, ref_sample); });
}


const char *gfs_last_error(void) {
    return g_err.c_str();
}

gfs_status gfs_device_count(int *out) {
    return guarded([&] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess) {
            n = 0;
            cudaGetLastError();
        }
        *out = n;
    });
}

gfs_status gfs_device_info(int device, int64_t *info8) {
    return guarded([&] {
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        int v = 0;
        info8[0] = prop.multiProcessorCount;
        info8[1] = (int64_t)prop.sharedMemPerBlockOptin;
        info8[2] = (int64_t)prop.sharedMemPerMultiprocessor;
        ck(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, device), "attribute");
        info8[3] = v;
        ck(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device), "attribute");
        info8[4] = v;
        ck(cudaDeviceGetAttribute(&v, cudaDevAttrClockRate, device), "attribute");
        info8[5] = v;
        info8[6] = prop.major * 10 + prop.minor;
        info8[7] = (int64_t)prop.l2CacheSize;
    });
}

gfs_status gfs_circuit_parse(const char *text, size_t len, gfs_circuit **out) {
    *out = nullptr;
    return guarded([&] {
        auto c = std::make_unique<gfs_circuit>();
        c->circuit = gfs::Circuit::parse(std::string_view(text, len));
        c->stats = c->circuit.stats();
        *out = c.release();
    });
}

gfs_status gfs_circuit_stats(const gfs_circuit *c, uint64_t *s) {
    return guarded([&] {
        s[0] = c->stats.num_qubits;
        s[1] = c->stats.num_measurements;
        s[2] = c->stats.num_detectors;
        s[3] = c->stats.num_observables;
        s[4] = c->stats.max_lookback;
        s[5] = c->stats.num_instances;
    });
}

void gfs_circuit_free(gfs_circuit *c) {
    delete c;
}

gfs_status gfs_program_info(const gfs_circuit *c, uint32_t mode, uint64_t *info8) {
    return guarded([&] {
        if (mode != GFS_MODE_DETECTIONS && mode != GFS_MODE_MEASUREMENTS) {
            throw std::invalid_argument("unknown sampling mode");
        }
        gfs::Program p = gfs::lower(c->circuit, mode == GFS_MODE_MEASUREMENTS ? gfs::SampleMode::MEASUREMENTS
                                                                           : gfs::SampleMode::DETECTIONS);
        info8[0] = p.ops.size();
        info8[1] = p.pool.size();
        info8[2] = p.num_rows;
        info8[3] = p.ring;
        info8[4] = p.chans.size();
        info8[5] = p.max_loop_depth;
        info8[6] = gfs::frame_smem_bytes(p.num_rows, p.ring, (uint32_t)p.num_observables, 1,
                                         p.tables.size() <= 32 * GFS_TABLE_LEN ? (uint32_t)p.tables.size() : 0,
                                         p.ops.size() <= 256 ? (uint32_t)p.ops.size() : 0);
        info8[7] = p.num_detectors;
    });
}

gfs_status gfs_circuit_reference_sample(const gfs_circuit *c, uint8_t *out, uint64_t nbytes) {
    return guarded([&] {
        const std::vector<uint8_t> bits = gfs::reference_sample(c->circuit);
        if (nbytes < bits.size()) {
            throw std::invalid_argument("reference sample buffer too small");
        }
        std::memset(out, 0, nbytes);
        std::memcpy(out, bits.data(), bits.size());
    });
}

gfs_status gfs_program_noise(const gfs_circuit *c, uint32_t mode, uint64_t *occurrences, double *hits_per_block) {
    return guarded([&] {
        if (mode != GFS_MODE_DETECTIONS && mode != GFS_MODE_MEASUREMENTS) {
            throw std::invalid_argument("unknown sampling mode");
        }
        gfs::Program p = gfs::lower(c->circuit, mode == GFS_MODE_MEASUREMENTS ? gfs::SampleMode::MEASUREMENTS
                                                                           : gfs::SampleMode::DETECTIONS);
        *occurrences = p.noise_occurrences;
        *hits_per_block = p.hits_per_block;
    });
}

gfs_status gfs_sampler_create(const gfs_circuit *c, uint32_t mode, uint64_t seed, int device, gfs_sampler **out) {
    *out = nullptr;
    return guarded([&] {
        if (mode != GFS_MODE_DETECTIONS && mode != GFS_MODE_MEASUREMENTS) {
            throw std::invalid_argument("unknown sampling mode");
        }
        auto s = std::make_unique<gfs_sampler>();
        s->init(c, mode, seed, device);
        *out = s.release();
    });
}

void gfs_sampler_free(gfs_sampler *s) {
    delete s;
}

gfs_status gfs_sample_detections(gfs_sampler *s, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dets_stride,
                                 uint8_t *obs, uint64_t obs_stride) {
    return guarded([&] {
        if (s->mode != GFS_MODE_DETECTIONS) {
            throw std::invalid_argument("sampler was not created in detection mode");
        }
        s->detections(shots, flags, dets, dets_stride, obs, obs_stride, false);
    });
}

gfs_status gfs_sample_detections_device(gfs_sampler *s, uint64_t shots, uint32_t flags, void *dets,
                                        uint64_t dets_stride, void *obs, uint64_t obs_stride) {
    return guarded([&] {
        if (s->mode != GFS_MODE_DETECTIONS) {
            throw std::invalid_argument("sampler was not created in detection mode");
        }
        s->detections(shots, flags, (uint8_t *)dets, dets_stride, (uint8_t *)obs, obs_stride, true);
    });
}

gfs_status gfs_sample_detections_device_noalloc(gfs_sampler *s, uint64_t shots, uint32_t flags, void *dets,
                                                uint64_t dets_stride, void *obs, uint64_t obs_stride) {
    return guarded([&] { detections_noalloc(s, shots, flags, (uint8_t *)dets, dets_stride, (uint8_t *)obs, obs_stride); });
}

gfs_status gfs_sample_measurements(gfs_sampler *s, uint64_t shots, uint32_t flags, const uint8_t *ref_sample,
                                   uint8_t *out, uint64_t out_stride) {
    return guarded([&] { s->measurements(shots, flags, ref_sample, out, out_stride); });
}

gfs_status gfs_sampler_last_timings(const gfs_sampler *s, double *out4, uint64_t *counts2) {
    return guarded([&] {
        out4[0] = s->t_frame;
        out4[1] = s->t_transpose;
        out4[2] = s->t_copy;
        out4[3] = s->t_total;
        if (counts2) {
            counts2[0] = s->n_frame;
            counts2[1] = s->n_transpose;
        }
    });
}

gfs_status gfs_sampler_set_shape(gfs_sampler *s, int blocks_per_cta, int threads, int grid) {
    return guarded([&] {
        if (blocks_per_cta != 1 && blocks_per_cta != 2 && blocks_per_cta != 4) {
            throw std::invalid_argument("blocks_per_cta must be 1, 2 or 4");
        }
        ck(cudaSetDevice(s->device), "cudaSetDevice");
        s->choose_shape(blocks_per_cta, threads, grid, s->ring_pref);
    });
}

gfs_status gfs_sampler_set_ring_placement(gfs_sampler *s, int placement) {
    return guarded([&] {
        if (placement < -1 || placement > 1) {
            throw std::invalid_argument("ring placement must be -1 (automatic), 0 (shared memory) or 1 (global memory)");
        }
        ck(cudaSetDevice(s->device), "cudaSetDevice");
        s->ring_pref = placement;
        s->choose_shape(s->shape.blocks_per_cta, s->shape.threads, 0, placement);
    });
}

gfs_status gfs_sampler_get_shape(const gfs_sampler *s, int *blocks_per_cta, int *threads, int *grid,
                                 uint64_t *smem_bytes) {
    return guarded([&] {
        const gfs::LaunchShape &sh = s->lean_active() ? s->shape_lean : s->shape;
        *blocks_per_cta = sh.blocks_per_cta;
        *threads = sh.threads;
        *grid = sh.grid;
        *smem_bytes = sh.smem;
    });
}

gfs_status gfs_sampler_set_frame_kernel(gfs_sampler *s, int kind) {
    return guarded([&] {
        if (kind < -1 || kind > 1) {
            throw std::invalid_argument("frame kernel must be -1 (automatic), 0 (generic) or 1 (lean when possible)");
        }
        s->lean_pref = kind;
    });
}

gfs_status gfs_sampler_get_frame_kernel(const gfs_sampler *s, int *kind) {
    return guarded([&] { *kind = s->lean_active() ? 1 : 0; });
}

gfs_status gfs_measure_smem_peak(int device, double *bytes_per_s) {
    return guarded([&] {
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(gfs::measure_smem_peak(bytes_per_s), "shared-memory probe");
    });
}

gfs_status gfs_measure_int_peaks(int device, double *lop3_per_s, double *philox_per_s) {
    return guarded([&] {
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(gfs::measure_int_peaks(lop3_per_s, philox_per_s), "integer-issue probe");
    });
}

gfs_status gfs_sampler_set_stream_position(gfs_sampler *s, uint64_t shot) {
    return guarded([&] {
        if (shot % 128) {
            throw std::invalid_argument("the stream position must be a multiple of 128 shots");
        }
        s->next_block = shot / 128;
    });
}

gfs_status gfs_sampler_get_stream_position(const gfs_sampler *s, uint64_t *shot) {
    return guarded([&] { *shot = s->next_block * 128; });
}

gfs_status gfs_sampler_set_chunk_shots(gfs_sampler *s, uint64_t shots) {
    return guarded([&] { s->chunk_shots = shots; });
}

gfs_status gfs_sampler_set_noise_mode(gfs_sampler *s, int mode) {
    return guarded([&] {
        if (mode < -1 || mode > 1) {
            throw std::invalid_argument("noise mode must be -1 (automatic), 0 (inline) or 1 (hit lists when possible)");
        }
        ck(cudaSetDevice(s->device), "cudaSetDevice");
        s->hits_pref = mode;
        s->choose_shape(s->shape.blocks_per_cta, s->shape.threads, 0, s->shape.ring_global ? 1 : 0);
    });
}

gfs_status gfs_sampler_last_noise_ms(const gfs_sampler *s, double *ms) {
    return guarded([&] { *ms = s->t_noise; });
}

gfs_status gfs_sampler_set_hit_capacity(gfs_sampler *s, uint64_t records) {
    return guarded([&] {
        s->hit_capacity_override = records;
        s->occs_blocks = 0;  // re-plan the regions
    });
}

gfs_status gfs_sampler_last_counts(const gfs_sampler *s, uint64_t *counts4) {
    return guarded([&] {
        counts4[0] = s->n_frame;
        counts4[1] = s->n_transpose;
        counts4[2] = s->n_noise;
        counts4[3] = s->n_hit_overflows;
    });
}

gfs_status gfs_sampler_autotune(gfs_sampler *s, uint64_t trial_shots, double *best_ms) {
    return guarded([&] {
        ck(cudaSetDevice(s->device), "cudaSetDevice");
        double ms = s->autotune(trial_shots ? trial_shots : (uint64_t)1 << 18);
        if (best_ms) {
            *best_ms = ms;
        }
    });
}

}  // extern "C"
