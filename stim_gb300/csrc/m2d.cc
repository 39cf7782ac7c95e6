// Measurements to detection events on the GPU: the host side of gfs_m2d_* (include/stim_gb300.h).
//
// Replaces CompiledMeasurementsToDetectionEventsConverter (src/stim/simulators/measurements_to_detection_events
// .pybind.cc:80-150) and its helper (measurements_to_detection_events.inl:29-131).  The reference walks the
// noiseless circuit once per batch with a frame simulator and XORs each detector's (and observable's)
// referenced measurement rows, inverting a row when the reference sample's parity of those measurements is
// 1.  Here the walk happens once, at creation: every output becomes a list of absolute measurement indices
// plus an expectation bit (the reference sample's parity), uploaded to the device.  A conversion then runs
// three kernels per chunk of shots: shot-major input bits into 128-shot measurement rows, the XOR fold, and
// the usual shot-major output transpose.
//
// Sweep bits: the reference's frame simulator turns sweep-controlled Paulis into extra flips of measurement
// results (and of observables' Pauli terms).  Without sweep data, or with all-zero sweep bits, those flips
// vanish and the fold is the whole answer.  Otherwise the frame kernel runs the circuit's noiseless copy with
// no randomization (the reference's aliased_noiseless_circuit and
// guarantee_anticommutation_via_frame_randomization = false) over the chunk's sweep table, and the fold XORs
// its detector and observable rows into the outputs.
#include "formats.h"
#include "sampler.h"

using namespace gfs_rt;

struct gfs_m2d {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t M = 0, D = 0, O = 0;
    uint64_t num_sweep_bits = 0;
    bool sweep_controlled = false;  // the circuit has sweep-controlled operations
    std::vector<uint32_t> off, idx;
    std::vector<uint8_t> expect;
    DevBuf d_off, d_idx, d_expect, sweep_in, sweep_rows;
    // Three pipeline slots: chunk k runs on slot k % 3 (its own stream and buffers), so chunk k's device->host
    // copy overlaps chunk k + 1's host->device copy and kernels, and chunk k + 2's copy in need not wait for it.
    static constexpr int kSlots = 3;
    cudaStream_t streams[kSlots] = {};
    DevBuf in_buf[kSlots], rows_buf[kSlots], det_buf[kSlots], obs_buf[kSlots], out_buf[kSlots];
    std::unique_ptr<gfs_sampler> sweep_sim;  // sweep-controlled circuits: the noiseless frame program

    ~gfs_m2d() {
        for (cudaStream_t s : streams) {
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        }
    }
};

namespace {

// Walks `c` with REPEAT blocks unrolled (the reference's for_each_operation, circuit.h:180-193): each
// DETECTOR and each OBSERVABLE_INCLUDE record target becomes absolute measurement indices.
struct Lists {
    std::vector<std::vector<uint32_t>> det;  // per detector
    std::vector<std::vector<uint32_t>> obs;  // per observable (all its OBSERVABLE_INCLUDE record targets)
    uint64_t meas = 0;
    uint64_t sweep_bits = 0;
    bool sweep_controlled = false;
};

void walk(const gfs::Circuit &c, Lists &l) {
    for (const gfs::Instruction &op : c.ops) {
        if (op.gate == GFS_REPEAT) {
            for (uint64_t r = 0; r < op.reps; r++) {
                walk(c.blocks[op.block], l);
            }
            continue;
        }
        auto absolute = [&](uint32_t t) -> uint32_t {
            const uint64_t k = t & GFS_T_VALUE_MASK;
            if (k == 0) {
                throw std::out_of_range("Lookback must be non-zero.");
            }
            if (k > l.meas) {
                throw std::out_of_range("Referred to a measurement record before the beginning of time.");
            }
            return (uint32_t)(l.meas - k);
        };
        if (op.gate == GFS_DETECTOR) {
            std::vector<uint32_t> refs;
            for (uint32_t t : op.targets) {
                if (t & GFS_T_RECORD) {
                    refs.push_back(absolute(t));
                }
            }
            l.det.push_back(std::move(refs));
            continue;
        }
        if (op.gate == GFS_OBSERVABLE_INCLUDE) {
            const size_t k = (size_t)op.args[0];
            if (l.obs.size() <= k) {
                l.obs.resize(k + 1);
            }
            for (uint32_t t : op.targets) {
                if (t & GFS_T_RECORD) {
                    l.obs[k].push_back(absolute(t));
                }
                // Pauli targets read the frame, which without sweep data stays zero in the reference.
            }
            continue;
        }
        for (uint32_t t : op.targets) {
            if (t & GFS_T_SWEEP) {
                l.sweep_controlled = true;
                l.sweep_bits = std::max<uint64_t>(l.sweep_bits, (uint64_t)(t & GFS_T_VALUE_MASK) + 1);
            }
        }
        l.meas += op.count_results();
        if (l.meas > 0xFFFFFFFFull) {
            throw std::invalid_argument("too many measurements for the GPU converter");
        }
    }
}

void create(gfs_m2d *m, const gfs_circuit *c, const uint8_t *ref, int device) {
    int count = 0;
    ck(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count) {
        throw std::invalid_argument("no CUDA device " + std::to_string(device));
    }
    Lists l;
    walk(c->circuit, l);
    m->device = device;
    m->M = l.meas;
    m->D = l.det.size();
    m->O = std::max<uint64_t>(l.obs.size(), c->stats.num_observables);
    l.obs.resize(m->O);
    m->num_sweep_bits = l.sweep_bits;
    m->sweep_controlled = l.sweep_controlled;
    if (l.sweep_controlled) {
        gfs::LowerOptions opts;
        opts.no_randomization = true;
        opts.sweep = true;
        m->sweep_sim = std::make_unique<gfs_sampler>();
        m->sweep_sim->init_program(gfs::lower(gfs::noiseless_copy(c->circuit), gfs::SampleMode::DETECTIONS, opts),
                                   GFS_MODE_DETECTIONS, 0, device);
        if (m->sweep_sim->prog.num_sweep_bits > m->num_sweep_bits) {
            throw std::logic_error("sweep bit count mismatch in the converter");
        }
    }
    const uint64_t n = m->D + m->O;
    m->off.assign(1, 0);
    m->expect.assign((n + 7) / 8, 0);
    uint64_t o = 0;
    for (auto *group : {&l.det, &l.obs}) {
        for (const std::vector<uint32_t> &refs : *group) {
            bool parity = false;
            for (uint32_t i : refs) {
                m->idx.push_back(i);
                if (ref) {
                    parity ^= (ref[i >> 3] >> (i & 7)) & 1;
                }
            }
            if (m->idx.size() > 0xFFFFFFFFull) {
                throw std::invalid_argument("too many record references for the GPU converter");
            }
            m->off.push_back((uint32_t)m->idx.size());
            if (parity) {
                m->expect[o >> 3] |= (uint8_t)(1u << (o & 7));
            }
            o++;
        }
    }
    ck(cudaSetDevice(device), "cudaSetDevice");
    for (cudaStream_t &st : m->streams) {
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    m->stream = m->streams[0];
    upload(m->d_off, m->off, device, m->stream);
    upload(m->d_idx, m->idx, device, m->stream);
    upload(m->d_expect, m->expect, device, m->stream);
    ck(cudaStreamSynchronize(m->stream), "upload");
}

void copy2d(void *dst, uint64_t dpitch, const void *src, uint64_t spitch, uint64_t width, uint64_t rows,
            cudaMemcpyKind kind, cudaStream_t s, const char *what) {
    if (!width || !rows) {
        return;
    }
    if (dpitch == width && spitch == width) {
        ck(cudaMemcpyAsync(dst, src, width * rows, kind, s), what);
    } else {
        ck(cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, rows, kind, s), what);
    }
}

void convert(gfs_m2d *m, uint64_t shots, const uint8_t *meas, uint64_t meas_stride, const uint8_t *sweep,
             uint64_t sweep_stride, uint32_t flags, uint8_t *dets, uint64_t dstride, uint8_t *obs, uint64_t ostride) {
    const uint64_t M = m->M, D = m->D, O = m->O;
    const uint64_t mrow = (M + 7) / 8;
    if (meas_stride < mrow) {
        throw std::invalid_argument("measurement row stride too small");
    }
    const uint64_t srow = (m->num_sweep_bits + 7) / 8;
    bool use_sweep = false;  // some sweep bit is set and some operation reads one
    if (sweep && m->sweep_controlled) {
        if (sweep_stride < srow) {
            throw std::invalid_argument("sweep row stride too small");
        }
        for (uint64_t s = 0; s < shots && !use_sweep; s++) {
            for (uint64_t b = 0; b < srow && !use_sweep; b++) {
                use_sweep = sweep[s * sweep_stride + b] != 0;
            }
        }
    }
    const bool packed = flags & GFS_BIT_PACKED;
    const uint64_t nd = D + ((flags & GFS_PREPEND_OBSERVABLES) ? O : 0) + ((flags & GFS_APPEND_OBSERVABLES) ? O : 0);
    const uint64_t drow = packed ? (nd + 7) / 8 : nd;
    const uint64_t orow = packed ? (O + 7) / 8 : O;
    if (dets && dstride < drow) {
        throw std::invalid_argument("dets row stride too small");
    }
    if (obs && ostride < orow) {
        throw std::invalid_argument("obs row stride too small");
    }
    ck(cudaSetDevice(m->device), "cudaSetDevice");
    // Chunks of up to 2^16 shots, fewer when a circuit's rows are large (about 1 GiB of device buffers).
    const uint64_t per_block = (M + D + O) * 16 + 128 * (mrow + drow + orow);
    uint64_t cb = std::max<uint64_t>(1, std::min<uint64_t>(512, ((uint64_t)1 << 30) / std::max<uint64_t>(1, per_block)));
    const uint64_t chunk = cb * 128;
    for (int k = 0; k < gfs_m2d::kSlots; k++) {
        m->in_buf[k].ensure(std::max<uint64_t>(16, chunk * mrow), m->device);
        m->rows_buf[k].ensure(std::max<uint64_t>(16, cb * M * 16), m->device);
        m->det_buf[k].ensure(std::max<uint64_t>(16, cb * D * 16), m->device);
        m->obs_buf[k].ensure(std::max<uint64_t>(16, cb * O * 16), m->device);
        m->out_buf[k].ensure(std::max<uint64_t>(16, chunk * (drow + orow)), m->device);
    }
    if (use_sweep) {
        m->sweep_in.ensure(std::max<uint64_t>(16, chunk * srow), m->device);
        // Room for the frame kernel's padding blocks (up to four 128-shot blocks per CTA slice).
        m->sweep_rows.ensure(std::max<uint64_t>(16, (cb + 4) * m->num_sweep_bits * 16), m->device);
    }
    if ((flags & GFS_PREPEND_OBSERVABLES) && (flags & GFS_APPEND_OBSERVABLES)) {
        throw std::invalid_argument("prepend and append observables together are not supported");
    }
    // Host->device copy and kernels of the chunk at `done` in slot k (sweep rows, when used, are XORed in).
    auto compute = [&](int k, uint64_t done, uint64_t cs, const uint4 *base_dets, const uint4 *base_obs) {
        cudaStream_t st = m->streams[k];
        const uint64_t nblk = (cs + 127) / 128;
        copy2d(m->in_buf[k].p, mrow, meas + done * meas_stride, meas_stride, mrow, cs, cudaMemcpyHostToDevice, st,
               "copy measurements");
        if (M == 0) {
            ck(cudaMemsetAsync(m->rows_buf[k].p, 0, 16, st), "memset");
        }
        gfs::RowsInArgs ra{(const uint8_t *)m->in_buf[k].p, mrow, cs, M, (uint4 *)m->rows_buf[k].p};
        ck(gfs::launch_rows_from_shots(ra, st), "rows kernel launch");
        gfs::FoldArgs fa{(const uint4 *)m->rows_buf[k].p, M, (const uint32_t *)m->d_off.p, (const uint32_t *)m->d_idx.p,
                         (const uint8_t *)m->d_expect.p, D, O, nblk, (uint4 *)m->det_buf[k].p,
                         (uint4 *)m->obs_buf[k].p};
        fa.base_dets = base_dets;
        fa.base_obs = base_obs;
        ck(gfs::launch_fold(fa, st), "fold kernel launch");
        const uint4 *dt = (const uint4 *)m->det_buf[k].p, *ot = (const uint4 *)m->obs_buf[k].p;
        uint8_t *dout = (uint8_t *)m->out_buf[k].p, *oout = dout + chunk * drow;
        auto tr = [&](const uint4 *s0, uint64_t n0, const uint4 *s1, uint64_t n1, uint8_t *out, uint64_t stride) {
            gfs::TransposeArgs t{};
            t.src0 = s0;
            t.n0 = n0;
            t.src1 = s1;
            t.n1 = n1;
            t.nshots = cs;
            t.out = out;
            t.out_stride = stride;
            t.bit_packed = packed ? 1 : 0;
            ck(gfs::launch_transpose(t, st), "transpose launch");
        };
        if (dets && drow) {
            if (flags & GFS_PREPEND_OBSERVABLES) {
                tr(ot, O, dt, D, dout, drow);
            } else if (flags & GFS_APPEND_OBSERVABLES) {
                tr(dt, D, ot, O, dout, drow);
            } else {
                tr(dt, D, nullptr, 0, dout, drow);
            }
        }
        if (obs && orow) {
            tr(ot, O, nullptr, 0, oout, orow);
        }
    };
    auto copy_out = [&](int k, uint64_t done, uint64_t cs) {
        cudaStream_t st = m->streams[k];
        uint8_t *dout = (uint8_t *)m->out_buf[k].p, *oout = dout + chunk * drow;
        if (dets && drow) {
            copy2d(dets + done * dstride, dstride, dout, drow, drow, cs, cudaMemcpyDeviceToHost, st, "copy dets");
        }
        if (obs && orow) {
            copy2d(obs + done * ostride, ostride, oout, orow, orow, cs, cudaMemcpyDeviceToHost, st, "copy obs");
        }
    };
    if (use_sweep) {
        // Sweep data: one chunk at a time on slot 0 (the frame program runs on its sampler's stream).
        for (uint64_t done = 0; done < shots;) {
            const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
            const uint64_t nblk = (cs + 127) / 128;
            copy2d(m->sweep_in.p, srow, sweep + done * sweep_stride, sweep_stride, srow, cs, cudaMemcpyHostToDevice,
                   m->streams[0], "copy sweep bits");
            gfs::RowsInArgs sa{(const uint8_t *)m->sweep_in.p, srow, cs, m->num_sweep_bits, (uint4 *)m->sweep_rows.p};
            ck(gfs::launch_rows_from_shots(sa, m->streams[0]), "rows kernel launch");
            ck(cudaStreamSynchronize(m->streams[0]), "sweep rows");
            gfs_sampler &sim = *m->sweep_sim;
            sim.sweep_rows = (const uint4 *)m->sweep_rows.p;
            sim.nsweep = (uint32_t)m->num_sweep_bits;
            sim.run_frame(nblk, 0);
            ck(cudaStreamSynchronize(sim.stream), "sweep frames");
            sim.sweep_rows = nullptr;
            if (sim.check_status()) {
                throw std::logic_error("noiseless frame program reported a hit-list overflow");
            }
            compute(0, done, cs, (const uint4 *)sim.det_tmp.p, (const uint4 *)sim.obs_tmp.p);
            copy_out(0, done, cs);
            ck(cudaStreamSynchronize(m->streams[0]), "convert");
            done += cs;
        }
        return;
    }
    // Chunk k's copy out is issued after chunk k + 1's copy in and kernels are queued (a copy to or from
    // pageable memory may hold the calling thread until it completes); a slot is reused once its previous
    // chunk has left.
    struct Pending {
        uint64_t done, cs;
    };
    Pending pend[gfs_m2d::kSlots] = {};
    bool used[gfs_m2d::kSlots] = {};
    int prev = -1;
    uint64_t n = 0;
    for (uint64_t done = 0; done < shots; n++) {
        const int k = (int)(n % gfs_m2d::kSlots);
        const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
        if (used[k]) {
            ck(cudaStreamSynchronize(m->streams[k]), "convert");
        }
        compute(k, done, cs, nullptr, nullptr);
        pend[k] = Pending{done, cs};
        used[k] = true;
        if (prev >= 0) {
            copy_out(prev, pend[prev].done, pend[prev].cs);
        }
        prev = k;
        done += cs;
    }
    if (prev >= 0) {
        copy_out(prev, pend[prev].done, pend[prev].cs);
    }
    for (cudaStream_t st : m->streams) {
        ck(cudaStreamSynchronize(st), "convert");
    }
}

// Files opened like the reference's RaiiFile (src/stim/io/raii_file.cc:44-66): no path, no file.
struct PathFile {
    FILE *f = nullptr;
    PathFile(const char *path, const char *mode) {
        if (path && *path) {
            f = fopen(path, mode);
            if (!f) {
                throw std::invalid_argument("Failed to open '" + std::string(path) + "' for " +
                                            (*mode == 'r' ? "reading." : "writing."));
            }
        }
    }
    ~PathFile() {
        if (f) {
            fclose(f);
        }
    }
};

// CompiledMeasurementsToDetectionEventsConverter.convert_file (measurements_to_detection_events.pybind.cc:45-77)
// through stream_measurements_to_detection_events_helper (measurements_to_detection_events.inl:190-294): records
// are read in chunks of 65,536 shots (measurements and, when given, as many sweep records), converted on the
// device by convert() and written in the requested formats, detection events with D / L prefixes and
// observables (obs_path) with L prefixes.
void convert_file(gfs_m2d *m, const char *meas_path, const char *meas_format, const char *sweep_path,
                  const char *sweep_format, const char *dets_path, const char *dets_format, bool append,
                  const char *obs_path, const char *obs_format) {
    const gfs::Format fin = gfs::parse_format(meas_format ? meas_format : "01");
    const gfs::Format fsweep = gfs::parse_format(sweep_format ? sweep_format : "01");
    const gfs::Format fout = gfs::parse_format(dets_format ? dets_format : "01");
    PathFile in(meas_path, "rb"), obs_out(obs_path, "wb"), sweep_in(sweep_path, "rb"), dets_out(dets_path, "wb");
    const gfs::Format fobs = gfs::parse_format(obs_format ? obs_format : "01");
    if (!in.f) {
        throw std::invalid_argument("measurements_filepath is required");
    }
    if (!dets_out.f) {
        throw std::invalid_argument("detection_events_filepath is required");
    }
    const uint64_t M = m->M, D = m->D, O = m->O, S = m->num_sweep_bits;
    gfs::RowReader meas_reader(in.f, fin, M);
    // The reference's record writers cannot write ptb64 one record at a time (measure_record_writer.cc:33-34).
    if ((obs_out.f && fobs == gfs::Format::PTB64) || fout == gfs::Format::PTB64) {
        throw std::invalid_argument("SAMPLE_FORMAT_PTB64 incompatible with SingleMeasurementRecord");
    }
    std::unique_ptr<gfs::RowReader> sweep_reader;
    if (sweep_in.f) {
        sweep_reader = std::make_unique<gfs::RowReader>(sweep_in.f, fsweep, S);
    }
    if (meas_reader.empty_records()) {
        throw std::invalid_argument(
            "Can't tell how many shots are in the measurement data.\n"
            "The circuit has no measurements and the measurement format encodes empty shots into no bytes.");
    }
    const uint64_t chunk = 1 << 16;
    const uint64_t mrow = (M + 7) / 8, srow = (S + 7) / 8, drow = (D + (append ? O : 0) + 7) / 8, orow = (O + 7) / 8;
    std::vector<uint8_t> meas(chunk * mrow + 1), sweep(chunk * srow + 1), dets(chunk * drow + 1), obs(chunk * orow + 1);
    const bool sweep_rows = sweep_reader && !sweep_reader->empty_records();
    uint64_t total = 0;
    for (;;) {
        uint64_t n = 0;
        while (n < chunk && meas_reader.read(meas.data() + n * mrow)) {
            n++;
        }
        if (sweep_reader) {
            uint64_t ns = 0;
            while (ns < chunk && sweep_reader->read(sweep.data() + ns * srow)) {
                ns++;
            }
            if (ns != n && sweep_rows) {
                std::string msg = "The sweep data contained a different number of shots than the measurement data.\n";
                msg += "There was " + std::to_string(n + total) + " shot records total.\n";
                if (ns < n) {
                    msg += "But there was " + std::to_string(n + ns) + " sweep records total.";
                } else {
                    msg += "But there was at least " + std::to_string(n + ns) + " sweep records.";
                }
                throw std::invalid_argument(msg);
            }
        }
        if (n == 0) {
            break;
        }
        total += n;
        convert(m, n, meas.data(), std::max<uint64_t>(1, mrow), sweep_rows ? sweep.data() : nullptr,
                std::max<uint64_t>(1, srow), GFS_BIT_PACKED | (append ? GFS_APPEND_OBSERVABLES : 0), dets.data(),
                std::max<uint64_t>(1, drow), obs_out.f ? obs.data() : nullptr, std::max<uint64_t>(1, orow));
        gfs::write_rows(dets_out.f, fout, dets.data(), std::max<uint64_t>(1, drow), n, D + (append ? O : 0), 'D', 'L',
                        D);
        if (obs_out.f) {
            gfs::write_rows(obs_out.f, fobs, obs.data(), std::max<uint64_t>(1, orow), n, O, 'L', 'L', 0);
        }
    }
}

}  // namespace

extern "C" {

gfs_status gfs_read_shot_data_file(const char *path, const char *format, uint64_t num_measurements,
                                   uint64_t num_detectors, uint64_t num_observables, uint8_t *out,
                                   uint64_t capacity_shots, uint64_t *shots) {
    return guarded([&] {
        const gfs::Format f = gfs::parse_format(format ? format : "01");
        PathFile in(path, "rb");
        if (!in.f) {
            throw std::invalid_argument("path is required");
        }
        gfs::RowReader reader(in.f, f, num_measurements, num_detectors, num_observables);
        const uint64_t nb = (num_measurements + num_detectors + num_observables + 7) / 8;
        std::vector<uint8_t> row(nb + 1);
        uint64_t k = 0;
        while (reader.read(row.data())) {
            if (k >= capacity_shots) {
                throw std::invalid_argument("the file holds more records than the output buffer");
            }
            std::copy(row.begin(), row.begin() + nb, out + k * nb);
            k++;
        }
        *shots = k;
    });
}

gfs_status gfs_write_shot_data_file(const uint8_t *rows, uint64_t stride, uint64_t shots, const char *path,
                                    const char *format, uint64_t num_measurements, uint64_t num_detectors,
                                    uint64_t num_observables) {
    return guarded([&] {
        if (num_measurements && (num_detectors || num_observables)) {
            throw std::invalid_argument("num_measurements and (num_detectors or num_observables)");
        }
        const gfs::Format f = gfs::parse_format(format ? format : "01");
        PathFile out(path, "wb");
        if (!out.f) {
            throw std::invalid_argument("path is required");
        }
        const uint64_t n = num_measurements + num_detectors + num_observables;
        const char c1 = num_measurements ? 'M' : 'D', c2 = num_measurements ? 'M' : 'L';
        gfs::write_rows(out.f, f, rows, std::max<uint64_t>(1, stride), shots, n, c1, c2,
                        num_measurements + num_detectors);
    });
}

gfs_status gfs_m2d_convert_file(gfs_m2d *m, const char *meas_path, const char *meas_format, const char *sweep_path,
                                const char *sweep_format, const char *dets_path, const char *dets_format,
                                int append_observables, const char *obs_path, const char *obs_format) {
    return guarded([&] {
        convert_file(m, meas_path, meas_format, sweep_path, sweep_format, dets_path, dets_format,
                     append_observables != 0, obs_path, obs_format);
    });
}

gfs_status gfs_m2d_create(const gfs_circuit *c, const uint8_t *ref_sample, int device, gfs_m2d **out) {
    return guarded([&] {
        auto m = std::make_unique<gfs_m2d>();
        create(m.get(), c, ref_sample, device);
        *out = m.release();
    });
}

void gfs_m2d_free(gfs_m2d *m) {
    delete m;
}

gfs_status gfs_m2d_stats(const gfs_m2d *m, uint64_t *stats4) {
    return guarded([&] {
        stats4[0] = m->M;
        stats4[1] = m->D;
        stats4[2] = m->O;
        stats4[3] = m->num_sweep_bits;
    });
}

gfs_status gfs_m2d_convert(gfs_m2d *m, uint64_t shots, const uint8_t *meas, uint64_t meas_stride,
                           const uint8_t *sweep, uint64_t sweep_stride, uint32_t flags, uint8_t *dets,
                           uint64_t dets_stride, uint8_t *obs, uint64_t obs_stride) {
    return guarded([&] { convert(m, shots, meas, meas_stride, sweep, sweep_stride, flags, dets, dets_stride, obs, obs_stride); });
}

}  // extern "C"
