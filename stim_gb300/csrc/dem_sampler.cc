// Detector-error-model sampling on the GPU: the host side of gfs_dem_* (include/stim_gb300.h).
//
// Replaces DemSampler<W> (src/stim/simulators/dem_sampler.inl:27-77) behind
// DetectorErrorModel.compile_sampler(seed=...).sample(shots, bit_packed, return_errors,
// recorded_errors_to_replay) (src/stim/simulators/dem_sampler.pybind.cc:40-80).  The reference draws every
// error row with biased_randomize_bits over all shots and XORs it into its symptoms' rows.  Here the model is
// parsed and grouped by probability once (dem.cc); a sample call runs, per chunk of 128-shot blocks, the
// sampling kernel (errors walked under the counter-based contract, symptoms XORed into detector rows) and the
// shot-major transposes.  Replayed errors take the converter's path instead: their rows are transposed in
// and folded into the outputs (each output the XOR of the mechanisms that list it).
#include "dem.h"
#include "sampler.h"

using namespace gfs_rt;

struct gfs_dem {
    int device = 0;
    cudaStream_t stream = nullptr;  // streams[0]
    uint64_t seed = 0;
    uint64_t next_block = 0;  // stream position, in 128-shot blocks
    gfs::DemModel model;
    gfs::DemLayout lay;
    DevBuf d_groups, d_units, d_sym_off, d_sym, d_tables, d_cg, d_cu0, d_cn, d_out_off, d_out_mech, d_expect;
    // Two pipeline slots: chunk k runs on slot k % 2, so its device->host copies overlap chunk k + 1's kernels.
    cudaStream_t streams[2] = {nullptr, nullptr};
    DevBuf det_buf[2], obs_buf[2], err_buf[2], in_buf[2], out_buf[2];

    ~gfs_dem() {
        for (cudaStream_t st : streams) {
            if (st) {
                cudaStreamSynchronize(st);
                cudaStreamDestroy(st);
            }
        }
    }
};

namespace {

void create(gfs_dem *d, const char *text, size_t len, uint64_t seed, int device) {
    d->model = gfs::parse_dem(std::string_view(text ? text : "", text ? len : 0));
    d->lay = gfs::layout_dem(d->model);
    int count = 0;
    ck(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count) {
        throw std::invalid_argument("no CUDA device " + std::to_string(device));
    }
    d->device = device;
    d->seed = seed;
    ck(cudaSetDevice(device), "cudaSetDevice");
    for (cudaStream_t &st : d->streams) {
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    d->stream = d->streams[0];
    const gfs::DemLayout &L = d->lay;
    upload(d->d_groups, L.groups, device, d->stream);
    upload(d->d_units, L.units, device, d->stream);
    upload(d->d_sym_off, d->model.sym_off, device, d->stream);
    upload(d->d_sym, d->model.sym, device, d->stream);
    upload(d->d_tables, L.tables, device, d->stream);
    upload(d->d_cg, L.chunk_group, device, d->stream);
    upload(d->d_cu0, L.chunk_unit0, device, d->stream);
    upload(d->d_cn, L.chunk_units, device, d->stream);
    upload(d->d_out_off, L.out_off, device, d->stream);
    upload(d->d_out_mech, L.out_mech, device, d->stream);
    std::vector<uint8_t> zeros((d->model.num_detectors + d->model.num_observables + 7) / 8 + 1, 0);
    upload(d->d_expect, zeros, device, d->stream);
    ck(cudaStreamSynchronize(d->stream), "upload");
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

void sample(gfs_dem *d, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dstride, uint8_t *obs,
            uint64_t ostride, uint8_t *errs, uint64_t estride, const uint8_t *replay, uint64_t rstride) {
    const uint64_t D = d->model.num_detectors, O = d->model.num_observables, E = d->model.num_errors();
    const bool packed = flags & GFS_BIT_PACKED;
    const uint64_t drow = packed ? (D + 7) / 8 : D, orow = packed ? (O + 7) / 8 : O, erow = packed ? (E + 7) / 8 : E;
    const uint64_t rrow = (E + 7) / 8;
    if ((dets && dstride < drow) || (obs && ostride < orow) || (errs && estride < erow)) {
        throw std::invalid_argument("output row stride too small");
    }
    if (replay && rstride < rrow) {
        throw std::invalid_argument("recorded error row stride too small");
    }
    ck(cudaSetDevice(d->device), "cudaSetDevice");
    const bool want_errs = errs != nullptr && !replay;
    const uint64_t per_block = (D + O) * 16 + ((want_errs || replay) ? E * 16 : 0) +
                               128 * (drow + orow + (want_errs ? erow : 0) + (replay ? rrow : 0));
    const uint64_t cb = std::max<uint64_t>(1, std::min<uint64_t>(512, ((uint64_t)1 << 30) / std::max<uint64_t>(1, per_block)));
    const uint64_t chunk = cb * 128;
    for (int k = 0; k < 2; k++) {
        d->det_buf[k].ensure(std::max<uint64_t>(16, cb * D * 16), d->device);
        d->obs_buf[k].ensure(std::max<uint64_t>(16, cb * O * 16), d->device);
        if (want_errs || replay) {
            d->err_buf[k].ensure(std::max<uint64_t>(16, cb * E * 16), d->device);
        }
        if (replay) {
            d->in_buf[k].ensure(std::max<uint64_t>(16, chunk * rrow), d->device);
        }
        d->out_buf[k].ensure(std::max<uint64_t>(16, chunk * (drow + orow + (want_errs ? erow : 0))), d->device);
    }
    const gfs::DemLayout &L = d->lay;
    // Kernels of the chunk at `done` in slot k, sampling from stream block `block0`.
    auto compute = [&](int k, uint64_t done, uint64_t cs, uint64_t block0) {
        cudaStream_t st = d->streams[k];
        const uint64_t nblk = (cs + 127) / 128;
        if (replay) {
            copy2d(d->in_buf[k].p, rrow, replay + done * rstride, rstride, rrow, cs, cudaMemcpyHostToDevice, st,
                   "copy recorded errors");
            gfs::RowsInArgs ra{(const uint8_t *)d->in_buf[k].p, rrow, cs, E, (uint4 *)d->err_buf[k].p};
            ck(gfs::launch_rows_from_shots(ra, st), "rows kernel launch");
            gfs::FoldArgs fa{(const uint4 *)d->err_buf[k].p, E, (const uint32_t *)d->d_out_off.p,
                             (const uint32_t *)d->d_out_mech.p, (const uint8_t *)d->d_expect.p, D, O, nblk,
                             (uint4 *)d->det_buf[k].p, (uint4 *)d->obs_buf[k].p};
            ck(gfs::launch_fold(fa, st), "fold kernel launch");
        } else {
            ck(cudaMemsetAsync(d->det_buf[k].p, 0, nblk * D * 16, st), "memset");
            ck(cudaMemsetAsync(d->obs_buf[k].p, 0, nblk * O * 16, st), "memset");
            if (want_errs) {
                ck(cudaMemsetAsync(d->err_buf[k].p, 0, nblk * E * 16, st), "memset");
            }
            gfs::DemArgs a{};
            a.groups = (const gfs::DemGroup *)d->d_groups.p;
            a.units = (const uint32_t *)d->d_units.p;
            a.sym_off = (const uint32_t *)d->d_sym_off.p;
            a.sym = (const uint32_t *)d->d_sym.p;
            a.tables = (const uint32_t *)d->d_tables.p;
            a.chunk_group = (const uint32_t *)d->d_cg.p;
            a.chunk_unit0 = (const uint32_t *)d->d_cu0.p;
            a.chunk_units = (const uint32_t *)d->d_cn.p;
            a.nchunks = (uint32_t)L.chunk_group.size();
            a.seed = d->seed;
            a.block0 = block0;
            a.nblk = nblk;
            a.D = D;
            a.O = O;
            a.E = E;
            a.dets = (uint4 *)d->det_buf[k].p;
            a.obs = (uint4 *)d->obs_buf[k].p;
            a.errs = want_errs ? (uint4 *)d->err_buf[k].p : nullptr;
            ck(gfs::launch_dem_sample(a, st), "dem kernel launch");
        }
        uint8_t *dout = (uint8_t *)d->out_buf[k].p, *oout = dout + chunk * drow, *eout = oout + chunk * orow;
        auto tr = [&](const uint4 *src, uint64_t n, uint8_t *out, uint64_t stride) {
            gfs::TransposeArgs t{};
            t.src0 = src;
            t.n0 = n;
            t.nshots = cs;
            t.out = out;
            t.out_stride = stride;
            t.bit_packed = packed ? 1 : 0;
            ck(gfs::launch_transpose(t, st), "transpose launch");
        };
        if (dets && drow) {
            tr((const uint4 *)d->det_buf[k].p, D, dout, drow);
        }
        if (obs && orow) {
            tr((const uint4 *)d->obs_buf[k].p, O, oout, orow);
        }
        if (want_errs && erow) {
            tr((const uint4 *)d->err_buf[k].p, E, eout, erow);
        }
    };
    auto copy_out = [&](int k, uint64_t done, uint64_t cs) {
        cudaStream_t st = d->streams[k];
        uint8_t *dout = (uint8_t *)d->out_buf[k].p, *oout = dout + chunk * drow, *eout = oout + chunk * orow;
        if (dets && drow) {
            copy2d(dets + done * dstride, dstride, dout, drow, drow, cs, cudaMemcpyDeviceToHost, st, "copy dets");
        }
        if (obs && orow) {
            copy2d(obs + done * ostride, ostride, oout, orow, orow, cs, cudaMemcpyDeviceToHost, st, "copy obs");
        }
        if (want_errs && erow) {
            copy2d(errs + done * estride, estride, eout, erow, erow, cs, cudaMemcpyDeviceToHost, st, "copy errs");
        }
    };
    // Chunk k's copies are issued after chunk k + 1's kernels are queued (a copy into pageable memory may hold
    // the calling thread until it completes); a slot is reused once its previous chunk has left.
    struct Pending {
        uint64_t done, cs;
    };
    Pending pend[2] = {};
    bool used[2] = {false, false};
    int prev = -1;
    uint64_t n = 0;
    for (uint64_t done = 0; done < shots; n++) {
        const int k = (int)(n & 1);
        const uint64_t cs = std::min<uint64_t>(shots - done, chunk);
        if (used[k]) {
            ck(cudaStreamSynchronize(d->streams[k]), "dem sample");
        }
        compute(k, done, cs, d->next_block);
        if (!replay) {
            d->next_block += (cs + 127) / 128;
        }
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
    for (cudaStream_t st : d->streams) {
        ck(cudaStreamSynchronize(st), "dem sample");
    }
    if (errs && replay && erow) {
        // Replayed errors are returned as given (as the reference returns its replayed error table).
        for (uint64_t s = 0; s < shots; s++) {
            if (packed) {
                std::memcpy(errs + s * estride, replay + s * rstride, rrow);
            } else {
                for (uint64_t e = 0; e < E; e++) {
                    errs[s * estride + e] = (replay[s * rstride + (e >> 3)] >> (e & 7)) & 1;
                }
            }
        }
    }
}

}  // namespace

extern "C" {

gfs_status gfs_dem_parse_stats(const char *text, size_t len, uint64_t *stats3) {
    return guarded([&] {
        const gfs::DemModel m = gfs::parse_dem(std::string_view(text ? text : "", text ? len : 0));
        stats3[0] = m.num_detectors;
        stats3[1] = m.num_observables;
        stats3[2] = m.num_errors();
    });
}

gfs_status gfs_dem_create(const char *text, size_t len, uint64_t seed, int device, gfs_dem **out) {
    return guarded([&] {
        auto d = std::make_unique<gfs_dem>();
        create(d.get(), text, len, seed, device);
        *out = d.release();
    });
}

void gfs_dem_free(gfs_dem *d) {
    delete d;
}

gfs_status gfs_dem_sample(gfs_dem *d, uint64_t shots, uint32_t flags, uint8_t *dets, uint64_t dets_stride,
                          uint8_t *obs, uint64_t obs_stride, uint8_t *errs, uint64_t errs_stride,
                          const uint8_t *replay, uint64_t replay_stride) {
    return guarded([&] {
        sample(d, shots, flags, dets, dets_stride, obs, obs_stride, errs, errs_stride, replay, replay_stride);
    });
}

}  // extern "C"
