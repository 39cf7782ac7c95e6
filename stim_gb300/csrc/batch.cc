// Batched sampling: the shots of many circuits in one persistent frame-kernel launch (batch_frame_kernel),
// followed by each circuit's shot-major transpose, captured once as a CUDA graph and replayed while the
// request geometry (shot counts, destinations, launch shape) stays the same.
//
// Each circuit keeps the random stream of its own sampler: circuit j's shots are the next shots of
// samplers[j] (block0 = its shot counter), so a batch returns bit for bit what the samplers' own
// sample calls would have returned, in the same order.  The reference has no batched mode; its nearest
// equivalent is one CompiledDetectorSampler per circuit (compiled_detector_sampler.pybind.cc:216-322).
#include <unordered_map>

#include "sampler.h"

struct gfs_batch {
    using DevBuf = gfs_rt::DevBuf;
    int device = 0;
    std::vector<gfs_sampler *> samplers;
    std::vector<uint32_t> order;  // circuits by estimated cost per 128-shot block, most expensive first
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    DevBuf d_desc, d_prefix, d_counter, d_status, det_arena, obs_arena, out_arena, ring_buf;
    gfs::LaunchShape shape{};
    int num_sms = 0;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> graph_key;
    double t_frame = 0, t_transpose = 0, t_copy = 0, t_total = 0;
    uint64_t n_frame = 0, n_transpose = 0, n_graph_launches = 0, n_graph_builds = 0;

    ~gfs_batch() {
        cudaSetDevice(device);
        if (stream) {
            cudaStreamSynchronize(stream);
        }
        if (exec) {
            cudaGraphExecDestroy(exec);
        }
        for (auto &e : ev) {
            if (e) {
                cudaEventDestroy(e);
            }
        }
        if (stream) {
            cudaStreamDestroy(stream);
        }
    }

    void init(gfs_sampler *const *s, size_t n) {
        if (n == 0) {
            throw std::invalid_argument("a batch needs at least one sampler");
        }
        samplers.assign(s, s + n);
        device = samplers[0]->device;
        for (auto *x : samplers) {
            if (!x) {
                throw std::invalid_argument("null sampler in batch");
            }
            if (x->mode != GFS_MODE_DETECTIONS) {
                throw std::invalid_argument("batched sampling needs samplers created in detection mode");
            }
            if (x->device != device) {
                throw std::invalid_argument("all samplers of a batch must be on the same device");
            }
        }
        order.resize(n);
        for (size_t j = 0; j < n; j++) {
            order[j] = (uint32_t)j;
        }
        std::stable_sort(order.begin(), order.end(),
                         [&](uint32_t a, uint32_t b) { return samplers[a]->prog.work > samplers[b]->prog.work; });
        ck(cudaSetDevice(device), "cudaSetDevice");
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &e : ev) {
            ck(cudaEventCreate(&e), "cudaEventCreate");
        }
        d_counter.ensure(16, device);
        d_status.ensure(16, device);
        ck(cudaMemsetAsync(d_status.p, 0, 16, stream), "memset");
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        num_sms = prop.multiProcessorCount;
        set_shape(1, 256, -1);
        ck(cudaStreamSynchronize(stream), "init");
    }

    size_t smem_for(int bpc, bool ring_global) const {
        size_t m = 0;
        for (auto *x : samplers) {
            m = std::max(m, x->smem_for(bpc, ring_global));
        }
        return m;
    }

    uint64_t ring_stride(int bpc) const {
        uint64_t m = 0;
        for (auto *x : samplers) {
            m = std::max<uint64_t>(m, (uint64_t)bpc * x->prog.ring);
        }
        return m;
    }

    // Resident 128-shot blocks per SM for a candidate shape (0 = does not fit).
    int resident(int bpc, int threads, bool ring_global, gfs::LaunchShape *out) const {
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        gfs::LaunchShape t{bpc, threads, 1, smem_for(bpc, ring_global), ring_global};
        if (t.smem > (size_t)prop.sharedMemPerBlockOptin) {
            return 0;
        }
        int per = 0;
        if (gfs::batch_frame_kernel_max_ctas_per_sm(t, &per) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        t.grid = per * num_sms;
        if (out) {
            *out = t;
        }
        return per * bpc;
    }

    // ring: 0 shared memory, 1 global memory, -1 whichever keeps more blocks resident.
    void set_shape(int bpc, int threads, int ring) {
        if (bpc != 1 && bpc != 2 && bpc != 4) {
            throw std::invalid_argument("blocks_per_cta must be 1, 2 or 4");
        }
        if (threads <= 0 || threads > 256 || threads % 32) {
            throw std::invalid_argument("threads per CTA must be a multiple of 32 in [32, 256]");
        }
        gfs::LaunchShape in_smem{}, in_global{};
        int rs = ring == 1 ? 0 : resident(bpc, threads, false, &in_smem);
        int rg = ring == 0 ? 0 : resident(bpc, threads, true, &in_global);
        if (rs == 0 && rg == 0) {
            throw std::invalid_argument("the largest circuit of the batch does not fit in shared memory with " +
                                        std::to_string(bpc) + " blocks per CTA");
        }
        bool global = ring == 1 || (ring < 0 && (rs == 0 || rg * 2 >= rs * 3));
        shape = global ? in_global : in_smem;
        drop_graph();
    }

    void drop_graph() {
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        graph_key.clear();
    }

    struct Plan {
        std::vector<gfs::KernelArgs> desc;  // in launch order
        std::vector<uint32_t> prefix;
        std::vector<uint64_t> det_off, obs_off, block0, nblk;  // per circuit (input order)
        uint64_t det_total = 0, obs_total = 0;
    };

    Plan plan(const uint64_t *shots) const {
        Plan pl;
        const size_t n = samplers.size();
        const uint64_t B = (uint64_t)shape.blocks_per_cta;
        pl.det_off.assign(n, 0);
        pl.obs_off.assign(n, 0);
        pl.block0.assign(n, 0);
        pl.nblk.assign(n, 0);
        // A sampler listed more than once continues its stream from one entry to the next.
        std::unordered_map<const gfs_sampler *, uint64_t> next;
        for (size_t j = 0; j < n; j++) {
            auto it = next.find(samplers[j]);
            uint64_t b0 = it == next.end() ? samplers[j]->next_block : it->second;
            pl.block0[j] = b0;
            pl.nblk[j] = (shots[j] + 127) / 128;
            next[samplers[j]] = b0 + pl.nblk[j];
        }
        uint64_t total = 0;
        pl.prefix.push_back(0);
        for (uint32_t j : order) {
            const gfs_sampler *s = samplers[j];
            const uint64_t nslices = (pl.nblk[j] + B - 1) / B;
            if (nslices == 0) {
                continue;
            }
            pl.det_off[j] = pl.det_total;
            pl.obs_off[j] = pl.obs_total;
            pl.det_total += nslices * B * s->prog.num_detectors;
            pl.obs_total += nslices * B * s->prog.num_observables;
            gfs::KernelArgs a{};
            a.ops = (const gfs::DevOp *)s->d_ops.p;
            a.pool = (const uint32_t *)s->d_pool.p;
            a.tables = (const uint32_t *)s->d_tables.p;
            a.chans = (const gfs::DevChan *)s->d_chans.p;
            a.qubit_orig = (const uint32_t *)s->d_orig.p;
            a.nrows = s->prog.num_rows;
            a.ring = s->prog.ring;
            a.nobs = (uint32_t)s->prog.num_observables;
            a.nslices = (uint32_t)nslices;
            a.ndet = s->prog.num_detectors;
            a.nmeas = 0;
            a.seed = s->seed;
            a.block0 = pl.block0[j];
            a.status = (uint32_t *)d_status.p;
            a.smem_table_words = s->smem_table_words();
            a.smem_ops = s->smem_ops();
            a.ring_global = nullptr;
            a.ring_cta_stride = shape.ring_global ? ring_stride(shape.blocks_per_cta) : 0;
            pl.desc.push_back(a);
            total += nslices;
            if (total > 0xFFFFFFFFull) {
                throw std::invalid_argument("batch has too many 128-shot slices for one launch");
            }
            pl.prefix.push_back((uint32_t)total);
        }
        return pl;
    }

    // Fills the arena pointers of the descriptors and uploads them; returns the number of work items.
    uint32_t upload_plan(Plan &pl) {
        det_arena.ensure(std::max<uint64_t>(16, pl.det_total * 16), device);
        obs_arena.ensure(std::max<uint64_t>(16, pl.obs_total * 16), device);
        if (shape.ring_global) {
            ring_buf.ensure(std::max<uint64_t>(16, (uint64_t)shape.grid * ring_stride(shape.blocks_per_cta) * 16),
                            device);
        }
        size_t k = 0;
        for (uint32_t j : order) {
            if (pl.nblk[j] == 0) {
                continue;
            }
            gfs::KernelArgs &a = pl.desc[k++];
            a.det_out = (uint4 *)det_arena.p + pl.det_off[j];
            a.obs_out = (uint4 *)obs_arena.p + pl.obs_off[j];
            a.ring_global = shape.ring_global ? (uint4 *)ring_buf.p : nullptr;
        }
        if (!pl.desc.empty()) {
            d_desc.ensure(pl.desc.size() * sizeof(gfs::KernelArgs), device);
            d_prefix.ensure(pl.prefix.size() * sizeof(uint32_t), device);
            ck(cudaMemcpyAsync(d_desc.p, pl.desc.data(), pl.desc.size() * sizeof(gfs::KernelArgs),
                               cudaMemcpyHostToDevice, stream),
               "descriptor upload");
            ck(cudaMemcpyAsync(d_prefix.p, pl.prefix.data(), pl.prefix.size() * sizeof(uint32_t),
                               cudaMemcpyHostToDevice, stream),
               "descriptor upload");
        }
        return pl.prefix.back();
    }

    void enqueue_frame(const Plan &pl, uint32_t items) {
        ck(cudaMemsetAsync(d_counter.p, 0, 4, stream), "memset");
        gfs::BatchArgs b{};
        b.circuits = (const gfs::KernelArgs *)d_desc.p;
        b.slice_prefix = (const uint32_t *)d_prefix.p;
        b.ncircuits = (uint32_t)pl.desc.size();
        b.total_slices = items;
        b.counter = (uint32_t *)d_counter.p;
        gfs::LaunchShape s = shape;
        s.grid = (int)std::min<uint64_t>((uint64_t)shape.grid, items);
        ck(gfs::launch_batch_frame_kernel(b, s, stream), "batch frame kernel launch");
    }

    void enqueue_transposes(const Plan &pl, const uint64_t *shots, uint32_t flags, uint8_t *const *dets,
                            const uint64_t *dstride, uint8_t *const *obs, const uint64_t *ostride) {
        const bool packed = flags & GFS_BIT_PACKED;
        for (size_t j = 0; j < samplers.size(); j++) {
            if (pl.nblk[j] == 0) {
                continue;
            }
            const gfs_sampler *s = samplers[j];
            const uint64_t D = s->prog.num_detectors, O = s->prog.num_observables;
            const uint4 *dt = (const uint4 *)det_arena.p + pl.det_off[j];
            const uint4 *ot = (const uint4 *)obs_arena.p + pl.obs_off[j];
            auto tr = [&](const uint4 *s0, uint64_t n0, const uint4 *s1, uint64_t n1, const uint4 *s2, uint64_t n2,
                          uint8_t *out, uint64_t stride) {
                gfs::TransposeArgs t{};
                t.src0 = s0;
                t.n0 = n0;
                t.src1 = s1;
                t.n1 = n1;
                t.src2 = s2;
                t.n2 = n2;
                t.nshots = shots[j];
                t.out = out;
                t.out_stride = stride;
                t.bit_packed = packed ? 1 : 0;
                ck(gfs::launch_transpose(t, stream), "transpose launch");
            };
            if (dets && dets[j]) {
                if ((flags & GFS_PREPEND_OBSERVABLES) && (flags & GFS_APPEND_OBSERVABLES)) {
                    tr(ot, O, dt, D, ot, O, dets[j], dstride[j]);
                } else if (flags & GFS_PREPEND_OBSERVABLES) {
                    tr(ot, O, dt, D, nullptr, 0, dets[j], dstride[j]);
                } else if (flags & GFS_APPEND_OBSERVABLES) {
                    tr(dt, D, ot, O, nullptr, 0, dets[j], dstride[j]);
                } else {
                    tr(dt, D, nullptr, 0, nullptr, 0, dets[j], dstride[j]);
                }
            }
            if (obs && obs[j]) {
                tr(ot, O, nullptr, 0, nullptr, 0, obs[j], ostride[j]);
            }
        }
    }

    void row_bytes(size_t j, uint32_t flags, uint64_t *drow, uint64_t *orow) const {
        const bool packed = flags & GFS_BIT_PACKED;
        const uint64_t D = samplers[j]->prog.num_detectors, O = samplers[j]->prog.num_observables;
        const uint64_t nd =
            D + ((flags & GFS_PREPEND_OBSERVABLES) ? O : 0) + ((flags & GFS_APPEND_OBSERVABLES) ? O : 0);
        *drow = packed ? (nd + 7) / 8 : nd;
        *orow = packed ? (O + 7) / 8 : O;
    }

    void check_status() {
        uint32_t st = 0;
        ck(cudaMemcpy(&st, d_status.p, 4, cudaMemcpyDeviceToHost), "status read");
        if (st) {
            cudaMemset(d_status.p, 0, 4);
            throw std::runtime_error("batch frame kernel reported error status " + std::to_string(st));
        }
    }

    // Samples every circuit into device destinations (dets[j] / obs[j] may be null to skip them).
    void sample_device(const uint64_t *shots, uint32_t flags, uint8_t *const *dets, const uint64_t *dstride,
                       uint8_t *const *obs, const uint64_t *ostride) {
        const size_t n = samplers.size();
        for (size_t j = 0; j < n; j++) {
            uint64_t drow, orow;
            row_bytes(j, flags, &drow, &orow);
            if (dets && dets[j] && dstride[j] < drow) {
                throw std::invalid_argument("dets row stride too small for circuit " + std::to_string(j));
            }
            if (obs && obs[j] && ostride[j] < orow) {
                throw std::invalid_argument("obs row stride too small for circuit " + std::to_string(j));
            }
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        t_frame = t_transpose = t_copy = t_total = 0;
        Plan pl = plan(shots);
        const uint32_t items = upload_plan(pl);
        if (items == 0) {
            return;
        }
        // The graph holds the counter reset, the batched frame kernel and the transposes; the descriptors
        // it reads (seeds, stream offsets) are uploaded before each replay.
        std::vector<uint64_t> key = {(uint64_t)shape.blocks_per_cta, (uint64_t)shape.threads, (uint64_t)shape.grid,
                                     shape.smem, (uint64_t)shape.ring_global, flags, items,
                                     (uint64_t)(uintptr_t)det_arena.p, (uint64_t)(uintptr_t)obs_arena.p,
                                     (uint64_t)(uintptr_t)d_desc.p, (uint64_t)(uintptr_t)d_prefix.p,
                                     (uint64_t)(uintptr_t)ring_buf.p};
        for (size_t j = 0; j < n; j++) {
            key.push_back(shots[j]);
            key.push_back(dets ? (uint64_t)(uintptr_t)dets[j] : 0);
            key.push_back(dets && dets[j] ? dstride[j] : 0);
            key.push_back(obs ? (uint64_t)(uintptr_t)obs[j] : 0);
            key.push_back(obs && obs[j] ? ostride[j] : 0);
        }
        if (!exec || key != graph_key) {
            drop_graph();
            cudaGraph_t graph = nullptr;
            ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "graph capture");
            try {
                enqueue_frame(pl, items);
                ck(cudaEventRecord(ev[1], stream), "event");
                enqueue_transposes(pl, shots, flags, dets, dstride, obs, ostride);
            } catch (...) {
                cudaStreamEndCapture(stream, &graph);
                if (graph) {
                    cudaGraphDestroy(graph);
                }
                throw;
            }
            ck(cudaStreamEndCapture(stream, &graph), "graph capture");
            cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            ck(e, "graph instantiate");
            graph_key = key;
            n_graph_builds++;
        }
        ck(cudaEventRecord(ev[0], stream), "event");
        ck(cudaGraphLaunch(exec, stream), "graph launch");
        ck(cudaEventRecord(ev[2], stream), "event");
        ck(cudaStreamSynchronize(stream), "batch sample");
        n_graph_launches++;
        n_frame++;
        for (size_t j = 0; j < n; j++) {
            if (pl.nblk[j]) {
                n_transpose += (dets && dets[j] ? 1 : 0) + (obs && obs[j] ? 1 : 0);
            }
        }
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, ev[0], ev[2]), "cudaEventElapsedTime");
        t_total = ms;
        if (cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess) {
            t_frame = ms;
            t_transpose = std::max(0.0, t_total - t_frame);
        } else {
            cudaGetLastError();
            t_frame = t_total;
        }
        check_status();
        for (size_t j = 0; j < n; j++) {
            samplers[j]->next_block = std::max(samplers[j]->next_block, pl.block0[j] + pl.nblk[j]);
        }
    }

    // Host destinations: sample into a device staging arena (rows padded to 32 bytes), then copy.
    void sample_host(const uint64_t *shots, uint32_t flags, uint8_t *const *dets, const uint64_t *dstride,
                     uint8_t *const *obs, const uint64_t *ostride) {
        const size_t n = samplers.size();
        std::vector<uint64_t> dr(n), orw(n), ds(n), os(n), off(n);
        uint64_t bytes = 0;
        for (size_t j = 0; j < n; j++) {
            row_bytes(j, flags, &dr[j], &orw[j]);
            if (dets && dets[j] && dstride[j] < dr[j]) {
                throw std::invalid_argument("dets row stride too small for circuit " + std::to_string(j));
            }
            if (obs && obs[j] && ostride[j] < orw[j]) {
                throw std::invalid_argument("obs row stride too small for circuit " + std::to_string(j));
            }
            ds[j] = pad32(dr[j]);
            os[j] = pad32(orw[j]);
            off[j] = bytes;
            bytes += shots[j] * (ds[j] + os[j]);
        }
        ck(cudaSetDevice(device), "cudaSetDevice");
        out_arena.ensure(std::max<uint64_t>(16, bytes), device);
        std::vector<uint8_t *> dd(n, nullptr), od(n, nullptr);
        for (size_t j = 0; j < n; j++) {
            uint8_t *base = (uint8_t *)out_arena.p + off[j];
            dd[j] = dets && dets[j] ? base : nullptr;
            od[j] = obs && obs[j] ? base + shots[j] * ds[j] : nullptr;
        }
        sample_device(shots, flags, dd.data(), ds.data(), od.data(), os.data());
        ck(cudaEventRecord(ev[0], stream), "event");
        for (size_t j = 0; j < n; j++) {
            if (shots[j] == 0) {
                continue;
            }
            if (dd[j] && dr[j]) {
                ck(cudaMemcpy2DAsync(dets[j], dstride[j], dd[j], ds[j], dr[j], shots[j], cudaMemcpyDeviceToHost,
                                     stream),
                   "copy dets");
            }
            if (od[j] && orw[j]) {
                ck(cudaMemcpy2DAsync(obs[j], ostride[j], od[j], os[j], orw[j], shots[j], cudaMemcpyDeviceToHost,
                                     stream),
                   "copy obs");
            }
        }
        ck(cudaEventRecord(ev[2], stream), "event");
        ck(cudaStreamSynchronize(stream), "batch copy");
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, ev[0], ev[2]), "cudaEventElapsedTime");
        t_copy = ms;
        t_total += ms;
    }

    // Times the batched frame kernel for each candidate launch shape on these shot counts and keeps the
    // fastest.  Samplers do not advance; results never depend on the shape.
    double autotune(const uint64_t *shots) {
        ck(cudaSetDevice(device), "cudaSetDevice");
        struct Cand {
            int bpc, threads, ring;
        };
        const Cand cands[] = {{1, 256, 0}, {1, 256, 1}, {1, 128, 0}, {1, 128, 1}, {2, 256, 0},
                              {2, 256, 1}, {2, 128, 0}, {2, 128, 1}, {4, 256, 0}, {4, 256, 1}};
        double best = -1;
        gfs::LaunchShape best_shape = shape;
        for (const Cand &c : cands) {
            gfs::LaunchShape t{};
            if (resident(c.bpc, c.threads, c.ring == 1, &t) == 0) {
                continue;
            }
            shape = t;
            Plan pl = plan(shots);
            const uint32_t items = upload_plan(pl);
            if (items == 0) {
                break;
            }
            float ms = 0, total = 0;
            for (int rep = 0; rep < 2; rep++) {
                ck(cudaEventRecord(ev[0], stream), "event");
                enqueue_frame(pl, items);
                ck(cudaEventRecord(ev[2], stream), "event");
                ck(cudaStreamSynchronize(stream), "autotune");
                ck(cudaEventElapsedTime(&ms, ev[0], ev[2]), "cudaEventElapsedTime");
                if (rep) {
                    total = ms;
                }
            }
            check_status();
            if (best < 0 || total < best) {
                best = total;
                best_shape = shape;
            }
        }
        shape = best_shape;
        drop_graph();
        return best;
    }
};

extern "C" {

gfs_status gfs_batch_create(gfs_sampler *const *samplers, size_t n, gfs_batch **out) {
    *out = nullptr;
    return guarded([&] {
        auto b = std::make_unique<gfs_batch>();
        b->init(samplers, n);
        *out = b.release();
    });
}

void gfs_batch_free(gfs_batch *b) {
    delete b;
}

gfs_status gfs_batch_sample_detections_device(gfs_batch *b, const uint64_t *shots, uint32_t flags, void *const *dets,
                                              const uint64_t *dets_stride, void *const *obs,
                                              const uint64_t *obs_stride) {
    return guarded([&] {
        b->sample_device(shots, flags, (uint8_t *const *)dets, dets_stride, (uint8_t *const *)obs, obs_stride);
    });
}

gfs_status gfs_batch_sample_detections(gfs_batch *b, const uint64_t *shots, uint32_t flags, uint8_t *const *dets,
                                       const uint64_t *dets_stride, uint8_t *const *obs, const uint64_t *obs_stride) {
    return guarded([&] { b->sample_host(shots, flags, dets, dets_stride, obs, obs_stride); });
}

gfs_status gfs_batch_set_shape(gfs_batch *b, int blocks_per_cta, int threads, int ring_placement) {
    return guarded([&] {
        if (ring_placement < -1 || ring_placement > 1) {
            throw std::invalid_argument("ring placement must be -1 (automatic), 0 (shared memory) or 1 (global memory)");
        }
        ck(cudaSetDevice(b->device), "cudaSetDevice");
        b->set_shape(blocks_per_cta, threads, ring_placement);
    });
}

gfs_status gfs_batch_get_shape(const gfs_batch *b, int *blocks_per_cta, int *threads, int *grid, uint64_t *smem_bytes,
                               int *ring_global) {
    return guarded([&] {
        *blocks_per_cta = b->shape.blocks_per_cta;
        *threads = b->shape.threads;
        *grid = b->shape.grid;
        *smem_bytes = b->shape.smem;
        *ring_global = b->shape.ring_global ? 1 : 0;
    });
}

gfs_status gfs_batch_autotune(gfs_batch *b, const uint64_t *shots, double *best_ms) {
    return guarded([&] {
        double ms = b->autotune(shots);
        if (best_ms) {
            *best_ms = ms;
        }
    });
}

gfs_status gfs_batch_last_timings(const gfs_batch *b, double *out4, uint64_t *counts4) {
    return guarded([&] {
        out4[0] = b->t_frame;
        out4[1] = b->t_transpose;
        out4[2] = b->t_copy;
        out4[3] = b->t_total;
        if (counts4) {
            counts4[0] = b->n_frame;
            counts4[1] = b->n_transpose;
            counts4[2] = b->n_graph_launches;
            counts4[3] = b->n_graph_builds;
        }
    });
}

}  // extern "C"
