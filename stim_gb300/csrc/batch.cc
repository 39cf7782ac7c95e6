// Batched sampling: the shots of many circuits in one persistent frame-kernel launch (batch_frame_kernel),
// followed by each circuit's shot-major transpose, captured once as a CUDA graph and replayed while the
// request geometry (shot counts, destinations, launch shape) stays the same.
//
// Each circuit keeps the random stream of its own sampler: circuit j's shots are the next shots of
// samplers[j] (block0 = its shot counter), so a batch returns bit for bit what the samplers' own
// sample calls would have returned, in the same order.  The reference has no batched mode; its nearest
// equivalent is one CompiledDetectorSampler per circuit (compiled_detector_sampler.pybind.cc:216-322).
#include <unordered_map>

#include "batch_engine.h"

struct gfs_batch {
    std::vector<gfs_sampler *> samplers;
    std::vector<const gfs_sampler *> progs;
    std::vector<uint32_t> order;  // circuits by estimated cost per 128-shot block, most expensive first
    gfs_rt::BatchEngine eng;
    gfs_rt::DevBuf out_arena;
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> graph_key;
    double t_frame = 0, t_transpose = 0, t_copy = 0, t_total = 0;
    uint64_t n_frame = 0, n_transpose = 0, n_graph_launches = 0, n_graph_builds = 0, n_hit_overflows = 0;

    ~gfs_batch() {
        drop_graph();
    }

    void init(gfs_sampler *const *s, size_t n) {
        if (n == 0) {
            throw std::invalid_argument("a batch needs at least one sampler");
        }
        samplers.assign(s, s + n);
        for (auto *x : samplers) {
            if (!x) {
                throw std::invalid_argument("null sampler in batch");
            }
            if (x->mode != GFS_MODE_DETECTIONS) {
                throw std::invalid_argument("batched sampling needs samplers created in detection mode");
            }
            if (x->device != samplers[0]->device) {
                throw std::invalid_argument("all samplers of a batch must be on the same device");
            }
            progs.push_back(x);
        }
        order.resize(n);
        for (size_t j = 0; j < n; j++) {
            order[j] = (uint32_t)j;
        }
        std::stable_sort(order.begin(), order.end(),
                         [&](uint32_t a, uint32_t b) { return samplers[a]->prog.work > samplers[b]->prog.work; });
        eng.init(samplers[0]->device);
        eng.default_shape(progs);
    }

    void set_shape(int bpc, int threads, int ring) {
        if (bpc != 1 && bpc != 2 && bpc != 4) {
            throw std::invalid_argument("blocks_per_cta must be 1, 2 or 4");
        }
        if (threads <= 0 || threads > 256 || threads % 32) {
            throw std::invalid_argument("threads per CTA must be a multiple of 32 in [32, 256]");
        }
        eng.set_shape(progs, bpc, threads, ring);
        drop_graph();
    }

    void drop_graph() {
        if (exec) {
            cudaSetDevice(eng.device);
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        graph_key.clear();
    }

    // Entries for these shot counts: circuit j continues samplers[j]'s stream (a sampler listed more than
    // once continues from one entry to the next).
    std::vector<gfs_rt::BatchEntry> entries(const uint64_t *shots, uint8_t *const *dets, const uint64_t *dstride,
                                            uint8_t *const *obs, const uint64_t *ostride) const {
        std::vector<gfs_rt::BatchEntry> es(samplers.size());
        std::unordered_map<const gfs_sampler *, uint64_t> next;
        for (size_t j = 0; j < samplers.size(); j++) {
            auto it = next.find(samplers[j]);
            const uint64_t b0 = it == next.end() ? samplers[j]->next_block : it->second;
            gfs_rt::BatchEntry &e = es[j];
            e.prog = samplers[j];
            e.seed = samplers[j]->seed;
            e.block0 = b0;
            e.shots = shots[j];
            e.dets = dets ? dets[j] : nullptr;
            e.dstride = dets && dets[j] ? dstride[j] : 0;
            e.obs = obs ? obs[j] : nullptr;
            e.ostride = obs && obs[j] ? ostride[j] : 0;
            next[samplers[j]] = b0 + (shots[j] + 127) / 128;
        }
        return es;
    }

    // Samples every circuit into device destinations (dets[j] / obs[j] may be null to skip them).
    void sample_device(const uint64_t *shots, uint32_t flags, uint8_t *const *dets, const uint64_t *dstride,
                       uint8_t *const *obs, const uint64_t *ostride) {
        const size_t n = samplers.size();
        for (size_t j = 0; j < n; j++) {
            uint64_t drow, orow;
            gfs_rt::layout_rows(samplers[j], flags, &drow, &orow);
            if (dets && dets[j] && dstride[j] < drow) {
                throw std::invalid_argument("dets row stride too small for circuit " + std::to_string(j));
            }
            if (obs && obs[j] && ostride[j] < orow) {
                throw std::invalid_argument("obs row stride too small for circuit " + std::to_string(j));
            }
        }
        ck(cudaSetDevice(eng.device), "cudaSetDevice");
        t_frame = t_transpose = t_copy = t_total = 0;
        const std::vector<gfs_rt::BatchEntry> es = entries(shots, dets, dstride, obs, ostride);
        const uint32_t items = eng.prepare(es, order);
        if (items == 0) {
            return;
        }
        // The graph holds the counter reset, the batched frame kernel and the transposes; the descriptors
        // it reads (seeds, stream offsets) are uploaded before each replay.
        const gfs::LaunchShape &sh = eng.shape;
        std::vector<uint64_t> key = {(uint64_t)sh.blocks_per_cta, (uint64_t)sh.threads, (uint64_t)sh.grid, sh.smem,
                                     (uint64_t)sh.ring_global, flags, items, (uint64_t)(uintptr_t)eng.det_arena.p,
                                     (uint64_t)(uintptr_t)eng.obs_arena.p, (uint64_t)(uintptr_t)eng.d_desc.p,
                                     (uint64_t)(uintptr_t)eng.d_prefix.p, (uint64_t)(uintptr_t)eng.ring_buf.p,
                                     (uint64_t)eng.lean, (uint64_t)eng.lean_shape.grid, eng.lean_shape.smem};
        for (const auto &e : es) {
            key.push_back(e.shots);
            key.push_back((uint64_t)(uintptr_t)e.dets);
            key.push_back(e.dstride);
            key.push_back((uint64_t)(uintptr_t)e.obs);
            key.push_back(e.ostride);
        }
        uint64_t calls = 0;
        if (!exec || key != graph_key) {
            drop_graph();
            cudaGraph_t graph = nullptr;
            ck(cudaStreamBeginCapture(eng.stream, cudaStreamCaptureModeThreadLocal), "graph capture");
            try {
                eng.enqueue_frame();
                // An external event-record node: it records ev[1] on every replay, splitting the frame kernel
                // from the transposes (a plain record made during capture would not be a timing point).
                ck(cudaEventRecordWithFlags(eng.ev[1], eng.stream, cudaEventRecordExternal), "event");
                calls = eng.enqueue_transposes(es, flags);
            } catch (...) {
                cudaStreamEndCapture(eng.stream, &graph);
                if (graph) {
                    cudaGraphDestroy(graph);
                }
                throw;
            }
            ck(cudaStreamEndCapture(eng.stream, &graph), "graph capture");
            cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            ck(e, "graph instantiate");
            graph_key = key;
            n_graph_builds++;
        } else {
            for (const auto &e : es) {
                calls += e.shots ? (e.dets ? 1 : 0) + (e.obs ? 1 : 0) : 0;
            }
        }
        ck(cudaEventRecord(eng.ev[0], eng.stream), "event");
        ck(cudaGraphLaunch(exec, eng.stream), "graph launch");
        ck(cudaEventRecord(eng.ev[2], eng.stream), "event");
        ck(cudaStreamSynchronize(eng.stream), "batch sample");
        n_graph_launches++;
        n_frame++;
        n_transpose += calls;
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, eng.ev[0], eng.ev[2]), "cudaEventElapsedTime");
        t_total = ms;
        if (cudaEventElapsedTime(&ms, eng.ev[0], eng.ev[1]) == cudaSuccess && ms > 0 && ms <= t_total) {
            t_frame = ms;
            t_transpose = t_total - t_frame;
        } else {
            cudaGetLastError();
            t_frame = t_total;
        }
        if (eng.check_status()) {
            // A hit list overflowed: redo the batch with inline noise (identical results), outside the graph.
            n_hit_overflows++;
            eng.force_inline = true;
            try {
                eng.prepare(es, order);
                eng.enqueue_frame();
                eng.enqueue_transposes(es, flags);
                ck(cudaStreamSynchronize(eng.stream), "batch sample");
                eng.check_status();
            } catch (...) {
                eng.force_inline = false;
                drop_graph();
                throw;
            }
            eng.force_inline = false;
            drop_graph();  // its descriptors were overwritten
        }
        for (const auto &e : es) {
            gfs_sampler *s = const_cast<gfs_sampler *>(e.prog);
            s->next_block = std::max(s->next_block, e.block0 + (e.shots + 127) / 128);
        }
    }

    // Host destinations: sample into a device staging arena (rows padded to 32 bytes), then copy.
    void sample_host(const uint64_t *shots, uint32_t flags, uint8_t *const *dets, const uint64_t *dstride,
                     uint8_t *const *obs, const uint64_t *ostride) {
        const size_t n = samplers.size();
        std::vector<uint64_t> dr(n), orw(n), ds(n), os(n), off(n);
        uint64_t bytes = 0;
        for (size_t j = 0; j < n; j++) {
            gfs_rt::layout_rows(samplers[j], flags, &dr[j], &orw[j]);
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
        ck(cudaSetDevice(eng.device), "cudaSetDevice");
        out_arena.ensure(std::max<uint64_t>(16, bytes), eng.device);
        std::vector<uint8_t *> dd(n, nullptr), od(n, nullptr);
        for (size_t j = 0; j < n; j++) {
            uint8_t *base = (uint8_t *)out_arena.p + off[j];
            dd[j] = dets && dets[j] ? base : nullptr;
            od[j] = obs && obs[j] ? base + shots[j] * ds[j] : nullptr;
        }
        sample_device(shots, flags, dd.data(), ds.data(), od.data(), os.data());
        const double kernels = t_total;
        ck(cudaEventRecord(eng.ev[0], eng.stream), "event");
        for (size_t j = 0; j < n; j++) {
            if (shots[j] == 0) {
                continue;
            }
            if (dd[j] && dr[j]) {
                ck(cudaMemcpy2DAsync(dets[j], dstride[j], dd[j], ds[j], dr[j], shots[j], cudaMemcpyDeviceToHost,
                                     eng.stream),
                   "copy dets");
            }
            if (od[j] && orw[j]) {
                ck(cudaMemcpy2DAsync(obs[j], ostride[j], od[j], os[j], orw[j], shots[j], cudaMemcpyDeviceToHost,
                                     eng.stream),
                   "copy obs");
            }
        }
        ck(cudaEventRecord(eng.ev[2], eng.stream), "event");
        ck(cudaStreamSynchronize(eng.stream), "batch copy");
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, eng.ev[0], eng.ev[2]), "cudaEventElapsedTime");
        t_copy = ms;
        t_total = kernels + ms;
    }

    // Times the batched frame kernel for each candidate launch shape on these shot counts and keeps the
    // fastest.  Samplers do not advance; results never depend on the shape.
    double autotune(const uint64_t *shots) {
        ck(cudaSetDevice(eng.device), "cudaSetDevice");
        struct Cand {
            int bpc, threads, ring;
        };
        const Cand cands[] = {{1, 256, 0}, {1, 256, 1}, {1, 128, 0}, {1, 128, 1}, {2, 256, 0},
                              {2, 256, 1}, {2, 128, 0}, {2, 128, 1}, {4, 256, 0}, {4, 256, 1}};
        const std::vector<gfs_rt::BatchEntry> es = entries(shots, nullptr, nullptr, nullptr, nullptr);
        double best = -1;
        gfs::LaunchShape best_shape = eng.shape;
        uint64_t best_stride = eng.ring_stride_cur;
        for (const Cand &c : cands) {
            try {
                eng.set_shape(progs, c.bpc, c.threads, c.ring);
            } catch (const std::invalid_argument &) {
                continue;
            }
            if ((c.ring == 1) != eng.shape.ring_global) {
                continue;
            }
            const uint32_t items = eng.prepare(es, order);
            if (items == 0) {
                break;
            }
            float ms = 0;
            for (int rep = 0; rep < 2; rep++) {
                ck(cudaEventRecord(eng.ev[0], eng.stream), "event");
                eng.enqueue_frame();
                ck(cudaEventRecord(eng.ev[2], eng.stream), "event");
                ck(cudaStreamSynchronize(eng.stream), "autotune");
                ck(cudaEventElapsedTime(&ms, eng.ev[0], eng.ev[2]), "cudaEventElapsedTime");
            }
            eng.check_status();
            if (best < 0 || ms < best) {
                best = ms;
                best_shape = eng.shape;
                best_stride = eng.ring_stride_cur;
            }
        }
        eng.shape = best_shape;
        eng.ring_stride_cur = best_stride;
        eng.set_lean_shape(progs);
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
        ck(cudaSetDevice(b->eng.device), "cudaSetDevice");
        b->set_shape(blocks_per_cta, threads, ring_placement);
    });
}

gfs_status gfs_batch_get_shape(const gfs_batch *b, int *blocks_per_cta, int *threads, int *grid, uint64_t *smem_bytes,
                               int *ring_global) {
    return guarded([&] {
        const gfs::LaunchShape &sh = b->eng.lean ? b->eng.lean_shape : b->eng.shape;
        *blocks_per_cta = sh.blocks_per_cta;
        *threads = sh.threads;
        *grid = sh.grid;
        *smem_bytes = sh.smem;
        *ring_global = sh.ring_global ? 1 : 0;
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
