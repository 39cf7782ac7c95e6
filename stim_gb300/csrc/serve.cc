// Request server: continuous batching of detection-sampling requests on one device.
//
// Clients submit (circuit text, shots, seed, destinations) from any thread.  One worker thread owns the
// device: it keeps lowered circuits in a device-resident cache keyed by circuit text, cuts requests into
// chunks of at most `max_chunk_shots` shots, and admits chunks first come first served into the next
// batch while the batch's HBM footprint (detector-major scratch plus shot-major staging) stays within
// its slot budget.  Two slots alternate: while one batch runs (one persistent batch_frame_kernel
// launch, transposes, device->host copies, all on the slot's stream), the worker forms and launches the
// next one, so requests that arrive while others are on the GPU join as soon as a slot and its memory
// free up, and the two batches overlap on the device.  A request's result depends only on (circuit,
// seed, shot index) -- chunk k of a request samples the request's stream from shot k*max_chunk_shots --
// so it is identical bit for bit whether it ran alone or mixed with others.
//
// The reference has no server; each request corresponds to
// stim.Circuit(text).compile_detector_sampler(seed=seed).sample(shots, ...)
// (src/stim/py/compiled_detector_sampler.pybind.cc:216-322).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "batch_engine.h"

namespace {

using Clock = std::chrono::steady_clock;

struct CachedProgram {
    std::string text;
    std::unique_ptr<gfs_sampler> s;  // owns the lowered program on the device
};

struct Request {
    uint64_t id = 0;
    std::shared_ptr<CachedProgram> prog;
    uint64_t seed = 0, shots = 0;
    uint32_t flags = 0;
    bool device_out = false;
    uint8_t *dets = nullptr, *obs = nullptr;
    uint64_t dstride = 0, ostride = 0;
    uint64_t drow = 0, orow = 0;   // bytes per shot of each output
    uint64_t issued = 0, done = 0;  // shots handed to batches / finished
    Clock::time_point t_submit, t_done;
    bool finished = false;
    bool failed = false;
    std::string error;
};

struct Chunk {
    std::shared_ptr<Request> req;
    uint64_t first = 0, shots = 0;  // shot offset within the request (a multiple of 128)
};

// A batch is split by launch-shape class: circuits whose own sampler takes several 128-shot blocks per CTA
// (small and medium circuits: wide CTAs, many items per phase) and circuits that take one block per CTA (the
// largest: shared memory allows few blocks per SM).  Each class runs as its own persistent launch on its own
// engine and stream, so a batch's shape no longer follows its largest circuit (one shared shape ran a mixed
// 160-request batch at 513 Gbit/s, the two classes back to back at 765).
constexpr int kClasses = 2;

struct Slot {
    gfs_rt::BatchEngine eng[kClasses];
    gfs_rt::DevBuf staging;  // shot-major rows for host destinations
    std::vector<Chunk> chunks;
    std::vector<size_t> members[kClasses];  // indices into chunks, per class
    std::vector<uint64_t> soff;             // staging offset of each chunk (host destinations)
    bool busy = false;
    uint64_t bits = 0;
};

}  // namespace

struct gfs_server {
    int device = 0;
    uint64_t slot_budget = 0;
    uint64_t max_chunk = 0;
    size_t max_entries = 1024;
    size_t cache_capacity = 4096;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;  // requests with shots not yet issued
    std::unordered_map<uint64_t, std::shared_ptr<Request>> live;
    std::unordered_map<std::string, std::shared_ptr<CachedProgram>> cache;
    std::list<std::string> lru;
    uint64_t next_id = 1;
    bool stop = false;

    // Statistics (under mu).
    std::vector<double> latencies_ms;
    uint64_t completed = 0, failed_count = 0, batches = 0, entries_total = 0, cache_hits = 0, cache_misses = 0;
    uint64_t bits_done = 0, max_queue = 0;
    // Admission counters: requests accepted into the queue, rejected at submission (invalid circuit or
    // arguments, circuit too large for the server), chunks admitted into batches.
    uint64_t submitted = 0, rejected = 0, chunks_admitted = 0;
    Clock::time_point t_first_submit{}, t_last_done{};
    bool any_submit = false;

    Slot slots[2];
    std::thread worker;

    ~gfs_server() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv_work.notify_all();
        if (worker.joinable()) {
            worker.join();
        }
    }

    void init(int dev, uint64_t hbm_budget, uint64_t chunk_shots) {
        device = dev;
        slot_budget = std::max<uint64_t>(hbm_budget / 2, (uint64_t)64 << 20);
        max_chunk = std::max<uint64_t>(128, (chunk_shots ? chunk_shots : (uint64_t)1 << 18) & ~(uint64_t)127);
        for (auto &s : slots) {
            for (auto &e : s.eng) {
                e.init(device);
            }
        }
        worker = std::thread([this] { run(); });
    }

    // Called with mu held.  A miss is lowered and uploaded by submit() on the caller's thread.
    std::shared_ptr<CachedProgram> lookup(const std::string &text) {
        auto it = cache.find(text);
        if (it != cache.end()) {
            cache_hits++;
            lru.remove(text);
            lru.push_front(text);
            return it->second;
        }
        cache_misses++;
        return nullptr;
    }

    uint64_t submit(const char *text, size_t len, uint64_t shots, uint64_t seed, uint32_t flags, bool device_out,
                    uint8_t *dets, uint64_t dstride, uint8_t *obs, uint64_t ostride) {
        try {
            return submit_checked(text, len, shots, seed, flags, device_out, dets, dstride, obs, ostride);
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            rejected++;
            throw;
        }
    }

    uint64_t submit_checked(const char *text, size_t len, uint64_t shots, uint64_t seed, uint32_t flags,
                            bool device_out, uint8_t *dets, uint64_t dstride, uint8_t *obs, uint64_t ostride) {
        const Clock::time_point t0 = Clock::now();  // latency includes lowering on a cache miss
        std::string key(text, len);
        std::shared_ptr<CachedProgram> prog;
        {
            std::lock_guard<std::mutex> lk(mu);
            prog = lookup(key);
        }
        if (!prog) {
            // Parse, lower and upload outside the lock (a sampler object owns the device copy).
            gfs::Circuit c = gfs::Circuit::parse(key);
            gfs_circuit gc;
            gc.circuit = std::move(c);
            gc.stats = gc.circuit.stats();
            auto p = std::make_shared<CachedProgram>();
            p->text = key;
            p->s = std::make_unique<gfs_sampler>();
            p->s->init(&gc, GFS_MODE_DETECTIONS, 0, device);
            if (p->s->shape.frames_global) {
                // Rejected here, alone, rather than failing the batch it would join.
                throw std::invalid_argument("circuit too large for the server: its frames do not fit in shared "
                                            "memory (sample it with a CompiledDetectorSampler instead)");
            }
            std::lock_guard<std::mutex> lk(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                prog = it->second;
            } else {
                cache[key] = p;
                lru.push_front(key);
                prog = p;
                while (cache.size() > cache_capacity && !lru.empty()) {
                    cache.erase(lru.back());  // requests in flight keep their program alive
                    lru.pop_back();
                }
            }
        }
        auto r = std::make_shared<Request>();
        r->prog = prog;
        r->seed = seed;
        r->shots = shots;
        r->flags = flags;
        r->device_out = device_out;
        r->dets = dets;
        r->obs = obs;
        r->dstride = dstride;
        r->ostride = ostride;
        gfs_rt::layout_rows(prog->s.get(), flags, &r->drow, &r->orow);
        if (dets && dstride < r->drow) {
            throw std::invalid_argument("dets row stride too small");
        }
        if (obs && ostride < r->orow) {
            throw std::invalid_argument("obs row stride too small");
        }
        r->t_submit = t0;
        uint64_t id;
        {
            std::lock_guard<std::mutex> lk(mu);
            id = r->id = next_id++;
            submitted++;
            if (!any_submit) {
                t_first_submit = r->t_submit;
                any_submit = true;
            }
            live[id] = r;
            if (shots == 0) {
                finish_locked(*r);
            } else {
                queue.push_back(r);
                max_queue = std::max<uint64_t>(max_queue, queue.size());
            }
        }
        cv_work.notify_one();
        return id;
    }

    void finish_locked(Request &r) {
        r.finished = true;
        r.t_done = Clock::now();
        t_last_done = r.t_done;
        if (r.failed) {
            failed_count++;
        } else {
            completed++;
            latencies_ms.push_back(std::chrono::duration<double, std::milli>(r.t_done - r.t_submit).count());
            const gfs_sampler *s = r.prog->s.get();
            bits_done += r.shots * (s->prog.num_detectors + s->prog.num_observables);
        }
        cv_done.notify_all();
    }

    // Bytes of device memory a chunk needs in a slot.
    static uint64_t footprint(const Request &r, uint64_t shots, int bpc) {
        const gfs_sampler *s = r.prog->s.get();
        const uint64_t blocks = ((shots + 127) / 128 + bpc - 1) / bpc * bpc;
        uint64_t f = blocks * (s->prog.num_detectors + s->prog.num_observables) * 16;
        if (!r.device_out) {
            f += shots * (pad32(r.drow) * (r.dets ? 1 : 0) + pad32(r.orow) * (r.obs ? 1 : 0));
        }
        return f;
    }

    // Fills `slot` with chunks (called with mu held): passes over the queue in arrival order, taking at most
    // one chunk per request per pass, until the slot's memory budget or entry limit is reached.  A long
    // request therefore shares each batch with requests that arrived after it instead of blocking them.
    // Returns false when nothing was taken.
    bool form_locked(Slot &slot) {
        slot.chunks.clear();
        uint64_t used = 0;
        bool progress = true;
        while (progress && slot.chunks.size() < max_entries && !queue.empty()) {
            progress = false;
            for (auto it = queue.begin(); it != queue.end() && slot.chunks.size() < max_entries;) {
                std::shared_ptr<Request> r = *it;
                uint64_t take = std::min<uint64_t>(r->shots - r->issued, max_chunk);
                while (take > 128 && used + footprint(*r, take, 4) > slot_budget) {
                    take = std::max<uint64_t>(128, ((take / 2) + 127) & ~(uint64_t)127);
                }
                if (used + footprint(*r, take, 4) > slot_budget) {
                    if (slot.chunks.empty() && used == 0) {
                        r->failed = true;
                        r->error = "request needs more device memory per 128 shots than the server's slot budget";
                        r->done += r->shots - r->issued;
                        r->issued = r->shots;
                        it = queue.erase(it);
                        if (r->done >= r->shots && !r->finished) {
                            finish_locked(*r);
                        }
                        continue;
                    }
                    ++it;
                    continue;
                }
                slot.chunks.push_back(Chunk{r, r->issued, take});
                chunks_admitted++;
                used += footprint(*r, take, 4);
                r->issued += take;
                progress = true;
                if (r->issued >= r->shots) {
                    it = queue.erase(it);
                } else {
                    ++it;
                }
            }
        }
        return !slot.chunks.empty();
    }

    static int shape_class(const Request &r) {
        return r.prog->s->shape.blocks_per_cta > 1 ? 0 : 1;
    }

    void launch(Slot &slot) {
        ck(cudaSetDevice(device), "cudaSetDevice");
        for (int g = 0; g < kClasses; g++) {
            slot.members[g].clear();
        }
        uint64_t staging = 0;
        std::vector<uint64_t> soff(slot.chunks.size(), 0);
        slot.bits = 0;
        for (size_t k = 0; k < slot.chunks.size(); k++) {
            const Chunk &c = slot.chunks[k];
            const Request &r = *c.req;
            slot.members[shape_class(r)].push_back(k);
            if (!r.device_out) {
                soff[k] = staging;
                staging += c.shots * (pad32(r.drow) * (r.dets ? 1 : 0) + pad32(r.orow) * (r.obs ? 1 : 0));
            }
            slot.bits += c.shots * (r.prog->s->prog.num_detectors + r.prog->s->prog.num_observables);
        }
        slot.staging.ensure(std::max<uint64_t>(16, staging), device);
        slot.soff = std::move(soff);
        for (int g = 0; g < kClasses; g++) {
            if (!slot.members[g].empty()) {
                launch_class(slot, g);
            }
        }
    }

    // One class of the slot's chunks as one persistent launch on the class's engine and stream.
    void launch_class(Slot &slot, int g) {
        gfs_rt::BatchEngine &eng = slot.eng[g];
        const std::vector<size_t> &mem = slot.members[g];
        std::vector<const gfs_sampler *> progs;
        std::vector<gfs_rt::BatchEntry> es(mem.size());
        for (size_t i = 0; i < mem.size(); i++) {
            const Chunk &c = slot.chunks[mem[i]];
            const Request &r = *c.req;
            progs.push_back(r.prog->s.get());
            gfs_rt::BatchEntry &e = es[i];
            e.prog = r.prog->s.get();
            e.seed = r.seed;
            e.block0 = c.first / 128;
            e.shots = c.shots;
            if (r.device_out) {
                e.dets = r.dets ? r.dets + c.first * r.dstride : nullptr;
                e.dstride = r.dstride;
                e.obs = r.obs ? r.obs + c.first * r.ostride : nullptr;
                e.ostride = r.ostride;
            } else {
                uint8_t *base = (uint8_t *)slot.staging.p + slot.soff[mem[i]];
                e.dets = r.dets ? base : nullptr;
                e.dstride = pad32(r.drow);
                e.obs = r.obs ? base + (r.dets ? c.shots * pad32(r.drow) : 0) : nullptr;
                e.ostride = pad32(r.orow);
            }
        }
        eng.default_shape(progs);
        if (eng.prepare(es, {}) == 0) {
            ck(cudaEventRecord(eng.ev[2], eng.stream), "event");
            return;
        }
        eng.enqueue_frame();
        enqueue_transposes(slot, g, es);
        for (size_t i = 0; i < mem.size(); i++) {
            const Chunk &c = slot.chunks[mem[i]];
            const Request &r = *c.req;
            if (r.device_out) {
                continue;
            }
            if (r.dets && r.drow) {
                ck(cudaMemcpy2DAsync(r.dets + c.first * r.dstride, r.dstride, es[i].dets, es[i].dstride, r.drow,
                                     c.shots, cudaMemcpyDeviceToHost, eng.stream),
                   "copy dets");
            }
            if (r.obs && r.orow) {
                ck(cudaMemcpy2DAsync(r.obs + c.first * r.ostride, r.ostride, es[i].obs, es[i].ostride, r.orow,
                                     c.shots, cudaMemcpyDeviceToHost, eng.stream),
                   "copy obs");
            }
        }
        ck(cudaEventRecord(eng.ev[2], eng.stream), "event");
    }

    // Transposes with each entry's own layout flags (entries `es` are class g's members in order).
    void enqueue_transposes(Slot &slot, int g, const std::vector<gfs_rt::BatchEntry> &es) {
        const std::vector<size_t> &mem = slot.members[g];
        std::vector<gfs_rt::BatchEntry> group(es.size());
        std::vector<uint32_t> flags_seen;
        for (size_t k : mem) {
            const uint32_t f = slot.chunks[k].req->flags;
            if (std::find(flags_seen.begin(), flags_seen.end(), f) == flags_seen.end()) {
                flags_seen.push_back(f);
            }
        }
        for (uint32_t f : flags_seen) {
            for (size_t i = 0; i < es.size(); i++) {
                const bool same = slot.chunks[mem[i]].req->flags == f;
                group[i] = same ? es[i] : gfs_rt::BatchEntry{};
                if (!same) {
                    group[i].shots = 0;
                }
            }
            slot.eng[g].enqueue_transposes(group, f);
        }
    }

    // True when every class launched for the slot has finished on the device.
    bool slot_ready(Slot &slot) {
        for (int g = 0; g < kClasses; g++) {
            if (!slot.members[g].empty() && cudaEventQuery(slot.eng[g].ev[2]) == cudaErrorNotReady) {
                return false;
            }
        }
        return true;
    }

    void sync_slot(Slot &slot) {
        for (auto &e : slot.eng) {
            cudaStreamSynchronize(e.stream);
        }
    }

    void complete(Slot &slot) {
        std::string err;
        for (int g = 0; g < kClasses; g++) {  // every class's launch has ended before the slot is released
            if (!slot.members[g].empty()) {
                cudaError_t e = cudaEventSynchronize(slot.eng[g].ev[2]);
                if (e != cudaSuccess && err.empty()) {
                    err = std::string("batch failed: ") + cudaGetErrorString(e);
                }
            }
        }
        for (int g = 0; g < kClasses && err.empty(); g++) {
            if (slot.members[g].empty()) {
                continue;
            }
            gfs_rt::BatchEngine &eng = slot.eng[g];
            try {
                if (eng.check_status()) {
                    // A hit list overflowed: redo this class with inline noise (identical results).
                    eng.force_inline = true;
                    try {
                        launch_class(slot, g);
                        ck(cudaEventSynchronize(eng.ev[2]), "batch redo");
                        eng.check_status();
                    } catch (...) {
                        eng.force_inline = false;
                        throw;
                    }
                    eng.force_inline = false;
                }
            } catch (const std::exception &x) {
                err = x.what();
            }
        }
        std::lock_guard<std::mutex> lk(mu);
        batches++;
        entries_total += slot.chunks.size();
        for (const Chunk &c : slot.chunks) {
            Request &r = *c.req;
            if (!err.empty() && !r.failed) {
                r.failed = true;
                r.error = err;
            }
            r.done += c.shots;
            if (r.done >= r.shots && !r.finished) {
                finish_locked(r);
            }
        }
        slot.chunks.clear();
        slot.busy = false;
    }

    void run() {
        int next_slot = 0;
        for (;;) {
            Slot *to_launch = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                const bool any_busy = slots[0].busy || slots[1].busy;
                if (!any_busy) {
                    cv_work.wait(lk, [&] { return stop || !queue.empty(); });
                    if (queue.empty() && stop) {
                        return;
                    }
                }
                Slot &cand = slots[next_slot];
                if (!cand.busy && !queue.empty() && form_locked(cand)) {
                    cand.busy = true;
                    to_launch = &cand;
                }
            }
            if (to_launch) {
                try {
                    launch(*to_launch);
                } catch (const std::exception &x) {
                    sync_slot(*to_launch);
                    std::lock_guard<std::mutex> lk(mu);
                    for (const Chunk &c : to_launch->chunks) {
                        Request &r = *c.req;
                        r.failed = true;
                        r.error = x.what();
                        r.done += c.shots;
                        if (r.done >= r.shots && !r.finished) {
                            finish_locked(r);
                        }
                    }
                    to_launch->chunks.clear();
                    to_launch->busy = false;
                }
                next_slot ^= 1;
                continue;
            }
            // Nothing to launch now.  The older batch in flight is the one in next_slot when that slot is
            // busy.  With both slots busy, block until the older one ends; with one busy and nothing
            // queued, poll it so that new arrivals can start in the free slot right away.
            Slot &old = slots[next_slot].busy ? slots[next_slot] : slots[next_slot ^ 1];
            if (!old.busy) {
                continue;
            }
            const bool both_busy = slots[0].busy && slots[1].busy;
            if (both_busy || slot_ready(old)) {
                complete(old);
            } else {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait_for(lk, std::chrono::microseconds(100), [&] { return stop || !queue.empty(); });
            }
        }
    }

    // Returns 1 when the request has finished (0 on timeout); throws with its error when it failed.
    int wait(uint64_t id, double timeout_s, double *latency_ms) {
        std::unique_lock<std::mutex> lk(mu);
        auto it = live.find(id);
        if (it == live.end()) {
            throw std::invalid_argument("unknown or already collected request " + std::to_string(id));
        }
        std::shared_ptr<Request> r = it->second;
        auto pred = [&] { return r->finished; };
        if (timeout_s < 0) {
            cv_done.wait(lk, pred);
        } else if (!cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
            return 0;
        }
        live.erase(id);
        if (latency_ms) {
            *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        }
        if (r->failed) {
            throw std::runtime_error(r->error);
        }
        return 1;
    }

    void stats(double *out) {
        std::lock_guard<std::mutex> lk(mu);
        std::vector<double> l = latencies_ms;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) {
            if (l.empty()) {
                return 0.0;
            }
            size_t i = (size_t)std::min<double>((double)l.size() - 1, std::ceil(q * (double)l.size()) - 1);
            return l[i];
        };
        const double span =
            any_submit ? std::chrono::duration<double>(t_last_done - t_first_submit).count() : 0.0;
        out[0] = (double)completed;
        out[1] = (double)failed_count;
        out[2] = pct(0.50);
        out[3] = pct(0.99);
        out[4] = span > 0 ? (double)bits_done / span / 1e9 : 0.0;
        out[5] = (double)batches;
        out[6] = batches ? (double)entries_total / (double)batches : 0.0;
        out[7] = (double)cache_hits;
        out[8] = (double)cache_misses;
        out[9] = (double)max_queue;
        out[10] = (double)bits_done;
        out[11] = span;
    }

    void counters(uint64_t *out) {
        std::lock_guard<std::mutex> lk(mu);
        uint64_t pending = 0;
        for (const auto &kv : live) {
            pending += kv.second->finished ? 0 : 1;
        }
        out[0] = submitted;
        out[1] = rejected;
        out[2] = completed;
        out[3] = failed_count;
        out[4] = queue.size();
        out[5] = pending;
        out[6] = max_queue;
        out[7] = chunks_admitted;
    }
};

extern "C" {

gfs_status gfs_server_create(int device, uint64_t hbm_budget_bytes, uint64_t max_chunk_shots, gfs_server **out) {
    *out = nullptr;
    return guarded([&] {
        int count = 0;
        ck(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if (device < 0 || device >= count) {
            throw std::invalid_argument("no CUDA device " + std::to_string(device));
        }
        auto s = std::make_unique<gfs_server>();
        s->init(device, hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)8 << 30, max_chunk_shots);
        *out = s.release();
    });
}

void gfs_server_free(gfs_server *s) {
    delete s;
}

gfs_status gfs_server_submit(gfs_server *s, const char *text, size_t len, uint64_t shots, uint64_t seed,
                             uint32_t flags, int device_out, void *dets, uint64_t dets_stride, void *obs,
                             uint64_t obs_stride, uint64_t *ticket) {
    return guarded([&] {
        *ticket = s->submit(text, len, shots, seed, flags, device_out != 0, (uint8_t *)dets, dets_stride,
                            (uint8_t *)obs, obs_stride);
    });
}

gfs_status gfs_server_wait(gfs_server *s, uint64_t ticket, double timeout_s, int *done, double *latency_ms) {
    return guarded([&] { *done = s->wait(ticket, timeout_s, latency_ms); });
}

gfs_status gfs_server_stats(gfs_server *s, double *out12) {
    return guarded([&] { s->stats(out12); });
}

gfs_status gfs_server_counters(gfs_server *s, uint64_t *out8) {
    return guarded([&] { s->counters(out8); });
}

}  // extern "C"
