// Batched frame sampling shared by the batch API (batch.cc) and the request server (serve.cc): a list of
// entries (a lowered program on the device, a seed, a stream position, a shot count, destinations) is
// planned into one work list of (entry, 128-shot slice) items, sampled by ONE persistent
// batch_frame_kernel launch, and turned shot-major by one transpose per entry and output.
#pragma once

#include <unordered_map>

#include "sampler.h"

namespace gfs_rt {

struct BatchEntry {
    const gfs_sampler *prog = nullptr;  // program owner (its own seed and stream position are not used)
    uint64_t seed = 0;
    uint64_t block0 = 0;  // first 128-shot block of this entry in its random stream
    uint64_t shots = 0;
    uint8_t *dets = nullptr;  // device destinations; null skips the output
    uint64_t dstride = 0;
    uint8_t *obs = nullptr;
    uint64_t ostride = 0;
};

inline void layout_rows(const gfs_sampler *s, uint32_t flags, uint64_t *drow, uint64_t *orow) {
    const bool packed = flags & GFS_BIT_PACKED;
    const uint64_t D = s->prog.num_detectors, O = s->prog.num_observables;
    const uint64_t nd = D + ((flags & GFS_PREPEND_OBSERVABLES) ? O : 0) + ((flags & GFS_APPEND_OBSERVABLES) ? O : 0);
    *drow = packed ? (nd + 7) / 8 : nd;
    *orow = packed ? (O + 7) / 8 : O;
}

struct BatchEngine {
    int device = 0;
    int num_sms = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // start, frame done, end
    DevBuf d_desc, d_prefix, d_counter, d_status, det_arena, obs_arena, ring_buf;
    DevBuf hit_arena, count_arena, d_wprefix;
    gfs::LaunchShape shape{};
    // The lean batched kernel (frame_lean.cu) in hit-list mode when every program has a lean phase list:
    // same blocks, threads and ring placement as `shape`, its own shared memory and grid.
    bool lean = false;
    gfs::LaunchShape lean_shape{};
    uint64_t ring_stride_cur = 0;
    bool force_inline = false;  // set while a batch is redone after a hit list overflowed
    // Occurrence tables planned for this engine's blocks per CTA, per program.
    struct OccPlan {
        std::unique_ptr<DevBuf> occs;
        uint64_t slice_cap = 0;
        int blocks = 0;
    };
    std::unordered_map<const gfs_sampler *, OccPlan> occ_plans;
    std::vector<uint64_t> wprefix;
    uint64_t noise_warps = 0;

    // Current plan (set by prepare()).
    std::vector<gfs::KernelArgs> desc;
    std::vector<uint32_t> prefix;
    std::vector<uint64_t> det_off, obs_off;  // per entry (input order), in uint4 units
    uint32_t items = 0;

    BatchEngine() = default;
    BatchEngine(const BatchEngine &) = delete;
    BatchEngine &operator=(const BatchEngine &) = delete;

    ~BatchEngine() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
            for (auto &e : ev) {
                if (e) {
                    cudaEventDestroy(e);
                }
            }
            cudaStreamDestroy(stream);
        }
    }

    void init(int dev) {
        device = dev;
        ck(cudaSetDevice(device), "cudaSetDevice");
        cudaDeviceProp prop;
        ck(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
        num_sms = prop.multiProcessorCount;
        smem_optin = prop.sharedMemPerBlockOptin;
        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        for (auto &e : ev) {
            ck(cudaEventCreate(&e), "cudaEventCreate");
        }
        d_counter.ensure(16, device);
        d_status.ensure(16, device);
        ck(cudaMemsetAsync(d_status.p, 0, 16, stream), "memset");
        ck(cudaStreamSynchronize(stream), "init");
    }

    // Shape for a set of programs: dynamic shared memory and ring stride of the largest; grid = one wave.
    // Returns false when it does not fit.
    // Hit-list mode for a batch: every program either lists its noise occurrences or has none, and no
    // sampler asked for inline noise.
    static bool hits_for(const std::vector<const gfs_sampler *> &progs) {
        for (auto *p : progs) {
            if (p->hits_pref == 0 || (p->prog.occs.empty() && p->prog.noise_occurrences > 0)) {
                return false;
            }
        }
        return true;
    }

    bool fit(const std::vector<const gfs_sampler *> &progs, int bpc, int threads, bool ring_global,
             gfs::LaunchShape *out, uint64_t *ring_stride) const {
        const bool hits = hits_for(progs);
        size_t smem = 0;
        uint64_t rs = 0;
        for (auto *p : progs) {
            smem = std::max(smem, p->smem_for(bpc, ring_global, hits, false));
            rs = std::max<uint64_t>(rs, (uint64_t)bpc * p->prog.ring);
        }
        gfs::LaunchShape t{bpc, threads, 1, smem, ring_global};
        t.hits = hits;
        if (t.smem > smem_optin) {
            return false;
        }
        int per = 0;
        if (gfs::batch_frame_kernel_max_ctas_per_sm(t, &per) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (per < 1) {
            return false;
        }
        t.grid = per * num_sms;
        *out = t;
        *ring_stride = ring_global ? rs : 0;
        return true;
    }

    // ring: 0 shared memory, 1 global memory, -1 whichever keeps more blocks resident per SM.
    void set_shape(const std::vector<const gfs_sampler *> &progs, int bpc, int threads, int ring) {
        gfs::LaunchShape a{}, b{};
        uint64_t ra = 0, rb = 0;
        const bool fa = ring != 1 && fit(progs, bpc, threads, false, &a, &ra);
        const bool fb = ring != 0 && fit(progs, bpc, threads, true, &b, &rb);
        if (!fa && !fb) {
            throw std::invalid_argument("the largest circuit does not fit in shared memory with " + std::to_string(bpc) +
                                        " blocks per CTA");
        }
        const int res_a = fa ? a.grid * bpc : 0, res_b = fb ? b.grid * bpc : 0;
        const bool global = !fa || (fb && ring < 0 && res_b * 2 >= res_a * 3) || ring == 1;
        shape = global ? b : a;
        ring_stride_cur = global ? rb : ra;
        set_lean_shape(progs);
    }

    void set_lean_shape(const std::vector<const gfs_sampler *> &progs) {
        lean = false;
        if (!shape.hits) {
            return;
        }
        size_t smem = 0;
        for (auto *p : progs) {
            if (!p->prog.lean_ok || p->lean_pref == 0) {
                return;
            }
            smem = std::max(smem, gfs::lean_smem_bytes(p->prog.num_rows, shape.ring_global ? 0 : p->prog.ring,
                                                       (uint32_t)p->prog.num_observables, shape.blocks_per_cta,
                                                       (uint32_t)p->prog.lean.size(), (uint32_t)p->prog.occs.size(),
                                                       shape.threads));
        }
        gfs::LaunchShape l = shape;
        l.smem = smem;
        int per = 0;
        if (smem > smem_optin || gfs::batch_frame_kernel_lean_max_ctas_per_sm(l, &per) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        if (per < 1) {
            return;
        }
        l.grid = per * num_sms;
        lean_shape = l;
        lean = true;
    }

    // Default shape without timing: four blocks per CTA when at least two such CTAs fit per SM (small
    // and medium circuits), else one block per CTA of 128 threads; ring placement by residency.
    void default_shape(const std::vector<const gfs_sampler *> &progs) {
        gfs::LaunchShape t{};
        uint64_t rs = 0;
        for (bool g : {false, true}) {
            if (fit(progs, 4, 256, g, &t, &rs) && t.grid >= 2 * num_sms) {
                set_shape(progs, 4, 256, g ? 1 : 0);
                return;
            }
        }
        set_shape(progs, 1, 128, -1);
    }

    // Plans the entries (launch order = `order`, or input order when empty), allocates the arenas and
    // uploads the descriptors.  Returns the number of work items.
    uint32_t prepare(const std::vector<BatchEntry> &entries, const std::vector<uint32_t> &order) {
        const uint64_t B = (uint64_t)shape.blocks_per_cta;
        const size_t n = entries.size();
        desc.clear();
        prefix.assign(1, 0);
        det_off.assign(n, 0);
        obs_off.assign(n, 0);
        uint64_t det_total = 0, obs_total = 0, total = 0, hit_total = 0, count_total = 0;
        const bool hits = shape.hits && !force_inline;
        std::vector<uint64_t> hit_off(n, 0), count_off(n, 0);
        wprefix.assign(1, 0);
        for (size_t k = 0; k < n; k++) {
            const size_t j = order.empty() ? k : order[k];
            const BatchEntry &e = entries[j];
            const gfs_sampler *s = e.prog;
            const uint64_t nslices = ((e.shots + 127) / 128 + B - 1) / B;
            if (nslices == 0) {
                continue;
            }
            det_off[j] = det_total;
            obs_off[j] = obs_total;
            det_total += nslices * B * s->prog.num_detectors;
            obs_total += nslices * B * s->prog.num_observables;
            gfs::KernelArgs a{};
            a.ops = (const gfs::DevOp *)s->d_ops.p;
            a.pool = (const uint32_t *)s->d_pool.p;
            a.tables = (const uint32_t *)s->d_tables.p;
            a.chans = (const gfs::DevChan *)s->d_chans.p;
            a.qubit_orig = (const uint32_t *)s->d_orig.p;
            a.reset_zero = s->prog.reset_norand ? 1u : 0u;
            a.nrows = s->prog.num_rows;
            a.ring = s->prog.ring;
            a.nobs = (uint32_t)s->prog.num_observables;
            a.nslices = (uint32_t)nslices;
            a.ndet = s->prog.num_detectors;
            a.nmeas = 0;
            a.seed = e.seed;
            a.block0 = e.block0;
            a.status = (uint32_t *)d_status.p;
            a.smem_table_words = 0;  // the same shared-memory layout in hit-list mode and its inline fallback
            a.smem_ops = s->smem_ops();
            a.ring_cta_stride = ring_stride_cur;
            if (s->prog.lean_ok) {
                a.lean = (const gfs::LeanPhase *)s->d_lean.p;
                a.lean_inst = (const uint64_t *)s->d_lean_inst.p;
                a.n_lean = (uint32_t)s->prog.lean.size();
            }
            if (hits) {
                const OccPlan &pl = occ_plan(s);
                a.n_occ = (uint32_t)s->prog.occs.size();
                a.slice_cap = pl.slice_cap;
                a.occs = a.n_occ ? (const gfs::NoiseOcc *)pl.occs->p : nullptr;
                a.occ_xform = lean ? s->occ_xform() : nullptr;  // records for the lean plan's moved hit phases
                a.smem_occ = s->smem_occ(true);
                hit_off[j] = hit_total;
                count_off[j] = count_total;
                hit_total += nslices * pl.slice_cap;
                count_total += nslices * a.n_occ;
                const uint64_t sb = (uint64_t)gfs::noise_slices_per_warp_for((int)B);
                wprefix.push_back(wprefix.back() + (nslices + sb - 1) / sb * a.n_occ);
            }
            desc.push_back(a);
            total += nslices;
            if (total > 0xFFFFFFFFull) {
                throw std::invalid_argument("batch has too many 128-shot slices for one launch");
            }
            prefix.push_back((uint32_t)total);
        }
        det_arena.ensure(std::max<uint64_t>(16, det_total * 16), device);
        obs_arena.ensure(std::max<uint64_t>(16, obs_total * 16), device);
        noise_warps = 0;
        if (hits) {
            hit_arena.ensure(std::max<uint64_t>(16, hit_total * 8), device);
            count_arena.ensure(std::max<uint64_t>(16, count_total * 4), device);
            noise_warps = wprefix.back();
            d_wprefix.ensure(wprefix.size() * sizeof(uint64_t), device);
            ck(cudaMemcpyAsync(d_wprefix.p, wprefix.data(), wprefix.size() * sizeof(uint64_t), cudaMemcpyHostToDevice,
                               stream),
               "descriptor upload");
        }
        if (shape.ring_global) {
            const uint64_t grid = std::max<uint64_t>((uint64_t)shape.grid, lean ? (uint64_t)lean_shape.grid : 0);
            ring_buf.ensure(std::max<uint64_t>(16, grid * ring_stride_cur * 16), device);
        }
        size_t k = 0;
        for (size_t q = 0; q < n; q++) {
            const size_t j = order.empty() ? q : order[q];
            if (entries[j].shots == 0) {
                continue;
            }
            gfs::KernelArgs &a = desc[k++];
            a.det_out = (uint4 *)det_arena.p + det_off[j];
            a.obs_out = (uint4 *)obs_arena.p + obs_off[j];
            a.ring_global = shape.ring_global ? (uint4 *)ring_buf.p : nullptr;
            if (hits) {
                a.hits = (uint64_t *)hit_arena.p + hit_off[j];
                a.hit_count = (uint32_t *)count_arena.p + count_off[j];
            }
        }
        if (!desc.empty()) {
            d_desc.ensure(desc.size() * sizeof(gfs::KernelArgs), device);
            d_prefix.ensure(prefix.size() * sizeof(uint32_t), device);
            ck(cudaMemcpyAsync(d_desc.p, desc.data(), desc.size() * sizeof(gfs::KernelArgs), cudaMemcpyHostToDevice,
                               stream),
               "descriptor upload");
            ck(cudaMemcpyAsync(d_prefix.p, prefix.data(), prefix.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                               stream),
               "descriptor upload");
        }
        items = prefix.back();
        return items;
    }

    void enqueue_frame() {
        ck(cudaMemsetAsync(d_counter.p, 0, 4, stream), "memset");
        gfs::BatchArgs b{};
        b.circuits = (const gfs::KernelArgs *)d_desc.p;
        b.slice_prefix = (const uint32_t *)d_prefix.p;
        b.ncircuits = (uint32_t)desc.size();
        b.total_slices = items;
        b.counter = (uint32_t *)d_counter.p;
        b.warp_prefix = (const uint64_t *)d_wprefix.p;
        b.total_noise_warps = noise_warps;
        if (lean && !force_inline) {
            gfs::LaunchShape l = lean_shape;
            l.grid = (int)std::min<uint64_t>((uint64_t)l.grid, items);
            ck(gfs::launch_batch_frame_kernel_lean(b, l, stream), "lean batch frame kernel launch");
            return;
        }
        gfs::LaunchShape s = shape;
        s.hits = shape.hits && !force_inline;
        if (shape.hits && force_inline) {
            s = inline_shape();
        }
        s.grid = (int)std::min<uint64_t>((uint64_t)s.grid, items);
        ck(gfs::launch_batch_frame_kernel(b, s, stream), "batch frame kernel launch");
    }

    // The current shape for the inline-noise batch kernel (same blocks, threads and ring placement).
    gfs::LaunchShape inline_shape() const {
        gfs::LaunchShape t = shape;
        t.hits = false;
        int per = 0;
        if (gfs::batch_frame_kernel_max_ctas_per_sm(t, &per) != cudaSuccess || per < 1) {
            cudaGetLastError();
            per = 1;
        }
        t.grid = per * num_sms;
        return t;
    }

    // Occurrence regions of program s planned for this engine's blocks per CTA (uploaded once).
    const OccPlan &occ_plan(const gfs_sampler *s) {
        OccPlan &pl = occ_plans[s];
        if (!pl.occs || pl.blocks != shape.blocks_per_cta) {
            std::vector<gfs::NoiseOcc> occs = s->prog.occs;
            pl.slice_cap = gfs::plan_hit_regions(occs, s->prog.occ_hits_per_block, (uint32_t)shape.blocks_per_cta,
                                                 s->hit_capacity_override);
            pl.occs = std::make_unique<DevBuf>();
            upload(*pl.occs, occs, device, stream);
            pl.blocks = shape.blocks_per_cta;
        }
        return pl;
    }

    // One transpose per entry and output.  Returns the number of transpose calls enqueued.
    uint64_t enqueue_transposes(const std::vector<BatchEntry> &entries, uint32_t flags) {
        const bool packed = flags & GFS_BIT_PACKED;
        uint64_t calls = 0;
        for (size_t j = 0; j < entries.size(); j++) {
            const BatchEntry &e = entries[j];
            if (e.shots == 0) {
                continue;
            }
            const uint64_t D = e.prog->prog.num_detectors, O = e.prog->prog.num_observables;
            const uint4 *dt = (const uint4 *)det_arena.p + det_off[j];
            const uint4 *ot = (const uint4 *)obs_arena.p + obs_off[j];
            auto tr = [&](const uint4 *s0, uint64_t n0, const uint4 *s1, uint64_t n1, const uint4 *s2, uint64_t n2,
                          uint8_t *out, uint64_t stride) {
                gfs::TransposeArgs t{};
                t.src0 = s0;
                t.n0 = n0;
                t.src1 = s1;
                t.n1 = n1;
                t.src2 = s2;
                t.n2 = n2;
                t.nshots = e.shots;
                t.out = out;
                t.out_stride = stride;
                t.bit_packed = packed ? 1 : 0;
                ck(gfs::launch_transpose(t, stream), "transpose launch");
                calls++;
            };
            if (e.dets) {
                if ((flags & GFS_PREPEND_OBSERVABLES) && (flags & GFS_APPEND_OBSERVABLES)) {
                    tr(ot, O, dt, D, ot, O, e.dets, e.dstride);
                } else if (flags & GFS_PREPEND_OBSERVABLES) {
                    tr(ot, O, dt, D, nullptr, 0, e.dets, e.dstride);
                } else if (flags & GFS_APPEND_OBSERVABLES) {
                    tr(dt, D, ot, O, nullptr, 0, e.dets, e.dstride);
                } else {
                    tr(dt, D, nullptr, 0, nullptr, 0, e.dets, e.dstride);
                }
            }
            if (e.obs) {
                tr(ot, O, nullptr, 0, nullptr, 0, e.obs, e.ostride);
            }
        }
        return calls;
    }

    // Reads and clears the kernels' status word (after the stream has drained).  Bits 1 and 2 are errors;
    // bit 4 (a hit list overflowed) is returned as true: the caller redoes the batch with inline noise.
    bool check_status() {
        uint32_t st = 0;
        ck(cudaMemcpy(&st, d_status.p, 4, cudaMemcpyDeviceToHost), "status read");
        if (st) {
            ck(cudaMemset(d_status.p, 0, 4), "status clear");
        }
        if (st & 3u) {
            throw std::runtime_error("batch frame kernel reported error status " + std::to_string(st));
        }
        return (st & 4u) != 0;
    }
};

}  // namespace gfs_rt
