// Frame-sampling kernels for sm_103a.
//
// frame_kernel<B, HITS>: one CTA owns a slice of B x 128 shots at a time (persistent, grid-stride over
// slices).  Its X/Z Pauli frames ([row][block] uint4, 128 shots per uint4), the measurement ring, the
// observable accumulators and the correlated-error flags live in shared memory for the whole circuit.  The
// CTA walks the device program (program.h): every op spreads its independent units over the threads,
// updates 128 shots per unit with 128-bit shared-memory loads/stores and bitwise logic, and ends with one
// __syncthreads().  The lowering orders each gate op's units so that a quarter-warp's eight 16-byte
// accesses fall in distinct bank groups.  Noise follows the counter-based stream of gfs_contract.h: with
// HITS, noise_kernel has already drawn every hit into per-occurrence record lists and the frame kernel only
// XORs them in; without, a thread owns a segment of 16 units x 128 shots and skips geometrically to its hits
// (noise next to a gate on the same targets is fused into the gate op).  Detection events stream to
// global memory as [block][detector] uint4 rows.
//
// noise_kernel<B>: one warp per (slice, noise occurrence), writing the hit records.
//
// batch_frame_kernel<B>: the frame kernel over many circuits' (circuit, slice) work items.
//
// transpose_tile_kernel: turns [block][row] bit-rows into shot-major bytes with 32x32 shuffle-butterfly
// bit transposes, replacing the reference's bit-by-bit numpy conversion (numpy.pybind.cc:20-63) and
// simd_bit_table::transpose_into (simd_bit_table.inl:192-208).
#include <algorithm>
#include <cstdio>

#include "frame_device.cuh"

namespace gfs {

// Gate op with noise fused before and/or after it.  The op's units are its instruction's units (the
// lowering fuses only single-run instructions whose noise targets are the same list), so the noise of
// unit u is keyed exactly as the standalone noise instruction would be.  Each lane takes one noise
// segment (sixteen units x 128 shots): it walks the pre-noise hits into those units' shared-memory rows,
// applies the gate to the sixteen units, then walks the post-noise hits.  The rows are the lane's own, so
// there are no atomics and no extra phase.
// The gate of one unit of a fused op (noise is applied separately, in place, by the segment owner).
template <int B>
__device__ __forceinline__ void gate_unit(const KernelArgs &p, uint32_t code, uint32_t sub, uint32_t a, uint32_t rb,
                                          uint64_t inst, uint32_t u, uint32_t blk, uint32_t block, uint4 *X, uint4 *Z,
                                          uint4 *R, uint32_t rec, uint32_t L, bool norand) {
    const bool pair = code == OP_2Q;
    const uint32_t i1 = __ldg(p.pool + a + (pair ? 2 * u : u)) * B + blk;
    if (pair) {
        const uint32_t i2 = __ldg(p.pool + a + 2 * u + 1) * B + blk;
        uint4 x1 = X[i1], z1 = Z[i1], x2 = X[i2], z2 = Z[i2];
        rule2v(sub, x1, z1, x2, z2);
        X[i1] = x1;
        Z[i1] = z1;
        X[i2] = x2;
        Z[i2] = z2;
    } else if (code == OP_1Q) {
        uint4 x = X[i1], z = Z[i1];
        rule1(sub, x, z);
        X[i1] = x;
        Z[i1] = z;
    } else if (code == OP_MEASURE) {
        measure_row(sub, X, Z, R, i1, wrap(rec + u, L) * B + blk, rand_row(p, norand, inst, rb + u, block),
                    p.ring_global != nullptr, norand);
    } else {  // OP_RESET
        reset_row(sub, X, Z, i1, rand_row(p, norand, inst, rb + u, block), norand);
    }
}

// Gate op with noise fused before and/or after it.  The op's units are its instruction's units (the
// lowering fuses only single-run instructions whose noise targets are the same list), so the noise of
// unit u is keyed exactly as the standalone noise instruction would be.  A warp takes 32 noise segments
// (sixteen units x 128 shots each): every lane walks its segment's pre-noise hits into those units'
// shared-memory rows; after a __syncwarp the warp applies the gate to the 128 units with consecutive lanes
// on consecutive units (so quarter-warps touch distinct banks); after another __syncwarp each lane walks
// its post-noise hits.  All rows stay within the warp: no atomics, no extra CTA phase.
template <int B>
__device__ __forceinline__ void fused_gate(const KernelArgs &p, const DevOp &op, uint32_t code, uint32_t sub,
                                           uint64_t inst, uint64_t gb0, const uint32_t *tables, uint4 *X, uint4 *Z,
                                           uint4 *R, uint32_t rec, uint32_t L, uint32_t tid, uint32_t nt) {
    const uint32_t n = op.n, a = op.a;
    const Fused pre = decode_fused(p, op.d, inst), post = decode_fused(p, op.c, inst);
    const bool pair = code == OP_2Q;
    const uint32_t nseg = (n + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
    const uint32_t items = nseg * B;  // (segment, block) pairs
    const uint32_t lane = tid & 31u;
    for (uint32_t item0 = tid - lane; item0 < items; item0 += nt) {  // warp-uniform trip count
        const uint32_t item = item0 + lane;
        const bool valid = item < items;
        const uint32_t q = item / B, blk = item % B;
        const uint32_t u0 = q * GFS_SEG_UNITS;
        const uint32_t un = valid ? min(GFS_SEG_UNITS, n - u0) : 0;
        const uint32_t block = (uint32_t)(gb0 + blk);
        if (pre.ch) {
            if (un) {
                walk_segment(*pre.ch, tables + pre.ch->table, p.seed, GFS_P_NOISE, pre.inst, q, block, un,
                             [&](uint32_t k, uint32_t shot, gfs_stream *st) {
                                 const uint32_t bits = hit_bits(pre.kind, *pre.ch, st);
                                 const uint32_t u = u0 + k;
                                 const uint32_t i1 = __ldg(p.pool + a + (pair ? 2 * u : u)) * B + blk;
                                 const uint32_t i2 = pair ? __ldg(p.pool + a + 2 * u + 1) * B + blk : i1;
                                 apply_bits(X, Z, i1, i2, shot, bits, false);
                             });
            }
            __syncwarp();
        }
        // The warp's items cover units [item0 / B * 4, ...) of B blocks: 128 (unit, block) gate items.
        const uint32_t ubase = (item0 / B) * GFS_SEG_UNITS;
#pragma unroll
        for (uint32_t m = 0; m < GFS_SEG_UNITS; m++) {
            const uint32_t j = m * 32 + lane;  // (unit, block) gate item of this warp, blocks fastest
            const uint32_t u = ubase + j / B, gb = j % B;
            if (u < n && (item0 + (j / B) / GFS_SEG_UNITS * B + gb) < items) {
                gate_unit<B>(p, code, sub, a, op.b, inst, u, gb, (uint32_t)(gb0 + gb), X, Z, R, rec, L,
                             (op.code & kNoRandomize) != 0);
            }
        }
        if (post.ch) {
            __syncwarp();
            if (un) {
                walk_segment(*post.ch, tables + post.ch->table, p.seed, GFS_P_NOISE, post.inst, q, block, un,
                             [&](uint32_t k, uint32_t shot, gfs_stream *st) {
                                 const uint32_t bits = hit_bits(post.kind, *post.ch, st);
                                 const uint32_t u = u0 + k;
                                 const uint32_t i1 = __ldg(p.pool + a + (pair ? 2 * u : u)) * B + blk;
                                 const uint32_t i2 = pair ? __ldg(p.pool + a + 2 * u + 1) * B + blk : i1;
                                 apply_bits(X, Z, i1, i2, shot, bits, false);
                             });
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------------------------------
// Precomputed noise.  noise_kernel walks the program once per slice, exactly as the frame kernel does,
// and draws every noise occurrence's hits (same contract, same streams) into a list of 64-bit records;
// the frame kernel in hit-list mode then only XORs the recorded bits into its shared-memory frames.
// This takes the Philox/geometric-skip work, its register pressure and its lane imbalance out of the
// frame kernel, whose CTAs wait on a barrier after every op.
//
// Record: bits 0..23 row (measurement flips: result index within the instruction), 24..47 second row
// (heralds: result index), 48..51 Pauli bits (X, Z on the first row, X, Z on the second), 52..60 shot
// within the slice (block * 128 + shot).  Records of one occurrence are contiguous but unordered (XOR
// and OR commute).
// ------------------------------------------------------------------------------------------------
// One noise occurrence resolved: channel, Pauli kind, stream purpose, units and where their rows are.
struct OccParams {
    const DevChan *ch;
    uint32_t code, sub, kind, purpose, n, a;
    bool pair, fused;
    uint64_t inst;
    const OccXform *xf;  // the lean plan moved this occurrence: transform its Paulis (program.h OccXform)
};

// The Pauli bits of a hit on rows (r1, r2) as they must be applied where the lean plan moved the occurrence.
__device__ __forceinline__ uint32_t xform_bits(const OccXform &x, const uint32_t *pool, uint32_t bits, uint32_t r1,
                                               uint32_t r2, bool pair) {
    bits = ((bits < 8 ? x.own_lo >> (4 * bits) : x.own_hi >> (4 * (bits - 8)))) & 15u;
    for (uint32_t f = 0; f < x.nf; f++) {
        const uint32_t tab = x.ftab[f];
        const uint32_t *mem = pool + x.fmem[f];
        if ((__ldg(mem + (r1 >> 5)) >> (r1 & 31)) & 1u) {
            bits = (bits & ~3u) | ((tab >> (2 * (bits & 3u))) & 3u);
        }
        if (pair && ((__ldg(mem + (r2 >> 5)) >> (r2 & 31)) & 1u)) {
            bits = (bits & 3u) | (((tab >> (2 * ((bits >> 2) & 3u))) & 3u) << 2);
        }
    }
    return bits;
}

// which = 0 for a noise op, 1 for the noise fused before a gate (op.d), 2 for the noise fused after it (op.c).
__device__ __forceinline__ OccParams occ_params(const KernelArgs &p, const DevOp &op, uint32_t which,
                                                uint64_t inst) {
    OccParams o;
    o.code = op.code & 0xFFu;
    o.sub = (op.code >> 8) & 0xFFu;
    o.a = op.a;
    o.n = op.n;
    o.purpose = GFS_P_NOISE;
    o.pair = false;
    o.fused = which != 0;
    o.inst = inst;
    o.xf = nullptr;
    if (which) {
        const uint32_t w = which == 1 ? op.d : op.c;
        o.ch = &p.chans[(w & kFusedChanMask) - 1];
        o.kind = (w >> 20) & 0xFu;
        o.inst = inst + (int64_t)(int8_t)(w >> 24);
        o.pair = o.code == OP_2Q;
    } else {
        o.ch = &p.chans[op.b];
        o.kind = o.sub;
        if (o.code == OP_NOISE) {
            o.pair = o.sub == KN_DEP2 || o.sub == KN_PC2;
        } else if (o.code == OP_MNOISE) {
            o.purpose = GFS_P_MNOISE;
            o.kind = KN_FLIP;
        } else if (o.code == OP_CORR_MASK) {
            o.n = 1;
        }
    }
    return o;
}

// The record of a hit on unit u at (block blk, shot), drawing the Pauli choice from the segment's stream
// as the contract orders it.
__device__ __forceinline__ uint64_t occ_record(const KernelArgs &p, const OccParams &o, uint32_t u, uint32_t blk,
                                               uint32_t shot, gfs_stream *st) {
    const uint32_t s9 = blk * 128 + shot;
    if (!o.fused && o.code == OP_MNOISE) {
        return hit_record(u, 0, 1, s9);
    }
    if (!o.fused && o.code == OP_CORR_MASK) {
        return hit_record(0, 0, 0, s9);
    }
    if (!o.fused && o.code == OP_HERALD) {
        const uint32_t c = gfs_stream_next(st);
        const uint32_t v = o.sub == 0 ? (c & 3u) : pauli_xz(gfs_choice_weighted(c, o.ch->cum, 4));
        return hit_record(__ldg(p.pool + o.a + u), u, v, s9);
    }
    uint32_t bits = hit_bits(o.kind, *o.ch, st);
    const uint32_t r1 = __ldg(p.pool + o.a + (o.pair ? 2 * u : u));
    const uint32_t r2 = o.pair ? __ldg(p.pool + o.a + 2 * u + 1) : r1;
    if (o.xf) {
        bits = xform_bits(*o.xf, p.pool, bits, r1, r2, o.pair);
    }
    return hit_record(r1, r2, bits, s9);
}

// One warp draws the hit records of one (slice, occurrence).  Screening rounds are dense: each lane draws
// the first Philox group of one segment, and the segments whose first draw leaves the segment (13% of them at
// p = 1e-3 with 2,048 trials) are done.  Segments with a hit are queued in shared memory with their three unused draws.  Lanes
// then walk queued segments hit by hit, exactly as gfs_next_hit would (same draws, same order); a lane whose
// segment ends takes the next queued one at once, and a new screening round runs whenever the queue can no
// longer refill the warp.  Every step each lane with a pending hit writes up to two records; the records of a step
// get consecutive slots (ballot prefix), so the stores coalesce and no atomics are needed.  No barriers:
// occurrences and slices are independent streams.
struct NoiseQueued {
    uint32_t item, u, d1, d2, d3;
};

// One warp draws occurrence k of the SB slices slice0 .. slice0 + nsub - 1 (B blocks each) into their regions
// of the hit list; count[s] (the warp's counters in shared memory) receives the records of slice slice0 + s
// (records past the region's capacity are counted but not written).  Items are (segment, slice, block), blocks
// fastest, so a warp screens the same segment of several blocks together; records of one step go to
// consecutive slots of their own slice's region (lanes of one slice grouped by __match_any_sync).  `q` is the
// warp's queue (64 entries).
template <int B, int SB>
__device__ __forceinline__ void noise_records(const KernelArgs &p, uint32_t slice0, uint32_t nsub, uint32_t k,
                                              uint32_t lane, NoiseQueued *q, uint32_t *count) {
    const NoiseOcc oc = p.occs[k];
    const DevOp op = p.ops[oc.pc];
    OccParams o = occ_params(p, op, oc.which, oc.inst);
    if (p.occ_xform && oc.xform) {
        o.xf = p.occ_xform + (oc.xform - 1);
    }
    if (lane < (uint32_t)SB) {
        count[lane] = 0;  // this warp's records per slice (shared memory)
    }
    __syncwarp();
    if (!o.ch->active) {
        return;
    }
    const DevChan &ch = *o.ch;
    const uint32_t *T = p.tables + ch.table;
    const bool always = ch.always != 0;
    const uint32_t nseg = (o.n + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
    constexpr uint32_t per_seg = (uint32_t)(B * SB);
    const uint32_t items = nseg * per_seg;
    const uint32_t kseed0 = (uint32_t)p.seed, kseed1 = (uint32_t)(p.seed >> 32);
    const uint32_t c3base = gfs_c3(o.purpose, o.inst, 0);
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t qn = 0;        // queued segments (warp-uniform)
    uint32_t screened = 0;  // items screened so far (warp-uniform)
    // This lane's segment walk.
    bool active = false;
    gfs_stream st;
    int32_t pos = -1, trials = 0;
    uint32_t u0 = 0, blk = 0, sub = 0;
    for (;;) {
        // Idle lanes take queued segments (the most recently queued first).
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
        if (idle && qn) {
            const uint32_t take = min((uint32_t)__popc(idle), qn);
            const uint32_t rank = __popc(idle & lt);
            if (!active && rank < take) {
                const NoiseQueued e = q[qn - 1 - rank];
                const uint32_t g = e.item / per_seg, r = e.item % per_seg;
                sub = r / B;
                blk = r % B;
                u0 = g * GFS_SEG_UNITS;
                trials = (int32_t)(min(GFS_SEG_UNITS, o.n - u0) * GFS_BLOCK_SHOTS);
                gfs_stream_init(&st, p.seed, o.purpose, o.inst, g,
                                (uint32_t)(p.block0 + (uint64_t)(slice0 + sub) * B + blk));
                if (always) {
                    pos = 0;
                } else {
                    // Group 0 was drawn when screening: u decided the first hit; d1..d3 come next.
                    st.group = 1;
                    st.left = 3;
                    st.b0 = e.d1;
                    st.b1 = e.d2;
                    st.b2 = e.d3;
                    pos = gfs_hit_after_draw(e.u, T, ch.inv_c, -1, trials);
                }
                active = pos >= 0;
            }
            qn -= take;
            __syncwarp();
        }
        // Screen the next 32 items when the queue could not refill the whole warp.
        if (qn < 32 && screened < items) {
            const uint32_t item = screened + lane;
            bool hit = false;
            uint32_t u = 0, d1 = 0, d2 = 0, d3 = 0;
            const uint32_t g = item / per_seg, r = item % per_seg;
            if (item < items && r / B < nsub) {
                if (always) {
                    hit = true;
                } else {
                    const uint32_t units = min(GFS_SEG_UNITS, o.n - g * GFS_SEG_UNITS);
                    const uint32_t block = (uint32_t)(p.block0 + (uint64_t)(slice0 + r / B) * B + r % B);
                    const gfs_u32x4 rr = gfs_philox(kseed0, kseed1, block, g, (uint32_t)o.inst, c3base);
                    u = rr.v[0];
                    d1 = rr.v[1];
                    d2 = rr.v[2];
                    d3 = rr.v[3];
                    hit = u >= __ldg(T + units * GFS_BLOCK_SHOTS);
                }
            }
            const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
            if (hit) {
                q[qn + __popc(mask & lt)] = NoiseQueued{item, u, d1, d2, d3};
            }
            qn += __popc(mask);
            screened += 32;
            __syncwarp();
            continue;
        }
        const uint32_t act = __ballot_sync(0xFFFFFFFFu, active);
        if (!act) {
            if (qn == 0 && screened >= items) {
                break;
            }
            continue;
        }
        // Up to two hits per active lane (the walk's next two), each lane's records into its own slice's region: the
        // lanes of one slice take consecutive places after the slice's count, which their first lane advances once.
        // Two per step halve the warp-level bookkeeping per hit (ballots, queue and screening checks, routing);
        // three or four per step cost more in code size and registers than they save.
        if (active) {
            const uint64_t r1 = occ_record(p, o, u0 + ((uint32_t)pos >> 7), blk, (uint32_t)pos & 127u, &st);
            pos = gfs_next_hit(&st, T, ch.inv_c, pos, trials, always);
            const bool two = pos >= 0;
            uint64_t r2 = 0;
            if (two) {
                r2 = occ_record(p, o, u0 + ((uint32_t)pos >> 7), blk, (uint32_t)pos & 127u, &st);
                pos = gfs_next_hit(&st, T, ch.inv_c, pos, trials, always);
            }
            const uint32_t sec = __ballot_sync(act, two);  // lanes with a second record
            uint32_t at;
            if (SB == 1) {
                at = count[0] + __popc(act & lt) + __popc(sec & lt);
                __syncwarp(act);
                if (lane == (uint32_t)(__ffs(act) - 1)) {
                    count[0] += __popc(act) + __popc(sec);
                }
            } else {
                const uint32_t peers = __match_any_sync(act, sub);
                const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
                uint32_t base = 0;
                if (lane == leader) {
                    base = count[sub];
                    count[sub] = base + __popc(peers) + __popc(peers & sec);
                }
                at = __shfl_sync(act, base, leader) + __popc(peers & lt) + __popc(peers & sec & lt);
            }
            uint64_t *const region = p.hits + (uint64_t)(slice0 + sub) * p.slice_cap + oc.off;
            if (at < oc.cap) {
                region[at] = r1;
            }
            if (two && at + 1 < oc.cap) {
                region[at + 1] = r2;
            }
            active = pos >= 0;
        }
        __syncwarp();
    }
}

// Warp w draws occurrence w % n_occ of the SB slices from (w / n_occ) * SB on into their regions.
template <int B, int SB>
__device__ __forceinline__ void noise_warp(const KernelArgs &p, uint64_t w, uint32_t warp, uint32_t lane,
                                           NoiseQueued (*queue)[64], uint32_t *counts) {
    const uint32_t slice0 = (uint32_t)(w / p.n_occ) * SB, k = (uint32_t)(w % p.n_occ);
    const uint32_t nsub = min((uint32_t)SB, p.nslices - slice0);
    uint32_t *count = counts + warp * SB;
    noise_records<B, SB>(p, slice0, nsub, k, lane, queue[warp], count);
    __syncwarp();
    if (lane == 0) {
        const uint32_t cap = p.occs[k].cap;
#pragma unroll
        for (int s = 0; s < SB; s++) {
            if ((uint32_t)s < nsub) {
                uint32_t c = count[s];
                if (c > cap) {
                    atomicOr(p.status, 4u);
                    c = 0;
                }
                p.hit_count[(uint64_t)(slice0 + s) * p.n_occ + k] = c;
            }
        }
    }
}

template <int B>
__host__ __device__ constexpr int noise_slices_per_warp() {
    return noise_slices_per_warp_for(B);
}

template <int B>
__global__ void __launch_bounds__(256) noise_kernel(const KernelArgs p) {
    constexpr int SB = noise_slices_per_warp<B>();
    __shared__ NoiseQueued queue[8][64];
    __shared__ uint32_t counts[8 * SB];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t w = (uint64_t)blockIdx.x * 8 + warp;
    if (w < (uint64_t)((p.nslices + SB - 1) / SB) * p.n_occ) {
        noise_warp<B, SB>(p, w, warp, lane, queue, counts);
    }
}

// The noise of a batch: warp w belongs to circuit j with warp_prefix[j] <= w < warp_prefix[j + 1].
template <int B>
__global__ void __launch_bounds__(256) batch_noise_kernel(const BatchArgs b) {
    constexpr int SB = noise_slices_per_warp<B>();
    __shared__ NoiseQueued queue[8][64];
    __shared__ uint32_t counts[8 * SB];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t w = (uint64_t)blockIdx.x * 8 + warp;
    if (w >= b.total_noise_warps) {
        return;
    }
    uint32_t lo = 0, hi = b.ncircuits;  // last j with warp_prefix[j] <= w
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (b.warp_prefix[mid] <= w) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    const KernelArgs &p = b.circuits[lo];
    noise_warp<B, SB>(p, w - b.warp_prefix[lo], warp, lane, queue, counts);
}

// Shared-memory layout of a CTA holding B blocks of 128 shots: X and Z frames [row][block], the
// measurement ring [ring row][block] (unless it is in global memory), observable accumulators, the
// correlated-error flags and mask, then the gap tables, the op stream, and the occurrence cache when they
// are cached.
struct FrameState {
    uint4 *X, *Z, *R, *O, *OCC, *MSK;
    const uint32_t *tables;
    const DevOp *ops;
    uint32_t *occ_off, *occ_cnt;  // hit-list mode with cached occurrences: region offsets, slice's counts
};

// Starts pulling occurrence `occ`'s records into L2 (one bulk prefetch; regions start on 16 bytes and
// hold an even number of records, so rounding the size up stays inside the region).
__device__ __forceinline__ void prefetch_occurrence(const KernelArgs &p, const uint32_t *occ_off,
                                                    const uint32_t *occ_cnt, uint32_t slice, uint32_t occ) {
    if (occ >= p.n_occ || !occ_cnt) {
        return;
    }
    uint32_t count;
    const uint64_t *h = occ_records(p, occ_off, occ_cnt, slice, occ, &count);
    const uint32_t bytes = ((count + 1) & ~1u) * 8u;
    if (bytes) {
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(h), "r"(bytes) : "memory");
    }
}

// Applies the records of occurrence `occ` of this slice: Pauli flips into the frames, measurement flips
// into the ring, heralds into the ring and frames; correlated-error hits are OR-ed into MSK (the caller
// clears it first and derives the mask afterwards).  The thread's first two records come from `pre`
// (loaded a phase earlier); it then loads its first two records of the next occurrence into `pre`, and
// thread 0 prefetches the records two occurrences ahead into L2.
template <int B>
__device__ __forceinline__ void apply_hits(const KernelArgs &p, const FrameState &st, uint32_t slice, uint32_t occ,
                                           uint32_t kind, uint4 *X, uint4 *Z, uint4 *R, uint4 *MSK, uint32_t rec,
                                           uint32_t L, uint32_t n, uint32_t tid, uint32_t nt, HitPre &pre) {
    if (occ >= p.n_occ) {  // the host counted fewer occurrences than the program has
        if (tid == 0) {
            atomicOr(p.status, 2u);
        }
        return;
    }
    if (tid == 0) {
        prefetch_occurrence(p, st.occ_off, st.occ_cnt, slice, occ + 2);
    }
    uint32_t count;
    const uint64_t *h = occ_records(p, st.occ_off, st.occ_cnt, slice, occ, &count);
    const HitPre cur = pre;
    hit_prefetch(p, st.occ_off, st.occ_cnt, slice, occ + 1, tid, nt, pre);
    if ((tid & ~31u) >= count) {  // no record for this warp (warp-uniform)
        return;
    }
    for (uint32_t i = tid; i < count; i += nt) {
        const uint64_t r = i == tid ? cur.r0
                           : i == tid + nt ? cur.r1
                                           : __ldcg(reinterpret_cast<const unsigned long long *>(h + i));
        const uint32_t ra = (uint32_t)r & kRowMask, rb = (uint32_t)(r >> 24) & kRowMask;
        const uint32_t bits = (uint32_t)(r >> 48) & 15u, s9 = (uint32_t)(r >> 52) & 511u;
        const uint32_t blk = s9 >> 7, shot = s9 & 127u;
        switch (kind) {
            case OCC_PAULI:
                apply_bits(X, Z, ra * B + blk, rb * B + blk, shot, bits, true);
                break;
            case OCC_FLIP:
                flip_bit(R, wrap(rec + L - n + ra, L) * B + blk, shot, true);
                break;
            case OCC_HERALD:
                atomic_or_bit(R, wrap(rec + L - n + rb, L) * B + blk, shot);
                apply_bits(X, Z, ra * B + blk, ra * B + blk, shot, bits, true);
                break;
            default:  // OCC_CORR
                atomic_or_bit(MSK, blk, shot);
                break;
        }
    }
}

// Lays out shared memory for circuit `p` and copies its gap tables and op stream in; the copies are
// visible after the next __syncthreads() (the first one in frame_slice).
template <int B>
__device__ __forceinline__ FrameState frame_state(const KernelArgs &p, uint4 *sm, bool frames_global = false) {
    FrameState st;
    const uint32_t nr = p.nrows, L = p.ring, NO = p.nobs;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    // Frames in shared memory, or (circuits too large for it; a compile-time choice of the kernel) in this CTA's
    // region of a global buffer.
    uint4 *const fr = frames_global ? p.frames_global + (size_t)blockIdx.x * p.frames_cta_stride : sm;
    uint4 *const after = frames_global ? sm : sm + (size_t)2 * nr * B;  // next free shared-memory entry
    st.X = fr;
    st.Z = st.X + (size_t)nr * B;
    // The measurement ring lives in shared memory, or (for large rings, to fit more CTAs per SM) in this
    // CTA's own region of a global scratch buffer, which stays L2-resident.
    st.R = p.ring_global ? p.ring_global + (size_t)blockIdx.x * p.ring_cta_stride : after;
    st.O = p.ring_global ? after : st.R + (size_t)L * B;
    st.OCC = st.O + (size_t)NO * B;
    st.MSK = st.OCC + B;
    // Gap tables are read on every noise draw; keep them in shared memory when the launch reserved room.
    st.tables = p.tables;
    uint32_t *st_tables = reinterpret_cast<uint32_t *>(st.MSK + B);
    if (p.smem_table_words) {
        for (uint32_t i = tid; i < p.smem_table_words; i += nt) {
            st_tables[i] = __ldg(p.tables + i);
        }
        st.tables = st_tables;
    }
    // The op stream is read by every thread at every op; keep it in shared memory when it is small.
    st.ops = p.ops;
    if (p.smem_ops) {
        DevOp *so = reinterpret_cast<DevOp *>(st_tables + ((p.smem_table_words + 3) & ~3u));
        const uint4 *src = reinterpret_cast<const uint4 *>(p.ops);
        uint4 *dst = reinterpret_cast<uint4 *>(so);
        for (uint32_t i = tid; i < p.smem_ops * (sizeof(DevOp) / sizeof(uint4)); i += nt) {
            dst[i] = __ldg(src + i);
        }
        st.ops = so;
    }
    st.occ_off = st.occ_cnt = nullptr;
    if (p.smem_occ) {
        uint32_t *oo = reinterpret_cast<uint32_t *>(st_tables + ((p.smem_table_words + 3) & ~3u)) +
                       (size_t)p.smem_ops * (sizeof(DevOp) / sizeof(uint32_t));
        for (uint32_t i = tid; i < p.smem_occ; i += nt) {
            oo[i] = __ldg(&p.occs[i].off);
        }
        st.occ_off = oo;
        st.occ_cnt = oo + p.smem_occ;
    }
    return st;
}

// ------------------------------------------------------------------------------------------------
// Compact unit lists (DevOp.g).  A thread owns the items i = tid + j * nt (item = unit * B + block) and
// first loads the list entries of up to J of them together, so an op costs one load latency per thread
// instead of one (or three, for detectors) per unit.
// ------------------------------------------------------------------------------------------------
template <int B, int J, bool HALF>
__device__ __forceinline__ void load_entries(const uint32_t *list, uint32_t items, uint32_t i0, uint32_t nt,
                                             uint32_t (&w)[J]) {
#pragma unroll
    for (int j = 0; j < J; j++) {
        const uint32_t i = i0 + (uint32_t)j * nt;
        if (HALF) {
            w[j] = i < items ? (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(list) + i / B) : 0u;
        } else {
            w[j] = i < items ? __ldg(list + i / B) : 0u;
        }
    }
}

// f(unit, block, entry) for every item of this thread.
template <int B, int J, bool HALF, typename F>
__device__ __forceinline__ void for_items(const uint32_t *list, uint32_t items, uint32_t tid, uint32_t nt, F f) {
    for (uint32_t i0 = tid; i0 < items; i0 += (uint32_t)J * nt) {
        uint32_t w[J];
        load_entries<B, J, HALF>(list, items, i0, nt, w);
#pragma unroll
        for (int j = 0; j < J; j++) {
            const uint32_t i = i0 + (uint32_t)j * nt;
            if (i < items) {
                f(i / B, i % B, w[j]);
            }
        }
    }
}

// CX / CZ over a compact pair list, two pairs at a time so that both pairs' loads are in flight together
// (the pairs of one op touch distinct rows, which the compiler cannot know).
template <int B>
__device__ __forceinline__ void cx_cz_compact(const uint32_t *list, bool cz, uint32_t items, uint4 *X, uint4 *Z,
                                              uint32_t tid, uint32_t nt) {
    constexpr int J = 4;
    for (uint32_t i0 = tid; i0 < items; i0 += (uint32_t)J * nt) {
        uint32_t w[J];
        load_entries<B, J, false>(list, items, i0, nt, w);
#pragma unroll
        for (int j = 0; j < J; j += 2) {
            const uint32_t ia = i0 + (uint32_t)j * nt, ib = ia + nt;
            if (ia < items) {
                const bool two = ib < items;
                const uint32_t ba = ia % B, bb = ib % B;
                const uint32_t a1 = (w[j] & 0xFFFFu) * B + ba, a2 = (w[j] >> 16) * B + ba;
                const uint32_t b1 = (w[j + 1] & 0xFFFFu) * B + bb, b2 = (w[j + 1] >> 16) * B + bb;
                if (!cz) {
                    const uint4 az1 = Z[a1], az2 = Z[a2], ax1 = X[a1], ax2 = X[a2];
                    const uint4 bz1 = Z[b1], bz2 = Z[b2], bx1 = X[b1], bx2 = X[b2];
                    Z[a1] = x4(az1, az2);
                    X[a2] = x4(ax2, ax1);
                    if (two) {
                        Z[b1] = x4(bz1, bz2);
                        X[b2] = x4(bx2, bx1);
                    }
                } else {
                    const uint4 az1 = Z[a1], az2 = Z[a2], ax1 = X[a1], ax2 = X[a2];
                    const uint4 bz1 = Z[b1], bz2 = Z[b2], bx1 = X[b1], bx2 = X[b2];
                    Z[a1] = x4(az1, ax2);
                    Z[a2] = x4(az2, ax1);
                    if (two) {
                        Z[b1] = x4(bz1, bx2);
                        Z[b2] = x4(bz2, bx1);
                    }
                }
            }
        }
    }
}

// Detectors over a compact lookback list: each reads at most two records; the records of four detectors are
// loaded before any result is stored.
template <int B>
__device__ __forceinline__ void detectors_compact(const uint32_t *list, uint32_t items, const uint4 *R, uint32_t rec,
                                                  uint32_t L, bool rg, uint4 *out, uint64_t ndet, uint64_t lb0,
                                                  uint64_t det_base, uint32_t tid, uint32_t nt) {
    constexpr int J = 4;
    for (uint32_t i0 = tid; i0 < items; i0 += (uint32_t)J * nt) {
        uint32_t w[J];
        load_entries<B, J, false>(list, items, i0, nt, w);
        uint4 acc[J];
#pragma unroll
        for (int j = 0; j < J; j++) {
            const uint32_t i = i0 + (uint32_t)j * nt;
            const uint32_t blk = i % B, k1 = w[j] & 0xFFFFu, k2 = w[j] >> 16;
            acc[j] = zero4();
            if (i < items && k1) {
                acc[j] = ring_ld(R, wrap(rec + L - k1, L) * B + blk, rg);
            }
            if (i < items && k2) {
                acc[j] = x4(acc[j], ring_ld(R, wrap(rec + L - k2, L) * B + blk, rg));
            }
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
            const uint32_t i = i0 + (uint32_t)j * nt;
            if (i < items) {
                out[(lb0 + i % B) * ndet + det_base + i / B] = acc[j];
            }
        }
    }
}

// Samples slice `slice` (blocks slice*B .. slice*B+B-1 of this launch) of circuit `p` from the start of
// the circuit to its end, leaving detection events, observables and measurements in global memory.
template <int B, bool HITS>
__device__ __forceinline__ void frame_slice(const KernelArgs &p, const FrameState &st, uint32_t slice) {
    const uint32_t nr = p.nrows, L = p.ring, NO = p.nobs;
    uint4 *const X = st.X, *const Z = st.Z, *const R = st.R, *const O = st.O, *const OCC = st.OCC,
               *const MSK = st.MSK;
    const uint32_t *const tables = st.tables;
    const DevOp *const ops = st.ops;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t *pool = p.pool;
    const uint64_t lb0 = (uint64_t)slice * B;
    const uint64_t gb0 = p.block0 + lb0;

    for (uint32_t i = tid; i < nr * B; i += nt) {
        uint32_t r = i / B, blk = i % B;
        X[i] = zero4();
        Z[i] = p.reset_zero ? zero4()
                            : u4(gfs_row_bits(p.seed, GFS_P_RESET, 0, __ldg(p.qubit_orig + r), (uint32_t)(gb0 + blk)));
    }
    for (uint32_t i = tid; i < NO * B; i += nt) {
        O[i] = zero4();
    }
    for (uint32_t i = tid; i < B; i += nt) {
        OCC[i] = zero4();
    }
    if (HITS && st.occ_cnt) {
        const uint32_t *cnt = p.hit_count + (uint64_t)slice * p.n_occ;
        for (uint32_t i = tid; i < p.smem_occ; i += nt) {
            st.occ_cnt[i] = __ldg(cnt + i);
        }
    }
    __syncthreads();
    if (HITS && tid == 0) {
        prefetch_occurrence(p, st.occ_off, st.occ_cnt, slice, 0);
        prefetch_occurrence(p, st.occ_off, st.occ_cnt, slice, 1);
    }
    HitPre pre;
    pre.r0 = pre.r1 = 0;
    if (HITS) {
        hit_prefetch(p, st.occ_off, st.occ_cnt, slice, 0, tid, nt, pre);
    }

    uint32_t rec = 0, occ = 0;
    uint64_t det_base = 0, meas_base = 0, inst_base = 0;
    int depth = 0;
    // The two outermost REPEAT levels keep their state in registers; deeper ones in local arrays.
    uint32_t lpc0 = 0, lpc1 = 0;
    uint64_t left0 = 0, left1 = 0, base0 = 0, base1 = 0, stride0 = 0, stride1 = 0;
    uint32_t loop_pc[kMaxLoopDepth + 1];
    uint64_t loop_left[kMaxLoopDepth + 1], loop_base[kMaxLoopDepth + 1], loop_stride[kMaxLoopDepth + 1];
    uint32_t pc = 0;

    for (;;) {
        const DevOp op = ops[pc];
        const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
        const uint64_t inst = inst_base + op.inst;
        const uint32_t n = op.n, a = op.a;
        if (code == OP_END) {
            break;
        }
        if (code == OP_LOOP_BEGIN) {
            if (depth >= kMaxLoopDepth) {
                if (tid == 0) {
                    atomicOr(p.status, 1u);
                }
                break;
            }
            const uint64_t reps = (uint64_t)op.a | ((uint64_t)op.b << 32);
            const uint64_t stride = (uint64_t)op.c | ((uint64_t)op.d << 32);
            if (depth == 0) {
                lpc0 = pc;
                left0 = reps;
                base0 = inst_base;
                stride0 = stride;
            } else if (depth == 1) {
                lpc1 = pc;
                left1 = reps;
                base1 = inst_base;
                stride1 = stride;
            } else {
                loop_pc[depth] = pc;
                loop_left[depth] = reps;
                loop_base[depth] = inst_base;
                loop_stride[depth] = stride;
            }
            depth++;
            inst_base = inst;
            pc++;
            continue;
        }
        if (code == OP_LOOP_END) {
            const int d = depth - 1;
            uint64_t left, stride, base;
            uint32_t lpc;
            if (d == 0) {
                left = --left0;
                stride = stride0;
                base = base0;
                lpc = lpc0;
            } else if (d == 1) {
                left = --left1;
                stride = stride1;
                base = base1;
                lpc = lpc1;
            } else {
                left = --loop_left[d];
                stride = loop_stride[d];
                base = loop_base[d];
                lpc = loop_pc[d];
            }
            if (left > 0) {
                inst_base += stride;
                pc = lpc + 1;
            } else {
                inst_base = base;
                depth = d;
                pc++;
            }
            continue;
        }

        const bool gate = code == OP_1Q || code == OP_2Q || code == OP_MEASURE || code == OP_RESET;
        if (!HITS && gate && (op.c | op.d)) {
            fused_gate<B>(p, op, code, sub, inst, gb0, tables, X, Z, R, rec, L, tid, nt);
            if (code == OP_MEASURE) {
                rec = wrap(rec + n, L);
            }
            __syncthreads();
            pc++;
            continue;
        }
        if (HITS && gate && (op.d & kFusedChanMask)) {  // noise before the gate
            apply_hits<B>(p, st, slice, occ++, OCC_PAULI, X, Z, R, MSK, rec, L, n, tid, nt, pre);
            __syncthreads();
        }

        // Gate units in bank-friendly order (a second list when the op carries fused noise).
        const uint32_t ga = (op.code & kGateOrderInB) ? op.b : a;
        const bool compact = (op.code & kCompact) != 0;
        const bool norand = (op.code & kNoRandomize) != 0;
        const bool rg = p.ring_global != nullptr;
        const uint32_t *const glist = pool + op.g;
        switch (code) {
            case OP_1Q:
                if (compact) {
                    for_items<B, 4, true>(glist, n * B, tid, nt, [&](uint32_t, uint32_t blk, uint32_t row) {
                        const uint32_t idx = row * B + blk;
                        uint4 x = X[idx], z = Z[idx];
                        rule1(sub, x, z);
                        X[idx] = x;
                        Z[idx] = z;
                    });
                    break;
                }
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t idx = __ldg(pool + ga + u) * B + blk;
                    uint4 x = X[idx], z = Z[idx];
                    switch (sub) {
                        case K1_H_XZ:
                            X[idx] = z;
                            Z[idx] = x;
                            break;
                        case K1_H_XY:
                            Z[idx] = x4(z, x);
                            break;
                        case K1_H_YZ:
                            X[idx] = x4(x, z);
                            break;
                        default:
                            rule1(sub, x, z);
                            X[idx] = x;
                            Z[idx] = z;
                            break;
                    }
                }
                break;

            case OP_2Q:
                if (compact) {
                    if (sub == K2_CX || sub == K2_CZ) {
                        cx_cz_compact<B>(glist, sub == K2_CZ, n * B, X, Z, tid, nt);
                        break;
                    }
                    for_items<B, 4, false>(glist, n * B, tid, nt, [&](uint32_t, uint32_t blk, uint32_t w) {
                        const uint32_t i1 = (w & 0xFFFFu) * B + blk, i2 = (w >> 16) * B + blk;
                        uint4 x1 = X[i1], z1 = Z[i1], x2 = X[i2], z2 = Z[i2];
                        rule2v(sub, x1, z1, x2, z2);
                        X[i1] = x1;
                        Z[i1] = z1;
                        X[i2] = x2;
                        Z[i2] = z2;
                    });
                    break;
                }
                if (sub == K2_CX || sub == K2_CZ) {
                    // Two independent pairs per iteration: both pairs' loads are in flight together.
                    const uint32_t items = n * B;
                    for (uint32_t i = tid; i < items; i += 2 * nt) {
                        const uint32_t i2b = i + nt;
                        const bool two = i2b < items;
                        const uint32_t ua = i / B, ba = i % B;
                        const uint32_t ub = two ? i2b / B : ua, bb = two ? i2b % B : ba;
                        const uint32_t a1 = __ldg(pool + ga + 2 * ua) * B + ba, a2 = __ldg(pool + ga + 2 * ua + 1) * B + ba;
                        const uint32_t b1 = __ldg(pool + ga + 2 * ub) * B + bb, b2 = __ldg(pool + ga + 2 * ub + 1) * B + bb;
                        uint4 az1 = Z[a1], az2 = Z[a2], ax1 = X[a1], ax2 = X[a2];
                        uint4 bz1 = Z[b1], bz2 = Z[b2], bx1 = X[b1], bx2 = X[b2];
                        if (sub == K2_CX) {
                            Z[a1] = x4(az1, az2);
                            X[a2] = x4(ax2, ax1);
                            if (two) {
                                Z[b1] = x4(bz1, bz2);
                                X[b2] = x4(bx2, bx1);
                            }
                        } else {
                            Z[a1] = x4(az1, ax2);
                            Z[a2] = x4(az2, ax1);
                            if (two) {
                                Z[b1] = x4(bz1, bx2);
                                Z[b2] = x4(bz2, bx1);
                            }
                        }
                    }
                    break;
                }
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t i1 = __ldg(pool + ga + 2 * u) * B + blk;
                    uint32_t i2 = __ldg(pool + ga + 2 * u + 1) * B + blk;
                    uint4 x1 = X[i1], z1 = Z[i1], x2 = X[i2], z2 = Z[i2];
                    rule2v(sub, x1, z1, x2, z2);
                    X[i1] = x1;
                    Z[i1] = z1;
                    X[i2] = x2;
                    Z[i2] = z2;
                }
                break;

            case OP_FEEDBACK:
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t k = __ldg(pool + a + 2 * u);
                    uint32_t rm = __ldg(pool + a + 2 * u + 1);
                    uint32_t idx = (rm & kRowMask) * B + blk;
                    uint4 v;
                    if (k & kFeedbackSweep) {  // sweep bit (k & ~kFeedbackSweep) < nsweep, checked by the host
                        v = p.sweep ? p.sweep[(lb0 + blk) * p.nsweep + (k & ~kFeedbackSweep)] : zero4();
                    } else {
                        v = ring_ld(R, wrap(rec + L - k, L) * B + blk, rg);
                    }
                    if ((rm >> 24) & kFeedbackX) {
                        X[idx] = x4(X[idx], v);
                    }
                    if ((rm >> 24) & kFeedbackZ) {
                        Z[idx] = x4(Z[idx], v);
                    }
                }
                break;

            case OP_MEASURE:
                if (compact) {
                    for_items<B, 4, true>(glist, n * B, tid, nt, [&](uint32_t u, uint32_t blk, uint32_t row) {
                        measure_row(sub, X, Z, R, row * B + blk, wrap(rec + u, L) * B + blk,
                                    rand_row(p, norand, inst, op.b + u, (uint32_t)(gb0 + blk)), rg, norand);
                    });
                } else {
                    for (uint32_t i = tid; i < n * B; i += nt) {
                        const uint32_t u = i / B, blk = i % B;
                        measure_row(sub, X, Z, R, __ldg(pool + a + u) * B + blk, wrap(rec + u, L) * B + blk,
                                    rand_row(p, norand, inst, op.b + u, (uint32_t)(gb0 + blk)), rg, norand);
                    }
                }
                rec = wrap(rec + n, L);
                break;

            case OP_RESET: {
                auto reset_unit = [&](uint32_t u, uint32_t blk, uint32_t row) {
                    reset_row(sub, X, Z, row * B + blk, rand_row(p, norand, inst, op.b + u, (uint32_t)(gb0 + blk)),
                              norand);
                };
                if (compact) {
                    for_items<B, 4, true>(glist, n * B, tid, nt, reset_unit);
                } else {
                    for (uint32_t i = tid; i < n * B; i += nt) {
                        reset_unit(i / B, i % B, __ldg(pool + a + i / B));
                    }
                }
                break;
            }

            case OP_RECORD_ZERO:
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    ring_st(R, wrap(rec + u, L) * B + blk, zero4(), rg);
                }
                rec = wrap(rec + n, L);
                break;

            case OP_NOISE:
            case OP_MNOISE: {
                if (HITS) {
                    apply_hits<B>(p, st, slice, occ++, code == OP_MNOISE ? OCC_FLIP : OCC_PAULI, X, Z, R, MSK, rec, L, n,
                                  tid, nt, pre);
                    break;
                }
                // Standalone noise: one segment per lane; rows may repeat within an instruction, so hits
                // are applied with shared atomics.
                const bool meas = code == OP_MNOISE;
                const DevChan &ch = p.chans[op.b];
                const uint32_t *T = tables + ch.table;
                const bool pair = !meas && (sub == KN_DEP2 || sub == KN_PC2);
                const uint32_t kind = meas ? (uint32_t)KN_FLIP : sub;
                const uint32_t nseg = (n + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
                for (uint32_t item = tid; item < nseg * B; item += nt) {
                    const uint32_t g = item / B, blk = item % B;
                    const uint32_t u0 = g * GFS_SEG_UNITS;
                    walk_segment(ch, T, p.seed, meas ? GFS_P_MNOISE : GFS_P_NOISE, inst, g, (uint32_t)(gb0 + blk),
                                 min(GFS_SEG_UNITS, n - u0), [&](uint32_t k, uint32_t shot, gfs_stream *st) {
                                     const uint32_t u = u0 + k;
                                     if (meas) {
                                         flip_bit(R, wrap(rec + L - n + u, L) * B + blk, shot, true);
                                         return;
                                     }
                                     const uint32_t bits = hit_bits(kind, ch, st);
                                     const uint32_t i1 = __ldg(pool + a + (pair ? 2 * u : u)) * B + blk;
                                     const uint32_t i2 = pair ? __ldg(pool + a + 2 * u + 1) * B + blk : i1;
                                     apply_bits(X, Z, i1, i2, shot, bits, true);
                                 });
                }
                break;
            }

            case OP_HERALD: {
                if (HITS) {
                    apply_hits<B>(p, st, slice, occ++, OCC_HERALD, X, Z, R, MSK, rec, L, n, tid, nt, pre);
                    break;
                }
                const DevChan &ch = p.chans[op.b];
                const uint32_t *T = tables + ch.table;
                const uint32_t nseg = (n + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
                for (uint32_t item = tid; item < nseg * B; item += nt) {
                    const uint32_t g = item / B, blk = item % B;
                    const uint32_t u0 = g * GFS_SEG_UNITS;
                    walk_segment(ch, T, p.seed, GFS_P_NOISE, inst, g, (uint32_t)(gb0 + blk),
                                 min(GFS_SEG_UNITS, n - u0), [&](uint32_t k, uint32_t shot, gfs_stream *st) {
                                     const uint32_t u = u0 + k;
                                     const uint32_t c = gfs_stream_next(st);
                                     const uint32_t idx = __ldg(pool + a + u) * B + blk;
                                     atomic_or_bit(R, wrap(rec + L - n + u, L) * B + blk, shot);
                                     const uint32_t v =
                                         sub == 0 ? (c & 3u) : pauli_xz(gfs_choice_weighted(c, ch.cum, 4));
                                     apply_bits(X, Z, idx, idx, shot, v, true);
                                 });
                }
                break;
            }

            case OP_CORR_MASK: {
                if (HITS) {
                    for (uint32_t blk = tid; blk < (uint32_t)B; blk += nt) {
                        MSK[blk] = zero4();
                    }
                    __syncthreads();
                    apply_hits<B>(p, st, slice, occ++, OCC_CORR, X, Z, R, MSK, rec, L, n, tid, nt, pre);
                    __syncthreads();
                    for (uint32_t blk = tid; blk < (uint32_t)B; blk += nt) {
                        const uint4 hits = MSK[blk];
                        const uint4 oc = sub == 0 ? zero4() : OCC[blk];
                        const uint4 mk = make_uint4(hits.x & ~oc.x, hits.y & ~oc.y, hits.z & ~oc.z, hits.w & ~oc.w);
                        OCC[blk] = make_uint4(oc.x | mk.x, oc.y | mk.y, oc.z | mk.z, oc.w | mk.w);
                        MSK[blk] = mk;
                    }
                    break;
                }
                const DevChan &ch = p.chans[op.b];
                for (uint32_t blk = tid; blk < (uint32_t)B; blk += nt) {
                    uint32_t hw[4] = {0, 0, 0, 0};
                    if (ch.active) {
                        walk_segment(ch, tables + ch.table, p.seed, GFS_P_NOISE, inst, 0, (uint32_t)(gb0 + blk), 1,
                                     [&](uint32_t, uint32_t shot, gfs_stream *) {
                                         hw[shot >> 5] |= 1u << (shot & 31);
                                     });
                    }
                    const uint4 hits = make_uint4(hw[0], hw[1], hw[2], hw[3]);
                    uint4 occ = sub == 0 ? zero4() : OCC[blk];
                    uint4 mk = make_uint4(hits.x & ~occ.x, hits.y & ~occ.y, hits.z & ~occ.z, hits.w & ~occ.w);
                    OCC[blk] = make_uint4(occ.x | mk.x, occ.y | mk.y, occ.z | mk.z, occ.w | mk.w);
                    MSK[blk] = mk;
                }
                break;
            }

            case OP_CORR_APPLY:
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t rm = __ldg(pool + a + u);
                    uint32_t idx = (rm & kRowMask) * B + blk;
                    uint4 mk = MSK[blk];
                    if ((rm >> 24) & 1) {
                        X[idx] = x4(X[idx], mk);
                    }
                    if ((rm >> 24) & 2) {
                        Z[idx] = x4(Z[idx], mk);
                    }
                }
                break;

            case OP_DETECTORS:
                if (compact) {
                    detectors_compact<B>(glist, n * B, R, rec, L, rg, p.det_out, p.ndet, lb0, det_base, tid, nt);
                    det_base += n;
                    break;
                }
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t s = __ldg(pool + a + u), e = __ldg(pool + a + u + 1);
                    uint4 acc = zero4();
                    for (uint32_t j = s; j < e; j++) {
                        uint32_t k = __ldg(pool + j);
                        acc = x4(acc, ring_ld(R, wrap(rec + L - k, L) * B + blk, rg));
                    }
                    p.det_out[(lb0 + blk) * p.ndet + det_base + u] = acc;
                }
                det_base += n;
                break;

            case OP_OBS:
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    uint32_t t = __ldg(pool + a + u);
                    uint4 v;
                    if (t & kTermRecord) {
                        v = ring_ld(R, wrap(rec + L - (t & kRowMask), L) * B + blk, rg);
                    } else {
                        uint32_t idx = (t & kRowMask) * B + blk;
                        v = zero4();
                        if (t & kTermX) {
                            v = x4(v, Z[idx]);
                        }
                        if (t & kTermZ) {
                            v = x4(v, X[idx]);
                        }
                    }
                    atomic_xor4(O, op.b * B + blk, v);
                }
                break;

            case OP_EMIT:
                for (uint32_t i = tid; i < n * B; i += nt) {
                    uint32_t u = i / B, blk = i % B;
                    p.meas_out[(lb0 + blk) * p.nmeas + meas_base + u] = ring_ld(R, wrap(rec + L - n + u, L) * B + blk, rg);
                }
                meas_base += n;
                break;

            default:
                if (tid == 0) {
                    atomicOr(p.status, 2u);
                }
                break;
        }
        if (HITS && gate && (op.c & kFusedChanMask)) {  // noise after the gate
            __syncthreads();
            apply_hits<B>(p, st, slice, occ++, OCC_PAULI, X, Z, R, MSK, rec, L, n, tid, nt, pre);
        }
        __syncthreads();
        pc++;
    }

    for (uint32_t i = tid; i < NO * B; i += nt) {
        uint32_t k = i / B, blk = i % B;
        p.obs_out[(lb0 + blk) * NO + k] = O[i];
    }
    __syncthreads();
}

// Register budget: 96 a thread keeps five 128-thread CTAs resident per SM (the usual shared-memory limit
// at large circuits) without spilling to local memory.
template <int B, bool HITS>
__global__ void __maxnreg__(96) frame_kernel(const KernelArgs p) {
    extern __shared__ uint4 sm[];
    const FrameState st = frame_state<B>(p, sm);
    for (uint32_t slice = blockIdx.x; slice < p.nslices; slice += gridDim.x) {
        frame_slice<B, HITS>(p, st, slice);
    }
}

// The same with the X / Z frames in a per-CTA global region (one block per CTA): circuits whose frames do not
// fit in shared memory.  Frame accesses go through L1 / L2; everything else is as in frame_kernel.
template <bool HITS>
__global__ void __maxnreg__(96) frame_kernel_global(const KernelArgs p) {
    extern __shared__ uint4 sm[];
    const FrameState st = frame_state<1>(p, sm, true);
    for (uint32_t slice = blockIdx.x; slice < p.nslices; slice += gridDim.x) {
        frame_slice<1, HITS>(p, st, slice);
    }
}

// Many circuits in one persistent launch: work items are (circuit, slice) pairs numbered circuit by
// circuit (b.slice_prefix[j] = first item of circuit j); CTAs claim items from a global counter, so
// expensive and cheap circuits balance across the SMs.  A CTA reloads the circuit's descriptor, gap tables
// and op stream only when its next item belongs to another circuit.
template <int B, bool HITS>
__global__ void __maxnreg__(96) batch_frame_kernel(const BatchArgs b) {
    extern __shared__ uint4 sm[];
    __shared__ KernelArgs cur;
    __shared__ uint32_t s_item, s_circ;
    uint32_t have = 0xFFFFFFFFu;
    FrameState st{};
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t item = atomicAdd(b.counter, 1u);
            s_item = item;
            if (item < b.total_slices) {
                uint32_t lo = 0, hi = b.ncircuits;  // last j with slice_prefix[j] <= item
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) / 2;
                    if (b.slice_prefix[mid] <= item) {
                        lo = mid;
                    } else {
                        hi = mid;
                    }
                }
                s_circ = lo;
                if (lo != have) {
                    cur = b.circuits[lo];
                }
            }
        }
        __syncthreads();
        const uint32_t item = s_item, j = s_circ;
        if (item >= b.total_slices) {
            break;
        }
        if (j != have) {
            st = frame_state<B>(cur, sm);
            have = j;
        }
        frame_slice<B, HITS>(cur, st, item - b.slice_prefix[j]);
    }
}

size_t frame_smem_bytes(uint32_t nrows, uint32_t ring, uint32_t nobs, int blocks_per_cta, uint32_t table_words,
                        uint32_t smem_ops, uint32_t smem_occ) {
    // `ring` = measurement-ring rows held in shared memory (0 when the ring is in global memory).
    return ((size_t)2 * nrows + ring + nobs + 2) * (size_t)blocks_per_cta * sizeof(uint4) +
           (size_t)((table_words + 3) & ~3u) * sizeof(uint32_t) + (size_t)smem_ops * sizeof(DevOp) +
           (size_t)2 * smem_occ * sizeof(uint32_t);
}

template <int B, bool H>
static cudaError_t launch_b(const KernelArgs &args, const LaunchShape &s, cudaStream_t stream) {
    cudaError_t e =
        cudaFuncSetAttribute(frame_kernel<B, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    frame_kernel<B, H><<<s.grid, s.threads, s.smem, stream>>>(args);
    return cudaGetLastError();
}

template <bool H>
static cudaError_t launch_global_frames(const KernelArgs &args, const LaunchShape &s, cudaStream_t stream) {
    cudaError_t e =
        cudaFuncSetAttribute(frame_kernel_global<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    frame_kernel_global<H><<<s.grid, s.threads, s.smem, stream>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_frame_kernel(const KernelArgs &args, const LaunchShape &shape, cudaStream_t stream) {
    const bool h = args.hits != nullptr;
    if (h != shape.hits) {
        return cudaErrorInvalidValue;
    }
    if (shape.frames_global) {
        if (shape.blocks_per_cta != 1 || !args.frames_global) {
            return cudaErrorInvalidValue;
        }
        return h ? launch_global_frames<true>(args, shape, stream) : launch_global_frames<false>(args, shape, stream);
    }
    switch (shape.blocks_per_cta) {
        case 1:
            return h ? launch_b<1, true>(args, shape, stream) : launch_b<1, false>(args, shape, stream);
        case 2:
            return h ? launch_b<2, true>(args, shape, stream) : launch_b<2, false>(args, shape, stream);
        case 4:
            return h ? launch_b<4, true>(args, shape, stream) : launch_b<4, false>(args, shape, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

template <int B>
static cudaError_t launch_noise_b(const KernelArgs &args, cudaStream_t stream) {
    constexpr int SB = noise_slices_per_warp<B>();
    const uint64_t warps = (uint64_t)((args.nslices + SB - 1) / SB) * args.n_occ;
    const uint64_t blocks = (warps + 7) / 8;
    if (blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    noise_kernel<B><<<(unsigned)blocks, 256, 0, stream>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_noise_kernel(const KernelArgs &args, int blocks_per_cta, cudaStream_t stream) {
    if (!args.hits || !args.hit_count || !args.occs || args.n_occ == 0) {
        return cudaErrorInvalidValue;
    }
    switch (blocks_per_cta) {
        case 1:
            return launch_noise_b<1>(args, stream);
        case 2:
            return launch_noise_b<2>(args, stream);
        case 4:
            return launch_noise_b<4>(args, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

template <int B, bool H>
static cudaError_t launch_batch_b(const BatchArgs &args, const LaunchShape &s, cudaStream_t stream) {
    cudaError_t e = cudaFuncSetAttribute(batch_frame_kernel<B, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    if (H) {
        const uint64_t blocks = (args.total_noise_warps + 7) / 8;
        if (blocks > 0x7FFFFFFFull) {
            return cudaErrorInvalidValue;
        }
        if (blocks) {
            batch_noise_kernel<B><<<(unsigned)blocks, 256, 0, stream>>>(args);
            e = cudaGetLastError();
            if (e != cudaSuccess) {
                return e;
            }
        }
    }
    batch_frame_kernel<B, H><<<s.grid, s.threads, s.smem, stream>>>(args);
    return cudaGetLastError();
}

template <int B>
static cudaError_t launch_batch_noise_b(const BatchArgs &args, cudaStream_t stream) {
    const uint64_t blocks = (args.total_noise_warps + 7) / 8;
    if (blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    if (blocks) {
        batch_noise_kernel<B><<<(unsigned)blocks, 256, 0, stream>>>(args);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

cudaError_t launch_batch_noise_kernel(const BatchArgs &args, int blocks_per_cta, cudaStream_t stream) {
    switch (blocks_per_cta) {
        case 1:
            return launch_batch_noise_b<1>(args, stream);
        case 2:
            return launch_batch_noise_b<2>(args, stream);
        case 4:
            return launch_batch_noise_b<4>(args, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_frame_kernel(const BatchArgs &args, const LaunchShape &shape, cudaStream_t stream) {
    const bool h = shape.hits;
    switch (shape.blocks_per_cta) {
        case 1:
            return h ? launch_batch_b<1, true>(args, shape, stream) : launch_batch_b<1, false>(args, shape, stream);
        case 2:
            return h ? launch_batch_b<2, true>(args, shape, stream) : launch_batch_b<2, false>(args, shape, stream);
        case 4:
            return h ? launch_batch_b<4, true>(args, shape, stream) : launch_batch_b<4, false>(args, shape, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

template <int B, bool H>
static cudaError_t occ_batch_b(const LaunchShape &s, int *out) {
    cudaError_t e = cudaFuncSetAttribute(batch_frame_kernel<B, H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, batch_frame_kernel<B, H>, s.threads, s.smem);
}

cudaError_t batch_frame_kernel_max_ctas_per_sm(const LaunchShape &shape, int *out) {
    const bool h = shape.hits;
    switch (shape.blocks_per_cta) {
        case 1:
            return h ? occ_batch_b<1, true>(shape, out) : occ_batch_b<1, false>(shape, out);
        case 2:
            return h ? occ_batch_b<2, true>(shape, out) : occ_batch_b<2, false>(shape, out);
        case 4:
            return h ? occ_batch_b<4, true>(shape, out) : occ_batch_b<4, false>(shape, out);
        default:
            return cudaErrorInvalidValue;
    }
}

template <int B, bool H>
static cudaError_t occ_b(const LaunchShape &s, int *out) {
    cudaError_t e =
        cudaFuncSetAttribute(frame_kernel<B, H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, frame_kernel<B, H>, s.threads, s.smem);
}

template <bool H>
static cudaError_t occ_global_frames(const LaunchShape &s, int *out) {
    cudaError_t e =
        cudaFuncSetAttribute(frame_kernel_global<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, frame_kernel_global<H>, s.threads, s.smem);
}

cudaError_t frame_kernel_max_ctas_per_sm(const LaunchShape &shape, int *out) {
    const bool h = shape.hits;
    if (shape.frames_global) {
        if (shape.blocks_per_cta != 1) {
            return cudaErrorInvalidValue;
        }
        return h ? occ_global_frames<true>(shape, out) : occ_global_frames<false>(shape, out);
    }
    switch (shape.blocks_per_cta) {
        case 1:
            return h ? occ_b<1, true>(shape, out) : occ_b<1, false>(shape, out);
        case 2:
            return h ? occ_b<2, true>(shape, out) : occ_b<2, false>(shape, out);
        case 4:
            return h ? occ_b<4, true>(shape, out) : occ_b<4, false>(shape, out);
        default:
            return cudaErrorInvalidValue;
    }
}

// Shot-major output, tiled: a CTA of 256 threads owns (one 128-shot block, 1024 concatenated rows).
// Phase 1: each warp loads 4 groups of 32 rows (one uint4 = 128 shots per row) and turns every 32x32 bit
// block around with a five-stage shuffle butterfly (recursive exchange of off-diagonal sub-blocks), leaving
// lane l with 32 rows of shot 32w + l; the words are staged in shared memory as [shot][32 words].
// Phase 2: each warp writes whole shot rows of the tile (128 bytes bit-packed, 1024 bytes unpacked) with
// coalesced 4-byte stores; a destination that is not 4-byte aligned is written as aligned words assembled
// with funnel shifts, and only the two partial words at the ends use byte stores.
__device__ __forceinline__ uint4 load_concat(const TransposeArgs &t, uint64_t blk, uint64_t r, uint64_t total) {
    uint4 v = zero4();
    if (r < t.n0) {
        v = t.src0[blk * t.n0 + r];
    } else if (r < t.n0 + t.n1) {
        v = t.src1[blk * t.n1 + (r - t.n0)];
    } else if (r < total) {
        v = t.src2[blk * t.n2 + (r - t.n0 - t.n1)];
    }
    if (t.xor_rows && r < total && ((t.xor_rows[r >> 3] >> (r & 7)) & 1)) {
        v = x4(v, make_uint4(~0u, ~0u, ~0u, ~0u));
    }
    return v;
}

// Lane r holds row r of a 32x32 bit matrix (bit c = column c); afterwards lane c holds column c.  Stage s
// (16, 8, 4, 2, 1) swaps the off-diagonal s x s sub-blocks between lanes l and l^s: the partner's word is
// rotated by s toward the bits this lane takes (left when lane bit s is clear, right when set) and merged
// under this lane's mask.  keep[k] / rot[k] depend only on the lane, so a stage is a shuffle, a funnel
// shift and one bitwise select.
struct Transpose32 {
    uint32_t keep[5], rot[5];
    __device__ __forceinline__ explicit Transpose32(uint32_t lane) {
        const uint32_t lo[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const uint32_t s = 16u >> k;
            const bool hi = (lane & s) != 0;
            keep[k] = hi ? ~lo[k] : lo[k];
            rot[k] = hi ? 32u - s : s;
        }
    }
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const {
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const uint32_t y = __shfl_xor_sync(0xFFFFFFFFu, x, 16u >> k);
            const uint32_t r = __funnelshift_l(y, y, rot[k]);
            x = (x & keep[k]) | (r & ~keep[k]);
        }
        return x;
    }
};

constexpr uint32_t kTileRows = 1024, kTileWords = kTileRows / 32;

// Word j of a shot's output chunk: the packed bits themselves, or four 0/1 bytes per nibble unpacked.
__device__ __forceinline__ uint32_t chunk_word(const uint32_t *row, int32_t j, int packed) {
    if (packed) {
        return row[j];
    }
    const uint32_t v = (row[j >> 3] >> (4 * (j & 7))) & 0xFu;
    return (v & 1u) | ((v >> 1) & 1u) << 8 | ((v >> 2) & 1u) << 16 | ((v >> 3) & 1u) << 24;
}

// Half-word j of a shot's output chunk (2-byte aligned destinations): packed bits, or two 0/1 bytes.
__device__ __forceinline__ uint32_t chunk_half(const uint32_t *row, int32_t j, int packed) {
    if (packed) {
        return reinterpret_cast<const uint16_t *>(row)[j];
    }
    const uint32_t v = (row[j >> 4] >> (2 * (j & 15))) & 3u;
    return (v & 1u) | (v >> 1) << 8;
}

// kSingle: one source, no row inversion (the detector, observable and measurement outputs of the samplers),
// so a row load is one bounds test and one 16-byte load from a per-block base pointer.
template <bool kSingle>
__global__ void __launch_bounds__(256) transpose_tile_kernel(const TransposeArgs t) {
    __shared__ uint32_t tile[128][kTileWords + 1];  // [shot][32-row word], padded against bank conflicts
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Row tiles vary fastest across the grid, so the CTAs writing the pieces of the same shot rows run
    // together and the 32-byte sectors they share are completed in L2 before eviction.
    const uint64_t blk = blockIdx.y;
    const uint64_t total = t.n0 + t.n1 + t.n2;
    const uint64_t r0 = (uint64_t)blockIdx.x * kTileRows;
    const Transpose32 transpose32(lane);
    uint4 v[4];
    if (kSingle) {
        const uint4 *src = t.src0 + blk * t.n0 + r0;
        const uint32_t avail = total - r0 < kTileRows ? (uint32_t)(total - r0) : kTileRows;
#pragma unroll
        for (uint32_t g = 0; g < 4; g++) {  // all four loads in flight before the shuffles
            const uint32_t r = 128 * warp + 32 * g + lane;
            v[g] = r < avail ? src[r] : zero4();
        }
    } else {
#pragma unroll
        for (uint32_t g = 0; g < 4; g++) {
            v[g] = load_concat(t, blk, r0 + 128 * warp + 32 * g + lane, total);
        }
    }
#pragma unroll
    for (uint32_t g = 0; g < 4; g++) {
        const uint32_t words[4] = {v[g].x, v[g].y, v[g].z, v[g].w};
#pragma unroll
        for (uint32_t w = 0; w < 4; w++) {
            tile[32 * w + lane][4 * warp + g] = transpose32(words[w]);
        }
    }
    __syncthreads();
    const uint64_t rows = total - r0 < kTileRows ? total - r0 : kTileRows;
    const int packed = t.bit_packed;
    const int32_t nbytes = (int32_t)(packed ? (rows + 7) / 8 : rows);
    const uint64_t left = t.nshots - blk * 128;
    const uint32_t nvalid = left < 128 ? (uint32_t)left : 128u;
    uint8_t *const base = t.out + blk * 128 * t.out_stride + (packed ? r0 / 8 : r0);
    // One warp per shot row.  Destinations 4-byte aligned get one 4-byte word per lane, 2-byte aligned ones
    // (even row strides, e.g. ceil(detectors / 8) = 1950 bytes) one half-word per lane, others bytes, lane q
    // writing unit 32k + q so that every store instruction covers 32 consecutive units: no funnel shifts,
    // no divergent edge handling.
    if (packed && nbytes == 4 * (int32_t)kTileWords) {
        // A full bit-packed tile: 128 bytes per shot row, one store per lane per row (two or four below 4-byte
        // alignment), no inner loops.
#pragma unroll 4
        for (uint32_t s = warp; s < nvalid; s += 8) {
            const uint32_t *row = tile[s];
            uint8_t *dst = base + s * t.out_stride;
            const uint32_t mis = (uint32_t)(uintptr_t)dst & 3u;
            if (mis == 0) {
                reinterpret_cast<uint32_t *>(dst)[lane] = row[lane];
            } else if (mis == 2) {
                const uint16_t *r16 = reinterpret_cast<const uint16_t *>(row);
                uint16_t *d16 = reinterpret_cast<uint16_t *>(dst);
                d16[lane] = r16[lane];
                d16[lane + 32] = r16[lane + 32];
            } else {
                const uint8_t *rb = reinterpret_cast<const uint8_t *>(row);
#pragma unroll
                for (uint32_t k = 0; k < 4; k++) {
                    dst[lane + 32 * k] = rb[lane + 32 * k];
                }
            }
        }
        return;
    }
    for (uint32_t s = warp; s < nvalid; s += 8) {
        const uint32_t *row = tile[s];
        uint8_t *dst = base + s * t.out_stride;
        const uint32_t mis = (uint32_t)(uintptr_t)dst & 3u;
        if (mis == 0) {
            uint32_t *d32 = reinterpret_cast<uint32_t *>(dst);
            const int32_t full = nbytes / 4;
            for (int32_t q = (int32_t)lane; q < full; q += 32) {
                d32[q] = chunk_word(row, q, packed);
            }
            if ((int32_t)lane < nbytes - 4 * full) {
                const int32_t b = 4 * full + (int32_t)lane;
                dst[b] = (uint8_t)(chunk_word(row, b >> 2, packed) >> (8 * (b & 3)));
            }
        } else if (mis == 2) {
            uint16_t *d16 = reinterpret_cast<uint16_t *>(dst);
            const int32_t full = nbytes / 2;
            for (int32_t q = (int32_t)lane; q < full; q += 32) {
                d16[q] = (uint16_t)chunk_half(row, q, packed);
            }
            if (lane == 0 && (nbytes & 1)) {
                dst[nbytes - 1] = (uint8_t)chunk_half(row, full, packed);
            }
        } else if (packed) {
            const uint8_t *rb = reinterpret_cast<const uint8_t *>(row);
            for (int32_t b = (int32_t)lane; b < nbytes; b += 32) {
                dst[b] = rb[b];
            }
        } else {
            for (int32_t b = (int32_t)lane; b < nbytes; b += 32) {
                dst[b] = (uint8_t)((row[b >> 5] >> (b & 31)) & 1u);
            }
        }
    }
}

cudaError_t launch_transpose(const TransposeArgs &args, cudaStream_t stream) {
    const uint64_t total = args.n0 + args.n1 + args.n2;
    if (total == 0 || args.nshots == 0) {
        return cudaSuccess;
    }
    const uint64_t tiles = (total + kTileRows - 1) / kTileRows;
    if (tiles > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    const uint64_t nblk = (args.nshots + 127) / 128;
    const bool single = args.n1 == 0 && args.n2 == 0 && args.xor_rows == nullptr;
    const uint64_t per_launch = 65535;  // grid.y limit; larger requests are split by 128-shot block
    for (uint64_t b0 = 0; b0 < nblk; b0 += per_launch) {
        TransposeArgs t = args;
        t.src0 = args.src0 ? args.src0 + b0 * args.n0 : nullptr;
        t.src1 = args.src1 ? args.src1 + b0 * args.n1 : nullptr;
        t.src2 = args.src2 ? args.src2 + b0 * args.n2 : nullptr;
        t.out = args.out + b0 * 128 * args.out_stride;
        t.nshots = args.nshots - b0 * 128;
        const uint64_t nb = nblk - b0 < per_launch ? nblk - b0 : per_launch;
        if (single) {
            transpose_tile_kernel<true><<<dim3((unsigned)tiles, (unsigned)nb), 256, 0, stream>>>(t);
        } else {
            transpose_tile_kernel<false><<<dim3((unsigned)tiles, (unsigned)nb), 256, 0, stream>>>(t);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            return e;
        }
    }
    return cudaSuccess;
}

// ------------------------------------------------------------------------------------------------
// Measurements to detection events.  rows_from_shots_kernel is the inverse of transpose_tile_kernel: a CTA
// of 256 threads owns (one 128-shot block, 1024 measurement rows).  Phase 1 stages the 128 shots' 128-byte
// pieces of their rows in shared memory (lane q reading byte 32k + q, so any row stride and alignment
// works); phase 2 turns each 32 x 32 bit block around with the shuffle butterfly (lane = shot in, lane =
// measurement out); phase 3 writes [block][row] uint4 rows with coalesced 16-byte stores.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) rows_from_shots_kernel(const RowsInArgs a) {
    __shared__ uint32_t tin[128][kTileWords + 1];  // [shot][word of the 1024-bit piece], padded
    __shared__ uint32_t tout[kTileRows][5];        // [row][32-shot group], stride 5 words: conflict-free
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t blk = blockIdx.y;
    const uint64_t r0 = (uint64_t)blockIdx.x * kTileRows;
    const uint64_t rows = a.nbits - r0 < kTileRows ? a.nbits - r0 : kTileRows;
    const uint32_t nbytes = (uint32_t)((rows + 7) / 8);
    for (uint32_t s = warp; s < 128; s += 8) {
        const uint64_t shot = blk * 128 + s;
        const uint8_t *src = a.in + shot * a.in_stride + r0 / 8;
        uint8_t *dst = reinterpret_cast<uint8_t *>(tin[s]);
        for (uint32_t b = lane; b < 4 * kTileWords; b += 32) {
            dst[b] = (shot < a.nshots && b < nbytes) ? src[b] : (uint8_t)0;
        }
    }
    __syncthreads();
    const Transpose32 transpose32(lane);
    for (uint32_t t = warp; t < 4 * kTileWords; t += 8) {
        const uint32_t g = t / kTileWords, w = t % kTileWords;
        tout[32 * w + lane][g] = transpose32(tin[32 * g + lane][w]);
    }
    __syncthreads();
    for (uint32_t r = tid; r < rows; r += 256) {
        a.out[blk * a.nbits + r0 + r] = make_uint4(tout[r][0], tout[r][1], tout[r][2], tout[r][3]);
    }
}

cudaError_t launch_rows_from_shots(const RowsInArgs &args, cudaStream_t stream) {
    if (args.nbits == 0 || args.nshots == 0) {
        return cudaSuccess;
    }
    const uint64_t tiles = (args.nbits + kTileRows - 1) / kTileRows;
    const uint64_t nblk = (args.nshots + 127) / 128;
    if (tiles > 0x7FFFFFFFull || nblk > 65535) {
        return cudaErrorInvalidValue;
    }
    rows_from_shots_kernel<<<dim3((unsigned)tiles, (unsigned)nblk), 256, 0, stream>>>(args);
    return cudaGetLastError();
}

// One thread per (block, output row), outputs of a block consecutive so that the block's measurement rows
// stay in L2 while its outputs are folded.
__global__ void __launch_bounds__(256) m2d_fold_kernel(const FoldArgs a) {
    const uint64_t total = a.D + a.O;
    const uint64_t n = a.nblk * total;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t blk = i / total, o = i % total;
        const uint4 *rows = a.rows + blk * a.nrows;
        uint4 acc = zero4();
        for (uint32_t j = __ldg(a.off + o), e = __ldg(a.off + o + 1); j < e; j++) {
            acc = x4(acc, rows[__ldg(a.idx + j)]);
        }
        if ((__ldg(a.expect + (o >> 3)) >> (o & 7)) & 1u) {
            acc = make_uint4(~acc.x, ~acc.y, ~acc.z, ~acc.w);
        }
        if (o < a.D) {
            if (a.base_dets) {
                acc = x4(acc, a.base_dets[blk * a.D + o]);
            }
            a.dets[blk * a.D + o] = acc;
        } else {
            if (a.base_obs) {
                acc = x4(acc, a.base_obs[blk * a.O + (o - a.D)]);
            }
            a.obs[blk * a.O + (o - a.D)] = acc;
        }
    }
}

cudaError_t launch_fold(const FoldArgs &args, cudaStream_t stream) {
    const uint64_t n = args.nblk * (args.D + args.O);
    if (n == 0) {
        return cudaSuccess;
    }
    const uint64_t grid = std::min<uint64_t>((n + 255) / 256, (uint64_t)1 << 20);
    m2d_fold_kernel<<<(unsigned)grid, 256, 0, stream>>>(args);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Detector-error-model sampling.  The same walk as noise_records (screening rounds of 32 segments, queued
// segments walked by lanes that refill as soon as their walk ends), over a chunk of one probability group's
// mechanisms; a hit on mechanism m at `shot` XORs the shot's bit into every symptom row of m (global
// atomics, the rows are per launch and L2-resident) and sets it in m's error row when errors are wanted.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void dem_apply(const DemArgs &a, uint64_t blk, uint32_t m, uint32_t shot) {
    const uint32_t bit = 1u << (shot & 31);
    for (uint32_t j = __ldg(a.sym_off + m), e = __ldg(a.sym_off + m + 1); j < e; j++) {
        const uint32_t o = __ldg(a.sym + j);
        uint4 *row = o < a.D ? a.dets + blk * a.D + o : a.obs + blk * a.O + (o - a.D);
        atomicXor(reinterpret_cast<uint32_t *>(row) + (shot >> 5), bit);
    }
    if (a.errs) {
        atomicOr(reinterpret_cast<uint32_t *>(a.errs + blk * a.E + m) + (shot >> 5), bit);
    }
}

__global__ void __launch_bounds__(256) dem_sample_kernel(const DemArgs a) {
    __shared__ NoiseQueued queue[8][64];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t w = (uint64_t)blockIdx.x * 8 + warp;
    if (w >= a.nblk * a.nchunks) {
        return;
    }
    NoiseQueued *q = queue[warp];
    const uint64_t blk = w / a.nchunks;
    const uint32_t chunk = (uint32_t)(w % a.nchunks);
    const uint32_t g = __ldg(a.chunk_group + chunk), cu0 = __ldg(a.chunk_unit0 + chunk);
    const uint32_t cn = __ldg(a.chunk_units + chunk);
    const DemGroup G = a.groups[g];
    const uint32_t *T = a.tables + G.table;
    const bool always = (G.flags & 2u) != 0;
    const uint32_t block = (uint32_t)(a.block0 + blk);
    const uint32_t seg0 = cu0 / GFS_DEM_SEG_UNITS;  // chunks start on segment boundaries
    const uint32_t items = (cn + GFS_DEM_SEG_UNITS - 1) / GFS_DEM_SEG_UNITS;
    const uint32_t kseed0 = (uint32_t)a.seed, kseed1 = (uint32_t)(a.seed >> 32);
    const uint32_t c3base = gfs_c3(GFS_P_DEM, g, 0);
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t qn = 0, screened = 0;
    bool active = false;
    gfs_stream st;
    int32_t pos = -1, trials = 0;
    uint32_t ubase = 0;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !active);
        if (idle && qn) {
            const uint32_t take = min((uint32_t)__popc(idle), qn);
            const uint32_t rank = __popc(idle & lt);
            if (!active && rank < take) {
                const NoiseQueued e = q[qn - 1 - rank];
                const uint32_t sg = seg0 + e.item;
                ubase = sg * GFS_DEM_SEG_UNITS;
                trials = (int32_t)(min(GFS_DEM_SEG_UNITS, G.n - ubase) * GFS_BLOCK_SHOTS);
                gfs_stream_init(&st, a.seed, GFS_P_DEM, g, sg, block);
                if (always) {
                    pos = 0;
                } else {
                    st.group = 1;
                    st.left = 3;
                    st.b0 = e.d1;
                    st.b1 = e.d2;
                    st.b2 = e.d3;
                    pos = gfs_hit_after_draw(e.u, T, G.inv_c, -1, trials);
                }
                active = pos >= 0;
            }
            qn -= take;
            __syncwarp();
        }
        if (qn < 32 && screened < items) {
            const uint32_t item = screened + lane;
            bool hit = false;
            uint32_t u = 0, d1 = 0, d2 = 0, d3 = 0;
            if (item < items) {
                if (always) {
                    hit = true;
                } else {
                    const uint32_t sg = seg0 + item;
                    const uint32_t units = min(GFS_DEM_SEG_UNITS, G.n - sg * GFS_DEM_SEG_UNITS);
                    const gfs_u32x4 r = gfs_philox(kseed0, kseed1, block, sg, g, c3base);
                    u = r.v[0];
                    d1 = r.v[1];
                    d2 = r.v[2];
                    d3 = r.v[3];
                    hit = u >= __ldg(T + units * GFS_BLOCK_SHOTS);
                }
            }
            const uint32_t mask = __ballot_sync(0xFFFFFFFFu, hit);
            if (hit) {
                q[qn + __popc(mask & lt)] = NoiseQueued{item, u, d1, d2, d3};
            }
            qn += __popc(mask);
            screened += 32;
            __syncwarp();
            continue;
        }
        const uint32_t act = __ballot_sync(0xFFFFFFFFu, active);
        if (!act) {
            if (qn == 0 && screened >= items) {
                break;
            }
            continue;
        }
        if (active) {
            const uint32_t m = __ldg(a.units + G.first + ubase + ((uint32_t)pos >> 7));
            dem_apply(a, blk, m, (uint32_t)pos & 127u);
            pos = gfs_next_hit(&st, T, G.inv_c, pos, trials, always);
            active = pos >= 0;
        }
    }
}

cudaError_t launch_dem_sample(const DemArgs &args, cudaStream_t stream) {
    const uint64_t warps = args.nblk * args.nchunks;
    if (warps == 0) {
        return cudaSuccess;
    }
    const uint64_t blocks = (warps + 7) / 8;
    if (blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    dem_sample_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Decoder feed.  The reference's sinter sampler (glue/sample/src/sinter/_decoding/_stim_then_decode_sampler.py:
// 170-190) counts detection events with eight numpy passes over the shot-major bytes and drops postselected
// shots with a numpy mask; here both run over the device rows before anything crosses the link, and only the
// kept rows are copied out.
// ------------------------------------------------------------------------------------------------

// Set bits over the flat detector bytes (16-byte aligned base): one 16-byte load per thread and step.
__global__ void __launch_bounds__(256) feed_popcount_kernel(const uint8_t *p, uint64_t n, unsigned long long *count) {
    const uint64_t n16 = n / 16;
    const uint4 *q = reinterpret_cast<const uint4 *>(p);
    unsigned long long c = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * 256 + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * 256) {
        const uint4 v = q[i];
        c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 15)) {
        c += __popc(p[16 * n16 + threadIdx.x]);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
    }
    if ((threadIdx.x & 31) == 0 && c) {
        atomicAdd(count, c);
    }
}

// One warp per shot, eight shots (of one group) per CTA: lanes test the mask's bytes; the CTA adds its kept shots
// to its group's count in group_kept (zeroed by the launcher).  feed_scan_kernel derives the dropped count.
__global__ void __launch_bounds__(256) feed_flags_kernel(const FeedArgs a) {
    __shared__ uint32_t kept_warp[8];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t s0 = (uint64_t)blockIdx.x * 8, s = s0 + warp;
    uint32_t keep = 0;
    if (s < a.nshots) {
        const uint8_t *row = a.dets + s * a.drow;
        uint32_t hit = 0;
        for (uint32_t k = lane; k < a.nmask; k += 32) {
            hit |= row[a.mask_idx[k]] & a.mask_bits[k];
        }
        keep = __any_sync(0xFFFFFFFFu, hit != 0) ? 0u : 1u;
        if (lane == 0) {
            a.keep[s] = (uint8_t)keep;
        }
    }
    if (lane == 0) {
        kept_warp[warp] = keep;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 8; w++) {
            t += kept_warp[w];
        }
        if (t) {
            atomicAdd(&a.group_kept[s0 / kFeedGroup], t);
        }
    }
}

__device__ __forceinline__ uint32_t warp_inclusive_sum(uint32_t x, uint32_t lane) {
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) {
            x += y;
        }
    }
    return x;
}

// Exclusive prefix sum of the groups' kept counts, in place: one CTA walks tiles of 1024 with a carry.
// Exclusive scan of the groups' kept counts in place; the shots the scan does not cover were dropped, and their
// number goes to dropped[0].
__global__ void __launch_bounds__(1024) feed_scan_kernel(uint32_t *v, uint32_t n, uint64_t nshots,
                                                         unsigned long long *dropped) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry_s;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        carry_s = 0;
    }
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t x = i < n ? v[i] : 0u;
        const uint32_t inc = warp_inclusive_sum(x, lane);
        if (lane == 31) {
            wsum[warp] = inc;
        }
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = wsum[lane];
            wsum[lane] = warp_inclusive_sum(w, lane) - w;
        }
        __syncthreads();
        const uint32_t carry = carry_s;
        if (i < n) {
            v[i] = carry + wsum[warp] + inc - x;
        }
        __syncthreads();
        if (threadIdx.x == 1023) {
            carry_s = carry + wsum[31] + inc;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        dropped[0] = (unsigned long long)(nshots - carry_s);
    }
}

// Copies n bytes with the widest unit dividing n (both rows start at multiples of n from 256-byte aligned
// bases, so that unit is aligned on both sides).
__device__ __forceinline__ void feed_copy_row(uint8_t *dst, const uint8_t *src, uint64_t n, uint32_t lane) {
    if ((n & 15) == 0) {
        for (uint64_t j = lane; j < n / 16; j += 32) {
            reinterpret_cast<uint4 *>(dst)[j] = reinterpret_cast<const uint4 *>(src)[j];
        }
    } else if ((n & 7) == 0) {
        for (uint64_t j = lane; j < n / 8; j += 32) {
            reinterpret_cast<uint2 *>(dst)[j] = reinterpret_cast<const uint2 *>(src)[j];
        }
    } else if ((n & 3) == 0) {
        for (uint64_t j = lane; j < n / 4; j += 32) {
            reinterpret_cast<uint32_t *>(dst)[j] = reinterpret_cast<const uint32_t *>(src)[j];
        }
    } else if ((n & 1) == 0) {
        for (uint64_t j = lane; j < n / 2; j += 32) {
            reinterpret_cast<uint16_t *>(dst)[j] = reinterpret_cast<const uint16_t *>(src)[j];
        }
    } else {
        for (uint64_t j = lane; j < n; j += 32) {
            dst[j] = src[j];
        }
    }
}

// Kept shots of a group get consecutive output rows from the group's scanned start: thread t ranks shots
// 4t .. 4t + 3 and writes each shot's output row (or 0xFFFFFFFF) to dst.
__global__ void __launch_bounds__(256) feed_rank_kernel(const FeedArgs a) {
    __shared__ uint32_t wsum[8];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t s0 = (uint64_t)blockIdx.x * kFeedGroup;
    uint32_t k[4], c = 0;
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
        const uint64_t s = s0 + 4 * tid + j;
        k[j] = s < a.nshots ? (uint32_t)a.keep[s] : 0u;
        c += k[j];
    }
    const uint32_t inc = warp_inclusive_sum(c, lane);
    if (lane == 31) {
        wsum[warp] = inc;
    }
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) {
        before += wsum[w];
    }
    uint32_t pos = a.group_kept[blockIdx.x] + before + inc - c;
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
        const uint64_t s = s0 + 4 * tid + j;
        if (s < a.nshots) {
            a.dst[s] = k[j] ? pos : 0xFFFFFFFFu;
        }
        pos += k[j];
    }
}

// One warp per shot copies a kept shot's detector and observable rows to its output row; eight shots per CTA,
// so the copy runs with the whole GPU's warps in flight.
__global__ void __launch_bounds__(256) feed_gather_kernel(const FeedArgs a) {
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t s = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (s >= a.nshots) {
        return;
    }
    const uint32_t r = a.dst[s];
    if (r == 0xFFFFFFFFu) {
        return;
    }
    feed_copy_row(a.cdets + (uint64_t)r * a.drow, a.dets + s * a.drow, a.drow, lane);
    if (a.orow) {
        feed_copy_row(a.cobs + (uint64_t)r * a.orow, a.obs + s * a.orow, a.orow, lane);
    }
}

__global__ void publish_words_kernel(const uint32_t *src, uint32_t *dst, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        dst[i] = src[i];
    }
}

cudaError_t launch_publish_words(const uint32_t *src, uint32_t *dst, uint32_t n, cudaStream_t stream) {
    publish_words_kernel<<<1, 32, 0, stream>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_feed_popcount(const FeedArgs &args, cudaStream_t stream) {
    const uint64_t n = args.nshots * args.drow;
    if (n == 0) {
        return cudaSuccess;
    }
    const uint64_t want = (n / 16 + 255) / 256;
    const unsigned grid = (unsigned)(want < 1 ? 1 : (want > 4096 ? 4096 : want));
    feed_popcount_kernel<<<grid, 256, 0, stream>>>(args.dets, n, args.counts);
    return cudaGetLastError();
}

cudaError_t launch_feed_flags(const FeedArgs &args, cudaStream_t stream) {
    const uint64_t groups = (args.nshots + kFeedGroup - 1) / kFeedGroup;
    if (groups == 0) {
        return cudaSuccess;
    }
    if (groups > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    const uint64_t blocks = (args.nshots + 7) / 8;
    if (blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaMemsetAsync(args.group_kept, 0, groups * sizeof(uint32_t), stream);
    if (e != cudaSuccess) {
        return e;
    }
    feed_flags_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
    return cudaGetLastError();
}

cudaError_t launch_feed_scan(const FeedArgs &args, cudaStream_t stream) {
    const uint64_t groups = (args.nshots + kFeedGroup - 1) / kFeedGroup;
    if (groups == 0) {
        return cudaSuccess;
    }
    if (groups > 0xFFFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    feed_scan_kernel<<<1, 1024, 0, stream>>>(args.group_kept, (uint32_t)groups, args.nshots, args.counts + 1);
    return cudaGetLastError();
}

cudaError_t launch_feed_compact(const FeedArgs &args, cudaStream_t stream) {
    const uint64_t groups = (args.nshots + kFeedGroup - 1) / kFeedGroup;
    if (groups == 0) {
        return cudaSuccess;
    }
    if (groups > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    feed_rank_kernel<<<(unsigned)groups, 256, 0, stream>>>(args);
    const uint64_t blocks = (args.nshots + 7) / 8;
    if (blocks > 0x7FFFFFFFull) {
        return cudaErrorInvalidValue;
    }
    feed_gather_kernel<<<(unsigned)blocks, 256, 0, stream>>>(args);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------
// Shared-memory throughput probe: every thread streams 128-bit load/XOR/store passes over a 64 KiB
// shared buffer with conflict-free addressing (consecutive lanes touch consecutive 16-byte words).
// Reports the bytes moved (loads + stores) per second over all SMs: the denominator of the frame
// kernel's shared-memory roofline.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(512) smem_probe_kernel(uint32_t iters, uint32_t *sink) {
    extern __shared__ uint4 buf[];
    const uint32_t n = 4096;  // 64 KiB of uint4
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        buf[i] = make_uint4(i, i * 3u, i * 5u, i * 7u);
    }
    __syncthreads();
    uint4 acc = zero4();
    uint32_t idx = threadIdx.x;
    for (uint32_t it = 0; it < iters; it++) {
#pragma unroll 8
        for (uint32_t k = 0; k < 8; k++) {
            uint32_t j = (idx + k * blockDim.x) & (n - 1);
            uint4 v = buf[j];
            acc = x4(acc, v);
            buf[j] = x4(v, make_uint4(it, k, it ^ k, 1u));
        }
    }
    if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9E3779B9u) {
        atomicAdd(sink, 1u);
    }
}

cudaError_t measure_smem_peak(double *bytes_per_s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return e;
    const size_t smem = 4096 * sizeof(uint4);
    e = cudaFuncSetAttribute(smem_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, smem_probe_kernel, 512, smem);
    if (e != cudaSuccess) return e;
    int grid = prop.multiProcessorCount * (per_sm > 0 ? per_sm : 1);
    uint32_t *sink = nullptr;
    e = cudaMalloc(&sink, 4);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const uint32_t iters = 4096;
    smem_probe_kernel<<<grid, 512, smem>>>(64, sink);  // warm-up
    cudaEventRecord(a);
    smem_probe_kernel<<<grid, 512, smem>>>(iters, sink);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess) return e;
    double bytes = (double)grid * 512.0 * iters * 8.0 * 2.0 * sizeof(uint4);
    *bytes_per_s = bytes / (ms * 1e-3);
    return cudaGetLastError();
}


// ------------------------------------------------------------------------------------------------
// Integer-issue probes (the denominators of the instruction-bound rooflines):
// * lop3_probe_kernel: eight independent chains of 3-input logic ops (lop3.b32 XOR3) per thread, the
//   operation the frame kernel's gate updates are made of; reports 32-bit logic ops per second.
// * philox_probe_kernel: back-to-back Philox4x32-10 calls (the contract's generator) on distinct counters,
//   four independent streams per thread; reports generator calls per second, the peak of the noise kernel's
//   random-draw work.
// Both run one full wave of 1024-thread CTAs on every SM.
// ------------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) lop3_probe_kernel(uint32_t iters, uint32_t *sink) {
    uint32_t a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        a[j] = threadIdx.x * 2654435761u + (uint32_t)j * 40503u + blockIdx.x;
    }
    const uint32_t b = blockIdx.x * 97u + 1u, c = threadIdx.x ^ 0x5bd1e995u;
    for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
#pragma unroll
            for (int j = 0; j < 8; j++) {
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[j]) : "r"(b), "r"(c + (uint32_t)k));
            }
        }
    }
    uint32_t x = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        x ^= a[j];
    }
    if (x == 0x9E3779B9u) {
        atomicAdd(sink, 1u);
    }
}

__global__ void __launch_bounds__(1024) philox_probe_kernel(uint32_t iters, uint32_t *sink) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    // The key is a run-time value, as the seed is in the sampling kernels (so its schedule is not folded).
    const uint32_t k0 = iters * 0x9E3779B9u + 17u, k1 = iters ^ 0x85EBCA6Bu;
    uint32_t x = 0;
    for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
        for (uint32_t j = 0; j < 4; j++) {
            const gfs_u32x4 r = gfs_philox(k0, k1, t, it, j, GFS_P_NOISE << 28);
            x ^= r.v[0] ^ r.v[1] ^ r.v[2] ^ r.v[3];
        }
    }
    if (x == 0x9E3779B9u) {
        atomicAdd(sink, 1u);
    }
}

// Runs `kernel` for one full wave (resident 1024-thread CTAs on every SM) and returns seconds.
template <typename K>
static cudaError_t time_probe(K kernel, uint32_t iters, double *seconds, double *threads) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 1024, 0);
    if (e != cudaSuccess) return e;
    const int grid = prop.multiProcessorCount * (per_sm > 0 ? per_sm : 1);
    uint32_t *sink = nullptr;
    e = cudaMalloc(&sink, 4);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    kernel<<<grid, 1024>>>(iters / 16 + 1, sink);  // warm-up
    cudaEventRecord(a);
    kernel<<<grid, 1024>>>(iters, sink);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess) return e;
    *seconds = ms * 1e-3;
    *threads = (double)grid * 1024.0;
    return cudaGetLastError();
}

cudaError_t measure_int_peaks(double *lop3_per_s, double *philox_per_s) {
    double s = 0, th = 0;
    const uint32_t lop_iters = 4096;
    cudaError_t e = time_probe(lop3_probe_kernel, lop_iters, &s, &th);
    if (e != cudaSuccess) return e;
    *lop3_per_s = th * lop_iters * 16.0 * 8.0 / s;
    const uint32_t ph_iters = 256;
    e = time_probe(philox_probe_kernel, ph_iters, &s, &th);
    if (e != cudaSuccess) return e;
    *philox_per_s = th * ph_iters * 4.0 / s;
    return cudaSuccess;
}

}  // namespace gfs
