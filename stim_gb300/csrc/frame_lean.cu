// Lean frame kernel for sm_103a: the frame kernel's work with the per-phase overhead cut down.
//
// A CTA owns a slice of B x 128 shots at a time (persistent, grid-stride over slices), with its X/Z frames,
// observables and (when it fits) the measurement ring in shared memory, exactly as frame_kernel does, and
// produces the same bits.  What differs is how it walks the program.  The lowering re-cuts the device program
// into a phase list (program.h LeanPhase: one 16-byte descriptor per barrier-separated step, fields resolved
// on the host, the noise fused into a gate split into its own hit phase), which the CTA keeps in shared
// memory.  Each thread works one phase ahead: before the barrier that ends phase k it has already done the
// loop bookkeeping that leads to phase k+1, read k+1's descriptor and loaded the unit-list entries of its
// first kLeanJ items of k+1 into registers.
//
// Hit records reach shared memory ahead of time: each hit phase copies (cp.async) the record that this thread
// applies first two noise occurrences later into a per-thread staging slot, so that when a hit phase starts its
// record is already in shared memory instead of a DRAM round trip away.  Phases whose successors only XOR into
// the same rows or touch disjoint state (consecutive hit phases, detectors next to Pauli hits) run without a
// barrier between them (program.h kLeanNoBarrier).
//
// Noise comes only from hit lists (noise_kernel runs first), so no Philox work or gap tables live here.
// Programs with correlated errors, heralds or sweep-controlled feedback, unit lists that are not compact,
// or more than two loop levels keep the generic kernel.
#include "frame_device.cuh"

namespace gfs {

namespace {

constexpr int kLeanJ = 6;  // unit-list entries per thread prefetched one phase ahead

struct LeanLoops {
    int depth;
    uint32_t lpc0, lpc1, left0, left1;
    uint64_t base0, base1, stride0, stride1;
};

// Executes the loop bookkeeping phases from `pc` on and returns the index of the next phase that does work
// (or LK_END).  Uniform across the CTA.
__device__ __forceinline__ uint32_t lean_next(const LeanPhase *ph, const uint64_t *lean_inst, uint32_t pc,
                                              LeanLoops &lp, uint64_t &inst_base) {
    for (;;) {
        const LeanPhase d = ph[pc];
        const uint32_t kind = d.op & 0xFFu;
        if (kind == LK_LOOP_BEGIN) {
            const uint64_t stride = (uint64_t)d.a | ((uint64_t)d.b << 32);
            if (lp.depth == 0) {
                lp.lpc0 = pc;
                lp.left0 = d.n;
                lp.base0 = inst_base;
                lp.stride0 = stride;
            } else {
                lp.lpc1 = pc;
                lp.left1 = d.n;
                lp.base1 = inst_base;
                lp.stride1 = stride;
            }
            lp.depth++;
            inst_base += __ldg(reinterpret_cast<const unsigned long long *>(lean_inst) + pc);
            pc++;
            continue;
        }
        if (kind == LK_LOOP_END) {
            if (lp.depth == 2) {
                if (--lp.left1 > 0) {
                    inst_base += lp.stride1;
                    pc = lp.lpc1 + 1;
                } else {
                    inst_base = lp.base1;
                    lp.depth = 1;
                    pc++;
                }
            } else {
                if (--lp.left0 > 0) {
                    inst_base += lp.stride0;
                    pc = lp.lpc0 + 1;
                } else {
                    inst_base = lp.base0;
                    lp.depth = 0;
                    pc++;
                }
            }
            continue;
        }
        return pc;
    }
}

// Unit-list entries of this thread's first kLeanJ items of phase `d` (items i = tid + j * nt, item = unit * B
// + block).  16-bit lists for one-qubit gates, measurements and resets, 32-bit words for pairs and detectors.
template <int B>
__device__ __forceinline__ void lean_prefetch(const LeanPhase &d, const uint32_t *pool, uint32_t tid, uint32_t nt,
                                              uint32_t (&E)[kLeanJ]) {
    const uint32_t kind = d.op & 0xFFu;
    const uint32_t items = d.n * B;
    if (kind == LK_1Q || kind == LK_MEAS || kind == LK_RESET) {
        const unsigned short *l = reinterpret_cast<const unsigned short *>(pool + d.a);
#pragma unroll
        for (int j = 0; j < kLeanJ; j++) {
            const uint32_t i = tid + (uint32_t)j * nt;
            E[j] = i < items ? (uint32_t)__ldg(l + i / B) : 0u;
        }
    } else if (kind == LK_CX || kind == LK_CZ || kind == LK_2Q || kind == LK_DETS2) {
        const uint32_t *l = pool + d.a;
#pragma unroll
        for (int j = 0; j < kLeanJ; j++) {
            const uint32_t i = tid + (uint32_t)j * nt;
            E[j] = i < items ? __ldg(l + i / B) : 0u;
        }
    }
}

// f(unit, block, entry) over this thread's items: the first kLeanJ from the prefetched entries, the rest (units
// beyond kLeanJ * nt items) loaded here.
template <int B, bool HALF, typename F>
__device__ __forceinline__ void lean_items(const uint32_t (&E)[kLeanJ], const uint32_t *list, uint32_t items,
                                           uint32_t tid, uint32_t nt, F f) {
#pragma unroll
    for (int j = 0; j < kLeanJ; j++) {
        const uint32_t i = tid + (uint32_t)j * nt;
        if (i < items) {
            f(i / B, i % B, E[j]);
        }
    }
    for (uint32_t i = tid + (uint32_t)kLeanJ * nt; i < items; i += nt) {
        const uint32_t w = HALF ? (uint32_t)__ldg(reinterpret_cast<const unsigned short *>(list) + i / B)
                                : __ldg(list + i / B);
        f(i / B, i % B, w);
    }
}

// CX / CZ over this thread's pairs, two pairs' loads in flight together.
template <int B>
__device__ __forceinline__ void lean_cx_cz(const uint32_t (&E)[kLeanJ], const uint32_t *list, bool cz, uint32_t items,
                                           uint4 *X, uint4 *Z, uint32_t tid, uint32_t nt) {
    auto pair2 = [&](uint32_t ia, uint32_t wa, uint32_t ib, uint32_t wb) {
        const bool two = ib < items;
        const uint32_t a1 = (wa & 0xFFFFu) * B + ia % B, a2 = (wa >> 16) * B + ia % B;
        const uint32_t b1 = (wb & 0xFFFFu) * B + ib % B, b2 = (wb >> 16) * B + ib % B;
        const uint4 az1 = Z[a1], az2 = Z[a2], ax1 = X[a1], ax2 = X[a2];
        uint4 bz1 = az1, bz2 = az2, bx1 = ax1, bx2 = ax2;
        if (two) {
            bz1 = Z[b1];
            bz2 = Z[b2];
            bx1 = X[b1];
            bx2 = X[b2];
        }
        if (!cz) {
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
    };
#pragma unroll
    for (int j = 0; j < kLeanJ; j += 2) {
        const uint32_t ia = tid + (uint32_t)j * nt;
        if (ia < items) {
            pair2(ia, E[j], ia + nt, E[j + 1]);
        }
    }
    for (uint32_t ia = tid + (uint32_t)kLeanJ * nt; ia < items; ia += 2 * nt) {
        const uint32_t ib = ia + nt;
        pair2(ia, __ldg(list + ia / B), ib, ib < items ? __ldg(list + ib / B) : 0u);
    }
}

// Staged hit records: slot (occ & 1) of stg holds, for each thread, the first record it applies of occurrence
// occ (record tid), copied there asynchronously two hit phases earlier.  oc[k] = {region offset, count} of
// occurrence k in this slice (two zero sentinels past the last).
__device__ __forceinline__ void lean_stage(uint64_t *slot, const uint64_t *hb, uint2 c, uint32_t tid) {
    if (tid < c.y) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(slot + tid)),
                     "l"(hb + c.x + tid)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");  // one group per call, empty or not
}

// Applies the records of noise occurrence `occ` (Pauli flips into the frames, or measurement flips into the last
// n results of the ring) and stages this thread's first record of occurrence occ + 2.
template <int B>
__device__ __forceinline__ void lean_hits(const uint2 *oc, uint64_t *stg, const uint64_t *hb, uint32_t occ,
                                          bool flips, uint4 *X, uint4 *Z, uint4 *R, uint32_t rec, uint32_t L,
                                          uint32_t n, uint32_t tid, uint32_t nt) {
    asm volatile("cp.async.wait_group 1;" ::: "memory");  // this occurrence's copies (not the next one's)
    const uint2 c = oc[occ];
    uint64_t *const slot = stg + (size_t)(occ & 1u) * nt;
    auto apply = [&](uint64_t r) {
        const uint32_t ra = (uint32_t)r & kRowMask, rb = (uint32_t)(r >> 24) & kRowMask;
        const uint32_t bits = (uint32_t)(r >> 48) & 15u, s9 = (uint32_t)(r >> 52) & 511u;
        const uint32_t blk = s9 >> 7, shot = s9 & 127u;
        if (flips) {
            flip_bit(R, wrap(rec + L - n + ra, L) * B + blk, shot, true);
        } else {
            apply_bits(X, Z, ra * B + blk, rb * B + blk, shot, bits, true);
        }
    };
    if (tid < c.y) {
        apply(slot[tid]);  // read (and used) before the slot is reused below
    }
    lean_stage(slot, hb, oc[occ + 2], tid);
    for (uint32_t i = tid + nt; i < c.y; i += nt) {
        apply(__ldcg(reinterpret_cast<const unsigned long long *>(hb + c.x + i)));
    }
}

struct LeanState {
    uint4 *X, *Z, *R, *O;
    const LeanPhase *ph;
    uint2 *oc;      // [n_occ + 2] {region offset, this slice's count}
    uint64_t *stg;  // [2][threads] staged first records
};

// Shared-memory layout: X and Z frames [row][block], the ring [row][block] unless it is in global memory,
// observables, the phase list, the occurrence table, then the record staging slots.
template <int B>
__device__ __forceinline__ LeanState lean_state(const KernelArgs &p, uint4 *sm) {
    LeanState st;
    const uint32_t nr = p.nrows, L = p.ring, NO = p.nobs;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    st.X = sm;
    st.Z = st.X + (size_t)nr * B;
    uint4 *after = st.Z + (size_t)nr * B;
    st.R = p.ring_global ? p.ring_global + (size_t)blockIdx.x * p.ring_cta_stride : after;
    st.O = p.ring_global ? after : st.R + (size_t)L * B;
    LeanPhase *ph = reinterpret_cast<LeanPhase *>(st.O + (size_t)NO * B);
    for (uint32_t i = tid; i < p.n_lean; i += nt) {
        ph[i] = p.lean[i];
    }
    st.ph = ph;
    st.oc = reinterpret_cast<uint2 *>(ph + p.n_lean);
    for (uint32_t i = tid; i < p.n_occ + 2; i += nt) {
        st.oc[i] = make_uint2(i < p.n_occ ? __ldg(&p.occs[i].off) : 0u, 0u);
    }
    st.stg = reinterpret_cast<uint64_t *>(st.oc + p.n_occ + 2);
    return st;
}

template <int B>
__device__ __forceinline__ void lean_slice(const KernelArgs &p, const LeanState &st, uint32_t slice) {
    const uint32_t nr = p.nrows, L = p.ring, NO = p.nobs;
    uint4 *const X = st.X, *const Z = st.Z, *const R = st.R, *const O = st.O;
    const LeanPhase *const ph = st.ph;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const uint32_t *const pool = p.pool;
    const uint64_t lb0 = (uint64_t)slice * B;
    const uint64_t gb0 = p.block0 + lb0;
    const bool rg = p.ring_global != nullptr;
    const uint32_t n_occ = p.n_occ;

    for (uint32_t i = tid; i < nr * B; i += nt) {
        const uint32_t r = i / B, blk = i % B;
        X[i] = zero4();
        Z[i] = p.reset_zero ? zero4()
                            : u4(gfs_row_bits(p.seed, GFS_P_RESET, 0, __ldg(p.qubit_orig + r), (uint32_t)(gb0 + blk)));
    }
    for (uint32_t i = tid; i < NO * B; i += nt) {
        O[i] = zero4();
    }
    {
        const uint32_t *cnt = p.hit_count + (uint64_t)slice * n_occ;
        for (uint32_t i = tid; i < n_occ; i += nt) {
            st.oc[i].y = __ldg(cnt + i);
        }
    }
    __syncthreads();
    const uint64_t *const hb = p.hits + (uint64_t)slice * p.slice_cap;
    lean_stage(st.stg, hb, st.oc[0], tid);
    lean_stage(st.stg + nt, hb, st.oc[1], tid);

    LeanLoops lp{};
    uint64_t inst_base = 0;
    uint32_t rec = 0, occ = 0;
    uint64_t det_base = 0, meas_base = 0;
    uint32_t pc = lean_next(ph, p.lean_inst, 0, lp, inst_base);
    LeanPhase d = ph[pc];
    uint32_t E[kLeanJ];
    lean_prefetch<B>(d, pool, tid, nt, E);

    for (;;) {
        const uint32_t kind = d.op & 0xFFu, sub = (d.op >> 8) & 0xFFu;
        const uint32_t n = d.n, items = n * B;
        if (kind == LK_END) {
            break;
        }
        const uint32_t *const list = pool + d.a;
        switch (kind) {
            case LK_HITS:
            case LK_FLIPS:
                if (occ >= n_occ) {  // the host counted fewer occurrences than the program has
                    if (tid == 0) {
                        atomicOr(p.status, 2u);
                    }
                    break;
                }
                lean_hits<B>(st.oc, st.stg, hb, occ++, kind == LK_FLIPS, X, Z, R, rec, L, n, tid, nt);
                break;
            case LK_1Q:
                lean_items<B, true>(E, list, items, tid, nt, [&](uint32_t, uint32_t blk, uint32_t row) {
                    const uint32_t idx = row * B + blk;
                    uint4 x = X[idx], z = Z[idx];
                    rule1(sub, x, z);
                    X[idx] = x;
                    Z[idx] = z;
                });
                break;
            case LK_CX:
            case LK_CZ:
                lean_cx_cz<B>(E, list, kind == LK_CZ, items, X, Z, tid, nt);
                break;
            case LK_2Q:
                lean_items<B, false>(E, list, items, tid, nt, [&](uint32_t, uint32_t blk, uint32_t w) {
                    const uint32_t i1 = (w & 0xFFFFu) * B + blk, i2 = (w >> 16) * B + blk;
                    uint4 x1 = X[i1], z1 = Z[i1], x2 = X[i2], z2 = Z[i2];
                    rule2v(sub, x1, z1, x2, z2);
                    X[i1] = x1;
                    Z[i1] = z1;
                    X[i2] = x2;
                    Z[i2] = z2;
                });
                break;
            case LK_MEAS: {
                const bool norand = (d.op & kLeanNoRandomize) != 0;
                const uint64_t inst = norand ? 0 : inst_base + p.lean_inst[pc];
                lean_items<B, true>(E, list, items, tid, nt, [&](uint32_t u, uint32_t blk, uint32_t row) {
                    measure_row(sub, X, Z, R, row * B + blk, wrap(rec + u, L) * B + blk,
                                rand_row(p, norand, inst, d.b + u, (uint32_t)(gb0 + blk)), rg, norand);
                });
                rec = wrap(rec + n, L);
                break;
            }
            case LK_RESET: {
                const bool norand = (d.op & kLeanNoRandomize) != 0;
                const uint64_t inst = norand ? 0 : inst_base + p.lean_inst[pc];
                lean_items<B, true>(E, list, items, tid, nt, [&](uint32_t u, uint32_t blk, uint32_t row) {
                    reset_row(sub, X, Z, row * B + blk, rand_row(p, norand, inst, d.b + u, (uint32_t)(gb0 + blk)),
                              norand);
                });
                break;
            }
            case LK_ZERO:
                for (uint32_t i = tid; i < items; i += nt) {
                    ring_st(R, wrap(rec + i / B, L) * B + i % B, zero4(), rg);
                }
                rec = wrap(rec + n, L);
                break;
            case LK_DETS2: {
                uint4 *const out = p.det_out;
                const uint64_t ndet = p.ndet;
                // All of this thread's prefetched detectors' records are loaded before any result is stored.
                uint4 acc[kLeanJ];
#pragma unroll
                for (int j = 0; j < kLeanJ; j++) {
                    const uint32_t i = tid + (uint32_t)j * nt;
                    const uint32_t blk = i % B, k1 = E[j] & 0xFFFFu, k2 = E[j] >> 16;
                    acc[j] = zero4();
                    if (i < items && k1) {
                        acc[j] = ring_ld(R, wrap(rec + L - k1, L) * B + blk, rg);
                    }
                    if (i < items && k2) {
                        acc[j] = x4(acc[j], ring_ld(R, wrap(rec + L - k2, L) * B + blk, rg));
                    }
                }
#pragma unroll
                for (int j = 0; j < kLeanJ; j++) {
                    const uint32_t i = tid + (uint32_t)j * nt;
                    if (i < items) {
                        out[(lb0 + i % B) * ndet + det_base + i / B] = acc[j];
                    }
                }
                for (uint32_t i = tid + (uint32_t)kLeanJ * nt; i < items; i += nt) {
                    const uint32_t w = __ldg(list + i / B), blk = i % B, k1 = w & 0xFFFFu, k2 = w >> 16;
                    uint4 a = zero4();
                    if (k1) {
                        a = ring_ld(R, wrap(rec + L - k1, L) * B + blk, rg);
                    }
                    if (k2) {
                        a = x4(a, ring_ld(R, wrap(rec + L - k2, L) * B + blk, rg));
                    }
                    out[(lb0 + blk) * ndet + det_base + i / B] = a;
                }
                det_base += n;
                break;
            }
            case LK_DETS:
                for (uint32_t i = tid; i < items; i += nt) {
                    const uint32_t u = i / B, blk = i % B;
                    const uint32_t s = __ldg(pool + d.a + u), e = __ldg(pool + d.a + u + 1);
                    uint4 acc = zero4();
                    for (uint32_t j = s; j < e; j++) {
                        acc = x4(acc, ring_ld(R, wrap(rec + L - __ldg(pool + j), L) * B + blk, rg));
                    }
                    p.det_out[(lb0 + blk) * p.ndet + det_base + u] = acc;
                }
                det_base += n;
                break;
            case LK_OBS:
                for (uint32_t i = tid; i < items; i += nt) {
                    const uint32_t u = i / B, blk = i % B;
                    const uint32_t t = __ldg(pool + d.a + u);
                    uint4 v;
                    if (t & kTermRecord) {
                        v = ring_ld(R, wrap(rec + L - (t & kRowMask), L) * B + blk, rg);
                    } else {
                        const uint32_t idx = (t & kRowMask) * B + blk;
                        v = zero4();
                        if (t & kTermX) {
                            v = x4(v, Z[idx]);
                        }
                        if (t & kTermZ) {
                            v = x4(v, X[idx]);
                        }
                    }
                    atomic_xor4(O, d.b * B + blk, v);
                }
                break;
            case LK_EMIT:
                for (uint32_t i = tid; i < items; i += nt) {
                    const uint32_t u = i / B, blk = i % B;
                    p.meas_out[(lb0 + blk) * p.nmeas + meas_base + u] =
                        ring_ld(R, wrap(rec + L - n + u, L) * B + blk, rg);
                }
                meas_base += n;
                break;
            case LK_FEEDBACK:
                for (uint32_t i = tid; i < items; i += nt) {
                    const uint32_t u = i / B, blk = i % B;
                    const uint32_t k = __ldg(pool + d.a + 2 * u), rm = __ldg(pool + d.a + 2 * u + 1);
                    const uint32_t idx = (rm & kRowMask) * B + blk;
                    const uint4 v = ring_ld(R, wrap(rec + L - k, L) * B + blk, rg);
                    if ((rm >> 24) & kFeedbackX) {
                        X[idx] = x4(X[idx], v);
                    }
                    if ((rm >> 24) & kFeedbackZ) {
                        Z[idx] = x4(Z[idx], v);
                    }
                }
                break;
            default:
                if (tid == 0) {
                    atomicOr(p.status, 2u);
                }
                break;
        }
        // Phase k+1 is resolved and its entries are on their way before the barrier that ends phase k.
        const bool bar = (d.op & kLeanNoBarrier) == 0;
        pc++;
        d = ph[pc];
        if ((d.op & 0xFFu) == LK_LOOP_BEGIN || (d.op & 0xFFu) == LK_LOOP_END) {
            pc = lean_next(ph, p.lean_inst, pc, lp, inst_base);
            d = ph[pc];
        }
        lean_prefetch<B>(d, pool, tid, nt, E);
        if (bar) {
            __syncthreads();
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // no copy may land in the staging slots of the next slice

    for (uint32_t i = tid; i < NO * B; i += nt) {
        const uint32_t k = i / B, blk = i % B;
        p.obs_out[(lb0 + blk) * NO + k] = O[i];
    }
    __syncthreads();
}

template <int B>
__global__ void __maxnreg__(96) frame_kernel_lean(const KernelArgs p) {
    extern __shared__ uint4 sm[];
    const LeanState st = lean_state<B>(p, sm);
    for (uint32_t slice = blockIdx.x; slice < p.nslices; slice += gridDim.x) {
        lean_slice<B>(p, st, slice);
    }
}

// Many circuits in one persistent launch (as batch_frame_kernel): CTAs claim (circuit, slice) work items from a
// global counter and reload a circuit's phase list and occurrence table only when the circuit changes.
template <int B>
__global__ void __maxnreg__(96) batch_frame_kernel_lean(const BatchArgs b) {
    extern __shared__ uint4 sm[];
    __shared__ KernelArgs cur;
    __shared__ uint32_t s_item, s_circ;
    uint32_t have = 0xFFFFFFFFu;
    LeanState st{};
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
            st = lean_state<B>(cur, sm);
            have = j;
        }
        lean_slice<B>(cur, st, item - b.slice_prefix[j]);
    }
}

template <int B>
cudaError_t lean_batch_launch_b(const BatchArgs &args, const LaunchShape &s, cudaStream_t stream) {
    cudaError_t e =
        cudaFuncSetAttribute(batch_frame_kernel_lean<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    e = launch_batch_noise_kernel(args, B, stream);
    if (e != cudaSuccess) {
        return e;
    }
    batch_frame_kernel_lean<B><<<s.grid, s.threads, s.smem, stream>>>(args);
    return cudaGetLastError();
}

template <int B>
cudaError_t lean_batch_occ_b(const LaunchShape &s, int *out) {
    cudaError_t e =
        cudaFuncSetAttribute(batch_frame_kernel_lean<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, batch_frame_kernel_lean<B>, s.threads, s.smem);
}

template <int B>
cudaError_t lean_launch_b(const KernelArgs &args, const LaunchShape &s, cudaStream_t stream) {
    cudaError_t e = cudaFuncSetAttribute(frame_kernel_lean<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    frame_kernel_lean<B><<<s.grid, s.threads, s.smem, stream>>>(args);
    return cudaGetLastError();
}

template <int B>
cudaError_t lean_occ_b(const LaunchShape &s, int *out) {
    cudaError_t e = cudaFuncSetAttribute(frame_kernel_lean<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s.smem);
    if (e != cudaSuccess) {
        return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, frame_kernel_lean<B>, s.threads, s.smem);
}

}  // namespace

size_t lean_smem_bytes(uint32_t nrows, uint32_t ring, uint32_t nobs, int blocks_per_cta, uint32_t n_lean,
                       uint32_t n_occ, int threads) {
    // `ring` = measurement-ring rows held in shared memory (0 when the ring is in global memory).
    return ((size_t)2 * nrows + ring + nobs) * (size_t)blocks_per_cta * sizeof(uint4) +
           (size_t)n_lean * sizeof(LeanPhase) + (size_t)(n_occ + 2) * sizeof(uint2) +
           (size_t)2 * threads * sizeof(uint64_t);
}

cudaError_t launch_frame_kernel_lean(const KernelArgs &args, const LaunchShape &shape, cudaStream_t stream) {
    if (!args.hits || !args.lean || args.n_lean == 0 || shape.frames_global || args.sweep || !args.occs) {
        return cudaErrorInvalidValue;
    }
    switch (shape.blocks_per_cta) {
        case 1:
            return lean_launch_b<1>(args, shape, stream);
        case 2:
            return lean_launch_b<2>(args, shape, stream);
        case 4:
            return lean_launch_b<4>(args, shape, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_batch_frame_kernel_lean(const BatchArgs &args, const LaunchShape &shape, cudaStream_t stream) {
    if (!shape.hits) {
        return cudaErrorInvalidValue;
    }
    switch (shape.blocks_per_cta) {
        case 1:
            return lean_batch_launch_b<1>(args, shape, stream);
        case 2:
            return lean_batch_launch_b<2>(args, shape, stream);
        case 4:
            return lean_batch_launch_b<4>(args, shape, stream);
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t batch_frame_kernel_lean_max_ctas_per_sm(const LaunchShape &shape, int *out) {
    switch (shape.blocks_per_cta) {
        case 1:
            return lean_batch_occ_b<1>(shape, out);
        case 2:
            return lean_batch_occ_b<2>(shape, out);
        case 4:
            return lean_batch_occ_b<4>(shape, out);
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t frame_kernel_lean_max_ctas_per_sm(const LaunchShape &shape, int *out) {
    switch (shape.blocks_per_cta) {
        case 1:
            return lean_occ_b<1>(shape, out);
        case 2:
            return lean_occ_b<2>(shape, out);
        case 4:
            return lean_occ_b<4>(shape, out);
        default:
            return cudaErrorInvalidValue;
    }
}

}  // namespace gfs
