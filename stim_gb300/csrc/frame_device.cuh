// Device helpers shared by the frame kernels (kernels.cu, frame_lean.cu): 128-shot row arithmetic, the
// per-gate frame rules applied to uint4 rows, measurement / reset of one row, noise-hit application, and the
// 64-bit hit-record format written by noise_kernel.
#pragma once

#include <cstdint>

#include "frame_rules.h"
#include "gfs_contract.h"
#include "kernels.h"

namespace gfs {

__device__ __forceinline__ uint4 x4(uint4 a, uint4 b) {
    return make_uint4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w);
}
__device__ __forceinline__ uint4 zero4() {
    return make_uint4(0, 0, 0, 0);
}
__device__ __forceinline__ uint4 u4(gfs_u32x4 v) {
    return make_uint4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ uint32_t wrap(uint32_t s, uint32_t L) {
    return s >= L ? s - L : s;
}
__device__ __forceinline__ void atomic_xor_bit(uint4 *base, uint32_t idx, uint32_t shot) {
    atomicXor(reinterpret_cast<uint32_t *>(base + idx) + (shot >> 5), 1u << (shot & 31));
}
__device__ __forceinline__ void atomic_or_bit(uint4 *base, uint32_t idx, uint32_t shot) {
    atomicOr(reinterpret_cast<uint32_t *>(base + idx) + (shot >> 5), 1u << (shot & 31));
}

__device__ __forceinline__ void rule2v(uint32_t sub, uint4 &x1, uint4 &z1, uint4 &x2, uint4 &z2) {
    rule2(sub, x1.x, z1.x, x2.x, z2.x);
    rule2(sub, x1.y, z1.y, x2.y, z2.y);
    rule2(sub, x1.z, z1.z, x2.z, z2.z);
    rule2(sub, x1.w, z1.w, x2.w, z2.w);
}

// Pauli pattern of a noise hit: bit0 = X on the unit's (first) row, bit1 = Z on it, bits 2-3 the same for
// the second row of a pair; for measurement flips (KN_FLIP) bit0 = flip.
__device__ __forceinline__ uint32_t pauli_xz(uint32_t v) {  // 0=I 1=X 2=Y 3=Z
    return (v == 1 || v == 2 ? 1u : 0u) | (v == 2 || v == 3 ? 2u : 0u);
}

// Draws the Pauli of one hit, consuming the channel's choice draw when it has one.  DEPOLARIZE1/2 keep
// the reference's bit layout of 1 + rng() % 3 / % 15 (frame_simulator.inl:663-690).
__device__ __forceinline__ uint32_t hit_bits(uint32_t kind, const DevChan &ch, gfs_stream *st) {
    switch (kind) {
        case KN_X:
        case KN_FLIP:
            return 1;
        case KN_Y:
            return 3;
        case KN_Z:
            return 2;
        case KN_DEP1:
            return 1 + gfs_choice_uniform(gfs_stream_next(st), 3);
        case KN_PC1:
            return pauli_xz(1 + gfs_choice_weighted(gfs_stream_next(st), ch.cum, 3));
        case KN_DEP2:
            return 1 + gfs_choice_uniform(gfs_stream_next(st), 15);
        default: {  // KN_PC2
            uint32_t v = 1 + gfs_choice_weighted(gfs_stream_next(st), ch.cum, 15);
            return pauli_xz(v >> 2) | (pauli_xz(v & 3) << 2);
        }
    }
}

// The hits of one segment (units [16g, 16g+16) x the 128 shots of a block), following gfs_contract.h:
// f(k, shot, stream) is called for each hit, on unit 4g + k at `shot`.  At small p the first Philox
// call of the segment usually shows there is no hit at all.
template <typename F>
__device__ __forceinline__ void walk_segment(const DevChan &ch, const uint32_t *T, uint64_t seed, uint32_t purpose,
                                             uint64_t inst, uint32_t seg, uint32_t block, uint32_t nunits, F f) {
    gfs_stream st;
    gfs_stream_init(&st, seed, purpose, inst, seg, block);
    const int32_t trials = (int32_t)(nunits * GFS_BLOCK_SHOTS);
    int32_t pos = -1;
    while ((pos = gfs_next_hit(&st, T, ch.inv_c, pos, trials, ch.always)) >= 0) {
        f((uint32_t)pos >> 7, (uint32_t)pos & 127u, &st);
    }
}

__device__ __forceinline__ void flip_bit(uint4 *base, uint32_t idx, uint32_t shot, bool atomic) {
    uint32_t *w = reinterpret_cast<uint32_t *>(base + idx) + (shot >> 5);
    if (atomic) {
        atomicXor(w, 1u << (shot & 31));
    } else {
        *w ^= 1u << (shot & 31);
    }
}

__device__ __forceinline__ void atomic_xor4(uint4 *base, uint32_t idx, uint4 m) {
    uint32_t *w = reinterpret_cast<uint32_t *>(base + idx);
    if (m.x) atomicXor(w + 0, m.x);
    if (m.y) atomicXor(w + 1, m.y);
    if (m.z) atomicXor(w + 2, m.z);
    if (m.w) atomicXor(w + 3, m.w);
}

// Applies the Pauli `bits` of one hit (bit0 = X / bit1 = Z on the first row, bits 2-3 on the second).
__device__ __forceinline__ void apply_bits(uint4 *X, uint4 *Z, uint32_t i1, uint32_t i2, uint32_t shot,
                                           uint32_t bits, bool atomic) {
    if (bits & 1) flip_bit(X, i1, shot, atomic);
    if (bits & 2) flip_bit(Z, i1, shot, atomic);
    if (bits & 4) flip_bit(X, i2, shot, atomic);
    if (bits & 8) flip_bit(Z, i2, shot, atomic);
}

// A noise channel fused into a gate op: DevOp c (after the gate) / d (before it).
struct Fused {
    const DevChan *ch;  // null when absent
    uint32_t kind;
    uint64_t inst;
};

__device__ __forceinline__ Fused decode_fused(const KernelArgs &p, uint32_t v, uint64_t inst) {
    Fused f;
    const uint32_t c = v & kFusedChanMask;
    f.ch = c ? &p.chans[c - 1] : nullptr;
    f.kind = (v >> 20) & 0xFu;
    f.inst = inst + (int64_t)(int8_t)(v >> 24);
    return f;
}

// Applies the one-qubit frame rule of a K1_* gate to 128 shots.
__device__ __forceinline__ void rule1(uint32_t sub, uint4 &x, uint4 &z) {
    rule1w(sub, x.x, z.x);
    rule1w(sub, x.y, z.y);
    rule1w(sub, x.z, z.z);
    rule1w(sub, x.w, z.w);
}

// The randomized row of unit u of a measurement / reset instance (zero when the lowering proved the row
// never reaches an output of this sampling mode).
__device__ __forceinline__ uint4 rand_row(const KernelArgs &p, bool norand, uint64_t inst, uint32_t unit,
                                          uint32_t block) {
    return norand ? zero4() : u4(gfs_row_bits(p.seed, GFS_P_RAND, inst, unit, block));
}

// Measurement-ring accesses.  When the ring is in global memory (rg) they go through L2 only: the ring is
// private to its CTA, and keeping it out of L1 leaves L1 to the op lists that every CTA on the SM reads.
__device__ __forceinline__ uint4 ring_ld(const uint4 *R, uint32_t i, bool rg) {
    return rg ? __ldcg(R + i) : R[i];
}
__device__ __forceinline__ void ring_st(uint4 *R, uint32_t i, uint4 v, bool rg) {
    if (rg) {
        __stcg(R + i, v);
    } else {
        R[i] = v;
    }
}

// Measurement of one row: the result goes to ring slot `slot`, the measured basis is re-randomized.  With
// norand the frame keeps what the reference's frame simulator keeps when it does not randomize
// (guarantee_anticommutation_via_frame_randomization = false, frame_simulator.inl:172-317): the randomized
// component is left as it was.  Where the lowering set norand to skip randomization, the randomized
// combination provably reaches no output, so keeping it gives the same outputs as a fresh draw.
__device__ __forceinline__ void measure_row(uint32_t sub, uint4 *X, uint4 *Z, uint4 *R, uint32_t idx, uint32_t slot,
                                            uint4 r, bool rg, bool norand) {
    const uint4 x = X[idx];
    switch (sub) {
        case KM_M:
            ring_st(R, slot, x, rg);
            if (!norand) {
                Z[idx] = r;
            }
            break;
        case KM_MX:
            ring_st(R, slot, Z[idx], rg);
            if (!norand) {
                X[idx] = r;
            }
            break;
        case KM_MY: {
            const uint4 y = x4(x, Z[idx]);
            ring_st(R, slot, y, rg);
            if (!norand) {
                X[idx] = x4(y, r);
                Z[idx] = r;
            }
            break;
        }
        case KM_MR:
            ring_st(R, slot, x, rg);
            X[idx] = zero4();
            if (!norand) {
                Z[idx] = r;
            }
            break;
        case KM_MRX:
            ring_st(R, slot, Z[idx], rg);
            Z[idx] = zero4();
            if (!norand) {
                X[idx] = r;
            }
            break;
        default: {  // KM_MRY
            const uint4 z = Z[idx];
            ring_st(R, slot, x4(x, z), rg);
            if (!norand) {
                Z[idx] = r;
                X[idx] = r;
            } else {
                X[idx] = z;
            }
            break;
        }
    }
}

// Reset of one row (same norand rule as measure_row).
__device__ __forceinline__ void reset_row(uint32_t sub, uint4 *X, uint4 *Z, uint32_t idx, uint4 r, bool norand) {
    if (sub == KR_R) {
        X[idx] = zero4();
        if (!norand) {
            Z[idx] = r;
        }
    } else if (sub == KR_RX) {
        Z[idx] = zero4();
        if (!norand) {
            X[idx] = r;
        }
    } else {  // KR_RY
        if (!norand) {
            X[idx] = r;
            Z[idx] = r;
        } else {
            X[idx] = Z[idx];
        }
    }
}


// Hit record (noise_kernel -> frame kernels): bits 0..23 row (measurement flips: result index within the
// instruction), 24..47 second row (heralds: result index), 48..51 Pauli bits (X, Z on the first row, X, Z on
// the second), 52..60 shot within the slice (block * 128 + shot).
__device__ __forceinline__ uint64_t hit_record(uint32_t a, uint32_t b, uint32_t bits, uint32_t s9) {
    return (uint64_t)(a & kRowMask) | ((uint64_t)(b & kRowMask) << 24) | ((uint64_t)(bits & 15u) << 48) |
           ((uint64_t)s9 << 52);
}

// Occurrence kinds (how the frame kernel applies a record).
enum : uint32_t { OCC_PAULI = 0, OCC_FLIP, OCC_HERALD, OCC_CORR };

// First record of occurrence `occ` in this slice, and its count.
__device__ __forceinline__ const uint64_t *occ_records(const KernelArgs &p, const uint32_t *occ_off,
                                                        const uint32_t *occ_cnt, uint32_t slice, uint32_t occ,
                                                        uint32_t *count) {
    *count = occ_cnt ? occ_cnt[occ] : p.hit_count[(uint64_t)slice * p.n_occ + occ];
    return p.hits + (uint64_t)slice * p.slice_cap + (occ_off ? occ_off[occ] : p.occs[occ].off);
}

// The records this thread applies first from the next occurrence (indices tid and tid + nt), loaded one
// hit phase ahead so that their latency overlaps the gate phases in between.  Records are read through L2
// only, so that they do not evict the op lists from L1.
struct HitPre {
    uint64_t r0, r1;
};

__device__ __forceinline__ void hit_prefetch(const KernelArgs &p, const uint32_t *occ_off, const uint32_t *occ_cnt,
                                             uint32_t slice, uint32_t occ, uint32_t tid, uint32_t nt, HitPre &h) {
    h.r0 = h.r1 = 0;
    if (occ < p.n_occ) {
        uint32_t count;
        const uint64_t *r = occ_records(p, occ_off, occ_cnt, slice, occ, &count);
        const unsigned long long *rr = reinterpret_cast<const unsigned long long *>(r);
        if (tid < count) {
            h.r0 = __ldcg(rr + tid);
        }
        if (tid + nt < count) {
            h.r1 = __ldcg(rr + tid + nt);
        }
    }
}

}  // namespace gfs
