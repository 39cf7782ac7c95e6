/*
 * gfs_contract.h -- the random-bit contract of the GPU frame sampler.
 *
 * The reference frame simulator (src/stim/simulators/frame_simulator.inl) draws its
 * randomness from one sequential std::mt19937_64 (frame_simulator.h:60), with
 * std::geometric_distribution skipping for noise (src/stim/util_bot/probability_util.h:33-71)
 * and raw 64-bit words for stabilizer randomization (frame_simulator.inl:152-163, 172-317).
 * That stream depends on batch size, SIMD width and libstdc++, so it cannot be reproduced
 * shot-by-shot on a GPU.  This header replaces it with a counter-based stream whose every bit
 * is a pure function of (seed, instruction instance, unit index, 128-shot block), so that:
 *
 *   - a CUDA kernel, the CPU oracle, and a harness that injects the same bits into the
 *     reference's own FrameSimulator all produce identical results shot for shot;
 *   - results for a shot do not depend on how shots are sliced across CTAs, launches or GPUs.
 *
 * Definitions (all integer arithmetic; no floating point result leaks into a bit):
 *
 *   block       b = global_shot_index >> 7          (128 shots; word w of a block = shots 32w..32w+31)
 *   instance    i = index of the instruction in the circuit with every REPEAT unrolled
 *                   (adjacent fusable instructions fused exactly as the reference parser does)
 *   unit        a target (1-qubit channels), a target pair (2-qubit channels), a measurement
 *               result (noisy measurements, heralds), or the single unit of E/ELSE_CORRELATED_ERROR
 *   segment     units [16g, 16g+16) x the 128 shots of a block; trial tau = (u - 16g) * 128 + shot
 *
 *   Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
 *   SC'11) with key (lo32(seed), hi32(seed)) and counter
 *       c0 = b, c1 = segment or qubit or result, c2 = lo32(i), c3 = purpose<<28 | (bits 32..39 of i)<<20 | group
 *
 *   RESET   purpose 1: z of qubit q at the start of a shot = Philox(b, q, 0, 1<<28)
 *   RAND    purpose 2: the randomized row of result/target r of instance i = Philox(b, r, i, 2<<28)
 *   NOISE   purpose 3: a sequential stream of 32-bit draws per segment, 4 per Philox call (group 0, 1, ...)
 *   MNOISE  purpose 4: the same for measurement-result flips (M(p), MR(p), MPP(p), ...)
 *   DEM     purpose 5: detector-error-model sampling.  The error mechanisms (error instructions with REPEAT
 *           unrolled) are grouped by probability, groups numbered by first appearance and each group's
 *           mechanisms kept in model order; group j is sampled like a noise instruction of instance j whose
 *           units are its mechanisms, with segments of GFS_DEM_SEG_UNITS units (same draws otherwise).
 *
 *   A segment's hits: pos = -1; repeat { pos += 1 + G(next draw); if pos >= trials: stop; hit(pos);
 *   if the channel picks a Pauli: choice = next draw }.  G(u) = max{k : u < T[k]} with
 *   T[k] = floor((1-p)^k * 2^32) computed in 64-bit fixed point, so P(G >= k) = (1-p)^k.
 *   p == 0 draws nothing and hits nothing; p >= 1 hits every trial without gap draws.
 *   A segment is the sixteen units one GPU lane walks: at small p one Philox call per lane and segment
 *   usually decides everything, and sixteen units (2,048 trials) keep the screening calls few while a
 *   segment rarely holds more than a few hits.
 */
#ifndef GFS_CONTRACT_H
#define GFS_CONTRACT_H

#include <stdint.h>
#if !defined(__CUDA_ARCH__)
#include <math.h>
#endif

#if defined(__CUDACC__)
#define GFS_HD __host__ __device__ __forceinline__
#else
#define GFS_HD static inline
#endif

#define GFS_BLOCK_SHOTS 128u
#define GFS_SEG_UNITS 16u
#define GFS_SEG_TRIALS (GFS_BLOCK_SHOTS * GFS_SEG_UNITS)
#define GFS_TABLE_LEN (GFS_SEG_TRIALS + 1u) /* T[0..512] */

#define GFS_P_RESET 1u
#define GFS_P_RAND 2u
#define GFS_P_NOISE 3u
#define GFS_P_MNOISE 4u
#define GFS_P_DEM 5u
/* DEM segments stay at 4 mechanisms: a sampled error does several dependent global updates, and shorter
 * walks keep more lanes busy per step. */
#define GFS_DEM_SEG_UNITS 4u

typedef struct gfs_u32x4 {
    uint32_t v[4];
} gfs_u32x4;

GFS_HD uint32_t gfs_mulhi32(uint32_t a, uint32_t b) {
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

/* Philox4x32 with 10 rounds; constants from the published algorithm. */
GFS_HD gfs_u32x4 gfs_philox(uint32_t k0, uint32_t k1, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; r++) {
        uint32_t lo0 = M0 * c0, hi0 = gfs_mulhi32(M0, c0);
        uint32_t lo1 = M1 * c2, hi1 = gfs_mulhi32(M1, c2);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    gfs_u32x4 out;
    out.v[0] = c0;
    out.v[1] = c1;
    out.v[2] = c2;
    out.v[3] = c3;
    return out;
}

GFS_HD uint32_t gfs_c3(uint32_t purpose, uint64_t instance, uint32_t group) {
    return (purpose << 28) | ((uint32_t)((instance >> 32) & 0xFFu) << 20) | (group & 0xFFFFFu);
}

/* 128 random bits for a whole-row randomization (RESET or RAND purposes). */
GFS_HD gfs_u32x4 gfs_row_bits(uint64_t seed, uint32_t purpose, uint64_t instance, uint32_t unit, uint32_t block) {
    return gfs_philox((uint32_t)seed, (uint32_t)(seed >> 32), block, unit, (uint32_t)instance,
                      gfs_c3(purpose, instance, 0));
}

/* Sequential draw stream of one segment. */
typedef struct gfs_stream {
    uint32_t k0, k1, c0, c1, c2, c3base;
    uint32_t group;
    uint32_t left;              /* draws left in b0..b3 */
    uint32_t b0, b1, b2, b3;    /* next draws, in order (kept in registers: no indexed access) */
} gfs_stream;

GFS_HD void gfs_stream_init(gfs_stream *s, uint64_t seed, uint32_t purpose, uint64_t instance, uint32_t segment,
                            uint32_t block) {
    s->k0 = (uint32_t)seed;
    s->k1 = (uint32_t)(seed >> 32);
    s->c0 = block;
    s->c1 = segment;
    s->c2 = (uint32_t)instance;
    s->c3base = gfs_c3(purpose, instance, 0);
    s->group = 0;
    s->left = 0;
    s->b0 = s->b1 = s->b2 = s->b3 = 0;
}

GFS_HD uint32_t gfs_stream_next(gfs_stream *s) {
    if (s->left == 0) {
        gfs_u32x4 r = gfs_philox(s->k0, s->k1, s->c0, s->c1, s->c2, s->c3base | (s->group & 0xFFFFFu));
        s->b0 = r.v[0];
        s->b1 = r.v[1];
        s->b2 = r.v[2];
        s->b3 = r.v[3];
        s->group++;
        s->left = 4;
    }
    uint32_t out = s->b0;
    s->b0 = s->b1;
    s->b1 = s->b2;
    s->b2 = s->b3;
    s->left--;
    return out;
}

/*
 * G(u) = max{k <= maxk : u < T[k]} (T[0] = 2^32).  `est` is any starting guess; the two walks make the
 * answer exact whatever the guess.  `table` holds T[0..GFS_SEG_TRIALS] (index 0 unused).
 */
GFS_HD uint32_t gfs_gap_fixup(uint32_t u, const uint32_t *table, int32_t est, int32_t maxk) {
    int32_t k = est < 0 ? 0 : (est > maxk ? maxk : est);
    while (k < maxk && u < table[k + 1]) {
        k++;
    }
    while (k > 0 && u >= table[k]) {
        k--;
    }
    return (uint32_t)k;
}

/*
 * Next hit of a segment after position `pos` (start with pos = -1), or -1 when the segment has no
 * further hits.  `always` marks p >= 1 (every trial hits, no draws); `inv_c` = 1 / -log2(1-p) only
 * seeds the lookup, so host and device may compute it with different log2 approximations.
 */
/*
 * The hit that draw `u` selects after position `pos` with `room` = trials - pos - 1 > 0 trials left, or -1
 * when u leaves the segment.  (Split out of gfs_next_hit so that a caller holding an already drawn value can
 * continue a walk exactly.)
 */
GFS_HD int32_t gfs_hit_after_draw(uint32_t u, const uint32_t *table, float inv_c, int32_t pos, int32_t room) {
    if (u < table[room]) {
        return -1;
    }
#if defined(__CUDA_ARCH__)
    float lg = __log2f((float)u + 0.5f);
#else
    float lg = log2f((float)u + 0.5f);
#endif
    float e = (32.0f - lg) * inv_c;
    if (!(e >= 0.0f)) { /* also catches NaN */
        e = 0.0f;
    }
    if (e > (float)room) {
        e = (float)room;
    }
    uint32_t g = gfs_gap_fixup(u, table, (int32_t)e, room - 1);
    return pos + 1 + (int32_t)g;
}

/*
 * Next hit of a segment after position `pos` (start with pos = -1), or -1 when the segment has no
 * further hits.  `always` marks p >= 1 (every trial hits, no draws); `inv_c` = 1 / -log2(1-p) only
 * seeds the lookup, so host and device may compute it with different log2 approximations.
 */
GFS_HD int32_t gfs_next_hit(gfs_stream *s, const uint32_t *table, float inv_c, int32_t pos, int32_t trials,
                            int always) {
    if (always) {
        return pos + 1 < trials ? pos + 1 : -1;
    }
    int32_t room = trials - pos - 1; /* a gap >= room leaves the segment */
    if (room <= 0) {
        return -1;
    }
    return gfs_hit_after_draw(gfs_stream_next(s), table, inv_c, pos, room);
}

/* Choice helpers. */
GFS_HD uint32_t gfs_choice_uniform(uint32_t c, uint32_t n) {
    return gfs_mulhi32(c, n);
}

/* Outcome index of a weighted choice: the first k with c < cum[k]; cum[n-1] == 2^32. */
GFS_HD uint32_t gfs_choice_weighted(uint32_t c, const uint64_t *cum, uint32_t n) {
    uint32_t k = 0;
    while (k + 1 < n && (uint64_t)c >= cum[k]) {
        k++;
    }
    return k;
}

#if !defined(__CUDA_ARCH__)
/*
 * Host-only: the threshold table T[0..GFS_SEG_TRIALS] for probability p in (0, 1).
 * (1-p) is converted once to 0.64 fixed point; powers are formed by 64x64->128 multiplies,
 * so every platform computes the same table from the same double p.
 */
static inline void gfs_build_gap_table(double p, uint32_t *table) {
    double q = 1.0 - p;
    uint64_t Q;
    if (q >= 1.0) {
        Q = UINT64_MAX;
    } else if (q <= 0.0) {
        Q = 0;
    } else {
        double scaled = q * 18446744073709551616.0; /* exact: multiply by 2^64 */
        Q = scaled >= 18446744073709551615.0 ? UINT64_MAX : (uint64_t)scaled;
    }
    uint64_t A = UINT64_MAX;
    table[0] = UINT32_MAX;
    for (uint32_t k = 1; k <= GFS_SEG_TRIALS; k++) {
        A = (uint64_t)(((unsigned __int128)A * (unsigned __int128)Q) >> 64);
        table[k] = (uint32_t)(A >> 32);
    }
}

/* Seed for the gap lookup: 1 / -log2(1-p), kept finite. */
static inline float gfs_inv_c(double p) {
    double c = -log2(1.0 - p);
    if (!(c > 1e-9)) {
        return 1e9f;
    }
    double v = 1.0 / c;
    return v > 1e9 ? 1e9f : (float)v;
}

/* Cumulative choice thresholds for weights w[0..n-1] (n <= 16); the last is 2^32. */
static inline void gfs_build_choice_table(const double *w, uint32_t n, uint64_t *cum) {
    double total = 0;
    for (uint32_t k = 0; k < n; k++) {
        total += w[k];
    }
    double acc = 0;
    for (uint32_t k = 0; k < n; k++) {
        acc += w[k];
        double frac = total > 0 ? acc / total : 0.0;
        double scaled = frac * 4294967296.0;
        uint64_t v = scaled >= 4294967296.0 ? (uint64_t)1 << 32 : (uint64_t)scaled;
        cum[k] = v;
    }
    if (n > 0) {
        cum[n - 1] = (uint64_t)1 << 32;
    }
}
#endif

#endif /* GFS_CONTRACT_H */
