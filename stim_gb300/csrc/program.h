// Device instruction stream of the frame-sampling kernel.
//
// The host lowers a parsed circuit into this compact program once per (circuit, mode).  REPEAT blocks stay
// loops (LOOP_BEGIN / LOOP_END with a repetition count), so a 25-round surface code is ~30 ops per round
// body instead of the reference's per-iteration re-walk of the instruction list (circuit.h:180-193).
// Every op acts on "units" (targets, pairs, detectors, terms) that are independent of one another, so
// the kernel spreads units over threads and puts one CTA barrier between consecutive ops.
#pragma once

#include <cstdint>

namespace gfs {

enum OpCode : uint32_t {
    OP_END = 0,
    OP_LOOP_BEGIN,   // n = body length in ops; a,b = reps lo/hi; c,d = instances per iteration lo/hi
    OP_LOOP_END,     // n = body length in ops
    OP_1Q,           // sub = K1_*; pool[a+i] = row
    OP_2Q,           // sub = K2_*; pool[a+2i], pool[a+2i+1] = rows
    OP_FEEDBACK,     // pool[a+2i] = lookback (or kFeedbackSweep | sweep bit), pool[a+2i+1] = row | mask<<24
                     // (1 = x, 2 = z)
    OP_MEASURE,      // sub = KM_*; pool[a+i] = row; b = first randomization unit
    OP_RESET,        // sub = KR_*; pool[a+i] = row; b = first randomization unit
    OP_RECORD_ZERO,  // append n zero results (MPAD, herald slots)
    OP_MNOISE,       // flip the last n results; b = channel
    OP_NOISE,        // sub = KN_*; pool[a + i*(1 or 2)] = rows; b = channel
    OP_CORR_MASK,    // sub = 0 (E: clear the occurred flags first) / 1 (ELSE); b = channel
    OP_CORR_APPLY,   // pool[a+i] = row | xz<<24
    OP_HERALD,       // sub = 0 HERALDED_ERASE / 1 HERALDED_PAULI_CHANNEL_1; pool[a+i] = row; b = channel;
                     // the herald results are the last n results (already zeroed)
    OP_DETECTORS,    // n detectors; pool[a+i] .. pool[a+i+1] = absolute pool range of lookbacks
    OP_OBS,          // b = observable index; pool[a+i] = term (rec: k | 1<<31; Pauli: row | X<<30 | Z<<29)
    OP_EMIT,         // copy the last n results to the measurement output
};

// Noise fused into a gate op (OP_1Q, OP_2Q, OP_MEASURE, OP_RESET): DevOp c = noise after the gate,
// d = noise before it.  Bits 0..19: channel index + 1 (0 = none); bits 20..23: KN_* kind; bits 24..31:
// signed offset of the noise instruction's instance from the gate's.  The lowering fuses a noise
// instruction only into an adjacent single-run gate with the same target list, so unit u of the gate
// is unit u of the noise instruction.

enum : uint32_t { K1_H_XZ = 0, K1_H_XY, K1_H_YZ, K1_C_XYZ, K1_C_ZYX };
enum : uint32_t {
    K2_CX = 0,
    K2_CY,
    K2_CZ,
    K2_XCX,
    K2_XCY,
    K2_YCX,
    K2_YCY,
    K2_SWAP,
    K2_ISWAP,
    K2_CXSWAP,
    K2_CZSWAP,
    K2_SWAPCX,
    K2_SQRT_XX,
    K2_SQRT_YY,
    K2_SQRT_ZZ,
};
enum : uint32_t { KM_M = 0, KM_MX, KM_MY, KM_MR, KM_MRX, KM_MRY };
enum : uint32_t { KR_R = 0, KR_RX, KR_RY };
enum : uint32_t { KN_X = 0, KN_Y, KN_Z, KN_DEP1, KN_PC1, KN_DEP2, KN_PC2, KN_FLIP };
constexpr uint32_t kFusedChanMask = (1u << 20) - 1;

// DevOp.code bit: the op's gate units are also listed, in bank-friendly order, at pool[b] (OP_1Q / OP_2Q
// ops with fused noise, whose pool[a] list keeps the noise instruction's unit order).
constexpr uint32_t kGateOrderInB = 1u << 24;

// DevOp.code bit: the op also has a compact unit list at pool[g] (see DevOp.g).
constexpr uint32_t kCompact = 1u << 25;
// DevOp.code bit (OP_MEASURE / OP_RESET): the rows this op randomizes never reach a detector or observable,
// so in detection sampling the kernel may write zeros instead of drawing them (results are unchanged).
constexpr uint32_t kNoRandomize = 1u << 26;

struct alignas(16) DevOp {
    uint32_t code;  // OpCode | sub << 8 | kGateOrderInB | kCompact | kNoRandomize
    uint32_t n;
    uint32_t a, b, c, d;
    uint64_t inst;  // instance offset of the source instruction within the enclosing loop iteration
    // Compact unit list (code & kCompact), in the order the gate is applied: OP_2Q one word per pair
    // (row1 | row2 << 16); OP_1Q / OP_MEASURE / OP_RESET one 16-bit row per unit (halfword 2 * g + u);
    // OP_DETECTORS one word per detector (lookback1 | lookback2 << 16, 0 = no record).  Used when every row
    // and lookback fits 16 bits and no detector reads more than two records.
    uint32_t g;
    uint32_t pad[3];
};
static_assert(sizeof(DevOp) == 48, "DevOp layout");

// A noise channel: hit probability p (gap table) plus the Pauli choice thresholds.
struct alignas(16) DevChan {
    uint32_t table;   // offset of T[0..1024] in the table pool
    uint32_t active;  // p > 0
    uint32_t always;  // p >= 1
    float inv_c;
    uint64_t cum[16];
};

// One noise occurrence of the program (a noise op, or the noise fused before / after a gate op) met by a
// pass over the program with loops unrolled: the op, the instance it runs as, and where its hit records
// go inside a slice's region of the hit list.
struct alignas(16) NoiseOcc {
    uint32_t pc;     // op index
    uint32_t which;  // 0 noise op, 1 noise fused before the gate (op.d), 2 after it (op.c)
    uint64_t inst;   // instance of the op (loop iteration applied)
    uint32_t off;    // first record within the slice region (even, so regions start on 16 bytes)
    uint32_t cap;    // records reserved
    uint32_t xform;  // 1 + index into the lean plan's OccXform table (0: the records' Paulis as drawn)
    uint32_t pad;
};

// The lean phase list moves some hit phases earlier, across the gates they follow, so that they run next to other
// hit phases without a barrier between (lower.cc move_lean_hits).  A Pauli P applied after a gate G whose frame
// update is the linear map M equals M^-1(P) applied before G, so when the lean kernel consumes the records,
// noise_kernel writes each moved occurrence's Pauli bits transformed: first by `own` (the inverse map of the gate
// the noise is fused to, a 16-entry table of 4-bit patterns: X, Z on the first row, X, Z on the second), then for
// each of `nf` one-qubit gates crossed by the row-local inverse map ftab (four 2-bit entries) on the rows of the
// crossed gate (bitmap of rows at pool word fmem).
struct OccXform {
    uint32_t own_lo, own_hi;  // entries 0-7 and 8-15, four bits each
    uint32_t nf;
    uint32_t ftab[2];
    uint32_t fmem[2];
    uint32_t pad;
};
static_assert(sizeof(OccXform) == 32, "OccXform layout");
static_assert(sizeof(NoiseOcc) == 32, "NoiseOcc layout");

// Phase list of the lean frame kernel (frame_lean.cu): the device program re-cut into the phases the kernel
// executes, each one barrier-separated step with its fields pre-resolved, so that a phase costs one 16-byte
// shared-memory read to decode.  Noise fused into a gate becomes its own hit phase before / after the gate
// (hit-list mode only: noise_kernel has drawn the hit records).  Built by the lowering when every op has a
// lean form (see Program::lean_ok).
enum LeanKind : uint32_t {
    LK_END = 0,
    LK_LOOP_BEGIN,  // n = repetitions; a | b << 32 = instances per iteration; the body follows
    LK_LOOP_END,    // a = phase index of the matching LK_LOOP_BEGIN
    LK_HITS,        // Pauli hit records of the next noise occurrence (into X / Z rows)
    LK_FLIPS,       // measurement-flip records of the next occurrence: n = results of the noisy instruction
    LK_1Q,          // sub = K1_*; a = compact list (16-bit rows, halfword index 2a + u)
    LK_CX,          // a = compact pair list (row1 | row2 << 16)
    LK_CZ,
    LK_2Q,          // sub = K2_*, other two-qubit gates; a = compact pair list
    LK_MEAS,        // sub = KM_*; a = compact list (16-bit rows); b = first randomization unit
    LK_RESET,       // sub = KR_*; a = compact list; b = first randomization unit
    LK_ZERO,        // n zero results appended (MPAD)
    LK_DETS2,       // n detectors; a = compact list (lookback1 | lookback2 << 16)
    LK_DETS,        // n detectors; a = CSR range offsets into the pool (as OP_DETECTORS)
    LK_OBS,         // b = observable index; a = pool offset of the n terms (as OP_OBS)
    LK_EMIT,        // copy the last n results to the measurement output
    LK_FEEDBACK,    // as OP_FEEDBACK (record-controlled Paulis only)
};
constexpr uint32_t kLeanNoRandomize = 1u << 16;  // LeanPhase.op flag: write zeros instead of randomization
// LeanPhase.op flag: no barrier after this phase, because every phase that can follow it touches disjoint state
// or only XORs into the same rows (hit phases commute with one another; detector phases read the ring and write
// detection rows, disjoint from the frames that Pauli hits change).
constexpr uint32_t kLeanNoBarrier = 1u << 17;

struct alignas(16) LeanPhase {
    uint32_t op;  // LeanKind | sub << 8 | flags
    uint32_t n;
    uint32_t a;
    uint32_t b;
};
static_assert(sizeof(LeanPhase) == 16, "LeanPhase layout");

constexpr uint32_t kFeedbackX = 1, kFeedbackZ = 2;
constexpr uint32_t kFeedbackSweep = 1u << 31;  // OP_FEEDBACK source: column of the sweep table, not a lookback
constexpr uint32_t kTermRecord = 1u << 31, kTermX = 1u << 30, kTermZ = 1u << 29;
constexpr uint32_t kRowMask = (1u << 24) - 1;
constexpr int kMaxLoopDepth = 16;

}  // namespace gfs
