// Lowering of a parsed circuit into the device program.
//
// Decompositions follow the reference exactly where they change which frame bits exist at a
// randomization point: MPP (gate_decomposition.cc:88-161), SPP/SPP_DAG (gate_decomposition.cc:163-250),
// MXX/MYY/MZZ (frame_simulator.inl:841-902 with decompose_pair_instruction_into_disjoint_segments,
// gate_decomposition.cc:319-347).  Instructions whose targets repeat are split into runs of distinct
// targets so the kernel may process every unit of an op in parallel with the reference's sequential
// result (frame_simulator.inl:278 notes the same hazard for MR).
#include "lower.h"

#include <algorithm>
#include <cmath>
#include <functional>
#include <iterator>
#include <map>
#include <stdexcept>
#include <unordered_map>
#include <unordered_set>

#include "frame_rules.h"
#include "gfs_contract.h"

namespace gfs {
namespace {

struct Lowerer {
    const Circuit &root;
    SampleMode mode;
    Program prog;
    std::vector<int32_t> row_of;  // qubit -> row
    std::map<std::vector<double>, uint32_t> chan_cache;
    uint64_t meas_seen = 0;  // results before this point on the first pass through every loop
    uint64_t mult = 1;       // product of the repetition counts of the enclosing loops
    uint64_t dets_unrolled = 0;
    uint64_t max_results_per_inst = 0;

    // pending detector group
    std::vector<std::vector<uint32_t>> pending_dets;
    uint64_t pending_inst = 0;

    LowerOptions opts;

    // The op and the noise slot (0 noise op, 1 fused before the gate, 2 after it) of each lean phase.
    std::vector<uint32_t> lean_pc, lean_which;

    Lowerer(const Circuit &c, SampleMode m, const LowerOptions &o) : root(c), mode(m), opts(o) {
    }

    uint32_t row(uint32_t t) const {
        return (uint32_t)row_of[t & GFS_T_VALUE_MASK];
    }

    // OP_FEEDBACK source word of sweep target `t` (LowerOptions::sweep).
    uint32_t sweep_source(uint32_t t) {
        const uint32_t k = t & GFS_T_VALUE_MASK;
        if (k >= kFeedbackSweep) {
            throw std::invalid_argument("sweep bit index too large for the GPU frame sampler");
        }
        prog.num_sweep_bits = std::max<uint64_t>(prog.num_sweep_bits, (uint64_t)k + 1);
        return kFeedbackSweep | k;
    }

    void collect_qubits(const Circuit &c, std::vector<uint8_t> &used) {
        for (const auto &op : c.ops) {
            if (op.gate == GFS_REPEAT) {
                collect_qubits(c.blocks[op.block], used);
                continue;
            }
            if (op.gate == GFS_MPAD) {
                continue;
            }
            for (auto t : op.targets) {
                if (t & (GFS_T_RECORD | GFS_T_SWEEP | GFS_T_COMBINER)) {
                    continue;
                }
                used[t & GFS_T_VALUE_MASK] = 1;
            }
        }
    }

    uint32_t channel(double p, const std::vector<double> &weights) {
        std::vector<double> key = weights;
        key.push_back(p);
        auto it = chan_cache.find(key);
        if (it != chan_cache.end()) {
            return it->second;
        }
        DevChan ch{};
        ch.active = p > 0;
        ch.always = p >= 1;
        ch.table = 0;
        ch.inv_c = 0;
        if (ch.active && !ch.always) {
            ch.table = (uint32_t)prog.tables.size();
            prog.tables.resize(prog.tables.size() + GFS_TABLE_LEN);
            gfs_build_gap_table(p, prog.tables.data() + ch.table);
            ch.inv_c = gfs_inv_c(p);
        }
        if (!weights.empty()) {
            gfs_build_choice_table(weights.data(), (uint32_t)weights.size(), ch.cum);
        }
        uint32_t id = (uint32_t)prog.chans.size();
        prog.chans.push_back(ch);
        prog.chan_p.push_back(p);
        chan_cache[key] = id;
        return id;
    }

    DevOp &emit(uint32_t code, uint32_t sub, uint32_t n, uint64_t inst) {
        DevOp op{};
        op.code = code | (sub << 8);
        op.n = n;
        op.a = (uint32_t)prog.pool.size();
        op.inst = inst;
        prog.ops.push_back(op);
        // Cost estimate per 128-shot block: units processed plus a fixed per-op overhead, times repetitions.
        const double w = ((double)n + 64.0) * (double)mult;
        prog.work = prog.work + w > 1e18 ? 1e18 : prog.work + w;
        return prog.ops.back();
    }

    void check_lookback(uint32_t k) {
        if (k == 0) {
            throw std::out_of_range("Lookback must be non-zero.");
        }
        if (k > meas_seen) {
            throw std::out_of_range("Referred to a measurement record before the beginning of time.");
        }
    }

    // Whether every record target of a detector / observable instruction reads a result already recorded.
    bool lookbacks_valid(const Instruction &op) const {
        for (auto t : op.targets) {
            const uint32_t k = t & GFS_T_VALUE_MASK;
            if (((op.gate == GFS_DETECTOR) || (t & GFS_T_RECORD)) && (k == 0 || k > meas_seen)) {
                return false;
            }
        }
        return true;
    }

    // ---- runs of distinct rows ----
    template <typename F>
    void distinct_runs(const std::vector<uint32_t> &rows, size_t stride, F flush) {
        std::unordered_set<uint32_t> seen;
        size_t start = 0;
        for (size_t k = 0; k < rows.size(); k += stride) {
            bool clash = false;
            for (size_t j = 0; j < stride; j++) {
                if (seen.count(rows[k + j])) {
                    clash = true;
                }
            }
            if (clash) {
                flush(start, k);
                seen.clear();
                start = k;
            }
            for (size_t j = 0; j < stride; j++) {
                seen.insert(rows[k + j]);
            }
        }
        if (start < rows.size()) {
            flush(start, rows.size());
        }
    }

    void emit_1q(uint32_t sub, const std::vector<uint32_t> &rows, uint64_t inst) {
        distinct_runs(rows, 1, [&](size_t a, size_t b) {
            emit(OP_1Q, sub, (uint32_t)(b - a), inst);
            prog.pool.insert(prog.pool.end(), rows.begin() + a, rows.begin() + b);
        });
    }

    void emit_2q(uint32_t sub, const std::vector<uint32_t> &rows, uint64_t inst) {
        distinct_runs(rows, 2, [&](size_t a, size_t b) {
            emit(OP_2Q, sub, (uint32_t)((b - a) / 2), inst);
            prog.pool.insert(prog.pool.end(), rows.begin() + a, rows.begin() + b);
        });
    }

    void emit_measure(uint32_t sub, const std::vector<uint32_t> &rows, uint32_t unit0, uint64_t inst) {
        distinct_runs(rows, 1, [&](size_t a, size_t b) {
            DevOp &op = emit(OP_MEASURE, sub, (uint32_t)(b - a), inst);
            op.b = unit0 + (uint32_t)a;
            prog.pool.insert(prog.pool.end(), rows.begin() + a, rows.begin() + b);
        });
    }

    void emit_results_tail(const Instruction &op, uint64_t nres, uint64_t inst) {
        if (!op.args.empty() && op.args[0] > 0 && nres) {
            DevOp &d = emit(OP_MNOISE, 0, (uint32_t)nres, inst);
            d.b = channel(op.args[0], {});
        }
        if (mode == SampleMode::MEASUREMENTS && nres) {
            emit(OP_EMIT, 0, (uint32_t)nres, inst);
        }
        meas_seen += nres;
        max_results_per_inst = std::max(max_results_per_inst, nres);
    }

    void flush_detectors() {
        if (pending_dets.empty()) {
            return;
        }
        uint32_t n = (uint32_t)pending_dets.size();
        emit(OP_DETECTORS, 0, n, pending_inst);
        size_t base = prog.pool.size();
        prog.pool.resize(base + n + 1);
        for (uint32_t i = 0; i < n; i++) {
            prog.pool[base + i] = (uint32_t)prog.pool.size();
            prog.pool.insert(prog.pool.end(), pending_dets[i].begin(), pending_dets[i].end());
        }
        prog.pool[base + n] = (uint32_t)prog.pool.size();
        dets_unrolled += (uint64_t)n * mult;
        pending_dets.clear();
    }

    // ---- two-qubit gates with classical controls ----
    void lower_two_qubit(const Instruction &op, uint64_t inst) {
        uint32_t sub = 0;
        bool reverse = false;
        switch (op.gate) {
            case GFS_CX: sub = K2_CX; break;
            case GFS_CY: sub = K2_CY; break;
            case GFS_CZ: sub = K2_CZ; break;
            case GFS_XCZ: sub = K2_CX; reverse = true; break;
            case GFS_YCZ: sub = K2_CY; reverse = true; break;
            case GFS_XCX: sub = K2_XCX; break;
            case GFS_XCY: sub = K2_XCY; break;
            case GFS_YCX: sub = K2_YCX; break;
            case GFS_YCY: sub = K2_YCY; break;
            case GFS_SWAP: sub = K2_SWAP; break;
            case GFS_ISWAP:
            case GFS_ISWAP_DAG: sub = K2_ISWAP; break;
            case GFS_CXSWAP: sub = K2_CXSWAP; break;
            case GFS_SWAPCX: sub = K2_SWAPCX; break;
            case GFS_CZSWAP: sub = K2_CZSWAP; break;
            case GFS_SQRT_XX:
            case GFS_SQRT_XX_DAG: sub = K2_SQRT_XX; break;
            case GFS_SQRT_YY:
            case GFS_SQRT_YY_DAG: sub = K2_SQRT_YY; break;
            case GFS_SQRT_ZZ:
            case GFS_SQRT_ZZ_DAG: sub = K2_SQRT_ZZ; break;
            default: throw std::invalid_argument("not a two-qubit gate");
        }
        // Split into runs; a run is either all quantum pairs or all feedback, with distinct rows.
        std::vector<uint32_t> qrows;
        std::vector<uint32_t> fb;  // lookback, row|mask
        std::unordered_set<uint32_t> seen;
        auto flush = [&]() {
            if (!qrows.empty()) {
                emit(OP_2Q, sub, (uint32_t)(qrows.size() / 2), inst);
                prog.pool.insert(prog.pool.end(), qrows.begin(), qrows.end());
                qrows.clear();
            }
            if (!fb.empty()) {
                emit(OP_FEEDBACK, 0, (uint32_t)(fb.size() / 2), inst);
                prog.pool.insert(prog.pool.end(), fb.begin(), fb.end());
                fb.clear();
            }
            seen.clear();
        };
        for (size_t k = 0; k < op.targets.size(); k += 2) {
            uint32_t c = op.targets[k] & ~GFS_T_INVERTED, t = op.targets[k + 1] & ~GFS_T_INVERTED;
            if (reverse) {
                std::swap(c, t);
            }
            bool cb = c & (GFS_T_RECORD | GFS_T_SWEEP), tb = t & (GFS_T_RECORD | GFS_T_SWEEP);
            if (!cb && !tb) {
                uint32_t r1 = row(c), r2 = row(t);
                if (!fb.empty() || seen.count(r1) || seen.count(r2)) {
                    flush();
                }
                seen.insert(r1);
                seen.insert(r2);
                qrows.push_back(r1);
                qrows.push_back(r2);
                continue;
            }
            uint32_t bit, q, mask;
            if (sub == K2_CZ) {
                if (cb && tb) {
                    continue;  // both classical: no effect
                }
                bit = cb ? c : t;
                q = cb ? t : c;
                mask = kFeedbackZ;
            } else if (tb) {
                throw std::invalid_argument(std::string(sub == K2_CX ? "Controlled X" : "Controlled Y") +
                                            " had a bit as its target, instead of its control.");
            } else {
                bit = c;
                q = t;
                mask = sub == K2_CX ? kFeedbackX : (kFeedbackX | kFeedbackZ);
            }
            uint32_t src;
            if (bit & GFS_T_SWEEP) {
                if (!opts.sweep) {
                    continue;  // sweep bits read as zero in the samplers
                }
                src = sweep_source(bit);
            } else {
                src = bit & GFS_T_VALUE_MASK;
                check_lookback(src);
            }
            uint32_t r = row(q);
            if (!qrows.empty() || seen.count(r)) {
                flush();
            }
            seen.insert(r);
            fb.push_back(src);
            fb.push_back(r | (mask << 24));
        }
        flush();
    }

    // ---- Pauli products (MPP, SPP) ----
    struct Product {
        std::vector<uint32_t> qubits;  // sorted, active
        std::vector<uint8_t> x, z;
        std::vector<uint32_t> bits;
    };

    std::vector<Product> read_products(const Instruction &op, const char *gname) {
        std::vector<Product> out;
        size_t k = 0;
        while (k < op.targets.size()) {
            size_t end = k + 1;
            while (end < op.targets.size() && (op.targets[end] & GFS_T_COMBINER)) {
                end += 2;
            }
            std::map<uint32_t, std::pair<uint8_t, uint8_t>> acc;
            bool imag = false;
            Product p;
            for (size_t j = k; j < end; j += 2) {
                uint32_t t = op.targets[j];
                if (t & (GFS_T_PAULI_X | GFS_T_PAULI_Z)) {
                    uint32_t q = t & GFS_T_VALUE_MASK;
                    uint8_t nx = (t & GFS_T_PAULI_X) ? 1 : 0, nz = (t & GFS_T_PAULI_Z) ? 1 : 0;
                    auto &e = acc[q];
                    if ((e.first & nz) ^ (e.second & nx)) {
                        imag = !imag;
                    }
                    e.first ^= nx;
                    e.second ^= nz;
                } else if (t & (GFS_T_RECORD | GFS_T_SWEEP)) {
                    p.bits.push_back(t);
                } else {
                    throw std::invalid_argument(std::string("Found an unsupported target in ") + gname + ".");
                }
            }
            if (imag) {
                throw std::invalid_argument(std::string("Acted on an anti-Hermitian operator (e.g. X0*Z0 instead of Y0) in ") +
                                            gname + ".");
            }
            for (auto &e : acc) {
                if (e.second.first || e.second.second) {
                    p.qubits.push_back(e.first);
                    p.x.push_back(e.second.first);
                    p.z.push_back(e.second.second);
                }
            }
            out.push_back(std::move(p));
            k = end;
        }
        return out;
    }

    // Emits the CX pairs (control, target) as layers in which every row appears at most once.  All
    // pairs passed here commute with one another (distinct controls, targets never controls).
    void emit_cx_layers(const std::vector<std::pair<uint32_t, uint32_t>> &pairs, uint64_t inst) {
        std::vector<std::pair<uint32_t, uint32_t>> rest = pairs;
        while (!rest.empty()) {
            std::unordered_set<uint32_t> used;
            std::vector<uint32_t> layer;
            std::vector<std::pair<uint32_t, uint32_t>> next;
            for (auto &pr : rest) {
                if (used.count(pr.first) || used.count(pr.second)) {
                    next.push_back(pr);
                } else {
                    used.insert(pr.first);
                    used.insert(pr.second);
                    layer.push_back(pr.first);
                    layer.push_back(pr.second);
                }
            }
            emit(OP_2Q, K2_CX, (uint32_t)(layer.size() / 2), inst);
            prog.pool.insert(prog.pool.end(), layer.begin(), layer.end());
            rest.swap(next);
        }
    }

    void lower_mpp(const Instruction &op, uint64_t inst) {
        auto prods = read_products(op, "MPP");
        uint32_t result = 0;
        std::vector<uint32_t> hxz, hyz, meas;
        std::vector<std::pair<uint32_t, uint32_t>> cnot;
        std::unordered_set<uint32_t> merged;
        uint32_t group_first = 0;
        auto flush = [&]() {
            if (meas.empty()) {
                return;
            }
            if (!hxz.empty()) emit_1q(K1_H_XZ, hxz, inst);
            if (!hyz.empty()) emit_1q(K1_H_YZ, hyz, inst);
            if (!cnot.empty()) emit_cx_layers(cnot, inst);
            emit_measure(KM_M, meas, group_first, inst);
            if (!cnot.empty()) emit_cx_layers(cnot, inst);
            if (!hyz.empty()) emit_1q(K1_H_YZ, hyz, inst);
            if (!hxz.empty()) emit_1q(K1_H_XZ, hxz, inst);
            hxz.clear();
            hyz.clear();
            meas.clear();
            cnot.clear();
            merged.clear();
        };
        for (auto &p : prods) {
            if (p.qubits.empty()) {
                flush();
                emit(OP_RECORD_ZERO, 0, 1, inst);
                result++;
                continue;
            }
            bool overlap = false;
            for (auto q : p.qubits) {
                overlap |= merged.count(q) > 0;
            }
            if (overlap) {
                flush();
            }
            if (meas.empty()) {
                group_first = result;
            }
            for (size_t j = 0; j < p.qubits.size(); j++) {
                uint32_t r = row_of[p.qubits[j]];
                merged.insert(p.qubits[j]);
                if (p.x[j]) {
                    (p.z[j] ? hyz : hxz).push_back(r);
                }
                if (j == 0) {
                    meas.push_back(r);
                } else {
                    cnot.push_back({r, (uint32_t)row_of[p.qubits[0]]});
                }
            }
            result++;
        }
        flush();
        emit_results_tail(op, result, inst);
    }

    void lower_spp(const Instruction &op, uint64_t inst) {
        auto prods = read_products(op, op.gate == GFS_SPP ? "SPP" : "SPP_DAG");
        for (auto &p : prods) {
            if (p.qubits.empty()) {
                continue;
            }
            std::vector<uint32_t> hxz, hyz;
            uint32_t focus = (uint32_t)row_of[p.qubits[0]];
            for (size_t j = 0; j < p.qubits.size(); j++) {
                uint32_t r = row_of[p.qubits[j]];
                if (p.x[j]) {
                    (p.z[j] ? hyz : hxz).push_back(r);
                }
            }
            auto cx_all = [&]() {
                for (size_t j = 1; j < p.qubits.size(); j++) {
                    emit(OP_2Q, K2_CX, 1, inst);
                    prog.pool.push_back((uint32_t)row_of[p.qubits[j]]);
                    prog.pool.push_back(focus);
                }
                for (auto b : p.bits) {
                    uint32_t src;
                    if (b & GFS_T_SWEEP) {
                        if (!opts.sweep) {
                            continue;
                        }
                        src = sweep_source(b);
                    } else {
                        src = b & GFS_T_VALUE_MASK;
                        check_lookback(src);
                    }
                    emit(OP_FEEDBACK, 0, 1, inst);
                    prog.pool.push_back(src);
                    prog.pool.push_back(focus | (kFeedbackX << 24));
                }
            };
            if (!hxz.empty()) emit_1q(K1_H_XZ, hxz, inst);
            if (!hyz.empty()) emit_1q(K1_H_YZ, hyz, inst);
            cx_all();
            emit_1q(K1_H_XY, {focus}, inst);
            cx_all();
            if (!hyz.empty()) emit_1q(K1_H_YZ, hyz, inst);
            if (!hxz.empty()) emit_1q(K1_H_XZ, hxz, inst);
        }
    }

    void lower_pair_measure(const Instruction &op, uint64_t inst) {
        uint32_t conj = op.gate == GFS_MYY ? K2_CY : K2_CX;
        bool reverse = op.gate == GFS_MZZ;
        uint32_t mk = op.gate == GFS_MXX ? KM_MX : op.gate == GFS_MYY ? KM_MY : KM_M;
        uint32_t result = 0;
        std::unordered_set<uint32_t> used;
        size_t flushed = 0;
        auto flush = [&](size_t end) {
            std::vector<uint32_t> pr, first;
            for (size_t k = flushed; k < end; k += 2) {
                uint32_t a = row(op.targets[k]), b = row(op.targets[k + 1]);
                if (reverse) {
                    pr.push_back(b);
                    pr.push_back(a);
                } else {
                    pr.push_back(a);
                    pr.push_back(b);
                }
                first.push_back(a);
            }
            emit_2q(conj, pr, inst);
            emit_measure(mk, first, result, inst);
            emit_2q(conj, pr, inst);
            result += (uint32_t)first.size();
            used.clear();
            flushed = end;
        };
        for (size_t k = 0; k < op.targets.size(); k += 2) {
            uint32_t q0 = op.targets[k] & GFS_T_VALUE_MASK, q1 = op.targets[k + 1] & GFS_T_VALUE_MASK;
            if (used.count(q0) || used.count(q1)) {
                flush(k);
            }
            used.insert(q0);
            used.insert(q1);
        }
        if (flushed < op.targets.size()) {
            flush(op.targets.size());
        }
        emit_results_tail(op, result, inst);
    }

    // ---- noise fused into adjacent gates ----
    struct Fuse {
        const Instruction *pre = nullptr;   // noise instruction just before the gate (instance inst - 1)
        const Instruction *post = nullptr;  // noise instruction just after it (instance inst + 1)
    };

    static bool noise_1q(gfs_gate g) {
        return g == GFS_X_ERROR || g == GFS_Y_ERROR || g == GFS_Z_ERROR || g == GFS_DEPOLARIZE1 ||
               g == GFS_PAULI_CHANNEL_1;
    }
    static bool noise_2q(gfs_gate g) {
        return g == GFS_DEPOLARIZE2 || g == GFS_PAULI_CHANNEL_2;
    }
    static bool gate_1q_fusable(gfs_gate g) {
        switch (g) {
            case GFS_H: case GFS_H_NXZ: case GFS_SQRT_Y: case GFS_SQRT_Y_DAG: case GFS_S: case GFS_S_DAG:
            case GFS_H_XY: case GFS_H_NXY: case GFS_SQRT_X: case GFS_SQRT_X_DAG: case GFS_H_YZ: case GFS_H_NYZ:
            case GFS_C_XYZ: case GFS_C_NXYZ: case GFS_C_XNYZ: case GFS_C_XYNZ: case GFS_C_ZYX: case GFS_C_NZYX:
            case GFS_C_ZNYX: case GFS_C_ZYNX: case GFS_M: case GFS_MX: case GFS_MY: case GFS_MR: case GFS_MRX:
            case GFS_MRY: case GFS_R: case GFS_RX: case GFS_RY:
                return true;
            default:
                return false;
        }
    }
    static bool gate_2q_fusable(gfs_gate g) {
        switch (g) {
            case GFS_CX: case GFS_CY: case GFS_CZ: case GFS_XCX: case GFS_XCY: case GFS_YCX: case GFS_YCY:
            case GFS_SWAP: case GFS_ISWAP: case GFS_ISWAP_DAG: case GFS_CXSWAP: case GFS_SWAPCX: case GFS_CZSWAP:
            case GFS_SQRT_XX: case GFS_SQRT_XX_DAG: case GFS_SQRT_YY: case GFS_SQRT_YY_DAG: case GFS_SQRT_ZZ:
            case GFS_SQRT_ZZ_DAG:
                return true;
            default:
                return false;
        }
    }

    static double noise_p(const Instruction &n) {
        if (n.gate == GFS_PAULI_CHANNEL_1 || n.gate == GFS_PAULI_CHANNEL_2) {
            double p = 0;
            for (double w : n.args) p += w;
            return p;
        }
        return n.args.empty() ? 0.0 : n.args[0];
    }

    // Whether noise instruction `n` may be fused into gate instruction `g` (same units, distinct rows).
    bool fusable(const Instruction &n, const Instruction &g) const {
        if (!(noise_p(n) > 0)) {
            return false;
        }
        bool one = noise_1q(n.gate) && gate_1q_fusable(g.gate);
        bool two = noise_2q(n.gate) && gate_2q_fusable(g.gate);
        if (!one && !two) {
            return false;
        }
        if (n.targets.size() != g.targets.size()) {
            return false;
        }
        std::unordered_set<uint32_t> seen;
        for (size_t k = 0; k < g.targets.size(); k++) {
            uint32_t gt = g.targets[k] & ~GFS_T_INVERTED, nt = n.targets[k];
            if (gt != nt || (gt & (GFS_T_RECORD | GFS_T_SWEEP | GFS_T_COMBINER))) {
                return false;
            }
            if (!seen.insert(gt).second) {
                return false;
            }
        }
        return true;
    }

    uint32_t fused_word(const Instruction *n, int delta) {
        if (!n) {
            return 0;
        }
        uint32_t kind;
        std::vector<double> weights;
        switch (n->gate) {
            case GFS_X_ERROR: kind = KN_X; break;
            case GFS_Y_ERROR: kind = KN_Y; break;
            case GFS_Z_ERROR: kind = KN_Z; break;
            case GFS_DEPOLARIZE1: kind = KN_DEP1; break;
            case GFS_DEPOLARIZE2: kind = KN_DEP2; break;
            case GFS_PAULI_CHANNEL_1: kind = KN_PC1; weights = n->args; break;
            default: kind = KN_PC2; weights = n->args; break;
        }
        uint32_t ch = channel(noise_p(*n), weights);
        if (ch + 1 > kFusedChanMask) {
            throw std::invalid_argument("too many distinct noise channels for the GPU frame sampler");
        }
        return (ch + 1) | (kind << 20) | ((uint32_t)(uint8_t)(int8_t)delta << 24);
    }

    // Emits a gate instruction with fused noise as a single op.
    void lower_fused(const Instruction &op, uint64_t inst, const Fuse &f) {
        std::vector<uint32_t> rows;
        for (auto t : op.targets) {
            rows.push_back(row(t));
        }
        uint32_t code, sub;
        uint32_t n = (uint32_t)rows.size();
        gfs_gate g = op.gate;
        if (gate_2q_fusable(g)) {
            code = OP_2Q;
            n /= 2;
            switch (g) {
                case GFS_CX: sub = K2_CX; break;
                case GFS_CY: sub = K2_CY; break;
                case GFS_CZ: sub = K2_CZ; break;
                case GFS_XCX: sub = K2_XCX; break;
                case GFS_XCY: sub = K2_XCY; break;
                case GFS_YCX: sub = K2_YCX; break;
                case GFS_YCY: sub = K2_YCY; break;
                case GFS_SWAP: sub = K2_SWAP; break;
                case GFS_ISWAP: case GFS_ISWAP_DAG: sub = K2_ISWAP; break;
                case GFS_CXSWAP: sub = K2_CXSWAP; break;
                case GFS_SWAPCX: sub = K2_SWAPCX; break;
                case GFS_CZSWAP: sub = K2_CZSWAP; break;
                case GFS_SQRT_XX: case GFS_SQRT_XX_DAG: sub = K2_SQRT_XX; break;
                case GFS_SQRT_YY: case GFS_SQRT_YY_DAG: sub = K2_SQRT_YY; break;
                default: sub = K2_SQRT_ZZ; break;
            }
        } else {
            switch (g) {
                case GFS_H: case GFS_H_NXZ: case GFS_SQRT_Y: case GFS_SQRT_Y_DAG: code = OP_1Q; sub = K1_H_XZ; break;
                case GFS_S: case GFS_S_DAG: case GFS_H_XY: case GFS_H_NXY: code = OP_1Q; sub = K1_H_XY; break;
                case GFS_SQRT_X: case GFS_SQRT_X_DAG: case GFS_H_YZ: case GFS_H_NYZ: code = OP_1Q; sub = K1_H_YZ; break;
                case GFS_C_XYZ: case GFS_C_NXYZ: case GFS_C_XNYZ: case GFS_C_XYNZ: code = OP_1Q; sub = K1_C_XYZ; break;
                case GFS_C_ZYX: case GFS_C_NZYX: case GFS_C_ZNYX: case GFS_C_ZYNX: code = OP_1Q; sub = K1_C_ZYX; break;
                case GFS_M: code = OP_MEASURE; sub = KM_M; break;
                case GFS_MX: code = OP_MEASURE; sub = KM_MX; break;
                case GFS_MY: code = OP_MEASURE; sub = KM_MY; break;
                case GFS_MR: code = OP_MEASURE; sub = KM_MR; break;
                case GFS_MRX: code = OP_MEASURE; sub = KM_MRX; break;
                case GFS_MRY: code = OP_MEASURE; sub = KM_MRY; break;
                case GFS_R: code = OP_RESET; sub = KR_R; break;
                case GFS_RX: code = OP_RESET; sub = KR_RX; break;
                default: code = OP_RESET; sub = KR_RY; break;
            }
        }
        uint32_t post = fused_word(f.post, +1), pre = fused_word(f.pre, -1);
        DevOp &d = emit(code, sub, n, inst);
        d.b = 0;
        d.c = post;
        d.d = pre;
        prog.pool.insert(prog.pool.end(), rows.begin(), rows.end());
        if (code == OP_MEASURE) {
            emit_results_tail(op, n, inst);
        }
    }

    void lower_instruction(const Instruction &op, uint64_t inst) {
        gfs_gate g = op.gate;
        if (g == GFS_DETECTOR) {
            // Sampling measurements, the reference never evaluates detectors or observables (frame_simulator.inl
            // :222-252 keep no detection data), so one that reads a record before the beginning of time is left
            // out instead of rejected; detection sampling rejects it as the reference does.
            if (mode == SampleMode::MEASUREMENTS && !lookbacks_valid(op)) {
                return;
            }
            if (pending_dets.empty()) {
                pending_inst = inst;
            }
            std::vector<uint32_t> lbs;
            for (auto t : op.targets) {
                uint32_t k = t & GFS_T_VALUE_MASK;
                check_lookback(k);
                lbs.push_back(k);
            }
            pending_dets.push_back(std::move(lbs));
            return;
        }
        switch (g) {
            case GFS_TICK:
            case GFS_QUBIT_COORDS:
            case GFS_SHIFT_COORDS:
            case GFS_I:
            case GFS_X:
            case GFS_Y:
            case GFS_Z:
            case GFS_II:
            case GFS_I_ERROR:
            case GFS_II_ERROR:
                return;
            default:
                break;
        }
        if (g == GFS_OBSERVABLE_INCLUDE) {
            if (mode == SampleMode::MEASUREMENTS && !lookbacks_valid(op)) {
                return;  // as for detectors above
            }
            uint32_t k_obs = (uint32_t)op.args[0];
            std::vector<uint32_t> terms;
            for (auto t : op.targets) {
                if (t & GFS_T_RECORD) {
                    check_lookback(t & GFS_T_VALUE_MASK);
                    terms.push_back((t & GFS_T_VALUE_MASK) | kTermRecord);
                } else {
                    uint32_t term = row(t);
                    if (t & GFS_T_PAULI_X) term |= kTermX;
                    if (t & GFS_T_PAULI_Z) term |= kTermZ;
                    terms.push_back(term);
                }
            }
            if (!terms.empty()) {
                DevOp &d = emit(OP_OBS, 0, (uint32_t)terms.size(), inst);
                d.b = k_obs;
                prog.pool.insert(prog.pool.end(), terms.begin(), terms.end());
            }
            return;
        }
        flush_detectors();
        std::vector<uint32_t> rows;
        for (auto t : op.targets) {
            if (!(t & (GFS_T_RECORD | GFS_T_SWEEP | GFS_T_COMBINER))) {
                rows.push_back(row(t));
            }
        }
        switch (g) {
            case GFS_H:
            case GFS_H_NXZ:
            case GFS_SQRT_Y:
            case GFS_SQRT_Y_DAG:
                emit_1q(K1_H_XZ, rows, inst);
                return;
            case GFS_S:
            case GFS_S_DAG:
            case GFS_H_XY:
            case GFS_H_NXY:
                emit_1q(K1_H_XY, rows, inst);
                return;
            case GFS_SQRT_X:
            case GFS_SQRT_X_DAG:
            case GFS_H_YZ:
            case GFS_H_NYZ:
                emit_1q(K1_H_YZ, rows, inst);
                return;
            case GFS_C_XYZ:
            case GFS_C_NXYZ:
            case GFS_C_XNYZ:
            case GFS_C_XYNZ:
                emit_1q(K1_C_XYZ, rows, inst);
                return;
            case GFS_C_ZYX:
            case GFS_C_NZYX:
            case GFS_C_ZNYX:
            case GFS_C_ZYNX:
                emit_1q(K1_C_ZYX, rows, inst);
                return;
            case GFS_M:
            case GFS_MX:
            case GFS_MY:
            case GFS_MR:
            case GFS_MRX:
            case GFS_MRY: {
                uint32_t sub = g == GFS_M    ? KM_M
                               : g == GFS_MX ? KM_MX
                               : g == GFS_MY ? KM_MY
                               : g == GFS_MR ? KM_MR
                               : g == GFS_MRX ? KM_MRX
                                              : KM_MRY;
                emit_measure(sub, rows, 0, inst);
                emit_results_tail(op, rows.size(), inst);
                return;
            }
            case GFS_R:
            case GFS_RX:
            case GFS_RY: {
                uint32_t sub = g == GFS_R ? KR_R : g == GFS_RX ? KR_RX : KR_RY;
                distinct_runs(rows, 1, [&](size_t a, size_t b) {
                    DevOp &d = emit(OP_RESET, sub, (uint32_t)(b - a), inst);
                    d.b = (uint32_t)a;
                    prog.pool.insert(prog.pool.end(), rows.begin() + a, rows.begin() + b);
                });
                return;
            }
            case GFS_MPAD: {
                emit(OP_RECORD_ZERO, 0, (uint32_t)op.targets.size(), inst);
                emit_results_tail(op, op.targets.size(), inst);
                return;
            }
            case GFS_MPP:
                lower_mpp(op, inst);
                return;
            case GFS_SPP:
            case GFS_SPP_DAG:
                lower_spp(op, inst);
                return;
            case GFS_MXX:
            case GFS_MYY:
            case GFS_MZZ:
                lower_pair_measure(op, inst);
                return;
            case GFS_X_ERROR:
            case GFS_Y_ERROR:
            case GFS_Z_ERROR:
            case GFS_DEPOLARIZE1:
            case GFS_DEPOLARIZE2: {
                double p = op.args[0];
                if (!(p > 0) || rows.empty()) {
                    return;
                }
                uint32_t sub = g == GFS_X_ERROR   ? KN_X
                               : g == GFS_Y_ERROR ? KN_Y
                               : g == GFS_Z_ERROR ? KN_Z
                               : g == GFS_DEPOLARIZE1 ? KN_DEP1
                                                      : KN_DEP2;
                uint32_t n = (uint32_t)(sub == KN_DEP2 ? rows.size() / 2 : rows.size());
                DevOp &d = emit(OP_NOISE, sub, n, inst);
                d.b = channel(p, {});
                prog.pool.insert(prog.pool.end(), rows.begin(), rows.end());
                return;
            }
            case GFS_PAULI_CHANNEL_1:
            case GFS_PAULI_CHANNEL_2: {
                double p = 0;
                for (double w : op.args) p += w;
                if (!(p > 0) || rows.empty()) {
                    return;
                }
                uint32_t sub = g == GFS_PAULI_CHANNEL_1 ? KN_PC1 : KN_PC2;
                uint32_t n = (uint32_t)(sub == KN_PC2 ? rows.size() / 2 : rows.size());
                DevOp &d = emit(OP_NOISE, sub, n, inst);
                d.b = channel(p, op.args);
                prog.pool.insert(prog.pool.end(), rows.begin(), rows.end());
                return;
            }
            case GFS_E:
            case GFS_ELSE_CORRELATED_ERROR: {
                DevOp &m = emit(OP_CORR_MASK, g == GFS_E ? 0 : 1, 1, inst);
                m.b = channel(op.args[0], {});
                std::map<uint32_t, uint32_t> xz;
                for (auto t : op.targets) {
                    uint32_t r = row(t);
                    uint32_t v = ((t & GFS_T_PAULI_X) ? 1u : 0u) | ((t & GFS_T_PAULI_Z) ? 2u : 0u);
                    xz[r] ^= v;
                }
                std::vector<uint32_t> units;
                for (auto &e : xz) {
                    if (e.second) {
                        units.push_back(e.first | (e.second << 24));
                    }
                }
                if (!units.empty()) {
                    emit(OP_CORR_APPLY, 0, (uint32_t)units.size(), inst);
                    prog.pool.insert(prog.pool.end(), units.begin(), units.end());
                }
                return;
            }
            case GFS_HERALDED_ERASE:
            case GFS_HERALDED_PAULI_CHANNEL_1: {
                uint32_t n = (uint32_t)rows.size();
                emit(OP_RECORD_ZERO, 0, n, inst);
                double p = 0;
                std::vector<double> w;
                if (g == GFS_HERALDED_ERASE) {
                    p = op.args[0];
                } else {
                    w = op.args;
                    for (double v : w) p += v;
                }
                if (p > 0 && n) {
                    DevOp &d = emit(OP_HERALD, g == GFS_HERALDED_ERASE ? 0 : 1, n, inst);
                    d.b = channel(p, w);
                    prog.pool.insert(prog.pool.end(), rows.begin(), rows.end());
                }
                if (mode == SampleMode::MEASUREMENTS && n) {
                    emit(OP_EMIT, 0, n, inst);
                }
                meas_seen += n;
                max_results_per_inst = std::max<uint64_t>(max_results_per_inst, n);
                return;
            }
            default:
                break;
        }
        if (gate_info(g).flags & GFS_F_PAIRS) {
            lower_two_qubit(op, inst);
            return;
        }
        throw std::invalid_argument(std::string("Not implemented in the GPU frame sampler: ") + gate_info(g).name);
    }

    std::unordered_map<const Circuit *, uint64_t> inst_memo;
    uint64_t instances(const Circuit &c) {
        auto it = inst_memo.find(&c);
        if (it != inst_memo.end()) {
            return it->second;
        }
        uint64_t v = c.stats().num_instances;
        inst_memo[&c] = v;
        return v;
    }

    uint64_t results_of(const Circuit &c) {
        return c.stats().num_measurements;
    }

    void lower_block(const Circuit &c, uint32_t depth) {
        prog.max_loop_depth = std::max(prog.max_loop_depth, depth);
        if (depth > (uint32_t)kMaxLoopDepth) {
            throw std::invalid_argument("REPEAT blocks nested deeper than the GPU sampler supports");
        }
        uint64_t flat = 0;
        // 0: lowered on its own; 1: noise fused after the previous instruction; 2: noise fused before the next.
        std::vector<uint8_t> fused(c.ops.size(), 0);
        for (size_t k = 0; k < c.ops.size(); k++) {
            const auto &op = c.ops[k];
            if (fused[k]) {  // noise lowered as part of a neighbouring gate
                flat += 1;
                continue;
            }
            if (op.gate != GFS_REPEAT && k + 1 < c.ops.size() && (noise_1q(op.gate) || noise_2q(op.gate)) &&
                c.ops[k + 1].gate != GFS_REPEAT && (gate_1q_fusable(c.ops[k + 1].gate) ||
                                                     gate_2q_fusable(c.ops[k + 1].gate)) &&
                fusable(op, c.ops[k + 1])) {
                fused[k] = 2;
                flat += 1;
                continue;
            }
            if (op.gate != GFS_REPEAT && (gate_1q_fusable(op.gate) || gate_2q_fusable(op.gate))) {
                Fuse f;
                if (k > 0 && fused[k - 1] == 2) {
                    f.pre = &c.ops[k - 1];
                }
                if (k + 1 < c.ops.size() && c.ops[k + 1].gate != GFS_REPEAT && fusable(c.ops[k + 1], op)) {
                    f.post = &c.ops[k + 1];
                    fused[k + 1] = 1;
                }
                if (f.pre || f.post) {
                    flush_detectors();
                    lower_fused(op, flat, f);
                    flat += 1;
                    continue;
                }
            }
            if (op.gate == GFS_REPEAT) {
                flush_detectors();
                const Circuit &body = c.blocks[op.block];
                uint64_t stride = instances(body);
                size_t begin = prog.ops.size();
                DevOp &lb = emit(OP_LOOP_BEGIN, 0, 0, flat);
                lb.a = (uint32_t)op.reps;
                lb.b = (uint32_t)(op.reps >> 32);
                lb.c = (uint32_t)stride;
                lb.d = (uint32_t)(stride >> 32);
                uint64_t seen_before = meas_seen;
                uint64_t saved_mult = mult;
                mult = (op.reps && mult > UINT64_MAX / op.reps) ? UINT64_MAX : mult * op.reps;
                lower_block(body, depth + 1);
                flush_detectors();
                mult = saved_mult;
                uint32_t body_len = (uint32_t)(prog.ops.size() - begin - 1);
                prog.ops[begin].n = body_len;
                DevOp &le = emit(OP_LOOP_END, 0, body_len, flat);
                (void)le;
                // The body was lowered against the first iteration's record length; later iterations
                // only see more results.
                uint64_t per_iter = meas_seen - seen_before;
                meas_seen = seen_before + per_iter * op.reps;
                flat += op.reps * stride;
            } else {
                lower_instruction(op, flat);
                flat += 1;
            }
        }
    }

    // Counts noise occurrences and expected hits with loop multiplicities (the noise kernel and the frame
    // kernel meet the occurrences in exactly this order), and lists them when there are not too many.
    void count_noise() {
        auto chan_hits = [&](uint32_t ch, uint64_t units) {
            double pr = std::min(1.0, std::max(0.0, prog.chan_p[ch]));
            return (double)units * GFS_BLOCK_SHOTS * pr;
        };
        // Occurrences and expected hits of op `op` (in the order pre, op, post).
        auto op_noise = [&](const DevOp &op, auto emit_occ) {
            const uint32_t code = op.code & 0xFFu;
            switch (code) {
                case OP_1Q:
                case OP_2Q:
                case OP_MEASURE:
                case OP_RESET:
                    if (op.d & kFusedChanMask) {
                        emit_occ(1u, chan_hits((op.d & kFusedChanMask) - 1, op.n));
                    }
                    if (op.c & kFusedChanMask) {
                        emit_occ(2u, chan_hits((op.c & kFusedChanMask) - 1, op.n));
                    }
                    break;
                case OP_NOISE:
                case OP_MNOISE:
                case OP_HERALD:
                    emit_occ(0u, chan_hits(op.b, op.n));
                    break;
                case OP_CORR_MASK:
                    emit_occ(0u, chan_hits(op.b, 1));
                    break;
                default:
                    break;
            }
        };
        // Totals with multiplicities.
        std::vector<double> mult_stack{1.0};
        double occ = 0, hits = 0;
        for (const DevOp &op : prog.ops) {
            const uint32_t code = op.code & 0xFFu;
            const double m = mult_stack.back();
            if (code == OP_LOOP_BEGIN) {
                mult_stack.push_back(m * (double)((uint64_t)op.a | ((uint64_t)op.b << 32)));
            } else if (code == OP_LOOP_END) {
                if (mult_stack.size() > 1) {
                    mult_stack.pop_back();
                }
            } else {
                op_noise(op, [&](uint32_t, double h) {
                    occ += m;
                    hits += m * h;
                });
            }
        }
        prog.noise_occurrences = occ > 1e18 ? (uint64_t)1e18 : (uint64_t)occ;
        prog.hits_per_block = hits;
        prog.occs.clear();
        prog.occ_hits_per_block.clear();
        if (prog.noise_occurrences == 0 || prog.noise_occurrences > kMaxNoiseOccurrences) {
            return;
        }
        // The list, walking the program the way the kernels do (same instance arithmetic).
        struct Loop {
            uint32_t pc;
            uint64_t left, base, stride;
        };
        std::vector<Loop> loops;
        uint64_t inst_base = 0;
        for (uint32_t pc = 0; pc < prog.ops.size();) {
            const DevOp &op = prog.ops[pc];
            const uint32_t code = op.code & 0xFFu;
            const uint64_t inst = inst_base + op.inst;
            if (code == OP_END) {
                break;
            }
            if (code == OP_LOOP_BEGIN) {
                loops.push_back({pc, (uint64_t)op.a | ((uint64_t)op.b << 32), inst_base,
                                 (uint64_t)op.c | ((uint64_t)op.d << 32)});
                inst_base = inst;
                pc++;
                continue;
            }
            if (code == OP_LOOP_END) {
                Loop &l = loops.back();
                if (--l.left > 0) {
                    inst_base += l.stride;
                    pc = l.pc + 1;
                } else {
                    inst_base = l.base;
                    loops.pop_back();
                    pc++;
                }
                continue;
            }
            op_noise(op, [&](uint32_t which, double h) {
                NoiseOcc o{};
                o.pc = pc;
                o.which = which;
                o.inst = inst;
                prog.occs.push_back(o);
                prog.occ_hits_per_block.push_back(h);
            });
            pc++;
        }
        if (prog.occs.size() != prog.noise_occurrences) {
            throw std::logic_error("noise occurrence count mismatch");
        }
    }

    // Reorders the units of every one- and two-qubit gate op so that each aligned group of 8 consecutive
    // units touches 8 distinct residues (row mod 8) on each side.  Threads take consecutive units, a
    // quarter-warp issues 8 lanes' 16-byte accesses together, and a row's 16 bytes sit in bank group
    // row mod 8, so such a group is free of shared-memory bank conflicts (for 2 and 4 blocks per CTA the
    // halves / quarters of a group stay distinct mod 4 / mod 2).  Units of one op act on distinct rows
    // and commute, so the order does not change any result.  Ops with fused noise keep their list (the
    // noise unit order is part of the random-bit contract) and get a second, reordered list at pool[b].
    void bank_order_gates() {
        for (DevOp &op : prog.ops) {
            const uint32_t code = op.code & 0xFFu;
            if ((code != OP_1Q && code != OP_2Q) || op.n < 16) {
                continue;
            }
            const uint32_t stride = code == OP_2Q ? 2 : 1;
            const uint32_t n = op.n;
            std::vector<uint32_t> units(prog.pool.begin() + op.a, prog.pool.begin() + op.a + (size_t)n * stride);
            std::vector<uint32_t> order;
            order.reserve(n);
            // Buckets by (first row mod 8, second row mod 8); one-qubit ops use residue 0 for the second.
            std::vector<std::vector<uint32_t>> bucket(64);
            for (uint32_t u = n; u-- > 0;) {
                const uint32_t c = units[(size_t)u * stride] & 7u;
                const uint32_t t = stride == 2 ? units[(size_t)u * stride + 1] & 7u : 0u;
                bucket[c * 8 + t].push_back(u);
            }
            // Greedy, group by group: each slot takes a unit from the bucket whose residues are least used so
            // far in the group (mod 8), in the slot's half of the group (mod 4: two blocks per CTA) and in its
            // pair (mod 2: four blocks per CTA); ties go to the fullest bucket, keeping later groups balanced.
            for (uint32_t left = n; left > 0;) {
                uint32_t l8c[8] = {0}, l8t[8] = {0}, l4c[4] = {0}, l4t[4] = {0}, l2c[2] = {0}, l2t[2] = {0};
                for (uint32_t slot = 0; slot < 8 && left > 0; slot++) {
                    if (slot % 4 == 0) {
                        std::fill(l4c, l4c + 4, 0u);
                        std::fill(l4t, l4t + 4, 0u);
                    }
                    if (slot % 2 == 0) {
                        l2c[0] = l2c[1] = l2t[0] = l2t[1] = 0;
                    }
                    int best = -1;
                    uint32_t best_cost = ~0u;
                    size_t best_size = 0;
                    for (uint32_t bk = 0; bk < 64; bk++) {
                        if (bucket[bk].empty()) {
                            continue;
                        }
                        const uint32_t c = bk / 8, t = bk % 8;
                        uint32_t cost = 4 * l8c[c] + 2 * l4c[c % 4] + l2c[c % 2];
                        if (stride == 2) {
                            cost += 4 * l8t[t] + 2 * l4t[t % 4] + l2t[t % 2];
                        }
                        if (cost < best_cost || (cost == best_cost && bucket[bk].size() > best_size)) {
                            best = (int)bk;
                            best_cost = cost;
                            best_size = bucket[bk].size();
                        }
                    }
                    order.push_back(bucket[best].back());
                    bucket[best].pop_back();
                    const uint32_t c = (uint32_t)best / 8, t = (uint32_t)best % 8;
                    l8c[c]++;
                    l8t[t]++;
                    l4c[c % 4]++;
                    l4t[t % 4]++;
                    l2c[c % 2]++;
                    l2t[t % 2]++;
                    left--;
                }
            }
            std::vector<uint32_t> out;
            out.reserve(units.size());
            for (uint32_t u : order) {
                for (uint32_t j = 0; j < stride; j++) {
                    out.push_back(units[(size_t)u * stride + j]);
                }
            }
            if (op.c | op.d) {
                op.b = (uint32_t)prog.pool.size();
                op.code |= kGateOrderInB;
                prog.pool.insert(prog.pool.end(), out.begin(), out.end());
            } else {
                std::copy(out.begin(), out.end(), prog.pool.begin() + op.a);
            }
        }
    }

    // Appends the compact unit lists (DevOp.g) of the gate, measurement, reset and detector ops: one load per
    // unit instead of two (pairs) or three dependent ones (detectors), and half the bytes, so a thread can
    // fetch all of its units' entries at once and a loop body's lists stay in L1.  Only when every row and
    // lookback fits 16 bits; detectors only when none reads more than two records.
    void build_compact_lists() {
        if (prog.num_rows > 0xFFFFu) {
            return;
        }
        for (DevOp &op : prog.ops) {
            const uint32_t code = op.code & 0xFFu;
            const uint32_t n = op.n;
            const uint32_t list = (op.code & kGateOrderInB) ? op.b : op.a;
            std::vector<uint32_t> words;
            if (code == OP_2Q) {
                for (uint32_t u = 0; u < n; u++) {
                    words.push_back(prog.pool[list + 2 * u] | (prog.pool[list + 2 * u + 1] << 16));
                }
            } else if (code == OP_1Q || code == OP_MEASURE || code == OP_RESET) {
                words.assign((n + 1) / 2, 0u);
                for (uint32_t u = 0; u < n; u++) {
                    words[u / 2] |= prog.pool[list + u] << (16 * (u % 2));
                }
            } else if (code == OP_DETECTORS) {
                bool ok = true;
                for (uint32_t u = 0; u < n && ok; u++) {
                    const uint32_t s = prog.pool[op.a + u], e = prog.pool[op.a + u + 1];
                    if (e - s > 2) {
                        ok = false;
                        break;
                    }
                    uint32_t w = 0;
                    for (uint32_t j = s; j < e; j++) {
                        const uint32_t k = prog.pool[j];
                        if (k == 0 || k > 0xFFFFu) {
                            ok = false;
                            break;
                        }
                        w |= k << (16 * (j - s));
                    }
                    words.push_back(w);
                }
                if (!ok) {
                    continue;
                }
            } else {
                continue;
            }
            op.g = (uint32_t)prog.pool.size();
            op.code |= kCompact;
            prog.pool.insert(prog.pool.end(), words.begin(), words.end());
        }
    }

    // Detection sampling: finds the measurement / reset ops whose randomized rows cannot change any detector
    // or observable, and marks them kNoRandomize (and the start-of-shot Z randomization, reset_norand).
    //
    // Every output is a GF(2)-linear function of the noise bits and of the randomization bits, because the
    // frame updates are XORs, copies and overwrites.  The pass walks the program backwards (loops unrolled)
    // keeping, for every row, the sorted sets of outputs that an X or a Z frame bit at that point flips
    // (the transpose of the forward map), and for every pending measurement result the outputs that read
    // it.  A randomized row whose set is empty has coefficient zero in every output, so writing zeros
    // instead of random bits leaves every detection event and observable unchanged for every noise
    // realisation.  The pass gives up (marks nothing) past a work limit.
    void analyze_randomization() {
        using Set = std::vector<uint32_t>;
        const uint32_t rows = prog.num_rows;
        std::vector<Set> xs(rows), zs(rows);
        const uint64_t R = (uint64_t)prog.ring + 1;
        std::vector<Set> pend(R);
        std::vector<uint8_t> ok(prog.ops.size(), 1);
        uint64_t meas = prog.stats.num_measurements, det = prog.stats.num_detectors;
        const uint32_t D = (uint32_t)prog.stats.num_detectors;
        uint64_t work = 0;
        const uint64_t kWorkLimit = 400000000ull;
        Set tmp;
        auto sdiff = [&](Set &a, const Set &b) {  // a ^= b
            if (b.empty()) {
                return;
            }
            tmp.clear();
            std::set_symmetric_difference(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(tmp));
            a.swap(tmp);
            work += a.size() + b.size();
        };
        auto toggle = [&](Set &a, uint32_t id) {
            auto it = std::lower_bound(a.begin(), a.end(), id);
            if (it != a.end() && *it == id) {
                a.erase(it);
            } else {
                a.insert(it, id);
            }
            work += 1 + a.size() / 8;
        };
        // S_before[k] = XOR of S_after[i] over the outputs i of the forward map that input k reaches.
        auto transpose = [&](uint32_t nv, uint32_t image[4], Set *after[4]) {
            Set before[4];
            for (uint32_t k = 0; k < nv; k++) {
                for (uint32_t i = 0; i < nv; i++) {
                    if ((image[k] >> i) & 1u) {
                        sdiff(before[k], *after[i]);
                    }
                }
            }
            for (uint32_t k = 0; k < nv; k++) {
                after[k]->swap(before[k]);
            }
        };
        bool failed = false;
        std::function<void(uint32_t, uint32_t)> walk = [&](uint32_t lo, uint32_t hi) {
            for (int64_t pc = (int64_t)hi - 1; pc >= (int64_t)lo && !failed; pc--) {
                if (work > kWorkLimit) {
                    failed = true;
                    return;
                }
                const DevOp &op = prog.ops[(size_t)pc];
                const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu, n = op.n;
                const uint32_t list = (op.code & kGateOrderInB) ? op.b : op.a;
                switch (code) {
                    case OP_LOOP_END: {
                        const int64_t lb = pc - (int64_t)n - 1;
                        const DevOp &b = prog.ops[(size_t)lb];
                        const uint64_t reps = (uint64_t)b.a | ((uint64_t)b.b << 32);
                        for (uint64_t r = 0; r < reps && !failed; r++) {
                            walk((uint32_t)lb + 1, (uint32_t)pc);
                        }
                        pc = lb;
                        break;
                    }
                    case OP_1Q:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t r = prog.pool[list + u];
                            uint32_t image[4];
                            for (uint32_t k = 0; k < 2; k++) {
                                uint32_t x = k == 0, z = k == 1;
                                rule1w(sub, x, z);
                                image[k] = (x & 1u) | ((z & 1u) << 1);
                            }
                            Set *after[4] = {&xs[r], &zs[r], nullptr, nullptr};
                            transpose(2, image, after);
                        }
                        break;
                    case OP_2Q:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t r1 = prog.pool[list + 2 * u], r2 = prog.pool[list + 2 * u + 1];
                            uint32_t image[4];
                            for (uint32_t k = 0; k < 4; k++) {
                                uint32_t v[4] = {k == 0, k == 1, k == 2, k == 3};
                                rule2(sub, v[0], v[1], v[2], v[3]);
                                image[k] = (v[0] & 1u) | ((v[1] & 1u) << 1) | ((v[2] & 1u) << 2) | ((v[3] & 1u) << 3);
                            }
                            Set *after[4] = {&xs[r1], &zs[r1], &xs[r2], &zs[r2]};
                            transpose(4, image, after);
                        }
                        break;
                    case OP_MEASURE:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t r = prog.pool[op.a + u];
                            Set &P = pend[(meas - n + u) % R];
                            Set &X = xs[r], &Z = zs[r];
                            const bool ybasis = sub == KM_MY || sub == KM_MRY;
                            const bool xbasis = sub == KM_MX || sub == KM_MRX;
                            if (ybasis) {
                                Set y = X;
                                sdiff(y, Z);
                                ok[(size_t)pc] &= y.empty();
                            } else {
                                ok[(size_t)pc] &= (xbasis ? X : Z).empty();
                            }
                            switch (sub) {
                                case KM_M:
                                    sdiff(X, P);
                                    Z.clear();
                                    break;
                                case KM_MX:
                                    sdiff(Z, P);
                                    X.clear();
                                    break;
                                case KM_MY:
                                    sdiff(X, P);
                                    Z = X;
                                    break;
                                case KM_MR:
                                    X = P;
                                    Z.clear();
                                    break;
                                case KM_MRX:
                                    Z = P;
                                    X.clear();
                                    break;
                                default:  // KM_MRY
                                    X = P;
                                    Z = P;
                                    break;
                            }
                            P.clear();
                        }
                        meas -= n;
                        break;
                    case OP_RESET:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t r = prog.pool[op.a + u];
                            Set &X = xs[r], &Z = zs[r];
                            if (sub == KR_RY) {
                                Set y = X;
                                sdiff(y, Z);
                                ok[(size_t)pc] &= y.empty();
                            } else {
                                ok[(size_t)pc] &= (sub == KR_RX ? X : Z).empty();
                            }
                            X.clear();
                            Z.clear();
                        }
                        break;
                    case OP_FEEDBACK:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t k = prog.pool[op.a + 2 * u], rm = prog.pool[op.a + 2 * u + 1];
                            if (k & kFeedbackSweep) {
                                continue;  // sweep data is an input, not randomness
                            }
                            const uint32_t r = rm & kRowMask;
                            Set &P = pend[(meas - k) % R];
                            if ((rm >> 24) & kFeedbackX) {
                                sdiff(P, xs[r]);
                            }
                            if ((rm >> 24) & kFeedbackZ) {
                                sdiff(P, zs[r]);
                            }
                        }
                        break;
                    case OP_RECORD_ZERO:
                        for (uint32_t u = 0; u < n; u++) {
                            pend[(meas - n + u) % R].clear();
                        }
                        meas -= n;
                        break;
                    case OP_DETECTORS:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t id = (uint32_t)(det - n + u);
                            for (uint32_t j = prog.pool[op.a + u]; j < prog.pool[op.a + u + 1]; j++) {
                                toggle(pend[(meas - prog.pool[j]) % R], id);
                            }
                        }
                        det -= n;
                        break;
                    case OP_OBS:
                        for (uint32_t u = 0; u < n; u++) {
                            const uint32_t t = prog.pool[op.a + u], id = D + op.b;
                            if (t & kTermRecord) {
                                toggle(pend[(meas - (t & kRowMask)) % R], id);
                            } else {
                                if (t & kTermX) {
                                    toggle(zs[t & kRowMask], id);
                                }
                                if (t & kTermZ) {
                                    toggle(xs[t & kRowMask], id);
                                }
                            }
                        }
                        break;
                    case OP_EMIT:
                        failed = true;
                        break;
                    default:  // noise, heralds, correlated errors, loop starts, end: no effect on the map
                        break;
                }
            }
        };
        walk(0, (uint32_t)prog.ops.size());
        if (failed || meas != 0 || det != 0) {
            return;
        }
        prog.reset_norand = true;
        for (uint32_t r = 0; r < rows; r++) {
            prog.reset_norand &= zs[r].empty();
        }
        for (size_t pc = 0; pc < prog.ops.size(); pc++) {
            const uint32_t code = prog.ops[pc].code & 0xFFu;
            if ((code == OP_MEASURE || code == OP_RESET) && ok[pc]) {
                prog.ops[pc].code |= kNoRandomize;
            }
        }
    }

    // The lean kernel's phase list (program.h LeanPhase): one phase per op, plus a hit phase for the noise fused
    // before / after a gate, in the order the generic kernel meets the noise occurrences.  Gives up (lean_ok =
    // false) on ops without a lean form.
    void build_lean() {
        prog.lean.clear();
        prog.lean_inst.clear();
        prog.occ_xform.clear();
        prog.lean_ok = false;
        lean_pc.clear();
        lean_which.clear();
        std::vector<uint32_t> open;  // phase indices of the open LK_LOOP_BEGINs
        uint32_t pc = 0, which = 0;
        auto add = [&](uint32_t kind, uint32_t sub, uint32_t flags, uint32_t n, uint32_t a, uint32_t b, uint64_t inst) {
            prog.lean.push_back(LeanPhase{kind | (sub << 8) | flags, n, a, b});
            prog.lean_inst.push_back(inst);
            lean_pc.push_back(pc);
            lean_which.push_back(which);
        };
        for (pc = 0; pc < prog.ops.size(); pc++) {
            const DevOp &op = prog.ops[pc];
            const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
            const bool compact = (op.code & kCompact) != 0;
            const uint32_t norand = (op.code & kNoRandomize) ? kLeanNoRandomize : 0u;
            const bool gate = code == OP_1Q || code == OP_2Q || code == OP_MEASURE || code == OP_RESET;
            if (gate && !compact) {
                return;
            }
            if (gate && (op.d & kFusedChanMask)) {
                which = 1;
                add(LK_HITS, 0, 0, op.n, 0, 0, op.inst);
            }
            which = 0;
            switch (code) {
                case OP_END:
                    add(LK_END, 0, 0, 0, 0, 0, 0);
                    break;
                case OP_LOOP_BEGIN: {
                    const uint64_t reps = (uint64_t)op.a | ((uint64_t)op.b << 32);
                    const uint64_t stride = (uint64_t)op.c | ((uint64_t)op.d << 32);
                    if (reps == 0 || reps > 0xFFFFFFFFull || open.size() >= 2) {
                        return;
                    }
                    open.push_back((uint32_t)prog.lean.size());
                    add(LK_LOOP_BEGIN, 0, 0, (uint32_t)reps, (uint32_t)stride, (uint32_t)(stride >> 32), op.inst);
                    break;
                }
                case OP_LOOP_END:
                    if (open.empty()) {
                        return;
                    }
                    add(LK_LOOP_END, 0, 0, 0, open.back(), 0, 0);
                    open.pop_back();
                    break;
                case OP_1Q:
                    add(LK_1Q, sub, 0, op.n, op.g, 0, op.inst);
                    break;
                case OP_2Q:
                    add(sub == K2_CX ? LK_CX : sub == K2_CZ ? LK_CZ : LK_2Q, sub, 0, op.n, op.g, 0, op.inst);
                    break;
                case OP_MEASURE:
                    add(LK_MEAS, sub, norand, op.n, op.g, op.b, op.inst);
                    break;
                case OP_RESET:
                    add(LK_RESET, sub, norand, op.n, op.g, op.b, op.inst);
                    break;
                case OP_RECORD_ZERO:
                    add(LK_ZERO, 0, 0, op.n, 0, 0, op.inst);
                    break;
                case OP_NOISE:
                    add(LK_HITS, 0, 0, op.n, 0, 0, op.inst);
                    break;
                case OP_MNOISE:
                    add(LK_FLIPS, 0, 0, op.n, 0, 0, op.inst);
                    break;
                case OP_DETECTORS:
                    if (compact) {
                        add(LK_DETS2, 0, 0, op.n, op.g, 0, op.inst);
                    } else {
                        add(LK_DETS, 0, 0, op.n, op.a, 0, op.inst);
                    }
                    break;
                case OP_OBS:
                    add(LK_OBS, 0, 0, op.n, op.a, op.b, op.inst);
                    break;
                case OP_EMIT:
                    add(LK_EMIT, 0, 0, op.n, 0, 0, op.inst);
                    break;
                case OP_FEEDBACK:
                    for (uint32_t u = 0; u < op.n; u++) {
                        if (prog.pool[op.a + 2 * u] & kFeedbackSweep) {
                            return;
                        }
                    }
                    add(LK_FEEDBACK, 0, 0, op.n, op.a, 0, op.inst);
                    break;
                default:  // correlated errors, heralds
                    return;
            }
            if (gate && (op.c & kFusedChanMask)) {
                which = 2;
                add(LK_HITS, 0, 0, op.n, 0, 0, op.inst);
            }
        }
        if (!open.empty() || prog.num_detectors > 0xFFFFFFFFull || prog.num_measurements > 0xFFFFFFFFull) {
            return;
        }
        move_lean_hits();
        mark_lean_barriers();
        prog.lean_ok = true;
    }

    // Rows touched by the units of op pc (gate rows, or the rows of a noise op); `pair` when units are pairs.
    void op_rows(uint32_t pc, std::vector<uint32_t> &rows, bool &pair) const {
        const DevOp &op = prog.ops[pc];
        const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
        pair = code == OP_2Q || (code == OP_NOISE && (sub == KN_DEP2 || sub == KN_PC2));
        const uint32_t k = pair ? 2u : 1u;
        rows.assign(prog.pool.begin() + op.a, prog.pool.begin() + op.a + (size_t)k * op.n);
    }

    // Moves hit phases earlier across the gates right before them when that lands them next to another phase they
    // commute with (a hit, flip or detector phase), so that the two run with no barrier between.  A Pauli P
    // applied after a gate with frame map M equals M^-1(P) applied before it (the maps are linear over GF(2)), so
    // a moved occurrence gets a transform of its records (program.h OccXform) that noise_kernel applies.  A hit
    // phase crosses: its own gate (the noise fused after a one- or two-qubit gate: the gate's inverse map on the
    // unit's 2 or 4 Pauli bits), up to two other one-qubit gates (their inverse map on the rows they act on), and
    // gates, measurements and resets on rows disjoint from its own (no change).  It never crosses another hit
    // phase, so the kernel still consumes the occurrences in order.
    void move_lean_hits() {
        if (prog.occs.empty()) {
            return;  // no hit lists, so no records to transform
        }
        std::vector<LeanPhase> &ph = prog.lean;
        const size_t n = ph.size();
        auto kind = [&](size_t i) { return ph[i].op & 0xFFu; };
        auto lands = [&](uint32_t k) {
            return k == LK_HITS || k == LK_FLIPS || k == LK_DETS2 || k == LK_DETS || k == LK_EMIT;
        };
        // Inverse one-qubit map of K1_* gate `sub` on (x, z) = bits 0, 1: entry v (2 bits each) = M^-1(v).
        auto inv1 = [](uint32_t sub) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < 4; w++) {
                uint32_t x = w & 1u, z = (w >> 1) & 1u;
                rule1w(sub, x, z);
                t |= w << (2 * ((x & 1u) | (z & 1u) << 1));
            }
            return t;
        };
        // Inverse two-qubit map of K2_* gate `sub` on (x1, z1, x2, z2) = bits 0..3 (4 bits per entry).
        auto inv2 = [](uint32_t sub, uint32_t &lo, uint32_t &hi) {
            uint64_t t = 0;
            for (uint32_t w = 0; w < 16; w++) {
                uint32_t x1 = w & 1u, z1 = (w >> 1) & 1u, x2 = (w >> 2) & 1u, z2 = (w >> 3) & 1u;
                rule2(sub, x1, z1, x2, z2);
                const uint32_t v = (x1 & 1u) | (z1 & 1u) << 1 | (x2 & 1u) << 2 | (z2 & 1u) << 3;
                t |= (uint64_t)w << (4 * v);
            }
            lo = (uint32_t)t;
            hi = (uint32_t)(t >> 32);
        };
        const uint64_t kIdLo = 0x76543210u, kIdHi = 0xFEDCBA98u;
        std::map<uint32_t, uint32_t> member_at;  // gate op -> pool offset of its row bitmap
        auto member_bitmap = [&](uint32_t gpc) {
            auto it = member_at.find(gpc);
            if (it != member_at.end()) {
                return it->second;
            }
            std::vector<uint32_t> rows;
            bool pr = false;
            op_rows(gpc, rows, pr);
            const uint32_t off = (uint32_t)prog.pool.size();
            prog.pool.resize(prog.pool.size() + (prog.num_rows + 31) / 32, 0u);
            for (uint32_t r : rows) {
                prog.pool[off + (r >> 5)] |= 1u << (r & 31);
            }
            member_at[gpc] = off;
            return off;
        };
        std::vector<uint32_t> xf_of(n, 0);  // 1 + index into prog.occ_xform of each phase
        std::vector<uint8_t> in_hit(prog.num_rows, 0);
        std::vector<uint32_t> hit_rows, gate_rows;
        for (size_t i = 0; i < n; i++) {
            if (kind(i) != LK_HITS) {
                continue;
            }
            const uint32_t hpc = lean_pc[i], hwhich = lean_which[i];
            const uint32_t hcode = prog.ops[hpc].code & 0xFFu;
            if (hwhich == 0 && hcode != OP_NOISE) {
                continue;
            }
            bool hpair = false;
            op_rows(hpc, hit_rows, hpair);
            for (uint32_t r : hit_rows) {
                in_hit[r] = 1;
            }
            OccXform x{};
            x.own_lo = (uint32_t)kIdLo;
            x.own_hi = (uint32_t)kIdHi;
            uint32_t fgate[2] = {0, 0};
            size_t j = i;
            while (j > 0) {
                const size_t g = j - 1;
                const uint32_t k = kind(g);
                if (k != LK_1Q && k != LK_CX && k != LK_CZ && k != LK_2Q && k != LK_MEAS && k != LK_RESET) {
                    break;
                }
                const uint32_t gpc = lean_pc[g];
                bool gpair = false;
                op_rows(gpc, gate_rows, gpair);
                bool disjoint = true;
                for (uint32_t r : gate_rows) {
                    disjoint &= in_hit[r] == 0;
                }
                if (disjoint) {
                    j = g;
                    continue;
                }
                const uint32_t gsub = (prog.ops[gpc].code >> 8) & 0xFFu;
                if (gpc == hpc && hwhich == 2 && g + 1 == i && (k == LK_1Q || k == LK_CX || k == LK_CZ || k == LK_2Q)) {
                    if (k == LK_1Q) {
                        const uint32_t t = inv1(gsub);
                        x.own_lo = (uint32_t)kIdLo;
                        for (uint32_t v = 0; v < 4; v++) {
                            x.own_lo = (x.own_lo & ~(15u << (4 * v))) | (((t >> (2 * v)) & 3u) << (4 * v));
                        }
                    } else {
                        inv2(gsub, x.own_lo, x.own_hi);
                    }
                    j = g;
                    continue;
                }
                if (k == LK_1Q && x.nf < 2) {
                    fgate[x.nf] = gpc;
                    x.ftab[x.nf] = inv1(gsub);
                    x.nf++;
                    j = g;
                    continue;
                }
                break;
            }
            for (uint32_t r : hit_rows) {
                in_hit[r] = 0;
            }
            if (j == i || j == 0 || !lands(kind(j - 1))) {
                continue;
            }
            for (uint32_t f = 0; f < x.nf; f++) {
                x.fmem[f] = member_bitmap(fgate[f]);
            }
            const bool identity = x.nf == 0 && x.own_lo == (uint32_t)kIdLo && x.own_hi == (uint32_t)kIdHi;
            if (!identity) {
                prog.occ_xform.push_back(x);
                xf_of[i] = (uint32_t)prog.occ_xform.size();
            }
            // Rotate phase i down to position j (every parallel list alike).
            auto rot = [&](auto &v) { std::rotate(v.begin() + j, v.begin() + i, v.begin() + i + 1); };
            rot(ph);
            rot(prog.lean_inst);
            rot(lean_pc);
            rot(lean_which);
            rot(xf_of);
        }
        if (prog.occ_xform.empty()) {
            return;
        }
        std::map<std::pair<uint32_t, uint32_t>, uint32_t> xf_at;
        for (size_t i = 0; i < n; i++) {
            if (xf_of[i]) {
                xf_at[{lean_pc[i], lean_which[i]}] = xf_of[i];
            }
        }
        for (NoiseOcc &o : prog.occs) {
            auto it = xf_at.find({o.pc, o.which});
            o.xform = it == xf_at.end() ? 0u : it->second;
        }
    }

    // Sets kLeanNoBarrier on the phases that every possible successor may follow without a barrier.
    void mark_lean_barriers() {
        std::vector<LeanPhase> &ph = prog.lean;
        const size_t n = ph.size();
        auto kind = [&](size_t i) { return ph[i].op & 0xFFu; };
        // The work phases that can run right after phase i (loop markers followed; both outcomes of a loop end).
        std::function<void(size_t, std::vector<size_t> &, int)> succ = [&](size_t j, std::vector<size_t> &out,
                                                                            int guard) {
            if (j >= n || guard > 8) {
                out.push_back(n);  // unknown: treat as needing a barrier
                return;
            }
            const uint32_t k = kind(j);
            if (k == LK_LOOP_BEGIN) {
                succ(j + 1, out, guard + 1);
            } else if (k == LK_LOOP_END) {
                succ(ph[j].a + 1, out, guard + 1);  // another iteration
                succ(j + 1, out, guard + 1);        // loop done
            } else {
                out.push_back(j);
            }
        };
        auto commutes = [&](uint32_t a, uint32_t b) {
            const bool ha = a == LK_HITS || a == LK_FLIPS, hb = b == LK_HITS || b == LK_FLIPS;
            const bool ra = a == LK_DETS2 || a == LK_DETS || a == LK_EMIT;
            const bool rb = b == LK_DETS2 || b == LK_DETS || b == LK_EMIT;
            if (ha && hb) {
                return true;  // XORs into frames / ring commute
            }
            if ((a == LK_HITS && rb) || (ra && b == LK_HITS)) {
                return true;  // frames vs ring reads and output rows: disjoint
            }
            return ra && rb;  // ring reads into distinct output rows
        };
        for (size_t i = 0; i < n; i++) {
            const uint32_t k = kind(i);
            if (k == LK_END || k == LK_LOOP_BEGIN || k == LK_LOOP_END) {
                continue;
            }
            std::vector<size_t> next;
            succ(i + 1, next, 0);
            bool ok = !next.empty();
            for (size_t j : next) {
                if (j >= n || kind(j) == LK_END || !commutes(k, kind(j))) {
                    ok = false;
                    break;
                }
            }
            if (ok) {
                ph[i].op |= kLeanNoBarrier;
            }
        }
    }

    void run() {
        prog.stats = root.stats();
        std::vector<uint8_t> used(prog.stats.num_qubits + 1, 0);
        collect_qubits(root, used);
        row_of.assign(used.size(), -1);
        for (size_t q = 0; q < used.size(); q++) {
            if (used[q]) {
                prog.qubit_orig.push_back((uint32_t)q);
            }
        }
        // Rows are the used qubits in a fixed pseudo-random order (Fisher-Yates with a 64-bit LCG), so
        // that the row residues mod 8 of any gate layer are spread out and bank_order_gates can form
        // conflict-free groups; generated codes otherwise put a layer's rows on few residues.  Which row
        // holds which qubit never affects results: the random streams are keyed by qubit and unit.
        uint64_t lcg = 0x9E3779B97F4A7C15ull;
        for (size_t k = prog.qubit_orig.size(); k > 1; k--) {
            lcg = lcg * 6364136223846793005ull + 1442695040888963407ull;
            const size_t j = (size_t)((lcg >> 33) % k);
            std::swap(prog.qubit_orig[k - 1], prog.qubit_orig[j]);
        }
        for (size_t r = 0; r < prog.qubit_orig.size(); r++) {
            row_of[prog.qubit_orig[r]] = (int32_t)r;
        }
        prog.num_rows = (uint32_t)prog.qubit_orig.size();
        if (prog.num_rows > kRowMask) {
            throw std::invalid_argument("too many qubits for the GPU frame sampler");
        }
        lower_block(root, 0);
        flush_detectors();
        emit(OP_END, 0, 0, 0);
        bank_order_gates();
        build_compact_lists();
        count_noise();
        prog.num_detectors = prog.stats.num_detectors;
        prog.num_observables = prog.stats.num_observables;
        prog.num_measurements = prog.stats.num_measurements;
        uint64_t ring = std::max<uint64_t>(std::max<uint64_t>(prog.stats.max_lookback, max_results_per_inst), 1);
        if (ring > (1u << 24)) {
            throw std::invalid_argument("measurement record window too large for the GPU frame sampler");
        }
        prog.ring = (uint32_t)ring;
        if (mode == SampleMode::DETECTIONS && dets_unrolled != prog.stats.num_detectors) {
            throw std::logic_error("detector count mismatch in lowering");
        }
        if (opts.no_randomization) {
            prog.reset_norand = true;
            for (DevOp &op : prog.ops) {
                const uint32_t code = op.code & 0xFFu;
                if (code == OP_MEASURE || code == OP_RESET) {
                    op.code |= kNoRandomize;
                }
            }
        } else if (mode == SampleMode::DETECTIONS) {
            analyze_randomization();
        }
        build_lean();
    }
};

}  // namespace

uint64_t plan_hit_regions(std::vector<NoiseOcc> &occs, const std::vector<double> &hits_per_block, uint32_t blocks,
                          uint64_t cap_override) {
    uint64_t off = 0;
    for (size_t k = 0; k < occs.size(); k++) {
        const double mean = hits_per_block[k] * blocks;
        double cap = std::ceil(mean + 8.0 * std::sqrt(mean) + 32.0);
        cap = std::min(cap, (double)blocks * GFS_BLOCK_SHOTS * (double)(1u << 24));  // at most every trial
        uint64_t c = (uint64_t)cap;
        if (cap_override) {
            c = std::min<uint64_t>(c, cap_override);
        }
        c = (c + 1) & ~(uint64_t)1;
        if (off + c > 0xFFFFFFFFull) {
            throw std::invalid_argument("hit-list region too large");
        }
        occs[k].off = (uint32_t)off;
        occs[k].cap = (uint32_t)c;
        off += c;
    }
    return off;
}

Program lower(const Circuit &circuit, SampleMode mode, const LowerOptions &opts) {
    Lowerer l(circuit, mode, opts);
    l.run();
    return std::move(l.prog);
}

Circuit noiseless_copy(const Circuit &c) {
    Circuit out;
    for (const Instruction &op : c.ops) {
        const uint32_t flags = gate_info(op.gate).flags;
        if (op.gate == GFS_HERALDED_ERASE || op.gate == GFS_HERALDED_PAULI_CHANNEL_1) {
            Instruction pad;
            pad.gate = GFS_MPAD;
            pad.targets.assign(op.targets.size(), 0u);
            out.ops.push_back(pad);
        } else if (flags & GFS_F_RESULTS) {
            Instruction m = op;
            m.args.clear();
            out.ops.push_back(m);
        } else if (!(flags & GFS_F_NOISY)) {
            out.ops.push_back(op);
        }
    }
    for (const Circuit &b : c.blocks) {
        out.blocks.push_back(noiseless_copy(b));
    }
    return out;
}

}  // namespace gfs
