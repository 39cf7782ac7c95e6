// ref_inject -- runs the REFERENCE's own stim::FrameSimulator on a circuit, with every random bit
// taken from the counter-based contract in gfs_contract.h instead of std::mt19937_64.
//
// Test infrastructure only: it is compiled from the reference's sources where they lie (never copied)
// by `make -C oracle ref`, and writes golden outputs that pin both the CPU oracle and the CUDA path.
//
// What runs unmodified in the reference: parsing (Circuit(text)), every Clifford gate, classical
// feedback, resets and measurements (FrameSimulator<W>::do_gate, frame_simulator.inl:914-1113), the
// MPP / pair-measurement decompositions (gate_decomposition.cc:88-161, 319-347), DETECTOR and
// OBSERVABLE_INCLUDE (frame_simulator.inl:221-252) and the reference sample
// (TableauSimulator<W>::reference_sample_circuit, tableau_simulator.inl:1435-1438).
//
// What is injected (the only places the reference consumes randomness):
//   * reset_all's z randomization (frame_simulator.inl:152-163);
//   * the post-collapse randomization of M/MX/MY/MR/MRX/MRY/R/RX/RY (frame_simulator.inl:172-317),
//     applied target by target, with guarantee_anticommutation_via_frame_randomization = false;
//   * measurement-result flips of noisy measurements (measure_record_batch.inl:48-54);
//   * every noise channel (frame_simulator.inl:632-695, 718-839).
//
// Usage: ref_inject CIRCUIT_FILE SEED NUM_SHOTS OUT_FILE
// Output (little endian): "GFSREF01", u64 shots, u64 dets, u64 obs, u64 meas, then shot-major bit-packed
// dets, obs, meas (measurement flips, before any reference-sample XOR), then the reference sample bits.

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <vector>

#include "gfs_contract.h"
#include "stim/circuit/gate_decomposition.h"
#include "stim/simulators/frame_simulator.h"
#include "stim/simulators/tableau_simulator.h"

using namespace stim;
constexpr size_t W = MAX_BITWORD_WIDTH;

struct Injector {
    FrameSimulator<W> &sim;
    uint64_t seed;
    size_t shots;
    size_t blocks;
    uint64_t instance = 0;

    Injector(FrameSimulator<W> &sim, uint64_t seed, size_t shots)
        : sim(sim), seed(seed), shots(shots), blocks((shots + 127) / 128) {
    }

    void set_row(simd_bits_range_ref<W> row, uint32_t purpose, uint64_t inst, uint32_t unit) {
        size_t nb = row.num_u64_padded() / 2;
        for (size_t b = 0; b < nb; b++) {
            gfs_u32x4 r = gfs_row_bits(seed, purpose, inst, unit, (uint32_t)b);
            row.u64[2 * b] = (uint64_t)r.v[0] | ((uint64_t)r.v[1] << 32);
            row.u64[2 * b + 1] = (uint64_t)r.v[2] | ((uint64_t)r.v[3] << 32);
        }
    }

    void reset_all() {
        sim.guarantee_anticommutation_via_frame_randomization = false;
        sim.reset_all();
        for (size_t q = 0; q < sim.num_qubits; q++) {
            set_row(sim.z_table[q], GFS_P_RESET, 0, (uint32_t)q);
        }
    }

    // Post-collapse randomization of one target, following the reference's per-gate rule.
    void randomize_after(GateType g, uint32_t q, uint32_t unit) {
        simd_bits<W> r(sim.batch_size);
        set_row(r, GFS_P_RAND, instance, unit);
        switch (g) {
            case GateType::M:
            case GateType::MR:
            case GateType::R:
                sim.z_table[q] = r;
                break;
            case GateType::MX:
            case GateType::MRX:
            case GateType::RX:
                sim.x_table[q] = r;
                break;
            case GateType::MY:
                // With randomization on: x ^= z; record; z = rand; x ^= z.  With it off x was restored.
                sim.x_table[q] ^= sim.z_table[q];
                sim.x_table[q] ^= r;
                sim.z_table[q] = r;
                break;
            case GateType::MRY:
            case GateType::RY:
                sim.z_table[q] = r;
                sim.x_table[q] = r;
                break;
            default:
                throw std::invalid_argument("no randomization rule");
        }
    }

    // Segment walk of the contract; calls hit(unit, shot, stream) for each hit.
    template <typename HIT>
    void for_hits(double p, uint32_t purpose, size_t num_units, HIT hit) {
        if (!(p > 0) || num_units == 0) {
            return;
        }
        bool always = p >= 1;
        std::vector<uint32_t> table(GFS_TABLE_LEN);
        float inv_c = 0;
        if (!always) {
            gfs_build_gap_table(p, table.data());
            inv_c = gfs_inv_c(p);
        }
        size_t nseg = (num_units + GFS_SEG_UNITS - 1) / GFS_SEG_UNITS;
        for (size_t b = 0; b < blocks; b++) {
            for (size_t g = 0; g < nseg; g++) {
                size_t u0 = g * GFS_SEG_UNITS;
                size_t nu = std::min<size_t>(GFS_SEG_UNITS, num_units - u0);
                int32_t trials = (int32_t)(nu * GFS_BLOCK_SHOTS);
                gfs_stream s;
                gfs_stream_init(&s, seed, purpose, instance, (uint32_t)g, (uint32_t)b);
                int32_t pos = -1;
                while ((pos = gfs_next_hit(&s, table.data(), inv_c, pos, trials, always)) >= 0) {
                    size_t unit = u0 + (size_t)pos / GFS_BLOCK_SHOTS;
                    size_t shot = b * GFS_BLOCK_SHOTS + (size_t)pos % GFS_BLOCK_SHOTS;
                    hit(unit, shot, &s);
                }
            }
        }
    }

    void flip_x(size_t q, size_t shot) {
        sim.x_table[q][shot] ^= true;
    }
    void flip_z(size_t q, size_t shot) {
        sim.z_table[q][shot] ^= true;
    }
    void apply_pauli_index(size_t q, size_t shot, uint32_t v) {  // 0=I 1=X 2=Y 3=Z
        if (v == 1 || v == 2) {
            flip_x(q, shot);
        }
        if (v == 2 || v == 3) {
            flip_z(q, shot);
        }
    }

    void flip_results(double p, size_t first_row, size_t n) {
        for_hits(p, GFS_P_MNOISE, n, [&](size_t unit, size_t shot, gfs_stream *) {
            if (shot < shots) {
                sim.m_record.storage[first_row + unit][shot] ^= true;
            }
        });
    }

    static CircuitInstruction single(GateType g, const GateTarget *t) {
        return CircuitInstruction(g, {}, SpanRef<const GateTarget>(t, t + 1), "");
    }

    void do_collapse(const CircuitInstruction &op) {
        size_t first = sim.m_record.stored;
        bool produces = GATE_DATA[op.gate_type].flags & GATE_PRODUCES_RESULTS;
        for (size_t k = 0; k < op.targets.size(); k++) {
            sim.do_gate(single(op.gate_type, &op.targets[k]));
            randomize_after(op.gate_type, op.targets[k].qubit_value(), (uint32_t)k);
        }
        if (produces && !op.args.empty()) {
            flip_results(op.args[0], first, op.targets.size());
        }
    }

    void do_mpp(const CircuitInstruction &op) {
        size_t first = sim.m_record.stored;
        uint32_t result = 0;
        decompose_mpp_operation(op, sim.num_qubits, [&](const CircuitInstruction &sub) {
            if (sub.gate_type == GateType::M) {
                for (size_t k = 0; k < sub.targets.size(); k++) {
                    sim.do_gate(single(GateType::M, &sub.targets[k]));
                    randomize_after(GateType::M, sub.targets[k].qubit_value(), result++);
                }
            } else if (sub.gate_type == GateType::MPAD) {
                for (size_t k = 0; k < sub.targets.size(); k++) {
                    sim.do_gate(single(GateType::MPAD, &sub.targets[k]));
                    result++;
                }
            } else {
                sim.do_gate(sub);
            }
        });
        if (!op.args.empty()) {
            flip_results(op.args[0], first, result);
        }
    }

    void do_pair_measure(const CircuitInstruction &op) {
        size_t first = sim.m_record.stored;
        uint32_t result = 0;
        GateType conj, meas;
        if (op.gate_type == GateType::MXX) {
            conj = GateType::CX;
            meas = GateType::MX;
        } else if (op.gate_type == GateType::MYY) {
            conj = GateType::CY;
            meas = GateType::MY;
        } else {
            conj = GateType::XCZ;
            meas = GateType::M;
        }
        decompose_pair_instruction_into_disjoint_segments(op, sim.num_qubits, [&](CircuitInstruction seg) {
            std::vector<GateTarget> ts;
            for (auto t : seg.targets) {
                ts.push_back(GateTarget::qubit(t.qubit_value()));
            }
            sim.do_gate(CircuitInstruction(conj, {}, ts, ""));
            for (size_t k = 0; k < ts.size(); k += 2) {
                sim.do_gate(single(meas, &ts[k]));
                randomize_after(meas, ts[k].qubit_value(), result++);
            }
            sim.do_gate(CircuitInstruction(conj, {}, ts, ""));
        });
        if (!op.args.empty()) {
            flip_results(op.args[0], first, result);
        }
    }

    void do_mpad(const CircuitInstruction &op) {
        size_t first = sim.m_record.stored;
        sim.do_gate(CircuitInstruction(GateType::MPAD, {}, op.targets, ""));
        if (!op.args.empty()) {
            flip_results(op.args[0], first, op.targets.size());
        }
    }

    void do_heralded(const CircuitInstruction &op) {
        size_t nt = op.targets.size();
        auto &rec = sim.m_record;
        rec.reserve_space_for_results(nt);
        for (size_t k = 0; k < nt; k++) {
            rec.storage[rec.stored + k].clear();
        }
        size_t first = rec.stored;
        if (op.gate_type == GateType::HERALDED_ERASE) {
            for_hits(op.args[0], GFS_P_NOISE, nt, [&](size_t u, size_t shot, gfs_stream *s) {
                uint32_t c = gfs_stream_next(s);
                size_t q = op.targets[u].qubit_value();
                rec.storage[first + u][shot] = true;
                if (c & 1) {
                    flip_x(q, shot);
                }
                if (c & 2) {
                    flip_z(q, shot);
                }
            });
        } else {
            double w[4] = {op.args[0], op.args[1], op.args[2], op.args[3]};
            uint64_t cum[4];
            gfs_build_choice_table(w, 4, cum);
            double total = w[0] + w[1] + w[2] + w[3];
            for_hits(total, GFS_P_NOISE, nt, [&](size_t u, size_t shot, gfs_stream *s) {
                uint32_t c = gfs_stream_next(s);
                size_t q = op.targets[u].qubit_value();
                rec.storage[first + u][shot] = true;
                apply_pauli_index(q, shot, gfs_choice_weighted(c, cum, 4));
            });
        }
        for (size_t k = 0; k < nt; k++) {
            for (size_t shot = shots; shot < rec.storage[first + k].num_bits_padded(); shot++) {
                rec.storage[first + k][shot] = false;
            }
        }
        rec.stored += nt;
        rec.unwritten += nt;
    }

    void do_correlated(const CircuitInstruction &op) {
        auto &occ = sim.last_correlated_error_occurred;
        if (op.gate_type == GateType::E) {
            occ.clear();
        }
        simd_bits<W> mask(sim.batch_size);
        for_hits(op.args[0], GFS_P_NOISE, 1, [&](size_t, size_t shot, gfs_stream *) {
            mask[shot] = true;
        });
        for (size_t k = 0; k < mask.num_u64_padded(); k++) {
            mask.u64[k] &= ~occ.u64[k];
            occ.u64[k] |= mask.u64[k];
        }
        for (auto t : op.targets) {
            if (t.data & TARGET_PAULI_X_BIT) {
                sim.x_table[t.qubit_value()] ^= mask;
            }
            if (t.data & TARGET_PAULI_Z_BIT) {
                sim.z_table[t.qubit_value()] ^= mask;
            }
        }
    }

    void do_noise(const CircuitInstruction &op) {
        const auto &ts = op.targets;
        switch (op.gate_type) {
            case GateType::X_ERROR:
                for_hits(op.args[0], GFS_P_NOISE, ts.size(), [&](size_t u, size_t shot, gfs_stream *) {
                    flip_x(ts[u].qubit_value(), shot);
                });
                break;
            case GateType::Y_ERROR:
                for_hits(op.args[0], GFS_P_NOISE, ts.size(), [&](size_t u, size_t shot, gfs_stream *) {
                    flip_x(ts[u].qubit_value(), shot);
                    flip_z(ts[u].qubit_value(), shot);
                });
                break;
            case GateType::Z_ERROR:
                for_hits(op.args[0], GFS_P_NOISE, ts.size(), [&](size_t u, size_t shot, gfs_stream *) {
                    flip_z(ts[u].qubit_value(), shot);
                });
                break;
            case GateType::DEPOLARIZE1:
                for_hits(op.args[0], GFS_P_NOISE, ts.size(), [&](size_t u, size_t shot, gfs_stream *s) {
                    uint32_t v = 1 + gfs_choice_uniform(gfs_stream_next(s), 3);
                    size_t q = ts[u].qubit_value();
                    if (v & 1) {
                        flip_x(q, shot);
                    }
                    if (v & 2) {
                        flip_z(q, shot);
                    }
                });
                break;
            case GateType::DEPOLARIZE2:
                for_hits(op.args[0], GFS_P_NOISE, ts.size() / 2, [&](size_t u, size_t shot, gfs_stream *s) {
                    uint32_t v = 1 + gfs_choice_uniform(gfs_stream_next(s), 15);
                    size_t q1 = ts[2 * u].qubit_value(), q2 = ts[2 * u + 1].qubit_value();
                    if (v & 1) {
                        flip_x(q1, shot);
                    }
                    if (v & 2) {
                        flip_z(q1, shot);
                    }
                    if (v & 4) {
                        flip_x(q2, shot);
                    }
                    if (v & 8) {
                        flip_z(q2, shot);
                    }
                });
                break;
            case GateType::PAULI_CHANNEL_1: {
                double w[3] = {op.args[0], op.args[1], op.args[2]};
                uint64_t cum[3];
                gfs_build_choice_table(w, 3, cum);
                for_hits(w[0] + w[1] + w[2], GFS_P_NOISE, ts.size(), [&](size_t u, size_t shot, gfs_stream *s) {
                    uint32_t v = 1 + gfs_choice_weighted(gfs_stream_next(s), cum, 3);
                    apply_pauli_index(ts[u].qubit_value(), shot, v);
                });
                break;
            }
            case GateType::PAULI_CHANNEL_2: {
                double w[15];
                double total = 0;
                for (int k = 0; k < 15; k++) {
                    w[k] = op.args[k];
                    total += w[k];
                }
                uint64_t cum[15];
                gfs_build_choice_table(w, 15, cum);
                for_hits(total, GFS_P_NOISE, ts.size() / 2, [&](size_t u, size_t shot, gfs_stream *s) {
                    uint32_t v = 1 + gfs_choice_weighted(gfs_stream_next(s), cum, 15);
                    apply_pauli_index(ts[2 * u].qubit_value(), shot, v >> 2);
                    apply_pauli_index(ts[2 * u + 1].qubit_value(), shot, v & 3);
                });
                break;
            }
            default:
                throw std::invalid_argument("not a noise channel");
        }
    }

    void do_op(const CircuitInstruction &op) {
        switch (op.gate_type) {
            case GateType::M:
            case GateType::MX:
            case GateType::MY:
            case GateType::MR:
            case GateType::MRX:
            case GateType::MRY:
            case GateType::R:
            case GateType::RX:
            case GateType::RY:
                do_collapse(op);
                break;
            case GateType::MPP:
                do_mpp(op);
                break;
            case GateType::MXX:
            case GateType::MYY:
            case GateType::MZZ:
                do_pair_measure(op);
                break;
            case GateType::MPAD:
                do_mpad(op);
                break;
            case GateType::HERALDED_ERASE:
            case GateType::HERALDED_PAULI_CHANNEL_1:
                do_heralded(op);
                break;
            case GateType::E:
            case GateType::ELSE_CORRELATED_ERROR:
                do_correlated(op);
                break;
            case GateType::X_ERROR:
            case GateType::Y_ERROR:
            case GateType::Z_ERROR:
            case GateType::DEPOLARIZE1:
            case GateType::DEPOLARIZE2:
            case GateType::PAULI_CHANNEL_1:
            case GateType::PAULI_CHANNEL_2:
                do_noise(op);
                break;
            default:
                sim.do_gate(op);
        }
        instance++;
    }
};

static void write_table(std::ofstream &out, const simd_bit_table<W> &t, size_t major, size_t shots) {
    size_t nbytes = (major + 7) / 8;
    std::vector<uint8_t> row(nbytes);
    for (size_t s = 0; s < shots; s++) {
        std::fill(row.begin(), row.end(), 0);
        for (size_t m = 0; m < major; m++) {
            if (t[m][s]) {
                row[m >> 3] |= (uint8_t)(1 << (m & 7));
            }
        }
        out.write((const char *)row.data(), (std::streamsize)nbytes);
    }
}

int main(int argc, char **argv) {
    if (argc != 5) {
        fprintf(stderr, "usage: ref_inject CIRCUIT SEED SHOTS OUT\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::stringstream ss;
    ss << in.rdbuf();
    Circuit circuit(ss.str());
    uint64_t seed = strtoull(argv[2], nullptr, 10);
    size_t shots = strtoull(argv[3], nullptr, 10);
    auto stats = circuit.compute_stats();

    FrameSimulator<W> sim(stats, FrameSimulatorMode::STORE_EVERYTHING_TO_MEMORY, shots, std::mt19937_64(0));
    Injector inj(sim, seed, shots);
    inj.reset_all();
    circuit.for_each_operation([&](const CircuitInstruction &op) {
        inj.do_op(op);
    });

    auto ref = TableauSimulator<W>::reference_sample_circuit(circuit);

    std::ofstream out(argv[4], std::ios::binary);
    out.write("GFSREF01", 8);
    uint64_t hdr[4] = {shots, stats.num_detectors, stats.num_observables, stats.num_measurements};
    out.write((const char *)hdr, sizeof(hdr));
    write_table(out, sim.det_record.storage, stats.num_detectors, shots);
    write_table(out, sim.obs_record, stats.num_observables, shots);
    write_table(out, sim.m_record.storage, stats.num_measurements, shots);
    std::vector<uint8_t> rb((stats.num_measurements + 7) / 8);
    for (size_t m = 0; m < stats.num_measurements; m++) {
        if (ref[m]) {
            rb[m >> 3] |= (uint8_t)(1 << (m & 7));
        }
    }
    out.write((const char *)rb.data(), (std::streamsize)rb.size());
    return 0;
}
