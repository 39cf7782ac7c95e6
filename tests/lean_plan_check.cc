// Checks the lean kernel's phase list (stim_gb300/csrc/lower.cc build_lean, move_lean_hits) on the CPU: the
// device program and the phase list are both walked over 32 shots at once (one 32-bit word per frame row), with
// the same Clifford rules (frame_rules.h) and the same pseudo-random Pauli hits for every noise occurrence; the
// phase list applies each moved occurrence's hits through its transform (program.h OccXform), as noise_kernel
// writes them for the lean kernel.  The frames measured at every measurement, and the final frames, must agree.
//
// Usage: lean_plan_check CIRCUIT_FILE  ->  prints "ok <phases> <occurrences> <moved>" or a mismatch, exit 1.
// Test infrastructure (tests/test_lean_plan.py compiles it); the product never uses it.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <vector>

#include "frame_rules.h"
#include "lower.h"

using namespace gfs;

namespace {

struct Hit {
    uint32_t unit, bits, lane;
};

// Deterministic hits of occurrence instance k: 1..3 hits on random units with random nonzero Paulis.
std::vector<Hit> hits_of(uint64_t k, uint32_t n, bool pair) {
    uint64_t x = 0x9E3779B97F4A7C15ull * (k + 1);
    auto next = [&]() {
        x ^= x >> 33;
        x *= 0xFF51AFD7ED558CCDull;
        x ^= x >> 29;
        return (uint32_t)(x >> 16);
    };
    std::vector<Hit> h;
    const uint32_t m = 1 + next() % 3;
    for (uint32_t i = 0; i < m && n; i++) {
        Hit t;
        t.unit = next() % n;
        t.bits = pair ? 1 + next() % 15 : 1 + next() % 3;
        t.lane = next() % 32;
        h.push_back(t);
    }
    return h;
}

struct Frames {
    std::vector<uint32_t> x, z;
    std::vector<uint32_t> log;  // (x, z) of every measured row, in order
    explicit Frames(uint32_t rows) : x(rows, 0), z(rows, 0) {
    }
    void pauli(uint32_t r, uint32_t xz, uint32_t lane) {
        if (xz & 1) x[r] ^= 1u << lane;
        if (xz & 2) z[r] ^= 1u << lane;
    }
    void measure(uint32_t r, bool reset) {
        log.push_back(x[r]);
        log.push_back(z[r]);
        if (reset) {
            x[r] = 0;
            z[r] = 0;
        }
    }
};

// The occurrence's rows for unit u: the fused gate's unit (pair for two-qubit gates) or the noise op's unit.
void occ_rows(const Program &p, const NoiseOcc &o, uint32_t u, uint32_t &r1, uint32_t &r2, bool &pair) {
    const DevOp &op = p.ops[o.pc];
    const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
    pair = o.which ? code == OP_2Q : (code == OP_NOISE && (sub == KN_DEP2 || sub == KN_PC2));
    r1 = p.pool[op.a + (pair ? 2 * u : u)];
    r2 = pair ? p.pool[op.a + 2 * u + 1] : r1;
}

void apply_hits(const Program &p, uint64_t k, Frames &f, bool transformed) {
    const NoiseOcc &o = p.occs[k];
    const DevOp &op = p.ops[o.pc];
    if (!o.which && (op.code & 0xFFu) != OP_NOISE) {
        return;  // measurement flips: no frame effect
    }
    uint32_t r1, r2;
    bool pair;
    occ_rows(p, o, 0, r1, r2, pair);
    for (const Hit &h : hits_of(k, op.n, pair)) {
        occ_rows(p, o, h.unit, r1, r2, pair);
        uint32_t bits = h.bits;
        if (transformed && o.xform) {
            const OccXform &x = p.occ_xform[o.xform - 1];
            const uint64_t own = (uint64_t)x.own_lo | ((uint64_t)x.own_hi << 32);
            bits = (uint32_t)(own >> (4 * bits)) & 15u;
            for (uint32_t g = 0; g < x.nf; g++) {
                const uint32_t *mem = p.pool.data() + x.fmem[g];
                if ((mem[r1 >> 5] >> (r1 & 31)) & 1u) {
                    bits = (bits & ~3u) | ((x.ftab[g] >> (2 * (bits & 3u))) & 3u);
                }
                if (pair && ((mem[r2 >> 5] >> (r2 & 31)) & 1u)) {
                    bits = (bits & 3u) | (((x.ftab[g] >> (2 * ((bits >> 2) & 3u))) & 3u) << 2);
                }
            }
        }
        f.pauli(r1, bits & 3u, h.lane);
        if (pair) {
            f.pauli(r2, (bits >> 2) & 3u, h.lane);
        }
    }
}

bool is_reset_measure(uint32_t sub) {
    return sub == KM_MR || sub == KM_MRX || sub == KM_MRY;
}

// The device program, loops unrolled, occurrences in order.
void walk_ops(const Program &p, Frames &f) {
    uint64_t k = 0;
    struct Loop {
        uint32_t pc;
        uint64_t left;
    };
    std::vector<Loop> loops;
    for (uint32_t pc = 0; pc < p.ops.size();) {
        const DevOp &op = p.ops[pc];
        const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
        if (code == OP_END) {
            break;
        }
        if (code == OP_LOOP_BEGIN) {
            loops.push_back({pc, (uint64_t)op.a | ((uint64_t)op.b << 32)});
            pc++;
            continue;
        }
        if (code == OP_LOOP_END) {
            if (--loops.back().left > 0) {
                pc = loops.back().pc + 1;
            } else {
                loops.pop_back();
                pc++;
            }
            continue;
        }
        const bool gate = code == OP_1Q || code == OP_2Q || code == OP_MEASURE || code == OP_RESET;
        if (gate && (op.d & kFusedChanMask)) {
            apply_hits(p, k++, f, false);
        }
        if (code == OP_1Q) {
            for (uint32_t u = 0; u < op.n; u++) {
                const uint32_t r = p.pool[op.a + u];
                rule1w(sub, f.x[r], f.z[r]);
            }
        } else if (code == OP_2Q) {
            for (uint32_t u = 0; u < op.n; u++) {
                const uint32_t a = p.pool[op.a + 2 * u], b = p.pool[op.a + 2 * u + 1];
                rule2(sub, f.x[a], f.z[a], f.x[b], f.z[b]);
            }
        } else if (code == OP_MEASURE) {
            for (uint32_t u = 0; u < op.n; u++) {
                f.measure(p.pool[op.a + u], is_reset_measure(sub));
            }
        } else if (code == OP_RESET) {
            for (uint32_t u = 0; u < op.n; u++) {
                const uint32_t r = p.pool[op.a + u];
                f.x[r] = f.z[r] = 0;
            }
        } else if (code == OP_NOISE || code == OP_MNOISE) {
            apply_hits(p, k++, f, false);
        }
        if (gate && (op.c & kFusedChanMask)) {
            apply_hits(p, k++, f, false);
        }
        pc++;
    }
    if (k != p.occs.size()) {
        std::printf("device program met %llu occurrences, the list has %zu\n", (unsigned long long)k, p.occs.size());
        std::exit(1);
    }
}

// The lean phase list, as frame_lean.cu walks it (compact unit lists, moved hit phases transformed).
void walk_lean(const Program &p, Frames &f) {
    const uint16_t *half = reinterpret_cast<const uint16_t *>(p.pool.data());
    uint64_t k = 0;
    struct Loop {
        uint32_t pc;
        uint64_t left;
    };
    std::vector<Loop> loops;
    for (uint32_t pc = 0; pc < p.lean.size();) {
        const LeanPhase &d = p.lean[pc];
        const uint32_t kind = d.op & 0xFFu, sub = (d.op >> 8) & 0xFFu;
        if (kind == LK_END) {
            break;
        }
        switch (kind) {
            case LK_LOOP_BEGIN:
                loops.push_back({pc, d.n});
                break;
            case LK_LOOP_END:
                if (--loops.back().left > 0) {
                    pc = loops.back().pc + 1;
                    continue;
                }
                loops.pop_back();
                break;
            case LK_HITS:
            case LK_FLIPS:
                apply_hits(p, k++, f, true);
                break;
            case LK_1Q:
                for (uint32_t u = 0; u < d.n; u++) {
                    const uint32_t r = half[2 * d.a + u];
                    rule1w(sub, f.x[r], f.z[r]);
                }
                break;
            case LK_CX:
            case LK_CZ:
            case LK_2Q:
                for (uint32_t u = 0; u < d.n; u++) {
                    const uint32_t w = p.pool[d.a + u], a = w & 0xFFFFu, b = w >> 16;
                    rule2(sub, f.x[a], f.z[a], f.x[b], f.z[b]);
                }
                break;
            case LK_MEAS:
                for (uint32_t u = 0; u < d.n; u++) {
                    f.measure(half[2 * d.a + u], is_reset_measure(sub));
                }
                break;
            case LK_RESET:
                for (uint32_t u = 0; u < d.n; u++) {
                    const uint32_t r = half[2 * d.a + u];
                    f.x[r] = f.z[r] = 0;
                }
                break;
            default:  // detectors, observables, zero results, emitted results: no frame effect
                break;
        }
        pc++;
    }
    if (k != p.occs.size()) {
        std::printf("phase list met %llu occurrences, the list has %zu\n", (unsigned long long)k, p.occs.size());
        std::exit(1);
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: lean_plan_check CIRCUIT_FILE\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::stringstream ss;
    ss << in.rdbuf();
    const Program p = lower(Circuit::parse(ss.str()), SampleMode::DETECTIONS);
    if (!p.lean_ok) {
        std::printf("no-lean\n");
        return 0;
    }
    if (p.occs.size() != p.noise_occurrences) {
        std::printf("skip: occurrences not listed\n");
        return 0;
    }
    Frames a(p.num_rows), b(p.num_rows);
    walk_ops(p, a);
    walk_lean(p, b);
    if (a.log != b.log) {
        size_t i = 0;
        while (i < a.log.size() && i < b.log.size() && a.log[i] == b.log[i]) {
            i++;
        }
        std::printf("measurement %zu differs (of %zu / %zu)\n", i / 2, a.log.size() / 2, b.log.size() / 2);
        return 1;
    }
    if (a.x != b.x || a.z != b.z) {
        std::printf("final frames differ\n");
        return 1;
    }
    size_t moved = 0;
    for (const NoiseOcc &o : p.occs) {
        moved += o.xform != 0;
    }
    std::printf("ok %zu %zu %zu\n", p.lean.size(), p.occs.size(), moved);
    return 0;
}
