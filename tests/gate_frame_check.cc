// Checks the frame update of every unitary gate against the reference's own tableau data, on the CPU: the
// reference's bulk_operations_consistent_with_tableau_data (src/stim/simulators/frame_simulator.test.cc:98-126)
// restated.  For each gate of tests/golden/gate_tableaus.txt (written by the reference's GATE_DATA), the one-gate
// circuit "NAME 0" / "NAME 0 1" is parsed and lowered by the product (stim_gb300/csrc/lower.cc), and its one- and
// two-qubit ops are applied with the product's frame rules (frame_rules.h) to the frames X0, Z0, X1, Z1 (one per bit
// lane); each result must be the gate's Heisenberg image of that Pauli, signs aside (a Pauli frame carries none).
//
// Usage: gate_frame_check TABLEAU_FILE  ->  prints "ok <gates>" or the mismatches, exit 1.
// Test infrastructure (tests/test_gate_frames.py compiles it); the product never uses it.
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "frame_rules.h"
#include "lower.h"

using namespace gfs;

namespace {

// 'I' / 'X' / 'Y' / 'Z' of the frame bits (x, z).
char pauli_char(uint32_t x, uint32_t z) {
    return x ? (z ? 'Y' : 'X') : (z ? 'Z' : '_');
}

// The images of X0, Z0 (, X1, Z1) under the gate's lowered program, one string per input Pauli.
bool images(const std::string &name, uint32_t n, std::vector<std::string> &out, std::string &err) {
    const std::string text = name + (n == 1 ? " 0" : " 0 1");
    Program p;
    try {
        p = lower(Circuit::parse(text), SampleMode::MEASUREMENTS);
    } catch (const std::exception &e) {
        err = e.what();
        return false;
    }
    std::vector<uint32_t> row_of(n, UINT32_MAX);
    for (uint32_t r = 0; r < p.num_rows && r < p.qubit_orig.size(); r++) {
        if (p.qubit_orig[r] < n) {
            row_of[p.qubit_orig[r]] = r;
        }
    }
    std::vector<uint32_t> x(p.num_rows, 0), z(p.num_rows, 0);
    for (uint32_t q = 0; q < n; q++) {
        if (row_of[q] == UINT32_MAX) {
            continue;  // an untouched qubit (a Pauli gate on it leaves no op): its frames stay as they are
        }
        x[row_of[q]] |= 1u << (2 * q);
        z[row_of[q]] |= 1u << (2 * q + 1);
    }
    for (const DevOp &op : p.ops) {
        const uint32_t code = op.code & 0xFFu, sub = (op.code >> 8) & 0xFFu;
        if (code == OP_END) {
            break;
        }
        if (code == OP_1Q) {
            for (uint32_t u = 0; u < op.n; u++) {
                const uint32_t r = p.pool[op.a + u];
                rule1w(sub, x[r], z[r]);
            }
        } else if (code == OP_2Q) {
            for (uint32_t u = 0; u < op.n; u++) {
                const uint32_t a = p.pool[op.a + 2 * u], b = p.pool[op.a + 2 * u + 1];
                rule2(sub, x[a], z[a], x[b], z[b]);
            }
        } else {
            err = "unexpected op code " + std::to_string(code);
            return false;
        }
    }
    out.clear();
    for (uint32_t lane = 0; lane < 2 * n; lane++) {
        std::string s;
        for (uint32_t q = 0; q < n; q++) {
            if (row_of[q] == UINT32_MAX) {
                const bool xb = lane == 2 * q, zb = lane == 2 * q + 1;
                s += pauli_char(xb, zb);
            } else {
                s += pauli_char((x[row_of[q]] >> lane) & 1u, (z[row_of[q]] >> lane) & 1u);
            }
        }
        out.push_back(s);
    }
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: gate_frame_check TABLEAU_FILE\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::string line;
    int gates = 0, bad = 0;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string tag, name;
        uint32_t n = 0;
        if (!(ls >> tag >> name >> n) || tag != "T" || (n != 1 && n != 2)) {
            continue;
        }
        std::vector<std::string> want;
        for (uint32_t k = 0; k < 2 * n; k++) {
            std::string img;
            ls >> img;
            want.push_back(img.substr(1));  // drop the sign
        }
        std::vector<std::string> got;
        std::string err;
        gates++;
        if (!images(name, n, got, err)) {
            std::printf("%s: %s\n", name.c_str(), err.c_str());
            bad++;
            continue;
        }
        for (uint32_t k = 0; k < 2 * n; k++) {
            if (got[k] != want[k]) {
                std::printf("%s: image of %c%u is %s, the reference's tableau says %s\n", name.c_str(), "XZ"[k & 1],
                            k / 2, got[k].c_str(), want[k].c_str());
                bad++;
            }
        }
    }
    if (bad) {
        return 1;
    }
    std::printf("ok %d\n", gates);
    return 0;
}
