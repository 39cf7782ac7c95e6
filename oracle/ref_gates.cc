// ref_gates -- prints the REFERENCE's gate vocabulary (stim::GATE_DATA, src/stim/gates/gates.h:192-390):
// every gate's canonical name, argument count, GateFlags bits, and every alias with the gate it names.
//
// Test infrastructure only: compiled from the reference's sources where they lie (never copied) by
// `make -C oracle ref`, run by tests/golden/make_gates.py, which commits its output as a fixture.  The product's
// table (stim_gb300/csrc/gfs_gates.h) is then checked against that fixture, so a wrong entry cannot hide behind
// the CPU oracle reading the same table.
//
// Usage: ref_gates  ->  one line per gate: "G <name> <arg_count> <flags>", then "A <alias> <canonical name>".

#include <cstdio>
#include <string>

#include "stim/gates/gates.h"

int main() {
    for (const stim::Gate &g : stim::GATE_DATA.items) {
        if (g.id == stim::GateType::NOT_A_GATE || g.name.empty()) {
            continue;
        }
        std::printf("G %s %u %u\n", std::string(g.name).c_str(), (unsigned)g.arg_count, (unsigned)g.flags);
    }
    for (const stim::GateDataMapHashEntry &e : stim::GATE_DATA.hashed_name_to_gate_type_table) {
        if (e.id == stim::GateType::NOT_A_GATE || e.expected_name.empty()) {
            continue;
        }
        const stim::Gate &g = stim::GATE_DATA[e.id];
        if (e.expected_name != g.name) {
            std::printf("A %s %s\n", std::string(e.expected_name).c_str(), std::string(g.name).c_str());
        }
    }
    return 0;
}
