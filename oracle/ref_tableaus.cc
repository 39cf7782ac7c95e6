// ref_tableaus -- prints the REFERENCE's Heisenberg images of every unitary gate (stim::GATE_DATA's tableau data,
// src/stim/gates/gates.h:273-285): for a one-qubit gate the images of X and Z, for a two-qubit gate the images of
// X0, Z0, X1, Z1, each as a signed Pauli string ("+XZ", "-Y_").
//
// Test infrastructure only: compiled from the reference's sources where they lie (never copied) by
// `make -C oracle ref`, run by tests/golden/make_gate_tableaus.py, which commits its output as a fixture.  The
// product's frame rules (stim_gb300/csrc/frame_rules.h, reached through the lowering of each gate) are checked
// against it by tests/gate_frame_check.cc, the reference's bulk_operations_consistent_with_tableau_data
// (src/stim/simulators/frame_simulator.test.cc:98-126) restated.
//
// Usage: ref_tableaus  ->  one line per unitary gate with one- or two-qubit tableau data (SPP / SPP_DAG, which take
// Pauli products of any size, have none): "T <name> <qubits> <image> ...".

#include <cstdio>
#include <stdexcept>
#include <string>

#include "stim/gates/gates.h"
#include "stim/stabilizers/tableau.h"

int main() {
    for (const stim::Gate &g : stim::GATE_DATA.items) {
        if (g.id == stim::GateType::NOT_A_GATE || g.name.empty() || !(g.flags & stim::GATE_IS_UNITARY)) {
            continue;
        }
        stim::Tableau<64> t(0);
        try {
            t = g.tableau<64>();
        } catch (const std::out_of_range &) {
            continue;
        }
        std::printf("T %s %zu", std::string(g.name).c_str(), t.num_qubits);
        for (size_t k = 0; k < t.num_qubits; k++) {
            std::printf(" %s %s", t.xs[k].str().c_str(), t.zs[k].str().c_str());
        }
        std::printf("\n");
    }
    return 0;
}
