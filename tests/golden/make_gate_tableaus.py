"""Writes tests/golden/gate_tableaus.txt: the REFERENCE's Heisenberg images of every unitary gate with one- or
two-qubit tableau data, as its own GATE_DATA holds them.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref REF=<reference tree>     # builds oracle/_ref/ref_tableaus from the reference's own sources
    python tests/golden/make_gate_tableaus.py

Each line is "T <name> <qubits>" followed by the images of X0, Z0 (and X1, Z1) as signed Pauli strings.
tests/test_gate_frames.py checks the product's frame rules, reached through the lowering of each gate, against it.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_TABLEAUS = os.path.join(ROOT, "oracle", "_ref", "ref_tableaus")


def main():
    out = subprocess.run([REF_TABLEAUS], check=True, capture_output=True, text=True).stdout
    lines = sorted(out.splitlines())
    with open(os.path.join(HERE, "gate_tableaus.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"{len(lines)} gates")


if __name__ == "__main__":
    main()
