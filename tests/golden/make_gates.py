"""Writes tests/golden/gates.txt: the REFERENCE's gate vocabulary as its own GATE_DATA holds it.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref REF=<reference tree>     # builds oracle/_ref/ref_gates from the reference's own sources
    python tests/golden/make_gates.py

Each line is "G <name> <arg_count> <GateFlags bits>" (arg_count 255 = any number, 254 = zero or one;
src/stim/gates/gates.h:44-49, 192-233) or "A <alias> <canonical name>".  tests/test_gate_table.py checks the
product's table (stim_gb300/csrc/gfs_gates.h) against it.
"""

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_GATES = os.path.join(ROOT, "oracle", "_ref", "ref_gates")


def main():
    out = subprocess.run([REF_GATES], check=True, capture_output=True, text=True).stdout
    lines = sorted(out.splitlines(), key=lambda s: (s[0] != "G", s))
    with open(os.path.join(HERE, "gates.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print(f"{sum(1 for s in lines if s[0] == 'G')} gates, {sum(1 for s in lines if s[0] == 'A')} aliases")


if __name__ == "__main__":
    main()
