"""The product's gate vocabulary (stim_gb300/csrc/gfs_gates.h) against the reference's own GATE_DATA.

tests/golden/gates.txt is written by tests/golden/make_gates.py from oracle/ref_gates.cc, which prints the
reference's table (src/stim/gates/gates.h:192-390) compiled from the reference's sources.  The CPU oracle parses
circuits with the same gfs_gates.h as the product, so the oracle cannot catch a wrong entry there; this test pins
every name, alias, argument count and flag word to the reference directly.
"""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "stim_gb300", "csrc")

# Prints the table the parser uses: "G name arg_count flags" per gate, "A alias canonical" per alias.
DUMP_C = r"""
#include <stdio.h>
#include "gfs_gates.h"
int main(void) {
    size_t n = sizeof(GFS_GATE_TABLE) / sizeof(GFS_GATE_TABLE[0]);
    for (size_t k = 0; k < n; k++) {
        int a = GFS_GATE_TABLE[k].arg_count;
        unsigned ac = a == GFS_ARGS_ANY ? 255u : a == GFS_ARGS_ZERO_OR_ONE ? 254u : (unsigned)a;
        printf("G %s %u %u\n", GFS_GATE_TABLE[k].name, ac, (unsigned)GFS_GATE_TABLE[k].flags);
    }
    size_t na = sizeof(GFS_GATE_ALIASES) / sizeof(GFS_GATE_ALIASES[0]);
    for (size_t k = 0; k < na; k++) {
        printf("A %s %s\n", GFS_GATE_ALIASES[k].name, gfs_gate_by_id(GFS_GATE_ALIASES[k].id)->name);
    }
    return 0;
}
"""


def parse(text):
    gates, aliases = {}, {}
    for line in text.splitlines():
        parts = line.split()
        if not parts:
            continue
        if parts[0] == "G":
            gates[parts[1]] = (int(parts[2]), int(parts[3]))
        elif parts[0] == "A":
            aliases[parts[1]] = parts[2]
    return gates, aliases


@pytest.fixture(scope="module")
def tables(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("gates")
    src, exe = d / "dump.c", d / "dump"
    src.write_text(DUMP_C)
    subprocess.run([cc, "-std=c11", "-I", CSRC, "-o", str(exe), str(src)], check=True)
    ours = parse(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout)
    with open(os.path.join(HERE, "golden", "gates.txt")) as f:
        ref = parse(f.read())
    return ours, ref


def test_every_gate_matches_the_reference(tables):
    (gates, _), (ref_gates, _) = tables
    for name, (args, flags) in gates.items():
        assert name in ref_gates, f"{name} is not a reference gate"
        assert (args, flags) == ref_gates[name], f"{name}: ours (args, flags) {(args, flags)}, reference {ref_gates[name]}"


def test_every_reference_gate_is_known(tables):
    (gates, _), (ref_gates, _) = tables
    assert sorted(set(ref_gates) - set(gates)) == []


def test_aliases_match_the_reference(tables):
    (_, aliases), (_, ref_aliases) = tables
    assert aliases == ref_aliases
