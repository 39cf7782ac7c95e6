"""Frame rules of every unitary gate against the reference's own tableau data, on the CPU (tests/gate_frame_check.cc;
the reference's bulk_operations_consistent_with_tableau_data, src/stim/simulators/frame_simulator.test.cc:98-126):
each gate of tests/golden/gate_tableaus.txt (the reference's GATE_DATA, tests/golden/make_gate_tableaus.py) is
lowered by the product and its ops applied with the product's frame rules to X0, Z0, X1, Z1; every result must be
the gate's Heisenberg image, signs aside.  The oracle restates the frame rules on its own, so this pins the
product's rules and gate-to-rule mapping directly to the reference."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "stim_gb300", "csrc")
TABLEAUS = os.path.join(HERE, "golden", "gate_tableaus.txt")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("gates") / "gate_frame_check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "gate_frame_check.cc"), os.path.join(CSRC, "lower.cc"),
                    os.path.join(CSRC, "circuit.cc"), "-o", str(exe)], check=True)
    return str(exe)


def test_fixture_covers_every_one_and_two_qubit_unitary():
    names = [line.split()[1] for line in open(TABLEAUS) if line.startswith("T ")]
    assert len(names) == 46
    for name in ["H", "S", "SQRT_X", "C_XYZ", "CX", "CZ", "ISWAP", "SQRT_ZZ_DAG", "SWAPCX", "CZSWAP", "I", "Y"]:
        assert name in names


def test_frame_rules_match_reference_tableaus(checker):
    out = subprocess.run([checker, TABLEAUS], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.split() == ["ok", "46"]
