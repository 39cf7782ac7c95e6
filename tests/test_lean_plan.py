"""The lean kernel's phase list against the device program, on the CPU (tests/lean_plan_check.cc): both are walked
over 32 shots with the same Clifford rules and the same Pauli hits for every noise occurrence, the phase list
applying each moved occurrence's hits through its transform; measured frames and final frames must agree."""

import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "stim_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("lean") / "lean_plan_check"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "lean_plan_check.cc"), os.path.join(CSRC, "lower.cc"),
                    os.path.join(CSRC, "circuit.cc"), "-o", str(exe)], check=True)
    return str(exe)


def circuit_files():
    names = ["surface_rz_d3_r3", "surface_rz_d25_r25", "surface_rx_d11_r11", "color_d5_r5", "color_d15_r15",
             "rep_d9_r9", "rep_d51_r51"]
    return [os.path.join(HERE, "golden", "circuits", n + ".stim") for n in names]


def fixture_circuits():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if "circuit" in np.load(f).files)


def run(checker, path):
    out = subprocess.run([checker, path], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    return out.stdout.split()


@pytest.mark.parametrize("path", circuit_files(), ids=os.path.basename)
def test_generated_codes(checker, path):
    res = run(checker, path)
    assert res[0] == "ok"
    assert int(res[3]) > 0  # some occurrences were moved (and transformed)


@pytest.mark.parametrize("name", fixture_circuits())
def test_reference_fixture_circuits(checker, name, tmp_path):
    path = tmp_path / "c.stim"
    path.write_text(str(np.load(os.path.join(HERE, "golden", name + ".npz"))["circuit"]))
    assert run(checker, str(path))[0] in ("ok", "no-lean", "skip:")
