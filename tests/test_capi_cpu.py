"""C ABI checks that need no GPU: the library loads, exports every declared symbol, parses circuits
with the reference's statistics and errors, and refuses to sample without a device (no CPU fallback)."""

import ctypes
import os
import re

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR, ROOT, golden_names
from oracle.oracle import OracleCircuit
from stim_gb300 import _native, workloads


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"\b(gfs_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _native.lib()
    syms = declared_symbols()
    assert len(syms) >= 14
    for name in syms:
        assert hasattr(L, name), name


@pytest.mark.parametrize("name", golden_names())
def test_parse_stats_match_reference(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    c = stim_gb300.Circuit(str(g["circuit"]))
    assert c.num_detectors == int(g["num_detectors"])
    assert c.num_observables == int(g["num_observables"])
    assert c.num_measurements == int(g["num_measurements"])
    o = OracleCircuit(str(g["circuit"]))
    assert c.num_qubits == o.num_qubits
    assert c.max_lookback == o.max_lookback
    assert c.num_instructions_unrolled == o.num_instances


def test_parse_large_surface_code():
    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_z", 25, 25, 0.001))
    assert (c.num_qubits, c.num_measurements, c.num_detectors, c.num_observables, c.max_lookback) == (
        1324, 16225, 15600, 1, 1248)


@pytest.mark.parametrize("text,err", [
    ("H 0\nCX 0", ValueError),
    ("X_ERROR(1.5) 0", ValueError),
    ("NOT_A_GATE 0", ValueError),
    ("REPEAT 0 {\nH 0\n}", ValueError),
    ("REPEAT 2 {\nH 0\n", ValueError),
    ("}", ValueError),
    ("H 0 rec[-1]", ValueError),
    ("CX 0 0", ValueError),
    ("MPP X0*", ValueError),
    ("DEPOLARIZE1(0.1, 0.2) 0", ValueError),
    ("H0", ValueError),
])
def test_parse_errors(text, err):
    with pytest.raises(err):
        stim_gb300.Circuit(text)
    with pytest.raises(ValueError):
        OracleCircuit(text)


def test_parse_fuses_like_the_reference():
    c = stim_gb300.Circuit("H 0\nH 1\nX_ERROR(0.1) 0\nX_ERROR(0.1) 1\nX_ERROR(0.2) 2\nTICK\nTICK\nREPEAT 3 {\nH 0\n}\nH 1")
    o = OracleCircuit("H 0\nH 1\nX_ERROR(0.1) 0\nX_ERROR(0.1) 1\nX_ERROR(0.2) 2\nTICK\nTICK\nREPEAT 3 {\nH 0\n}\nH 1")
    assert c.num_instructions_unrolled == o.num_instances == 1 + 1 + 1 + 2 + 3 + 1


def test_sampling_without_gpu_raises_instead_of_falling_back():
    if _native.device_count() > 0:
        pytest.skip("a CUDA device is present")
    c = stim_gb300.Circuit("X_ERROR(1) 0\nM 0\nDETECTOR rec[-1]")
    with pytest.raises((RuntimeError, ValueError)):
        c.compile_detector_sampler(seed=1)


@pytest.mark.parametrize("name", golden_names())
def test_lowering_succeeds_on_host(name):
    g = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    c = stim_gb300.Circuit(str(g["circuit"]))
    for mode in ("detections", "measurements"):
        info = c.program_info(mode)
        assert info["detectors"] == c.num_detectors
        assert info["rows"] <= c.num_qubits
        assert info["ring"] >= max(1, c.max_lookback)


def test_lowering_keeps_repeat_as_loops():
    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_z", 25, 25, 0.001))
    info = c.program_info()
    assert info["loop_depth"] == 1
    assert info["rows"] == 1249
    assert info["ops"] < 200  # the 24-round body is emitted once, not unrolled
    assert 3 * info["smem_bytes_per_block"] <= 227 * 1024  # three CTAs per SM


def test_noise_occurrence_accounting():
    # Occurrences with loops unrolled: the d=3 memory experiment has its noise in a 2-round REPEAT body.
    from stim_gb300 import _native

    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.001))
    info = c.program_info()
    assert info["noise_occurrences"] > 0
    # Expected hits per 128-shot block ~ p x (noisy units) x 128 shots.
    assert 0 < info["hits_per_block"] < 10000
    c0 = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.0))
    assert c0.program_info()["noise_occurrences"] == 0
    assert _native.lib() is not None


@pytest.mark.parametrize("name", golden_names())
def test_reference_sample_matches_reference_tableau(name):
    # The reference's own TableauSimulator::reference_sample_circuit output, stored with each fixture.
    g = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    c = stim_gb300.Circuit(str(g["circuit"]))
    np.testing.assert_array_equal(c.reference_sample(bit_packed=True), g["ref_sample"])
    bits = c.reference_sample()
    assert bits.dtype == np.bool_ and bits.shape == (c.num_measurements,)
    np.testing.assert_array_equal(np.packbits(bits, bitorder="little"), g["ref_sample"])


def test_reference_sample_random_small_circuits():
    d = np.load(os.path.join(GOLDEN_DIR, "refsample_random.npz"))
    for text, row, n in zip(d["circuits"], d["samples"], d["lengths"]):
        got = stim_gb300.Circuit(str(text)).reference_sample(bit_packed=True)
        np.testing.assert_array_equal(got, row[:n], err_msg=str(text))


def test_reference_sample_multi_target_circuits():
    # Measurements, resets and pair measurements on several entangled targets at once: which random outcome the
    # reference forces to 0 depends on the order it collapses an instruction's targets in (X / Y bases ascending
    # by qubit, Z in the order given; pair measurements per run of disjoint pairs).
    d = np.load(os.path.join(GOLDEN_DIR, "refsample_multi.npz"))
    for text, row, n in zip(d["circuits"], d["samples"], d["lengths"]):
        got = stim_gb300.Circuit(str(text)).reference_sample(bit_packed=True)
        np.testing.assert_array_equal(got, row[:n], err_msg=str(text))


def test_binding_example_compiles_and_runs(tmp_path):
    # The host half of the binding the integration notes show (tests/binding_example.cc), compiled against
    # include/stim_gb300.h and linked to the library: parse, counts, reference sample, and sampler creation, which
    # without a GPU must fail with GFS_ERR_CUDA and a message.
    import shutil
    import subprocess

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib_dir = os.path.dirname(_native.lib()._name)
    exe = tmp_path / "binding_example"
    subprocess.run([cxx, "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "binding_example.cc"), "-L", lib_dir, "-lstim_gb300",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.strip()
    assert re.fullmatch(r"measurements 4 reference 1000 sampler (0|3 message)", out), out
