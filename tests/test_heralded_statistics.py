"""Statistics of heralded noise as the reference's own tests state them (src/stim/simulators/frame_simulator.test.cc:
1553-1684, heralded_erase_detect_statistics / heralded_pauli_channel_1_statistics / the same offset by two qubits):
a pair measured in the X and Z bases around a heralded channel, three detectors (the two pair parities and the
herald), 2^18 shots binned by their detection pattern.  The oracle (CPU) and the GPU sampler (both noise modes,
bit for bit equal to the oracle) must land inside the reference's tolerances."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

SHOTS = 1 << 18

ERASE = """
    MXX {a} {b}
    MZZ {a} {b}
    HERALDED_ERASE(0.1) {a}
    MXX {a} {b}
    MZZ {a} {b}
    DETECTOR rec[-1] rec[-4]
    DETECTOR rec[-2] rec[-5]
    DETECTOR rec[-3]
"""
PAULI = """
    MXX {a} {b}
    MZZ {a} {b}
    HERALDED_PAULI_CHANNEL_1(0.05, 0.10, 0.15, 0.25) {a}
    MXX {a} {b}
    MZZ {a} {b}
    DETECTOR rec[-1] rec[-4]
    DETECTOR rec[-2] rec[-5]
    DETECTOR rec[-3]
"""
# (bin, expected fraction, tolerance); bins 1-3 (a flip without a herald) must be empty.
WANT_ERASE = [(0, 0.9, 0.05), (4, 0.025, 0.02), (5, 0.025, 0.02), (6, 0.025, 0.02), (7, 0.025, 0.02)]
WANT_PAULI = [(0, 0.45, 0.05), (4, 0.05, 0.04), (5, 0.10, 0.04), (6, 0.25, 0.04), (7, 0.15, 0.04)]
CASES = [("erase", ERASE, 0, 1, WANT_ERASE), ("erase_offset_by_2", ERASE, 2, 3, WANT_ERASE),
         ("pauli_channel_1", PAULI, 0, 1, WANT_PAULI)]


def check_bins(dets, want):
    bins = np.bincount(dets[:, 0] & 7, minlength=8)
    n = dets.shape[0]
    assert bins[1] == bins[2] == bins[3] == 0
    for b, frac, tol in want:
        assert abs(bins[b] / n - frac) <= tol, (b, bins[b] / n, frac)


@pytest.mark.parametrize("name,template,a,b,want", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference_statistics(name, template, a, b, want):
    d, _, _ = OracleCircuit(template.format(a=a, b=b)).sample(SHOTS, 7, threads=8)
    check_bins(d, want)


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("name,template,a,b,want", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_reference_statistics(name, template, a, b, want, noise_mode):
    text = template.format(a=a, b=b)
    s = stim_gb300.Circuit(text).compile_detector_sampler(seed=7)
    s.set_noise_mode(noise_mode)
    d = s.sample(SHOTS, bit_packed=True)
    check_bins(d, want)
    np.testing.assert_array_equal(d, OracleCircuit(text).sample(SHOTS, 7, threads=8)[0])


# src/stim/simulators/frame_simulator_pybind_test.py:406-414 (test_repro_heralded_pauli_channel_1_bug): a herald with
# only the "heralded identity" and X branches set fires on some shots, and the unheralded qubit stays 0.
HERALD_REPRO = "R 0 1\nHERALDED_PAULI_CHANNEL_1(0.2, 0.2, 0, 0) 1\nM 0"


def test_oracle_heralded_pauli_channel_repro():
    _, _, m = OracleCircuit(HERALD_REPRO).sample(1024, 9, dets=False, obs=False, meas=True)
    r = np.unpackbits(m, axis=1, bitorder="little")[:, :2]
    assert r[:, 0].sum() > 0 and r[:, 1].sum() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
def test_gpu_heralded_pauli_channel_repro(noise_mode):
    s = stim_gb300.Circuit(HERALD_REPRO).compile_sampler(seed=9)
    s.set_noise_mode(noise_mode)
    r = s.sample(1024)
    assert r[:, 0].sum() > 0 and r[:, 1].sum() == 0
