"""CORRELATED_ERROR / ELSE_CORRELATED_ERROR chains as the reference's own test states them
(src/stim/simulators/frame_simulator.test.cc:425-572, FrameSimulator.correlated_error): deterministic chains with
probabilities 0 and 1 give exact measurement records, and a 0.5 / 0.25 / 0.75 chain gives the stated rates
(X0: 1/2, X1: 1/2 * 1/4, X2: 1/2 * 3/4 * 3/4).  Measurements are the raw flips (reference sample all zeros), as the
reference test samples them; the oracle on the CPU, the GPU sampler in both noise modes."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

CHAINS = [
    ("CORRELATED_ERROR(0) X0 X1\nELSE_CORRELATED_ERROR(0) X1 X2\nELSE_CORRELATED_ERROR(0) X2 X3\nM 0 1 2 3", [0, 0, 0, 0]),
    ("CORRELATED_ERROR(1) X0 X1\nELSE_CORRELATED_ERROR(0) X1 X2\nELSE_CORRELATED_ERROR(0) X2 X3\nM 0 1 2 3", [1, 1, 0, 0]),
    ("CORRELATED_ERROR(0) X0 X1\nELSE_CORRELATED_ERROR(1) X1 X2\nELSE_CORRELATED_ERROR(0) X2 X3\nM 0 1 2 3", [0, 1, 1, 0]),
    ("CORRELATED_ERROR(0) X0 X1\nELSE_CORRELATED_ERROR(0) X1 X2\nELSE_CORRELATED_ERROR(1) X2 X3\nM 0 1 2 3", [0, 0, 1, 1]),
    ("CORRELATED_ERROR(1) X0 X1\nELSE_CORRELATED_ERROR(1) X1 X2\nELSE_CORRELATED_ERROR(0) X2 X3\nM 0 1 2 3", [1, 1, 0, 0]),
    ("CORRELATED_ERROR(1) X0 X1\nELSE_CORRELATED_ERROR(1) X1 X2\nELSE_CORRELATED_ERROR(1) X2 X3\nM 0 1 2 3", [1, 1, 0, 0]),
    ("CORRELATED_ERROR(1) X0 X1\nELSE_CORRELATED_ERROR(1) X1 X2\nELSE_CORRELATED_ERROR(1) X2 X3\n"
     "CORRELATED_ERROR(1) X3 X4\nM 0 1 2 3 4", [1, 1, 0, 1, 1]),
]
RATES = "CORRELATED_ERROR(0.5) X0\nELSE_CORRELATED_ERROR(0.25) X1\nELSE_CORRELATED_ERROR(0.75) X2\nM 0 1 2"
SHOTS = 10000


def unpack(m, n):
    return np.unpackbits(m, axis=1, bitorder="little")[:, :n]


def check_rates(bits):
    hits = bits.sum(axis=0)
    assert 0.45 * SHOTS < hits[0] < 0.55 * SHOTS
    assert (0.125 - 0.05) * SHOTS < hits[1] < (0.125 + 0.05) * SHOTS
    assert (0.28125 - 0.05) * SHOTS < hits[2] < (0.28125 + 0.05) * SHOTS


@pytest.mark.parametrize("text,want", CHAINS)
def test_oracle_chains(text, want):
    _, _, m = OracleCircuit(text).sample(64, 3, dets=False, obs=False, meas=True)
    assert (unpack(m, len(want)) == np.array(want, dtype=np.uint8)).all()


def test_oracle_chain_rates():
    _, _, m = OracleCircuit(RATES).sample(SHOTS, 5, dets=False, obs=False, meas=True)
    check_rates(unpack(m, 3))


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("text,want", CHAINS)
def test_gpu_chains(text, want, noise_mode):
    s = stim_gb300.Circuit(text).compile_sampler(skip_reference_sample=True, seed=3)
    s.set_noise_mode(noise_mode)
    m = s.sample(64, bit_packed=True)
    assert (unpack(m, len(want)) == np.array(want, dtype=np.uint8)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
def test_gpu_chain_rates(noise_mode):
    s = stim_gb300.Circuit(RATES).compile_sampler(skip_reference_sample=True, seed=5)
    s.set_noise_mode(noise_mode)
    m = s.sample(SHOTS, bit_packed=True)
    check_rates(unpack(m, 3))
    _, _, om = OracleCircuit(RATES).sample(SHOTS, 5, dets=False, obs=False, meas=True)
    np.testing.assert_array_equal(m, om)
