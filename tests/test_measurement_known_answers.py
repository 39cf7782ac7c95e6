"""Noisy measurements, measure-resets, Pauli-product measurements and Pauli observable terms as the reference's own
tests state them (src/stim/simulators/frame_simulator.test.cc:1177-1457 noisy_measurement_{x,y,z} and
noisy_measurement_reset_{x,y,z}, measure_pauli_product_4body, non_deterministic_pauli_product_detectors;
:1685-1744 observable_include_paulis_r{z,y,x}; frame_simulator_util.test.cc:223-426, the same noisy measurements
as detection events, one detector per measurement).  Raw measurement flips (reference sample all zeros) as the
reference tests sample them; the oracle on the CPU, the GPU samplers in both noise modes."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

# (basis, measurement, error that flips a measurement in that basis, whether the measurement resets)
NOISY = [("X", "MX", "Z_ERROR", False), ("Y", "MY", "Z_ERROR", False), ("Z", "MZ", "X_ERROR", False),
         ("X", "MRX", "Z_ERROR", True), ("Y", "MRY", "Z_ERROR", True), ("Z", "MRZ", "X_ERROR", True)]
MPP4 = """
    X_ERROR(0.5) 0 1 2 3
    Z_ERROR(0.5) 0 1 2 3
    MPP X0*X1*X2*X3
    MX 0 1 2 3 4 5
    MPP X2*X3*X4*X5
    MPP Z0*Z1*Z4*Z5 !Y0*Y1*Y4*Y5
"""
RANDOM_PRODUCTS = ["MPP Z8*X9\nDETECTOR rec[-1]", "MPP X9\nDETECTOR rec[-1]", "MX 9\nDETECTOR rec[-1]"]
OBS_PAULIS = "R{b} 0\nOBSERVABLE_INCLUDE(0) X0\nOBSERVABLE_INCLUDE(1) Y0\nOBSERVABLE_INCLUDE(2) Z0"


def meas_oracle(text, shots, seed):
    c = stim_gb300.Circuit(text)
    _, _, m = OracleCircuit(text).sample(shots, seed, dets=False, obs=False, meas=True, threads=4)
    return np.unpackbits(m, axis=1, bitorder="little")[:, :c.num_measurements]


def meas_gpu(text, shots, seed, noise_mode):
    s = stim_gb300.Circuit(text).compile_sampler(skip_reference_sample=True, seed=seed)
    s.set_noise_mode(noise_mode)
    return s.sample(shots).astype(np.uint8)


def with_detectors(text):
    """The circuit with one detector per measurement, in order (the detection-event form of the tests)."""
    n = stim_gb300.Circuit(text).num_measurements
    return text + "".join(f"\nDETECTOR rec[-{n - k}]" for k in range(n))


def dets_oracle(text, shots, seed):
    d, _, _ = OracleCircuit(with_detectors(text)).sample(shots, seed, obs=False, threads=4)
    return np.unpackbits(d, axis=1, bitorder="little")[:, :stim_gb300.Circuit(text).num_measurements]


def dets_gpu(text, shots, seed, noise_mode):
    s = stim_gb300.Circuit(with_detectors(text)).compile_detector_sampler(seed=seed)
    s.set_noise_mode(noise_mode)
    return s.sample(shots).astype(np.uint8)


def check_noisy(sample, basis, m, err, resets):
    r = sample(f"R{basis} 0\n{m}(0.05) 0\n{m} 0", 10000)
    assert not r[:, 1].any()
    assert 300 < r[:, 0].sum() < 700
    r = sample(f"R{basis} 0 1\n{err}(1) 0 1\n{m}(0.05) 0 1\n{m} 0 1", 5000)
    assert 10000 - 700 < r[:, 0].sum() + r[:, 1].sum() < 10000 - 300
    assert r[:, 2].sum() == r[:, 3].sum() == (0 if resets else 5000)


def check_mpp4(r):
    x0123, x0, x1, x2, x3, x4, x5, x2345, mz0145, y0145 = (r[:, k] for k in range(10))
    assert (x0123 == x0 ^ x1 ^ x2 ^ x3).all()
    assert (x2345 == x2 ^ x3 ^ x4 ^ x5).all()
    assert (y0145 ^ mz0145 == x0123 ^ x2345).all()


def check_obs_paulis(obs, basis):
    x0, y0, z0 = obs.sum(axis=0)
    random_pair, zero = {"Z": ((x0, y0), z0), "Y": ((x0, z0), y0), "X": ((y0, z0), x0)}[basis]
    assert random_pair[0] == random_pair[1] and 300 < random_pair[0] < 700
    assert zero == 0


@pytest.mark.parametrize("basis,m,err,resets", NOISY, ids=[n[1] for n in NOISY])
def test_oracle_noisy_measurements(basis, m, err, resets):
    check_noisy(lambda text, shots: meas_oracle(text, shots, 3), basis, m, err, resets)


@pytest.mark.parametrize("basis,m,err,resets", NOISY, ids=[n[1] for n in NOISY])
def test_oracle_noisy_measurement_detectors(basis, m, err, resets):
    check_noisy(lambda text, shots: dets_oracle(text, shots, 4), basis, m, err, resets)


def test_oracle_pauli_products():
    check_mpp4(meas_oracle(MPP4, 10, 5))
    for text in RANDOM_PRODUCTS:
        d, _, _ = OracleCircuit(text).sample(1000, 6)
        assert 400 < (d[:, 0] & 1).sum() < 600


@pytest.mark.parametrize("basis", ["Z", "Y", "X"])
def test_oracle_observable_paulis(basis):
    _, o, _ = OracleCircuit(OBS_PAULIS.format(b=basis)).sample(1024, 7)
    check_obs_paulis(np.unpackbits(o, axis=1, bitorder="little")[:, :3], basis)


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("basis,m,err,resets", NOISY, ids=[n[1] for n in NOISY])
def test_gpu_noisy_measurements(basis, m, err, resets, noise_mode):
    check_noisy(lambda text, shots: meas_gpu(text, shots, 3, noise_mode), basis, m, err, resets)


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("basis,m,err,resets", NOISY, ids=[n[1] for n in NOISY])
def test_gpu_noisy_measurement_detectors(basis, m, err, resets, noise_mode):
    check_noisy(lambda text, shots: dets_gpu(text, shots, 4, noise_mode), basis, m, err, resets)


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
def test_gpu_pauli_products(noise_mode):
    check_mpp4(meas_gpu(MPP4, 10, 5, noise_mode))
    for text in RANDOM_PRODUCTS:
        s = stim_gb300.Circuit(text).compile_detector_sampler(seed=6)
        s.set_noise_mode(noise_mode)
        assert 400 < s.sample(1000).sum() < 600


@pytest.mark.gpu
@pytest.mark.parametrize("basis", ["Z", "Y", "X"])
def test_gpu_observable_paulis(basis):
    s = stim_gb300.Circuit(OBS_PAULIS.format(b=basis)).compile_detector_sampler(seed=7)
    _, o = s.sample(1024, separate_observables=True)
    check_obs_paulis(o.astype(np.int64), basis)
