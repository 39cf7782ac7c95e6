"""The reference's FrameSimulator tests that fix exact outputs, restated against this package
(src/stim/simulators/frame_simulator.test.cc):

* :289-330 sample_batch_measurements_writing_results_to_disk, :331-372 big_circuit_measurements,
  :373-408 run_length_measurement_formats, :409-424 big_circuit_random_measurements;
* :706-826 classical_controls (record-controlled Paulis, the record holding flips against the reference sample);
* :839-860 stream_huge_case (400,000 measurements per shot), :861-977 block_results / stream_results /
  stream_many_shots (long loops, odd shot counts);
* :978-1026 measure_y_without_reset_doesnt_reset, :1027-1176 resets_vs_measurements;
* :1458-1473 ignores_sweep_controls_when_given_no_sweep_data.

The reference's `sample_batch_measurements(circuit, ref, ...)` returns measurement flips XOR `ref`; with `ref` all
zeros that is this package's compile_sampler(skip_reference_sample=True), and with the circuit's own reference
sample it is compile_sampler().  Deterministic cases run on the oracle (CPU) and on the GPU sampler in both noise
modes."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

# frame_simulator.test.cc:706-826: (circuit, measurement results of every shot).
CLASSICAL_CONTROLS = [
    ("M 0\nCX rec[-1] 1\nM 1", [0, 0]),
    ("M !0\nCX rec[-1] 1\nM 1", [0, 0]),
    ("X_ERROR(1) 0\nM !0\nCX rec[-1] 1\nM 1", [1, 1]),
    ("X_ERROR(1) 0\nM 0\nCX rec[-1] 1\nM 1", [1, 1]),
    ("X_ERROR(1) 0\nM 0\nH 1\nCZ rec[-1] 1\nH 1\nM 1", [1, 1]),
    ("X_ERROR(1) 0\nM 0\nCY rec[-1] 1\nM 1", [1, 1]),
]

FLIPS = """
    H_XZ 0 1 2
    H_YZ 3 4 5
    X_ERROR(1) 0 3 6
    Y_ERROR(1) 1 4 7
    Z_ERROR(1) 2 5 8
"""
# frame_simulator.test.cc:1027-1176: (circuit, measurement flips of every shot).
RESETS_VS_MEASUREMENTS = [
    ("RX 0\nRY 1\nRZ 2\nH_XZ 0\nH_YZ 1\nM 0 1 2", [0, 0, 0]),
    (FLIPS + "MX 0 1 2\nMY 3 4 5\nMZ 6 7 8", [0, 1, 1, 1, 0, 1, 1, 1, 0]),
    (FLIPS + "MX !0 !1 !2\nMY !3 !4 !5\nMZ !6 !7 !8", [0, 1, 1, 1, 0, 1, 1, 1, 0]),
    (FLIPS + "MRX 0 1 2\nMRY 3 4 5\nMRZ 6 7 8\nH_XZ 0\nH_YZ 3\nM 0 3 6", [0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 0, 0]),
    (FLIPS + "MRX !0 !1 !2\nMRY !3 !4 !5\nMRZ !6 !7 !8\nH_XZ 0\nH_YZ 3\nM 0 3 6",
     [0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 0, 0]),
    ("H_XZ 0\nH_YZ 1\nZ_ERROR(1) 0 1\nX_ERROR(1) 2\nMRX 0 0\nMRY 1 1\nMRZ 2 2", [1, 0, 1, 0, 1, 0]),
]

# frame_simulator.test.cc:978-1026: (circuit, whether each measurement flips in every shot).
MEASURE_Y = [
    ("RY 0\nMY 0\nMY 0\nZ_ERROR(1) 0\nMY 0\nMY 0\nZ_ERROR(1) 0\nMY 0\nMY 0", [0, 0, 1, 1, 0, 0]),
    ("RY 0\nMRY 0\nMRY 0\nZ_ERROR(1) 0\nMRY 0\nMRY 0\nZ_ERROR(1) 0\nMRY 0\nMRY 0", [0, 0, 1, 0, 1, 0]),
]
DETERMINISTIC = CLASSICAL_CONTROLS + RESETS_VS_MEASUREMENTS + MEASURE_Y
SWEEP = "CNOT sweep[0] 0\nM 0\nDETECTOR rec[-1]"


def oracle_flips(text, shots, seed=3):
    o = OracleCircuit(text)
    _, _, m = o.sample(shots, seed, dets=False, obs=False, meas=True)
    return np.unpackbits(m, axis=1, bitorder="little")[:, :o.num_measurements]


@pytest.mark.parametrize("text,want", DETERMINISTIC)
def test_oracle_deterministic_flips(text, want):
    np.testing.assert_array_equal(oracle_flips(text, 100), np.array([want] * 100, dtype=np.uint8))


def test_oracle_classical_control_of_random_flip():
    r = oracle_flips("X_ERROR(0.5) 0\nM 0\nCX rec[-1] 1\nM 1", 1000)
    assert (r[:, 0] == r[:, 1]).all()
    assert 400 < r[:, 0].sum() < 600


def test_oracle_ignores_sweep_controls():
    o = OracleCircuit(SWEEP)
    d, _, m = o.sample(1000, 5, dets=True, obs=False, meas=True)
    assert not d.any() and not m.any()


def gpu_sampler(text, noise_mode, seed=7, **kw):
    s = stim_gb300.Circuit(text).compile_sampler(seed=seed, **kw)
    s.set_noise_mode(noise_mode)
    return s


NOISE_MODES = pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])


@pytest.mark.gpu
@NOISE_MODES
@pytest.mark.parametrize("text,want", DETERMINISTIC)
def test_gpu_deterministic_flips(text, want, noise_mode):
    r = gpu_sampler(text, noise_mode, skip_reference_sample=True).sample(100)
    np.testing.assert_array_equal(r, np.array([want] * 100, dtype=np.bool_))


@pytest.mark.gpu
@NOISE_MODES
def test_gpu_classical_control_of_random_flip(noise_mode):
    r = gpu_sampler("X_ERROR(0.5) 0\nM 0\nCX rec[-1] 1\nM 1", noise_mode, skip_reference_sample=True).sample(1000)
    assert (r[:, 0] == r[:, 1]).all()
    assert 400 < r[:, 0].sum() < 600


@pytest.mark.gpu
@NOISE_MODES
def test_gpu_ignores_sweep_controls(noise_mode):
    c = stim_gb300.Circuit(SWEEP)
    assert not gpu_sampler(SWEEP, noise_mode, skip_reference_sample=True).sample(1000).any()
    s = c.compile_detector_sampler(seed=7)
    s.set_noise_mode(noise_mode)
    assert not s.sample(1000).any()


@pytest.mark.gpu
def test_gpu_measurements_writing_results_to_disk(tmp_path):
    # frame_simulator.test.cc:289-330: X 0, then M 1 0 2 3 with the circuit's reference sample.
    c = stim_gb300.Circuit("X 0\nM 1\nM 0\nM 2\nM 3")
    s = c.compile_sampler()
    np.testing.assert_array_equal(s.sample(10, bit_packed=True), np.full((10, 1), 2, dtype=np.uint8))
    path = tmp_path / "out"
    s.sample_write(5, filepath=str(path), format="01")
    assert path.read_text() == "0100\n" * 5
    s.sample_write(5, filepath=str(path), format="b8")
    assert path.read_bytes() == b"\x02" * 5
    s.sample_write(64, filepath=str(path), format="ptb64")
    assert path.read_bytes() == b"\x00" * 8 + b"\xff" * 8 + b"\x00" * 16


@pytest.mark.gpu
def test_gpu_big_circuit_measurements(tmp_path):
    # frame_simulator.test.cc:331-372: X on every third of 1,250 qubits, then M on each.
    text = "".join(f"X {k}\n" for k in range(0, 1250, 3)) + "".join(f"M {k}\n" for k in range(1250))
    s = stim_gb300.Circuit(text).compile_sampler()
    want = np.arange(1250) % 3 == 0
    np.testing.assert_array_equal(s.sample(750), np.broadcast_to(want, (750, 1250)))
    path = tmp_path / "out"
    s.sample_write(750, filepath=str(path), format="01")
    line = "".join("01"[int(b)] for b in want) + "\n"
    assert path.read_text() == line * 750
    s.sample_write(750, filepath=str(path), format="b8")
    row = np.packbits(want, bitorder="little").tobytes()
    assert path.read_bytes() == row * 750


@pytest.mark.gpu
def test_gpu_run_length_measurement_formats(tmp_path):
    # frame_simulator.test.cc:373-408: X on 100, 500, 501, 551, 1200 of 1,250 measured qubits.
    text = "X 100 500 501 551 1200\n" + "".join(f"M {k}\n" for k in range(1250))
    s = stim_gb300.Circuit(text).compile_sampler()
    path = tmp_path / "out"
    s.sample_write(3, filepath=str(path), format="hits")
    assert path.read_text() == "100,500,501,551,1200\n" * 3
    s.sample_write(3, filepath=str(path), format="dets")
    assert path.read_text() == "shot M100 M500 M501 M551 M1200\n" * 3
    s.sample_write(3, filepath=str(path), format="r8")
    assert path.read_bytes() == bytes([100, 255, 400 - 255 - 1, 0, 49, 255, 255, 1200 - 551 - 255 * 2 - 1,
                                       1250 - 1200 - 1]) * 3


@pytest.mark.gpu
def test_gpu_big_circuit_random_measurements():
    # frame_simulator.test.cc:409-424: 270 qubits in |+>, measured in Z: no shot is all zeros.
    text = "".join(f"H_XZ {k}\n" for k in range(270)) + "".join(f"M {k}\n" for k in range(270))
    r = stim_gb300.Circuit(text).compile_sampler(seed=11).sample(1000)
    assert r.any(axis=1).all()


@pytest.mark.gpu
@NOISE_MODES
def test_gpu_stream_huge_case(tmp_path, noise_mode):
    # frame_simulator.test.cc:839-860: 400,000 measurements per shot, qubit 2 always flipped.
    s = gpu_sampler("X_ERROR(1) 2\nREPEAT 100000 {\n    M 0 1 2 3\n}", noise_mode)
    path = tmp_path / "out"
    s.sample_write(256, filepath=str(path), format="b8")
    data = np.fromfile(path, dtype=np.uint8)
    assert data.size == 256 * 100000 * 4 // 8
    assert (data == 0x44).all()


@pytest.mark.gpu
@NOISE_MODES
@pytest.mark.parametrize("shots", [1, 3])
def test_gpu_block_results(tmp_path, noise_mode, shots):
    # frame_simulator.test.cc:861-907, 908-930, 952-977: 10,000 iterations of X_ERROR(1) 0, MR 0, M 0 0.
    s = gpu_sampler("REPEAT 10000 {\n    X_ERROR(1) 0\n    MR 0\n    M 0 0\n}", noise_mode)
    path = tmp_path / "out"
    s.sample_write(shots, filepath=str(path), format="01")
    assert path.read_text() == ("100" * 10000 + "\n") * shots


@pytest.mark.gpu
@NOISE_MODES
def test_gpu_stream_many_shots(tmp_path, noise_mode):
    # frame_simulator.test.cc:931-951: 2,049 shots (a partial 128-shot block), qubit 1 always flipped.
    s = gpu_sampler("X_ERROR(1) 1\nM 0 1 2", noise_mode)
    path = tmp_path / "out"
    s.sample_write(2049, filepath=str(path), format="01")
    assert path.read_text() == "010\n" * 2049


def test_bad_detector_rejected():
    # frame_simulator_util.test.cc:46-48: a bare record target is not a circuit.
    with pytest.raises(ValueError):
        stim_gb300.Circuit("rec[-1]")
