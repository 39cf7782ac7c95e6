"""The reference's measurements-to-detection-events tests, restated against this package
(src/stim/simulators/measurements_to_detection_events.test.cc): :25-143 single_detector_no_sweep_data,
:145-215 sweep_data, :217-243 empty_cases, :245-297 big_shots / big_data, :299-370 append_observables,
:372-428 file_01_to_dets_{no,yes}_obs, :430-506 with_error_propagation, :508-571 many_shots /
many_measurements_and_detectors, :573-600 file_01_to_01_yes_obs, :602-676 empty inputs.

A detector fires when its measurements' parity differs from their parity in the circuit's reference sample (sweep
bits flipping the results they control).  The oracle on the CPU takes the cases without sweep bits; the GPU
converter takes all of them, through convert and convert_file."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

# single_detector_no_sweep_data: (circuit, value of the one recorded measurement bit, detection event).
SINGLE = [
    ("M 0\nDETECTOR rec[-1]", 0, 0),
    ("M !0\nDETECTOR rec[-1]", 0, 1),
    ("X 0\nM 0\nDETECTOR rec[-1]", 0, 1),
    ("M 0\nDETECTOR rec[-1]", 1, 1),
    ("M !0\nDETECTOR rec[-1]", 1, 0),
    ("X 0\nM 0\nDETECTOR rec[-1]", 1, 0),
    ("M 0 1\nDETECTOR rec[-1]", 1, 0),
    ("M 0 1\nDETECTOR rec[-2]", 1, 1),
    ("M 0 1\nDETECTOR rec[-1] rec[-2]", 1, 1),
    ("M 0 1\nDETECTOR", 1, 0),
]
BIG = "M 0 !1\nREPEAT {n} {{\n    DETECTOR rec[-2]\n    DETECTOR rec[-1]\n}}"
APPEND = ["X 0\nM 0\nOBSERVABLE_INCLUDE(9) rec[-1]",
          "X 0\nM 0\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(9) rec[-1]\nDETECTOR rec[-1]"]
FILE_CIRCUIT = "X 0\nM 0\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(9) rec[-1]\nDETECTOR\nDETECTOR rec[-1]"


def measurement_rows(circuit_text, shots, first_bit):
    n = stim_gb300.Circuit(circuit_text).num_measurements
    m = np.zeros((shots, n), dtype=np.bool_)
    if n:
        m[:, 0] = bool(first_bit)
    return m


def oracle_m2d(text, meas_bool):
    c = stim_gb300.Circuit(text)
    o = OracleCircuit(text)
    ref = c.reference_sample(bit_packed=True)
    d, obs = o.m2d(np.packbits(meas_bool, axis=1, bitorder="little"), ref if ref.size else None)
    unpack = lambda a, n: np.unpackbits(a, axis=1, bitorder="little")[:, :n].astype(np.bool_)
    return unpack(d, o.num_detectors), unpack(obs, o.num_observables)


@pytest.mark.parametrize("text,bit,want", SINGLE)
def test_oracle_single_detector(text, bit, want):
    d, _ = oracle_m2d(text, measurement_rows(text, 256, bit))
    assert (d[:, 0] == bool(want)).all()


@pytest.mark.parametrize("reps,shots", [(50, 512), (200, 256)])
def test_oracle_big(reps, shots):
    text = BIG.format(n=reps)
    d, _ = oracle_m2d(text, measurement_rows(text, shots, 0))
    assert d.shape == (shots, 2 * reps)
    assert not d[:, 0::2].any() and d[:, 1::2].all()


def test_oracle_append_observables():
    d, o = oracle_m2d(APPEND[0], measurement_rows(APPEND[0], 256, 0))
    assert d.shape == (256, 0) and o.shape == (256, 10)
    assert o[:, 9].all() and not o[:, :9].any()
    d, o = oracle_m2d(APPEND[1], measurement_rows(APPEND[1], 256, 0))
    assert d.all() and o[:, 9].all() and not o[:, :9].any()


def test_empty_circuit_counts():
    # empty_cases: no detectors, whatever the measurements.
    for text in ["", "X 0\nM 0"]:
        c = stim_gb300.Circuit(text)
        assert c.num_detectors == 0 and c.num_observables == 0


def gpu_convert(text, meas_bool, sweep=None, append=False):
    conv = stim_gb300.Circuit(text).compile_m2d_converter()
    return conv.convert(measurements=meas_bool, sweep_bits=sweep, separate_observables=False,
                        append_observables=append)


@pytest.mark.gpu
@pytest.mark.parametrize("text,bit,want", SINGLE)
def test_gpu_single_detector(text, bit, want):
    d = gpu_convert(text, measurement_rows(text, 256, bit))
    assert d.shape == (256, 1) and (d[:, 0] == bool(want)).all()


@pytest.mark.gpu
def test_gpu_sweep_data():
    meas = np.zeros((11, 10), dtype=np.bool_)
    for k in range(10):
        meas[k, 9 - k] = True
    sweep = np.zeros((11, 4), dtype=np.bool_)
    for k in range(1, 5):
        sweep[k, k - 1] = True
        sweep[k + 5, k - 1] = True
    sweep[10, :] = True
    text = """
        CNOT sweep[0] 1 sweep[0] 2
        CNOT sweep[1] 3 sweep[1] 4
        CNOT sweep[3] 8 sweep[3] 9
        CNOT sweep[2] 8 sweep[2] 7
        X 3
        X_ERROR(1) 4
        M 0 1 2 3 4 5 6 7 8 9
    """ + "".join(f"DETECTOR rec[-{k}]\n" for k in range(9, 0, -1))
    want = ["..1.....1", "111....1.", "...1..1..", "..1..111.", "..1.1..11", "..11.....", "11.......",
            ".1.1.....", "1.1...11.", "..1....11", "11.1..1.1"]
    want = np.array([[ch == "1" for ch in row] for row in want], dtype=np.bool_)
    np.testing.assert_array_equal(gpu_convert(text, meas, sweep), want)


@pytest.mark.gpu
@pytest.mark.parametrize("reps,shots", [(50, 512), (200, 256)])
def test_gpu_big(reps, shots):
    text = BIG.format(n=reps)
    d = gpu_convert(text, measurement_rows(text, shots, 0))
    assert d.shape == (shots, 2 * reps)
    assert not d[:, 0::2].any() and d[:, 1::2].all()


@pytest.mark.gpu
def test_gpu_append_observables():
    d = gpu_convert(APPEND[0], measurement_rows(APPEND[0], 256, 0), append=True)
    assert d.shape == (256, 10) and d[:, 9].all() and not d[:, :9].any()
    d = gpu_convert(APPEND[1], measurement_rows(APPEND[1], 256, 0), append=True)
    assert d.shape == (256, 12)
    assert d[:, 0].all() and d[:, 1].all() and d[:, 11].all() and not d[:, 2:11].any()
    d = gpu_convert(APPEND[0], measurement_rows(APPEND[0], 256, 0))
    assert d.shape == (256, 0)
    d = gpu_convert(APPEND[1], measurement_rows(APPEND[1], 256, 0))
    assert d.shape == (256, 2) and d.all()


@pytest.mark.gpu
@pytest.mark.parametrize("text", ["", "X 0\nM 0"])
def test_gpu_empty_cases(text):
    c = stim_gb300.Circuit(text)
    d = gpu_convert(text, np.zeros((256, c.num_measurements), dtype=np.bool_))
    assert d.shape == (256, 0)


def convert_file(tmp_path, text, data, fmt_out, append, sweep=None, fmt_in="01"):
    src, out = tmp_path / "in", tmp_path / "out"
    src.write_bytes(data)
    kw = {}
    if sweep is not None:
        (tmp_path / "sweep").write_text(sweep)
        kw = {"sweep_bits_filepath": str(tmp_path / "sweep"), "sweep_bits_format": "01"}
    stim_gb300.Circuit(text).compile_m2d_converter().convert_file(
        measurements_filepath=str(src), measurements_format=fmt_in, detection_events_filepath=str(out),
        detection_events_format=fmt_out, append_observables=append, **kw)
    return out.read_text()


@pytest.mark.gpu
def test_gpu_file_01_to_dets_and_01(tmp_path):
    assert convert_file(tmp_path, FILE_CIRCUIT, b"0\n0\n1\n", "dets", False) == "shot D0 D2\nshot D0 D2\nshot\n"
    assert convert_file(tmp_path, FILE_CIRCUIT, b"0\n0\n1\n", "dets", True) == (
        "shot D0 D2 L9\nshot D0 D2 L9\nshot\n")
    assert convert_file(tmp_path, FILE_CIRCUIT, b"0\n0\n1\n", "01", True) == (
        "1010000000001\n1010000000001\n0000000000000\n")


@pytest.mark.gpu
def test_gpu_file_with_error_propagation(tmp_path):
    text = """
        CX sweep[0] 0
        CX sweep[1] 1
        CZ sweep[2] 0
        CZ sweep[3] 1
        H 0 1
        CZ 0 1
        M 0
        MX 1
        DETECTOR rec[-1] rec[-2]
    """
    meas = b"00\n" * 6 + b"01\n" * 2 + b"11\n" * 2
    sweep = "0000\n1000\n0100\n0010\n0001\n1111\n0000\n1111\n0000\n1111\n"
    got = convert_file(tmp_path, text, meas, "dets", True, sweep=sweep)
    assert got == ("shot\nshot\nshot D0\nshot\nshot\nshot D0\n"
                   "shot D0\nshot\n"
                   "shot\nshot D0\n")


@pytest.mark.gpu
def test_gpu_file_many_shots_and_many_detectors(tmp_path):
    text = "X 0\nM 0\nDETECTOR rec[-1]\nDETECTOR rec[-1]"
    assert convert_file(tmp_path, text, b"0\n1\n" * 500, "dets", True) == "shot D0 D1\nshot\n" * 500
    text = "REPEAT 500 {\n    M 0 1\n    DETECTOR rec[-2]\n    DETECTOR rec[-1]\n}"
    want = "shot" + "".join(f" D{2 * k + 1}" for k in range(500)) + "\n"
    assert convert_file(tmp_path, text, b"01" * 500 + b"\n", "dets", True) == want


@pytest.mark.gpu
def test_gpu_file_empty_inputs(tmp_path):
    assert convert_file(tmp_path, "", b"", "01", True) == ""
    assert convert_file(tmp_path, "", b"\n\n", "01", True) == "\n\n"
    # empty_input_b8_empty_sweep_b8: with no measurements, b8 cannot tell how many shots there are.
    with pytest.raises(ValueError, match="how many shots"):
        convert_file(tmp_path, "", b"", "01", True, fmt_in="b8")
