"""The reference's own Python tests of the sampler surface, restated against this package
(src/stim/py/compiled_detector_sampler_pybind_test.py:23-214, compiled_measurement_sampler_pybind_test.py:21-190):
the same circuits, calls and expected arrays / files / errors, so a caller switching packages sees the same
behaviour.  (test_manual_output_buffer is in test_gpu_parity.py.)"""

import pathlib

import numpy as np
import pytest

import stim_gb300

pytestmark = pytest.mark.gpu

SAMPLE = """
    X_ERROR(1) 0
    M 0 1 2
    DETECTOR rec[-3] rec[-2]
    DETECTOR rec[-3] rec[-1]
    DETECTOR rec[-1] rec[-2]
    OBSERVABLE_INCLUDE(0) rec[-3]
    OBSERVABLE_INCLUDE(3) rec[-2] rec[-1]
    OBSERVABLE_INCLUDE(0) rec[-2]
"""


def rows(row, n=5, dtype=np.bool_):
    return np.array([row] * n, dtype=dtype)


def test_detector_sampler_trivial():
    c = stim_gb300.Circuit("X_ERROR(1) 0\nM 0\nDETECTOR rec[-1]")
    np.testing.assert_array_equal(c.compile_detector_sampler().sample(shots=2), rows([1], 2))


def test_detector_sampler_layouts():
    c = stim_gb300.Circuit(SAMPLE)
    s = c.compile_detector_sampler
    np.testing.assert_array_equal(s().sample(5), rows([1, 1, 0]))
    np.testing.assert_array_equal(s().sample(5, prepend_observables=True), rows([1, 0, 0, 0, 1, 1, 0]))
    np.testing.assert_array_equal(s().sample(5, append_observables=True), rows([1, 1, 0, 1, 0, 0, 0]))
    dets, obs = s().sample(5, separate_observables=True)
    np.testing.assert_array_equal(dets, rows([1, 1, 0]))
    np.testing.assert_array_equal(obs, rows([1, 0, 0, 0]))
    dets, obs = s().sample(5, separate_observables=True, bit_packed=True)
    np.testing.assert_array_equal(dets, rows([3], dtype=np.uint8))
    np.testing.assert_array_equal(obs, rows([1], dtype=np.uint8))
    np.testing.assert_array_equal(s().sample(5, append_observables=True, prepend_observables=True),
                                  rows([1, 0, 0, 0, 1, 1, 0, 1, 0, 0, 0]))
    np.testing.assert_array_equal(s().sample_bit_packed(5), rows([0b011], dtype=np.uint8))
    np.testing.assert_array_equal(s().sample(5, bit_packed=True), rows([0b011], dtype=np.uint8))


def test_detector_sampler_write(tmp_path):
    c = stim_gb300.Circuit(SAMPLE)
    path = tmp_path / "tmp.dat"
    c.compile_detector_sampler().sample_write(5, filepath=str(path), format="b8")
    assert path.read_bytes() == b"\x03" * 5
    c.compile_detector_sampler().sample_write(5, filepath=pathlib.Path(path), format="b8")
    assert path.read_bytes() == b"\x03" * 5
    c.compile_detector_sampler().sample_write(5, filepath=str(path), format="01", prepend_observables=True)
    assert path.read_text().splitlines(keepends=True) == ["1000110\n"] * 5
    c.compile_detector_sampler().sample_write(5, filepath=str(path), format="01", append_observables=True)
    assert path.read_text().splitlines(keepends=True) == ["1101000\n"] * 5


@pytest.mark.parametrize("as_path", [False, True])
def test_write_obs_file(tmp_path, as_path):
    c = stim_gb300.Circuit("""
        X_ERROR(1) 1
        MR 0 1
        DETECTOR rec[-2]
        DETECTOR rec[-2]
        DETECTOR rec[-2]
        DETECTOR rec[-1]
        DETECTOR rec[-2]
        DETECTOR rec[-2]
        OBSERVABLE_INCLUDE(1) rec[-1]
        OBSERVABLE_INCLUDE(2) rec[-2]
    """)
    det, obs = tmp_path / "det", tmp_path / "obs"
    c.compile_detector_sampler().sample_write(shots=100, filepath=det if as_path else str(det), format="dets",
                                              obs_out_filepath=obs if as_path else str(obs), obs_out_format="hits")
    assert det.read_text() == "shot D3\n" * 100
    assert obs.read_text() == "1\n" * 100


def test_samplers_actually_fill_arrays():
    c = stim_gb300.Circuit("X_ERROR(1) 0\nM 0\nDETECTOR rec[-1]")
    assert np.all(c.compile_detector_sampler().sample(shots=10000))
    assert np.all(c.compile_sampler().sample(shots=10000))


def test_measurement_sampler_sample():
    c = stim_gb300.Circuit("X 0 1 2 3 4 5 6 7     10\nM 0 1 2 3 4 5 6 7 8 9 10")
    np.testing.assert_array_equal(c.compile_sampler().sample_bit_packed(shots=1), [[255, 4]])
    np.testing.assert_array_equal(c.compile_sampler().sample(shots=1, bit_packed=True), [[255, 4]])


@pytest.mark.parametrize("text", [
    "RX 0\nRY 1\nRZ 2\nH 0\nH_YZ 1\nM 0 1 2",
    "H 0\nH_YZ 1\nMRX 0\nMRY 1\nMRZ 2\nH 0\nH_YZ 1\nM 0 1 2",
    "H 0\nH_YZ 1\nMRX 0\nMRY 1\nMRZ 2",
])
def test_measurements_vs_resets(text):
    assert not np.any(stim_gb300.Circuit(text).compile_sampler().sample(shots=100))


def test_measurement_sample_write(tmp_path):
    c = stim_gb300.Circuit("X 0 4 5\nM 0 1 2 3 4 5 6")
    path = tmp_path / "tmp.dat"
    c.compile_sampler().sample_write(5, filepath=str(path), format="b8")
    assert path.read_bytes() == b"\x31" * 5
    c.compile_sampler().sample_write(5, filepath=str(path), format="01")
    assert path.read_text().splitlines(keepends=True) == ["1000110\n"] * 5


def test_skip_reference_sample():
    x, xe = stim_gb300.Circuit("X 0\nM 0"), stim_gb300.Circuit("X_ERROR(1) 0\nM 0")
    np.testing.assert_array_equal(x.compile_sampler().sample(1), [[True]])
    np.testing.assert_array_equal(x.compile_sampler(skip_reference_sample=False).sample(1), [[True]])
    np.testing.assert_array_equal(x.compile_sampler(skip_reference_sample=True).sample(1), [[False]])
    np.testing.assert_array_equal(xe.compile_sampler(skip_reference_sample=False).sample(1), [[True]])
    np.testing.assert_array_equal(xe.compile_sampler(skip_reference_sample=True).sample(1), [[True]])


def test_reference_sample_init():
    x = stim_gb300.Circuit("X 0\nM 0")
    np.testing.assert_array_equal(x.compile_sampler(reference_sample=None).sample(1), [[True]])
    np.testing.assert_array_equal(x.compile_sampler(reference_sample=np.array([False])).sample(1), [[False]])
    np.testing.assert_array_equal(x.compile_sampler(reference_sample=x.reference_sample()).sample(1), [[True]])
    xe = stim_gb300.Circuit("X_ERROR(1) 0\n M 0")
    np.testing.assert_array_equal(xe.compile_sampler(reference_sample=np.array([False])).sample(1), [[True]])
    ref = xe.reference_sample()
    np.testing.assert_array_equal(xe.compile_sampler(reference_sample=ref).sample(1), [[True]])
    with pytest.raises(ValueError):
        xe.compile_sampler(reference_sample=ref, skip_reference_sample=True)
    for text, shots in [("H 0\n X 1\n CNOT 0 1\n H 0 1\n MPP X0*X1", 10),
                        ("H 0\n X 1\n CNOT 0 1\n H 0 1 2\n MPP Y1*Y2 X1*X2 Z1*Z2", 11)]:
        c = stim_gb300.Circuit(text)
        np.testing.assert_array_equal(c.compile_sampler(reference_sample=c.reference_sample(), seed=0).sample(shots),
                                      c.compile_sampler(seed=0).sample(shots))


def test_repr():
    c = stim_gb300.Circuit("""
        X 0
        M 0
    """)
    want = "stim_gb300.Circuit('''\n    X 0\n    M 0\n''')"
    assert repr(c.compile_sampler()) == f"stim_gb300.CompiledMeasurementSampler({want})"
    assert repr(c.compile_sampler(skip_reference_sample=True)) == (
        f"stim_gb300.CompiledMeasurementSampler({want}, skip_reference_sample=True)")
    assert repr(c.compile_detector_sampler()) == f"stim_gb300.CompiledDetectorSampler({want})"


# From src/stim/circuit/circuit_pybind_test.py:216-260, 520-570, 2079-2090.
def test_compiled_sampler_reprs_evaluate():
    empty = stim_gb300.Circuit()
    assert repr(empty.compile_sampler()) == "stim_gb300.CompiledMeasurementSampler(stim_gb300.Circuit())"
    assert repr(empty.compile_detector_sampler()) == "stim_gb300.CompiledDetectorSampler(stim_gb300.Circuit())"
    c = stim_gb300.Circuit("M 0\nH 0 1 2 3 4\nM 0 1 2 3 4")
    r = repr(c.compile_sampler())
    assert r == ("stim_gb300.CompiledMeasurementSampler(stim_gb300.Circuit('''\n    M 0\n    H 0 1 2 3 4\n"
                 "    M 0 1 2 3 4\n'''))")
    assert repr(eval(r, {"stim_gb300": stim_gb300})) == r
    d = stim_gb300.Circuit("M 0\nDETECTOR rec[-1]")
    r = repr(d.compile_detector_sampler())
    assert repr(eval(r, {"stim_gb300": stim_gb300})) == r


@pytest.mark.parametrize("compile_name,text", [
    ("compile_sampler", "H 0\nM 0"),
    ("compile_detector_sampler", "X_ERROR(0.5) 0\nM 0\nDETECTOR rec[-1]"),
])
def test_sampling_seeded(compile_name, text):
    c = stim_gb300.Circuit(text)
    compile_ = getattr(c, compile_name)
    with pytest.raises(ValueError, match="seed"):
        compile_(seed=-1)
    with pytest.raises(ValueError, match="seed"):
        compile_(seed=object())
    assert not np.array_equal(compile_().sample(256), compile_().sample(256))
    assert not np.array_equal(compile_(seed=None).sample(256), compile_(seed=None).sample(256))
    s1, s2, s3 = compile_(seed=5).sample(256), compile_(seed=5).sample(256), compile_(seed=6).sample(256)
    assert np.array_equal(s1, s2)
    assert not np.array_equal(s1, s3)


def test_tagged_instructions_sample():
    c = stim_gb300.Circuit("R[test1] 0\nX_ERROR[test2](0.25) 0\nM[test3](0.25) 0\nDETECTOR[test4](1, 2) rec[-1]")
    assert 200 < np.sum(c.compile_detector_sampler().sample(shots=1000)) < 600
    assert 200 < np.sum(c.compile_sampler().sample(shots=1000)) < 600
    c.compile_m2d_converter()
