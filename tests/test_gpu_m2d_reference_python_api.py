"""The reference's own Python tests of the measurements-to-detection-events converter
(src/stim/simulators/measurements_to_detection_events_test.py:22-300), restated against this package: files with and
without sweep bits, arrays bool and bit-packed (and the legacy bit_pack_result), swept, separate observables,
noiseless conversion, the explicit-observables error, and anticommuting observable pieces."""

import numpy as np
import pytest

import stim_gb300

pytestmark = pytest.mark.gpu

SWEPT = """
    X_ERROR(0.1) 0
    X 0
    CNOT sweep[0] 0
    M 0
    DETECTOR rec[-1]
    OBSERVABLE_INCLUDE(0) rec[-1]
"""
REP = "REPEAT 100 {\n X_ERROR(0.1) 0\n X 0\n MR 0\n DETECTOR rec[-1]\n}\n"


def pack(a):
    return np.packbits(np.asarray(a, dtype=np.bool_), axis=1, bitorder="little")


def test_convert_file_without_and_with_sweep_bits(tmp_path):
    conv = stim_gb300.Circuit(SWEPT).compile_m2d_converter()
    (tmp_path / "m.01").write_text("0\n1\n")
    conv.convert_file(measurements_filepath=str(tmp_path / "m.01"),
                      detection_events_filepath=str(tmp_path / "d.01"), append_observables=False)
    assert (tmp_path / "d.01").read_text() == "1\n0\n"
    (tmp_path / "m.b8").write_bytes(bytes([0, 1, 0, 1]))
    (tmp_path / "s.hits").write_text("\n\n0\n0\n")
    conv.convert_file(measurements_filepath=str(tmp_path / "m.b8"), measurements_format="b8",
                      sweep_bits_filepath=str(tmp_path / "s.hits"), sweep_bits_format="hits",
                      detection_events_filepath=str(tmp_path / "d.dets"), detection_events_format="dets",
                      append_observables=True)
    assert (tmp_path / "d.dets").read_text() == "shot D0 L0\nshot\nshot\nshot D0 L0\n"
    conv.convert_file(measurements_filepath=str(tmp_path / "m.b8"), measurements_format="b8",
                      sweep_bits_filepath=str(tmp_path / "s.hits"), sweep_bits_format="hits",
                      detection_events_filepath=str(tmp_path / "d.dets"), detection_events_format="dets",
                      obs_out_filepath=str(tmp_path / "o.hits"), obs_out_format="hits")
    assert (tmp_path / "d.dets").read_text() == "shot D0\nshot\nshot\nshot D0\n"
    assert (tmp_path / "o.hits").read_text() == "0\n\n\n0\n"


def test_convert():
    conv = stim_gb300.Circuit(SWEPT).compile_m2d_converter()
    r = conv.convert(measurements=np.array([[0], [1]], dtype=np.bool_), append_observables=False)
    assert r.dtype == np.bool_ and r.shape == (2, 1)
    np.testing.assert_array_equal(r, [[1], [0]])
    r = conv.convert(measurements=np.array([[0], [1]], dtype=np.bool_), append_observables=True)
    assert r.shape == (2, 2)
    np.testing.assert_array_equal(r, [[1, 1], [0, 0]])
    r = conv.convert(measurements=np.array([[0], [1], [0], [1]], dtype=np.bool_),
                     sweep_bits=np.array([[0], [0], [1], [1]], dtype=np.bool_), append_observables=True)
    np.testing.assert_array_equal(r, [[1, 1], [0, 0], [0, 0], [1, 1]])


def test_convert_bit_packed():
    conv = stim_gb300.Circuit(REP).compile_m2d_converter()
    meas = np.array([[0] * 100, [1] * 100], dtype=np.bool_)
    want = np.array([[1] * 100, [0] * 100], dtype=np.bool_)
    for m in (meas, pack(meas)):
        r = conv.convert(measurements=m, append_observables=False)
        assert r.dtype == np.bool_ and r.shape == (2, 100)
        np.testing.assert_array_equal(r, want)
        for kw in ({"bit_pack_result": True}, {"bit_packed": True}):
            r = conv.convert(measurements=m, append_observables=False, **kw)
            assert r.dtype == np.uint8 and r.shape == (2, 13)
            np.testing.assert_array_equal(r, pack(want))


def test_convert_bit_packed_swept():
    conv = stim_gb300.Circuit("REPEAT 100 {\n CNOT sweep[0] 0\n X_ERROR(0.1) 0\n X 0\n MR 0\n DETECTOR rec[-1]\n}\n"
                              ).compile_m2d_converter()
    meas = np.array([[0] * 100, [1] * 100], dtype=np.bool_)
    sweeps = np.array([[1], [0]], dtype=np.bool_)
    want = np.zeros((2, 100), dtype=np.bool_)
    for m in (meas, pack(meas)):
        for s in (sweeps, pack(sweeps)):
            np.testing.assert_array_equal(conv.convert(measurements=m, sweep_bits=s, append_observables=False), want)
            np.testing.assert_array_equal(
                conv.convert(measurements=m, sweep_bits=s, append_observables=False, bit_pack_result=True), pack(want))


def test_convert_bit_packed_separate_observables():
    conv = stim_gb300.Circuit(REP + "OBSERVABLE_INCLUDE(0) rec[-1]\nOBSERVABLE_INCLUDE(6) rec[-2]\n"
                                    "OBSERVABLE_INCLUDE(14) rec[-3]\n").compile_m2d_converter()
    meas = np.array([[0] * 100, [1] * 100], dtype=np.bool_)
    want_d = np.array([[1] * 100, [0] * 100], dtype=np.bool_)
    want_o = np.array([[1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1], [0] * 15], dtype=np.bool_)
    for m in (meas, pack(meas)):
        d, o = conv.convert(measurements=m, separate_observables=True)
        assert d.dtype == o.dtype == np.bool_ and d.shape == (2, 100) and o.shape == (2, 15)
        np.testing.assert_array_equal(d, want_d)
        np.testing.assert_array_equal(o, want_o)
        d, o = conv.convert(measurements=m, separate_observables=True, bit_pack_result=True)
        assert d.dtype == o.dtype == np.uint8 and d.shape == (2, 13) and o.shape == (2, 2)
        np.testing.assert_array_equal(d, pack(want_d))
        np.testing.assert_array_equal(o, pack(want_o))


def test_noiseless_conversion():
    conv = stim_gb300.Circuit("MR 0\nDETECTOR rec[-1]\nX 0\nMR 0\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(0) rec[-1]"
                              ).compile_m2d_converter()
    meas = np.array([[0, 0], [0, 1], [1, 0], [1, 1]], dtype=np.bool_)
    d, o = conv.convert(measurements=meas, separate_observables=True)
    np.testing.assert_array_equal(d, [[0, 1], [0, 0], [1, 1], [1, 0]])
    np.testing.assert_array_equal(o, [[1], [0], [1], [0]])


def test_needs_append_or_separate():
    conv = stim_gb300.Circuit("").compile_m2d_converter()
    ms = np.zeros((50, 0), dtype=np.bool_)
    with pytest.raises(ValueError, match="explicitly specify either separate"):
        conv.convert(measurements=ms)
    d1 = conv.convert(measurements=ms, append_observables=True)
    d2, d3 = conv.convert(measurements=ms, separate_observables=True)
    d4, d5 = conv.convert(measurements=ms, separate_observables=True, append_observables=True)
    for x in (d2, d3, d4, d5):
        np.testing.assert_array_equal(d1, x)


def test_anticommuting_pieces_combining_into_deterministic_observable():
    c = stim_gb300.Circuit("MX 0\nOBSERVABLE_INCLUDE(0) rec[-1]\nMX 0\nOBSERVABLE_INCLUDE(0) rec[-1]")
    m = c.compile_sampler().sample_bit_packed(shots=1000)
    _, obs = c.compile_m2d_converter().convert(measurements=m, separate_observables=True)
    assert not obs.any()
