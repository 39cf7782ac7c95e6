"""The reference's own Python tests of result-file reading and writing (src/stim/io/read_write_pytest.py:24-312),
restated against this package's read_shot_data_file / write_shot_data_file (host code, no GPU): exact contents,
the errors the reference raises (message fragments), the legacy bit_pack argument, and round trips in every
format with str and pathlib paths."""

import itertools
import pathlib

import numpy as np
import pytest

import stim_gb300


def test_read_shot_data_file_01(tmp_path):
    path = str(tmp_path / "file.01")
    pathlib.Path(path).write_text("0001110011\n0000000000\n")
    with pytest.raises(ValueError, match="expected data length"):
        stim_gb300.read_shot_data_file(path=path, format="01", num_measurements=9)
    with pytest.raises(ValueError, match="ended in middle"):
        stim_gb300.read_shot_data_file(path=path, format="01", num_measurements=11)
    r = stim_gb300.read_shot_data_file(path=path, format="01", num_measurements=10)
    assert r.dtype == np.bool_ and r.shape == (2, 10)
    np.testing.assert_array_equal(r, [[0, 0, 0, 1, 1, 1, 0, 0, 1, 1], [0] * 10])
    r = stim_gb300.read_shot_data_file(path=path, format="01", num_measurements=10, bit_pack=True)
    assert r.dtype == np.uint8 and r.shape == (2, 2)
    np.testing.assert_array_equal(r, [[0x38, 0x03], [0x00, 0x00]])


def test_read_shot_data_file_dets(tmp_path):
    path = str(tmp_path / "file.dets")
    pathlib.Path(path).write_text("shot\nshot D0 D5 L0\n")
    with pytest.raises(ValueError, match="D0"):
        stim_gb300.read_shot_data_file(path=path, format="dets", num_measurements=9)
    with pytest.raises(ValueError, match="D5"):
        stim_gb300.read_shot_data_file(path=path, format="dets", num_measurements=0, num_detectors=5,
                                       num_observables=2)
    r = stim_gb300.read_shot_data_file(path=path, format="dets", num_measurements=0, num_detectors=10,
                                       num_observables=2)
    assert r.dtype == np.bool_ and r.shape == (2, 12)
    np.testing.assert_array_equal(r, [[0] * 12, [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]])
    d, o = stim_gb300.read_shot_data_file(path=path, format="dets", num_measurements=0, num_detectors=10,
                                          num_observables=2, separate_observables=True)
    assert d.shape == (2, 10) and o.shape == (2, 2) and d.dtype == o.dtype == np.bool_
    np.testing.assert_array_equal(d, [[0] * 10, [1, 0, 0, 0, 0, 1, 0, 0, 0, 0]])
    np.testing.assert_array_equal(o, [[0, 0], [1, 0]])
    d, o = stim_gb300.read_shot_data_file(path=path, format="dets", num_measurements=0, num_detectors=10,
                                          num_observables=2, separate_observables=True, bit_packed=True)
    assert d.dtype == o.dtype == np.uint8 and d.shape == (2, 2) and o.shape == (2, 1)
    np.testing.assert_array_equal(d, [[0, 0], [0b00100001, 0]])
    np.testing.assert_array_equal(o, [[0], [1]])


def test_write_shot_data_file_01(tmp_path):
    path = str(tmp_path / "file.01")
    data = np.array([[0, 1, 0], [0, 1, 1]])
    with pytest.raises(ValueError, match="4 bits per shot.+bool_"):
        stim_gb300.write_shot_data_file(data=data.astype(np.bool_), path=path, format="01", num_measurements=4)
    with pytest.raises(ValueError, match="4 bits per shot.+uint8"):
        stim_gb300.write_shot_data_file(data=data.astype(np.uint8), path=path, format="01", num_measurements=4)
    with pytest.raises(ValueError, match="num_measurements and"):
        stim_gb300.write_shot_data_file(data=data.astype(np.bool_), path=path, format="01", num_measurements=1,
                                        num_detectors=2)
    stim_gb300.write_shot_data_file(data=data.astype(np.bool_), path=path, format="01", num_measurements=3)
    assert pathlib.Path(path).read_text() == "010\n011\n"
    stim_gb300.write_shot_data_file(data=np.array([[0x38, 0x03], [0x00, 0x00]], dtype=np.uint8), path=path,
                                    format="01", num_measurements=13)
    assert pathlib.Path(path).read_text() == "0001110011000\n0000000000000\n"


def test_read_data_file_partial_and_big_b8(tmp_path):
    path = tmp_path / "tmp.b8"
    path.write_bytes(b"\0" * 273)
    with pytest.raises(ValueError, match="middle of record"):
        stim_gb300.read_shot_data_file(path=str(path), format="b8", num_detectors=2185, num_observables=0)
    path.write_bytes(b"\0" * 274000)
    assert stim_gb300.read_shot_data_file(path=str(path), format="b8", num_detectors=2185,
                                          num_observables=0).shape == (1000, 2185)


def test_read_01_shots(tmp_path):
    path = tmp_path / "shots"
    path.write_text("0000\n0101\n")
    np.testing.assert_array_equal(stim_gb300.read_shot_data_file(path=str(path), format="01", num_measurements=4),
                                  [[0, 0, 0, 0], [0, 1, 0, 1]])


@pytest.mark.parametrize("fmt,bit_packed,path_type", list(itertools.product(
    ["01", "b8", "r8", "ptb64", "hits", "dets"], [False, True], ["str", "path"])))
def test_read_write_round_trips(tmp_path, fmt, bit_packed, path_type):
    data = np.random.default_rng(1).integers(2, size=(320, 500)).astype(np.bool_)
    arg = data if not bit_packed else np.packbits(data, axis=1, bitorder="little")
    path = tmp_path / "shots" if path_type == "path" else str(tmp_path / "shots")
    stim_gb300.write_shot_data_file(data=arg, path=path, format=fmt, num_measurements=500)
    back = stim_gb300.read_shot_data_file(path=path, format=fmt, num_measurements=500, bit_pack=bit_packed)
    np.testing.assert_array_equal(arg, back)
