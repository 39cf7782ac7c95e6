"""The reference's result-reader tests, restated against this package's read_shot_data_file (host code, no GPU;
src/stim/io/measure_record_reader.test.cc:60-136 Format01 / FormatB8 / FormatHits / FormatR8 / FormatR8_LongGap,
:327-457 multiple records, short and huge dets records, D and L prefixes, invalid input, repeated hits,
:769-830 Windows newlines): each file and the bits the reference reads from it."""

import numpy as np
import pytest

import stim_gb300

F8 = [3, 4, 5, 6, 7, 12, 13, 14, 15, 16, 17]


def read(tmp_path, data, fmt, **counts):
    path = tmp_path / "data"
    path.write_bytes(data)
    return stim_gb300.read_shot_data_file(path=str(path), format=fmt, **counts).astype(np.uint8)


def rows(n, *sets):
    a = np.zeros((len(sets), n), dtype=np.uint8)
    for k, s in enumerate(sets):
        a[k, list(s)] = 1
    return a


@pytest.mark.parametrize("fmt,data", [
    ("01", b"000111110000111111\n"), ("b8", b"\xf8\xf0\x03"), ("hits", b"3,4,5,6,7,12,13,14,15,16,17\n"),
    ("r8", bytes([3, 0, 0, 0, 0, 4, 0, 0, 0, 0, 0, 0])),
])
def test_one_record_in_each_format(tmp_path, fmt, data):
    np.testing.assert_array_equal(read(tmp_path, data, fmt, num_measurements=18), rows(18, F8))


def test_r8_long_gap(tmp_path):
    np.testing.assert_array_equal(read(tmp_path, b"\xff\xff\x02\x20", "r8", num_measurements=8 * 64 + 32 + 1),
                                  rows(545, [512]))


def test_multiple_and_short_records(tmp_path):
    assert read(tmp_path, b"111011001\n010000000\n101100011\n", "01", num_measurements=9).shape == (3, 9)
    np.testing.assert_array_equal(read(tmp_path, b"shot M0\nshot M1\nshot M0\nshot\n", "dets", num_measurements=2),
                                  rows(2, [0], [1], [0], []))


def test_dets_prefixes_and_huge_observables(tmp_path):
    got = read(tmp_path, b"shot L1000\nshot D2 L999\n", "dets", num_detectors=10, num_observables=1500)
    np.testing.assert_array_equal(got, rows(1510, [1010], [2, 1009]))
    got = read(tmp_path, b"shot D0 D3 D5 L1 L2\n", "dets", num_detectors=7, num_observables=4)
    np.testing.assert_array_equal(got, rows(11, [0, 3, 5, 8, 9]))


@pytest.mark.parametrize("fmt,data", [("01", b"012\n"), ("hits", b"100,1\n"), ("dets", b"D2\n")])
def test_invalid_input(tmp_path, fmt, data):
    with pytest.raises(ValueError):
        read(tmp_path, data, fmt, num_measurements=3)


def test_repeated_hits_cancel(tmp_path):
    np.testing.assert_array_equal(read(tmp_path, b"1,1\n", "hits", num_measurements=3), rows(3, []))


@pytest.mark.parametrize("fmt,data", [
    ("01", b"01\r\n01\r\n"), ("hits", b"1\r\n1\r\n"), ("dets", b"shot M1\r\n\r\n\n   shot M1\r\n\n"),
])
def test_windows_newlines(tmp_path, fmt, data):
    np.testing.assert_array_equal(read(tmp_path, data, fmt, num_measurements=2), rows(2, [1], [1]))


def test_windows_newlines_four_bits(tmp_path):
    np.testing.assert_array_equal(read(tmp_path, b"3\r\n1\r\n", "hits", num_measurements=4), rows(4, [3], [1]))
    np.testing.assert_array_equal(read(tmp_path, b"shot M3\r\n\r\n\n   shot M1\r\n\n", "dets", num_measurements=4),
                                  rows(4, [3], [1]))
