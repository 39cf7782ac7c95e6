"""The reference's result-writer tests, restated against this package (src/stim/io/measure_record_writer.test.cc:
26-165 Format01 / FormatB8 / FormatHits / FormatDets / FormatDets_EmptyRecords / FormatDets_MultipleRecords /
FormatR8 / FormatR8_LongGap, :167-212 write_table_data_small, :390-443 write_bits_{01,b8,r8}_{a,b}).

Each case is a record of bits and the exact bytes the reference writes for it.  On the CPU the records go through
write_shot_data_file (the host writer); on the GPU a circuit whose measurements (or detectors and observables) come
out as that record in every shot goes through sample_write, so the device format kernels are held to the same
bytes."""

import numpy as np
import pytest

import stim_gb300

# (name, record bits set, record length, {format: expected bytes of one shot})
RECORDS = [
    # Format01 / FormatB8 / FormatHits / FormatR8: bytes 0xF8, bit 0, bytes 0xF8, bit 1.
    ("f8_0_f8_1", [3, 4, 5, 6, 7, 12, 13, 14, 15, 16, 17], 18, {
        "01": b"000111110000111111\n",
        "b8": bytes([0xF8, 0xF0, 0x03]),
        "hits": b"3,4,5,6,7,12,13,14,15,16,17\n",
        "r8": bytes([3, 0, 0, 0, 0, 4, 0, 0, 0, 0, 0, 0]),
    }),
    # FormatR8_LongGap: 512 zeros, a one, 32 zeros.
    ("long_gap", [512], 545, {"r8": bytes([255, 255, 2, 32])}),
    # write_bits_*_a: bits of bytes 0x00, 0xFF, first 11.
    ("bits_a", [8, 9, 10], 11, {"01": b"00000000111\n", "b8": bytes([0x00, 0x07]), "r8": bytes([8, 0, 0, 0])}),
    # write_bits_*_b: bits of bytes 0xFF, 0x00, first 11.
    ("bits_b", list(range(8)), 11, {"01": b"11111111000\n", "b8": bytes([0xFF, 0x00]),
                                    "r8": bytes([0] * 8 + [3])}),
    # write_table_data_small: four measurements, the second one set.
    ("table_small", [1], 4, {"01": b"0100\n", "hits": b"1\n", "dets": b"shot M1\n", "r8": bytes([1, 2]),
                             "b8": bytes([2])}),
    # FormatDets_EmptyRecords: nothing set.
    ("empty", [], 1, {"dets": b"shot\n", "hits": b"\n"}),
]
CASES = [(name, bits, n, fmt, want) for name, bits, n, fmts in RECORDS for fmt, want in fmts.items()]
IDS = [f"{c[0]}-{c[3]}" for c in CASES]


def record_rows(bits, n, shots):
    a = np.zeros((shots, n), dtype=np.bool_)
    a[:, bits] = True
    return a


@pytest.mark.parametrize("name,bits,n,fmt,want", CASES, ids=IDS)
def test_host_writer(tmp_path, name, bits, n, fmt, want):
    path = tmp_path / "out"
    stim_gb300.write_shot_data_file(data=record_rows(bits, n, 3), path=str(path), format=fmt, num_measurements=n)
    assert path.read_bytes() == want * 3


def test_host_writer_dets_detectors_and_observables(tmp_path):
    # FormatDets: D bits 0xF8, 0, 0xF8 (17 detectors), then L bits 0, 1.
    path = tmp_path / "out"
    rows = record_rows([3, 4, 5, 6, 7, 12, 13, 14, 15, 16, 18], 19, 2)
    stim_gb300.write_shot_data_file(data=rows, path=str(path), format="dets", num_detectors=17, num_observables=2)
    assert path.read_text() == "shot D3 D4 D5 D6 D7 D12 D13 D14 D15 D16 L1\n" * 2


def test_host_writer_dets_multiple_records(tmp_path):
    # FormatDets_MultipleRecords: two shots of three / four detectors and two / three observables, written as
    # rows of four detectors and three observables.
    path = tmp_path / "out"
    rows = np.array([[0, 0, 1, 0, 0, 1, 0], [1, 0, 0, 1, 1, 0, 1]], dtype=np.bool_)
    stim_gb300.write_shot_data_file(data=rows, path=str(path), format="dets", num_detectors=4, num_observables=3)
    assert path.read_text() == "shot D2 L1\nshot D0 D3 L0 L2\n"


def test_host_writer_table_small_observable_and_ptb64(tmp_path):
    # write_table_data_small: with one detector before the observables, the set bit is L0; ptb64 over 64 shots
    # with the bit set in shots 0-4 only.
    path = tmp_path / "out"
    rows = record_rows([1], 4, 5)
    stim_gb300.write_shot_data_file(data=rows, path=str(path), format="dets", num_detectors=1, num_observables=3)
    assert path.read_text() == "shot L0\n" * 5
    rows = np.zeros((64, 4), dtype=np.bool_)
    rows[:5, 1] = True
    stim_gb300.write_shot_data_file(data=rows, path=str(path), format="ptb64", num_measurements=4)
    assert path.read_bytes() == b"\x00" * 8 + b"\x1f" + b"\x00" * 7 + b"\x00" * 16


def record_circuit(bits, n, flip_gate="X"):
    """Measurements 0..n-1 of qubits 0..n-1, the qubits in `bits` flipped first: every shot records `bits`.  With
    X the flips are part of the reference sample (measurement results); with X_ERROR(1) they are errors against it
    (detection events)."""
    flip = (f"{flip_gate} " + " ".join(map(str, bits)) + "\n") if bits else ""
    return flip + "M " + " ".join(map(str, range(n)))


@pytest.mark.gpu
@pytest.mark.parametrize("name,bits,n,fmt,want", CASES, ids=IDS)
def test_gpu_writer(tmp_path, name, bits, n, fmt, want):
    path = tmp_path / "out"
    stim_gb300.Circuit(record_circuit(bits, n)).compile_sampler().sample_write(5, filepath=str(path), format=fmt)
    assert path.read_bytes() == want * 5


@pytest.mark.gpu
def test_gpu_writer_dets_detectors_and_observables(tmp_path):
    # FormatDets through the detection sampler: 17 detectors (0xF8, 0, 0xF8) and observables (0, 1) appended.
    text = (record_circuit([3, 4, 5, 6, 7, 12, 13, 14, 15, 16, 18], 19, "X_ERROR(1)") + "\n" +
            "".join(f"DETECTOR rec[-{19 - k}]\n" for k in range(17)) +
            "OBSERVABLE_INCLUDE(0) rec[-2]\nOBSERVABLE_INCLUDE(1) rec[-1]")
    path = tmp_path / "out"
    stim_gb300.Circuit(text).compile_detector_sampler().sample_write(3, filepath=str(path), format="dets",
                                                                      append_observables=True)
    assert path.read_text() == "shot D3 D4 D5 D6 D7 D12 D13 D14 D15 D16 L1\n" * 3


# FormatDets_EmptyRecords in every format: records of no bits (a circuit without measurements, a detection sampler
# without detectors or observables).
EMPTY_RECORD = {"01": b"\n", "b8": b"", "r8": b"\x00", "hits": b"\n", "dets": b"shot\n", "ptb64": b""}


@pytest.mark.parametrize("fmt", sorted(EMPTY_RECORD))
def test_host_writer_empty_records(tmp_path, fmt):
    path = tmp_path / "out"
    stim_gb300.write_shot_data_file(data=np.zeros((64, 0), dtype=np.bool_), path=str(path), format=fmt,
                                    num_measurements=0)
    assert path.read_bytes() == EMPTY_RECORD[fmt] * 64


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", sorted(EMPTY_RECORD))
def test_gpu_writer_empty_records(tmp_path, fmt):
    path = tmp_path / "out"
    stim_gb300.Circuit("H 0").compile_sampler().sample_write(64, filepath=str(path), format=fmt)
    assert path.read_bytes() == EMPTY_RECORD[fmt] * 64
    stim_gb300.Circuit("M 0").compile_detector_sampler().sample_write(128, filepath=str(path), format=fmt)
    assert path.read_bytes() == EMPTY_RECORD[fmt] * 128
