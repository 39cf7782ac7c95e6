"""Result-file readers (host code) against files written by the reference's own CLI (tests/golden/m2d_files/,
made by make_m2d_files.py): every format decodes to the same records as the b8 file; malformed data raises the
reference's messages."""

import glob
import os

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR

FILES_DIR = os.path.join(GOLDEN_DIR, "m2d_files")
FORMATS = ["01", "b8", "r8", "ptb64", "hits", "dets"]
OUT_FORMATS = ["01", "b8", "r8", "hits", "dets"]


def file_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(FILES_DIR, "*.npz")))


def load_files(name):
    return np.load(os.path.join(FILES_DIR, name + ".npz"))


def counts(g):
    c = stim_gb300.Circuit(str(g["circuit"]))
    return c


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("name", file_cases())
def test_reader_decodes_every_format_like_b8(name, fmt, tmp_path):
    g = load_files(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    kinds = [("meas", c.num_measurements)]
    if bool(g["has_sweep"]):
        kinds.append(("sweep", int(max(int(t[6:-1]) for t in str(g["circuit"]).split() if t.startswith("sweep[")) + 1)))
    for kind, n in kinds:
        want_path, path = tmp_path / f"{kind}.b8", tmp_path / f"{kind}.{fmt}"
        g[f"{kind}_b8"].tofile(want_path)
        g[f"{kind}_{fmt}"].tofile(path)
        want = stim_gb300.read_shot_data_file(path=want_path, format="b8", num_measurements=n, bit_packed=True)
        got = stim_gb300.read_shot_data_file(path=path, format=fmt, num_measurements=n, bit_packed=True)
        assert want.shape == (128, (n + 7) // 8)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("name", file_cases())
def test_reader_reads_detector_outputs_with_prefixes(name, tmp_path):
    g = load_files(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    D, O = c.num_detectors, c.num_observables
    g["out_b8"].tofile(tmp_path / "o.b8")
    g["out_dets"].tofile(tmp_path / "o.dets")
    want = stim_gb300.read_shot_data_file(path=tmp_path / "o.b8", format="b8", num_detectors=D, num_observables=O)
    d, o = stim_gb300.read_shot_data_file(path=tmp_path / "o.dets", format="dets", num_detectors=D,
                                          num_observables=O, separate_observables=True)
    np.testing.assert_array_equal(np.concatenate([d, o], axis=1), want)


@pytest.mark.parametrize("fmt,data,msg", [
    ("01", b"0110\n01", "01 data ended in middle of record"),
    ("01", b"0120\n", "Unexpected character in 01 format data"),
    ("01", b"01101\n", "01 data didn't end with a newline"),
    ("b8", b"\x01\x02\x03", "b8 data ended in middle of record"),
    ("hits", b"1,x\n", "HITS data wasn't comma-separated"),
    ("hits", b"9\n", "hit index is too large"),
    ("r8", b"\x09", "r8 data jumped past expected end"),
    ("r8", b"\xff", "End of file before end of r8 data"),
    ("dets", b"shot M1 X2\n", "Unrecognized DETS prefix"),
    ("dets", b"shot M9\n", "DETS data had a value larger than expected"),
    ("dets", b"shit M1\n", "DETS data didn't start with 'shot'"),
    ("dets", b"shot M1,M2\n", "DETS data wasn.t single-space-separated"),
    ("dets", b"shot M1  M2\n", "Unrecognized DETS prefix"),
    ("ptb64", b"\x00" * 20, "ptb64 data ended in middle of 64 record group"),
])
def test_reader_errors_match_reference_messages(fmt, data, msg, tmp_path):
    p = tmp_path / "bad"
    p.write_bytes(data)
    with pytest.raises(ValueError, match=msg):
        stim_gb300.read_shot_data_file(path=p, format=fmt, num_measurements=4 if fmt != "b8" else 16)


@pytest.mark.parametrize("fmt", OUT_FORMATS)
@pytest.mark.parametrize("name", file_cases())
def test_writer_reproduces_reference_files(name, fmt, tmp_path):
    # write_shot_data_file on the records of the reference's b8 output gives the reference's file in every format
    # it writes (detection events with observables appended: D then L tokens in dets).
    g = load_files(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    D, O = c.num_detectors, c.num_observables
    g["out_b8"].tofile(tmp_path / "o.b8")
    rows = stim_gb300.read_shot_data_file(path=tmp_path / "o.b8", format="b8", num_detectors=D, num_observables=O,
                                          bit_packed=True)
    stim_gb300.write_shot_data_file(data=rows, path=tmp_path / "w", format=fmt, num_detectors=D, num_observables=O)
    assert (tmp_path / "w").read_bytes() == g[f"out_{fmt}"].tobytes()
    # Bool input and measurement records round-trip through every format, ptb64 included.
    bits = stim_gb300.read_shot_data_file(path=tmp_path / "o.b8", format="b8", num_measurements=D + O)
    for f2 in FORMATS:
        stim_gb300.write_shot_data_file(data=bits, path=tmp_path / "m", format=f2, num_measurements=D + O)
        back = stim_gb300.read_shot_data_file(path=tmp_path / "m", format=f2, num_measurements=D + O)
        np.testing.assert_array_equal(back, bits)


def test_writer_argument_errors(tmp_path):
    with pytest.raises(ValueError, match="num_measurements and"):
        stim_gb300.write_shot_data_file(data=np.zeros((2, 3), bool), path=tmp_path / "x", format="01",
                                        num_measurements=1, num_detectors=2)
    with pytest.raises(ValueError, match="Must specify"):
        stim_gb300.write_shot_data_file(data=np.zeros((2, 3), bool), path=tmp_path / "x", format="01")
