"""The reference's command-line tests of `stim detect`, `stim sample`, `stim m2d` and `stim sample_dem`, restated
against this package (src/stim/cmd/command_detect.test.cc:21-233, command_sample.test.cc:73-420,
command_m2d.test.cc:22-176, command_sample_dem.test.cc:22-51): the CLI's output is what sample_write / convert_file
write, and `--prepend_observables` / `--append_observables` / `--skip_reference_sample` / `--obs_out` are the
arguments of the same meaning.  (`m2d --ran_without_feedback` has no counterpart in the reference's Python
converter, which this package mirrors, and is left out.)

Exact outputs for deterministic circuits; for random ones the reference's `deviation` check
(command_sample.test.cc:37-71): every sampled line must be an expected one, and each expected line's rate must lie
within 5 standard deviations of its probability.  The oracle on the CPU (its measurement flips XOR the host reference
sample), the GPU samplers on the GB300."""

import math
from collections import Counter

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

# command_detect.test.cc:21-183: (circuit, prepend, append, detection-event line of every shot).
LOOP = """
M 2
M 2
{flip}REPEAT 3 {{
  R 2
  CNOT 0 2 1 2
  DETECTOR rec[-1] rec[-2]
  M 2
}}
M 0 1
OBSERVABLE_INCLUDE(0) {obs}
"""
DETECT = [
    ("M 0", False, False, ""),
    ("M 0\nDETECTOR rec[-1]", False, False, "0"),
    ("X_ERROR(1) 0\nM 0\nDETECTOR rec[-1]", False, False, "1"),
    ("DETECTOR", False, False, "0"),
    ("X_ERROR(1) 0\nMR 0\nDETECTOR rec[-1]", False, False, "1"),
    ("X_ERROR(1) 0\nM 0\nM 0\nDETECTOR rec[-1] rec[-2]", False, False, "0"),
    ("X_ERROR(1) 0\nMR 0\nMR 0\nDETECTOR rec[-1] rec[-2]", False, False, "1"),
    (LOOP.format(flip="", obs="rec[-2] rec[-1]"), False, False, "000"),
    (LOOP.format(flip="", obs="rec[-2] rec[-1]"), True, False, "0000"),
    (LOOP.format(flip="X_ERROR(1) 0 1\n", obs="rec[-2]"), True, False, "1000"),
    (LOOP.format(flip="X_ERROR(1) 0 1\n", obs="rec[-2]"), False, True, "0001"),
]

# command_sample.test.cc:73-138, 317-336: (circuit, measurement line of every shot).
SAMPLE_EXACT = [("M 0", "0"), ("X 0\nM 0", "1"), ("M !0", "1"), ("X 0\nR 0\nM 0", "0"), ("X 0\nMR 0\nMR 0", "10")]

# command_sample.test.cc:160-315: (circuit, shots, {line: probability}).
FOUR = lambda p: {"00": (1 - p) ** 2, "01": (1 - p) * p, "10": (1 - p) * p, "11": p * p}
DISTRIBUTIONS = [
    ("H 0\nCNOT 0 1\nM 0 1", 10000, {"00": 0.5, "11": 0.5}),
    ("H 0\nCNOT 0 1\nSQRT_X 0 1\nM 0 1", 10000, {"10": 0.5, "01": 0.5}),
    ("H 0\nCNOT 0 1\nSQRT_Y 0 1\nM 0 1", 10000, {"00": 0.5, "11": 0.5}),
    ("X_ERROR(0.1) 0 1\nM 0 1", 100000, FOUR(0.1)),
    ("H 0 1\nX_ERROR(0.1) 0 1\nH 0 1\nM 0 1", 10, {"00": 1}),
    ("H 0 1\nZ_ERROR(0.1) 0 1\nH 0 1\nM 0 1", 100000, FOUR(0.1)),
    ("Z_ERROR(0.1) 0 1\nM 0 1", 10, {"00": 1}),
    ("Y_ERROR(0.1) 0 1\nM 0 1", 100000, FOUR(0.1)),
    ("H_YZ 0 1\nY_ERROR(0.1) 0 1\nH_YZ 0 1\nM 0 1", 10, {"00": 1}),
    ("DEPOLARIZE1(0.3) 0 1\nM 0 1", 100000, FOUR(0.2)),
    ("H 0 1\nDEPOLARIZE1(0.3) 0 1\nH 0 1\nM 0 1", 100000, FOUR(0.2)),
    ("H_YZ 0 1\nDEPOLARIZE1(0.3) 0 1\nH_YZ 0 1\nM 0 1", 100000, FOUR(0.2)),
    ("DEPOLARIZE2(0.1) 0 1\nM 0 1", 100000,
     {"00": 0.1 * 3 / 15 + 0.9, "01": 0.1 * 4 / 15, "10": 0.1 * 4 / 15, "11": 0.1 * 4 / 15}),
    ("H 0\nH_YZ 1\nDEPOLARIZE2(0.3) 0 1\nH 0\nH_YZ 1\nM 0 1", 100000,
     {"00": 0.3 * 3 / 15 + 0.7, "01": 0.3 * 4 / 15, "10": 0.3 * 4 / 15, "11": 0.3 * 4 / 15}),
]
# command_sample.test.cc:338-386: H S S H flips |0> to |1>; the flips alone (no reference sample) stay 0.
HSSH = "H 0\nS 0\nS 0\nH 0\nM 0"


def deviation(lines, expected):
    """The reference's distribution check (command_sample.test.cc:37-71): "" when it passes, else the reason."""
    actual = Counter(lines)
    for line in actual:
        if line not in expected:
            return f"Sampled {line} which was not expected."
    total = sum(actual.values())
    if total == 0:
        return "No samples."
    if abs(sum(expected.values()) - 1) > 1e-5:
        return "Expected distribution doesn't add up to 1."
    for line, rate in expected.items():
        allowed = 5 * math.sqrt(rate * (1 - rate) / total)
        if rate - allowed < 0 or rate + allowed > 1:
            return "Not enough samples to bound results away from extremes."
        if abs(rate - actual[line] / total) > allowed:
            return f"Actual rate {actual[line] / total} of sample '{line}' is more than 5 standard deviations"
    return ""


def lines_of(bits):
    return ["".join("1" if b else "0" for b in row) for row in np.asarray(bits)]


def oracle_measurements(text, shots, seed, skip_reference=False):
    o = OracleCircuit(text)
    _, _, m = o.sample(shots, seed, dets=False, obs=False, meas=True, threads=4)
    flips = np.unpackbits(m, axis=1, bitorder="little")[:, :o.num_measurements].astype(np.bool_)
    if skip_reference:
        return flips
    return flips ^ stim_gb300.Circuit(text).reference_sample()


def oracle_detections(text, shots, prepend, append):
    o = OracleCircuit(text)
    d, obs, _ = o.sample(shots, 1)
    d = np.unpackbits(d, axis=1, bitorder="little")[:, :o.num_detectors]
    obs = np.unpackbits(obs, axis=1, bitorder="little")[:, :o.num_observables]
    return np.concatenate(([obs] if prepend else []) + [d] + ([obs] if append else []), axis=1)


def test_deviation_rejects_what_the_reference_rejects():
    # command_sample.test.cc:140-158 intentional_failures.
    assert deviation(["00", "10", "11"], {"00": 0.5, "11": 0.5}) == "Sampled 10 which was not expected."
    assert deviation(["0"] * 500 + ["1"] * 500, {"0": 0.1, "1": 0.9}) != ""
    assert deviation(["0"] * 500 + ["1"] * 500, {"0": 0.5, "1": 0.5}) == ""


@pytest.mark.parametrize("text,prepend,append,want", DETECT)
def test_oracle_detect(text, prepend, append, want):
    assert lines_of(oracle_detections(text, 2, prepend, append)) == [want] * 2


@pytest.mark.parametrize("text,want", SAMPLE_EXACT)
def test_oracle_sample_exact(text, want):
    assert lines_of(oracle_measurements(text, 2, 5)) == [want] * 2


@pytest.mark.parametrize("text,shots,expected", DISTRIBUTIONS)
def test_oracle_distributions(text, shots, expected):
    assert deviation(lines_of(oracle_measurements(text, shots, 11)), expected) == ""


def test_oracle_skip_reference_sample():
    assert deviation(lines_of(oracle_measurements(HSSH, 10, 3, skip_reference=True)), {"0": 1}) == ""
    assert deviation(lines_of(oracle_measurements(HSSH, 10, 3)), {"1": 1}) == ""


def test_oracle_detect_mpp_counts():
    # command_detect.test.cc:185-196: a Z8*X9 product is random.
    d = oracle_detections("MPP Z8*X9\nDETECTOR rec[-1]", 1000, False, False)
    assert 400 < 1000 - d.sum() < 600


@pytest.mark.gpu
@pytest.mark.parametrize("shots", [1, 2])
@pytest.mark.parametrize("text,prepend,append,want", DETECT)
def test_gpu_detect(tmp_path, text, prepend, append, want, shots):
    path = tmp_path / "out"
    stim_gb300.Circuit(text).compile_detector_sampler().sample_write(
        shots, filepath=str(path), format="01", prepend_observables=prepend, append_observables=append)
    assert path.read_text() == (want + "\n") * shots


@pytest.mark.gpu
@pytest.mark.parametrize("shots", [0, 1, 2])
@pytest.mark.parametrize("text,want", SAMPLE_EXACT)
def test_gpu_sample_exact(tmp_path, text, want, shots):
    path = tmp_path / "out"
    stim_gb300.Circuit(text).compile_sampler().sample_write(shots, filepath=str(path), format="01")
    assert path.read_text() == (want + "\n") * shots


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("text,shots,expected", DISTRIBUTIONS)
def test_gpu_distributions(text, shots, expected, noise_mode):
    s = stim_gb300.Circuit(text).compile_sampler(seed=11)
    s.set_noise_mode(noise_mode)
    assert deviation(lines_of(s.sample(shots)), expected) == ""


@pytest.mark.gpu
def test_gpu_skip_reference_sample():
    c = stim_gb300.Circuit(HSSH)
    for shots in (1, 10):
        assert deviation(lines_of(c.compile_sampler(skip_reference_sample=True).sample(shots)), {"0": 1}) == ""
        assert deviation(lines_of(c.compile_sampler().sample(shots)), {"1": 1}) == ""


@pytest.mark.gpu
def test_gpu_detect_mpp_counts(tmp_path):
    path = tmp_path / "out"
    stim_gb300.Circuit("MPP Z8*X9\nDETECTOR rec[-1]").compile_detector_sampler().sample_write(
        1000, filepath=str(path), format="01")
    text = path.read_text()
    assert len(text) == 2000 and text[1::2] == "\n" * 1000
    assert 400 < text[0::2].count("0") < 600


@pytest.mark.gpu
@pytest.mark.parametrize("compile_name,text", [("compile_sampler", "H 0\nM 0"),
                                               ("compile_detector_sampler", "X_ERROR(0.5) 0\nM 0\nDETECTOR rec[-1]")])
def test_gpu_seeded_sampling(tmp_path, compile_name, text):
    # command_sample.test.cc:388-420, command_detect.test.cc:198-233: equal seeds give equal files, others differ.
    c = stim_gb300.Circuit(text)

    def run(seed):
        path = tmp_path / "out"
        getattr(c, compile_name)(seed=seed).sample_write(256, filepath=str(path), format="01")
        return path.read_text()

    assert run(5) == run(5)
    assert run(5) != run(6)
    assert run(None) != run(None)


# command_m2d.test.cc:22-62: X 0, M 0 1, D0 = rec[-2], D1 = rec[-1], L2 = rec[-1]; inputs 00, 01, 10, 11.
M2D = "X 0\nM 0 1\nDETECTOR rec[-2]\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(2) rec[-1]"
M2D_IN = "00\n01\n10\n11\n"
M2D_CASES = [
    (False, True, "shot D0\nshot D0 D1 L2\nshot\nshot D1 L2\n"),
    (False, False, "shot D0\nshot D0 D1\nshot\nshot D1\n"),
    (True, False, "shot\nshot D1\nshot D0\nshot D0 D1\n"),
]
# command_m2d.test.cc:64-120: records controlling Paulis change the reference sample, not the conversion.
FEEDBACK = """
CX 0 2 1 2
M 2
CX rec[-1] 2
DETECTOR rec[-1]
TICK
CX 0 2 1 2
M 2
CX rec[-1] 2
DETECTOR rec[-1] rec[-2]
TICK
CX 0 2 1 2
M 2
CX rec[-1] 2
DETECTOR rec[-1] rec[-2]
TICK
M 0 1
DETECTOR rec[-1] rec[-2] rec[-3]
OBSERVABLE_INCLUDE(0) rec[-1]
"""
FEEDBACK_IN = "00000\n10000\n01000\n00100\n00010\n00001\n"
FEEDBACK_OUT = "shot\nshot D0 D1\nshot D1 D2\nshot D2 D3\nshot D3\nshot D3 L0\n"
# command_m2d.test.cc:158-176: observables of Pauli terms only; the conversion ignores the terms.
UNPHYSICAL = """
QUBIT_COORDS(0, 0) 0
QUBIT_COORDS(1, 0) 1
QUBIT_COORDS(0, 1) 2
QUBIT_COORDS(1, 1) 3
OBSERVABLE_INCLUDE(0) X0 X1
OBSERVABLE_INCLUDE(1) Z0 Z2
MPP X0*X1*X2*X3 Z0*Z1 Z2*Z3
DEPOLARIZE1(0.001) 0 1 2 3
MPP X0*X1*X2*X3 Z0*Z1 Z2*Z3
DETECTOR rec[-1] rec[-4]
DETECTOR rec[-2] rec[-5]
DETECTOR rec[-3] rec[-6]
OBSERVABLE_INCLUDE(0) X0 X1
OBSERVABLE_INCLUDE(1) Z0 Z2
"""


def parse01(text):
    return np.array([[ch == "1" for ch in line] for line in text.splitlines()], dtype=np.bool_)


def dets_lines(d, o, append):
    out = []
    for dr, orow in zip(d, o):
        line = "shot" + "".join(f" D{k}" for k in np.nonzero(dr)[0])
        if append:
            line += "".join(f" L{k}" for k in np.nonzero(orow)[0])
        out.append(line + "\n")
    return "".join(out)


def oracle_m2d_dets(text, data01, skip, append):
    c, o = stim_gb300.Circuit(text), OracleCircuit(text)
    ref = None if skip else c.reference_sample(bit_packed=True)
    packed = np.packbits(parse01(data01), axis=1, bitorder="little")
    d, ob = o.m2d(packed, ref if ref is not None and ref.size else None)
    d = np.unpackbits(d, axis=1, bitorder="little")[:, :o.num_detectors]
    ob = np.unpackbits(ob, axis=1, bitorder="little")[:, :o.num_observables]
    return d, ob


@pytest.mark.parametrize("skip,append,want", M2D_CASES)
def test_oracle_m2d_command(skip, append, want):
    assert dets_lines(*oracle_m2d_dets(M2D, M2D_IN, skip, append), append) == want


def test_oracle_m2d_feedback_and_unphysical_observables():
    assert dets_lines(*oracle_m2d_dets(FEEDBACK, FEEDBACK_IN, False, True), True) == FEEDBACK_OUT
    d, ob = oracle_m2d_dets(UNPHYSICAL, "000000\n100100\n000110\n", False, False)
    assert lines_of(d) == ["000", "000", "011"] and lines_of(ob) == ["00", "00", "00"]


def m2d_file(tmp_path, text, data01, out_format, skip=False, append=False, obs=False):
    src, out, obs_path = tmp_path / "in", tmp_path / "out", tmp_path / "obs"
    src.write_text(data01)
    conv = stim_gb300.Circuit(text).compile_m2d_converter(skip_reference_sample=skip)
    conv.convert_file(measurements_filepath=str(src), measurements_format="01", detection_events_filepath=str(out),
                      detection_events_format=out_format, append_observables=append,
                      obs_out_filepath=str(obs_path) if obs else None, obs_out_format="01")
    return out.read_text(), (obs_path.read_text() if obs else None)


@pytest.mark.gpu
@pytest.mark.parametrize("skip,append,want", M2D_CASES)
def test_gpu_m2d_command(tmp_path, skip, append, want):
    assert m2d_file(tmp_path, M2D, M2D_IN, "dets", skip=skip, append=append)[0] == want


@pytest.mark.gpu
def test_gpu_m2d_feedback(tmp_path):
    assert m2d_file(tmp_path, FEEDBACK, FEEDBACK_IN, "dets", append=True)[0] == FEEDBACK_OUT


@pytest.mark.gpu
@pytest.mark.parametrize("index,obs_line", [(0, "0\n"), (10, "00000000000\n")])
def test_gpu_m2d_obs_file_sizes(tmp_path, index, obs_line):
    # command_m2d.test.cc:122-156: 1,024 detectors and an observables file of 1 or 11 observables.
    text = f"M 0\nREPEAT 1024 {{\n    DETECTOR rec[-1]\n}}\nOBSERVABLE_INCLUDE({index}) rec[-1]"
    assert m2d_file(tmp_path, text, "0\n", "01", obs=True) == ("0" * 1024 + "\n", obs_line)


@pytest.mark.gpu
def test_gpu_m2d_unphysical_observables(tmp_path):
    assert m2d_file(tmp_path, UNPHYSICAL, "000000\n100100\n000110\n", "01", obs=True) == (
        "000\n000\n011\n", "00\n00\n00\n")


@pytest.mark.gpu
def test_gpu_sample_dem_command(tmp_path):
    # command_sample_dem.test.cc:22-51: an empty model gives one empty line; error(0) D0, error(1) D1 L2 at seed 0.
    det, obs = tmp_path / "det", tmp_path / "obs"
    stim_gb300.DetectorErrorModel("").compile_sampler(seed=0).sample_write(
        1, det_out_file=str(det), det_out_format="01", obs_out_file=None)
    assert det.read_text() == "\n"
    stim_gb300.DetectorErrorModel("error(0) D0\nerror(1) D1 L2").compile_sampler(seed=0).sample_write(
        5, det_out_file=str(det), det_out_format="01", obs_out_file=str(obs), obs_out_format="01")
    assert det.read_text() == "01\n" * 5
    assert obs.read_text() == "001\n" * 5
