"""The reference's command-line tests of `stim detect` and `stim sample`, restated against this package's samplers
(src/stim/cmd/command_detect.test.cc:21-196, command_sample.test.cc:73-420): the CLI's 01 output is what
sample_write(format="01") writes, and `--prepend_observables` / `--append_observables` / `--skip_reference_sample`
are the samplers' arguments of the same names.

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
