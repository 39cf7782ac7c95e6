"""Result files as the reference's own sampler tests state them (src/stim/simulators/frame_simulator_util.test.cc:
31-160: sample_test_detection_events, ..._writing_results_to_disk with dets / hits and observables prepended or
appended, stream_many_shots, block_results_single_shot / triple_shot): deterministic circuits, exact bytes."""

import numpy as np
import pytest

import stim_gb300

pytestmark = pytest.mark.gpu

OBS4 = """
    X_ERROR(1) 0
    M 0 1
    DETECTOR rec[-1]
    DETECTOR rec[-2]
    OBSERVABLE_INCLUDE(4) rec[-2]
"""
BLOCKS = """
    REPEAT 10000 {
        M 0
        X_ERROR(1) 0
        M 0
        R 0
        DETECTOR rec[-1] rec[-2]
        M 0
        DETECTOR rec[-1]
        DETECTOR rec[-1]
    }
"""


def write(tmp_path, text, shots, fmt, **kw):
    path = tmp_path / "out"
    stim_gb300.Circuit(text).compile_detector_sampler(seed=1).sample_write(shots, filepath=str(path), format=fmt, **kw)
    return path.read_bytes()


def test_x_error_one_gives_ones():
    d = stim_gb300.Circuit("X_ERROR(1) 0\nM 0\nDETECTOR rec[-1]\n").compile_detector_sampler(seed=1).sample(5)
    assert d.shape == (5, 1) and d.all()


@pytest.mark.parametrize("fmt,kw,want", [
    ("dets", {}, b"shot D1\nshot D1\n"),
    ("dets", {"prepend_observables": True}, b"shot L4 D1\nshot L4 D1\n"),
    ("dets", {"append_observables": True}, b"shot D1 L4\nshot D1 L4\n"),
    ("hits", {"append_observables": True}, b"1,6\n1,6\n"),
])
def test_observables_in_dets_and_hits(tmp_path, fmt, kw, want):
    assert write(tmp_path, OBS4, 2, fmt, **kw) == want


def test_stream_many_shots(tmp_path):
    text = "X_ERROR(1) 1\nM 0 1 2\nDETECTOR rec[-1]\nDETECTOR rec[-2]\nDETECTOR rec[-3]\n"
    assert write(tmp_path, text, 2048, "01") == b"010\n" * 2048


@pytest.mark.parametrize("shots", [1, 3])
def test_block_results(tmp_path, shots):
    assert write(tmp_path, BLOCKS, shots, "01", append_observables=True) == (b"100" * 10000 + b"\n") * shots
