"""The CPU oracle against fixtures produced by the reference's own FrameSimulator on the same injected
random stream (tests/golden/make_golden.py, oracle/ref_inject.cc).  This is what pins the oracle."""

import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, golden_names
from oracle.oracle import OracleCircuit


def load(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name):
    g = load(name)
    c = OracleCircuit(str(g["circuit"]))
    assert c.num_detectors == int(g["num_detectors"])
    assert c.num_observables == int(g["num_observables"])
    assert c.num_measurements == int(g["num_measurements"])
    d, o, m = c.sample(int(g["shots"]), int(g["seed"]), meas=True, threads=2)
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])
    np.testing.assert_array_equal(m, g["meas"])


def test_oracle_noiseless_surface_code_has_no_detection_events():
    g = load("surface_rx_d11_r11_p0")
    assert not g["dets"].any()
    c = OracleCircuit(str(g["circuit"]))
    d, o, _ = c.sample(1024, 99, threads=4)
    assert not d.any() and not o.any()


def test_oracle_obs_data_known_answer():
    # frame_simulator_util.test.cc:427-474: first 399 detectors fire in every shot, observable byte 0x3.
    g = load("obs_data_1001")
    bits = np.unpackbits(g["dets"], axis=1, bitorder="little")[:, :999]
    assert bits[:, :399].all() and not bits[:, 399:].any()
    assert (g["obs"][:, 0] == 0x3).all()


def test_oracle_results_do_not_depend_on_slicing():
    g = load("surface_rx_d5_r5_p0.01")
    c = OracleCircuit(str(g["circuit"]))
    d1, _, _ = c.sample(1024, 2, threads=1)
    d2, _, _ = c.sample(512, 2, first_shot=512, threads=3)
    np.testing.assert_array_equal(d1[512:], d2)
