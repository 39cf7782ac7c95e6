"""MPAD and pair measurements (MXX / MYY / MZZ) as the reference's own tests state them
(src/stim/simulators/frame_simulator.test.cc:1489-1543: mpad, mxxyyzz_basis, mxxyyzz_inversion): measurement records
(reference sample included) with fixed values or fixed relations between results, whatever the random outcomes.
The oracle's flips XOR the host reference sample on the CPU; the GPU measurement sampler in both noise modes."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

SHOTS = 100
MPAD = "MPAD 0 1"
BASIS = "RX 0 1\nMXX 0 1\nRY 0 1\nMYY 0 1\nRZ 0 1\nMZZ 0 1"
INVERSION = "MXX 0 1 0 !1 !0 1 !0 !1\nMYY 0 1 0 !1 !0 1 !0 !1\nMZZ 0 1 0 !1 !0 1 !0 !1"


def check(text, s):
    if text == MPAD:
        assert (s[:, 0] == 0).all() and (s[:, 1] == 1).all()
    elif text == BASIS:
        assert not s[:, :3].any()
    else:
        for b in (0, 4, 8):
            assert (s[:, b + 1] == 1 - s[:, b]).all()
            assert (s[:, b + 2] == 1 - s[:, b]).all()
            assert (s[:, b + 3] == s[:, b]).all()
        assert (s[:, 8] == 1 ^ s[:, 0] ^ s[:, 4]).all()
    return s


@pytest.mark.parametrize("text", [MPAD, BASIS, INVERSION], ids=["mpad", "basis", "inversion"])
def test_oracle_records(text):
    c = stim_gb300.Circuit(text)
    ref = c.reference_sample(bit_packed=True)
    _, _, m = OracleCircuit(text).sample(SHOTS, 9, dets=False, obs=False, meas=True)
    s = np.unpackbits(m ^ ref[None, :], axis=1, bitorder="little")[:, :c.num_measurements]
    check(text, s)
    if text == INVERSION:
        assert 0 < s[:, 0].sum() < SHOTS  # the outcomes are random, only their relations are fixed


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("text", [MPAD, BASIS, INVERSION], ids=["mpad", "basis", "inversion"])
def test_gpu_records(text, noise_mode):
    c = stim_gb300.Circuit(text)
    sm = c.compile_sampler(seed=9)
    sm.set_noise_mode(noise_mode)
    s = sm.sample(SHOTS).astype(np.uint8)
    check(text, s)
    ref = c.reference_sample(bit_packed=True)
    _, _, m = OracleCircuit(text).sample(SHOTS, 9, dets=False, obs=False, meas=True)
    np.testing.assert_array_equal(s, np.unpackbits(m ^ ref[None, :], axis=1, bitorder="little")[:, :c.num_measurements])
