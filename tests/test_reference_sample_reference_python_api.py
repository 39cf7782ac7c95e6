"""The reference's own Python test of Circuit.reference_sample (src/stim/circuit/circuit_pybind_test.py:1497-1523),
restated against this package's host reference sample (no GPU): no measurements give an empty sample, the sample is
deterministic, the parity of X0*X1, Y0*Y1, Z0*Z1 on a Bell pair is odd, and the bit-packed form is the unpacked
one padded with zeros."""

import numpy as np

import stim_gb300


def test_reference_sample():
    assert len(stim_gb300.Circuit("H 0\nCNOT 0 1").reference_sample()) == 0
    text = "H 0 1\nCX 0 2 1 3\nMPP X0*X1 Y0*Y1 Z0*Z1\n"
    c = stim_gb300.Circuit(text)
    np.testing.assert_array_equal(c.reference_sample(), c.reference_sample())
    assert np.sum(c.reference_sample()) % 2 == 1
    c = stim_gb300.Circuit(text + "X " + " ".join(map(str, range(0, 100, 2))) + "\n" +
                           "M " + " ".join(map(str, range(100))))
    packed = c.reference_sample(bit_packed=True)
    unpacked = np.unpackbits(packed, bitorder="little")
    expected = c.reference_sample(bit_packed=False)
    padded = np.zeros_like(unpacked)
    padded[:len(expected)] = expected
    np.testing.assert_array_equal(unpacked, padded)
