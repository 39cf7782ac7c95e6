"""Circuit counts as the reference's own Python tests state them (src/stim/circuit/circuit_pybind_test.py:24-45,
350-384): qubits, measurements, detectors and observables of small circuits, through REPEAT blocks nested to
10^12 iterations (counted, not unrolled).  Host code (the parser), no GPU."""

import stim_gb300


def test_counts_of_small_circuits():
    c = stim_gb300.Circuit()
    assert c.num_qubits == c.num_measurements == 0
    c = stim_gb300.Circuit("X 3")
    assert (c.num_qubits, c.num_measurements) == (4, 0)
    c = stim_gb300.Circuit("X 3\nM 0")
    assert (c.num_qubits, c.num_measurements) == (4, 1)


def test_num_detectors():
    assert stim_gb300.Circuit().num_detectors == 0
    assert stim_gb300.Circuit("DETECTOR").num_detectors == 1
    assert stim_gb300.Circuit("REPEAT 1000 {\n DETECTOR\n}").num_detectors == 1000
    assert stim_gb300.Circuit("""
        DETECTOR
        REPEAT 1000000 {
            REPEAT 1000000 {
                M 0
                DETECTOR rec[-1]
            }
        }
    """).num_detectors == 1000000 ** 2 + 1


def test_num_observables():
    assert stim_gb300.Circuit().num_observables == 0
    assert stim_gb300.Circuit("OBSERVABLE_INCLUDE(0)").num_observables == 1
    assert stim_gb300.Circuit("OBSERVABLE_INCLUDE(1)").num_observables == 2
    assert stim_gb300.Circuit("""
        M 0
        OBSERVABLE_INCLUDE(2)
        REPEAT 1000000 {
            REPEAT 1000000 {
                M 0
                OBSERVABLE_INCLUDE(3) rec[-1]
            }
            OBSERVABLE_INCLUDE(4)
        }
    """).num_observables == 5


def _nest(depth, body, reps=999999):
    for _ in range(depth):
        body = f"REPEAT {reps} {{\n{body}\n}}"
    return body


def test_counts_of_the_reference_circuit_tests():
    # src/stim/circuit/circuit.test.cc:589-898 (count_qubits, count_detectors_num_observables, max_lookback,
    # count_measurements): counts through nested loops without unrolling, saturating at 2^64 - 1.
    C = stim_gb300.Circuit
    small = "H 0\nM 0 1\nREPEAT 2 {\n    X 1\n    REPEAT 3 {\n        Y 2\n        M 2\n    }\n}"
    assert C().num_qubits == 0 and C(small).num_qubits == 3
    assert C("H 0\nM 0 1\n" + _nest(4, "X 1\n" + _nest(1, "Y 2\nM 2"))).num_qubits == 3
    c = C("M 0 1 2\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(5) rec[-1]")
    assert (c.num_detectors, c.num_observables) == (1, 6)
    c = C("M 0 1\n" + _nest(4, "DETECTOR rec[-1]\nOBSERVABLE_INCLUDE(2) rec[-1]", 1000))
    assert (c.num_detectors, c.num_observables) == (10 ** 12, 3)
    c = C("M 0 1\n" + _nest(13, "DETECTOR rec[-1]"))
    assert (c.num_detectors, c.num_observables) == (2 ** 64 - 1, 0)
    assert C().max_lookback == 0 and C("M 0 1 2 3 4 5 6").max_lookback == 0
    assert C("M 0 1 2 3 4 5 6\nREPEAT 2 {\n    CNOT rec[-4] 0\n    REPEAT 3 {\n        CNOT rec[-1] 0\n    }\n}"
             ).max_lookback == 4
    assert C("M 0 1 2 3 4 5\n" + _nest(5, "CNOT rec[-5] 0")).max_lookback == 5
    assert C().num_measurements == 0 and C(small).num_measurements == 8
    assert C(_nest(3, "M 0")).num_measurements == 999999 ** 3
    assert C(_nest(9, "M 0")).num_measurements == 2 ** 64 - 1
    for text, n in [("MPP X0 Z1 Y2", 3), ("MPP X0 Z1*Y2", 2), ("MPP X0*X1*X2*X3*X4 Z5 Z6", 3), ("MXX 0 1 2 3", 2),
                    ("MYY 0 1 2 3", 2), ("MZZ 0 1 2 3", 2), ("MPP X0*X1 Z0*Z1 Y0*Y1", 3),
                    ("HERALDED_ERASE(0.01) 0 1 2", 3)]:
        assert C(text).num_measurements == n
