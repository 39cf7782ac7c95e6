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
