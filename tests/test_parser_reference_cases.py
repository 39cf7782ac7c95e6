"""The reference's circuit-parser tests, restated against this package's host parser (no GPU;
src/stim/circuit/circuit.test.cc:23-170 from_text, :172-208 parse_mpp, :210-252 parse_spp / parse_spp_dag,
:254-315 parse_tag, :317-330 parse_sweep_bits, :415-444 append_op_validation (as text), :446-496 repeat / tick /
detector / X_ERROR / PAULI_CHANNEL_1 / PAULI_CHANNEL_2 validation, :503-523 classical_controls, :1025-1034
zero_repetitions_not_allowed, :1213-1223 NaN probability and MPAD): every text the reference rejects raises
ValueError (its std::invalid_argument), every text it accepts parses, with the measurement counts it implies."""

import pytest

import stim_gb300

REJECTED = [
    # from_text
    "H a", "H(1)", "X_ERROR 1", "H 9999999999999999999999999999999999999999999", "H -1", "CNOT 0 a",
    "CNOT 0 99999999999999999999999999999999", "CNOT 0 -1", "DETECTOR 1 2", "CX 1 1", "SWAP 1 1",
    "DEPOLARIZE2(1) 1 1", "DETEstdCTOR rec[-1]", "DETECTOR rec[0]", "DETECTOR rec[1]", "DETECTOR rec[-999999999999]",
    "OBSERVABLE_INCLUDE rec[-1]", "OBSERVABLE_INCLUDE(-1) rec[-1]", "CORRELATED_ERROR(1) B1",
    "CORRELATED_ERROR(1) X 1", "CORRELATED_ERROR(1) X\n", "CORRELATED_ERROR(1) 1", "ELSE_CORRELATED_ERROR(1) 1 2",
    "CORRELATED_ERROR(1) 1 2", "CORRELATED_ERROR(1) A", "CNOT 0\nCNOT 1",
    # parse_mpp, parse_spp, parse_spp_dag, parse_sweep_bits
    "H *", "MPP 0", "MPP *", "MPP * X1", "MPP * X1 *", "MPP X1 *", "MPP X1 * * Y2", "MPP X1**Y2", "MPP(1.1) X1**Y2",
    "MPP(-0.5) X1**Y2", "MPP X1*rec[-1]", "MPP rec[-1]", "MPP sweep[0]", "SPP 1", "SPP rec[-1]", "SPP sweep[0]",
    "SPP rec[-1]*X0", "SPP_DAG 1", "SPP_DAG rec[-1]", "SPP_DAG sweep[0]", "SPP_DAG rec[-1]*X0", "H sweep[0]",
    "X sweep[0]",
    # append_op_validation, as text
    "CNOT 0", "X X0", "X Z0", "X !0", "X(0.5) 0", "M X0", "M Z0", "M(1.5) 0", "M(-1.5) 0", "M(0.125, 0.25) 0",
    "CORRELATED_ERROR X0", "CORRELATED_ERROR(0.1, 0.2) X0", "CNOT 0 0",
    # repeat / tick / detector / error-argument validation
    "REPEAT 100 {", "REPEAT 100 {{\n}", "REPEAT {\n}", "H {", "H {\n}", "TICK 1", "DETECTOR 1",
    "X_ERROR(-0.1) 1", "X_ERROR(1.1) 1", "X_ERROR(0.1, 0.1) 1", "PAULI_CHANNEL_1 1", "PAULI_CHANNEL_1(0.1) 1",
    "PAULI_CHANNEL_1(0.1,0.1) 1", "PAULI_CHANNEL_1(0.1,0.1,0.1,0.1) 1", "PAULI_CHANNEL_1(-1,0,0) 1",
    "PAULI_CHANNEL_1(0.1,0.5,0.6) 1", "PAULI_CHANNEL_2(0.1,0,0,0,0,0,0,0,0,0,0.1,0,0,0,0.1) 1",
    "PAULI_CHANNEL_2(0.4,0,0,0,0,0.4,0,0,0,0,0,0,0,0,0.4) 1 2", "PAULI_CHANNEL_2(0,0,0,0,0,0,0,0,0,0,0,0,0,0) 1 2",
    "PAULI_CHANNEL_2(0,0,0,0,0,0,0,0,0,0,0,0,0,0,0,0) 1 2",
    # classical control of a qubit-only gate, zero repetitions, NaN, MPAD of a non-bit
    "M 0\nXCX rec[-1] 1", "REPEAT 0 {\n    M 0\n    OBSERVABLE_INCLUDE(0) rec[-1]\n}", "X_ERROR(nan) 0", "MPAD 2",
    "MPAD sweep[-1]",
    # an empty argument reads as 0 (the reference's read_normal_double), which these gates cannot take
    "H() 0", "TICK()", "H( ) 0", "X_ERROR(0.1,) 0",
]

# (text, measurements it records)
ACCEPTED = [
    ("# not an operation", 0), ("H 0", 0), ("h 0", 0), ("H 0     ", 0), ("     H 0     ", 0), ("\tH 0\t\t", 0),
    ("H 0  # comment", 0), ("H 23", 0), ("DEPOLARIZE1(0.125) 4 5  # comment", 0), ("  \t Cnot 5 6  # comment   ", 0),
    ("", 0), ("# Comment\n\n\n# More", 0), ("H 0 \n H 1", 0), ("# EPR\nH 0\nCNOT 0 1", 0), ("M 0 !0 1 !1", 4),
    ("H 0\nM 0\nM 1\nM 2\nSWAP 0 1\nM 0\nM 10", 5), ('X 0\nREPEAT 2 {\n  Y 1\n  Y 2 #####"\n} #####"', 0),
    ("M 0\nREPEAT 5 {\n  M 1 2\n  M 3\n} #####", 16), ("CORRELATED_ERROR(0.125) X90 Y91 Z92 X93", 0),
    ("MPP X1*Y2 Z3 * Z4\nMPP Z5", 3), ("MPP(0.125) X1*Y2 Z3 * Z4\nMPP Z5", 3), ("MPP X1*X1", 1), ("SPP", 0),
    ("SPP X0 X1*Y2*Z3", 0), ("SPP X1 Z2", 0), ("SPP_DAG", 0), ("SPP_DAG X0 X1*Y2*Z3", 0), ("SPP_DAG X1 Z2", 0),
    ("H[test] 3 5", 0), ("H[] 3 5", 0), ("H[test \\B\\C\\r\\n] 3 5", 0),
    ("X_ERROR[test](0.125)\nX_ERROR[no_fuse](0.125) 1\nX_ERROR(0.125) 2\nX_ERROR[](0.125) 3\n"
     "REPEAT[looper] 5 {\n    CX[within] 0 1\n}", 0),
    ("CNOT sweep[2] 5", 0), ("CNOT 0 1\nM !0\nM(0.125) !0", 2),
    ("CORRELATED_ERROR(0.1) X0\nCORRELATED_ERROR(0.1) Z0", 0),
    ("X_ERROR(0.5) 0", 0), ("X_ERROR(0) 1", 0), ("X_ERROR(0.1) 1", 0), ("X_ERROR(1) 1", 0),
    ("PAULI_CHANNEL_1(0,0,0) 1", 0), ("PAULI_CHANNEL_1(0.1,0.2,0.6) 1", 0), ("PAULI_CHANNEL_1(1,0,0) 1", 0),
    ("PAULI_CHANNEL_1(0.33333333334,0.33333333334,0.33333333334) 1", 0),
    ("PAULI_CHANNEL_2(0,0,0,0,0,0,0,0,0,0,0,0,0,0,0) 1 2", 0),
    ("PAULI_CHANNEL_2(0.1,0,0,0,0,0,0,0,0,0,0.1,0,0,0,0.1) 1 2", 0),
    ("ZCX 0 1\nZCX rec[-1] 1\nZCY rec[-2] 1\nZCZ rec[-4] 1", 0), ("MPAD 0 1", 2), ("H 0\r\nH 1\r\n", 0),
    # an empty argument reads as 0, as the reference's parser reads it (found by comparing acceptance with the
    # reference's own `stim sample` / `stim detect` on random texts)
    ("X_ERROR() 0", 0), ("X_ERROR( ) 0", 0), ("M() 0", 1), ("QUBIT_COORDS() 0", 0), ("DETECTOR()", 0),
    ("MPP() X0", 1), ("PAULI_CHANNEL_1(,,) 0", 0), ("PAULI_CHANNEL_1(0.1,,) 0", 0), ("REPEAT() 2 {\n}", 0),
]


@pytest.mark.parametrize("text", REJECTED)
def test_rejected_like_the_reference(text):
    with pytest.raises(ValueError):
        stim_gb300.Circuit(text)


@pytest.mark.parametrize("text,measurements", ACCEPTED)
def test_accepted_like_the_reference(text, measurements):
    assert stim_gb300.Circuit(text).num_measurements == measurements


@pytest.mark.parametrize("text", ["M 0\nDETECTOR rec[-3]", "OBSERVABLE_INCLUDE(0) rec[-3]",
                                  "REPEAT 3 {\n    M 0\n    DETECTOR rec[-2]\n}"])
def test_unreadable_detectors_matter_only_to_detection_sampling(text):
    # The reference's measurement sampler keeps no detection data (frame_simulator.inl:222-252), so `stim sample`
    # takes these circuits while `stim detect` rejects them (std::out_of_range, IndexError in Python).
    c = stim_gb300.Circuit(text)
    c.program_info("measurements")
    with pytest.raises(IndexError, match="before the beginning of time"):
        c.program_info("detections")
