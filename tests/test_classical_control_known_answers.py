"""Classical control as the reference's own tests state it (src/stim/simulators/frame_simulator.test.cc:573-705):
a measurement record may control a Pauli on a qubit (CX/CY/XCZ/YCZ with the record on the control side), never
the reverse (the circuit is rejected with a ValueError, the reference's std::invalid_argument).  The rejections are
host-side (parser / lowering, no GPU); the controlled flips on the oracle and on the GPU sampler."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit

QUANTUM_CONTROLS_CLASSICAL = ["M 0\nCNOT 1 rec[-1]", "M 0\nCY 1 rec[-1]", "M 0\nYCZ rec[-1] 1",
                              "M 0\nXCZ rec[-1] 1", "M 0\nSWAP 1 rec[-1]"]
CLASSICAL_CONTROLS_QUANTUM = [f"X_ERROR(1) 0\nM !0\n{g}\nM 1" for g in
                              ("CX rec[-1] 1", "CY rec[-1] 1", "XCZ 1 rec[-1]", "YCZ 1 rec[-1]")]


@pytest.mark.parametrize("text", QUANTUM_CONTROLS_CLASSICAL)
def test_quantum_cannot_control_classical(text):
    with pytest.raises(ValueError):
        stim_gb300.Circuit(text).program_info("measurements")


@pytest.mark.parametrize("text", CLASSICAL_CONTROLS_QUANTUM)
def test_oracle_classical_can_control_quantum(text):
    _, _, m = OracleCircuit(text).sample(64, 1, dets=False, obs=False, meas=True)
    assert (np.unpackbits(m, axis=1, bitorder="little")[:, :2] == 1).all()


@pytest.mark.gpu
@pytest.mark.parametrize("noise_mode", [0, 1], ids=["inline", "hit_lists"])
@pytest.mark.parametrize("text", CLASSICAL_CONTROLS_QUANTUM)
def test_gpu_classical_can_control_quantum(text, noise_mode):
    s = stim_gb300.Circuit(text).compile_sampler(skip_reference_sample=True, seed=1)
    s.set_noise_mode(noise_mode)
    assert s.sample(64).all()
