"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

* golden fixtures: outputs of the reference's own FrameSimulator on the injected stream, bit-exact;
* larger sizes: the CPU oracle on the same seeds, bit-exact;
* invariants: chunking, launch shape and stream continuation do not change any bit;
* noiseless circuits give exactly zero detection events.
"""

import os

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR, golden_names
from oracle.oracle import OracleCircuit
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu


def load(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


@pytest.mark.parametrize("name", golden_names())
def test_detections_match_reference_golden(name):
    g = load(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_detector_sampler(seed=int(g["seed"]))
    d, o = s.sample(int(g["shots"]), separate_observables=True, bit_packed=True)
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])


@pytest.mark.parametrize("name", golden_names())
def test_measurements_match_reference_golden(name):
    g = load(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_sampler(skip_reference_sample=True, seed=int(g["seed"]))
    m = s.sample(int(g["shots"]), bit_packed=True)
    np.testing.assert_array_equal(m, g["meas"])
    s2 = c.compile_sampler(reference_sample=g["ref_sample"], seed=int(g["seed"]))
    m2 = s2.sample(int(g["shots"]), bit_packed=True)
    np.testing.assert_array_equal(m2, g["meas"] ^ g["ref_sample"][None, :])
    # Default: the host computes the reference sample itself.
    s3 = c.compile_sampler(seed=int(g["seed"]))
    m3 = s3.sample(int(g["shots"]), bit_packed=True)
    np.testing.assert_array_equal(m3, g["meas"] ^ g["ref_sample"][None, :])


def _unpack(a, n):
    return np.unpackbits(a, axis=1, bitorder="little")[:, :n].astype(np.bool_)


def test_layout_flags_match_packed_golden():
    g = load("all_gates_s5")
    c = stim_gb300.Circuit(str(g["circuit"]))
    D, O, shots, seed = c.num_detectors, c.num_observables, int(g["shots"]), int(g["seed"])
    dets = _unpack(g["dets"], D)
    obs = _unpack(g["obs"], O)
    cases = [
        (dict(), dets),
        (dict(append_observables=True), np.concatenate([dets, obs], axis=1)),
        (dict(prepend_observables=True), np.concatenate([obs, dets], axis=1)),
        (dict(prepend_observables=True, append_observables=True), np.concatenate([obs, dets, obs], axis=1)),
    ]
    for kw, want in cases:
        for packed in (False, True):
            s = c.compile_detector_sampler(seed=seed)
            got = s.sample(shots, bit_packed=packed, **kw)
            if packed:
                got = _unpack(got, want.shape[1])
            np.testing.assert_array_equal(got, want, err_msg=str((kw, packed)))


def test_manual_output_buffers():
    text = """
        X_ERROR(1) 0
        M 0
        DETECTOR
        DETECTOR
        DETECTOR rec[-1]
        DETECTOR rec[-1]
        DETECTOR rec[-1]
        DETECTOR
        DETECTOR
        DETECTOR rec[-1]
        DETECTOR rec[-1]
        OBSERVABLE_INCLUDE(0) rec[-1]
    """
    s = stim_gb300.Circuit(text).compile_detector_sampler()
    for bad in [np.zeros((17, 8), np.bool_), np.zeros((17, 10), np.bool_), np.zeros((18, 9), np.bool_),
                np.zeros((17, 9), np.uint8)]:
        with pytest.raises(ValueError):
            s.sample(shots=17, dets_out=bad)
    buf = np.zeros((17, 9), dtype=np.bool_)
    assert s.sample(shots=17, dets_out=buf) is buf
    assert np.array_equal(buf, [[0, 0, 1, 1, 1, 0, 0, 1, 1]] * 17)
    buf = np.zeros((17, 2), dtype=np.uint8)
    assert s.sample(shots=17, dets_out=buf, bit_packed=True) is buf
    assert np.array_equal(buf, [[0b10011100, 0b1]] * 17)
    buf = np.zeros((2, 17), dtype=np.uint8).transpose()
    assert s.sample(shots=17, dets_out=buf, bit_packed=True) is buf
    assert np.array_equal(buf, [[0b10011100, 0b1]] * 17)
    obs = np.zeros((17, 1), dtype=np.bool_)
    s.sample(shots=17, obs_out=obs)
    assert obs.all()


def test_separate_with_append_raises():
    s = stim_gb300.Circuit("M 0\nDETECTOR rec[-1]").compile_detector_sampler()
    with pytest.raises(ValueError):
        s.sample(10, separate_observables=True, append_observables=True)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
@pytest.mark.parametrize("p", [0.001, 0.005])
def test_surface_d11_matches_oracle(seed, p):
    # The plain-GPU configuration: rotated memory-X, distance 11, 11 rounds, 2^20 shots, seeds 0..3.
    text = workloads.code_circuit("surface_code:rotated_memory_x", 11, 11, p)
    shots = 1 << 20
    gd, go = stim_gb300.Circuit(text).compile_detector_sampler(seed=seed).sample(
        shots, separate_observables=True, bit_packed=True)
    od, oo, _ = OracleCircuit(text).sample(shots, seed, threads=_THREADS)
    np.testing.assert_array_equal(gd, od)
    np.testing.assert_array_equal(go, oo)


_THREADS = max(1, min(32, os.cpu_count() or 1))


@pytest.mark.parametrize("mode,shots,autotune", [(1, 1 << 20, True), (1, 1 << 17, False), (0, 1 << 17, False)])
def test_surface_d25_benchmark_chunk_matches_oracle(mode, shots, autotune):
    # The benchmarked step: distance 25, 25 rounds, p = 1e-3, seed 0, hit-list noise with the launch shape the
    # autotuner picks (as the benchmark does) over a whole 2^20-shot chunk, and both noise modes at the default
    # shape.  The oracle is pinned to the reference's own FrameSimulator on this circuit by the
    # surface_rz_d25_r25_p0.001 fixture.
    text = workloads.code_circuit("surface_code:rotated_memory_z", 25, 25, 0.001)
    s = stim_gb300.Circuit(text).compile_detector_sampler(seed=0)
    s.set_noise_mode(mode)
    if autotune:
        s.autotune(1 << 18)
    gd, go = s.sample(shots, separate_observables=True, bit_packed=True)
    od, oo, _ = OracleCircuit(text).sample(shots, 0, threads=_THREADS)
    np.testing.assert_array_equal(gd, od)
    np.testing.assert_array_equal(go, oo)
    assert gd.any()
    t = s.last_timings()
    assert t["frame_launches"] >= 1
    if mode == 0:
        assert t["noise_launches"] == 0


def test_noiseless_surface_d11_gives_zero_detection_events():
    text = workloads.code_circuit("surface_code:rotated_memory_x", 11, 11, 0.0)
    d = stim_gb300.Circuit(text).compile_detector_sampler(seed=5).sample(1 << 18, bit_packed=True)
    assert not d.any()


@pytest.mark.parametrize("n,depth,seed", [(64, 200, 21), (128, 200, 22), (256, 200, 23), (512, 200, 24)])
def test_random_clifford_matches_oracle(n, depth, seed):
    text = workloads.random_clifford_circuit(n, depth, seed)
    shots = 2048
    gd, go = stim_gb300.Circuit(text).compile_detector_sampler(seed=seed).sample(
        shots, separate_observables=True, bit_packed=True)
    od, oo, _ = OracleCircuit(text).sample(shots, seed, threads=8)
    np.testing.assert_array_equal(gd, od)
    np.testing.assert_array_equal(go, oo)


def test_chunking_shape_and_continuation_do_not_change_bits():
    text = workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.01)
    c = stim_gb300.Circuit(text)
    ref = c.compile_detector_sampler(seed=9).sample(4096, bit_packed=True)
    for shape in [(1, 256), (2, 256), (4, 256), (1, 128), (2, 64)]:
        s = c.compile_detector_sampler(seed=9)
        s.set_launch_shape(*shape)
        np.testing.assert_array_equal(s.sample(4096, bit_packed=True), ref, err_msg=str(shape))
    s = c.compile_detector_sampler(seed=9)
    s.set_chunk_shots(384)
    np.testing.assert_array_equal(s.sample(4096, bit_packed=True), ref)
    s = c.compile_detector_sampler(seed=9)
    a = s.sample(1024, bit_packed=True)
    b = s.sample(3072, bit_packed=True)
    np.testing.assert_array_equal(np.concatenate([a, b]), ref)


def test_lookback_errors_match_reference():
    with pytest.raises(IndexError):
        stim_gb300.Circuit("M 0\nDETECTOR rec[-2]").compile_detector_sampler()
    with pytest.raises(ValueError):
        stim_gb300.Circuit("M 0\nCX 0 rec[-1]").compile_detector_sampler()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", golden_names())
def test_every_noise_mode_matches_golden(name, mode):
    # Mode 1 (the default) draws the hit lists with a separate kernel; mode 0 draws noise inside the frame
    # program.  Both must reproduce the reference's goldens.
    g = load(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_detector_sampler(seed=int(g["seed"]))
    s.set_noise_mode(mode)
    d, o = s.sample(int(g["shots"]), separate_observables=True, bit_packed=True)
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])
    if mode == 0:
        assert s.last_timings()["noise_launches"] == 0


@pytest.mark.parametrize("device_out", [False, True])
def test_hit_list_overflow_falls_back_to_inline_noise(device_out):
    from stim_gb300 import _native

    text = workloads.code_circuit("surface_code:rotated_memory_x", 5, 5, 0.02)
    c = stim_gb300.Circuit(text)
    want = c.compile_detector_sampler(seed=9)
    want.set_noise_mode(0)
    d0, o0 = want.sample(5000, bit_packed=True, separate_observables=True)
    s = c.compile_detector_sampler(seed=9)
    _native.check(_native.lib().gfs_sampler_set_hit_capacity(s._h, 4))  # far below the expected hits
    if device_out:
        torch = pytest.importorskip("torch")
        d = torch.zeros((5000, d0.shape[1]), dtype=torch.uint8, device="cuda")
        o = torch.zeros((5000, 1), dtype=torch.uint8, device="cuda")
        _native.check(_native.lib().gfs_sample_detections_device(s._h, 5000, _native.BIT_PACKED, d.data_ptr(),
                                                                 d.shape[1], o.data_ptr(), 1))
        d, o = d.cpu().numpy(), o.cpu().numpy()
    else:
        d, o = s.sample(5000, bit_packed=True, separate_observables=True)
    np.testing.assert_array_equal(d, d0)
    np.testing.assert_array_equal(o, o0)
    assert s.last_timings()["hit_overflows"] >= 1
    # The stream continues exactly where it would have.
    np.testing.assert_array_equal(s.sample(300, bit_packed=True), want.sample(300, bit_packed=True))


def _wide_circuit(n=9000, rounds=3):
    """A circuit whose frames (2 x 9000 rows x 16 B per 128 shots) exceed shared memory."""
    q = " ".join(map(str, range(n)))
    lines = ["R " + q, "X_ERROR(0.01) " + q]
    for _ in range(rounds):
        lines.append("CX " + " ".join(f"{2 * i} {2 * i + 1}" for i in range(n // 2)))
        lines.append("DEPOLARIZE1(0.001) " + q)
        lines.append("MR " + " ".join(str(2 * i + 1) for i in range(n // 2)))
        lines += ["DETECTOR rec[-%d]" % (k + 1) for k in range(0, n // 2, 97)]
    lines.append("M " + " ".join(str(2 * i) for i in range(n // 2)))
    lines += ["DETECTOR rec[-%d] rec[-%d]" % (k + 1, k + 1 + n // 2) for k in range(0, n // 2, 101)]
    lines.append("OBSERVABLE_INCLUDE(0) rec[-1] rec[-2]")
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("mode", [0, 1])
def test_circuit_too_large_for_shared_memory_matches_oracle(mode):
    # Frames in a per-CTA global region (one block per CTA); bit-exact against the oracle in both noise modes.
    text = _wide_circuit()
    c = stim_gb300.Circuit(text)
    assert c.program_info()["smem_bytes_per_block"] > 227 * 1024
    s = c.compile_detector_sampler(seed=17)
    s.set_noise_mode(mode)
    shots = 1500
    gd, go = s.sample(shots, separate_observables=True, bit_packed=True)
    od, oo, _ = OracleCircuit(text).sample(shots, 17, threads=8)
    np.testing.assert_array_equal(gd, od)
    np.testing.assert_array_equal(go, oo)
    assert gd.any()


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("name", golden_names())
def test_both_frame_kernels_match_golden(name, kernel):
    # Hit-list noise through the generic frame kernel (0) and the lean one (1, used by default wherever the
    # program has a lean phase list); both must reproduce the reference's goldens bit for bit.
    g = load(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_detector_sampler(seed=int(g["seed"]))
    s.set_noise_mode(1)
    s.set_frame_kernel(kernel)
    d, o = s.sample(int(g["shots"]), separate_observables=True, bit_packed=True)
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])
    m = c.compile_sampler(skip_reference_sample=True, seed=int(g["seed"]))
    m.set_noise_mode(1)
    m.set_frame_kernel(kernel)
    np.testing.assert_array_equal(m.sample(int(g["shots"]), bit_packed=True), g["meas"])
    if kernel == 0:
        assert s.launch_shape()["kernel"] == "generic"


def test_lean_kernel_is_used_for_generated_codes():
    for family, d in [("surface_code:rotated_memory_z", 25), ("repetition_code:memory", 9),
                      ("color_code:memory_xyz", 5)]:
        s = stim_gb300.Circuit(workloads.code_circuit(family, d, d, 0.001)).compile_detector_sampler(seed=1)
        assert s.launch_shape()["kernel"] == "lean", family


@pytest.mark.parametrize("shape", [(1, 128), (1, 256), (2, 128), (4, 256)])
def test_lean_kernel_shapes_match_oracle(shape):
    text = workloads.code_circuit("surface_code:rotated_memory_x", 11, 11, 0.005)
    s = stim_gb300.Circuit(text).compile_detector_sampler(seed=4)
    s.set_launch_shape(*shape)
    assert s.launch_shape()["kernel"] == "lean"
    gd, go = s.sample(20000, separate_observables=True, bit_packed=True)
    od, oo, _ = OracleCircuit(text).sample(20000, 4, threads=_THREADS)
    np.testing.assert_array_equal(gd, od)
    np.testing.assert_array_equal(go, oo)
