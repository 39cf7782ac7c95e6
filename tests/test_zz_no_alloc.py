"""The allocation-free detection entry point, gfs_sample_detections_device_noalloc.

That entry point is for callers that must not allocate or free device memory while they sample, for
example a real-time decoding loop whose HBM is reserved up front by its own pool allocator, or a loop
that cannot afford cudaMalloc's implicit synchronization.  Its scratch is a fixed 64 MiB device array
inside the library instead of cudaMalloc'd buffers.  These tests check, through the C ABI, that it gives
exactly the bits of the ordinary device entry point, on two calls in a row (the second continues the
random stream), and that a circuit too large for the fixed array is rejected with a clear error.

This file is collected last so that, if it fails, a run that stops at the first failure has already run
every other test.
"""

import os

import numpy as np
import pytest

import stim_gb300
from stim_gb300 import _native, workloads

pytestmark = pytest.mark.gpu


def _buffers(torch, shots, rows, cols_obs):
    dev = "cuda:0"
    return (torch.zeros((shots, rows), dtype=torch.uint8, device=dev),
            torch.zeros((shots, cols_obs), dtype=torch.uint8, device=dev))


def _call(entry, sampler, shots, flags, dets, obs):
    _native.check(entry(sampler._h, shots, flags, dets.data_ptr(), dets.stride(0),
                        obs.data_ptr(), obs.stride(0)))


@pytest.mark.parametrize("family,d,p,shots,flags", [
    # 40,000 shots of d=25 need two passes through the fixed array (it holds 268 blocks of 128 shots).
    ("surface_code:rotated_memory_z", 25, 0.001, 40000, _native.BIT_PACKED),
    ("surface_code:rotated_memory_x", 5, 0.01, 5000, _native.APPEND_OBSERVABLES),
    ("color_code:memory_xyz", 5, 0.02, 3000, _native.BIT_PACKED | _native.PREPEND_OBSERVABLES),
])
def test_noalloc_matches_existing_entry_point_on_two_calls(family, d, p, shots, flags):
    torch = pytest.importorskip("torch")
    L = _native.lib()
    circ = stim_gb300.Circuit(workloads.code_circuit(family, d, d, p))
    D, O = circ.num_detectors, circ.num_observables
    packed = bool(flags & _native.BIT_PACKED)
    nd = D + (O if flags & _native.PREPEND_OBSERVABLES else 0) + (O if flags & _native.APPEND_OBSERVABLES else 0)
    width = (lambda n: (n + 7) // 8) if packed else (lambda n: n)
    existing = circ.compile_detector_sampler(seed=1234)
    noalloc = circ.compile_detector_sampler(seed=1234)
    for call in range(2):
        da, oa = _buffers(torch, shots, width(nd), width(O))
        db, ob = _buffers(torch, shots, width(nd), width(O))
        _call(L.gfs_sample_detections_device, existing, shots, flags, da, oa)
        _call(L.gfs_sample_detections_device_noalloc, noalloc, shots, flags, db, ob)
        torch.cuda.synchronize()
        assert torch.equal(da, db), f"detection events differ on call {call}"
        assert torch.equal(oa, ob), f"observables differ on call {call}"
        assert int(da.sum()) > 0
    assert noalloc.last_timings()["frame_launches"] >= 1


def test_noalloc_rejects_circuits_beyond_its_fixed_scratch():
    torch = pytest.importorskip("torch")
    L = _native.lib()
    # 4.2 million detectors need 67.2 MB of scratch per 128-shot block, more than the 64 MiB array.
    circ = stim_gb300.Circuit("REPEAT 4200000 {\n    M 0\n    DETECTOR rec[-1]\n}\n")
    s = circ.compile_detector_sampler(seed=1)
    shots = 128
    dets, obs = _buffers(torch, shots, (circ.num_detectors + 7) // 8, 1)
    with pytest.raises(ValueError, match="allocation-free entry point holds"):
        _call(L.gfs_sample_detections_device_noalloc, s, shots, _native.BIT_PACKED, dets, obs)


def test_noalloc_matches_reference_fixture_at_distance_25():
    # The benchmarked circuit (distance 25, 25 rounds, p = 1e-3): the allocation-free entry point reproduces
    # the detection events and observable flips that the reference's own FrameSimulator produced on the same
    # injected random stream (tests/golden/surface_rz_d25_r25_p0.001.npz), on two calls in a row.
    torch = pytest.importorskip("torch")
    L = _native.lib()
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                  "surface_rz_d25_r25_p0.001.npz")))
    circ = stim_gb300.Circuit(str(g["circuit"]))
    s = circ.compile_detector_sampler(seed=int(g["seed"]))
    total = int(g["shots"])
    half = total // 2
    for k, (lo, hi) in enumerate([(0, half), (half, total)]):
        dets, obs = _buffers(torch, hi - lo, g["dets"].shape[1], g["obs"].shape[1])
        _call(L.gfs_sample_detections_device_noalloc, s, hi - lo, _native.BIT_PACKED, dets, obs)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(dets.cpu().numpy(), g["dets"][lo:hi], err_msg=f"call {k}")
        np.testing.assert_array_equal(obs.cpu().numpy(), g["obs"][lo:hi], err_msg=f"call {k}")


def test_noalloc_rejects_a_ring_that_needs_global_memory_and_later_calls_still_work():
    torch = pytest.importorskip("torch")
    L = _native.lib()
    # A lookback of 20,000 measurements: the ring (20,000 rows x 16 bytes per 128 shots) only fits in global
    # memory, which the allocation-free entry point does not use.
    text = "REPEAT 20000 {\n    X_ERROR(0.1) 0\n    M 0\n}\nDETECTOR rec[-1] rec[-20000]\n"
    circ = stim_gb300.Circuit(text)
    s = circ.compile_detector_sampler(seed=3)
    dets, obs = _buffers(torch, 256, 1, 1)
    with pytest.raises(ValueError, match="measurement ring does not fit in shared memory"):
        _call(L.gfs_sample_detections_device_noalloc, s, 256, _native.BIT_PACKED, dets, obs)
    # The rejected call leaves no CUDA error behind: the ordinary entry point still samples this circuit.
    _call(L.gfs_sample_detections_device, s, 256, _native.BIT_PACKED, dets, obs)
    torch.cuda.synchronize()
    assert int(dets.sum()) > 0
