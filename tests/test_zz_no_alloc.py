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
