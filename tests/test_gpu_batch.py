"""Batched sampling (many circuits in one persistent launch, replayed as a CUDA graph) and the launch-shape
autotuners: every bit equals what the circuits' own samplers return one call at a time, which the other
GPU tests tie to the reference's goldens and the oracle."""

import os

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu

MIX = [
    ("surface_rz_d3_r3_p0.001", 4096),
    ("surface_rx_d5_r5_p0.01", 1000),
    ("rep_d9_r9_p0.02", 0),
    ("color_d5_r5_p0.01", 1024),
    ("all_gates_s5", 333),
    ("feedback", 1024),
    ("random_clifford_n128_d200_s3", 256),
    ("surface_rx_d11_r11_p0.005", 512),
]


def load(name):
    return dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))


def make(names_shots):
    out = []
    for name, shots in names_shots:
        g = load(name)
        out.append((stim_gb300.Circuit(str(g["circuit"])), int(g["seed"]), shots, g))
    return out


def singles(items, calls):
    res = []
    samplers = [c.compile_detector_sampler(seed=seed) for c, seed, _, _ in items]
    for _ in range(calls):
        res.append([s.sample(shots, bit_packed=True, separate_observables=True)
                    for s, (_, _, shots, _) in zip(samplers, items)])
    return res


def test_batch_matches_single_samplers_and_goldens():
    items = make(MIX)
    batch = stim_gb300.BatchSampler([c.compile_detector_sampler(seed=seed) for c, seed, _, _ in items])
    shots = [s for _, _, s, _ in items]
    got = [batch.sample(shots, bit_packed=True, separate_observables=True) for _ in range(3)]
    want = singles(items, 3)
    for call in range(3):
        for j in range(len(items)):
            np.testing.assert_array_equal(got[call][j][0], want[call][j][0])
            np.testing.assert_array_equal(got[call][j][1], want[call][j][1])
    # First call from a fresh sampler = the reference's golden shots.
    for j, (_, _, n, g) in enumerate(items):
        k = min(n, int(g["shots"]))
        np.testing.assert_array_equal(got[0][j][0][:k], g["dets"][:k])
        np.testing.assert_array_equal(got[0][j][1][:k], g["obs"][:k])
    t = batch.last_timings()
    assert t["graph_launches"] == 3 and t["graph_builds"] == 1


@pytest.mark.parametrize("shape", [(1, 256, 0), (1, 128, 1), (2, 256, -1), (4, 256, 1)])
def test_batch_launch_shapes_do_not_change_results(shape):
    items = make(MIX)
    batch = stim_gb300.BatchSampler([c.compile_detector_sampler(seed=seed) for c, seed, _, _ in items])
    try:
        batch.set_launch_shape(*shape)
    except ValueError:
        pytest.skip("shape does not fit the largest circuit")
    shots = [s for _, _, s, _ in items]
    got = batch.sample(shots, bit_packed=False, append_observables=True)
    want = [c.compile_detector_sampler(seed=seed).sample(n, append_observables=True) for c, seed, n, _ in items]
    for a, b in zip(got, want):
        np.testing.assert_array_equal(a, b)


def test_batch_repeated_sampler_continues_stream():
    g = load("surface_rz_d3_r3_p0.001")
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_detector_sampler(seed=int(g["seed"]))
    batch = stim_gb300.BatchSampler([s, s, s])
    got = batch.sample([1000, 1500, 1596], bit_packed=True, separate_observables=True)
    d = np.concatenate([x[0] for x in got])
    o = np.concatenate([x[1] for x in got])
    # 1000 shots occupy 8 blocks of 128; the next entry starts at shot 1024 like a second sample() call.
    ref = c.compile_detector_sampler(seed=int(g["seed"]))
    parts = [ref.sample(n, bit_packed=True, separate_observables=True) for n in (1000, 1500, 1596)]
    np.testing.assert_array_equal(d, np.concatenate([p[0] for p in parts]))
    np.testing.assert_array_equal(o, np.concatenate([p[1] for p in parts]))
    np.testing.assert_array_equal(got[0][0], g["dets"][:1000])


def test_batch_autotune_and_device_outputs():
    torch = pytest.importorskip("torch")
    wl = workloads.batched_workload(num_circuits=12, seed=5, d_choices=(3, 5, 7, 9), shots_hi=1 << 14)
    circuits = [stim_gb300.Circuit(w["text"]) for w in wl]
    batch = stim_gb300.BatchSampler([c.compile_detector_sampler(seed=w["seed"]) for c, w in zip(circuits, wl)])
    shots = [w["shots"] for w in wl]
    ms = batch.autotune(shots)
    assert ms > 0
    bufs = [torch.zeros((n, (c.num_detectors + 7) // 8), dtype=torch.uint8, device="cuda")
            for n, c in zip(shots, circuits)]
    obufs = [torch.zeros((n, 1), dtype=torch.uint8, device="cuda") for n in shots]
    batch.sample_device(shots, [b.data_ptr() for b in bufs], [b.shape[1] for b in bufs],
                        [b.data_ptr() for b in obufs], [1] * len(obufs))
    torch.cuda.synchronize()
    for c, w, b, ob in zip(circuits, wl, bufs, obufs):
        d, o = c.compile_detector_sampler(seed=w["seed"]).sample(w["shots"], bit_packed=True,
                                                                  separate_observables=True)
        np.testing.assert_array_equal(b.cpu().numpy(), d)
        np.testing.assert_array_equal(ob.cpu().numpy(), o)


def test_sampler_autotune_keeps_results():
    g = load("surface_rx_d11_r11_p0.005")
    c = stim_gb300.Circuit(str(g["circuit"]))
    s = c.compile_detector_sampler(seed=int(g["seed"]))
    ms = s.autotune(1 << 14)
    assert ms > 0
    d, o = s.sample(int(g["shots"]), bit_packed=True, separate_observables=True)
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])


def test_batch_hit_list_overflow_falls_back_to_inline_noise():
    from stim_gb300 import _native

    items = make(MIX)
    samplers = [c.compile_detector_sampler(seed=seed) for c, seed, _, _ in items]
    for s in samplers:
        _native.check(_native.lib().gfs_sampler_set_hit_capacity(s._h, 2))  # far below the expected hits
    batch = stim_gb300.BatchSampler(samplers)
    shots = [s for _, _, s, _ in items]
    got = [batch.sample(shots, bit_packed=True, separate_observables=True) for _ in range(2)]
    want = singles(items, 2)
    for call in range(2):
        for j in range(len(items)):
            np.testing.assert_array_equal(got[call][j][0], want[call][j][0])
            np.testing.assert_array_equal(got[call][j][1], want[call][j][1])
