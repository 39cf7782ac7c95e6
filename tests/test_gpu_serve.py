"""Request server: continuous batching, device-resident circuit cache, and result identity between a
request served alone and the same request served in a mix (bit-exact: tolerance zero)."""

import random
import threading
import time

import numpy as np
import pytest

import stim_gb300
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu


def _mix(seed, n):
    rng = random.Random(seed)
    fams = [("surface_code:rotated_memory_x", [3, 5, 7, 9]), ("repetition_code:memory", [3, 9, 25]),
            ("color_code:memory_xyz", [3, 5, 7]), ("surface_code:rotated_memory_z", [3, 5, 11])]
    out = []
    for _ in range(n):
        fam, ds = fams[rng.randrange(len(fams))]
        d = ds[rng.randrange(len(ds))]
        p = float(f"{10 ** rng.uniform(-4, -2):.3g}")
        shots = int(10 ** rng.uniform(1, 4.3))
        out.append((workloads.code_circuit(fam, d, d, p), shots, rng.randrange(1 << 40)))
    return out


def _alone(text, shots, seed, **kw):
    return stim_gb300.Circuit(text).compile_detector_sampler(seed=seed).sample(shots, **kw)


def test_served_results_equal_alone_results():
    reqs = _mix(1, 40)
    with stim_gb300.Server(max_chunk_shots=1024) as sv:
        results = [None] * len(reqs)

        def client(idx):
            rng = random.Random(idx)
            for k in range(idx, len(reqs), 4):
                text, shots, seed = reqs[k]
                time.sleep(rng.uniform(0, 0.003))
                results[k] = sv.submit(text, shots, seed=seed, bit_packed=True, separate_observables=True)

        threads = [threading.Thread(target=client, args=(i,)) for i in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        outs = [r.result() for r in results]
        st = sv.stats()
    for (text, shots, seed), (d, o) in zip(reqs, outs):
        d0, o0 = _alone(text, shots, seed, bit_packed=True, separate_observables=True)
        np.testing.assert_array_equal(d, d0)
        np.testing.assert_array_equal(o, o0)
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["cache_hits"] + st["cache_misses"] == len(reqs)
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_continuous_batching_admits_arrivals_while_busy():
    big = workloads.code_circuit("surface_code:rotated_memory_z", 15, 15, 0.001)
    small = workloads.code_circuit("repetition_code:memory", 5, 5, 0.01)
    # A small memory budget spreads the big request over several batches (about four chunks each).
    with stim_gb300.Server(hbm_budget=128 << 20, max_chunk_shots=1 << 14) as sv:
        r_big = sv.submit(big, 1 << 18, seed=3, bit_packed=True, append_observables=True)
        time.sleep(0.002)
        r_small = [sv.submit(small, 500 + 100 * k, seed=k, append_observables=True) for k in range(8)]
        outs = [r.result() for r in r_small]
        d_big = r_big.result()
        st = sv.stats()
    assert st["batches"] > 2
    assert st["chunks_per_batch"] > 1.0
    # Small requests submitted after the big one finish before it: they joined batches while it ran.
    assert max(r.latency_ms for r in r_small) < r_big.latency_ms
    for k, out in enumerate(outs):
        np.testing.assert_array_equal(out, _alone(small, 500 + 100 * k, k, append_observables=True))
    np.testing.assert_array_equal(d_big, _alone(big, 1 << 18, 3, bit_packed=True, append_observables=True))


def test_server_device_destinations_and_errors():
    torch = pytest.importorskip("torch")
    text = workloads.code_circuit("surface_code:rotated_memory_x", 5, 5, 0.005)
    c = stim_gb300.Circuit(text)
    shots = 3000
    d = torch.zeros((shots, (c.num_detectors + 7) // 8), dtype=torch.uint8, device="cuda")
    o = torch.zeros((shots, 1), dtype=torch.uint8, device="cuda")
    with stim_gb300.Server(max_chunk_shots=1024) as sv:
        r = sv.submit_device(text, shots, seed=11, dets_ptr=d.data_ptr(), dets_stride=d.shape[1],
                             obs_ptr=o.data_ptr(), obs_stride=1)
        r.result()
        z = sv.submit(text, 0, seed=1, bit_packed=True)
        assert z.result().shape == (0, (c.num_detectors + 7) // 8)
        with pytest.raises(ValueError):
            sv.submit("NOT_A_GATE 0\n", 10, seed=1)
    d0, o0 = _alone(text, shots, 11, bit_packed=True, separate_observables=True)
    np.testing.assert_array_equal(d.cpu().numpy(), d0)
    np.testing.assert_array_equal(o.cpu().numpy(), o0)


def test_oversized_circuit_is_rejected_alone():
    # A circuit whose frames exceed shared memory fails at submission; the requests around it are served.
    from test_gpu_parity import _wide_circuit

    small = workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.01)
    with stim_gb300.Server(device=0) as server:
        a = server.submit(small, 5000, seed=1, bit_packed=True)
        with pytest.raises(ValueError, match="too large for the server"):
            server.submit(_wide_circuit(), 1000, seed=2, bit_packed=True).result()
        b = server.submit(small, 5000, seed=3, bit_packed=True)
        want_a = stim_gb300.Circuit(small).compile_detector_sampler(seed=1).sample(5000, bit_packed=True)
        np.testing.assert_array_equal(a.result(), want_a)
        assert b.result().shape == want_a.shape
        k = server.counters()
        assert (k["submitted"], k["rejected"], k["completed"], k["failed"]) == (2, 1, 2, 0)
        assert k["queued"] == 0 and k["pending"] == 0 and k["chunks_admitted"] >= 2
