"""Sharding one shot stream by shot range on the GPU: samplers whose stream positions come from
stim_gb300.shard_range reproduce, concatenated, a single sampler's shots (what each rank of bench.py under
torchrun does, one GPU at a time here)."""

import numpy as np
import pytest

import stim_gb300
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3, 8])
def test_shards_reproduce_one_stream(world):
    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_x", 7, 7, 0.005))
    total = 100_000
    want, want_o = c.compile_detector_sampler(seed=77).sample(total, bit_packed=True, separate_observables=True)
    parts, parts_o = [], []
    for rank in range(world):
        first, n = stim_gb300.shard_range(total, rank, world)
        s = c.compile_detector_sampler(seed=77)
        s.set_stream_position(first)
        d, o = s.sample(n, bit_packed=True, separate_observables=True)
        assert s.stream_position() == first + (n + 127) // 128 * 128
        parts.append(d)
        parts_o.append(o)
    np.testing.assert_array_equal(np.concatenate(parts), want)
    np.testing.assert_array_equal(np.concatenate(parts_o), want_o)


def test_stream_position_must_be_block_aligned():
    s = stim_gb300.Circuit("X_ERROR(0.1) 0\nM 0\nDETECTOR rec[-1]").compile_detector_sampler(seed=1)
    with pytest.raises(ValueError):
        s.set_stream_position(100)
