"""Native-RNG GPU runs against the reference's own CPU sampler: per-detector and per-observable flip rates
agree within 5-sigma binomial bounds (2^18 shots each side), and noiseless circuits fire nothing."""

import numpy as np
import pytest

import stim_gb300
from stats_util import counts_from_packed, load_rates, max_abs_z, rate_cases
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", rate_cases())
def test_gpu_rates_match_reference_sampler(name, mode):
    g = load_rates(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    n = int(g["shots"])
    s = c.compile_detector_sampler(seed=987654321 + mode)
    s.set_noise_mode(mode)
    d, o = s.sample(n, bit_packed=True, separate_observables=True)
    dz = max_abs_z(g["det_counts"], n, counts_from_packed(d, c.num_detectors), n)
    oz = max_abs_z(g["obs_counts"], n, counts_from_packed(o, c.num_observables), n)
    assert dz < 5.0 and oz < 5.0, (dz, oz)


def test_noiseless_d11_gives_no_detection_events_at_2_20_shots():
    c = stim_gb300.Circuit(workloads.code_circuit("surface_code:rotated_memory_x", 11, 11, 0.0))
    d, o = c.compile_detector_sampler(seed=5).sample(1 << 20, bit_packed=True, separate_observables=True)
    assert not d.any() and not o.any()
