"""The random-bit contract's noise matches the reference's native sampler in distribution: per-detector and
per-observable flip rates of the CPU oracle (same contract as the GPU kernels) against counts from the
reference's own `stim detect` (its mt19937_64 stream), within 5 sigma."""

import pytest

from oracle.oracle import OracleCircuit
from stats_util import counts_from_packed, load_rates, max_abs_z, rate_cases

SHOTS = 1 << 14


@pytest.mark.parametrize("name", rate_cases())
def test_oracle_rates_match_reference_sampler(name):
    g = load_rates(name)
    c = OracleCircuit(str(g["circuit"]))
    d, o, _ = c.sample(SHOTS, 1234, threads=4)
    dz = max_abs_z(g["det_counts"], int(g["shots"]), counts_from_packed(d, c.num_detectors), SHOTS)
    oz = max_abs_z(g["obs_counts"], int(g["shots"]), counts_from_packed(o, c.num_observables), SHOTS)
    assert dz < 5.0 and oz < 5.0, (dz, oz)
