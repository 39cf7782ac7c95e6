"""The CUDA detector-error-model sampler (through the C ABI): replayed errors against the reference CLI's
`stim sample_dem --replay_err_in`; contract sampling bit-exact against the oracle (errors included) and
continuing its stream across calls; native-RNG rates within 5 sigma of the reference's own sampler."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleDem
from stats_util import counts_from_packed, max_abs_z
from test_dem_oracle import dem_cases, load_dem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", dem_cases())
def test_dem_replay_matches_reference_cli(name):
    g = load_dem(name)
    s = stim_gb300.DetectorErrorModel(str(g["model"])).compile_sampler(seed=1)
    shots = g["replay"].shape[0]
    d, o, e = s.sample(shots, bit_packed=True, return_errors=True, recorded_errors_to_replay=g["replay"])
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])
    np.testing.assert_array_equal(e, g["replay"])
    # Unpacked replay input and output.
    E = s.num_errors
    eb = np.unpackbits(g["replay"], axis=1, bitorder="little")[:, :E].astype(bool)
    d2, o2, _ = s.sample(shots, recorded_errors_to_replay=eb)
    np.testing.assert_array_equal(d2, np.unpackbits(g["dets"], axis=1, bitorder="little")[:, :s.num_detectors])


@pytest.mark.parametrize("shots", [128, 1000, 70_000])
@pytest.mark.parametrize("name", dem_cases())
def test_dem_sampling_matches_oracle(name, shots):
    g = load_dem(name)
    text = str(g["model"])
    s = stim_gb300.DetectorErrorModel(text).compile_sampler(seed=42)
    d, o, e = s.sample(shots, bit_packed=True, return_errors=True)
    od, oo, oe = OracleDem(text).sample(shots, 42, errors=True)
    np.testing.assert_array_equal(d, od)
    np.testing.assert_array_equal(o, oo)
    np.testing.assert_array_equal(e, oe)
    # The next call continues the stream at the next 128-shot block.
    first = (shots + 127) // 128 * 128
    d2, o2, _ = s.sample(256, bit_packed=True)
    od2, oo2, _ = OracleDem(text).sample(256, 42, first_shot=first)
    np.testing.assert_array_equal(d2, od2)
    np.testing.assert_array_equal(o2, oo2)


def test_dem_probability_zero_and_one_are_exact():
    g = load_dem("hand")
    d, o, _ = stim_gb300.DetectorErrorModel(str(g["model"])).compile_sampler(seed=3).sample(4096)
    assert d[:, 4].all() and o[:, 2].all()   # error(1) D4 L2, nothing else touches them
    assert not d[:, 3].any()                 # error(0) D3


@pytest.mark.parametrize("name", dem_cases())
def test_dem_rates_match_reference_sampler(name):
    g = load_dem(name)
    n = 1 << 18
    s = stim_gb300.DetectorErrorModel(str(g["model"])).compile_sampler(seed=2024)
    d, o, _ = s.sample(n, bit_packed=True)
    dz = max_abs_z(g["det_counts"], int(g["rate_shots"]), counts_from_packed(d, s.num_detectors), n)
    oz = max_abs_z(g["obs_counts"], int(g["rate_shots"]), counts_from_packed(o, s.num_observables), n)
    assert dz < 5.0 and oz < 5.0, (dz, oz)
