"""Detector error models on the CPU: the oracle's and the library's parsers against the counts the reference's
own CLI reports; the oracle's replay against the reference's `stim sample_dem --replay_err_in`; and the
oracle's contract sampling against the reference's native sampler within 5-sigma binomial bounds
(tests/golden/make_dem.py)."""

import glob
import os

import numpy as np
import pytest

import stim_gb300
from conftest import GOLDEN_DIR
from oracle.oracle import OracleDem
from stats_util import counts_from_packed, max_abs_z

DEM_DIR = os.path.join(GOLDEN_DIR, "dem")


def dem_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(DEM_DIR, "*.npz")))


def load_dem(name):
    return np.load(os.path.join(DEM_DIR, name + ".npz"))


@pytest.mark.parametrize("name", dem_cases())
def test_dem_counts_match_reference(name):
    g = load_dem(name)
    want = (int(g["num_detectors"]), int(g["num_observables"]), int(g["num_errors"]))
    o = OracleDem(str(g["model"]))
    assert (o.num_detectors, o.num_observables, o.num_errors) == want
    m = stim_gb300.DetectorErrorModel(str(g["model"]))  # host-only parse in the library
    assert (m.num_detectors, m.num_observables, m.num_errors) == want


@pytest.mark.parametrize("name", dem_cases())
def test_oracle_dem_replay_matches_reference(name):
    g = load_dem(name)
    d, o, e = OracleDem(str(g["model"])).sample(g["replay"].shape[0], errors=True, replay=g["replay"])
    np.testing.assert_array_equal(d, g["dets"])
    np.testing.assert_array_equal(o, g["obs"])
    np.testing.assert_array_equal(e, g["replay"])


@pytest.mark.parametrize("name", dem_cases())
def test_oracle_dem_rates_match_reference_sampler(name):
    g = load_dem(name)
    n = 1 << 16
    m = OracleDem(str(g["model"]))
    d, o, _ = m.sample(n, 99)
    dz = max_abs_z(g["det_counts"], int(g["rate_shots"]), counts_from_packed(d, m.num_detectors), n)
    oz = max_abs_z(g["obs_counts"], int(g["rate_shots"]), counts_from_packed(o, m.num_observables), n)
    assert dz < 5.0 and oz < 5.0, (dz, oz)


def test_dem_parse_errors():
    for bad in ["error(1.5) D0", "error(0.1) ^ D0", "error(0.1) D0 ^ ^ D1", "detector L0", "repeat 2 {\nerror(0.1) D0",
                "}", "fault(0.1) D0", "logical_observable D0"]:
        with pytest.raises((ValueError, IndexError)):
            stim_gb300.DetectorErrorModel(bad)
