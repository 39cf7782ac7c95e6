"""The reference's DEM sampler unit tests, restated against this package (src/stim/simulators/dem_sampler.test.cc:
24-48 basic_sizing, :50-75 resample_basic_probabilities, :77-102 resample_combinations): empty and declaration-only
models sample nothing; each mechanism fires at its probability (0, 1 and the ranges in between), a mechanism's
symptoms fire together (D1 with L0, D4 with D5 across the `^` separator), and three mechanisms over three detectors
keep the parity of the detectors even.  The oracle on the CPU, the GPU sampler on the GB300, twice each (as the
reference resamples twice)."""

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleDem

BASIC = "error(0) D0\nerror(0.25) D1 L0\nerror(0.5) D2\nerror(0.75) D3\nerror(1) D4 ^ D5"
COMBINATIONS = "error(0.1) D0 D1\nerror(0.2) D1 D2\nerror(0.3) D2 D0"
SIZING = [("", 700, 0, 0), ("logical_observable L2000\ndetector D1000", 200, 1001, 2001)]


def unpack(a, n):
    return np.unpackbits(a, axis=1, bitorder="little")[:, :n].astype(np.bool_)


def oracle_sample(text, shots, seed):
    m = OracleDem(text)
    d, o, _ = m.sample(shots, seed)
    return unpack(d, m.num_detectors), unpack(o, m.num_observables)


def gpu_sample(text, shots, seed):
    d, o = stim_gb300.DetectorErrorModel(text).compile_sampler(seed=seed).sample(shots)[:2]
    return d, o


def check_sizing(sample, text, shots, nd, no):
    d, o = sample(text, shots, 3)
    assert d.shape == (shots, nd) and o.shape == (shots, no)
    assert not d.any() and not o.any()


def check_basic(d, o):
    n = d.shape[0]
    assert d[:, 0].sum() == 0
    assert 0 < d[:, 1].sum() < 500
    assert 250 < d[:, 2].sum() < 750
    assert 500 < d[:, 3].sum() < 1000
    assert d[:, 4].sum() == n
    np.testing.assert_array_equal(d[:, 1], o[:, 0])
    np.testing.assert_array_equal(d[:, 4], d[:, 5])


def check_combinations(d):
    assert 240 < d[:, 0].sum() < 440
    assert 160 < d[:, 1].sum() < 360
    assert 280 < d[:, 2].sum() < 480
    assert not (d[:, 0] ^ d[:, 1] ^ d[:, 2]).any()


@pytest.mark.parametrize("text,shots,nd,no", SIZING)
def test_oracle_sizing(text, shots, nd, no):
    check_sizing(oracle_sample, text, shots, nd, no)


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_basic_probabilities_and_combinations(seed):
    check_basic(*oracle_sample(BASIC, 1000, seed))
    check_combinations(oracle_sample(COMBINATIONS, 1000, seed)[0])


@pytest.mark.gpu
@pytest.mark.parametrize("text,shots,nd,no", SIZING)
def test_gpu_sizing(text, shots, nd, no):
    check_sizing(gpu_sample, text, shots, nd, no)


@pytest.mark.gpu
def test_gpu_basic_probabilities_and_combinations():
    basic = stim_gb300.DetectorErrorModel(BASIC).compile_sampler(seed=1)
    comb = stim_gb300.DetectorErrorModel(COMBINATIONS).compile_sampler(seed=1)
    for _ in range(2):
        check_basic(*basic.sample(1000)[:2])
        check_combinations(comb.sample(1000)[0])
