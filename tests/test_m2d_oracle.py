"""The oracle's measurements-to-detection-events restatement against outputs of the reference's own CLI
(`stim m2d --append_observables`, with and without --skip_reference_sample; tests/golden/make_m2d.py)."""

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR
from oracle.oracle import OracleCircuit

M2D_DIR = os.path.join(GOLDEN_DIR, "m2d")


def m2d_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(M2D_DIR, "*.npz")))


def load_m2d(name):
    return np.load(os.path.join(M2D_DIR, name + ".npz"))


def split_appended(packed, D, O):
    """Appended detector + observable rows -> (detector bits, observable bits) as bool arrays."""
    bits = np.unpackbits(packed, axis=1, bitorder="little")[:, :D + O].astype(bool)
    return bits[:, :D], bits[:, D:]


def unpack(packed, n):
    return np.unpackbits(packed, axis=1, bitorder="little")[:, :n].astype(bool)


@pytest.mark.parametrize("skip", [False, True])
@pytest.mark.parametrize("name", m2d_cases())
def test_oracle_m2d_matches_reference_cli(name, skip):
    g = load_m2d(name)
    D, O = int(g["num_detectors"]), int(g["num_observables"])
    c = OracleCircuit(str(g["circuit"]))
    d, o = c.m2d(g["meas"], None if skip else g["ref_sample"])
    want_d, want_o = split_appended(g["out_skip" if skip else "out"], D, O)
    np.testing.assert_array_equal(unpack(d, D), want_d)
    np.testing.assert_array_equal(unpack(o, O), want_o)


def test_m2d_fixtures_cover_sampled_and_random_rows():
    assert len(m2d_cases()) >= 8
    g = load_m2d("surface_rz_d3_r3")
    D, O = int(g["num_detectors"]), int(g["num_observables"])
    d, _ = split_appended(g["out"], D, O)
    half = d.shape[0] // 2
    assert d[:half].mean() < 0.1  # sampled rows: few detection events
    assert 0.3 < d[half:].mean() < 0.7  # random rows: about half


M2D_SWEEP_DIR = os.path.join(GOLDEN_DIR, "m2d_sweep")


def m2d_sweep_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(M2D_SWEEP_DIR, "*.npz")))


def load_m2d_sweep(name):
    return np.load(os.path.join(M2D_SWEEP_DIR, name + ".npz"))


@pytest.mark.parametrize("name", m2d_sweep_cases())
def test_sweep_fixtures_agree_with_oracle_where_sweep_bits_are_zero(name):
    # The oracle's converter has no sweep data; on the shots whose sweep rows are all zero the reference's
    # sweep-aware output must equal it (pins the fixtures' measurement / reference-sample side).
    g = load_m2d_sweep(name)
    D, O = int(g["num_detectors"]), int(g["num_observables"])
    zero = ~g["sweep"].any(axis=1)
    assert zero.sum() >= 7
    d, o = OracleCircuit(str(g["circuit"])).m2d(g["meas"][zero], g["ref_sample"])
    want_d, want_o = split_appended(g["out"][zero], D, O)
    np.testing.assert_array_equal(unpack(d, D), want_d)
    np.testing.assert_array_equal(unpack(o, O), want_o)
    # And the sweep data matters on the other shots (the fixtures exercise it).
    dd, oo = OracleCircuit(str(g["circuit"])).m2d(g["meas"][~zero], g["ref_sample"])
    got = np.concatenate([unpack(dd, D), unpack(oo, O)], axis=1)
    assert (got != np.concatenate(split_appended(g["out"][~zero], D, O), axis=1)).any()
