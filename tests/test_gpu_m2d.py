"""The CUDA measurements-to-detection-events converter (through the C ABI) against the reference CLI's
`stim m2d` outputs, in every output layout; plus a size-independent property at scale: converting the
GPU measurement sampler's records gives exactly the GPU detection sampler's events for the same seed
(both follow the same random-bit contract)."""

import numpy as np
import pytest

import stim_gb300
from stim_gb300 import workloads
from test_m2d_oracle import load_m2d, m2d_cases, split_appended, unpack

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", m2d_cases())
def test_m2d_matches_reference_cli_in_every_layout(name):
    g = load_m2d(name)
    D, O = int(g["num_detectors"]), int(g["num_observables"])
    c = stim_gb300.Circuit(str(g["circuit"]))
    conv = c.compile_m2d_converter()
    meas = g["meas"]
    want_d, want_o = split_appended(g["out"], D, O)
    # Appended, bit-packed: byte-identical to the reference's b8 output.
    out = conv.convert(measurements=meas, append_observables=True, bit_packed=True)
    np.testing.assert_array_equal(out, g["out"])
    # Separate, unpacked bool.
    d, o = conv.convert(measurements=meas, separate_observables=True, append_observables=False)
    assert d.dtype == np.bool_ and d.shape == (meas.shape[0], D)
    np.testing.assert_array_equal(d, want_d)
    np.testing.assert_array_equal(o, want_o)
    # Detectors only, from bool measurement input.
    mb = unpack(meas, c.num_measurements)
    d = conv.convert(measurements=mb, separate_observables=False, append_observables=False, bit_packed=True)
    np.testing.assert_array_equal(unpack(d, D), want_d)


@pytest.mark.parametrize("name", m2d_cases())
def test_m2d_skip_reference_sample_matches_reference_cli(name):
    g = load_m2d(name)
    c = stim_gb300.Circuit(str(g["circuit"]))
    out = c.compile_m2d_converter(skip_reference_sample=True).convert(
        measurements=g["meas"], append_observables=True, bit_packed=True)
    np.testing.assert_array_equal(out, g["out_skip"])


def test_m2d_argument_errors_match_reference():
    c = stim_gb300.Circuit("M 0 1\nDETECTOR rec[-1]\nOBSERVABLE_INCLUDE(0) rec[-2]")
    conv = c.compile_m2d_converter()
    with pytest.raises(ValueError, match="explicitly specify"):
        conv.convert(measurements=np.zeros((3, 2), dtype=np.bool_))
    with pytest.raises(ValueError):
        conv.convert(measurements=np.zeros((3, 3), dtype=np.bool_), append_observables=False)
    assert conv.convert(measurements=np.zeros((0, 2), dtype=np.bool_), append_observables=True).shape == (0, 2)


def test_m2d_ignores_zero_sweep_bits_and_rejects_others_on_swept_circuits():
    c = stim_gb300.Circuit("CX sweep[0] 0\nM 0\nDETECTOR rec[-1]")
    conv = c.compile_m2d_converter()
    meas = np.array([[0], [1]], dtype=np.uint8)
    zero = np.zeros((2, 1), dtype=np.uint8)
    d = conv.convert(measurements=meas, sweep_bits=zero, append_observables=False, bit_packed=True)
    np.testing.assert_array_equal(d, meas)
    with pytest.raises(ValueError, match="sweep"):
        conv.convert(measurements=meas, sweep_bits=np.ones((2, 1), dtype=np.uint8), append_observables=False)


@pytest.mark.parametrize("family,d,p,shots", [
    ("surface_code:rotated_memory_z", 25, 0.001, 1 << 17),
    ("surface_code:rotated_memory_x", 11, 0.005, 1 << 18),
    ("color_code:memory_xyz", 7, 0.01, 100_003),
])
def test_m2d_of_sampled_measurements_equals_detection_sampler(family, d, p, shots):
    text = workloads.code_circuit(family, d, d, p)
    c = stim_gb300.Circuit(text)
    meas = c.compile_sampler(seed=123).sample(shots, bit_packed=True)
    got_d, got_o = c.compile_m2d_converter().convert(measurements=meas, separate_observables=True,
                                                     append_observables=False, bit_packed=True)
    want_d, want_o = c.compile_detector_sampler(seed=123).sample(shots, separate_observables=True, bit_packed=True)
    np.testing.assert_array_equal(got_d, want_d)
    np.testing.assert_array_equal(got_o, want_o)
    assert got_d.any()
