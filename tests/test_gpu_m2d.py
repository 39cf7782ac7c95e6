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


def test_m2d_sweep_bit_flips_the_results_it_controls():
    c = stim_gb300.Circuit("CX sweep[0] 0\nM 0\nDETECTOR rec[-1]")
    conv = c.compile_m2d_converter()
    meas = np.array([[0], [1]], dtype=np.uint8)
    zero = np.zeros((2, 1), dtype=np.uint8)
    d = conv.convert(measurements=meas, sweep_bits=zero, append_observables=False, bit_packed=True)
    np.testing.assert_array_equal(d, meas)
    d = conv.convert(measurements=meas, sweep_bits=np.ones((2, 1), dtype=np.uint8), append_observables=False,
                     bit_packed=True)
    np.testing.assert_array_equal(d, meas ^ 1)


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


from test_m2d_oracle import load_m2d_sweep, m2d_sweep_cases  # noqa: E402


@pytest.mark.parametrize("name", m2d_sweep_cases())
def test_m2d_sweep_bits_match_reference_cli(name):
    g = load_m2d_sweep(name)
    D, O, S = int(g["num_detectors"]), int(g["num_observables"]), int(g["num_sweep_bits"])
    c = stim_gb300.Circuit(str(g["circuit"]))
    conv = c.compile_m2d_converter()
    assert conv.num_sweep_bits == S
    out = conv.convert(measurements=g["meas"], sweep_bits=g["sweep"], append_observables=True, bit_packed=True)
    np.testing.assert_array_equal(out, g["out"])
    # Bool sweep input, separate observables.
    want_d, want_o = split_appended(g["out"], D, O)
    d, o = conv.convert(measurements=g["meas"], sweep_bits=unpack(g["sweep"], S), separate_observables=True,
                        append_observables=False)
    np.testing.assert_array_equal(d, want_d)
    np.testing.assert_array_equal(o, want_o)


def _swept_circuit():
    text = workloads.code_circuit("surface_code:rotated_memory_x", 7, 7, 0.005)
    lines = text.splitlines()
    out = []
    for k, line in enumerate(lines):
        out.append(line)
        if line.strip().startswith(("CX ", "H ")) and k % 2 == 0:
            out.append(f"CX sweep[{k % 11}] {k % 97}")
            out.append(f"CZ sweep[{(k + 3) % 11}] {(k * 7) % 97}")
    return "\n".join(out) + "\n"


def test_m2d_sweep_is_affine_at_scale():
    # Over GF(2) the conversion is affine in (measurements, sweep bits):
    # out(m, s) = out(m, 0) ^ out(0, s) ^ out(0, 0).  150,000 shots take three converter chunks.
    c = stim_gb300.Circuit(_swept_circuit())
    conv = c.compile_m2d_converter()
    S = conv.num_sweep_bits
    assert S == 11
    shots = 150_000
    rng = np.random.default_rng(8)
    m = rng.integers(0, 256, (shots, (c.num_measurements + 7) // 8), dtype=np.uint8)
    s = rng.integers(0, 256, (shots, (S + 7) // 8), dtype=np.uint8)
    s[:, -1] &= (1 << (S % 8)) - 1
    zm, zs = np.zeros_like(m), np.zeros_like(s)

    def conv_(mm, ss):
        return conv.convert(measurements=mm, sweep_bits=ss, append_observables=True, bit_packed=True)

    ms, m0, s0, z = conv_(m, s), conv_(m, zs), conv_(zm, s), conv_(zm, zs)
    np.testing.assert_array_equal(ms, m0 ^ s0 ^ z)
    assert (s0 != z).any()   # the sweep bits flip something
    # Zero sweep data is the same as none.
    np.testing.assert_array_equal(m0, conv.convert(measurements=m, append_observables=True, bit_packed=True))


from test_m2d_files import FORMATS, OUT_FORMATS, file_cases, load_files  # noqa: E402


@pytest.mark.parametrize("name", file_cases())
def test_convert_file_matches_reference_cli_in_every_format(name, tmp_path):
    g = load_files(name)
    conv = stim_gb300.Circuit(str(g["circuit"])).compile_m2d_converter()
    swept = bool(g["has_sweep"])
    for fin in FORMATS:
        meas = tmp_path / f"m.{fin}"
        g[f"meas_{fin}"].tofile(meas)
        sweep = None
        if swept:
            sweep = tmp_path / f"s.{fin}"
            g[f"sweep_{fin}"].tofile(sweep)
        for fout in OUT_FORMATS:
            out, det, obs = tmp_path / "o", tmp_path / "d", tmp_path / "l"
            conv.convert_file(measurements_filepath=meas, measurements_format=fin, sweep_bits_filepath=sweep,
                              sweep_bits_format=fin, detection_events_filepath=out, detection_events_format=fout,
                              append_observables=True)
            assert out.read_bytes() == g[f"out_{fout}"].tobytes(), (fin, fout)
            conv.convert_file(measurements_filepath=meas, measurements_format=fin, sweep_bits_filepath=sweep,
                              sweep_bits_format=fin, detection_events_filepath=det, detection_events_format=fout,
                              obs_out_filepath=obs, obs_out_format=fout)
            assert det.read_bytes() == g[f"det_{fout}"].tobytes(), (fin, fout)
            assert obs.read_bytes() == g[f"obs_{fout}"].tobytes(), (fin, fout)
    with pytest.raises(ValueError, match="SAMPLE_FORMAT_PTB64 incompatible"):
        conv.convert_file(measurements_filepath=tmp_path / "m.b8", measurements_format="b8",
                          detection_events_filepath=tmp_path / "x", detection_events_format="ptb64")
    with pytest.raises(ValueError, match="Failed to open"):
        conv.convert_file(measurements_filepath=tmp_path / "missing.b8", measurements_format="b8",
                          detection_events_filepath=tmp_path / "x")


def test_convert_file_sweep_record_count_must_match(tmp_path):
    c = stim_gb300.Circuit("CX sweep[0] 0\nM 0\nDETECTOR rec[-1]")
    conv = c.compile_m2d_converter()
    (tmp_path / "m.01").write_text("0\n1\n1\n")
    (tmp_path / "s.01").write_text("1\n1\n")
    with pytest.raises(ValueError, match="different number of shots"):
        conv.convert_file(measurements_filepath=tmp_path / "m.01", sweep_bits_filepath=tmp_path / "s.01",
                          detection_events_filepath=tmp_path / "o.01")
    (tmp_path / "s.01").write_text("1\n0\n1\n")
    conv.convert_file(measurements_filepath=tmp_path / "m.01", sweep_bits_filepath=tmp_path / "s.01",
                      detection_events_filepath=tmp_path / "o.01")
    assert (tmp_path / "o.01").read_text() == "1\n1\n0\n"
