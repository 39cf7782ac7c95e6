"""The reference's own Python tests of the DEM sampler (src/stim/simulators/dem_sampler_pybind_test.py), restated
against this package: sampling with recorded errors replayed, sample_write with error files and replay from a
file, and the observable array filled."""

import numpy as np
import pytest

import stim_gb300

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bit_packed", [False, True])
def test_dem_sampler_sample(bit_packed):
    s = stim_gb300.DetectorErrorModel("error(0.125) D0\nerror(0.25) D1").compile_sampler()
    d, o, e = s.sample(shots=100, return_errors=True, bit_packed=bit_packed)
    rd, ro, _ = s.sample(shots=100, recorded_errors_to_replay=e, bit_packed=bit_packed)
    np.testing.assert_array_equal(d, rd)
    np.testing.assert_array_equal(o, ro)


def test_dem_sampler_sample_write(tmp_path):
    s = stim_gb300.DetectorErrorModel("""
       error(0) D0
       error(0) D1
       error(0) D0
       error(1) D1 D2 L0
       error(0) D0
    """).compile_sampler()
    s.sample_write(shots=1, det_out_file=tmp_path / "dets.01", det_out_format="01", obs_out_file=tmp_path / "obs.01",
                   obs_out_format="01", err_out_file=tmp_path / "err.hits", err_out_format="hits")
    assert (tmp_path / "dets.01").read_text() == "011\n"
    assert (tmp_path / "obs.01").read_text() == "1\n"
    assert (tmp_path / "err.hits").read_text() == "3\n"
    replaying = stim_gb300.DetectorErrorModel("""
       error(1) D0
       error(1) D1
       error(1) D0
       error(1) D1 D2 L0
       error(1) D0
    """).compile_sampler()
    replaying.sample_write(shots=1, det_out_file=tmp_path / "dets.01", det_out_format="01",
                           obs_out_file=tmp_path / "obs.01", obs_out_format="01", err_out_file=tmp_path / "err2.01",
                           err_out_format="01", replay_err_in_file=tmp_path / "err.hits", replay_err_in_format="hits")
    assert (tmp_path / "dets.01").read_text() == "011\n"
    assert (tmp_path / "obs.01").read_text() == "1\n"
    assert (tmp_path / "err2.01").read_text() == "00010\n"
    with pytest.raises(ValueError, match="Expected more error data"):
        replaying.sample_write(shots=2, det_out_file=None, obs_out_file=None,
                               replay_err_in_file=tmp_path / "err.hits", replay_err_in_format="hits")


def test_dem_sample_write_many_chunks(tmp_path):
    # More shots than one chunk of a large model: the files hold every shot in order, equal to sample().
    lines = [f"error(0.01) D{k} D{k + 1}" for k in range(3000)] + ["error(0.02) D0 L0"]
    dem = stim_gb300.DetectorErrorModel("\n".join(lines))
    shots = 3 * 1024
    dem.compile_sampler(seed=4).sample_write(shots, det_out_file=tmp_path / "d.b8", det_out_format="b8",
                                             obs_out_file=tmp_path / "o.01", obs_out_format="01")
    d, o, _ = dem.compile_sampler(seed=4).sample(shots, bit_packed=True)
    assert (tmp_path / "d.b8").read_bytes() == d.tobytes()
    got_o = stim_gb300.read_shot_data_file(path=tmp_path / "o.01", format="01", num_observables=1, bit_packed=True)
    np.testing.assert_array_equal(got_o, o)


def test_dem_sampler_actually_fills_obs_array():
    _, obs, _ = stim_gb300.DetectorErrorModel("error(1) L0").compile_sampler().sample(shots=10000)
    assert np.all(obs)
