"""Error counts of detector error models as the reference's own Python test states them
(src/stim/dem/detector_error_model_pybind_test.py:191-208, test_count_errors): declarations and shifts are not
errors; REPEAT blocks multiply.  Host code (the DEM parser), no GPU."""

import stim_gb300


def test_count_errors():
    assert stim_gb300.DetectorErrorModel().num_errors == 0
    assert stim_gb300.DetectorErrorModel("""
        logical_observable L100
        detector D100
        shift_detectors(100, 100, 100) 100
        error(0.125) D100
    """).num_errors == 1
    assert stim_gb300.DetectorErrorModel("""
        error(0.125) D0
        REPEAT 100 {
            REPEAT 5 {
                error(0.25) D1
            }
        }
    """).num_errors == 501
