"""Error counts of detector error models as the reference's own Python test states them
(src/stim/dem/detector_error_model_pybind_test.py:191-208, test_count_errors): declarations and shifts are not
errors; REPEAT blocks multiply.  Also the counts, rejections and parses of the reference's C++ model tests.  Host
code (the DEM parser), no GPU."""

import pytest

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


@pytest.mark.parametrize("text,detectors,observables", [
    # src/stim/dem/detector_error_model.test.cc:377-410 (count_detectors, count_observables), :892-896.
    ("", 0, 0), ("error(0.3) D2 L1000", 3, 1001), ("shift_detectors 5", 0, 0), ("shift_detectors 5\ndetector D3", 9, 0),
    ("shift_detectors 50\nrepeat 1000 {\n    detector D0\n    error(0.1) D0 D1\n    shift_detectors 4\n}", 4048, 0),
    ("error(0.3) L2 D9999", 10000, 3), ("shift_detectors 5\nlogical_observable L3", 0, 4),
    ("error(0.125) D0\r\ndetector(5) D10\r\n", 11, 0),
])
def test_counts_of_the_reference_dem_tests(text, detectors, observables):
    m = stim_gb300.DetectorErrorModel(text)
    assert (m.num_detectors, m.num_observables) == (detectors, observables)


def test_observable_count_through_loops():
    m = stim_gb300.DetectorErrorModel(
        "shift_detectors 50\nrepeat 1000 {\n    logical_observable L5\n    error(0.1) D0 D1 L6\n    shift_detectors 4\n}")
    assert m.num_observables == 7


@pytest.mark.parametrize("text", [
    # detector_error_model.test.cc:64-148: probabilities outside [0, 1], separators at an end or doubled, detector /
    # observable declarations of the other kind of target.
    "error(1.5) D0", "error(-0.5) D0", "error(0.25) ^", "error(0.25) ^ L0", "error(0.25) L0 ^", "error(0.25) L0 ^ ^ D4",
    "detector L4", "detector ^", "logical_observable D4", "logical_observable ^",
])
def test_rejected_like_the_reference(text):
    with pytest.raises(ValueError):
        stim_gb300.DetectorErrorModel(text)


def test_tagged_and_nested_models_parse():
    # detector_error_model.test.cc:177-262 (round_trip_str, parse, parse_tag).
    stim_gb300.DetectorErrorModel(
        "error(0.125) D0\nrepeat 100 {\n    repeat 200 {\n        error[test-tag](0.25) D0 D1 L0 ^ D2\n"
        "        shift_detectors(1.5, 3) 10\n        detector(0.5) D0\n        detector D1\n    }\n"
        "    error(0.375) D0 D1\n    shift_detectors 20\n    logical_observable L0\n}")
    m = stim_gb300.DetectorErrorModel(
        "error[test1](0.125) D0\nrepeat[test2] 10 {\n    shift_detectors[test3](1.5, 3) 10\n"
        "    detector[test4](0.5) D0\n}\nlogical_observable[test5] L0")
    assert (m.num_observables, m.num_errors) == (1, 1)
    m = stim_gb300.DetectorErrorModel(
        "error(0.125) D0\nerror(0.125) D5\nerror(0.25) D5 ^ L4\nshift_detectors(1.5, 2) 60\nrepeat 100 {\n"
        "    error(0.125) D0\n    error(0.125) D5\n    error(0.25) D5 ^ L4\n    shift_detectors(1.5, 2) 60\n}")
    assert (m.num_observables, m.num_errors) == (5, 303)


# Spacing and argument rules of the reference's model parser (circuit.h read_parens_arguments and
# read_until_next_line_arg, shared with circuits), found by comparing acceptance with the reference's own
# `stim sample_dem` on random texts.
@pytest.mark.parametrize("text", ["error() D0", "error( ) D0", "error(\t0.1\t) D0", "detector(1,,2) D0",
                                  "error(0.1)", "error(0.1)#c", "repeat 2 {}", "repeat 2 { detector D0\n}"])
def test_accepted_like_the_reference_parser(text):
    stim_gb300.DetectorErrorModel(text)


@pytest.mark.parametrize("text", ["error (0.1) D0", "error(0.1)D0", "repeat 2 {\ndetector D0 }",
                                  "repeat 2 {\ndetector D0}", "repeat(2) 3 {\n}", "error(0.1x) D0", "error(inf) D0"])
def test_rejected_like_the_reference_parser(text):
    with pytest.raises(ValueError):
        stim_gb300.DetectorErrorModel(text)
