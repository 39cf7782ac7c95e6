"""sinter glue on the host: classify_discards_and_errors against the reference's own known-answer cases
(tests/golden/sinter/, read from sinter's test file by make_sinter.py), and the compiled sampler's bookkeeping
(counts, postselection discards, prediction checks, the decode_via_files fallback) over a stub device sampler."""

import collections
import json
import os
import types

import numpy as np
import pytest

from stim_gb300 import sinter_sampler as ss

CASES = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sinter", "classify_cases.json")))["cases"]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_classify_matches_reference_cases(k):
    c = CASES[k]
    counter = collections.Counter() if c["count_combos"] else None
    mask = c["postselected_observables_mask"]
    got = ss.classify_discards_and_errors(
        actual_obs=np.array(c["actual_obs"], dtype=np.uint8), predictions=np.array(c["predictions"], dtype=np.uint8),
        postselected_observables_mask=None if mask is None else np.array(mask),
        out_count_observable_error_combos=counter, num_obs=c["num_obs"])
    assert list(got) == c["expected"]
    if counter is not None:
        assert dict(counter) == c["expected_combos"]


class StubDeviceSampler:
    """Stands in for CompiledDetectorSampler.sample_for_decoder: fixed rows, postselection and counts done
    with numpy the way the reference's sampler does them."""

    def __init__(self, dets, obs):
        self.dets, self.obs = dets, obs

    def sample_for_decoder(self, shots, *, postselection_mask=None):
        d, o = self.dets[:shots], self.obs[:shots]
        events = sum(int(np.count_nonzero(d & (1 << b))) for b in range(8))
        drop = np.zeros(shots, dtype=bool) if postselection_mask is None else np.any(d & postselection_mask, axis=1)
        return d[~drop], o[~drop], int(drop.sum()), events


class ZeroDecoder:
    def __init__(self, extra_byte=False):
        self.extra_byte = extra_byte

    def compile_decoder_for_dem(self, *, dem):
        outer = self

        class Compiled:
            def decode_shots_bit_packed(self, *, bit_packed_detection_event_data):
                n = bit_packed_detection_event_data.shape[0]
                out = np.zeros((n, (dem.num_observables + 7) // 8 + (1 if outer.extra_byte else 0)), np.uint8)
                if outer.extra_byte:
                    out[:, -1] = bit_packed_detection_event_data[:, 0] & 1   # discard shots with detector 0 set
                return out

        return Compiled()


def _task(num_det=12, num_obs=3, post=None, post_obs=None):
    circuit = "\n".join(["X_ERROR(0.5) " + " ".join(str(q) for q in range(num_det)), "M " + " ".join(
        str(q) for q in range(num_det))] + [f"DETECTOR rec[-{num_det - q}]" for q in range(num_det)] +
        [f"OBSERVABLE_INCLUDE({k}) rec[-{num_det - k}]" for k in range(num_obs)])
    dem = types.SimpleNamespace(num_detectors=num_det, num_observables=num_obs, to_file=None)
    del dem.to_file
    return types.SimpleNamespace(circuit=circuit, detector_error_model=dem, postselection_mask=post,
                                 postselected_observables_mask=post_obs, decoder="zero")


def _rows(shots, num_det, num_obs, seed):
    rng = np.random.default_rng(seed)
    d = np.packbits(rng.integers(0, 2, (shots, num_det), dtype=np.uint8), axis=1, bitorder="little")
    o = np.packbits(rng.integers(0, 2, (shots, num_obs), dtype=np.uint8), axis=1, bitorder="little")
    return d, o


def _compiled(task, stub, decoder, **kw):
    ss_obj = ss.CompiledStimThenDecodeSampler.__new__(ss.CompiledStimThenDecodeSampler)
    ss_obj.task = task
    ss_obj.compiled_decoder = ss._compile_decoder(decoder, task, kw.get("tmp_dir"))
    ss_obj.stim_sampler = stub
    ss_obj.count_observable_error_combos = kw.get("combos", False)
    ss_obj.count_detection_events = kw.get("events", False)
    ss_obj.num_det = task.detector_error_model.num_detectors
    ss_obj.num_obs = task.detector_error_model.num_observables
    return ss_obj


@pytest.mark.parametrize("post", [None, np.array([0b101, 0], np.uint8)])
@pytest.mark.parametrize("extra_byte", [False, True])
def test_compiled_sampler_counts(post, extra_byte):
    task = _task(post=post, post_obs=np.array([1], np.uint8))
    d, o = _rows(500, 12, 3, 5)
    c = _compiled(task, StubDeviceSampler(d, o), ZeroDecoder(extra_byte), events=True, combos=True)
    st = c.sample(500)
    # Expected, straight from the rows.
    drop1 = np.zeros(500, bool) if post is None else np.any(d & post, axis=1)
    kd, ko = d[~drop1], o[~drop1]
    drop2 = (kd[:, 0] & 1).astype(bool) if extra_byte else np.zeros(len(kd), bool)
    ko = ko[~drop2]
    drop3 = (ko[:, 0] & 1).astype(bool)          # observable 0 postselected, prediction 0
    ko = ko[~drop3]
    assert st.shots == 500
    assert st.discards == int(drop1.sum() + drop2.sum() + drop3.sum())
    assert st.errors == int(np.count_nonzero(np.any(ko != 0, axis=1)))
    assert st.custom_counts["detectors_checked"] == 12 * 500
    assert st.custom_counts["detection_events"] == int(np.unpackbits(d).sum())
    assert sum(v for k, v in st.custom_counts.items() if k.startswith("obs_mistake_mask=")) == st.errors


def test_prediction_shape_is_checked():
    task = _task()
    d, o = _rows(64, 12, 3, 1)

    class Bad:
        def compile_decoder_for_dem(self, *, dem):
            return types.SimpleNamespace(
                decode_shots_bit_packed=lambda *, bit_packed_detection_event_data: np.zeros((3, 1), np.uint8))

    with pytest.raises(ValueError, match="num_shots - num_discards_1"):
        _compiled(task, StubDeviceSampler(d, o), Bad()).sample(64)


class FileDecoder:
    """A decoder with only decode_via_files: predicts observable k = detector k."""

    def compile_decoder_for_dem(self, *, dem):
        raise NotImplementedError()

    def decode_via_files(self, *, num_shots, num_obs, num_dets, dem_path, dets_b8_in_path,
                         obs_predictions_b8_out_path, tmp_dir):
        assert dem_path.exists() and tmp_dir.is_dir()
        d = np.fromfile(dets_b8_in_path, dtype=np.uint8).reshape(num_shots, (num_dets + 7) // 8)
        bits = np.unpackbits(d, axis=1, bitorder="little")[:, :num_obs]
        np.packbits(bits, axis=1, bitorder="little").tofile(obs_predictions_b8_out_path)


def test_decode_via_files_fallback(tmp_path):
    task = _task()
    d, o = _rows(300, 12, 3, 9)
    with pytest.raises(ValueError, match="no temporary directory"):
        _compiled(task, StubDeviceSampler(d, o), FileDecoder())
    st = _compiled(task, StubDeviceSampler(d, o), FileDecoder(), tmp_dir=tmp_path).sample(300)
    pred = np.packbits(np.unpackbits(d, axis=1, bitorder="little")[:, :3], axis=1, bitorder="little")
    assert st.errors == int(np.count_nonzero(np.any(pred != o, axis=1)))
