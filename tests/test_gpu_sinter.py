"""The decoder feed on the GPU (gfs_sample_for_decoder through CompiledDetectorSampler.sample_for_decoder and
the sinter adapter): kept rows, discard and detection-event counts bit-exact against the oracle's shots with
the reference sinter sampler's numpy rules (_stim_then_decode_sampler.py:170-190) applied to them; multi-chunk
calls and the stream position agree with plain sampling."""

import collections
import types

import numpy as np
import pytest

import stim_gb300
from oracle.oracle import OracleCircuit
from stim_gb300 import sinter_sampler as ss
from stim_gb300 import workloads

pytestmark = pytest.mark.gpu


def _reference_rules(d, o, mask):
    """The reference sampler's own counting and postselection over shot-major bit-packed rows."""
    events = sum(int(np.count_nonzero(d & (1 << b))) for b in range(8))
    drop = np.zeros(d.shape[0], bool) if mask is None else np.any(d & mask, axis=1)
    return d[~drop], o[~drop], int(drop.sum()), events


def _mask(num_det, dets, seed):
    m = np.zeros((num_det + 7) // 8, np.uint8)
    for k in np.random.default_rng(seed).choice(num_det, size=dets, replace=False):
        m[k // 8] |= 1 << (k % 8)
    return m


@pytest.mark.parametrize("shots", [1, 1000, 5000])
@pytest.mark.parametrize("ndet_mask", [0, 1, 6, 10_000])
@pytest.mark.parametrize("family", ["surface_code:rotated_memory_x", "color_code:memory_xyz"])
def test_feed_matches_oracle(family, shots, ndet_mask):
    text = workloads.code_circuit(family, 5, 5, 0.01)
    c = stim_gb300.Circuit(text)
    mask = None if ndet_mask == 0 else _mask(c.num_detectors, min(ndet_mask, c.num_detectors), ndet_mask)
    s = c.compile_detector_sampler(seed=11)
    d, o, discards, events = s.sample_for_decoder(shots, postselection_mask=mask)
    od, oo, _ = OracleCircuit(text).sample(shots, 11, threads=8)
    wd, wo, wdisc, wev = _reference_rules(od, oo, mask)
    np.testing.assert_array_equal(d, wd)
    np.testing.assert_array_equal(o, wo)
    assert (discards, events) == (wdisc, wev)
    assert s.stream_position() == (shots + 127) // 128 * 128


def test_feed_ignores_mask_bits_past_the_last_detector():
    text = workloads.code_circuit("color_code:memory_xyz", 3, 3, 0.05)
    c = stim_gb300.Circuit(text)
    D = c.num_detectors
    assert D % 8
    mask = np.zeros((D + 7) // 8, np.uint8)
    mask[-1] = 0xFF & ~((1 << (D % 8)) - 1)        # only bits past the last detector
    d, o, discards, _ = c.compile_detector_sampler(seed=2).sample_for_decoder(4096, postselection_mask=mask)
    assert discards == 0 and d.shape[0] == 4096


@pytest.mark.parametrize("use_mask", [False, True])
def test_feed_multi_chunk_agrees_with_plain_sampling(use_mask):
    # d=25 rows are 1,950 bytes: 300,000 shots take two chunks of the feed's 512 MiB row buffer.
    text = workloads.code_circuit("surface_code:rotated_memory_z", 25, 25, 0.001)
    c = stim_gb300.Circuit(text)
    mask = _mask(c.num_detectors, 40, 3) if use_mask else None
    shots = 300_000
    s = c.compile_detector_sampler(seed=5)
    d, o, discards, events = s.sample_for_decoder(shots, postselection_mask=mask)
    pd, po = c.compile_detector_sampler(seed=5).sample(shots, bit_packed=True, separate_observables=True)
    wd, wo, wdisc, wev = _reference_rules(pd, po, mask)
    assert (discards, events) == (wdisc, wev)
    assert d.shape == wd.shape and np.array_equal(d, wd) and np.array_equal(o, wo)
    assert s.stream_position() == (shots + 127) // 128 * 128
    # The next call continues the stream exactly as plain sampling does.
    d2, o2, _, _ = s.sample_for_decoder(1000)
    p = c.compile_detector_sampler(seed=5)
    p.set_stream_position(s.stream_position() - (1000 + 127) // 128 * 128)
    pd2, po2 = p.sample(1000, bit_packed=True, separate_observables=True)
    np.testing.assert_array_equal(d2, pd2)
    np.testing.assert_array_equal(o2, po2)


class ParityDecoder:
    """Predicts observable 0 as the parity of the first detector row byte (wrong often: errors to count)."""

    def compile_decoder_for_dem(self, *, dem):
        num_obs = dem.num_observables

        class Compiled:
            def decode_shots_bit_packed(self, *, bit_packed_detection_event_data):
                d = bit_packed_detection_event_data
                out = np.zeros((d.shape[0], (num_obs + 7) // 8), np.uint8)
                out[:, 0] = np.unpackbits(d[:, :1], axis=1).sum(axis=1) & 1
                return out

        return Compiled()


def test_sinter_adapter_matches_reference_rules_on_oracle_shots():
    text = workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.02)
    c = stim_gb300.Circuit(text)
    mask = _mask(c.num_detectors, 3, 1)
    dem = types.SimpleNamespace(num_detectors=c.num_detectors, num_observables=c.num_observables)
    task = types.SimpleNamespace(circuit=text, detector_error_model=dem, postselection_mask=mask,
                                 postselected_observables_mask=None, decoder="parity")
    sampler = ss.StimThenDecodeSampler(decoder=ParityDecoder(), count_observable_error_combos=True,
                                       count_detection_events=True, seed=21)
    st = sampler.compiled_sampler_for_task(task).sample(20_000)
    od, oo, _ = OracleCircuit(text).sample(20_000, 21, threads=8)
    kd, ko, disc, events = _reference_rules(od, oo, mask)
    pred = ParityDecoder().compile_decoder_for_dem(dem=dem).decode_shots_bit_packed(bit_packed_detection_event_data=kd)
    combos = collections.Counter()
    d2, errors = ss.classify_discards_and_errors(actual_obs=ko, predictions=pred, postselected_observables_mask=None,
                                                 out_count_observable_error_combos=combos, num_obs=c.num_observables)
    assert st.shots == 20_000
    assert st.discards == disc + d2
    assert st.errors == errors > 0
    assert st.custom_counts["detection_events"] == events
    assert st.custom_counts["detectors_checked"] == c.num_detectors * 20_000
    for k, v in combos.items():
        assert st.custom_counts[k] == v


def test_feed_reuses_caller_arrays():
    text = workloads.code_circuit("surface_code:rotated_memory_z", 5, 5, 0.02)
    c = stim_gb300.Circuit(text)
    mask = _mask(c.num_detectors, 4, 9)
    shots = 3000
    d = np.full((shots, (c.num_detectors + 7) // 8), 0xAB, dtype=np.uint8)
    o = np.full((shots, (c.num_observables + 7) // 8), 0xCD, dtype=np.uint8)
    kd, ko, disc, ev = c.compile_detector_sampler(seed=4).sample_for_decoder(shots, postselection_mask=mask,
                                                                             dets_out=d, obs_out=o)
    assert kd.base is d or np.shares_memory(kd, d)
    wd, wo, wdisc, wev = c.compile_detector_sampler(seed=4).sample_for_decoder(shots, postselection_mask=mask)
    np.testing.assert_array_equal(kd, wd)
    np.testing.assert_array_equal(ko, wo)
    assert (disc, ev) == (wdisc, wev)
    with pytest.raises(ValueError):
        c.compile_detector_sampler(seed=4).sample_for_decoder(shots, dets_out=np.zeros((shots, 1), np.uint8))
