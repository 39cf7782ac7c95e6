"""sinter glue: a sampler that draws shots on the GPU and hands them to a decoder.

Mirrors sinter's default sampler, StimThenDecodeSampler
(glue/sample/src/sinter/_decoding/_stim_then_decode_sampler.py:15-46, 147-222), and its
classify_discards_and_errors (:49-84).  The sampling half runs on the device through
``CompiledDetectorSampler.sample_for_decoder``: detection events are counted and postselected shots dropped
before the rows cross to the host, so the decoder receives only the kept shots' bit-packed rows.  The decoding
half is the caller's decoder, unchanged: ``decoder.compile_decoder_for_dem(dem=...)`` and
``decode_shots_bit_packed``, or ``decode_via_files`` through a temporary directory when the decoder compiles
nothing (:87-144).

With sinter installed the classes derive from ``sinter.Sampler`` / ``sinter.CompiledSampler`` and return
``sinter.AnonTaskStats``, so an instance can be passed wherever sinter takes a sampler (for example as a value
of ``custom_decoders`` in ``sinter.collect``).  Without sinter, a task is any object with ``circuit``,
``detector_error_model``, ``postselection_mask`` and ``postselected_observables_mask`` attributes, and
``AnonTaskStats`` below holds the same fields.
"""

from __future__ import annotations

import collections
import dataclasses
import pathlib
import secrets
import time
from typing import Optional

import numpy as np

from . import Circuit

try:  # pragma: no cover - depends on the environment
    import sinter as _sinter

    _SamplerBase = _sinter.Sampler
    _CompiledSamplerBase = _sinter.CompiledSampler
    _CompiledDecoderBase = _sinter.CompiledDecoder
    AnonTaskStats = _sinter.AnonTaskStats
except ImportError:
    _sinter = None
    _SamplerBase = object
    _CompiledSamplerBase = object
    _CompiledDecoderBase = object

    @dataclasses.dataclass(frozen=True)
    class AnonTaskStats:
        """The statistics one ``sample`` call returns (sinter's AnonTaskStats fields)."""

        shots: int = 0
        errors: int = 0
        discards: int = 0
        seconds: float = 0
        custom_counts: collections.Counter = dataclasses.field(default_factory=collections.Counter)


def classify_discards_and_errors(*, actual_obs: np.ndarray, predictions: np.ndarray,
                                 postselected_observables_mask, out_count_observable_error_combos,
                                 num_obs: int) -> tuple:
    """Counts (discards, errors) of bit-packed observable rows against a decoder's predictions.

    A prediction row one byte longer than the observable rows signals a discard through a nonzero last byte;
    a mispredicted observable under ``postselected_observables_mask`` discards the shot too; any other
    mispredicted bit is an error.  With a counter, each error also counts its mistake pattern under the key
    ``"obs_mistake_mask="`` followed by one character per observable, ``E`` for a wrong one and ``_``
    otherwise.  Same rules as sinter's function of the same name."""
    actual = np.asarray(actual_obs)
    pred = np.asarray(predictions)
    discards = 0
    if pred.shape[1] == actual.shape[1] + 1:
        flagged = pred[:, -1] != 0
        discards += int(np.count_nonzero(flagged))
        actual = actual[~flagged]
        pred = pred[~flagged, :-1]
    if postselected_observables_mask is not None:
        flagged = np.any(((actual ^ pred) & postselected_observables_mask) != 0, axis=1)
        discards += int(np.count_nonzero(flagged))
        actual = actual[~flagged]
        pred = pred[~flagged]
    wrong = np.any(actual != pred, axis=1)
    if out_count_observable_error_combos is not None:
        for diff in actual[wrong] ^ pred[wrong]:
            bits = np.unpackbits(diff, count=num_obs, bitorder="little")
            out_count_observable_error_combos["obs_mistake_mask=" + "".join("E" if b else "_" for b in bits)] += 1
    return discards, int(np.count_nonzero(wrong))


class DiskDecoder(_CompiledDecoderBase):
    """Runs a decoder that compiles nothing through its ``decode_via_files`` (dem, b8 detection events in,
    b8 predictions out), in a fresh directory under ``tmp_dir``."""

    def __init__(self, decoder, task, tmp_dir: pathlib.Path):
        self.decoder = decoder
        tmp_dir = pathlib.Path(tmp_dir)
        while True:
            top = tmp_dir / f"disk_decoder_{secrets.randbits(64)}"
            try:
                top.mkdir()
                break
            except FileExistsError:
                continue
        self.top = top
        self.decoder_dir = top / "dec"
        self.decoder_dir.mkdir()
        dem = task.detector_error_model
        self.num_obs = dem.num_observables
        self.num_dets = dem.num_detectors
        self.dem_path = top / "dem.dem"
        if hasattr(dem, "to_file"):
            dem.to_file(self.dem_path)
        else:
            self.dem_path.write_text(str(dem))
        self.dets_path = top / "dets.b8"
        self.obs_path = top / "obs.b8"

    def decode_shots_bit_packed(self, *, bit_packed_detection_event_data: np.ndarray) -> np.ndarray:
        shots = bit_packed_detection_event_data.shape[0]
        np.ascontiguousarray(bit_packed_detection_event_data, dtype=np.uint8).tofile(self.dets_path)
        self.decoder.decode_via_files(num_shots=shots, num_obs=self.num_obs, num_dets=self.num_dets,
                                      dem_path=self.dem_path, dets_b8_in_path=self.dets_path,
                                      obs_predictions_b8_out_path=self.obs_path, tmp_dir=self.decoder_dir)
        row = (self.num_obs + 7) // 8
        pred = np.fromfile(self.obs_path, dtype=np.uint8, count=row * shots)
        if pred.shape != (row * shots,):
            raise ValueError("the decoder wrote fewer predictions than shots")
        self.obs_path.unlink()
        self.dets_path.unlink()
        return pred.reshape((shots, row))


def _compile_decoder(decoder, task, tmp_dir):
    try:
        return decoder.compile_decoder_for_dem(dem=task.detector_error_model)
    except NotImplementedError:
        pass
    if tmp_dir is None:
        raise ValueError(f"Decoder {getattr(task, 'decoder', decoder)!r} didn't implement `compile_decoder_for_dem`, "
                         "but no temporary directory was provided for falling back to `decode_via_files`.")
    return DiskDecoder(decoder, task, tmp_dir)


def _as_circuit(c) -> Circuit:
    return c if isinstance(c, Circuit) else Circuit(str(c))


class StimThenDecodeSampler(_SamplerBase):
    """Samples shots on the GPU, then decodes them with ``decoder``.

    Same constructor arguments as sinter's StimThenDecodeSampler, plus ``device`` (CUDA device index) and
    ``seed`` (None: a fresh random seed per task, as sinter's ``compile_detector_sampler()`` without a seed
    gives)."""

    def __init__(self, *, decoder, count_observable_error_combos: bool = False,
                 count_detection_events: bool = False, tmp_dir: Optional[pathlib.Path] = None,
                 device: int = 0, seed: Optional[int] = None):
        self.decoder = decoder
        self.count_observable_error_combos = count_observable_error_combos
        self.count_detection_events = count_detection_events
        self.tmp_dir = tmp_dir
        self.device = device
        self.seed = seed

    def compiled_sampler_for_task(self, task) -> "CompiledStimThenDecodeSampler":
        return CompiledStimThenDecodeSampler(
            decoder=self.decoder, task=task, count_observable_error_combos=self.count_observable_error_combos,
            count_detection_events=self.count_detection_events, tmp_dir=self.tmp_dir, device=self.device,
            seed=self.seed)


class CompiledStimThenDecodeSampler(_CompiledSamplerBase):
    """One task's sampler: a compiled GPU detector sampler and a compiled decoder."""

    def __init__(self, *, decoder, task, count_observable_error_combos: bool, count_detection_events: bool,
                 tmp_dir, device: int = 0, seed: Optional[int] = None, stim_sampler=None):
        self.task = task
        self.compiled_decoder = _compile_decoder(decoder, task, tmp_dir)
        circuit = _as_circuit(task.circuit)
        self.stim_sampler = stim_sampler if stim_sampler is not None else circuit.compile_detector_sampler(
            seed=secrets.randbits(64) if seed is None else seed, device=device)
        self.count_observable_error_combos = count_observable_error_combos
        self.count_detection_events = count_detection_events
        self.num_det = circuit.num_detectors
        self.num_obs = circuit.num_observables

    def sample(self, suggested_shots: int) -> AnonTaskStats:
        t0 = time.monotonic()
        shots = int(suggested_shots)
        dets, actual_obs, discards_1, events = self.stim_sampler.sample_for_decoder(
            shots, postselection_mask=self.task.postselection_mask)
        custom_counts = collections.Counter()
        if self.count_detection_events:
            custom_counts["detectors_checked"] += self.num_det * shots
            custom_counts["detection_events"] += events
        predictions = self.compiled_decoder.decode_shots_bit_packed(bit_packed_detection_event_data=dets)
        if not isinstance(predictions, np.ndarray):
            raise ValueError("not isinstance(predictions, np.ndarray)")
        if predictions.dtype != np.uint8:
            raise ValueError("predictions.dtype != np.uint8")
        if len(predictions.shape) != 2:
            raise ValueError("len(predictions.shape) != 2")
        if predictions.shape[0] != shots - discards_1:
            raise ValueError("predictions.shape[0] != num_shots - num_discards_1")
        if predictions.shape[1] < actual_obs.shape[1]:
            raise ValueError("predictions.shape[1] < actual_obs.shape[1]")
        if predictions.shape[1] > actual_obs.shape[1] + 1:
            raise ValueError("predictions.shape[1] > actual_obs.shape[1] + 1")
        discards_2, errors = classify_discards_and_errors(
            actual_obs=actual_obs, predictions=predictions,
            postselected_observables_mask=self.task.postselected_observables_mask,
            out_count_observable_error_combos=custom_counts if self.count_observable_error_combos else None,
            num_obs=self.num_obs)
        return AnonTaskStats(shots=shots, errors=errors, discards=discards_1 + discards_2,
                             seconds=time.monotonic() - t0, custom_counts=custom_counts)
