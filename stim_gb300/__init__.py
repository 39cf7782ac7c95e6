"""GB300 frame sampler: a drop-in for the reference's bulk detection-event and measurement samplers.

Mirrors the Python surface of the reference's compiled samplers:

* ``Circuit.compile_detector_sampler(*, seed=None)`` (src/stim/circuit/circuit.pybind.cc:827-831)
  -> ``CompiledDetectorSampler.sample(shots, *, prepend_observables, append_observables,
  separate_observables, bit_packed, dets_out, obs_out)`` (src/stim/py/compiled_detector_sampler.pybind.cc:34-86,
  216-322);
* ``Circuit.compile_sampler(*, skip_reference_sample=False, seed=None, reference_sample=None)``
  (circuit.pybind.cc:588-595, compiled_measurement_sampler.pybind.cc:63-83) -> ``.sample(shots, *, bit_packed)``.

Everything runs through the C ABI of libstim_gb300.so on a CUDA device.  Random streams are the
counter-based contract of csrc/gfs_contract.h: the same seed gives the same shots on every run, every
slicing and every GPU, but not the reference's mt19937_64 stream (which the reference itself documents as
unstable across versions and machines).
"""

import ctypes
import os
import shutil
import tempfile

import numpy as np

from . import _native
from ._native import check, lib

__all__ = ["shard_range", "Circuit", "CompiledDetectorSampler", "CompiledMeasurementSampler",
           "CompiledMeasurementsToDetectionEventsConverter", "DetectorErrorModel", "CompiledDemSampler",
           "BatchSampler", "Server", "device_count", "read_shot_data_file", "write_shot_data_file"]


def device_count() -> int:
    return _native.device_count()


def shard_range(total_shots: int, rank: int, world: int):
    """(first_shot, shots) of `rank`'s share when `world` ranks sample `total_shots` shots of one stream: whole
    128-shot blocks, as even as possible, in rank order.  No collective is needed: every shot's bits depend
    only on (circuit, seed, global shot index)."""
    if world < 1 or not 0 <= rank < world or total_shots < 0:
        raise ValueError("need 0 <= rank < world and total_shots >= 0")
    blocks = (total_shots + 127) // 128
    lo = blocks * rank // world
    hi = blocks * (rank + 1) // world
    first = lo * 128
    return first, max(0, min(total_shots, hi * 128) - first)


def _seed_value(seed):
    if seed is None:
        return int.from_bytes(os.urandom(8), "little")
    if isinstance(seed, bool) or not isinstance(seed, (int, np.integer)) or not (0 <= int(seed) < 2**64):
        raise ValueError("Expected seed to be None or a 64 bit unsigned integer.")
    return int(seed)


def read_shot_data_file(*, path, format: str = "01", num_measurements=None, num_detectors=None,
                        num_observables=None, separate_observables: bool = False, bit_packed: bool = False,
                        bit_pack: bool = False):
    """Reads a result file (formats "01", "b8", "r8", "ptb64", "hits", "dets") as the reference's
    stim.read_shot_data_file does (src/stim/io/read_write.pybind.cc:97-145): records of num_measurements +
    num_detectors + num_observables bits; bool arrays, or bit-packed uint8 rows (bit_pack is the reference's
    legacy name for bit_packed); observables split off with separate_observables."""
    bit_packed = bool(bit_packed) or bool(bit_pack)
    if num_measurements is None and num_detectors is None and num_observables is None:
        raise ValueError("Must specify num_measurements, num_detectors, num_observables.")
    nm, nd, no = (int(v or 0) for v in (num_measurements, num_detectors, num_observables))
    n = nm + nd + no
    nb = (n + 7) // 8
    p = _path(path)
    size = os.path.getsize(p.decode()) if os.path.exists(p.decode()) else 0
    # An upper bound on the records a file of this size can hold in this format.
    cap = {"b8": size // nb if nb else 0, "01": size // (n + 1), "ptb64": (size // (8 * n)) * 64 if n else 0,
           "dets": size // 5}.get(str(format), size) + 1
    buf = np.zeros((cap, max(1, nb)), dtype=np.uint8)
    shots = ctypes.c_uint64()
    check(lib().gfs_read_shot_data_file(p, str(format).encode(), nm, nd, no, _ptr(buf), cap, ctypes.byref(shots)))
    rows = buf[:shots.value, :nb]

    def part(lo, count):
        bits = np.unpackbits(rows, axis=1, bitorder="little")[:, lo:lo + count].astype(bool)
        return np.packbits(bits, axis=1, bitorder="little") if bit_packed else bits

    if separate_observables:
        return part(0, n - no), part(n - no, no)
    return part(0, n)


def write_shot_data_file(*, data, path, format: str = "01", num_measurements=None, num_detectors=None,
                         num_observables=None) -> None:
    """Writes shot records to a result file as the reference's stim.write_shot_data_file does
    (src/stim/io/read_write.pybind.cc:147-183): `data` is a bool array (shots, bits) or bit-packed uint8 rows
    (shots, ceil(bits / 8)); bits = num_measurements, or num_detectors + num_observables."""
    if num_measurements is None and num_detectors is None and num_observables is None:
        raise ValueError("Must specify num_measurements, num_detectors, num_observables.")
    nm, nd, no = (int(v or 0) for v in (num_measurements, num_detectors, num_observables))
    if nm and (nd or no):
        raise ValueError("num_measurements and (num_detectors or num_observables)")
    n = nm + nd + no
    a = np.asarray(data)
    if a.ndim != 2 or a.dtype not in (np.bool_, np.uint8):
        raise ValueError("data must be a 2-dimensional numpy array with dtype=np.uint8 or dtype=np.bool_")
    # The reference's messages for a wrong row width (src/stim/py/numpy.pybind.cc:256-263, 290-296).
    if a.dtype == np.bool_:
        if a.shape[1] != n:
            raise ValueError(f"Expected {n} bits per shot. Got unpacked boolean data (dtype=np.bool_) but "
                             f"data.shape[1]={a.shape[1]}")
        rows = np.packbits(a, axis=1, bitorder="little")
    else:
        if a.shape[1] != (n + 7) // 8:
            raise ValueError(f"Expected {n} bits per shot. Got bit packed data (dtype=np.uint8) but "
                             f"data.shape[1]={a.shape[1]} != math.ceil({n} / 8)={(n + 7) // 8}")
        rows = a
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    if rows.shape[1] == 0:
        rows = np.zeros((rows.shape[0], 1), dtype=np.uint8)
    check(lib().gfs_write_shot_data_file(_ptr(rows), rows.shape[1], rows.shape[0], _path(path),
                                         str(format).encode(), nm, nd, no))


class Circuit:
    """A parsed .stim circuit (parsing happens in the library's C++ host code)."""

    def __init__(self, text: str = ""):
        if not isinstance(text, str):
            text = str(text)
        self._text = text
        h = ctypes.c_void_p()
        data = text.encode()
        check(lib().gfs_circuit_parse(data, len(data), ctypes.byref(h)))
        self._h = h
        s = (ctypes.c_uint64 * 6)()
        check(lib().gfs_circuit_stats(self._h, s))
        (self.num_qubits, self.num_measurements, self.num_detectors, self.num_observables,
         self.max_lookback, self.num_instructions_unrolled) = [int(v) for v in s]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_circuit_free(h)
            self._h = None

    def __str__(self):
        return self._text

    def __repr__(self):
        return f"stim_gb300.Circuit({self._text!r})"

    def program_info(self, mode: str = "detections") -> dict:
        """Lowers the circuit on the host (no GPU needed) and describes the device program."""
        info = (ctypes.c_uint64 * 8)()
        m = _native.MODE_MEASUREMENTS if mode == "measurements" else _native.MODE_DETECTIONS
        check(lib().gfs_program_info(self._h, m, info))
        keys = ["ops", "pool_words", "rows", "ring", "channels", "loop_depth", "smem_bytes_per_block", "detectors"]
        out = dict(zip(keys, [int(v) for v in info]))
        occ, hits = ctypes.c_uint64(), ctypes.c_double()
        check(lib().gfs_program_noise(self._h, m, ctypes.byref(occ), ctypes.byref(hits)))
        out["noise_occurrences"] = occ.value
        out["hits_per_block"] = hits.value
        return out

    def reference_sample(self, *, bit_packed: bool = False) -> np.ndarray:
        """The noiseless run with random outcomes forced to 0 (the reference's Circuit.reference_sample),
        computed on the host."""
        M = self.num_measurements
        out = np.zeros((M + 7) // 8, dtype=np.uint8)
        check(lib().gfs_circuit_reference_sample(self._h, _ptr(out) if out.size else None, out.size))
        if bit_packed:
            return out
        return np.unpackbits(out, bitorder="little")[:M].astype(np.bool_)

    def compile_detector_sampler(self, *, seed=None, device: int = 0) -> "CompiledDetectorSampler":
        return CompiledDetectorSampler(self, seed=seed, device=device)

    def compile_sampler(self, *, skip_reference_sample: bool = False, seed=None, reference_sample=None,
                        device: int = 0) -> "CompiledMeasurementSampler":
        return CompiledMeasurementSampler(self, skip_reference_sample=skip_reference_sample, seed=seed,
                                          reference_sample=reference_sample, device=device)

    def compile_m2d_converter(self, *, skip_reference_sample: bool = False,
                              device: int = 0) -> "CompiledMeasurementsToDetectionEventsConverter":
        return CompiledMeasurementsToDetectionEventsConverter(self, skip_reference_sample=skip_reference_sample,
                                                              device=device)


def _circuit_repr(c) -> str:
    """The circuit as a Python expression: its lines, stripped and indented by four spaces, in a triple-quoted
    literal (the layout of the reference's circuit_repr)."""
    body = "".join(f"    {ln.strip()}\n" for ln in str(c).splitlines() if ln.strip())
    if not body:
        return "stim_gb300.Circuit()"
    return "stim_gb300.Circuit('''\n" + body + "''')"


class _SamplerBase:
    _mode = None

    def __init__(self, circuit, seed, device):
        if not isinstance(circuit, Circuit):
            circuit = Circuit(str(circuit))
        self._circuit = circuit
        h = ctypes.c_void_p()
        check(lib().gfs_sampler_create(circuit._h, self._mode, _seed_value(seed), int(device), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_sampler_free(h)
            self._h = None

    # -- tuning / introspection (no counterpart in the reference) --
    def set_launch_shape(self, blocks_per_cta: int, threads: int = 256, grid: int = 0):
        check(lib().gfs_sampler_set_shape(self._h, blocks_per_cta, threads, grid))

    def launch_shape(self):
        b, t, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        sm = ctypes.c_uint64()
        check(lib().gfs_sampler_get_shape(self._h, ctypes.byref(b), ctypes.byref(t), ctypes.byref(g),
                                          ctypes.byref(sm)))
        k = ctypes.c_int()
        check(lib().gfs_sampler_get_frame_kernel(self._h, ctypes.byref(k)))
        return {"blocks_per_cta": b.value, "threads": t.value, "grid": g.value, "smem_bytes": sm.value,
                "kernel": "lean" if k.value == 1 else "generic"}

    def set_frame_kernel(self, kind: int):
        """Frame kernel of hit-list launches: -1 automatic, 0 generic, 1 lean when the program has a lean phase
        list.  Results are identical."""
        check(lib().gfs_sampler_set_frame_kernel(self._h, int(kind)))

    def set_ring_placement(self, placement: int):
        """-1 automatic, 0 shared memory, 1 global memory (per-CTA, L2-resident)."""
        check(lib().gfs_sampler_set_ring_placement(self._h, int(placement)))

    def set_chunk_shots(self, shots: int):
        check(lib().gfs_sampler_set_chunk_shots(self._h, int(shots)))

    def set_stream_position(self, shot: int):
        """Global index of the next shot (a multiple of 128): ranks sampling one stream by shot range set
        disjoint positions (see shard_range)."""
        check(lib().gfs_sampler_set_stream_position(self._h, int(shot)))

    def stream_position(self) -> int:
        v = ctypes.c_uint64()
        check(lib().gfs_sampler_get_stream_position(self._h, ctypes.byref(v)))
        return v.value

    def autotune(self, trial_shots: int = 0) -> float:
        """Times the frame kernel for each candidate launch shape and keeps the fastest (results never
        depend on the shape; the stream position does not move).  Returns the best time in ms."""
        ms = ctypes.c_double()
        check(lib().gfs_sampler_autotune(self._h, int(trial_shots), ctypes.byref(ms)))
        return ms.value

    def set_noise_mode(self, mode: int):
        """-1 automatic, 0 noise drawn inside the frame kernel, 1 noise drawn into hit lists by a separate
        kernel.  Results are identical."""
        check(lib().gfs_sampler_set_noise_mode(self._h, int(mode)))

    def last_timings(self):
        t = (ctypes.c_double * 4)()
        c = (ctypes.c_uint64 * 4)()
        check(lib().gfs_sampler_last_timings(self._h, t, None))
        check(lib().gfs_sampler_last_counts(self._h, c))
        nm = ctypes.c_double()
        check(lib().gfs_sampler_last_noise_ms(self._h, ctypes.byref(nm)))
        return {"frame_ms": t[0], "noise_ms": nm.value, "transpose_ms": t[1], "copy_ms": t[2], "total_ms": t[3],
                "frame_launches": int(c[0]), "transpose_launches": int(c[1]), "noise_launches": int(c[2]),
                "hit_overflows": int(c[3])}


def _out_array(out, shape, packed):
    dtype = np.uint8 if packed else np.bool_
    if out is None:
        return np.empty(shape, dtype=dtype), None
    if not isinstance(out, np.ndarray) or out.dtype != dtype:
        raise ValueError("Output buffer wasn't a numpy.ndarray[%s]." % ("np.uint8" if packed else "np.bool_"))
    if out.ndim != 2:
        raise ValueError("Output buffer wasn't two dimensional.")
    if tuple(out.shape) != tuple(shape):
        raise ValueError(f"Expected output buffer to have shape=({shape[0]}, {shape[1]}) but its shape is "
                         f"({out.shape[0]}, {out.shape[1]}).")
    if out.flags.c_contiguous or (out.shape[1] <= 1 and out.strides[0] > 0):
        return out, None
    return np.empty(shape, dtype=dtype), out


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class CompiledDetectorSampler(_SamplerBase):
    """Samples detection events and observable flips (replaces CompiledDetectorSampler + FrameSimulator)."""

    _mode = _native.MODE_DETECTIONS

    def __init__(self, circuit, *, seed=None, device: int = 0):
        super().__init__(circuit, seed, device)

    def __repr__(self):
        # As the reference's CompiledDetectorSampler.repr (compiled_detector_sampler.pybind.cc:143-149).
        return f"stim_gb300.CompiledDetectorSampler({_circuit_repr(self._circuit)})"

    def sample_bit_packed(self, shots: int, *, prepend_observables: bool = False, append_observables: bool = False):
        """Deprecated in the reference: sample(shots, bit_packed=True, ...) (compiled_detector_sampler.pybind.cc:324-356)."""
        return self.sample(shots, prepend_observables=prepend_observables, append_observables=append_observables,
                           bit_packed=True)

    def sample(self, shots: int, *, prepend_observables: bool = False, append_observables: bool = False,
               separate_observables: bool = False, bit_packed: bool = False, dets_out=None, obs_out=None):
        if separate_observables and (append_observables or prepend_observables):
            raise ValueError("Can't specify separate_observables=True with append_observables=True or "
                             "prepend_observables=True")
        shots = int(shots)
        if shots < 0:
            raise ValueError("shots must be non-negative")
        c = self._circuit
        D, O = c.num_detectors, c.num_observables
        nd = D + (O if prepend_observables else 0) + (O if append_observables else 0)
        width = (lambda n: (n + 7) // 8) if bit_packed else (lambda n: n)
        dets, dets_user = _out_array(dets_out, (shots, width(nd)), bit_packed)
        want_obs = separate_observables or obs_out is not None
        obs = obs_user = None
        if want_obs:
            obs, obs_user = _out_array(obs_out, (shots, width(O)), bit_packed)
        flags = ((_native.PREPEND_OBSERVABLES if prepend_observables else 0)
                 | (_native.APPEND_OBSERVABLES if append_observables else 0)
                 | (_native.BIT_PACKED if bit_packed else 0))
        if shots:
            check(lib().gfs_sample_detections(
                self._h, shots, flags, _ptr(dets), dets.strides[0] if dets.size else max(1, dets.shape[1]),
                _ptr(obs) if obs is not None else None,
                (obs.strides[0] if obs.size else max(1, obs.shape[1])) if obs is not None else 0))
        if dets_user is not None:
            dets_user[...] = dets
            dets = dets_user
        if obs_user is not None:
            obs_user[...] = obs
            obs = obs_user
        if separate_observables:
            return dets, obs
        return dets

    def sample_for_decoder(self, shots: int, *, postselection_mask=None, dets_out=None, obs_out=None):
        """Samples ``shots`` shots for a decoder, as sinter's StimThenDecodeSampler does
        (glue/sample/src/sinter/_decoding/_stim_then_decode_sampler.py:170-190), with the counting and the
        postselection done on the device.

        Returns ``(dets, obs, num_discards, num_detection_events)``: the kept shots' bit-packed detector and
        observable rows in shot order, the number of shots dropped because a detection event fell under
        ``postselection_mask`` (uint8, ``ceil(num_detectors / 8)`` bytes, or None), and the number of
        detection events over all sampled shots before dropping.  dets_out / obs_out (optional) are caller-owned
        uint8 arrays of shape (shots, row bytes) reused across calls; the kept rows are views of their first rows."""
        shots = int(shots)
        if shots < 0:
            raise ValueError("shots must be non-negative")
        c = self._circuit
        drow, orow = (c.num_detectors + 7) // 8, (c.num_observables + 7) // 8
        mask = None
        if postselection_mask is not None:
            mask = np.ascontiguousarray(np.asarray(postselection_mask), dtype=np.uint8).reshape(-1)
            if mask.shape[0] != drow:
                raise ValueError(f"postselection_mask must have {drow} bytes, got {mask.shape[0]}")
        dets, _ = _out_array(dets_out, (shots, drow), True)
        obs, _ = _out_array(obs_out, (shots, orow), True)
        out = (ctypes.c_uint64 * 3)()
        if shots:
            check(lib().gfs_sample_for_decoder(
                self._h, shots, _ptr(mask) if mask is not None else None, _ptr(dets), max(1, drow), _ptr(obs),
                max(1, orow), out))
        kept = int(out[0])
        return dets[:kept], obs[:kept], int(out[1]), int(out[2])

    def sample_write(self, shots: int, *, filepath, format: str = "01", obs_out_filepath=None,
                     obs_out_format: str = "01", prepend_observables: bool = False,
                     append_observables: bool = False) -> None:
        """Samples detection events and writes them to a file in a result format ("01", "b8", "r8", "hits",
        "dets", "ptb64"), observables prepended, appended or written to ``obs_out_filepath``, as the
        reference's CompiledDetectorSampler.sample_write does (compiled_detector_sampler.pybind.cc:357-415)."""
        flags = ((_native.PREPEND_OBSERVABLES if prepend_observables else 0)
                 | (_native.APPEND_OBSERVABLES if append_observables else 0))
        check(lib().gfs_sample_write_detections(
            self._h, int(shots), _path(filepath), str(format).encode(), flags,
            _path(obs_out_filepath) if obs_out_filepath is not None else None, str(obs_out_format).encode()))


def _path(p):
    if isinstance(p, os.PathLike):
        p = os.fspath(p)
    if not isinstance(p, str):
        raise ValueError(f"Don't know how to write to {p!r}")
    return p.encode()


class CompiledMeasurementSampler(_SamplerBase):
    """Samples measurement results = reference sample XOR frame flips (replaces CompiledMeasurementSampler)."""

    _mode = _native.MODE_MEASUREMENTS

    def __init__(self, circuit, *, skip_reference_sample: bool = False, seed=None, reference_sample=None,
                 device: int = 0):
        super().__init__(circuit, seed, device)
        M = self._circuit.num_measurements
        self._skip = bool(skip_reference_sample)
        if reference_sample is not None:
            if skip_reference_sample:
                raise ValueError("skip_reference_sample = True but reference_sample is not None.")
            ref = np.asarray(reference_sample)
            if ref.dtype == np.bool_:
                if ref.shape != (M,):
                    raise ValueError("reference_sample has the wrong number of bits")
                ref = np.packbits(ref, bitorder="little")
            elif ref.dtype == np.uint8:
                if ref.shape != ((M + 7) // 8,):
                    raise ValueError("reference_sample has the wrong number of bytes")
            else:
                raise ValueError("reference_sample must be a numpy bool or uint8 array")
            self._ref = np.ascontiguousarray(ref, dtype=np.uint8)
        elif skip_reference_sample:
            self._ref = None
        else:
            self._ref = self._circuit.reference_sample(bit_packed=True)

    def __repr__(self):
        # As the reference's CompiledMeasurementSampler.repr (compiled_measurement_sampler.pybind.cc:47-56).
        skip = ", skip_reference_sample=True" if self._skip else ""
        return f"stim_gb300.CompiledMeasurementSampler({_circuit_repr(self._circuit)}{skip})"

    def sample_bit_packed(self, shots: int):
        """Deprecated in the reference: sample(shots, bit_packed=True) (compiled_measurement_sampler.pybind.cc:210-241)."""
        return self.sample(shots, bit_packed=True)

    def sample_write(self, shots: int, *, filepath, format: str = "01") -> None:
        """Samples measurements and writes them to a file in a result format ("01", "b8", "r8", "hits",
        "dets", "ptb64"), as the reference's CompiledMeasurementSampler.sample_write does."""
        check(lib().gfs_sample_write_measurements(self._h, int(shots), _path(filepath), str(format).encode(),
                                                  _ptr(self._ref) if self._ref is not None else None))

    def sample(self, shots: int, *, bit_packed: bool = False):
        shots = int(shots)
        M = self._circuit.num_measurements
        out = np.empty((shots, (M + 7) // 8 if bit_packed else M), dtype=np.uint8 if bit_packed else np.bool_)
        if shots:
            check(lib().gfs_sample_measurements(
                self._h, shots, _native.BIT_PACKED if bit_packed else 0,
                _ptr(self._ref) if self._ref is not None else None, _ptr(out),
                out.strides[0] if out.size else max(1, out.shape[1])))
        return out


class CompiledMeasurementsToDetectionEventsConverter:
    """Converts measurement records into detection events and observable flips on the GPU (replaces the
    reference's CompiledMeasurementsToDetectionEventsConverter, measurements_to_detection_events.pybind.cc).
    A detector fires when the parity of its measurements differs from their parity in the circuit's
    reference sample (all zeros with skip_reference_sample=True)."""

    def __init__(self, circuit, *, skip_reference_sample: bool = False, device: int = 0):
        if not isinstance(circuit, Circuit):
            circuit = Circuit(str(circuit))
        self._circuit = circuit
        ref = None if skip_reference_sample else circuit.reference_sample(bit_packed=True)
        h = ctypes.c_void_p()
        check(lib().gfs_m2d_create(circuit._h, _ptr(ref) if ref is not None and ref.size else None, int(device),
                                   ctypes.byref(h)))
        self._h = h
        self._ref = ref
        s = (ctypes.c_uint64 * 4)()
        check(lib().gfs_m2d_stats(self._h, s))
        self.num_measurements, self.num_detectors, self.num_observables, self.num_sweep_bits = [int(v) for v in s]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_m2d_free(h)
            self._h = None

    @staticmethod
    def _packed(a, nbits, what):
        """Bit-packed uint8 rows (shots, ceil(nbits / 8)) from a bool (shots, nbits) or packed uint8 array."""
        a = np.asarray(a)
        if a.ndim != 2:
            raise ValueError(f"{what} must be a 2d numpy array")
        if a.dtype == np.bool_:
            if a.shape[1] != nbits:
                raise ValueError(f"Expected {what}.shape[1] == {nbits} but got {a.shape[1]}")
            return np.ascontiguousarray(np.packbits(a, axis=1, bitorder="little"))
        if a.dtype == np.uint8:
            if a.shape[1] != (nbits + 7) // 8:
                raise ValueError(f"Expected bit packed {what}.shape[1] == {(nbits + 7) // 8} but got {a.shape[1]}")
            return np.ascontiguousarray(a)
        raise ValueError(f"{what} must be a numpy array of bool or of bit packed uint8")

    def convert(self, *, measurements, sweep_bits=None, separate_observables=None, append_observables=None,
                bit_packed: bool = False, bit_pack_result: bool = False, dets_out=None, obs_out=None):
        """As the reference's convert (bit_pack_result is its legacy name for bit_packed,
        measurements_to_detection_events.pybind.cc:84-86); dets_out / obs_out (optional, no counterpart in the
        reference) are caller-owned arrays of the result's shape and dtype, reused across calls to avoid touching
        fresh pages on every call."""
        bit_packed = bool(bit_packed) or bool(bit_pack_result)
        if separate_observables is None and append_observables is None:
            raise ValueError("To ignore observable flip data, you must explicitly specify either "
                             "separate_observables=False or append_observables=False.")
        separate = bool(separate_observables)
        append = bool(append_observables)
        m = self._packed(measurements, self.num_measurements, "measurements")
        shots = m.shape[0]
        sw = None
        if sweep_bits is not None:
            sw = self._packed(sweep_bits, self.num_sweep_bits, "sweep_bits")
            if sw.shape[0] != shots:
                raise ValueError("Need sweep_bits.shape[0] == measurements.shape[0]")
        D, O = self.num_detectors, self.num_observables
        nd = D + (O if append else 0)
        width = (lambda n: (n + 7) // 8) if bit_packed else (lambda n: n)
        dets, dets_user = _out_array(dets_out, (shots, width(nd)), bit_packed)
        obs = obs_user = None
        if separate:
            obs, obs_user = _out_array(obs_out, (shots, width(O)), bit_packed)
        flags = (_native.APPEND_OBSERVABLES if append else 0) | (_native.BIT_PACKED if bit_packed else 0)
        if shots:
            check(lib().gfs_m2d_convert(
                self._h, shots, _ptr(m) if m.size else None, max(1, m.shape[1]),
                _ptr(sw) if sw is not None and sw.size else None, max(1, sw.shape[1]) if sw is not None else 0,
                flags, _ptr(dets) if dets.size else None, max(1, dets.shape[1]),
                _ptr(obs) if obs is not None and obs.size else None, max(1, obs.shape[1]) if obs is not None else 0))
        if dets_user is not None:
            dets_user[...] = dets
            dets = dets_user
        if obs_user is not None:
            obs_user[...] = obs
            obs = obs_user
        if separate:
            return dets, obs
        return dets


    def convert_file(self, *, measurements_filepath, measurements_format: str = "01", sweep_bits_filepath=None,
                     sweep_bits_format: str = "01", detection_events_filepath, detection_events_format: str = "01",
                     append_observables: bool = False, obs_out_filepath=None, obs_out_format: str = "01") -> None:
        """Reads measurement data from a file and writes detection events to another file, as the reference's
        convert_file does (measurements_to_detection_events.pybind.cc:45-77, 211-222); formats "01", "b8", "r8",
        "ptb64", "hits", "dets"."""
        check(lib().gfs_m2d_convert_file(
            self._h, _path(measurements_filepath), str(measurements_format).encode(),
            _path(sweep_bits_filepath) if sweep_bits_filepath is not None else None,
            str(sweep_bits_format).encode(), _path(detection_events_filepath),
            str(detection_events_format).encode(), 1 if append_observables else 0,
            _path(obs_out_filepath) if obs_out_filepath is not None else None, str(obs_out_format).encode()))


class DetectorErrorModel:
    """A detector error model in the reference's text format (parsed and validated by the library's C++ host
    code; src/stim/dem/detector_error_model.cc:195-360)."""

    def __init__(self, text: str = ""):
        if not isinstance(text, str):
            text = str(text)
        self._text = text
        s = (ctypes.c_uint64 * 3)()
        data = text.encode()
        check(lib().gfs_dem_parse_stats(data, len(data), s))
        self.num_detectors, self.num_observables, self.num_errors = [int(v) for v in s]

    def __str__(self):
        return self._text

    def __repr__(self):
        return f"stim_gb300.DetectorErrorModel({self._text!r})"

    def compile_sampler(self, *, seed=None, device: int = 0) -> "CompiledDemSampler":
        return CompiledDemSampler(self, seed=seed, device=device)


class CompiledDemSampler:
    """Samples detection events, observable flips and (optionally) the errors themselves from a detector error
    model on the GPU (replaces the reference's DemSampler, src/stim/simulators/dem_sampler.pybind.cc:40-80).
    Draws follow the counter-based contract of csrc/gfs_contract.h (purpose DEM), not the reference's
    mt19937_64 stream; replayed errors give exactly the reference's symptoms."""

    def __init__(self, dem, *, seed=None, device: int = 0):
        if not isinstance(dem, DetectorErrorModel):
            dem = DetectorErrorModel(str(dem))
        self._dem = dem
        data = dem._text.encode()
        h = ctypes.c_void_p()
        check(lib().gfs_dem_create(data, len(data), _seed_value(seed), int(device), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_dem_free(h)
            self._h = None

    @property
    def num_detectors(self):
        return self._dem.num_detectors

    @property
    def num_observables(self):
        return self._dem.num_observables

    @property
    def num_errors(self):
        return self._dem.num_errors

    def sample(self, shots: int, *, bit_packed: bool = False, return_errors: bool = False,
               recorded_errors_to_replay=None, dets_out=None, obs_out=None):
        """As the reference's sample; dets_out / obs_out (optional, no counterpart in the reference) are
        caller-owned arrays of the result's shape and dtype, reused across calls."""
        shots = int(shots)
        if shots < 0:
            raise ValueError("shots must be non-negative")
        D, O, E = self.num_detectors, self.num_observables, self.num_errors
        width = (lambda n: (n + 7) // 8) if bit_packed else (lambda n: n)
        dtype = np.uint8 if bit_packed else np.bool_
        dets, dets_user = _out_array(dets_out, (shots, width(D)), bit_packed)
        obs, obs_user = _out_array(obs_out, (shots, width(O)), bit_packed)
        errs = np.empty((shots, width(E)), dtype=dtype) if return_errors else None
        replay = None
        if recorded_errors_to_replay is not None:
            replay = CompiledMeasurementsToDetectionEventsConverter._packed(recorded_errors_to_replay, E,
                                                                             "recorded_errors_to_replay")
            if replay.shape[0] != shots:
                raise ValueError("recorded_errors_to_replay.shape[0] != shots")
        if shots:
            check(lib().gfs_dem_sample(
                self._h, shots, _native.BIT_PACKED if bit_packed else 0,
                _ptr(dets) if dets.size else None, max(1, dets.shape[1]),
                _ptr(obs) if obs.size else None, max(1, obs.shape[1]),
                _ptr(errs) if errs is not None and errs.size else None, max(1, errs.shape[1]) if errs is not None else 0,
                _ptr(replay) if replay is not None and replay.size else None,
                max(1, replay.shape[1]) if replay is not None else 0))
        if dets_user is not None:
            dets_user[...] = dets
            dets = dets_user
        if obs_user is not None:
            obs_user[...] = obs
            obs = obs_user
        return dets, obs, errs

    def sample_write(self, shots: int, *, det_out_file, det_out_format: str = "01", obs_out_file,
                     obs_out_format: str = "01", err_out_file=None, err_out_format: str = "01",
                     replay_err_in_file=None, replay_err_in_format: str = "01") -> None:
        """As the reference's DemSampler.sample_write (dem_sampler.pybind.cc:274-380, dem_sampler.inl:75-130):
        detection events (D<k>), observable flips (L<k>) and the sampled errors (M<k>) to files (None: not
        written), optionally replaying errors read from a file.  Works in chunks of shots, each written after the
        previous one, so memory stays bounded whatever the shot count."""
        shots = int(shots)
        if shots < 0:
            raise ValueError("shots must be non-negative")
        D, O, E = self.num_detectors, self.num_observables, self.num_errors
        replay = None
        if replay_err_in_file is not None:
            replay = read_shot_data_file(path=replay_err_in_file, format=replay_err_in_format, num_measurements=E,
                                         bit_packed=True)
            if replay.shape[0] < shots:
                raise ValueError("Expected more error data for the requested number of shots.")
        outs = [(det_out_file, det_out_format, dict(num_detectors=D)),
                (obs_out_file, obs_out_format, dict(num_observables=O)),
                (err_out_file, err_out_format, dict(num_measurements=E))]
        if any(f is not None and str(fmt) == "ptb64" for f, fmt, _ in outs) and shots % 64:
            raise ValueError("shots must be a multiple of 64 to use ptb64 format.")
        for f, _, _ in outs:
            if f is not None:
                open(os.fspath(f), "wb").close()
        chunk = max(64, min(1 << 20, ((256 << 23) // max(1, D + O + E)) // 64 * 64))
        with tempfile.TemporaryDirectory() as tmp:
            part = os.path.join(tmp, "part")
            for done in range(0, shots, chunk):
                cs = min(chunk, shots - done)
                d, o, e = self.sample(cs, bit_packed=True, return_errors=err_out_file is not None,
                                      recorded_errors_to_replay=None if replay is None else replay[done:done + cs])
                for (f, fmt, counts), data in zip(outs, (d, o, e)):
                    if f is None:
                        continue
                    write_shot_data_file(data=data, path=part, format=fmt, **counts)
                    with open(part, "rb") as src, open(os.fspath(f), "ab") as dst:
                        shutil.copyfileobj(src, dst)


class BatchSampler:
    """The next shots of many detection samplers in one persistent kernel launch (replayed as a CUDA graph).

    Entry j of a call returns exactly what ``samplers[j].sample(shots[j], ...)`` would have returned at that
    point and advances that sampler the same way.  No counterpart in the reference, where each circuit has
    its own CompiledDetectorSampler (compiled_detector_sampler.pybind.cc:216-322).
    """

    def __init__(self, samplers):
        self._samplers = list(samplers)
        if not self._samplers:
            raise ValueError("a batch needs at least one sampler")
        for s in self._samplers:
            if not isinstance(s, CompiledDetectorSampler):
                raise ValueError("BatchSampler takes CompiledDetectorSampler objects")
        arr = (ctypes.c_void_p * len(self._samplers))(*[s._h.value for s in self._samplers])
        h = ctypes.c_void_p()
        check(lib().gfs_batch_create(arr, len(self._samplers), ctypes.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_batch_free(h)
            self._h = None

    def __len__(self):
        return len(self._samplers)

    def _shots(self, shots):
        shots = [int(x) for x in shots]
        if len(shots) != len(self._samplers):
            raise ValueError("need one shot count per sampler")
        if any(x < 0 for x in shots):
            raise ValueError("shots must be non-negative")
        return (ctypes.c_uint64 * len(shots))(*shots), shots

    def _rows(self, flags_packed, prepend, append):
        out = []
        for s in self._samplers:
            c = s._circuit
            D, O = c.num_detectors, c.num_observables
            nd = D + (O if prepend else 0) + (O if append else 0)
            out.append(((nd + 7) // 8, (O + 7) // 8) if flags_packed else (nd, O))
        return out

    def sample(self, shots, *, bit_packed: bool = False, prepend_observables: bool = False,
               append_observables: bool = False, separate_observables: bool = False):
        """Returns a list with one entry per sampler, shaped like CompiledDetectorSampler.sample's result."""
        if separate_observables and (append_observables or prepend_observables):
            raise ValueError("Can't specify separate_observables=True with append_observables=True or "
                             "prepend_observables=True")
        cshots, shots = self._shots(shots)
        n = len(shots)
        rows = self._rows(bit_packed, prepend_observables, append_observables)
        dtype = np.uint8 if bit_packed else np.bool_
        dets = [np.empty((k, r[0]), dtype=dtype) for k, r in zip(shots, rows)]
        obs = [np.empty((k, r[1]), dtype=dtype) for k, r in zip(shots, rows)] if separate_observables else None
        flags = ((_native.PREPEND_OBSERVABLES if prepend_observables else 0)
                 | (_native.APPEND_OBSERVABLES if append_observables else 0)
                 | (_native.BIT_PACKED if bit_packed else 0))
        dptr = (ctypes.c_void_p * n)(*[d.ctypes.data if d.size else None for d in dets])
        dstr = (ctypes.c_uint64 * n)(*[max(1, d.strides[0]) if d.size else max(1, d.shape[1]) for d in dets])
        if obs is not None:
            optr = (ctypes.c_void_p * n)(*[o.ctypes.data if o.size else None for o in obs])
            ostr = (ctypes.c_uint64 * n)(*[max(1, o.strides[0]) if o.size else max(1, o.shape[1]) for o in obs])
        else:
            optr = ostr = None
        check(lib().gfs_batch_sample_detections(self._h, cshots, flags, dptr, dstr, optr, ostr))
        if separate_observables:
            return list(zip(dets, obs))
        return dets

    def sample_device(self, shots, dets_ptrs, dets_strides, obs_ptrs=None, obs_strides=None, *,
                      bit_packed: bool = True, prepend_observables: bool = False, append_observables: bool = False):
        """Writes each circuit's shot-major rows to caller-owned device buffers (raw device pointers)."""
        cshots, shots = self._shots(shots)
        n = len(shots)
        flags = ((_native.PREPEND_OBSERVABLES if prepend_observables else 0)
                 | (_native.APPEND_OBSERVABLES if append_observables else 0)
                 | (_native.BIT_PACKED if bit_packed else 0))
        dptr = (ctypes.c_void_p * n)(*[int(p) if p else None for p in dets_ptrs])
        dstr = (ctypes.c_uint64 * n)(*[int(x) for x in dets_strides])
        optr = ostr = None
        if obs_ptrs is not None:
            optr = (ctypes.c_void_p * n)(*[int(p) if p else None for p in obs_ptrs])
            ostr = (ctypes.c_uint64 * n)(*[int(x) for x in obs_strides])
        check(lib().gfs_batch_sample_detections_device(self._h, cshots, flags, dptr, dstr, optr, ostr))

    def set_launch_shape(self, blocks_per_cta: int, threads: int = 256, ring_placement: int = -1):
        check(lib().gfs_batch_set_shape(self._h, int(blocks_per_cta), int(threads), int(ring_placement)))

    def launch_shape(self):
        b, t, g, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        sm = ctypes.c_uint64()
        check(lib().gfs_batch_get_shape(self._h, ctypes.byref(b), ctypes.byref(t), ctypes.byref(g),
                                        ctypes.byref(sm), ctypes.byref(r)))
        return {"blocks_per_cta": b.value, "threads": t.value, "grid": g.value, "smem_bytes": sm.value,
                "ring_global": bool(r.value)}

    def autotune(self, shots) -> float:
        """Times each candidate launch shape on these shot counts and keeps the fastest; returns its ms."""
        cshots, _ = self._shots(shots)
        ms = ctypes.c_double()
        check(lib().gfs_batch_autotune(self._h, cshots, ctypes.byref(ms)))
        return ms.value

    def last_timings(self):
        t = (ctypes.c_double * 4)()
        c = (ctypes.c_uint64 * 4)()
        check(lib().gfs_batch_last_timings(self._h, t, c))
        return {"frame_ms": t[0], "transpose_ms": t[1], "copy_ms": t[2], "total_ms": t[3],
                "frame_launches": int(c[0]), "transpose_launches": int(c[1]), "graph_launches": int(c[2]),
                "graph_builds": int(c[3])}


class ServerRequest:
    """A submitted request; ``result()`` waits and returns what
    ``Circuit(text).compile_detector_sampler(seed=seed).sample(shots, ...)`` returns."""

    def __init__(self, server, ticket, dets, obs, separate):
        self._server = server
        self._ticket = ticket
        self._dets = dets
        self._obs = obs
        self._separate = separate
        self._done = False
        self.latency_ms = None

    def done(self, timeout: float = 0.0) -> bool:
        if not self._done:
            d = ctypes.c_int()
            lat = ctypes.c_double()
            check(lib().gfs_server_wait(self._server._h, self._ticket, float(timeout), ctypes.byref(d),
                                        ctypes.byref(lat)))
            if d.value:
                self._done = True
                self.latency_ms = lat.value
        return self._done

    def result(self, timeout: float = -1.0):
        if not self.done(timeout):
            raise TimeoutError("request not finished")
        if self._dets is None:
            return None
        if self._separate:
            return self._dets, self._obs
        return self._dets


class Server:
    """Continuous-batching request server on one device (see gfs_server_* in include/stim_gb300.h)."""

    def __init__(self, device: int = 0, hbm_budget: int = 8 << 30, max_chunk_shots: int = 1 << 18):
        h = ctypes.c_void_p()
        check(lib().gfs_server_create(int(device), int(hbm_budget), int(max_chunk_shots), ctypes.byref(h)))
        self._h = h
        self._texts = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            lib().gfs_server_free(h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _text(self, circuit):
        t = circuit if isinstance(circuit, (str, bytes)) else str(circuit)
        return t.encode() if isinstance(t, str) else t

    def submit(self, circuit, shots: int, *, seed: int, bit_packed: bool = False, prepend_observables: bool = False,
               append_observables: bool = False, separate_observables: bool = False, num_detectors: int = None,
               num_observables: int = None) -> ServerRequest:
        """Queues a detection-sampling request with host (numpy) results."""
        if separate_observables and (append_observables or prepend_observables):
            raise ValueError("Can't specify separate_observables=True with append_observables=True or "
                             "prepend_observables=True")
        text = self._text(circuit)
        if num_detectors is None or num_observables is None:
            c = circuit if isinstance(circuit, Circuit) else self._texts.get(text)
            if c is None:
                c = Circuit(text.decode())
                self._texts[text] = c
            num_detectors, num_observables = c.num_detectors, c.num_observables
        D, O = int(num_detectors), int(num_observables)
        nd = D + (O if prepend_observables else 0) + (O if append_observables else 0)
        width = (lambda n: (n + 7) // 8) if bit_packed else (lambda n: n)
        dtype = np.uint8 if bit_packed else np.bool_
        shots = int(shots)
        dets = np.empty((shots, width(nd)), dtype=dtype)
        obs = np.empty((shots, width(O)), dtype=dtype) if separate_observables else None
        flags = ((_native.PREPEND_OBSERVABLES if prepend_observables else 0)
                 | (_native.APPEND_OBSERVABLES if append_observables else 0)
                 | (_native.BIT_PACKED if bit_packed else 0))
        t = ctypes.c_uint64()
        check(lib().gfs_server_submit(
            self._h, text, len(text), shots, _seed_value(seed), flags, 0,
            _ptr(dets) if dets.size else None, max(1, dets.strides[0]) if dets.size else max(1, dets.shape[1]),
            (_ptr(obs) if obs.size else None) if obs is not None else None,
            (max(1, obs.strides[0]) if obs.size else max(1, obs.shape[1])) if obs is not None else 0,
            ctypes.byref(t)))
        return ServerRequest(self, t.value, dets, obs, separate_observables)

    def submit_device(self, circuit, shots: int, *, seed: int, dets_ptr: int, dets_stride: int, obs_ptr: int = 0,
                      obs_stride: int = 0, bit_packed: bool = True) -> ServerRequest:
        """Queues a request whose bit-packed (or unpacked) results go to caller-owned device memory."""
        text = self._text(circuit)
        t = ctypes.c_uint64()
        check(lib().gfs_server_submit(self._h, text, len(text), int(shots), _seed_value(seed),
                                      _native.BIT_PACKED if bit_packed else 0, 1, int(dets_ptr) or None,
                                      int(dets_stride), int(obs_ptr) or None, int(obs_stride), ctypes.byref(t)))
        return ServerRequest(self, t.value, None, None, False)

    def stats(self) -> dict:
        o = (ctypes.c_double * 12)()
        check(lib().gfs_server_stats(self._h, o))
        keys = ["completed", "failed", "p50_ms", "p99_ms", "gbits", "batches", "chunks_per_batch", "cache_hits",
                "cache_misses", "max_queue", "bits", "seconds"]
        return dict(zip(keys, list(o)))

    def counters(self) -> dict:
        """Admission counters: submitted, rejected (at submission), completed, failed, queued (now), pending (not
        finished), max_queue, chunks_admitted."""
        o = (ctypes.c_uint64 * 8)()
        check(lib().gfs_server_counters(self._h, o))
        keys = ["submitted", "rejected", "completed", "failed", "queued", "pending", "max_queue", "chunks_admitted"]
        return dict(zip(keys, [int(v) for v in o]))
