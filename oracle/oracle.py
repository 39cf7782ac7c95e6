"""ctypes binding of the CPU oracle (oracle/stim_oracle.c).

Test infrastructure only: imported by tests/, by __graft_entry__.smoke() as the checker, and by
bench.py's CPU-baseline leg.  The product package never imports this module.
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the committed Makefile (plain gcc, no reference sources needed)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE, _LIB_PATH], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_parse.restype = ctypes.c_void_p
        L.oracle_parse.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_sample.restype = ctypes.c_int
        L.oracle_sample.argtypes = [
            ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t,
        ]
        L.oracle_m2d.restype = ctypes.c_int
        L.oracle_m2d.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_dem_parse.restype = ctypes.c_void_p
        L.oracle_dem_parse.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.oracle_dem_free.argtypes = [ctypes.c_void_p]
        L.oracle_dem_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_dem_sample.restype = ctypes.c_int
        L.oracle_dem_sample.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


class OracleCircuit:
    """A parsed circuit in the oracle."""

    def __init__(self, text: str):
        err = ctypes.create_string_buffer(512)
        self._h = lib().oracle_parse(text.encode(), err, 512)
        if not self._h:
            raise ValueError(err.value.decode())
        s = (ctypes.c_uint64 * 6)()
        lib().oracle_stats(self._h, s)
        (self.num_qubits, self.num_measurements, self.num_detectors,
         self.num_observables, self.max_lookback, self.num_instances) = [int(v) for v in s]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_free(self._h)
            self._h = None

    def sample(self, shots: int, seed: int, *, first_shot: int = 0, threads: int = 1,
               dets: bool = True, obs: bool = True, meas: bool = False):
        """Returns (dets, obs, meas) as shot-major bit-packed uint8 arrays (None where not asked)."""

        def buf(n, want):
            if not want:
                return None
            return np.zeros((shots, (n + 7) // 8), dtype=np.uint8)

        d = buf(self.num_detectors, dets)
        o = buf(self.num_observables, obs)
        m = buf(self.num_measurements, meas)
        err = ctypes.create_string_buffer(512)

        def ptr(a):
            return None if a is None else a.ctypes.data_as(ctypes.c_void_p)

        rc = lib().oracle_sample(self._h, seed & (2**64 - 1), first_shot, shots, threads,
                                 ptr(d), ptr(o), ptr(m), err, 512)
        if rc != 0:
            raise ValueError(err.value.decode())
        return d, o, m

    def m2d(self, meas_packed, ref_sample_packed=None):
        """Detection events and observable flips (bit-packed) of bit-packed measurement rows."""
        meas = np.ascontiguousarray(meas_packed, dtype=np.uint8)
        shots = meas.shape[0]
        d = np.zeros((shots, (self.num_detectors + 7) // 8), dtype=np.uint8)
        o = np.zeros((shots, (self.num_observables + 7) // 8), dtype=np.uint8)
        ref = None if ref_sample_packed is None else np.ascontiguousarray(ref_sample_packed, dtype=np.uint8)
        err = ctypes.create_string_buffer(512)

        def ptr(a):
            return None if a is None or a.size == 0 else a.ctypes.data_as(ctypes.c_void_p)

        rc = lib().oracle_m2d(self._h, shots, ptr(meas), ptr(ref), ptr(d), ptr(o), err, 512)
        if rc != 0:
            raise ValueError(err.value.decode())
        return d, o


class OracleDem:
    """A detector error model parsed by the oracle."""

    def __init__(self, text: str):
        err = ctypes.create_string_buffer(512)
        self._h = lib().oracle_dem_parse(text.encode(), err, 512)
        if not self._h:
            raise ValueError(err.value.decode())
        s = (ctypes.c_uint64 * 3)()
        lib().oracle_dem_stats(self._h, s)
        self.num_detectors, self.num_observables, self.num_errors = [int(v) for v in s]

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_dem_free(self._h)
            self._h = None

    def sample(self, shots: int, seed: int = 0, *, first_shot: int = 0, errors: bool = False, replay=None):
        """(dets, obs, errs) bit-packed; replay = bit-packed recorded errors (then seed is unused)."""
        d = np.zeros((shots, (self.num_detectors + 7) // 8), dtype=np.uint8)
        o = np.zeros((shots, (self.num_observables + 7) // 8), dtype=np.uint8)
        e = np.zeros((shots, (self.num_errors + 7) // 8), dtype=np.uint8) if errors else None
        r = None if replay is None else np.ascontiguousarray(replay, dtype=np.uint8)

        def ptr(a):
            return None if a is None or a.size == 0 else a.ctypes.data_as(ctypes.c_void_p)

        lib().oracle_dem_sample(self._h, seed & (2**64 - 1), first_shot, shots, ptr(d), ptr(o), ptr(e), ptr(r))
        return d, o, e
