"""ctypes binding of libstim_gb300.so (include/stim_gb300.h).

The product path has exactly one implementation: the CUDA library.  If it cannot be built or loaded,
or there is no CUDA device, calls raise; there is no CPU fallback.
"""

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
_lock = threading.Lock()
_lib = None

GFS_OK = 0
GFS_ERR_INVALID_ARGUMENT = 1
GFS_ERR_OUT_OF_RANGE = 2
GFS_ERR_CUDA = 3
GFS_ERR_OUT_OF_MEMORY = 4
GFS_ERR_INTERNAL = 5

MODE_DETECTIONS = 0
MODE_MEASUREMENTS = 1

PREPEND_OBSERVABLES = 1
APPEND_OBSERVABLES = 2
BIT_PACKED = 4

_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64


def _declare(L):
    L.gfs_last_error.restype = ctypes.c_char_p
    L.gfs_last_error.argtypes = []
    sigs = {
        "gfs_device_count": [ctypes.POINTER(ctypes.c_int)],
        "gfs_device_info": [ctypes.c_int, ctypes.POINTER(ctypes.c_int64)],
        "gfs_circuit_parse": [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_vp)],
        "gfs_circuit_stats": [_vp, ctypes.POINTER(_u64)],
        "gfs_program_info": [_vp, ctypes.c_uint32, ctypes.POINTER(_u64)],
        "gfs_circuit_reference_sample": [_vp, _vp, _u64],
        "gfs_sample_write_detections": [_vp, _u64, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint32,
                                        ctypes.c_char_p, ctypes.c_char_p],
        "gfs_sample_write_measurements": [_vp, _u64, ctypes.c_char_p, ctypes.c_char_p, _vp],
        "gfs_program_noise": [_vp, ctypes.c_uint32, ctypes.POINTER(_u64), ctypes.POINTER(ctypes.c_double)],
        "gfs_sampler_create": [_vp, ctypes.c_uint32, _u64, ctypes.c_int, ctypes.POINTER(_vp)],
        "gfs_sample_detections": [_vp, _u64, ctypes.c_uint32, _vp, _u64, _vp, _u64],
        "gfs_sample_detections_device": [_vp, _u64, ctypes.c_uint32, _vp, _u64, _vp, _u64],
        "gfs_sample_detections_device_noalloc": [_vp, _u64, ctypes.c_uint32, _vp, _u64, _vp, _u64],
        "gfs_sample_for_decoder": [_vp, _u64, _vp, _vp, _u64, _vp, _u64, ctypes.POINTER(_u64)],
        "gfs_sample_measurements": [_vp, _u64, ctypes.c_uint32, _vp, _vp, _u64],
        "gfs_sampler_last_timings": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_u64)],
        "gfs_sampler_set_shape": [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        "gfs_sampler_get_shape": [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_u64)],
        "gfs_sampler_set_chunk_shots": [_vp, _u64],
        "gfs_sampler_set_stream_position": [_vp, _u64],
        "gfs_sampler_get_stream_position": [_vp, ctypes.POINTER(_u64)],
        "gfs_sampler_set_ring_placement": [_vp, ctypes.c_int],
        "gfs_measure_smem_peak": [ctypes.c_int, ctypes.POINTER(ctypes.c_double)],
        "gfs_measure_int_peaks": [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)],
        "gfs_sampler_autotune": [_vp, _u64, ctypes.POINTER(ctypes.c_double)],
        "gfs_sampler_set_noise_mode": [_vp, ctypes.c_int],
        "gfs_sampler_set_frame_kernel": [_vp, ctypes.c_int],
        "gfs_sampler_get_frame_kernel": [_vp, ctypes.POINTER(ctypes.c_int)],
        "gfs_sampler_set_hit_capacity": [_vp, _u64],
        "gfs_sampler_last_noise_ms": [_vp, ctypes.POINTER(ctypes.c_double)],
        "gfs_sampler_last_counts": [_vp, ctypes.POINTER(_u64)],
        "gfs_batch_create": [ctypes.POINTER(_vp), ctypes.c_size_t, ctypes.POINTER(_vp)],
        "gfs_batch_sample_detections_device": [_vp, ctypes.POINTER(_u64), ctypes.c_uint32, ctypes.POINTER(_vp),
                                               ctypes.POINTER(_u64), ctypes.POINTER(_vp), ctypes.POINTER(_u64)],
        "gfs_batch_sample_detections": [_vp, ctypes.POINTER(_u64), ctypes.c_uint32, ctypes.POINTER(_vp),
                                        ctypes.POINTER(_u64), ctypes.POINTER(_vp), ctypes.POINTER(_u64)],
        "gfs_batch_set_shape": [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int],
        "gfs_batch_get_shape": [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_u64), ctypes.POINTER(ctypes.c_int)],
        "gfs_batch_autotune": [_vp, ctypes.POINTER(_u64), ctypes.POINTER(ctypes.c_double)],
        "gfs_batch_last_timings": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_u64)],
        "gfs_server_create": [ctypes.c_int, _u64, _u64, ctypes.POINTER(_vp)],
        "gfs_server_submit": [_vp, ctypes.c_char_p, ctypes.c_size_t, _u64, _u64, ctypes.c_uint32, ctypes.c_int,
                              _vp, _u64, _vp, _u64, ctypes.POINTER(_u64)],
        "gfs_server_wait": [_vp, _u64, ctypes.c_double, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)],
        "gfs_server_stats": [_vp, ctypes.POINTER(ctypes.c_double)],
        "gfs_server_counters": [_vp, ctypes.POINTER(_u64)],
        "gfs_m2d_create": [_vp, _vp, ctypes.c_int, ctypes.POINTER(_vp)],
        "gfs_m2d_stats": [_vp, ctypes.POINTER(_u64)],
        "gfs_m2d_convert": [_vp, _u64, _vp, _u64, _vp, _u64, ctypes.c_uint32, _vp, _u64, _vp, _u64],
        "gfs_read_shot_data_file": [ctypes.c_char_p, ctypes.c_char_p, _u64, _u64, _u64, _vp, _u64,
                                    ctypes.POINTER(_u64)],
        "gfs_write_shot_data_file": [_vp, _u64, _u64, ctypes.c_char_p, ctypes.c_char_p, _u64, _u64, _u64],
        "gfs_m2d_convert_file": [_vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                 ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p],
        "gfs_dem_parse_stats": [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_u64)],
        "gfs_dem_create": [ctypes.c_char_p, ctypes.c_size_t, _u64, ctypes.c_int, ctypes.POINTER(_vp)],
        "gfs_dem_sample": [_vp, _u64, ctypes.c_uint32, _vp, _u64, _vp, _u64, _vp, _u64, _vp, _u64],
    }
    for name, args in sigs.items():
        f = getattr(L, name)
        f.restype = ctypes.c_int
        f.argtypes = args
    for name in ("gfs_circuit_free", "gfs_sampler_free", "gfs_batch_free", "gfs_server_free", "gfs_m2d_free",
                 "gfs_dem_free"):
        f = getattr(L, name)
        f.restype = None
        f.argtypes = [_vp]


def library_path() -> str:
    return os.path.join(_HERE, "_lib", "libstim_gb300.so")


def lib():
    """Loads (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            from . import build as _build
            path = _build.build()
            L = ctypes.CDLL(path)
            _declare(L)
            _lib = L
    return _lib


def check(status: int):
    if status == GFS_OK:
        return
    msg = lib().gfs_last_error().decode(errors="replace")
    if status == GFS_ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == GFS_ERR_OUT_OF_RANGE:
        raise IndexError(msg)
    if status == GFS_ERR_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def measure_smem_peak(device: int = 0) -> float:
    """Shared-memory load+store bytes/s of the device, from the library's probe kernel."""
    v = ctypes.c_double(0)
    check(lib().gfs_measure_smem_peak(int(device), ctypes.byref(v)))
    return v.value


def measure_int_peaks(device: int = 0) -> dict:
    """Integer-issue peaks of the device from the library's probe kernels: 32-bit lop3 ops/s and Philox4x32-10
    calls/s."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    check(lib().gfs_measure_int_peaks(int(device), ctypes.byref(a), ctypes.byref(b)))
    return {"lop3_per_s": a.value, "philox_per_s": b.value}


def device_info(device: int = 0) -> dict:
    v = (ctypes.c_int64 * 8)()
    check(lib().gfs_device_info(int(device), v))
    keys = ["sms", "smem_per_cta_optin", "smem_per_sm", "pageable_memory_access",
            "pageable_uses_host_page_tables", "sm_clock_khz", "cc", "l2_bytes"]
    return dict(zip(keys, [int(x) for x in v]))


def device_count() -> int:
    n = ctypes.c_int(0)
    check(lib().gfs_device_count(ctypes.byref(n)))
    return n.value
