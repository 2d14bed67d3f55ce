"""ctypes binding of libmmcgb.so (the C ABI declared in include/mmcgb.h).

The library is loaded from ``mmc_gb300/lib`` only; there is no CPU fallback.
If the shared library is missing, loading raises ``NativeLibraryError`` so that
a GPU path never silently degrades.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

_LIBPATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libmmcgb.so")
_lock = threading.Lock()
_lib = None


class NativeLibraryError(RuntimeError):
    pass


class MmcgbError(RuntimeError):
    """A non-zero mmcgb_status, with the library's message."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"mmcgb error {code}: {msg}")
        self.code = code


STATUS = {0: "OK", 1: "E_ARG", 2: "E_CUDA", 3: "E_MESH", 4: "E_SOURCE", 5: "E_BUDGET", 6: "E_NOMEM"}


class MeshDesc(C.Structure):
    _fields_ = [
        ("nn", C.c_int32), ("ne", C.c_int32),
        ("node", C.c_void_p), ("elem", C.c_void_p), ("label", C.c_void_p), ("facenb", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [
        ("nphoton", C.c_uint64), ("photon_offset", C.c_uint64), ("seed", C.c_uint64),
        ("srcpos", C.c_float * 3), ("srcdir", C.c_float * 3),
        ("srctype", C.c_int32), ("e0", C.c_int32),
        ("tstart", C.c_float), ("tend", C.c_float), ("tstep", C.c_float),
        ("isreflect", C.c_int32), ("isspecular", C.c_int32), ("voidtime", C.c_int32),
        ("issavedet", C.c_int32), ("issaveseed", C.c_int32), ("issaveexit", C.c_int32),
        ("ismomentum", C.c_int32),
        ("minenergy", C.c_float), ("roulettesize", C.c_float), ("nout", C.c_float), ("unitinmm", C.c_float),
        ("outputtype", C.c_int32), ("basisorder", C.c_int32), ("isnormalized", C.c_int32),
        ("maxdetphoton", C.c_uint32),
        ("nmedia", C.c_int32), ("media", C.c_void_p),
        ("detnum", C.c_int32), ("detpos", C.c_void_p),
        ("replayseed", C.c_void_p), ("replayweight", C.c_void_p), ("replaytime", C.c_void_p),
        ("accum_f64", C.c_int32), ("step_budget", C.c_uint64),
        ("threads", C.c_int32), ("blocks", C.c_int32), ("fast_math", C.c_int32), ("phased", C.c_int32),
        ("srcparam1", C.c_float * 4), ("srcparam2", C.c_float * 4), ("focus", C.c_float), ("srcpattern", C.c_void_p),
        ("issaveref", C.c_int32), ("method", C.c_int32), ("gridstep", C.c_float), ("maxjumpdebug", C.c_uint32),
        ("phase_chunk", C.c_uint64), ("accumulate", C.c_int32), ("srcnum", C.c_int32),
        ("nodemua", C.c_void_p), ("nodemusp", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("field", C.c_void_p), ("detp", C.c_void_p), ("seeds", C.c_void_p),
        ("photon_weight", C.c_void_p), ("photon_steps", C.c_void_p), ("photon_det", C.c_void_p),
        ("detected", C.c_uint32), ("saved", C.c_uint32), ("reclen", C.c_int32), ("maxgate", C.c_int32),
        ("energytot", C.c_double), ("energyesc", C.c_double), ("normalizer", C.c_double),
        ("raytet", C.c_uint64), ("aborted", C.c_uint64), ("outside", C.c_uint64), ("traj", C.c_void_p),
        ("ntraj", C.c_uint32), ("dref", C.c_void_p),
        ("kernel_ms", C.c_float), ("energy_src", C.c_void_p),
    ]


class DeviceOut(C.Structure):
    _fields_ = [("field_raw", C.c_void_p), ("detp", C.c_void_p), ("seeds", C.c_void_p),
                ("detcount", C.c_void_p), ("energy", C.c_void_p), ("counters", C.c_void_p),
                ("energy_src", C.c_void_p)]


EXPORTS = [
    "mmcgb_abi_version", "mmcgb_last_error", "mmcgb_config_defaults", "mmcgb_mesh_create",
    "mmcgb_mesh_destroy", "mmcgb_mesh_info", "mmcgb_mesh_export", "mmcgb_mesh_locate",
    "mmcgb_simulate", "mmcgb_simulate_batch", "mmcgb_run", "mmcgb_session_begin", "mmcgb_session_launch",
    "mmcgb_session_sync", "mmcgb_session_end", "mmcgb_prepare_host", "mmcgb_normalize_host",
    "mmcgb_session_launch_batch", "mmcgb_session_stream", "mmcgb_session_launch_batch_on",
    "mmcgb_session_launch_repeat", "mmcgb_grid_info", "mmcgb_check_config",
    "mmcgb_session_device_buffers", "mmcgb_l2_read_bandwidth", "mmcgb_session_phase_window",
    "mmcgb_session_launch_batches",
]


def library_path() -> str:
    return _LIBPATH


def load():
    """Loads libmmcgb.so (building nothing); raises NativeLibraryError if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(_LIBPATH):
            raise NativeLibraryError(
                f"{_LIBPATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(_LIBPATH)
        lib.mmcgb_abi_version.restype = C.c_int32
        lib.mmcgb_last_error.restype = C.c_char_p
        lib.mmcgb_config_defaults.argtypes = [C.POINTER(Config)]
        lib.mmcgb_config_defaults.restype = None
        lib.mmcgb_mesh_create.argtypes = [C.POINTER(MeshDesc), C.c_int32, C.POINTER(C.c_void_p)]
        lib.mmcgb_mesh_destroy.argtypes = [C.c_void_p]
        lib.mmcgb_mesh_info.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        lib.mmcgb_mesh_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.mmcgb_mesh_locate.argtypes = [C.c_void_p, C.POINTER(C.c_float * 3)]
        lib.mmcgb_simulate.argtypes = [C.c_void_p, C.POINTER(Config), C.POINTER(Result)]
        lib.mmcgb_simulate_batch.argtypes = [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(Config), C.POINTER(Result)]
        lib.mmcgb_run.argtypes = [C.POINTER(MeshDesc), C.POINTER(Config), C.c_int32, C.POINTER(Result)]
        lib.mmcgb_session_begin.argtypes = [C.c_void_p, C.POINTER(Config), C.c_void_p, C.POINTER(C.c_void_p)]
        lib.mmcgb_session_launch.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
        lib.mmcgb_session_sync.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        lib.mmcgb_session_end.argtypes = [C.c_void_p, C.c_void_p]
        lib.mmcgb_prepare_host.argtypes = [C.POINTER(MeshDesc)] + [C.c_void_p] * 6
        lib.mmcgb_normalize_host.argtypes = [C.POINTER(MeshDesc), C.POINTER(Config), C.c_void_p, C.c_double,
                                             C.c_double, C.c_void_p, C.POINTER(C.c_double)]
        lib.mmcgb_session_stream.argtypes = [C.c_void_p]
        lib.mmcgb_session_stream.restype = C.c_void_p
        lib.mmcgb_session_launch_batch.argtypes = [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                                   C.POINTER(C.c_uint64)]
        lib.mmcgb_session_launch_batch_on.argtypes = [C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_uint64),
                                                      C.POINTER(C.c_uint64), C.c_void_p]
        lib.mmcgb_session_launch_repeat.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_int32]
        lib.mmcgb_session_launch_batches.argtypes = [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_void_p),
                                                     C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_void_p]
        lib.mmcgb_session_phase_window.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_int32),
                                                    C.POINTER(C.c_uint64)]
        lib.mmcgb_l2_read_bandwidth.argtypes = [C.c_int32, C.c_uint64, C.c_int32, C.POINTER(C.c_double)]
        lib.mmcgb_session_device_buffers.argtypes = [C.c_void_p, C.POINTER(DeviceOut)]
        lib.mmcgb_check_config.argtypes = [C.POINTER(MeshDesc), C.POINTER(Config), C.POINTER(C.c_int32)]
        lib.mmcgb_grid_info.argtypes = [C.c_void_p, C.c_float, C.POINTER(C.c_int32), C.POINTER(C.c_float)]
        for name in ("mmcgb_session_launch_batch", "mmcgb_session_launch_batch_on", "mmcgb_session_launch_repeat",
                     "mmcgb_grid_info", "mmcgb_check_config", "mmcgb_session_device_buffers", "mmcgb_l2_read_bandwidth", "mmcgb_session_phase_window",
                     "mmcgb_session_launch_batches", "mmcgb_prepare_host", "mmcgb_normalize_host", "mmcgb_session_begin", "mmcgb_session_launch", "mmcgb_session_sync", "mmcgb_session_end",
                     "mmcgb_mesh_create", "mmcgb_mesh_destroy", "mmcgb_mesh_info", "mmcgb_mesh_export",
                     "mmcgb_mesh_locate", "mmcgb_simulate", "mmcgb_simulate_batch", "mmcgb_run"):
            getattr(lib, name).restype = C.c_int32
        if lib.mmcgb_abi_version() != 6:
            raise NativeLibraryError("libmmcgb ABI version mismatch")
        _lib = lib
        return lib


def check(code: int):
    if code != 0:
        msg = load().mmcgb_last_error().decode(errors="replace")
        raise MmcgbError(code, f"{STATUS.get(code, '?')}: {msg}")
