"""ctypes binding of the C ABI in include/branson_gb300.h.

The library is loaded from the in-tree build (branson_gb300/_build/).  There
is no CPU fallback: if the shared library or a usable sm_103 GPU is missing,
the calls raise ``BransonError``.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

LIB_PATH = os.environ.get("BRANSON_GB300_LIB", _build.LIB)

OK, ERR_INVALID, ERR_CUDA, ERR_CAPACITY, ERR_STATE, ERR_DEVICE, ERR_NO_DEVICE = range(7)
REFLECT, VACUUM, ELEMENT, SOURCE, PROCESSOR = range(5)
EXIT, PASS, CENSUS, SCATTER, KILLED, BOUND = range(6)
HISTORY, EVENT = 0, 1
OPTIONS = {"event_round_cap": 0, "event_check_every": 1, "event_tail_fraction": 2, "transport_blocks": 3,
           "transport_threads": 4, "pipeline_min_photons": 5, "zero_copy": 6}
BATCH_OPTIONS = {"graph": 0, "transport_blocks": 1}
FIELDS = {"T_e": 0, "T_r": 1, "op_a": 2, "op_s": 3, "f": 4, "emission_E": 5, "census_E": 6,
          "source_E": 7, "abs_E": 8, "track_E": 9}


class BransonError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [("ngx", C.c_uint32), ("ngy", C.c_uint32), ("ngz", C.c_uint32), ("n_groups", C.c_uint32),
                ("x_planes", C.c_void_p), ("y_planes", C.c_void_p), ("z_planes", C.c_void_p),
                ("cell_region", C.c_void_p), ("n_regions", C.c_uint32), ("regions", C.c_void_p),
                ("bc", C.c_int32 * 6), ("T_source", C.c_double)]


PHOTON_FIELDS = (("pos_x", np.float64), ("pos_y", np.float64), ("pos_z", np.float64),
                 ("dir_x", np.float64), ("dir_y", np.float64), ("dir_z", np.float64),
                 ("E", np.float64), ("E0", np.float64), ("life_dx", np.float64),
                 ("cell", np.uint32), ("group", np.uint32), ("descriptor", np.uint8),
                 ("source_type", np.uint8), ("rng_stream", np.uint64), ("rng_counter", np.uint64))


class PhotonsHost(C.Structure):
    _fields_ = [(name, C.c_void_p) for name, _ in PHOTON_FIELDS]


class EnergyDiag(C.Structure):
    _fields_ = [("total_photon_E", C.c_double), ("emission_E", C.c_double), ("census_E", C.c_double),
                ("source_E", C.c_double), ("pre_mat_E", C.c_double), ("n_new_photons", C.c_uint64),
                ("n_initial_census", C.c_uint64)]


class TransportDiag(C.Structure):
    _fields_ = [("n_transported", C.c_uint64), ("n_census", C.c_uint64), ("n_segments", C.c_uint64),
                ("census_E", C.c_double), ("exit_E", C.c_double), ("absorbed_E", C.c_double),
                ("post_mat_E", C.c_double), ("device_flags", C.c_uint32), ("reserved", C.c_uint32)]


class StepParams(C.Structure):
    _fields_ = [("step", C.c_uint32), ("algorithm", C.c_uint32), ("dt", C.c_double), ("next_dt", C.c_double)]


class AdjointInfo(C.Structure):
    _fields_ = [("n_histories", C.c_uint64), ("n_segments", C.c_uint64), ("n_long", C.c_uint64),
                ("max_E", C.c_double), ("max_life", C.c_double), ("coef_max", C.c_double),
                ("visit_bound", C.c_double), ("grad_scale", C.c_int32), ("device_flags", C.c_uint32),
                ("replay_ms", C.c_float), ("reserved", C.c_float)]


_lib: Optional[C.CDLL] = None

# (name, restype, argtypes) of every exported entry point in include/branson_gb300.h
SIGNATURES = (
    ("bgs_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_uint64, C.c_void_p, C.c_uint32, C.c_uint64]),
    ("bgs_destroy", C.c_int, [C.c_void_p]),
    ("bgs_last_error", C.c_char_p, [C.c_void_p]),
    ("bgs_status_string", C.c_char_p, [C.c_int]),
    ("bgs_version", C.c_char_p, []),
    ("bgs_set_mesh", C.c_int, [C.c_void_p, C.POINTER(MeshDesc)]),
    ("bgs_n_cells", C.c_uint32, [C.c_void_p]),
    ("bgs_get_cell_field", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("bgs_set_cell_field", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("bgs_calculate_photon_energy", C.c_int, [C.c_void_p, C.c_uint32, C.c_double, C.POINTER(EnergyDiag)]),
    ("bgs_source", C.c_int, [C.c_void_p, C.c_uint32, C.c_double]),
    ("bgs_transport", C.c_int, [C.c_void_p, C.c_double, C.c_uint32, C.POINTER(TransportDiag)]),
    ("bgs_update_temperature", C.c_int, [C.c_void_p, C.c_double, C.POINTER(TransportDiag)]),
    ("bgs_step", C.c_int, [C.c_void_p, C.POINTER(StepParams), C.POINTER(TransportDiag)]),
    ("bgs_synchronize", C.c_int, [C.c_void_p]),
    ("bgs_bank_size", C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    ("bgs_comb_census", C.c_int, [C.c_void_p, C.c_int64, C.c_uint32, C.c_uint64, C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_uint64)]),
    ("bgs_get_photons", C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.POINTER(PhotonsHost)]),
    ("bgs_set_photons", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(PhotonsHost)]),
    ("bgs_replicated_transport", C.c_int,
     [C.c_void_p, C.c_uint64, C.POINTER(PhotonsHost), C.c_double, C.c_uint32, C.c_void_p, C.c_void_p,
      C.POINTER(PhotonsHost), C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("bgs_transport_device_noalloc", C.c_int,
     [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
      C.POINTER(C.c_int32), C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64,
      C.POINTER(PhotonsHost), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bgs_adjoint_forward", C.c_int,
     [C.c_void_p, C.POINTER(StepParams), C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("bgs_adjoint_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bgs_adjoint_counts", C.c_int, [C.c_void_p, C.c_void_p]),
    ("bgs_adjoint_get_info", C.c_int, [C.c_void_p, C.POINTER(AdjointInfo)]),
    ("bgs_adjoint_release", C.c_int, [C.c_void_p]),
    ("bgs_batch_create", C.c_int, [C.POINTER(C.c_void_p), C.c_uint32, C.POINTER(C.c_void_p)]),
    ("bgs_batch_destroy", C.c_int, [C.c_void_p]),
    ("bgs_batch_last_error", C.c_char_p, [C.c_void_p]),
    ("bgs_batch_step", C.c_int, [C.c_void_p, C.POINTER(StepParams), C.POINTER(TransportDiag)]),
    ("bgs_batch_synchronize", C.c_int, [C.c_void_p]),
    ("bgs_batch_set_option", C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    ("bgs_batch_last_transport_ms", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint64)]),
    ("bgs_batch_adjoint_forward", C.c_int,
     [C.c_void_p, C.POINTER(StepParams), C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("bgs_batch_adjoint_backward", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p, C.c_void_p]),
    ("bgs_set_option", C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    ("bgs_last_transport_ms", C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_uint32)]),
    ("bgs_kernel_launch_count", C.c_uint64, [C.c_void_p]),
)


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the in-tree shared library (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise BransonError(ERR_STATE, f"{LIB_PATH} is not built")
            _build.build()
        lib = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class PhotonArrays:
    """Host structure-of-arrays photon buffers (optionally page-locked)."""

    def __init__(self, n: int, pinned: bool = False):
        self.n = n
        self._pinned = []
        self.arrays = {}
        for name, dt in PHOTON_FIELDS:
            if pinned and n > 0:
                self.arrays[name] = _pinned_empty(n, dt, self._pinned)
            else:
                self.arrays[name] = np.zeros(n, dt)

    def __getitem__(self, name: str) -> np.ndarray:
        return self.arrays[name]

    def struct(self, omit=()) -> PhotonsHost:
        return PhotonsHost(*[None if name in omit else ptr(self.arrays[name]) for name, _ in PHOTON_FIELDS])

    def subset(self, n: int) -> "PhotonArrays":
        out = PhotonArrays(0)
        out.n = n
        out.arrays = {k: v[:n] for k, v in self.arrays.items()}
        return out


def _pinned_empty(n: int, dtype, keep: list) -> np.ndarray:
    """page-locked host array through the CUDA runtime (cudaMallocHost)."""
    rt = _cudart()
    p = C.c_void_p()
    nbytes = int(n) * np.dtype(dtype).itemsize
    if rt.cudaMallocHost(C.byref(p), C.c_size_t(nbytes)) != 0:
        raise BransonError(ERR_CUDA, "cudaMallocHost failed")
    buf = (C.c_char * nbytes).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dtype, count=n)
    keep.append(_PinnedOwner(rt, p))
    return arr


class _PinnedOwner:
    def __init__(self, rt, p):
        self.rt, self.p = rt, p

    def __del__(self):
        try:
            self.rt.cudaFreeHost(self.p)
        except Exception:
            pass


_rt = None


def _cudart():
    global _rt
    if _rt is None:
        load()
        import ctypes.util
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                _rt = C.CDLL(name)
                break
            except OSError:
                continue
        if _rt is None:
            raise BransonError(ERR_CUDA, "libcudart not found")
        _rt.cudaMallocHost.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        _rt.cudaFreeHost.argtypes = [C.c_void_p]
    return _rt
