"""ctypes binding of libkvmc (include/kvmc.h).

The library is the only compute path: if it is missing or no sm_103 GPU is
present, calls raise instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("KVMC_LIBRARY", PKG / "_build" / "libkvmc.so"))

KVMC_OK = 0
KVMC_ERR_ARGUMENT = 1
KVMC_ERR_BOUNDS = 2
KVMC_ERR_SINGULAR = 3
KVMC_ERR_CUDA = 4
KVMC_ERR_NUMERIC = 5
KVMC_ERR_NO_DEVICE = 6
KVMC_ERR_UNSUPPORTED = 7

PLAIN_FP64 = 0
MIXED_FP32 = 1
ACCEPT_REFERENCE = 0
ACCEPT_METROPOLIS = 1


class KvmcError(RuntimeError):
    """Base class; `code` is the kvmc_status value."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class ArgumentError(KvmcError, ValueError):
    """Julia ArgumentError / AssertionError / DimensionMismatch."""


class BoundsError(KvmcError, IndexError):
    """Julia BoundsError."""


class SingularException(KvmcError):
    """Julia LinearAlgebra.SingularException (or the singular-start ErrorException)."""


class DeviceError(KvmcError):
    """CUDA failure, missing or unsupported device, non-finite numbers."""


_ERRORS = {KVMC_ERR_ARGUMENT: ArgumentError, KVMC_ERR_BOUNDS: BoundsError, KVMC_ERR_SINGULAR: SingularException}


class LatticeDesc(C.Structure):
    _fields_ = [("n1", C.c_int32), ("n2", C.c_int32), ("pbc", C.c_int32 * 2), ("antipbc", C.c_int32 * 2),
                ("t", C.c_double)]


class Link(C.Structure):
    _fields_ = [("label1", C.c_int32), ("label2", C.c_int32), ("dx", C.c_int32), ("dy", C.c_int32),
                ("amplitude", C.c_double)]


class ModelDesc(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("n_up", C.c_int32), ("n_down", C.c_int32), ("n_bonds", C.c_int32),
                ("bonds", C.POINTER(C.c_int32)), ("U_up", C.POINTER(C.c_double)), ("U_down", C.POINTER(C.c_double)),
                ("U_up_imag", C.POINTER(C.c_double)), ("U_down_imag", C.POINTER(C.c_double))]


class BatchDesc(C.Structure):
    _fields_ = [("n_walkers", C.c_int32), ("precision", C.c_int32), ("accept_rule", C.c_int32),
                ("refresh_interval", C.c_int32), ("measure_interval", C.c_int32), ("delay_k", C.c_int32),
                ("device", C.c_int32), ("seed", C.c_uint64), ("w_placement", C.c_int32)]


class SweepStats(C.Structure):
    _fields_ = [("proposals", C.c_int64), ("accepted", C.c_int64), ("measurements", C.c_int64),
                ("sum_energy", C.c_double), ("sum_energy2", C.c_double), ("refreshes", C.c_int64),
                ("max_drift", C.c_double), ("bad_walkers", C.c_int32), ("launches", C.c_int32),
                ("fp64_redos", C.c_int64)]


# name -> argtypes (all return c_int)
_P = C.c_void_p
_SIGS = {
    "kvmc_lattice_sites": [C.POINTER(LatticeDesc), C.POINTER(C.c_int32)],
    "kvmc_hopping_matrix": [C.POINTER(LatticeDesc), C.POINTER(Link), C.c_int32, C.POINTER(Link), C.c_int32,
                            C.c_double, _P],
    "kvmc_bonds_from_hopping": [C.c_int32, _P, C.POINTER(C.c_int32), _P],
    "kvmc_create": [C.POINTER(ModelDesc), C.POINTER(BatchDesc), C.POINTER(_P)],
    "kvmc_destroy": [_P],
    "kvmc_last_error": [_P, C.c_char_p, C.c_size_t],
    "kvmc_init": [_P, _P, _P, _P],
    "kvmc_sweep": [_P, C.c_int64, C.POINTER(SweepStats)],
    "kvmc_advance": [_P, C.c_int64, C.POINTER(SweepStats)],
    "kvmc_measure": [_P, _P],
    "kvmc_eval_ratios": [_P, C.c_int32, _P, _P],
    "kvmc_apply_moves": [_P, _P],
    "kvmc_refresh": [_P],
    "kvmc_get_state": [_P, _P, _P, _P],
    "kvmc_set_state": [_P, _P, _P, _P],
    "kvmc_get_w": [_P, _P, _P],
    "kvmc_walker_stats": [_P, _P, _P, _P, _P, _P, _P],
    "kvmc_reset_stats": [_P],
    "kvmc_walker_drift": [_P, _P],
    "kvmc_set_drift_tolerance": [_P, C.c_double],
    "kvmc_enable_timing": [_P, C.c_int32],
    "kvmc_kernel_time": [_P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)],
    "kvmc_region_timer": [_P, C.c_int32, C.POINTER(C.c_double)],
    "kvmc_get_config": [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "kvmc_version": [C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
    "kvmc_device_name": [C.c_int32, C.c_char_p, C.c_size_t, C.POINTER(C.c_int32)],
    "kvmc_refresh_static": [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, _P, _P],
    "kvmc_ansatz_hopping": [C.POINTER(LatticeDesc), C.POINTER(Link), C.c_int32, C.POINTER(Link), C.c_int32,
                            C.c_double, _P, _P, _P],
    "kvmc_set_log_derivatives": [_P, C.c_int32, _P, _P, _P, _P],
    "kvmc_measure_grad": [_P, _P, _P],
    "kvmc_grad_sums": [_P, _P],
    "kvmc_walker_logdet": [_P, _P],
    "kvmc_set_tuning": [_P, C.c_int32, C.c_int32],
    "kvmc_group_create": [_P, C.c_int32, C.POINTER(_P)],
    "kvmc_group_destroy": [_P],
    "kvmc_group_advance": [_P, C.c_int64, _P, C.POINTER(C.c_double)],
    "kvmc_group_last_error": [_P, C.c_char_p, C.c_size_t],
}
EXPORTS = tuple(_SIGS)

_lib = None


def load():
    """Loads libkvmc.so (raises OSError when it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise OSError(f"libkvmc.so not found at {LIB_PATH}; run __graft_entry__.build() first")
        lib = C.CDLL(str(LIB_PATH))
        for name, args in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int
        _lib = lib
    return _lib


def last_error(handle=None) -> str:
    buf = C.create_string_buffer(1024)
    load().kvmc_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, handle=None):
    if rc != KVMC_OK:
        raise _ERRORS.get(rc, DeviceError)(rc, last_error(handle))


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def as_c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)
