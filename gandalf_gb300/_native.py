"""ctypes binding of libgsph_gb300.so (the C ABI in include/gsph_gb300.h).

There is no fallback: if the library is missing or fails to load, every entry point
raises.  Build it with ``gandalf_gb300.build.build()`` (nvcc, sm_103a).
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

GSPH_OK = 0
ERRORS = {-1: "GSPH_ERR_INVALID", -2: "GSPH_ERR_CUDA", -3: "GSPH_ERR_UNSUPPORTED",
          -4: "GSPH_ERR_STATE", -5: "GSPH_ERR_NOT_CONVERGED", -6: "GSPH_ERR_CAPACITY"}

FIELDS = ["h", "rho", "invomega", "zeta", "hfactor", "pressure", "sound", "u", "div_v", "dudt",
          "ax", "ay", "az", "agx", "agy", "agz", "gpot", "hrangesqd", "gpot_hydro"]
FIELD_ID = {k: i for i, k in enumerate(FIELDS)}


class KdkConfig(ctypes.Structure):
    _fields_ = [("nlevels", ctypes.c_int32), ("level_diff_max", ctypes.c_int32), ("courant_mult", ctypes.c_double),
                ("accel_mult", ctypes.c_double), ("energy_mult", ctypes.c_double)]


class KdkStatus(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nresync", ctypes.c_int64), ("level_max", ctypes.c_int64),
                ("level_step", ctypes.c_int64), ("nsteps", ctypes.c_int64), ("t", ctypes.c_double),
                ("timestep", ctypes.c_double), ("dt_max", ctypes.c_double), ("active_updates", ctypes.c_int64),
                ("status", ctypes.c_uint32)]


class KdkTiming(ctypes.Structure):
    _fields_ = [("ms_build", ctypes.c_double), ("ms_density", ctypes.c_double), ("ms_forces", ctypes.c_double),
                ("density_pairs", ctypes.c_int64), ("hydro_pairs", ctypes.c_int64), ("direct_pairs", ctypes.c_int64),
                ("cell_pairs", ctypes.c_int64), ("steps", ctypes.c_int64), ("repeat_passes", ctypes.c_int64)]


KDK_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "u", "dt", "tlast", "level", "nstep", "nlast", "levelneib"]


class Config(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("nleafmax", ctypes.c_int32),
                ("hydro_forces", ctypes.c_int32), ("self_gravity", ctypes.c_int32),
                ("eos", ctypes.c_int32), ("multipole", ctypes.c_int32),
                ("periodic", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("h_fac", ctypes.c_double), ("h_converge", ctypes.c_double),
                ("alpha_visc", ctypes.c_double), ("beta_visc", ctypes.c_double),
                ("gamma_eos", ctypes.c_double), ("temp0", ctypes.c_double),
                ("mu_bar", ctypes.c_double), ("thetamaxsqd", ctypes.c_double),
                ("boxmin", ctypes.c_double * 3), ("boxmax", ctypes.c_double * 3),
                ("compensated", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class FieldOffsets(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in (
        "r", "v", "m", "h", "u", "rho", "invomega", "zeta", "hfactor", "hrangesqd", "pressure",
        "sound", "div_v", "dudt", "a", "atree", "gpot", "gpot_hydro", "flags", "level", "levelneib")]


GSPH_FLAG_ACTIVE = 2   # the reference's `active` particle flag bit


class Tuning(ctypes.Structure):
    _fields_ = [("nleafmax", ctypes.c_int32), ("near_depth", ctypes.c_int32), ("cell_depth", ctypes.c_int32),
                ("gather_depth", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("ncell", ctypes.c_int64), ("nleaf", ctypes.c_int64),
                ("ltot", ctypes.c_int64), ("density_pairs", ctypes.c_int64),
                ("hydro_pairs", ctypes.c_int64), ("direct_pairs", ctypes.c_int64),
                ("cell_pairs", ctypes.c_int64), ("exact_checks", ctypes.c_int64),
                ("heavy_density", ctypes.c_int64), ("heavy_forces", ctypes.c_int64),
                ("status", ctypes.c_uint32), ("launches", ctypes.c_uint32),
                ("ms_build", ctypes.c_double), ("ms_density", ctypes.c_double),
                ("ms_hmax", ctypes.c_double), ("ms_forces", ctypes.c_double),
                ("ms_total", ctypes.c_double)]


# name -> (restype, argtypes); the list every test checks the library exports
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
SIGNATURES = {
    "gsph_abi_version": (_I32, []),
    "gsph_config_defaults": (None, [ctypes.POINTER(Config)]),
    "gsph_create": (_P, [ctypes.POINTER(Config), _I32]),
    "gsph_destroy": (None, [_P]),
    "gsph_last_error": (ctypes.c_char_p, [_P]),
    "gsph_create_error": (_I32, []),
    "gsph_set_particles": (_I32, [_P, _I64] + [_D] * 9),
    "gsph_set_particles_device": (_I32, [_P, _I64] + [_P] * 9),
    "gsph_set_particles_aos": (_I32, [_P, _P, _I64, _I64, ctypes.POINTER(FieldOffsets)]),
    "gsph_build_tree": (_I32, [_P]),
    "gsph_update_all_sph_properties": (_I32, [_P]),
    "gsph_update_all_sph_hydro_forces": (_I32, [_P]),
    "gsph_update_all_sph_forces": (_I32, [_P]),
    "gsph_step": (_I32, [_P]),
    "gsph_step_graph": (_I32, [_P]),
    "gsph_get_field": (_I32, [_P, _I32, _D]),
    "gsph_get_field_device": (_I32, [_P, _I32, _P]),
    "gsph_get_particles_aos": (_I32, [_P, _P, _I64, _I64, ctypes.POINTER(FieldOffsets)]),
    "gsph_update_active_particle_counters": (_I32, [_P, _P, _I64, _I64, ctypes.POINTER(FieldOffsets)]),
    "gsph_get_maximum_smoothing_length": (_I32, [_P, _D]),
    "gsph_get_stats": (_I32, [_P, ctypes.POINTER(Stats)]),
    "gsph_set_recording": (_I32, [_P, _I32, _I32]),
    "gsph_get_sph_neighbours": (_I64, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]),
    "gsph_get_direct_summary": (_I32, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64)]),
    "gsph_set_list_recording": (_I32, [_P, _I32, _I32]),
    "gsph_get_direct_lists": (_I64, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]),
    "gsph_get_cell_lists": (_I64, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32)]),
    "gsph_get_cell_summary": (_I32, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_uint64)]),
    "gsph_set_stream": (_I32, [_P, _P]),
    "gsph_fma_peak_gflops": (ctypes.c_double, [_I32, _I32]),
    "gsph_kdtree_order_noalloc": (_I32, [_P, _P, _P, _P, _I32, _I32, _P, _P]),
    "gsph_get_tuning": (_I32, [_P, ctypes.POINTER(Tuning)]),
    "gsph_set_tuning": (_I32, [_P, ctypes.POINTER(Tuning)]),
    "gsph_autotune": (_I32, [_P, _I32, ctypes.POINTER(Tuning), ctypes.POINTER(Tuning), _D, _I32,
                             ctypes.POINTER(ctypes.c_int32)]),
    "gsph_get_tree": (_I32, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                             ctypes.POINTER(ctypes.c_int32), _D]),
    "gsph_set_stars": (_I32, [_P, _I64] + [_D] * 8),
    "gsph_update_all_star_gas_forces": (_I32, [_P]),
    "gsph_get_star_forces": (_I32, [_P] + [_D] * 7),
    "gsph_kdk_config_defaults": (None, [ctypes.POINTER(KdkConfig)]),
    "gsph_kdk_setup": (_I32, [_P, ctypes.POINTER(KdkConfig)]),
    "gsph_kdk_steps": (_I32, [_P, _I32, _I32]),
    "gsph_kdk_get_status": (_I32, [_P, ctypes.POINTER(KdkStatus)]),
    "gsph_kdk_get_state": (_I32, [_P, _I32, _D]),
    "gsph_kdk_get_timing": (_I32, [_P, ctypes.POINTER(KdkTiming)]),
    "gsph_batch_create": (_P, [ctypes.POINTER(_P), _I32]),
    "gsph_batch_destroy": (None, [_P]),
    "gsph_batch_step": (_I32, [_P]),
    "gsph_batch_last_error": (ctypes.c_char_p, [_P]),
    "gsph_batch_stats": (_I32, [_P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)]),
}

ABI_VERSION = 3

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the CUDA library (raises if it is missing; there is no CPU path)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with gandalf_gb300.build.build()")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.gsph_abi_version() != ABI_VERSION:
        raise RuntimeError("libgsph_gb300.so ABI version mismatch")
    if path is None:
        _lib = lib
    return lib
