"""ctypes declarations of include/tam.h (the C ABI of libtam.so).

This module mirrors the header one-to-one: the same struct layouts, enum
values and entry points.  It is the binding a Python caller (or the tests)
uses; a Fortran caller would use the iso_c_binding interface module
include/tam.f90 instead.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtam.so")

# enum tam_status
TAM_OK, TAM_E_INVALID, TAM_E_CUDA, TAM_E_NOMEM, TAM_E_IO, TAM_E_PARSE, TAM_E_STATE, TAM_E_DEVICE, TAM_E_NODEV = range(9)
TAM_MODE_REFERENCE, TAM_MODE_CONFIG = 0, 1
TAM_FP64, TAM_FP32 = 0, 1
TAM_PULSE_GAUSSIAN, TAM_PULSE_TOPHAT, TAM_PULSE_TRIANGULAR = 0, 1, 2
TAM_SRC_DISK, TAM_SRC_GAUSSIAN = 0, 1
TAM_BC_DIRICHLET, TAM_BC_ROBIN = 0, 1
TAM_DEVERR_STEP_CAP, TAM_DEVERR_NAN, TAM_DEVERR_NEG_T = 0x1, 0x2, 0x4
(TAM_F_TEMP, TAM_F_RHOKAP, TAM_F_JMEAN, TAM_F_JMEAN_GLOBAL, TAM_F_TISSUE, TAM_F_THRESTIME, TAM_F_KAPPA,
 TAM_F_DENSITY, TAM_F_HEATCAP, TAM_F_COEFF, TAM_F_ALPHA, TAM_F_Q, TAM_F_WATER, TAM_F_MATERIAL) = range(14)
TAM_MAX_MATERIALS = 16
TAM_NOALLOC_MAX_VOXELS = 2097152
TALLY_NAMES = ("absorbed", "specular", "reflected", "transmitted", "side", "roulette_net", "missed",
               "voxel_steps", "scatters", "overflow")

STATUS_NAMES = {0: "TAM_OK", 1: "TAM_E_INVALID", 2: "TAM_E_CUDA", 3: "TAM_E_NOMEM", 4: "TAM_E_IO",
                5: "TAM_E_PARSE", 6: "TAM_E_STATE", 7: "TAM_E_DEVICE", 8: "TAM_E_NODEV"}


class Params(C.Structure):
    _fields_ = [
        ("nphotons", C.c_int64),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("n1", C.c_double), ("n2", C.c_double),
        ("total_time", C.c_double),
        ("loops", C.c_int32),
        ("repetition_rate_1", C.c_double),
        ("power", C.c_double),
        ("energy_per_pixel", C.c_double),
        ("ablate_temp", C.c_double),
        ("pulses_to_do", C.c_int32),
        ("pulse_type", C.c_int32),
        ("nxg", C.c_int32), ("nyg", C.c_int32), ("nzg", C.c_int32),
        ("numproc", C.c_int32),
        ("mode", C.c_int32),
        ("precision", C.c_int32),
        ("device", C.c_int32),
    ]


class Material(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("mua", "mus", "g", "n", "k", "rho", "c")]


class Config(C.Structure):
    _fields_ = [
        ("nmat", C.c_int32),
        ("mat", Material * TAM_MAX_MATERIALS),
        ("n_ambient", C.c_double),
        ("source", C.c_int32),
        ("source_radius", C.c_double),
        ("fresnel", C.c_int32),
        ("roulette", C.c_int32),
        ("roulette_w", C.c_double), ("roulette_m", C.c_double),
        ("T0", C.c_double),
        ("bc_type", C.c_int32 * 6),
        ("bc_T", C.c_double * 6), ("bc_h", C.c_double * 6), ("bc_Tamb", C.c_double * 6),
        ("dt_factor", C.c_double),
        ("dt", C.c_double),
        ("opscale", C.c_double),
        ("boil", C.c_int32),
        ("T_boil", C.c_double), ("lw", C.c_double),
        ("T_abl", C.c_double),
        ("arrhenius", C.c_int32),
        ("A", C.c_double), ("Ea", C.c_double), ("Rgas", C.c_double), ("T_lo", C.c_double), ("T_hi", C.c_double),
        ("thr", C.c_double * 3),
        ("retrace_fraction", C.c_double),
        ("retrace_check", C.c_int32),
        ("max_steps", C.c_int64),
        ("isolation", C.c_int32),
    ]


class State(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "time", "delt", "total_time", "pulse_count", "repetition_count", "laser_on", "pulse_length",
        "real_pulse_length", "volume_voxel", "mass_voxel", "qvapor", "dx", "dy", "dz")] + [
        ("laser_flag", C.c_int32), ("pulse_flag", C.c_int32), ("pulses_done", C.c_int32), ("counter", C.c_int32),
        ("n_ablated", C.c_int64), ("mc_passes", C.c_int64)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_U32 = C.POINTER(C.c_uint32)

# (name, restype, argtypes)
SIGNATURES = [
    ("tam_version", C.c_char_p, []),
    ("tam_abi_version", C.c_int, []),
    ("tam_struct_size", C.c_int64, [C.c_int32]),
    ("tam_params_default", C.c_int, [C.POINTER(Params)]),
    ("tam_config_default", C.c_int, [C.POINTER(Config)]),
    ("tam_read_input_params", C.c_int, [C.c_char_p, C.POINTER(Params)]),
    ("tam_read_config", C.c_int, [C.c_char_p, C.POINTER(Config)]),
    ("tam_create", C.c_int, [C.POINTER(Params), C.POINTER(Config), C.POINTER(_P)]),
    ("tam_destroy", C.c_int, [_P]),
    ("tam_last_error", C.c_char_p, [_P]),
    ("tam_set_stream", C.c_int, [_P, _P]),
    ("tam_device_errors", C.c_int, [_P, _U32]),
    ("tam_init_opt", C.c_int, [_P]),
    ("tam_gridset", C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    ("tam_init_thermal", C.c_int, [_P, _D]),
    ("tam_field_bytes", C.c_int, [_P, C.c_int, C.POINTER(C.c_int64)]),
    ("tam_upload", C.c_int, [_P, C.c_int, _P, C.c_int64]),
    ("tam_download", C.c_int, [_P, C.c_int, _P, C.c_int64]),
    ("tam_mc_pass", C.c_int, [_P, C.c_int64, C.c_uint64, C.c_uint32, _D]),
    ("tam_heat_steps", C.c_int, [_P, C.c_int32, _D]),
    ("tam_arrhenius", C.c_int, [_P]),
    ("tam_update_props", C.c_int, [_P, C.c_double]),
    ("tam_step_coupled", C.c_int, [_P, C.c_int32, C.c_uint64]),
    ("tam_run", C.c_int, [_P, C.c_uint64, C.c_int64, C.POINTER(C.c_int64)]),
    ("tam_finalize", C.c_int, [_P]),
    ("tam_get_tallies", C.c_int, [_P, _D, _D, _D]),
    ("tam_get_tallies_ex", C.c_int, [_P, _D, C.c_int32]),
    ("tam_get_state", C.c_int, [_P, C.POINTER(State)]),
    ("tam_get_timing", C.c_int, [_P, _D, _D, C.POINTER(C.c_int64)]),
    ("tam_batch_step_coupled", C.c_int, [C.POINTER(_P), C.c_int32, C.c_int32, C.POINTER(C.c_uint64)]),
    ("tam_batch_run", C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(C.c_uint64), C.c_int64,
                                C.POINTER(C.c_int64)]),
    ("tam_batch_heat_steps", C.c_int, [C.POINTER(_P), C.c_int32, C.c_int32]),
    ("tam_batch_mc_pass", C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_uint32)]),
    ("tam_batch_autotune", C.c_int, [C.POINTER(_P), C.c_int32, C.c_int32, C.POINTER(C.c_int64), C.c_int32]),
    ("tam_autotune", C.c_int, [_P, C.c_int64, C.c_int32, C.POINTER(C.c_int64), C.c_int32]),
    ("tam_save_state", C.c_int, [_P, C.c_char_p]),
    ("tam_load_state", C.c_int, [_P, C.c_char_p]),
    ("tam_kernel_launches", C.c_int64, []),
    ("tam_set_tuning", C.c_int, [_P, C.c_char_p, C.c_int64]),
    ("tam_write_output", C.c_int, [_P, C.c_char_p]),
    ("tam_measure_tally_atomics", C.c_int, [C.c_int64, C.c_int32, C.POINTER(C.c_double)]),
    ("tam_selftest_philox", C.c_int, [_U32, _U32, _U32, C.c_int64]),
    ("tam_mc_pass_noalloc", C.c_int, [C.POINTER(Params), _P, _P, C.c_int64, C.c_uint64, C.c_uint32, C.c_double, _P]),
]

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libtam.so (built in-tree by tam_gb300.build) and declare its ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"libtam.so not built ({p}); run tam_gb300.build.build() or __graft_entry__.build()")
    lib = C.CDLL(p)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
