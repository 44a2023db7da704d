"""ctypes binding of libffea_gb300.so (include/ffea_gpu.h).

The library is the product: there is no Python or CPU fallback.  Importing
this module does not load it; the first call to ``lib()`` does, and raises if
the library was not built (``python -m ffea_gb300.build`` or
``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class FfeaGpuError(RuntimeError):
    """A call across the C ABI returned FFEA_GPU_ERROR."""


class Mesh(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("num_elements", ctypes.c_int32),
        ("pos", _dp),
        ("vel", _dp),
        ("topology", _ip),
        ("material", _dp),
        ("stokes_drag", _dp),
        ("num_pinned", ctypes.c_int32),
        ("pinned", _ip),
    ]


SCRIPT_PATH_MAX = 1024


class ScriptParams(ctypes.Structure):
    """ffea_gpu_script_params"""
    _fields_ = [
        ("dt", ctypes.c_double),
        ("kT", ctypes.c_double),
        ("epsilon2", ctypes.c_double),
        ("stokes_visc", ctypes.c_double),
        ("num_steps", ctypes.c_int64),
        ("check", ctypes.c_int32),
        ("rng_seed", ctypes.c_int32),
        ("max_iterations_cg", ctypes.c_int32),
        ("calc_noise", ctypes.c_int32),
        ("calc_stokes", ctypes.c_int32),
        ("restart", ctypes.c_int32),
        ("num_blobs", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("trajectory_out_fname", ctypes.c_char * SCRIPT_PATH_MAX),
        ("measurement_out_fname", ctypes.c_char * SCRIPT_PATH_MAX),
        ("checkpoint_in", ctypes.c_char * SCRIPT_PATH_MAX),
        ("checkpoint_out", ctypes.c_char * SCRIPT_PATH_MAX),
    ]


class Params(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("kT", ctypes.c_double),
        ("epsilon2", ctypes.c_double),
        ("max_iterations_cg", ctypes.c_int32),
        ("calc_noise", ctypes.c_int32),
        ("calc_stokes", ctypes.c_int32),
        ("solver", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("rng_seed", ctypes.c_int32),
        ("true_residual", ctypes.c_int32),
        ("preconditioner", ctypes.c_int32),
    ]


# name -> (restype, argtypes); the full set declared by include/ffea_gpu.h
SIGNATURES = {
    "ffea_gpu_create": (ctypes.c_int, [ctypes.POINTER(Mesh), ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]),
    "ffea_gpu_create_batch": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(Mesh), ctypes.POINTER(Params),
                                             ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "ffea_gpu_destroy": (None, [ctypes.c_void_p]),
    "ffea_gpu_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ffea_gpu_get_nodes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp, _dp]),
    "ffea_gpu_set_nodes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp]),
    "ffea_gpu_set_external_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, _ip, _dp]),
    "ffea_gpu_get_rng_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _u64p]),
    "ffea_gpu_set_rng_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _u64p]),
    "ffea_gpu_energies": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp]),
    "ffea_gpu_measurements": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, _dp]),
    "ffea_gpu_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _ip, _ip, _dp, _ip]),
    "ffea_gpu_get_rhs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp]),
    "ffea_gpu_get_element_forces": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp]),
    "ffea_gpu_solver_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp]),
    "ffea_gpu_solver_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _dp, _dp]),
    "ffea_gpu_rng_draws": (ctypes.c_int, [_u64p, ctypes.c_uint64, ctypes.c_int64, _dp]),
    "ffea_gpu_ffea_seed": (ctypes.c_int, [ctypes.c_int32, _u64p]),
    "ffea_gpu_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "ffea_gpu_kernel_launches": (ctypes.c_int64, []),
    "ffea_gpu_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64)]),
    "ffea_gpu_set_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ffea_gpu_phase_times": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "ffea_gpu_kernel_times": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "ffea_gpu_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "ffea_gpu_set_graph_mode": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ffea_gpu_step_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ffea_gpu_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "ffea_gpu_cg_loop_count": (ctypes.c_int64, [ctypes.c_void_p]),
    "ffea_gpu_diag_spmv": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, _dp]),
    "ffea_gpu_diag_coarse": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "ffea_gpu_diag_coarse_half": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                                 ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_uint16),
                                                 ctypes.POINTER(ctypes.c_float)]),
    "ffea_gpu_script_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "ffea_gpu_script_free": (None, [ctypes.c_void_p]),
    "ffea_gpu_script_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ScriptParams)]),
    "ffea_gpu_script_get_blob": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(Mesh),
                                                ctypes.POINTER(Params)]),
    "ffea_gpu_script_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    "ffea_gpu_diag_cg_vectors": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp]),
    "ffea_gpu_diag_sgemm": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_void_p]),
    "ffea_gpu_preconditioner": (ctypes.c_int, [ctypes.c_void_p]),
    "ffea_gpu_selftest_barrier_timeout": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, _ip]),
    "ffea_gpu_set_smoother_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32,
                                                     ctypes.POINTER(ctypes.c_float)]),
    "ffea_gpu_mpnn_num_params": (ctypes.c_int, []),
    "ffea_gpu_mpnn_apply": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "ffea_gpu_mpnn_loss_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), _dp,
                                               ctypes.POINTER(ctypes.c_float)]),
    "ffea_gpu_mpnn_probe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32] + [ctypes.POINTER(ctypes.c_float)] * 5),
    "ffea_gpu_energies_noalloc": (ctypes.c_int, [ctypes.c_void_p] * 5 + [ctypes.c_int32, ctypes.c_int32,
                                                                          ctypes.c_void_p, ctypes.c_void_p]),
    "ffea_gpu_ssint_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "ffea_gpu_ssint_destroy": (None, [ctypes.c_void_p]),
    "ffea_gpu_ssint_forces": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_int64)]),
    "ffea_gpu_ssint_forces_device": (ctypes.c_int, [ctypes.c_void_p] * 4),
    "ffea_gpu_ssint_synchronize": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "ffea_gpu_ssint_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "ffea_gpu_ssint_set_pbc": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "ffea_gpu_ssint_blob_corr": (ctypes.c_int, [ctypes.c_int32, _dp, _dp, _dp]),
    "ffea_gpu_ssint_set_sticky_wall": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
}

_lib = None


def lib_path() -> str:
    return os.environ.get("FFEA_GB300_LIB", LIB)


def lib():
    """Load the library (once).  Raises if it is missing: no fallback path exists."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise FfeaGpuError(f"{path} is missing: build it with __graft_entry__.build() "
                               "(there is no CPU fallback for the GB300 blob update)")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(2048)
    lib().ffea_gpu_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise FfeaGpuError(f"{what}: {last_error()}" if what else last_error())


def ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)
