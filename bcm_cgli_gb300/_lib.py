"""Loader for the in-tree CUDA library ``_build/libbcm_gb300.so``.

There is no CPU fallback: if the library is missing or cannot be loaded the
import of the GPU API raises, so a product path can never silently run
anything but the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbcm_gb300.so")

_lib = None

dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class BcmgError(RuntimeError):
    pass


class CaseDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("ncube", C.c_int), ("mpi_ncube", C.c_int),
        ("mu_L", C.c_double), ("rho0", C.c_double), ("U0", C.c_double), ("Uin", C.c_double),
        ("P0", C.c_double), ("deltaT", C.c_double), ("deltaTau", C.c_double), ("e", C.c_double),
        ("precision", C.c_int),
        ("cube_size", C.c_void_p), ("csl", C.c_void_p), ("adj_number", C.c_void_p),
        ("FWS", C.c_void_p),
        ("nxl", C.c_int), ("nxu", C.c_int), ("nyl", C.c_int), ("nyu", C.c_int),
        ("nzl", C.c_int), ("nzu", C.c_int),
        ("xl", C.c_void_p), ("xu", C.c_void_p), ("yl", C.c_void_p), ("yu", C.c_void_p),
        ("zl", C.c_void_p), ("zu", C.c_void_p),
        ("nminus", C.c_int), ("w_minus", C.c_void_p), ("gc_minus", C.c_void_p),
        ("ip_minus", C.c_void_p),
        ("nplus", C.c_int), ("w_plus", C.c_void_p), ("gc_plus", C.c_void_p),
        ("ip_plus", C.c_void_p),
    ]


class Tuning(C.Structure):
    _fields_ = [("flux_tile", C.c_int), ("lusgs_threads", C.c_int), ("flux_form", C.c_int),
                ("flux_ms", C.c_double * 3), ("lusgs_ms", C.c_double * 2)]


# int (*)(void *user, int phase, void *stream): the exchange hook of sharded runs
EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_void_p)


class RefConfig(C.Structure):
    _fields_ = [("ncube_x", C.c_int), ("mpi_ncube", C.c_int), ("mu_L", C.c_double),
                ("rho0", C.c_double), ("U0", C.c_double), ("Uin", C.c_double),
                ("P0", C.c_double)]


def _declare(L):
    L.bcmg_last_error.restype = C.c_char_p
    L.bcmg_version.restype = C.c_char_p
    L.bcmg_set_reference_config.argtypes = [C.POINTER(RefConfig)]
    L.bcmg_set_reference_precision.argtypes = [C.c_int]
    L.bcmg_release_host_arrays.argtypes = []
    L.bcmg_release_host_arrays.restype = None
    L.bcmg_set_host_pinning.argtypes = [C.c_int]
    L.bcmg_set_host_pinning.restype = None
    L.bcmg_set_twin_scratch_kept.argtypes = [C.c_int]
    L.bcmg_set_twin_scratch_kept.restype = None
    L.bcmg_get_reference_config.argtypes = [C.POINTER(RefConfig)]
    L.BCM_Flux_XYZ_Viscous_Runge_kutta.argtypes = [
        C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, ip, ip, dp, dp, dp, dp,
        dp, dp, dp, dp, dp]
    L.BCM_Flux_XYZ_Viscous_Runge_kutta.restype = None
    L.BCM_X_boundary_condition.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, dp]
    L.BCM_Y_boundary_condition.argtypes = [C.c_int, C.c_int, ip, ip, dp]
    L.BCM_Z_boundary_condition.argtypes = [C.c_int, C.c_int, ip, ip, dp]
    for f in (L.BCM_X_boundary_condition, L.BCM_Y_boundary_condition,
              L.BCM_Z_boundary_condition):
        f.restype = None
    for f in (L.BCM_Ghostcell_minus, L.BCM_Ghostcell_plus):
        f.argtypes = [C.c_int, C.POINTER(C.c_int), dp, ip, ip, ip, dp]
        f.restype = None
    L.BCM_Interface.restype = None
    P = C.c_void_p
    L.bcmg_case_create.argtypes = [C.POINTER(CaseDesc), C.POINTER(P)]
    L.bcmg_case_create_shard.argtypes = [C.POINTER(CaseDesc), C.c_int, C.POINTER(P)]
    L.bcmg_shard_plan.argtypes = [C.c_int, P, P, P, C.c_int, C.c_int, C.POINTER(C.c_int), P,
                                  C.POINTER(C.c_int), P]
    L.bcmg_shard_bands.argtypes = [C.c_int, P, P, P, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_int), P]
    L.bcmg_case_set_exchange.argtypes = [P, EXCHANGE_FN, P]
    L.bcmg_case_set_halo.argtypes = [P, C.c_int, P, P, P, P]
    L.bcmg_case_halo_bytes.argtypes = [P, C.c_int, C.POINTER(C.c_size_t),
                                       C.POINTER(C.c_size_t)]
    L.bcmg_case_halo_pack.argtypes = [P, C.c_int, P]
    L.bcmg_case_halo_unpack.argtypes = [P, C.c_int, P]
    L.bcmg_case_norm_sums.argtypes = [P, C.POINTER(P)]
    L.bcmg_case_norm_sums_host.argtypes = [P, P, C.c_int]
    L.bcmg_case_advance_async.argtypes = [P, C.c_int, C.c_int]
    L.bcmg_case_copy_state_async.argtypes = [P, C.c_int, P, P, P]
    L.bcmg_case_get_norms.argtypes = [P, P, P]
    L.bcmg_case_destroy.argtypes = [P]
    L.bcmg_case_destroy.restype = None
    L.bcmg_case_set_state.argtypes = [P, P, P, P]
    L.bcmg_case_get_state.argtypes = [P, P, P, P]
    L.bcmg_case_get_scratch.argtypes = [P, P, P, P, P]
    L.bcmg_case_stage.argtypes = [P, C.c_int]
    L.bcmg_case_advance.argtypes = [P, C.c_int, C.c_int, C.c_int, P, P]
    L.bcmg_case_sync.argtypes = [P]
    L.bcmg_case_device_state.argtypes = [P, P, P, P]
    L.bcmg_case_launch_count.argtypes = [P]
    L.bcmg_case_launch_count.restype = C.c_longlong
    L.bcmg_case_time_flux.argtypes = [P, C.c_int, C.POINTER(C.c_double)]
    L.bcmg_case_set_profiling.argtypes = [P, C.c_int]
    L.bcmg_case_profile.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    L.bcmg_case_timer_mark.argtypes = [P, C.c_int]
    L.bcmg_case_timer_elapsed.argtypes = [P, C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.bcmg_batch_create.argtypes = [C.c_int, C.POINTER(CaseDesc), C.POINTER(P)]
    L.bcmg_case_set_method.argtypes = [P, C.c_int, C.c_double, C.c_double]
    L.bcmg_case_mirror.argtypes = [P, P]
    L.bcmg_case_mirror_current.argtypes = [P, P]
    L.bcmg_case_set_tuning.argtypes = [P, C.POINTER(Tuning)]
    L.bcmg_case_set_face_copies.argtypes = [P, C.c_int]
    L.bcmg_case_set_mirror_each_stage.argtypes = [P, C.c_int]
    L.bcmg_case_set_concurrent_ghosts.argtypes = [P, C.c_int]
    L.bcmg_case_concurrent_ghosts.argtypes = [P]
    L.bcmg_case_autotune.argtypes = [P, C.c_int, C.POINTER(Tuning)]
    L.bcmg_case_output_q.argtypes = [P, C.c_int, C.c_int, C.c_char_p]
    L.bcmg_case_output_x.argtypes = [P, C.c_int, C.c_int, C.c_char_p, P]
    L.bcmg_case_output_wait.argtypes = [P]
    L.bcmg_case_advance_converged.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_int, P, P, P]
    L.bcmg_case_ncase.argtypes = [P]
    L.bcmg_case_case_cubes.argtypes = [P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.bcmg_case_set_case_state.argtypes = [P, C.c_int, P, P, P]
    L.bcmg_case_get_case_state.argtypes = [P, C.c_int, P, P, P]
    L.bcmg_probe_fp64_rate.argtypes = [C.POINTER(C.c_double)]
    L.bcmg_ibm_schedule.argtypes = [C.c_int, ip, ip, C.c_int, C.c_int, ip]
    L.bcmg_interface_tasks.argtypes = [C.c_int, ip, ip, ip, ip, C.c_int]
    L.bcmg_interface_plan.argtypes = [C.c_int, C.c_int, ip, ip, P, P, P, C.c_int, P, C.c_int,
                                      ip, ip, C.c_int]
    L.bcmg_interface_closing_plan.argtypes = [C.c_int, C.c_int, ip, ip, P, P, P, C.c_int, P,
                                              C.c_int, ip, ip, C.c_int]
    L.bcmg_ghost_beside_plan.argtypes = [C.c_int, C.c_int, P, P, P, P, C.c_int, P, P, C.c_int,
                                         ip, C.c_int, ip]
    L.bcmg_ibm_preprocess.argtypes = [
        C.c_int, C.c_int, dp, ip, dp, dp, dp, ip, C.c_int, dp, C.c_int, C.POINTER(C.c_int), ip,
        ip, dp, C.POINTER(C.c_int), ip, ip, dp]
    L.BCM_Immersed_boundary.argtypes = [
        C.c_int, C.c_int, C.c_int, P, C.c_double, C.c_double, C.c_double, C.c_double,
        C.c_double, C.c_double, dp, ip, dp, dp, dp, P, P, P, ip, P]
    L.BCM_Immersed_boundary.restype = None
    L.BCM_FWS_Interface.argtypes = [C.c_int] * 8 + [P] * 11 + [P] * 4 + [P] * 3 + [ip, ip, P, P,
                                                                                   P, ip]
    L.BCM_FWS_Interface.restype = None
    L.bcmg_fws_interface.argtypes = [C.c_int, C.c_int, ip, ip, ip]
    L.bcmg_fws_band_pack.argtypes = [C.c_int, C.c_int, ip, C.c_int, ip, ip]
    L.bcmg_fws_band_unpack.argtypes = [C.c_int, C.c_int, ip, C.c_int, ip, ip]
    return L


def lib():
    """The loaded library (raises BcmgError when it is not built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise BcmgError(
                f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def check(code: int):
    if code != 0:
        msg = lib().bcmg_last_error()
        raise BcmgError(f"bcm_gb300 error {code}: {msg.decode() if msg else '?'}")


def last_error():
    m = lib().bcmg_last_error()
    return m.decode() if m else None
