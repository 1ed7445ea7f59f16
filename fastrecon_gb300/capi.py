"""ctypes bindings to libfastrecon_gb300.so (the C ABI in include/fastrecon_gb300.h).

Device buffers are passed as raw addresses (ints), e.g. ``tensor.data_ptr()``
of a CUDA tensor; streams as ``torch.cuda.Stream.cuda_stream`` or 0.  The
library is loaded from the package's ``_lib`` directory; there is no
fallback: if it cannot be loaded every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libfastrecon_gb300.so")

FR_PLAN_CHECKERBOARD = 1
FR_PLAN_NO_TAP_LISTS = 4
FR_PLAN_ACCUMULATE = 8
FR_PLAN_DETERMINISTIC = 16
FR_RECON_DEAPODIZE = 1
FR_RECON_CUFFT = 2
FR_RECON_PRUNED_FFT = 4
FR_RECON_DETERMINISTIC = 8

_lib = None


class FastreconError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {detail} (status {status})")
        self.status = status


class PlanDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("grid_size", C.c_uint), ("kernel_width", C.c_float), ("lut_length", C.c_int),
                ("lut", C.POINTER(C.c_float)), ("tile", C.c_int * 3), ("coil_group", C.c_int), ("chunk", C.c_int),
                ("flags", C.c_uint)]


class ReconDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("recon_size", C.c_uint), ("overgrid_factor", C.c_float),
                ("kernel_width", C.c_float), ("lut_length", C.c_int), ("out_size", C.c_uint * 3),
                ("channels", C.c_int), ("max_samples", C.c_size_t), ("tile", C.c_int * 3), ("coil_group", C.c_int),
                ("flags", C.c_uint), ("grid_budget", C.c_size_t)]


_VP = C.c_void_p
_SIGS = {
    "fr_status_string": (C.c_char_p, [C.c_int]),
    "fr_last_error": (C.c_char_p, []),
    "fr_version": (C.c_char_p, []),
    "fr_kb_lut": (C.c_int, [C.c_float, C.c_float, C.c_int, C.POINTER(C.c_float)]),
    "fr_lut_index_table": (C.c_int, [C.c_float, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float)]),
    "fr_plan_create": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(_VP)]),
    "fr_plan_destroy": (C.c_int, [_VP]),
    "fr_plan_set_trajectory": (C.c_int, [_VP, _VP, C.c_size_t, _VP]),
    "fr_plan_normalized_trajectory": (C.c_int, [_VP, _VP, _VP]),
    "fr_plan_bounds": (C.c_int, [_VP, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                 C.POINTER(C.c_float)]),
    "fr_plan_sample_ranges": (C.c_int, [_VP, _VP, _VP, _VP]),
    "fr_plan_stats": (C.c_int, [_VP, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                C.POINTER(C.c_longlong)]),
    "fr_plan_bins": (C.c_int, [_VP, _VP, _VP, _VP]),
    "fr_plan_tap_words": (C.c_int, [_VP, C.POINTER(C.c_int)]),
    "fr_plan_profile": (C.c_int, [_VP, C.c_int]),
    "fr_plan_profile_read": (C.c_int, [_VP, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "fr_kernel_launches": (C.c_longlong, []),
    "fr_grid": (C.c_int, [_VP, _VP, _VP, C.c_int, _VP, _VP]),
    "fr_grid_partitioned": (C.c_int, [C.POINTER(PlanDesc), _VP, C.c_size_t, _VP, _VP, C.c_int, _VP, C.c_size_t, _VP]),
    "fr_grid_noalloc": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_uint, C.c_float, C.POINTER(C.c_float), C.c_int,
                                  _VP, _VP, C.c_int, _VP, _VP]),
    "fr_batch_create": (C.c_int, [C.POINTER(PlanDesc), C.POINTER(_VP)]),
    "fr_batch_destroy": (C.c_int, [_VP]),
    "fr_batch_set_trajectories": (C.c_int, [_VP, _VP, C.POINTER(C.c_size_t), C.c_int, _VP]),
    "fr_batch_stats": (C.c_int, [_VP, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                 C.POINTER(C.c_longlong), C.POINTER(C.c_int)]),
    "fr_batch_grid": (C.c_int, [_VP, _VP, _VP, C.c_int, _VP, _VP]),
    "fr_batch_capture": (C.c_int, [_VP, _VP, _VP, C.c_int, _VP, _VP]),
    "fr_batch_replay": (C.c_int, [_VP, _VP]),
    "fr_batch_autotune": (C.c_int, [C.POINTER(PlanDesc), _VP, C.POINTER(C.c_size_t), C.c_int, _VP, _VP, C.c_int, _VP,
                                    C.c_int, C.POINTER(PlanDesc), C.POINTER(C.c_float), _VP]),
    "fr_dcf_analytic": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_float, _VP, _VP]),
    "fr_degrid": (C.c_int, [_VP, _VP, C.c_int, _VP, _VP]),
    "fr_grid_update": (C.c_int, [_VP, _VP, _VP, C.c_size_t, C.c_size_t, _VP, C.c_int, _VP, _VP]),
    "fr_grid_real": (C.c_int, [_VP, _VP, _VP, _VP]),
    "fr_dcf_pipe": (C.c_int, [_VP, C.c_int, _VP, _VP]),
    "fr_density_counts": (C.c_int, [_VP, C.POINTER(C.c_int), C.c_int, _VP, _VP]),
    "fr_dcf_features": (C.c_int, [_VP, _VP, _VP, C.POINTER(C.c_int), C.c_int, C.c_float, _VP, _VP]),
    "fr_mlp_forward": (C.c_int, [_VP, _VP, C.c_size_t, C.c_uint, C.c_float, _VP, _VP]),
    "fr_mlp_workspace_bytes": (C.c_size_t, [C.c_size_t]),
    "fr_mlp_backward": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP, _VP, _VP]),
    "fr_mlp_adam": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                              _VP]),
    "fr_mlp_to_bf16": (C.c_int, [_VP, _VP, C.c_int, _VP]),
    "fr_fft_create": (C.c_int, [C.c_int, C.POINTER(C.c_uint), C.c_int, C.c_int, C.POINTER(_VP)]),
    "fr_fft_execute": (C.c_int, [_VP, _VP, _VP]),
    "fr_fft_destroy": (C.c_int, [_VP]),
    "fr_fft_crop_sos_create": (C.c_int, [C.c_int, C.c_uint, C.c_int, C.POINTER(C.c_uint), C.POINTER(_VP)]),
    "fr_fft_crop_sos_execute": (C.c_int, [_VP, _VP, _VP, _VP, _VP]),
    "fr_fft_crop_sos_destroy": (C.c_int, [_VP]),
    "fr_fft_shift": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_uint), _VP]),
    "fr_crop": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint), _VP, _VP]),
    "fr_sos": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint), _VP, _VP, _VP]),
    "fr_normalize_trajectory": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_uint, _VP, C.POINTER(C.c_float), _VP]),
    "fr_transform_trajectory": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_float, C.c_float, _VP]),
    "fr_real_to_complex": (C.c_int, [_VP, C.c_size_t, _VP, _VP]),
    "fr_low_filter": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_uint), C.c_int, _VP]),
    "fr_normalize_channels": (C.c_int, [_VP, C.c_int, C.c_int, C.POINTER(C.c_uint), _VP]),
    "fr_sos_map": (C.c_int, [_VP, _VP, C.c_int, C.c_int, C.POINTER(C.c_uint), C.POINTER(C.c_uint), _VP, _VP]),
    "fr_recon_create": (C.c_int, [C.POINTER(ReconDesc), C.POINTER(_VP)]),
    "fr_recon_destroy": (C.c_int, [_VP]),
    "fr_recon_run": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP]),
    "fr_recon_run_host": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP]),
    "fr_recon_submit_host": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP]),
    "fr_recon_sync": (C.c_int, [_VP, _VP]),
    "fr_recon_plan": (C.c_int, [_VP, C.POINTER(_VP)]),
    "fr_recon_stage_ms": (C.c_int, [_VP, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_float)]),
}


def exported_symbols():
    """Names of every entry point the binding expects the library to export."""
    return list(_SIGS)


def load(path: str | None = None):
    """Load (once) and return the ctypes handle; raises if the library is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FastreconError(-1, "load", f"{p} not built; run __graft_entry__.build() or "
                                         "python fastrecon_gb300/build.py")
    lib = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int, where: str):
    if status != 0:
        lib = load()
        raise FastreconError(status, where, (lib.fr_status_string(status) or b"").decode() + ": " +
                             (lib.fr_last_error() or b"").decode())


def u3(vals):
    a = (C.c_uint * 3)()
    for i, v in enumerate(list(vals)[:3]):
        a[i] = int(v)
    return a
