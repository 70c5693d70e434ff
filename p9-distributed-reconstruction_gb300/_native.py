"""ctypes binding of libp9idg.so (declarations mirror include/p9idg.h).

The library is the product: there is no fallback.  If it is missing, loading raises
NativeLibraryMissing; compute calls on a machine without a GPU return P9IDG_NO_DEVICE.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libp9idg.so")

OK = 0
INVALID_ARGUMENT = 1
CANNOT_PLACE = 2
SUBGRID_OUT_OF_GRID = 3
INVALID_GRID = 4
OUT_OF_MEMORY = 5
CUDA_ERROR = 6
NO_DEVICE = 7
UNSUPPORTED = 8
DEVICE_CHECK_FAILED = 9

MODE_FP32 = 0
MODE_TC_BF16X3 = 1
MODE_TC_FP16X3 = 2

STAGES = ["gridder", "subgrid_ifft_add", "split_subgrid_fft", "degridder", "layer_fft", "h2d", "d2h", "convert"]


class NativeLibraryMissing(RuntimeError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("vis_count", ctypes.c_int64), ("grid_size", ctypes.c_int32), ("subgrid_size", ctypes.c_int32),
                ("kernel_size", ctypes.c_int32), ("max_timesteps", ctypes.c_int32), ("scale_arcsec", ctypes.c_float),
                ("wlayer_count", ctypes.c_int32), ("wstep", ctypes.c_double)]


class SubgridC(ctypes.Structure):
    _fields_ = [("baseline_idx", ctypes.c_int32), ("time_sample_start", ctypes.c_int32),
                ("time_sample_count", ctypes.c_int32), ("u_pixel", ctypes.c_int32), ("v_pixel", ctypes.c_int32),
                ("w_lambda", ctypes.c_int32)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("num_subgrids", ctypes.c_int64), ("input_visibilities", ctypes.c_int64),
                ("gridded_visibilities", ctypes.c_int64), ("work_items", ctypes.c_int64),
                ("nbl", ctypes.c_int32), ("nt", ctypes.c_int32), ("nch", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("requested_mode", ctypes.c_int32), ("tc_w_term", ctypes.c_double), ("tc_order", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


# Largest |dw r| of the tensor-core forms: first order (P9IDG_TC_MAX_W_TERM) and second order
# (P9IDG_TC_MAX_W_TERM2)
TC_MAX_W_TERM = 0.01
TC_MAX_W_TERM2 = 0.03


# name -> (restype, argtypes); every symbol include/p9idg.h declares
P = ctypes.c_void_p
i32, i64, dbl, f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_float
SIGNATURES = {
    "p9idg_plan_create": (i32, [P, P, i32, i32, P, i32, ctypes.POINTER(P)]),
    "p9idg_plan_create_from_subgrids": (i32, [P, P, i64, P, i32, i32, P, i32, ctypes.POINTER(P)]),
    "p9idg_plan_num_subgrids": (i32, [P, ctypes.POINTER(i64)]),
    "p9idg_plan_get_subgrids": (i32, [P, P, i64]),
    "p9idg_plan_get_info": (i32, [P, ctypes.POINTER(PlanInfo)]),
    "p9idg_plan_set_mode": (i32, [P, i32]),
    "p9idg_plan_set_tc_order": (i32, [P, i32]),
    "p9idg_plan_set_taper": (i32, [P, P]),
    "p9idg_plan_set_stream": (i32, [P, P]),
    "p9idg_plan_get_stream": (i32, [P, ctypes.POINTER(P)]),
    "p9idg_plan_destroy": (None, [P]),
    "p9idg_grid": (i32, [P, P, P, P]),
    "p9idg_degrid": (i32, [P, P, P, P]),
    "p9idg_grid_w": (i32, [P, P, P, P]),
    "p9idg_degrid_w": (i32, [P, P, P, P]),
    "p9idg_grid_psf": (i32, [P, P, P, P]),
    "p9idg_to_image": (i32, [P, P, P, P]),
    "p9idg_calculate_psf": (i32, [P, P, P, P]),
    "p9idg_wstack_ifft_float": (i32, [P, i32, i32, i64, P]),
    "p9idg_fft_forward_float": (i32, [P, i32, dbl, P]),
    "p9idg_fft_backward_float": (i32, [P, i32, dbl, P]),
    "p9idg_fft_shift": (i32, [P, i32, i32]),
    "p9idg_grid_w_device": (i32, [P, P, P]),
    "p9idg_degrid_w_device": (i32, [P, P, P]),
    "p9idg_grid_device": (i32, [P, P, P]),
    "p9idg_degrid_device": (i32, [P, P, P]),
    "p9idg_wstack_image_device": (i32, [P, P, P, i32]),
    "p9idg_synchronize": (i32, [P]),
    "p9idg_grid_w_device_noalloc": (i32, [P, P, i64, P, i32, i32, P, i32, P, P, P]),
    "p9idg_plan_enable_timing": (i32, [P, i32]),
    "p9idg_plan_stage_times": (i32, [P, P, P]),
    "p9idg_debug_fail_device_allocations": (i32, [i64]),
    "p9idg_debug_tc_wait": (i32, [i64, i32]),
    "p9idg_plan_reset_timing": (i32, [P]),
    "p9idg_last_error": (ctypes.c_char_p, []),
    "p9idg_version": (ctypes.c_char_p, []),
    "p9idg_device_count": (i32, []),
    "p9idg_measure_sincos_peak": (i32, [ctypes.POINTER(dbl), ctypes.POINTER(dbl)]),
    "p9idg_tc_selftest": (i32, [i32, i32, ctypes.POINTER(dbl)]),
    "p9idg_plan_set_chunking": (i32, [P, i32, i32]),
    "p9idg_batch_create": (i32, [ctypes.POINTER(P), i32, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P),
                                 ctypes.POINTER(P), ctypes.POINTER(P)]),
    "p9idg_batch_grid_w": (i32, [P]),
    "p9idg_batch_degrid_w": (i32, [P]),
    "p9idg_batch_capture_graph": (i32, [P]),
    "p9idg_batch_run": (i32, [P]),
    "p9idg_batch_set_schedule": (i32, [P, i32]),
    "p9idg_batch_synchronize": (i32, [P]),
    "p9idg_batch_latencies": (i32, [P, P]),
    "p9idg_batch_get_stream": (i32, [P, ctypes.POINTER(P)]),
    "p9idg_batch_destroy": (None, [P]),
    "p9idg_autotune": (i32, [P, P, i32, i32, P, i32, i32, P, i32, P]),
    "p9idg_plan_get_params": (i32, [P, P]),
    "p9idg_plan_init_device": (i32, [P]),
    "p9idg_plan_set_host_access": (i32, [P, i32]),
    "p9idg_plan_get_host_access": (i32, [P, ctypes.POINTER(i32)]),
    "p9idg_cd_create": (i32, [i32, P, i32, i32, ctypes.POINTER(P)]),
    "p9idg_cd_max_lipschitz": (i32, [P, ctypes.POINTER(f32)]),
    "p9idg_cd_get_maps": (i32, [P, P, P]),
    "p9idg_cd_psf2_size": (i32, [P, ctypes.POINTER(i32), ctypes.POINTER(i32)]),
    "p9idg_cd_set_stream": (i32, [P, P]),
    "p9idg_cd_deconvolve": (i32, [P, P, P, f32, f32, i32, f32, P]),
    "p9idg_cd_deconvolve_device": (i32, [P, P, P, f32, f32, i32, f32, P]),
    "p9idg_cd_deconvolve_path": (i32, [P, P, P, f32, f32, f32, i32, i32, f32, P]),
    "p9idg_cd_get_abs_max_diff": (i32, [P, P, P, f32, f32, ctypes.POINTER(f32)]),
    "p9idg_cd_get_abs_max_diff_device": (i32, [P, P, P, f32, f32, ctypes.POINTER(f32)]),
    "p9idg_cd_reset_lipschitz_map": (i32, [P, P, i32, i32]),
    "p9idg_cd_destroy": (None, [P]),
    "p9idg_convolver_create": (i32, [P, i32, i32, i32, i32, ctypes.POINTER(P)]),
    "p9idg_convolver_create_correlation": (i32, [P, i32, i32, i32, ctypes.POINTER(P)]),
    "p9idg_convolver_convolve": (i32, [P, P, i32, P]),
    "p9idg_convolver_convolve_device": (i32, [P, P, i32, P]),
    "p9idg_convolver_destroy": (None, [P]),
    "p9idg_psf_padded_fourier_correlation": (i32, [P, i32, i32, i32, i32, P]),
    "p9idg_psf_squared": (i32, [P, i32, i32, P]),
    "p9idg_psf_amap": (i32, [P, i32, i32, i32, i32, P]),
    "p9idg_major_cycle_serial_cd": (i32, [P, P, P, P, P, P, P, P, ctypes.POINTER(i32)]),
    "p9idg_major_cycle_serial_cd_device": (i32, [P, P, P, P, P, P, P, P, ctypes.POINTER(i32)]),
    "p9idg_fits_shape": (i32, [ctypes.c_char_p, ctypes.POINTER(i32), ctypes.POINTER(i32), P, i32]),
    "p9idg_fits_read_uvw": (i32, [ctypes.c_char_p, i32, i32, P]),
    "p9idg_fits_read_frequencies": (i32, [ctypes.c_char_p, P, i64]),
    "p9idg_fits_read_visibilities": (i32, [ctypes.c_char_p, i32, i32, i32, i32, dbl, P]),
    "p9idg_fits_read_flags": (i32, [ctypes.c_char_p, i32, i32, i32, i32, P]),
    "p9idg_fits_read_image": (i32, [ctypes.c_char_p, i32, P, i64]),
    "p9idg_fits_write_image": (i32, [ctypes.c_char_p, i32, P, i32, i32]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryMissing(
                f"{LIB_PATH} is not built; run __graft_entry__.build() (nvcc for sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().p9idg_last_error().decode(errors="replace")
