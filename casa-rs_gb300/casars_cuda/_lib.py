"""ctypes binding of libcasars_cuda.so (declarations mirror include/casars_cuda.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises, and nothing falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libcasars_cuda.so")

CR_OK, CR_INVALID, CR_NO_SAMPLES, CR_BUFFER_SMALL, CR_CUDA, CR_NORMALIZATION, CR_TIMEOUT = range(7)
CR_HOST, CR_DEVICE = 0, 1
CR_WEIGHT_NATURAL, CR_WEIGHT_UNIFORM, CR_WEIGHT_BRIGGS = 0, 1, 2
STOP_REASONS = {0: None, 1: "GlobalThresholdReached", 2: "CycleThresholdReached",
                3: "NsigmaThresholdReached", 4: "NoCleanablePixels"}

_d, _f, _i32, _i64, _p = C.c_double, C.c_float, C.c_int32, C.c_int64, C.c_void_p
_err = C.POINTER(C.c_char_p)


class Geometry(C.Structure):
    _fields_ = [("nx", _i32), ("ny", _i32), ("cell_x_rad", _d), ("cell_y_rad", _d)]


class GridInfo(C.Structure):
    _fields_ = [("grid_nx", _i64), ("grid_ny", _i64), ("blc_x", _i64), ("blc_y", _i64),
                ("du", _d), ("dv", _d), ("oversampling", _i32)]


class WProjInfo(C.Structure):
    _fields_ = [("planes", _i32), ("sampling", _i32), ("w_scale", _d), ("max_support", _i32),
                ("kernel_width", _i32), ("cube_elements", _i64)]


class VisBatch(C.Structure):
    _fields_ = [("n", _i64), ("u", _p), ("v", _p), ("w", _p), ("weight", _p),
                ("sumwt_factor", _p), ("gridable", _p), ("vis", _p), ("location", _i32)]


class CubeBatch(C.Structure):
    _fields_ = [("rows", _i64), ("channels", _i32), ("u_m", _p), ("v_m", _p),
                ("lambda_scale", _p), ("vis", _p), ("weight", _p), ("flags", _p),
                ("location", _i32)]


class RowRuns(C.Structure):
    _fields_ = [("rows", _i64), ("channels", _i32), ("correlations", _i32), ("uvw_m", _p),
                ("lambda_scale", _p), ("data", _p), ("flag", _p), ("weight", _p),
                ("weight_spectrum", _p), ("gridable", _p), ("location", _i32)]


class Polarization(C.Structure):
    _fields_ = [("mode", _i32), ("corr0", _i32), ("corr1", _i32), ("transform", _i32),
                ("sumwt_factor", _f)]


class RowFeedConfig(C.Structure):
    _fields_ = [("max_live_row_blocks", _i32), ("row_block_rows", _i64), ("channels", _i32),
                ("correlations", _i32), ("lambda_scale", _p), ("polarization", Polarization),
                ("has_flag", _i32), ("has_weight_spectrum", _i32), ("has_gridable", _i32)]


class RowBlock(C.Structure):
    _fields_ = [("slot", _i32), ("max_rows", _i64), ("uvw_m", _p), ("data", _p), ("flag", _p),
                ("weight", _p), ("weight_spectrum", _p), ("gridable", _p)]


class RowFeedSummary(C.Structure):
    _fields_ = [("row_blocks", _i64), ("streamed_samples", _i64), ("source_bytes", _i64),
                ("live_row_block_high_water", _i32), ("producer_send_blocked_s", _d),
                ("consumer_recv_blocked_s", _d), ("consumer_elapsed_s", _d),
                ("producer_consumer_overlap_s", _d)]


class Beam(C.Structure):
    _fields_ = [("major_fwhm_rad", _d), ("minor_fwhm_rad", _d), ("position_angle_rad", _d)]


class Sums(C.Structure):
    _fields_ = [("normalization_sumwt", _d), ("reported_sumwt", _d), ("gridded", _i64),
                ("skipped", _i64), ("unique_records", _i64), ("taps", _i64)]


class PsfState(C.Structure):
    _fields_ = [("psf_peak", _f), ("normalization_sumwt", _f), ("reported_sumwt", _f)]


class Timings(C.Structure):
    _fields_ = [("plan_ms", _f), ("grid_ms", _f), ("degrid_ms", _f), ("fft_ms", _f),
                ("other_ms", _f), ("grid_kernel_ms", _f), ("degrid_kernel_ms", _f)]


# name -> (restype, argtypes); the exported symbol set checked by the tests
SIGNATURES = {
    "cr_version": (C.c_char_p, []),
    "cr_free_error": (None, [C.c_void_p]),
    "cr_ctx_create": (C.c_int, [_i32, C.POINTER(_p), _err]),
    "cr_ctx_destroy": (None, [_p]),
    "cr_ctx_set_stream": (C.c_int, [_p, _p, _err]),
    "cr_ctx_stream": (_p, [_p]),
    "cr_ctx_synchronize": (C.c_int, [_p, _err]),
    "cr_ctx_last_timings": (C.c_int, [_p, C.POINTER(Timings)]),
    "cr_ctx_launch_count": (_i64, [_p]),
    "cr_ctx_workspace_bytes": (_i64, [_p]),
    "cr_ctx_set_cube_graphs": (C.c_int, [_p, _i32]),
    "cr_ctx_set_wait_limits": (C.c_int, [_p, _i64, _i64]),
    "cr_ctx_set_cube_grid_chunk": (C.c_int, [_p, _i32]),
    "cr_ctx_set_image_fft_precision": (C.c_int, [_p, _i32]),
    "cr_ctx_set_image_fft_engine": (C.c_int, [_p, _i32]),
    "cr_ctx_set_alloc_limit": (C.c_int, [_p, _i64]),
    "cr_ctx_set_timings": (C.c_int, [_p, _i32]),
    "cr_accumulator_create": (C.c_int, [_p, _p, C.POINTER(_p), _err]),
    "cr_accumulator_destroy": (None, [_p]),
    "cr_accumulator_add": (C.c_int, [_p, _p, C.POINTER(VisBatch), C.POINTER(Sums), _err]),
    "cr_accumulator_finish": (C.c_int, [_p, _p, _p, _p, _i32, C.POINTER(PsfState),
                                        C.POINTER(Sums), _err]),
    "cr_clark": (C.c_int, [_p, _p, _p, _p, _p, _i32, _i32, _i32, _i32, _f, _f, _f, _f, _i64, _p,
                           _p, _p, _p, C.POINTER(_i64), C.POINTER(_i32), C.POINTER(_f), _err]),
    "cr_hogbom_planes": (C.c_int, [_p, _p, _p, _p, _p, _i32, _i32, _i32, _p, _i32, _f, _f, _f,
                                   _f, _p, _i64, _i32, _p, _p, _p, _p, _p, _p, _p, _err]),
    "cr_gridder_create": (C.c_int, [_p, C.POINTER(Geometry), _d, _i32, C.POINTER(_p),
                                    C.POINTER(GridInfo), _err]),
    "cr_gridder_destroy": (None, [_p]),
    "cr_gridder_tables": (C.c_int, [_p, _p, _p, _p, _err]),
    "cr_wproj_create": (C.c_int, [_p, _p, _d, _i32, _i32, _i32, _i32, C.POINTER(_p),
                                  C.POINTER(WProjInfo), _err]),
    "cr_wproj_destroy": (None, [_p]),
    "cr_wproj_tables": (C.c_int, [_p, _p, _p, _p, _err]),
    "cr_grid_dirty": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _p, _i32,
                                C.POINTER(Sums), _err]),
    "cr_degrid": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _i32, _p, _i32, _err]),
    "cr_grid_residual": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _i32, _p, _i32,
                                   C.POINTER(Sums), _err]),
    "cr_plan_create": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), C.POINTER(_p),
                                 C.POINTER(Sums), _err]),
    "cr_plan_destroy": (None, [_p]),
    "cr_plan_grid_dirty": (C.c_int, [_p, _p, _p, _p, _i32, _err]),
    "cr_plan_degrid": (C.c_int, [_p, _p, _p, _i32, _p, _i32, _err]),
    "cr_plan_grid_residual": (C.c_int, [_p, _p, _p, _i32, _p, _i32, _err]),
    "cr_cube_grid_dirty": (C.c_int, [_p, _p, C.POINTER(CubeBatch), _i32, _f, _p, _p, _i32,
                                     _p, _err]),
    "cr_cube_degrid": (C.c_int, [_p, _p, C.POINTER(CubeBatch), _i32, _f, _p, _i32, _p, _i32,
                                 _err]),
    "cr_cube_grid_degrid": (C.c_int, [_p, _p, C.POINTER(CubeBatch), _i32, _f, _p, _p, _p, _i32,
                                      _p, _i32, _p, _err]),
    "cr_cube_plan_create": (C.c_int, [_p, _p, C.POINTER(CubeBatch), _i32, _f, C.POINTER(_p),
                                       _p, _err]),
    "cr_cube_plan_destroy": (None, [_p]),
    "cr_cube_plan_channels": (_i32, [_p]),
    "cr_cube_plan_set_fft_precision": (C.c_int, [_p, _i32]),
    "cr_cube_plan_grid_dirty": (C.c_int, [_p, _p, _p, _p, _i32, _err]),
    "cr_cube_plan_degrid": (C.c_int, [_p, _p, _p, _i32, _p, _i32, _err]),
    "cr_cube_plan_grid_residual": (C.c_int, [_p, _p, _p, _i32, _p, _p, _i32, _err]),
    "cr_cube_plan_dirty_images": (C.c_int, [_p, _p, _p, _p, _i32, _p, _err]),
    "cr_cube_plan_residual_images": (C.c_int, [_p, _p, _p, _i32, _p, _p, _p, _i32, _err]),
    "cr_cube_sample_taps": (C.c_int, [_p, _p, C.POINTER(CubeBatch), _i32, _f, _p, _p, _p, _p,
                                      _p, _i32, _err]),
    "cr_fit_beam": (C.c_int, [_p, _p, _i32, _i32, _i32, _d, _d, _f, C.POINTER(Beam),
                              C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_f), _err]),
    "cr_restore": (C.c_int, [_p, _p, _p, _i32, _i32, _i32, _d, _d, C.POINTER(Beam), _p, _i32,
                             _err]),
    "cr_psf_sidelobe": (C.c_int, [_p, _p, _i32, _i32, _i32, _d, _d, C.POINTER(Beam),
                                  C.POINTER(_f), _err]),
    "cr_plan_residual_image": (C.c_int, [_p, _p, _p, _i32, C.POINTER(PsfState), _p, _i32,
                                         _err]),
    "cr_grid_to_image": (C.c_int, [_p, _p, _p, _p, _i32, _f, _p, _i32, _err]),
    "cr_image_to_grid": (C.c_int, [_p, _p, _p, _p, _i32, _p, _i32, _err]),
    "cr_dirty_image": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _p, _i32,
                                 C.POINTER(PsfState), C.POINTER(Sums), _err]),
    "cr_residual_image": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _i32,
                                    C.POINTER(PsfState), _p, _i32, C.POINTER(Sums), _err]),
    "cr_predict": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _i32, _p, _i32, _err]),
    "cr_adjoint": (C.c_int, [_p, _p, _p, C.POINTER(VisBatch), _p, _i32, _err]),
    "cr_apply_weighting": (C.c_int, [_p, _p, C.POINTER(VisBatch), _i32, _f, _p, _i32,
                                     C.POINTER(_f), _err]),
    "cr_row_runs_prepare": (C.c_int, [_p, C.POINTER(RowRuns), C.POINTER(Polarization), _p, _p, _p,
                                       _p, _p, _p, _p, _p, _p, _i32, C.POINTER(_i64), _err]),
    "cr_row_feed_create": (C.c_int, [_p, _p, C.POINTER(RowFeedConfig), C.POINTER(_p), _err]),
    "cr_row_feed_destroy": (None, [_p]),
    "cr_row_feed_acquire": (C.c_int, [_p, C.POINTER(RowBlock), _err]),
    "cr_row_feed_submit": (C.c_int, [_p, _i32, _i64, _err]),
    "cr_row_feed_finish": (C.c_int, [_p, _p, _p, _i32, C.POINTER(PsfState), C.POINTER(Sums),
                                     C.POINTER(RowFeedSummary), _err]),
    "cr_polarization_for_plane": (C.c_int, [_i32, _p, _i32, C.POINTER(Polarization), _err]),
    "cr_apply_weighting_rows": (C.c_int, [_p, _p, C.POINTER(VisBatch), _p, _p, _i32, _f, _p, _i32,
                                          _p, _err]),
    "cr_apply_weighting_plane": (C.c_int, [_p, _p, C.POINTER(VisBatch), _i32, _f, _p, _i32,
                                     C.POINTER(_f), _err]),
    "cr_hogbom": (C.c_int, [_p, _p, _p, _p, _p, _i32, _i32, _i32, _f, _f, _f, _f, _i64, _i32,
                            _p, _p, _p, _p, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i32),
                            _err]),
    "cr_hogbom_plane": (C.c_int, [_p, _p, _p, _p, _p, _i32, _i32, _i32, _f, _f, _f, _f, _i64,
                                  _i32, _p, _p, _p, _p, C.POINTER(_i64), C.POINTER(_i64),
                                  _err]),
    "cr_multiscale_create": (C.c_int, [_p, _p, _p, _i32, _i32, _i32, _p, _i32, _f,
                                       C.POINTER(_p), _err]),
    "cr_multiscale_destroy": (None, [_p]),
    "cr_multiscale_set_residual": (C.c_int, [_p, _p, _i32, _err]),
    "cr_multiscale_residual": (C.c_int, [_p, _p, _i32, _err]),
    "cr_multiscale_peak": (C.c_int, [_p, C.POINTER(_i32), C.POINTER(_f), _err]),
    "cr_multiscale_minor_cycle": (C.c_int, [_p, _p, _i32, _f, _f, _f, _f, _i64, _p, _p, _p, _p,
                                            _p, C.POINTER(_i64), C.POINTER(_i64),
                                            C.POINTER(_i32), _err]),
    "cr_probe_tap_rate": (C.c_int, [_p, _i64, _i32, C.POINTER(_d), C.POINTER(_d), _err]),
    "cr_robust_rms": (C.c_int, [_p, _p, _p, _i32, _i32, _i32, _i32, _p, _i32, _p, _p, _p,
                                _err]),
    "cr_hogbom_noalloc": (C.c_int, [_p, _p, _p, _p, _p, _i32, _i32, _f, _f, _f, _f, _i64, _i32,
                                    _p, _p, _p, _p, C.POINTER(_i64), C.POINTER(_i64),
                                    C.POINTER(_i32), _err]),
}

_LIB = None
_LOCK = threading.Lock()


class CasarsCudaError(RuntimeError):
    """A non-zero status from the C ABI (mirrors casa-imaging's ImagingError)."""

    KINDS = {CR_INVALID: "InvalidRequest", CR_NO_SAMPLES: "NoUsableSamples",
             CR_BUFFER_SMALL: "BufferTooSmall", CR_CUDA: "Cuda",
             CR_NORMALIZATION: "Normalization", CR_TIMEOUT: "Timeout"}

    def __init__(self, code: int, message: str):
        self.code = code
        self.kind = self.KINDS.get(code, f"Status{code}")
        super().__init__(f"{self.kind}: {message}")


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load (not build) the library; raise if it is absent."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build it with `python casa-rs_gb300/build.py` "
                "(there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def call(name: str, *args):
    """Call an ABI function that takes a trailing char** err; raise on error."""
    lib = load()
    err = C.c_char_p()
    rc = getattr(lib, name)(*args, C.byref(err))
    if rc != CR_OK:
        msg = err.value.decode() if err.value else ""
        if err.value:
            lib.cr_free_error(C.cast(err, C.c_void_p))
        raise CasarsCudaError(rc, f"{name}: {msg}")
    return rc
