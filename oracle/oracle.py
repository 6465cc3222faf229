"""Python face of the FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker or as the CPU timing baseline.  The product
library in casa-rs_gb300/ never imports it.

The heavy loops live in casa_oracle.c; this module adds the parts the
reference delegates to rustfft 6.4.1 (the centred 2-D DFT, restated here with
numpy's float64 pocketfft) and the image-domain normalisation.  Each function
cites the reference function (file:line, relative to crates/casa-imaging/src)
it restates.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        _LIB = C.CDLL(path)
        _declare(_LIB)
    return _LIB


_d = C.c_double
_f = C.c_float
_i32 = C.c_int32
_i64 = C.c_int64
_p = C.c_void_p


class Accum(C.Structure):
    _fields_ = [("normalization_sumwt", _d), ("reported_sumwt", _d),
                ("gridded", _i64), ("skipped", _i64)]


class StdParams(C.Structure):
    _fields_ = [("gnx", _i64), ("gny", _i64), ("oversampling", _i32), ("support", _i32),
                ("du", _d), ("dv", _d), ("taps", _p), ("tap_rows", _i32)]


class WpParams(C.Structure):
    _fields_ = [("gnx", _i64), ("gny", _i64), ("du", _d), ("dv", _d), ("planes", _i32),
                ("sampling", _i32), ("w_scale", _d), ("width", _i32), ("support", _p),
                ("kernels", _p), ("norm_radius", _i32), ("norm_table", _p)]


def _declare(L):
    sig = {
        "oc_casa_composite_padded_len": (_i64, [_i64, _d]),
        "oc_image_blc": (None, [_i64, _i64, C.POINTER(_i64)]),
        "oc_grdsf": (_d, [_d]),
        "oc_spheroidal_kernel": (_f, [_d, _d]),
        "oc_std_kernel_table": (None, [_i32, _i32, _p]),
        "oc_std_tap_rows": (_i32, [_i32]),
        "oc_std_normalized_taps": (None, [_p, _i32, _i32, _i32, _p]),
        "oc_correction_axis": (None, [_i64, _p]),
        "oc_gridder_correction_axis": (None, [_i64, _p]),
        "oc_sinc_axis": (None, [_i64, _i64, _p]),
        "oc_std_plan": (C.c_int, [C.POINTER(StdParams), _d, _d, C.POINTER(_i64),
                                  C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)]),
        "oc_std_grid_dirty": (None, [C.POINTER(StdParams), _i64, _p, _p, _p, _p, _p, _p, _p,
                                     _p, C.POINTER(Accum), _i32]),
        "oc_std_degrid": (None, [C.POINTER(StdParams), _p, _i64, _p, _p, _p]),
        "oc_std_residual": (None, [C.POINTER(StdParams), _p, _i64, _p, _p, _p, _p, _p, _p,
                                   _p, _p, C.POINTER(Accum), _i32]),
        "oc_wproj_suggested_planes": (_i64, [_i64, _i64, _d, _d, _d]),
        "oc_wproj_max_uvw": (_d, [_d, _d, C.c_int]),
        "oc_wproj_build": (C.c_int, [_i64, _i64, _d, _d, _i64, _i64, _d, _i32, C.c_int, _i32,
                                     _i32, _i32, _i32, _i32, C.POINTER(_d), _p,
                                     C.POINTER(_i32), _p, _p]),
        "oc_wproj_plane_index": (_i32, [C.POINTER(WpParams), _d]),
        "oc_wproj_plan": (C.c_int, [C.POINTER(WpParams), _d, _d, _d, C.POINTER(_i64),
                                    C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64),
                                    C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_d)]),
        "oc_wproj_grid_dirty": (None, [C.POINTER(WpParams), _i64, _p, _p, _p, _p, _p, _p,
                                       _p, _p, _p, C.POINTER(Accum), _i32]),
        "oc_wproj_degrid": (None, [C.POINTER(WpParams), _p, _i64, _p, _p, _p, _p, _i32]),
        "oc_wproj_residual": (None, [C.POINTER(WpParams), _p, _i64, _p, _p, _p, _p, _p, _p,
                                     _p, _p, C.POINTER(Accum), _i32]),
        "oc_density_cell": (C.c_int, [_i64, _i64, _d, _d, _d, _d, C.c_int, C.POINTER(_i64),
                                      C.POINTER(_i64)]),
        "oc_density_grid": (None, [_i64, _i64, _d, _d, _i64, _p, _p, _p, _p]),
        "oc_density_grid_conv": (None, [_i64, _i64, _d, _d, _i64, _p, _p, _p, C.c_int, _p]),
        "oc_reweight_conv": (None, [_i64, _i64, _d, _d, _i64, _p, _p, _p, _p, C.c_int, _f,
                                    C.c_int, _p]),
        "oc_std_plan_many": (None, [C.POINTER(StdParams), _i64, _p, _p, _p, _p, _p, _p]),
        "oc_briggs_f2": (_f, [_p, _i64, _f]),
        "oc_briggs_denominator": (_f, [_f, _f]),
        "oc_reweight": (None, [_i64, _i64, _d, _d, _i64, _p, _p, _p, _p, C.c_int, _f, _p]),
        "oc_peak_location": (C.c_int, [_p, _p, _i64, _i64, C.POINTER(_i64), C.POINTER(_i64),
                                       C.POINTER(_f)]),
        "oc_minor_cycle_stop_reason": (C.c_int, [_f, _f, _f, _f]),
        "oc_hogbom": (_i64, [_p, _p, _p, _p, _i64, _i64, _f, _f, _f, _f, _i64, C.c_int, _p,
                             _p, _p, _p, C.POINTER(_i32), C.POINTER(_i64)]),
        "oc_subtract_shifted_psf": (None, [_p, _p, _i64, _i64, _i64, _i64, _f]),
        "oc_peak_relative": (C.c_int, [_p, _p, _i64, _i64, _f, C.POINTER(_i64),
                                       C.POINTER(_i64), C.POINTER(_f)]),
        "oc_hogbom_plane": (_i64, [_p, _p, _p, _p, _i64, _i64, _f, _f, _f, _f, _i64, C.c_int,
                                   _p, _p, _p, _p, C.POINTER(_i64)]),
        "oc_wproj_grid_dirty_f32": (None, [C.POINTER(WpParams), _p, _i64, _p, _p, _p, _p, _p, _p,
                                           _p, _p, _p, C.POINTER(Accum), _i32]),
        "oc_wproj_degrid_f32": (None, [C.POINTER(WpParams), _p, _p, _i64, _p, _p, _p, _p, _i32]),
        "oc_mean_stddev": (None, [_p, _i64, C.POINTER(_d), C.POINTER(_d)]),
        "oc_chauvenet_max_zscore": (_d, [C.c_uint64]),
        "oc_chauvenet_clip": (_i64, [_p, _i64, _d, _i32]),
        "oc_madfm": (_d, [_p, _i64, C.POINTER(_d)]),
        "oc_robust_rms": (_f, [_p, _p, _i64, C.POINTER(_d), C.POINTER(_i64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _ptr(a):
    return None if a is None else a.ctypes.data


def _c(a, dtype):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


# --------------------------------------------------------------------------
# geometry
# --------------------------------------------------------------------------
def padded_len(image_len: int, padding: float = 1.2) -> int:
    """casa_composite_padded_len (gridder.rs:4152-4173)."""
    return int(lib().oc_casa_composite_padded_len(image_len, padding))


def image_blc(grid_len: int, image_len: int) -> int:
    """image_blc (gridder.rs:401-404)."""
    out = _i64()
    lib().oc_image_blc(grid_len, image_len, C.byref(out))
    return int(out.value)


def grdsf(nu: float) -> float:
    return float(lib().oc_grdsf(nu))


def correction_axis(size: int) -> np.ndarray:
    """build_correction_axis (gridder.rs:4175-4188)."""
    out = np.zeros(size, np.float32)
    lib().oc_correction_axis(size, _ptr(out))
    return out


def sinc_axis(size: int, conv_sampling: int) -> np.ndarray:
    """build_sinc_axis (gridder.rs:4211-4228)."""
    out = np.zeros(size, np.float32)
    lib().oc_sinc_axis(size, conv_sampling, _ptr(out))
    return out


def std_taps(oversampling: int, support: int = 3) -> np.ndarray:
    """Kernel table and normalised tap rows (gridder.rs:407-416, 2026-2051)."""
    tlen = oversampling * (support + 1)
    table = np.zeros(tlen, np.float32)
    lib().oc_std_kernel_table(oversampling, support, _ptr(table))
    rows = int(lib().oc_std_tap_rows(oversampling))
    taps = np.zeros((rows, 2 * support + 1), np.float32)
    lib().oc_std_normalized_taps(_ptr(table), tlen, oversampling, support, _ptr(taps))
    return taps


# --------------------------------------------------------------------------
# centred FFTs (fft.rs:600-630; rustfft's DFT restated as float64 pocketfft)
# --------------------------------------------------------------------------
def centered_ifft2(grid: np.ndarray) -> np.ndarray:
    """ifftshift -> inverse DFT scaled by 1/(Nx Ny) -> fftshift (fft.rs:611-624)."""
    g = np.asarray(grid, np.complex128)
    return np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(g)))


def centered_fft2(grid: np.ndarray) -> np.ndarray:
    """ifftshift -> unscaled forward DFT -> fftshift (fft.rs:34, 600-630)."""
    g = np.asarray(grid, np.complex128)
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(g)))


# --------------------------------------------------------------------------
# standard gridder
# --------------------------------------------------------------------------
@dataclass
class Geometry:
    nx: int
    ny: int
    cell_x: float
    cell_y: float


class StdGridder:
    """StandardGridder (gridder.rs:322-443) at a chosen oversampling."""

    def __init__(self, geom: Geometry, oversampling: int = 100, padding: float = 1.2):
        self.geom = geom
        self.os = oversampling
        self.gnx = padded_len(geom.nx, padding)
        self.gny = padded_len(geom.ny, padding)
        self.blc_x = image_blc(self.gnx, geom.nx)
        self.blc_y = image_blc(self.gny, geom.ny)
        self.du = 1.0 / (self.gnx * geom.cell_x)
        self.dv = 1.0 / (self.gny * geom.cell_y)
        self.taps = std_taps(oversampling)
        self.corr_x = correction_axis(self.gnx)
        self.corr_y = correction_axis(self.gny)
        self._p = StdParams(self.gnx, self.gny, oversampling, 3, self.du, self.dv,
                            self.taps.ctypes.data, self.taps.shape[0])

    def plan(self, u: float, v: float):
        x0, y0, wx, wy = _i64(), _i64(), _i64(), _i64()
        ok = lib().oc_std_plan(C.byref(self._p), u, v, C.byref(x0), C.byref(y0), C.byref(wx),
                               C.byref(wy))
        return (int(x0.value), int(y0.value), int(wx.value), int(wy.value)) if ok else None

    def plan_many(self, u, v):
        """sample_tap_span over arrays: (start x, start y, x tap row, y tap row),
        -1 where the sample is rejected."""
        u, v = _c(u, np.float64), _c(v, np.float64)
        out = [np.zeros(len(u), np.int32) for _ in range(4)]
        lib().oc_std_plan_many(C.byref(self._p), len(u), _ptr(u), _ptr(v), *[_ptr(o) for o in out])
        return out

    def grid_dirty(self, u, v, weight, vis, sumwt_factor=None, gridable=None, threads=1):
        """accumulate_dirty_psf_and_residual_standard_streaming_grid (lib.rs:68306-68500)."""
        n = len(u)
        u, v = _c(u, np.float64), _c(v, np.float64)
        weight, sumwt_factor = _c(weight, np.float32), _c(sumwt_factor, np.float32)
        gridable = _c(gridable, np.uint8)
        vis = _c(vis, np.complex64)
        psf = np.zeros((self.gnx, self.gny), np.complex128)
        dirty = np.zeros((self.gnx, self.gny), np.complex128)
        acc = Accum()
        lib().oc_std_grid_dirty(C.byref(self._p), n, _ptr(u), _ptr(v), _ptr(weight),
                                _ptr(sumwt_factor), _ptr(gridable), _ptr(vis), _ptr(psf),
                                _ptr(dirty), C.byref(acc), threads)
        return psf, dirty, acc

    def degrid(self, model_grid, u, v):
        """degrid_sample_taps_planned_normalized (gridder.rs:1278-1312), FP64."""
        g = _c(model_grid, np.complex128)
        u, v = _c(u, np.float64), _c(v, np.float64)
        pred = np.zeros(len(u), np.complex128)
        lib().oc_std_degrid(C.byref(self._p), _ptr(g), len(u), _ptr(u), _ptr(v), _ptr(pred))
        return pred

    def residual(self, model_grid, u, v, weight, vis, sumwt_factor=None, gridable=None,
                 threads=1):
        """degrid_model_and_grid_residual_taps_planned_f64 (gridder.rs:1315-1396)."""
        n = len(u)
        g = _c(model_grid, np.complex128)
        u, v = _c(u, np.float64), _c(v, np.float64)
        weight, sumwt_factor = _c(weight, np.float32), _c(sumwt_factor, np.float32)
        gridable = _c(gridable, np.uint8)
        vis = _c(vis, np.complex64)
        res = np.zeros((self.gnx, self.gny), np.complex128)
        pred = np.zeros(n, np.complex128)
        acc = Accum()
        lib().oc_std_residual(C.byref(self._p), _ptr(g), n, _ptr(u), _ptr(v), _ptr(weight),
                              _ptr(sumwt_factor), _ptr(gridable), _ptr(vis), _ptr(res),
                              _ptr(pred), C.byref(acc), threads)
        return res, pred, acc

    # image-domain stages --------------------------------------------------
    def corrected_image(self, raw: np.ndarray) -> np.ndarray:
        """corrected_image_from_grid_f64 (gridder.rs:1646-1657)."""
        nx, ny = self.geom.nx, self.geom.ny
        sub = raw[self.blc_x:self.blc_x + nx, self.blc_y:self.blc_y + ny].real
        corr = (self.corr_x[self.blc_x:self.blc_x + nx, None].astype(np.float64)
                * self.corr_y[None, self.blc_y:self.blc_y + ny].astype(np.float64))
        return sub * corr

    def apodize(self, model: np.ndarray) -> np.ndarray:
        """apodize_model (gridder.rs:1554-1570)."""
        out = np.zeros((self.gnx, self.gny), np.complex128)
        nx, ny = self.geom.nx, self.geom.ny
        corr = (self.corr_x[self.blc_x:self.blc_x + nx, None].astype(np.float64)
                * self.corr_y[None, self.blc_y:self.blc_y + ny].astype(np.float64))
        out[self.blc_x:self.blc_x + nx, self.blc_y:self.blc_y + ny] = model * corr
        return out

    def model_grid(self, model: np.ndarray) -> np.ndarray:
        """centered_fft2(apodize_model(model)) (lib.rs:69000; gridder.rs:1554)."""
        return centered_fft2(self.apodize(model))

    def dirty_products(self, psf_grid, dirty_grid, acc: Accum):
        """dirty_grids_to_psf_and_residual_owned (lib.rs:48987-49130)."""
        if acc.normalization_sumwt <= 0.0:
            raise ValueError("no usable samples")
        psf = self.corrected_image(centered_ifft2(psf_grid)) / acc.normalization_sumwt
        peak = float(np.max(np.abs(psf)))
        psf = psf / peak
        res = self.corrected_image(centered_ifft2(dirty_grid)) / acc.normalization_sumwt / peak
        return psf, res, peak


# --------------------------------------------------------------------------
# W-projection
# --------------------------------------------------------------------------
class WProjector:
    """WProjector (gridder.rs:3391-3855), FP64 kernels."""

    def __init__(self, geom: Geometry, gridder: StdGridder, max_abs_w: float, planes=None,
                 sampling=None, support_min=0, support_max=0, threads=8, max_width=4096):
        self.geom = geom
        self.gridder = gridder
        explicit = planes is not None
        if planes is None:
            planes = max(1, int(lib().oc_wproj_suggested_planes(
                geom.nx, geom.ny, geom.cell_x, geom.cell_y, max_abs_w)))
        if sampling is None:
            sampling = 4 if planes > 1 else 1
        self.planes = planes
        self.sampling = sampling
        self.norm_radius = (sampling + 1) // 2
        L = 2 * self.norm_radius + 1
        conv = max(gridder.gnx, gridder.gny)
        quarter = conv // 2 - 1
        if support_min > 0:
            cap = min(max_width, support_max * sampling + self.norm_radius + 1)
        else:
            cap = min(max_width, max(quarter // sampling - 1, 1) * sampling + self.norm_radius + 1,
                      quarter)
        kern = np.zeros((planes, cap, cap), np.complex128)
        norm = np.zeros((planes, L, L), np.float64)
        support = np.zeros(planes, np.int32)
        w_scale = _d()
        width = _i32()
        rc = lib().oc_wproj_build(geom.nx, geom.ny, geom.cell_x, geom.cell_y, gridder.gnx,
                                  gridder.gny, max_abs_w, planes, int(explicit), sampling,
                                  support_min, support_max, cap, threads, C.byref(w_scale),
                                  _ptr(support), C.byref(width), _ptr(kern), _ptr(norm))
        if rc != 0:
            raise ValueError(f"oc_wproj_build failed with status {rc}")
        W = int(width.value)
        flat = kern.reshape(-1)[: planes * W * W]
        self.kernels = np.ascontiguousarray(flat.reshape(planes, W, W))
        self.norm = norm
        self.support = support
        self.width = W
        self.w_scale = float(w_scale.value)
        self._bind()

    @classmethod
    def from_arrays(cls, geom, gridder, w_scale, support, kernels, norm, sampling):
        """A projector over given kernel arrays (for timing with kernels built elsewhere)."""
        self = cls.__new__(cls)
        self.geom, self.gridder = geom, gridder
        self.planes = len(support)
        self.sampling = sampling
        self.norm_radius = (sampling + 1) // 2
        self.kernels = np.ascontiguousarray(kernels, np.complex128)
        self.norm = np.ascontiguousarray(norm, np.float64)
        self.support = np.ascontiguousarray(support, np.int32)
        self.width = self.kernels.shape[1]
        self.w_scale = float(w_scale)
        self._bind()
        return self

    def _bind(self):
        g = self.gridder
        self._p = WpParams(g.gnx, g.gny, g.du, g.dv, self.planes, self.sampling, self.w_scale,
                           self.width, self.support.ctypes.data, self.kernels.ctypes.data,
                           self.norm_radius, self.norm.ctypes.data)

    def plan(self, u, v, w):
        lx, ly, ox, oy = _i64(), _i64(), _i64(), _i64()
        pl, cj, nrm = _i32(), _i32(), _d()
        ok = lib().oc_wproj_plan(C.byref(self._p), u, v, w, C.byref(lx), C.byref(ly),
                                 C.byref(ox), C.byref(oy), C.byref(pl), C.byref(cj),
                                 C.byref(nrm))
        if not ok:
            return None
        return dict(loc_x=lx.value, loc_y=ly.value, off_x=ox.value, off_y=oy.value,
                    plane=pl.value, conj=bool(cj.value), normalization=nrm.value)

    def grid_dirty(self, u, v, w, weight, vis, sumwt_factor=None, gridable=None, threads=1):
        n = len(u)
        u, v, w = _c(u, np.float64), _c(v, np.float64), _c(w, np.float64)
        weight, sumwt_factor = _c(weight, np.float32), _c(sumwt_factor, np.float32)
        gridable = _c(gridable, np.uint8)
        vis = _c(vis, np.complex64)
        g = self.gridder
        psf = np.zeros((g.gnx, g.gny), np.complex128)
        dirty = np.zeros((g.gnx, g.gny), np.complex128)
        acc = Accum()
        lib().oc_wproj_grid_dirty(C.byref(self._p), n, _ptr(u), _ptr(v), _ptr(w), _ptr(weight),
                                  _ptr(sumwt_factor), _ptr(gridable), _ptr(vis), _ptr(psf),
                                  _ptr(dirty), C.byref(acc), threads)
        return psf, dirty, acc

    def degrid(self, model_grid, u, v, w, threads=1):
        g = _c(model_grid, np.complex128)
        u, v, w = _c(u, np.float64), _c(v, np.float64), _c(w, np.float64)
        pred = np.zeros(len(u), np.complex128)
        lib().oc_wproj_degrid(C.byref(self._p), _ptr(g), len(u), _ptr(u), _ptr(v), _ptr(w),
                              _ptr(pred), threads)
        return pred

    def residual(self, model_grid, u, v, w, weight, vis, sumwt_factor=None, gridable=None,
                 threads=1):
        n = len(u)
        g = _c(model_grid, np.complex128)
        u, v, w = _c(u, np.float64), _c(v, np.float64), _c(w, np.float64)
        weight, sumwt_factor = _c(weight, np.float32), _c(sumwt_factor, np.float32)
        gridable = _c(gridable, np.uint8)
        vis = _c(vis, np.complex64)
        gr = self.gridder
        res = np.zeros((gr.gnx, gr.gny), np.complex128)
        acc = Accum()
        lib().oc_wproj_residual(C.byref(self._p), _ptr(g), n, _ptr(u), _ptr(v), _ptr(w),
                                _ptr(weight), _ptr(sumwt_factor), _ptr(gridable), _ptr(vis),
                                _ptr(res), C.byref(acc), threads)
        return res, acc

    # the reference's Complex32 precision (timed CPU baseline) -------------
    def _k32(self):
        if getattr(self, "_kernels32", None) is None:
            self._kernels32 = np.ascontiguousarray(self.kernels.astype(np.complex64))
        return self._kernels32

    def grid_dirty_f32(self, u, v, w, weight, vis, threads=1):
        """grid_sample_planned_pair (gridder.rs:3702-3724) on Complex32 grids."""
        n = len(u)
        u, v, w = _c(u, np.float64), _c(v, np.float64), _c(w, np.float64)
        weight, vis = _c(weight, np.float32), _c(vis, np.complex64)
        g = self.gridder
        psf = np.zeros((g.gnx, g.gny), np.complex64)
        dirty = np.zeros((g.gnx, g.gny), np.complex64)
        acc = Accum()
        lib().oc_wproj_grid_dirty_f32(C.byref(self._p), _ptr(self._k32()), n, _ptr(u), _ptr(v),
                                      _ptr(w), _ptr(weight), None, None, _ptr(vis), _ptr(psf),
                                      _ptr(dirty), C.byref(acc), threads)
        return psf, dirty, acc

    def degrid_f32(self, model_grid, u, v, w, threads=1):
        """degrid_sample_planned (gridder.rs:3726-3747) in Complex32."""
        g = _c(model_grid, np.complex64)
        u, v, w = _c(u, np.float64), _c(v, np.float64), _c(w, np.float64)
        pred = np.zeros(len(u), np.complex64)
        lib().oc_wproj_degrid_f32(C.byref(self._p), _ptr(self._k32()), _ptr(g), len(u), _ptr(u),
                                  _ptr(v), _ptr(w), _ptr(pred), threads)
        return pred

    # image-domain stages --------------------------------------------------
    def _sinc(self):
        g = self.gridder
        return sinc_axis(max(g.gnx, g.gny), self.sampling).astype(np.float64)

    def corrected_image(self, raw):
        """corrected_w_project_image_from_grid (gridder.rs:1685-1715)."""
        g = self.gridder
        nx, ny = self.geom.nx, self.geom.ny
        s = self._sinc()
        sub = raw[g.blc_x:g.blc_x + nx, g.blc_y:g.blc_y + ny]
        corr = (g.corr_x[g.blc_x:g.blc_x + nx, None].astype(np.float64)
                * g.corr_y[None, g.blc_y:g.blc_y + ny].astype(np.float64))
        sf = s[g.blc_x:g.blc_x + nx, None] * s[None, g.blc_y:g.blc_y + ny]
        out = np.where(np.abs(sf) > 1e-6, (sub * (corr / np.where(sf == 0, 1, sf))).real, 0.0)
        return out

    def apodize(self, model):
        """apodize_w_project_model (gridder.rs:1572-1592)."""
        g = self.gridder
        nx, ny = self.geom.nx, self.geom.ny
        sx = sinc_axis(g.gnx, self.sampling).astype(np.float64)
        sy = sinc_axis(g.gny, self.sampling).astype(np.float64)
        f = (g.corr_x[g.blc_x:g.blc_x + nx, None].astype(np.float64)
             * g.corr_y[None, g.blc_y:g.blc_y + ny].astype(np.float64)
             * sx[g.blc_x:g.blc_x + nx, None] * sy[None, g.blc_y:g.blc_y + ny])
        out = np.zeros((g.gnx, g.gny), np.complex128)
        out[g.blc_x:g.blc_x + nx, g.blc_y:g.blc_y + ny] = model * f
        return out

    def model_grid(self, model):
        return centered_fft2(self.apodize(model))

    def dirty_products(self, psf_grid, dirty_grid, acc: Accum):
        """compute_dirty_psf_and_residual_w_project_streaming (lib.rs:70539-70590)."""
        if acc.normalization_sumwt <= 0.0:
            raise ValueError("no usable samples")
        psf = 2.0 * self.corrected_image(centered_ifft2(psf_grid)) / acc.normalization_sumwt
        peak = float(np.max(np.abs(psf)))
        psf = psf / peak
        res = 2.0 * self.corrected_image(centered_ifft2(dirty_grid)) / acc.normalization_sumwt
        res = res / peak
        return psf, res, peak


# --------------------------------------------------------------------------
# weighting
# --------------------------------------------------------------------------
def density_cell(geom: Geometry, u: float, v: float, convention: int = 0):
    cx, cy = _i64(), _i64()
    ok = lib().oc_density_cell(geom.nx, geom.ny, geom.cell_x, geom.cell_y, u, v, convention,
                               C.byref(cx), C.byref(cy))
    return (int(cx.value), int(cy.value)) if ok else None


def density_grid(geom: Geometry, u, v, weight, convention: int = 0):
    """build_density_grid_serial (weighting.rs:1729-1854); convention 1 is the
    cube PerPlane rounding (weighting.rs:1470-1483)."""
    u, v, weight = _c(u, np.float64), _c(v, np.float64), _c(weight, np.float32)
    d = np.zeros((geom.nx, geom.ny), np.float32)
    lib().oc_density_grid_conv(geom.nx, geom.ny, geom.cell_x, geom.cell_y, len(u), _ptr(u),
                               _ptr(v), _ptr(weight), convention, _ptr(d))
    return d


def briggs_f2(density, robust: float) -> float:
    d = _c(density, np.float32)
    return float(lib().oc_briggs_f2(_ptr(d), d.size, robust))


def briggs_denominator(density: float, f2: float) -> float:
    return float(lib().oc_briggs_denominator(density, f2))


def apply_weighting(geom: Geometry, u, v, weight, mode: str = "natural", robust: float = 0.0,
                    convention: int = 0, build_u=None, build_v=None):
    """apply_weighting_with_density_source (weighting.rs:1055-1180): Combined
    density (convention 0) or the cube's PerPlane density (convention 1).
    build_u / build_v: the density is built there and looked up at u, v (the
    streaming row path, weighting.rs:646-756 and 333-380)."""
    u, v, weight = _c(u, np.float64), _c(v, np.float64), _c(weight, np.float32)
    if mode == "natural":
        return weight.copy(), None, 0.0
    d = density_grid(geom, u if build_u is None else build_u,
                     v if build_v is None else build_v, weight, convention)
    m = {"uniform": 1, "briggs": 2}[mode]
    f2 = briggs_f2(d, robust) if m == 2 else 0.0
    out = np.zeros_like(weight)
    lib().oc_reweight_conv(geom.nx, geom.ny, geom.cell_x, geom.cell_y, len(u), _ptr(u), _ptr(v),
                           _ptr(weight), _ptr(d), m, f2, convention, _ptr(out))
    return out, d, f2


# --------------------------------------------------------------------------
# Hogbom
# --------------------------------------------------------------------------
def peak_location(image, mask=None):
    img = _c(image, np.float32)
    mk = _c(mask, np.uint8)
    px, py, val = _i64(), _i64(), _f()
    ok = lib().oc_peak_location(_ptr(img), _ptr(mk), img.shape[0], img.shape[1], C.byref(px),
                                C.byref(py), C.byref(val))
    return ((int(px.value), int(py.value)), float(val.value)) if ok else None


def stop_reason(peak_abs, threshold, cycle_threshold, nsigma_threshold) -> int:
    return int(lib().oc_minor_cycle_stop_reason(peak_abs, threshold, cycle_threshold,
                                                nsigma_threshold))


def hogbom(residual, psf, gain, niter, threshold=0.0, cycle_threshold=0.0,
           nsigma_threshold=0.0, mask=None, model=None, inclusive=True):
    """run_hogbom_minor_cycle_cpu_with_progress (lib.rs:59748-59883)."""
    res = np.array(residual, np.float32, copy=True, order="C")
    p = _c(psf, np.float32)
    nx, ny = res.shape
    mdl = np.zeros_like(res) if model is None else np.array(model, np.float32, copy=True)
    mk = _c(mask, np.uint8)
    cap = niter + 1
    cx = np.zeros(cap, np.int32)
    cy = np.zeros(cap, np.int32)
    cp = np.zeros(cap, np.float32)
    cf = np.zeros(cap, np.float32)
    stop = _i32()
    reported = _i64()
    n = lib().oc_hogbom(_ptr(mdl), _ptr(res), _ptr(p), _ptr(mk), nx, ny, gain, threshold,
                        cycle_threshold, nsigma_threshold, niter, int(inclusive), _ptr(cx),
                        _ptr(cy), _ptr(cp), _ptr(cf), C.byref(stop), C.byref(reported))
    return dict(model=mdl, residual=res, x=cx[:n], y=cy[:n], peak=cp[:n], flux=cf[:n],
                stop_reason=int(stop.value), actual=int(n), reported=int(reported.value))


def peak_relative(image, tol, mask=None):
    """finite_peak_location_masked_with_relative_tolerance (lib.rs:73998-74026)."""
    img = _c(image, np.float32)
    mk = _c(mask, np.uint8)
    px, py, val = _i64(), _i64(), _f()
    ok = lib().oc_peak_relative(_ptr(img), _ptr(mk), img.shape[0], img.shape[1], float(tol),
                                C.byref(px), C.byref(py), C.byref(val))
    return ((int(px.value), int(py.value)), float(val.value)) if ok else None


def hogbom_plane(residual, psf, gain, cycle_limit, cycle_threshold, tol, threshold=0.0,
                 mask=None, model=None, inclusive=True):
    """run_hogbom_plane_minor_cycle (lib.rs:64630-64680)."""
    res = np.array(residual, np.float32, copy=True, order="C")
    p = _c(psf, np.float32)
    nx, ny = res.shape
    mdl = np.zeros_like(res) if model is None else np.array(model, np.float32, copy=True)
    mk = _c(mask, np.uint8)
    cap = cycle_limit + 1
    cx = np.zeros(cap, np.int32)
    cy = np.zeros(cap, np.int32)
    cp = np.zeros(cap, np.float32)
    cf = np.zeros(cap, np.float32)
    reported = _i64()
    n = lib().oc_hogbom_plane(_ptr(mdl), _ptr(res), _ptr(p), _ptr(mk), nx, ny, gain, threshold,
                              cycle_threshold, float(tol), cycle_limit, int(inclusive), _ptr(cx),
                              _ptr(cy), _ptr(cp), _ptr(cf), C.byref(reported))
    return dict(model=mdl, residual=res, x=cx[:n], y=cy[:n], peak=cp[:n], flux=cf[:n],
                actual=int(n), reported=int(reported.value))


# --------------------------------------------------------------------------
# robust RMS and the n-sigma threshold
# --------------------------------------------------------------------------
def mean_stddev(values):
    """mean_stddev (lib.rs:74560-74576): sequential FP64 sums, sample variance."""
    v = _c(values, np.float32)
    m, s = _d(), _d()
    lib().oc_mean_stddev(_ptr(v), len(v), C.byref(m), C.byref(s))
    return float(m.value), float(s.value)


def chauvenet_max_zscore(npts: int) -> float:
    """chauvenet_max_zscore (lib.rs:74578-74622)."""
    return float(lib().oc_chauvenet_max_zscore(int(npts)))


def chauvenet_clip(values, zscore: float, max_iterations: int) -> np.ndarray:
    """apply_chauvenet_clipping (lib.rs:74512-74558): the kept values, in order."""
    v = np.array(values, np.float32, copy=True)
    n = lib().oc_chauvenet_clip(_ptr(v), len(v), float(zscore), int(max_iterations))
    return v[:n]


def madfm(values):
    """casacore madfm (casa-lattices statistics.rs:1367-1379): (median, madfm)."""
    v = _c(values, np.float32)
    med = _d()
    mad = lib().oc_madfm(_ptr(v), len(v), C.byref(med))
    return float(med.value), float(mad)


def robust_rms(residual, mask=None):
    """robust_rms_jy_per_beam (lib.rs:74130-74183): returns (rms float32,
    madfm FP64, number of values it was taken over)."""
    r = _c(residual, np.float32).reshape(-1)
    mk = None if mask is None else _c(np.asarray(mask, np.uint8), np.uint8).reshape(-1)
    mad, cnt = _d(), _i64()
    rms = lib().oc_robust_rms(_ptr(r), _ptr(mk), len(r), C.byref(mad), C.byref(cnt))
    return float(np.float32(rms)), float(mad.value), int(cnt.value)


def nsigma_threshold(residual, nsigma: float, mask=None) -> float:
    """nsigma_threshold_jy_per_beam (lib.rs:74474-74484), float32."""
    if not nsigma > 0.0:
        return 0.0
    return float(np.float32(nsigma) * np.float32(robust_rms(residual, mask)[0]))


def radians_from_arcsec(a: float) -> float:
    return a / 3600.0 * math.pi / 180.0


# --------------------------------------------------------------------------
# Cotton-Schwab major/minor controller
# --------------------------------------------------------------------------
def threshold_reached_with_tolerance(peak_abs: float, threshold: float) -> bool:
    """threshold_reached_with_tolerance (lib.rs:74628-74635), float32."""
    f32 = np.float32
    p, t = f32(peak_abs), f32(threshold)
    if t <= 0:
        return bool(p <= t)
    tol = max(f32(0.01) * t, f32(2.0e-8))
    return bool(p <= t or abs(p - t) <= tol)


def tolerant_clean_stop_reason(peak_abs, threshold, nsigma_threshold):
    """tolerant_clean_stop_reason (lib.rs:74637-74651)."""
    if threshold_reached_with_tolerance(peak_abs, threshold):
        return "GlobalThresholdReached"
    if nsigma_threshold > threshold and threshold_reached_with_tolerance(peak_abs,
                                                                         nsigma_threshold):
        return "NsigmaThresholdReached"
    return None


def clean_cycle_threshold(peak, sidelobe, cyclefactor, min_frac, max_frac, threshold) -> float:
    """clean_cycle_threshold (lib.rs:74120-74127), float32."""
    f32 = np.float32
    frac = min(max(f32(sidelobe) * f32(cyclefactor), f32(min_frac)), f32(max_frac))
    return float(max(f32(peak) * f32(frac), f32(threshold)))


_STOP_NAMES = {0: None, 1: "GlobalThresholdReached", 2: "CycleThresholdReached",
               3: "NsigmaThresholdReached", 4: "NoCleanablePixels"}


def cotton_schwab(residual, psf, refresh, niter, gain=0.1, threshold=0.0, minor_cycle_length=2000,
                  cyclefactor=1.0, min_psf_fraction=0.05, max_psf_fraction=0.8,
                  major_cycle_limit=None, sidelobe=0.0, inclusive=True, model=None,
                  cycle_threshold_override=None, nsigma=0.0):
    """run_hogbom_cotton_schwab (lib.rs:59354-59636) without mask; `nsigma`
    > 0 adds the robust-RMS threshold nsigma_threshold_jy_per_beam at each
    cycle start and after each refresh (lib.rs:59395-59396, 59563-59564).
    `refresh(model) -> residual` is the measured major cycle.
    `model` continues from an earlier model; `cycle_threshold_override`
    replaces the per-cycle threshold (the cube-wide threshold of
    run_standard_mfs_cube_clean).  Returns a dict with model, residual,
    major cycles, iterations, the stop reason, the per-cycle thresholds and
    the component list."""
    f32 = np.float32
    res = np.array(residual, np.float32, copy=True)
    model = np.zeros_like(res) if model is None else np.array(model, np.float32, copy=True)
    actual = reported = major = 0
    stop = None
    min_peak = f32(np.max(np.abs(res)))
    needs_refresh = False
    comps, thresholds, nsig_thresholds = [], [], []
    while reported < niter:
        if major_cycle_limit is not None and major >= major_cycle_limit:
            stop = "MajorCycleLimitReached"
            break
        pk = peak_location(res)
        if pk is None:
            stop = "NoCleanablePixels"
            break
        peak = abs(pk[1])
        nsig = nsigma_threshold(res, nsigma)
        nsig_thresholds.append(nsig)
        s = tolerant_clean_stop_reason(peak, threshold, nsig)
        if s is not None:
            stop = s
            break
        cyc_niter = min(niter - reported, minor_cycle_length)
        thr = clean_cycle_threshold(peak, sidelobe, cyclefactor, min_psf_fraction,
                                    max_psf_fraction, threshold)
        if cycle_threshold_override is not None:
            thr = float(cycle_threshold_override)
        thresholds.append(thr)
        out = hogbom(res, psf, gain, cyc_niter, threshold=threshold, cycle_threshold=thr,
                     nsigma_threshold=nsig, model=model, inclusive=inclusive)
        model, res = out["model"], out["residual"]
        comps.extend(zip(zip(out["x"].tolist(), out["y"].tolist()), out["flux"].tolist()))
        actual += out["actual"]
        reported += out["reported"]
        reason = _STOP_NAMES[out["stop_reason"]]
        updated = out["actual"] > 0
        stop_after = None
        if reason is not None:
            if updated and reason in ("CycleThresholdReached", "NsigmaThresholdReached"):
                pass
            elif reason in ("CycleThresholdReached", "NsigmaThresholdReached"):
                stop = reason
            else:
                stop = reason
                stop_after = reason
        if not updated:
            break
        needs_refresh = True
        minor_peak = f32(np.max(np.abs(res)))
        if minor_peak < min_peak:
            min_peak = minor_peak
        elif min_peak > 0 and (minor_peak - min_peak) / min_peak > f32(0.1):
            stop = "DivergenceDetected"
            break
        if reported >= niter:
            stop = "IterationLimitReached"
            break
        res = np.asarray(refresh(model), np.float32)
        major += 1
        needs_refresh = False
        nsig = nsigma_threshold(res, nsigma)
        if stop_after is not None:
            break
        s = tolerant_clean_stop_reason(f32(np.max(np.abs(res))), threshold, nsig)
        if s is not None:
            stop = s
            break
    if niter > 0 and stop is None:
        stop = "IterationLimitReached"
    if needs_refresh:
        res = np.asarray(refresh(model), np.float32)
    return dict(model=model, residual=res, major_cycles=major, actual=actual, reported=reported,
                stop_reason=stop, thresholds=thresholds, components=comps,
                nsigma_thresholds=nsig_thresholds)


def cube_clean(planes, niter, gain=0.1, threshold=0.0, minor_cycle_length=2000, cyclefactor=1.0,
               min_psf_fraction=0.05, max_psf_fraction=0.8, major_cycle_limit=None,
               inclusive=True, nsigma=0.0):
    """run_standard_mfs_cube_clean (casa-imaging lib.rs:3026-3210) over
    planes in ascending order.  Each plane is a dict with residual, psf,
    refresh(model) -> residual and sidelobe (its PSF sidelobe level).  Per
    synchronized pass every active plane (residual peak above the cube-wide
    cycle threshold) runs one major cycle of its own controller
    (run_standard_mfs_prepared_clean_plane_one_major_cycle, lib.rs:46465-46520:
    niter = the remaining global budget, one major cycle, the cube threshold
    as override).  Then the plane results of
    complete_standard_mfs_prepared_clean_plane (lib.rs:46343-46460)."""
    f32 = np.float32
    n = len(planes)
    res = [np.array(p["residual"], np.float32, copy=True) for p in planes]
    model = [np.zeros_like(r) for r in res]
    absmax = lambda a: f32(np.max(np.abs(a))) if a.size else f32(0)
    finite_max = lambda vals: max([f32(v) for v in vals if np.isfinite(v)] + [f32(0)])
    cyc = lambda peak, sl: clean_cycle_threshold(peak, sl, cyclefactor, min_psf_fraction,
                                                 max_psf_fraction, threshold)
    initial_peak = finite_max([absmax(r) for r in res])
    max_sidelobe = finite_max([p["sidelobe"] for p in planes])
    first_thr = cyc(initial_peak, max_sidelobe)
    at_or_below = sum(1 for r in res if absmax(r) <= f32(first_thr))
    plane_iters = [0] * n
    plane_stop = [None] * n
    comps = [[] for _ in range(n)]
    completed = major = 0
    thresholds, actives = [], []
    while True:
        peak = finite_max([absmax(r) for r in res])
        thr = cyc(peak, max_sidelobe)
        t = f32(threshold)
        reached = peak <= t or (t > 0 and abs(peak - t) / t < f32(0.01))
        if reached or completed >= niter:
            break
        if major_cycle_limit is not None and major >= major_cycle_limit:
            break
        active = [i for i in range(n) if absmax(res[i]) > f32(thr)]
        if not active:
            break
        major += 1
        cycle_niter = niter - completed
        thresholds.append(thr)
        actives.append(active)
        pass_iters = 0
        for i in active:
            out = cotton_schwab(res[i], planes[i]["psf"], planes[i]["refresh"], cycle_niter,
                                gain=gain, threshold=threshold,
                                minor_cycle_length=minor_cycle_length, cyclefactor=cyclefactor,
                                min_psf_fraction=min_psf_fraction,
                                max_psf_fraction=max_psf_fraction, major_cycle_limit=1,
                                sidelobe=max_sidelobe, inclusive=inclusive, model=model[i],
                                cycle_threshold_override=thr, nsigma=nsigma)
            model[i], res[i] = out["model"], out["residual"]
            comps[i].extend(out["components"])
            plane_iters[i] += out["reported"]
            plane_stop[i] = out["stop_reason"]
            pass_iters += out["reported"]
        completed += pass_iters
        if pass_iters == 0:
            break
    final_thr = cyc(finite_max([absmax(r) for r in res]), max_sidelobe)
    stops = []
    for i in range(n):
        if plane_iters[i] >= niter:
            stops.append("IterationLimitReached")
            continue
        s = tolerant_clean_stop_reason(absmax(res[i]), threshold,
                                       nsigma_threshold(res[i], nsigma))
        if s is None:
            s = plane_stop[i]
            if s in (None, "MajorCycleLimitReached"):
                s = "CycleThresholdReached"
        stops.append(s)
    return dict(models=model, residuals=res, plane_iterations=plane_iters, plane_stops=stops,
                components=comps, minor_iterations=completed, major_cycles=major,
                thresholds=thresholds, active=actives, initial_peak=float(initial_peak),
                max_sidelobe=float(max_sidelobe), final_cycle_threshold=final_thr,
                planes_at_or_below_initial_threshold=at_or_below)
