"""Host-side mirror of the deconvolution side of the reference's serial major cycle.

Names and argument meaning follow Distributed-Reconstruction: Core/Deconvolution/FastSerialCD.cs
(the IDeconvolver of the serial major cycle), Core/PaddedConvolver.cs, the PSF helpers of
Core/Common.cs, and SingleReconstruction/MajorCycle.cs:33-134 (ReconstructSerialCD).  Images are
numpy float32[n, n]; the coordinate descent, the PSF^2 and Lipschitz maps and the FFT
correlations run on the GPU through the C ABI.  PSF.Cut, CalcMaxSidelobe and CalcMaxLipschitz
are the reference's own small host loops (slicing and one reduction) and stay on the host.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import _native as nat
from .idg import GriddingConstants, P9IDGError, _check, _check_inputs, _plan_for, _ptr

MAJOR_EPSILON = 1e-4  # MajorCycle.cs:18 (1e-4f)


class Rectangle:
    """Common.Rectangle (Common.cs:373-399)."""

    def __init__(self, y, x, yEnd, xEnd):
        self.Y, self.X, self.YEnd, self.XEnd = int(y), int(x), int(yEnd), int(xEnd)

    def YExtent(self):
        return self.YEnd - self.Y

    def XExtent(self):
        return self.XEnd - self.X


@dataclasses.dataclass
class DeconvolutionResult:
    """IDeconvolver.cs:9-21 (elapsed time in milliseconds)."""
    Converged: bool
    IterationCount: int
    ElapsedMs: float


class _CdResult(ctypes.Structure):
    _fields_ = [("converged", ctypes.c_int32), ("iterations", ctypes.c_int32), ("elapsed_ms", ctypes.c_double)]


class McParams(ctypes.Structure):
    _fields_ = [("psf_cut_factor", ctypes.c_int32), ("max_major_cycles", ctypes.c_int32),
                ("deconv_iterations", ctypes.c_int32), ("reserved", ctypes.c_int32), ("lambda_", ctypes.c_float),
                ("alpha", ctypes.c_float), ("deconv_epsilon", ctypes.c_float), ("major_epsilon", ctypes.c_float)]


class McCycle(ctypes.Structure):
    _fields_ = [("max_dirty", ctypes.c_float), ("max_b", ctypes.c_float), ("current_lambda", ctypes.c_float),
                ("abs_max", ctypes.c_float), ("deconvolved", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("iterations", ctypes.c_int32), ("reserved", ctypes.c_int32), ("grid_ms", ctypes.c_double),
                ("image_ms", ctypes.c_double), ("deconv_ms", ctypes.c_double), ("degrid_ms", ctypes.c_double),
                ("objective", ctypes.c_double)]


def _f32(a, writable=False):
    a = np.asarray(a)
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        if writable:
            raise TypeError("in-place arrays must be C-contiguous float32")
        a = np.ascontiguousarray(a, np.float32)
    return a


def _square(psf):
    psf = _f32(psf)
    if psf.ndim != 2 or psf.shape[0] != psf.shape[1]:
        raise ValueError("the PSF must be a square 2-D array (FFT.Shift uses the row count)")
    return psf


class FastSerialCD:
    """FastSerialCD(totalSize, psf) (FastSerialCD.cs:31-46) on the GPU."""

    def __init__(self, totalSize: Rectangle, psf):
        if totalSize.YExtent() != totalSize.XExtent() or totalSize.Y or totalSize.X:
            raise ValueError("total size must be a square image at (0, 0)")
        psf = _square(psf)
        self.n = totalSize.YExtent()
        self._h = ctypes.c_void_p()
        _check(nat.lib().p9idg_cd_create(self.n, _ptr(psf), psf.shape[0], psf.shape[1], ctypes.byref(self._h)))

    @property
    def MaxLipschitz(self) -> float:
        v = ctypes.c_float()
        _check(nat.lib().p9idg_cd_max_lipschitz(self._h, ctypes.byref(v)))
        return v.value

    def maps(self):
        """(PSF^2, Lipschitz map) as the deconvolver holds them."""
        h, w = ctypes.c_int32(), ctypes.c_int32()
        _check(nat.lib().p9idg_cd_psf2_size(self._h, ctypes.byref(h), ctypes.byref(w)))
        psf2 = np.zeros((h.value, w.value), np.float32)
        amap = np.zeros((self.n, self.n), np.float32)
        _check(nat.lib().p9idg_cd_get_maps(self._h, _ptr(psf2), _ptr(amap)))
        return psf2, amap

    def _images(self, x, g, writable):
        x, g = _f32(x, writable), _f32(g, writable)
        for a, name in ((x, "xImage"), (g, "bMap")):
            if a.shape != (self.n, self.n):
                raise ValueError(f"{name} has shape {a.shape}; the deconvolver's image is {(self.n, self.n)}")
        return x, g

    def Deconvolve(self, xImage, bMap, lambda_, alpha, maxIteration, epsilon=1e-4) -> DeconvolutionResult:
        """Updates xImage and bMap (float32, C-contiguous) in place, as the reference does."""
        x, g = self._images(xImage, bMap, True)
        r = _CdResult()
        _check(nat.lib().p9idg_cd_deconvolve(self._h, _ptr(x), _ptr(g), float(lambda_), float(alpha), int(maxIteration),
                                             float(epsilon), ctypes.byref(r)))
        return DeconvolutionResult(bool(r.converged), r.iterations, r.elapsed_ms)

    def deconvolve_device(self, d_x: int, d_bmap: int, lambda_, alpha, maxIteration, epsilon=1e-4):
        r = _CdResult()
        _check(nat.lib().p9idg_cd_deconvolve_device(self._h, ctypes.c_void_p(d_x), ctypes.c_void_p(d_bmap),
                                                    float(lambda_), float(alpha), int(maxIteration), float(epsilon),
                                                    ctypes.byref(r)))
        return DeconvolutionResult(bool(r.converged), r.iterations, r.elapsed_ms)

    def DeconvolvePath(self, xImage, bMap, lambdaMin, lambdaFactor, alpha, maxPathIteration=10, maxIteration=100,
                       epsilon=1e-4) -> DeconvolutionResult:
        x, g = self._images(xImage, bMap, True)
        r = _CdResult()
        _check(nat.lib().p9idg_cd_deconvolve_path(self._h, _ptr(x), _ptr(g), float(lambdaMin), float(lambdaFactor),
                                                  float(alpha), int(maxPathIteration), int(maxIteration),
                                                  float(epsilon), ctypes.byref(r)))
        return DeconvolutionResult(bool(r.converged), r.iterations, r.elapsed_ms)

    def GetAbsMaxDiff(self, xImage, gradients, lambda_, alpha) -> float:
        x, g = self._images(xImage, gradients, False)
        v = ctypes.c_float()
        _check(nat.lib().p9idg_cd_get_abs_max_diff(self._h, _ptr(x), _ptr(g), float(lambda_), float(alpha),
                                                   ctypes.byref(v)))
        return v.value

    def ResetLipschitzMap(self, psf):
        psf = _square(psf)
        _check(nat.lib().p9idg_cd_reset_lipschitz_map(self._h, _ptr(psf), psf.shape[0], psf.shape[1]))

    def destroy(self):
        if getattr(self, "_h", None) and self._h.value:
            nat.lib().p9idg_cd_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class PaddedConvolver:
    """PaddedConvolver(Complex[,] kernel, Rectangle kernelSize) (PaddedConvolver.cs:36-41) on the GPU."""

    def __init__(self, kernel, kernelSize: Rectangle):
        k = np.ascontiguousarray(kernel, np.complex128)
        self._h = ctypes.c_void_p()
        _check(nat.lib().p9idg_convolver_create(_ptr(k), k.shape[0], k.shape[1], kernelSize.YExtent(),
                                                kernelSize.XExtent(), ctypes.byref(self._h)))

    @classmethod
    def correlation(cls, psf, totalSize: Rectangle) -> "PaddedConvolver":
        """= PaddedConvolver(PSF.CalcPaddedFourierCorrelation(psf, totalSize), psf rectangle), built on the GPU."""
        psf = _square(psf)
        self = cls.__new__(cls)
        self._h = ctypes.c_void_p()
        _check(nat.lib().p9idg_convolver_create_correlation(_ptr(psf), psf.shape[0], psf.shape[1], totalSize.YEnd,
                                                            ctypes.byref(self._h)))
        return self

    def Convolve(self, image) -> np.ndarray:
        img = _f32(image)
        out = np.zeros_like(img)
        _check(nat.lib().p9idg_convolver_convolve(self._h, _ptr(img), img.shape[0], _ptr(out)))
        return out

    def convolve_device(self, d_image: int, n: int, d_out: int):
        _check(nat.lib().p9idg_convolver_convolve_device(self._h, ctypes.c_void_p(d_image), int(n),
                                                         ctypes.c_void_p(d_out)))

    def destroy(self):
        if getattr(self, "_h", None) and self._h.value:
            nat.lib().p9idg_convolver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class PSF:
    """Common.PSF (Common.cs:44-227)."""

    @staticmethod
    def CalcPaddedFourierCorrelation(psf, padding: Rectangle) -> np.ndarray:
        psf = _f32(psf)
        out = np.zeros((padding.YEnd + psf.shape[0], padding.XEnd + psf.shape[1]), np.complex128)
        _check(nat.lib().p9idg_psf_padded_fourier_correlation(_ptr(psf), psf.shape[0], psf.shape[1], padding.YEnd,
                                                              padding.XEnd, _ptr(out)))
        return out

    @staticmethod
    def CalcPSFSquared(psf) -> np.ndarray:
        psf = _square(psf)
        out = np.zeros((2 * psf.shape[0], 2 * psf.shape[1]), np.float32)
        _check(nat.lib().p9idg_psf_squared(_ptr(psf), psf.shape[0], psf.shape[1], _ptr(out)))
        return out

    @staticmethod
    def CalcAMap(psf, totalSize: Rectangle) -> np.ndarray:
        psf = _f32(psf)
        out = np.zeros((totalSize.YEnd, totalSize.XEnd), np.float32)
        _check(nat.lib().p9idg_psf_amap(_ptr(psf), psf.shape[0], psf.shape[1], totalSize.YEnd, totalSize.XEnd,
                                        _ptr(out)))
        return out

    @staticmethod
    def Cut(psf, factor=2) -> np.ndarray:
        psf = _square(psf)
        m = psf.shape[0] // factor
        off = psf.shape[0] // 2 - m // 2
        return psf[off:off + m, off:off + m].copy()

    @staticmethod
    def CalcMaxSidelobe(fullPsf, cutFactor=2) -> float:
        psf = _square(fullPsf)
        n = psf.shape[0]
        m = n // cutFactor
        off = n // 2 - m // 2
        a = np.abs(psf)
        a[off:off + m, off:off + m] = 0.0
        return float(max(0.0, a.max()))

    @staticmethod
    def CalcMaxLipschitz(psf) -> float:
        p = _f32(psf)
        return float(np.sum((p * p).astype(np.float64)))


class MajorCycle:
    """SingleReconstruction/MajorCycle.cs."""

    @staticmethod
    def _params(psfCutFactor, maxMajorCycle, lambda_, alpha, deconvIterations, deconvEpsilon):
        return McParams(int(psfCutFactor), int(maxMajorCycle), int(deconvIterations), 0, float(lambda_),
                        float(alpha), float(deconvEpsilon), np.float32(MAJOR_EPSILON))

    @staticmethod
    def _cycles(arr, n):
        return [{k: getattr(arr[i], k) for k, _ in McCycle._fields_ if k != "reserved"} for i in range(n)]

    @staticmethod
    def ReconstructSerialCD(c: GriddingConstants, metadata, visibilities, uvw, frequencies, flags, psfCutFactor,
                            maxMajorCycle, lambda_, alpha, deconvIterations, deconvEpsilon) -> dict:
        """MajorCycle.ReconstructSerialCD (MajorCycle.cs:33-134) without the FITS writes: returns
        dict(model=xImage, residual=last dirty image, psf=PSF, cycles=[per-cycle record])."""
        plan = _plan_for(c, metadata, uvw, frequencies)
        vis = np.ascontiguousarray(visibilities, np.complex128)
        fl = np.ascontiguousarray(flags, np.uint8)
        _check_inputs(plan, c, vis=vis, uvw=uvw, flags=fl)
        N = c.GridSize
        model = np.zeros((N, N), np.float32)
        resid = np.zeros((N, N), np.float32)
        psf = np.zeros((N, N), np.float32)
        cyc = (McCycle * max(1, int(maxMajorCycle)))()
        n = ctypes.c_int32()
        p = MajorCycle._params(psfCutFactor, maxMajorCycle, lambda_, alpha, deconvIterations, deconvEpsilon)
        _check(nat.lib().p9idg_major_cycle_serial_cd(plan.handle, ctypes.byref(p), _ptr(vis), _ptr(fl), _ptr(model),
                                                     _ptr(resid), _ptr(psf), cyc, ctypes.byref(n)))
        return dict(model=model, residual=resid, psf=psf, cycles=MajorCycle._cycles(cyc, n.value))

    @staticmethod
    def reconstruct_serial_cd_device(plan, d_vis: int, d_flags: int, d_model: int, d_residual: int, d_psf: int,
                                     psfCutFactor, maxMajorCycle, lambda_, alpha, deconvIterations,
                                     deconvEpsilon) -> list:
        """The same loop on device buffers (complex64 visibilities, uint8 flags, float32 images)."""
        cyc = (McCycle * max(1, int(maxMajorCycle)))()
        n = ctypes.c_int32()
        p = MajorCycle._params(psfCutFactor, maxMajorCycle, lambda_, alpha, deconvIterations, deconvEpsilon)
        _check(nat.lib().p9idg_major_cycle_serial_cd_device(
            plan.handle, ctypes.byref(p), ctypes.c_void_p(d_vis), ctypes.c_void_p(d_flags), ctypes.c_void_p(d_model),
            ctypes.c_void_p(d_residual), ctypes.c_void_p(d_psf) if d_psf else None, cyc, ctypes.byref(n)))
        return MajorCycle._cycles(cyc, n.value)


__all__ = ["FastSerialCD", "PaddedConvolver", "PSF", "MajorCycle", "Rectangle", "DeconvolutionResult",
           "MAJOR_EPSILON", "P9IDGError"]
