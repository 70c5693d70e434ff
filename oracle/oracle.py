"""ctypes bindings for the FP64 CPU oracle (oracle/idg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, the smoke check and the
CPU-baseline leg of the benchmark, as the checker.  The product never imports
this module.  Parity is unpinned against the reference itself (the C#
reference cannot run here and ships no golden vectors); see idg_oracle.c.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libidg_oracle.so")

OK, INVALID_ARGUMENT, CANNOT_PLACE, SUBGRID_OUT_OF_GRID, INVALID_GRID, OUT_OF_MEMORY = range(6)

SUBGRID_DTYPE = np.dtype([("baseline_idx", "<i4"), ("time_sample_start", "<i4"), ("time_sample_count", "<i4"),
                          ("u_pixel", "<i4"), ("v_pixel", "<i4"), ("w_lambda", "<i4")])


class OracleError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what}: oracle status {code}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("vis_count", ctypes.c_int64), ("grid_size", ctypes.c_int32), ("subgrid_size", ctypes.c_int32),
                ("kernel_size", ctypes.c_int32), ("max_timesteps", ctypes.c_int32), ("scale_arcsec", ctypes.c_float),
                ("wlayer_count", ctypes.c_int32), ("wstep", ctypes.c_double)]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i32, i64 = ctypes.c_int32, ctypes.c_int64
        L.oc_partition.argtypes = [P, P, i32, i32, P, i32, ctypes.POINTER(P), ctypes.POINTER(i64)]
        L.oc_free.argtypes = [P]
        L.oc_fft1d.argtypes = [P, i64, P, ctypes.c_int, ctypes.c_int]
        L.oc_fft2d.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oc_gridder_forward.argtypes = [P, P, i64, P, i32, P, P, i32, P, P]
        L.oc_gridder_backward.argtypes = [P, P, i64, P, P, i32, P, i32, P, P]
        L.oc_subgrid_fft_forward.argtypes = [P, i64, P]
        L.oc_subgrid_fft_backward.argtypes = [P, i64, P]
        L.oc_adder_add.argtypes = [P, P, i64, P, P]
        L.oc_adder_split.argtypes = [P, P, i64, P, P]
        L.oc_adder_wstack_add.argtypes = [P, P, i64, P, P]
        L.oc_adder_wstack_split.argtypes = [P, P, i64, P, P]
        L.oc_shift_complex.argtypes = [P, ctypes.c_int]
        L.oc_shift_double.argtypes = [P, ctypes.c_int]
        L.oc_shift_float.argtypes = [P, ctypes.c_int]
        L.oc_wstack_ifft_float.argtypes = [P, ctypes.c_int, ctypes.c_int, i64, P]
        L.oc_fft_backward_real.argtypes = [P, ctypes.c_int, i64, P]
        L.oc_fft_forward_float.argtypes = [P, ctypes.c_int, ctypes.c_double, P]
        L.oc_idg_grid.argtypes = [P, P, i64, P, P, i32, P, i32, P]
        L.oc_idg_grid_w.argtypes = [P, P, i64, P, P, i32, P, i32, P]
        L.oc_idg_degrid.argtypes = [P, P, i64, P, P, i32, i32, P, i32, P]
        L.oc_idg_degrid_w.argtypes = [P, P, i64, P, P, i32, i32, P, i32, P]
        L.oc_unit_vis.argtypes = [P, i64, P]
        L.oc_vis_subtract.argtypes = [P, P, P, i64, P]
        L.oc_num_threads.restype = ctypes.c_int
        L.oc_set_num_threads.argtypes = [ctypes.c_int]
        f32, f64 = ctypes.c_float, ctypes.c_double
        L.ocd_elastic_net_penalty.argtypes = [P, i32, i32, f32, f32]
        L.ocd_elastic_net_penalty.restype = f64
        L.ocd_get_max.argtypes = [P, i64]
        L.ocd_get_max.restype = f32
        L.ocd_residual_penalty.argtypes = [P, i64]
        L.ocd_residual_penalty.restype = f64
        L.ocd_max_lipschitz.argtypes = [P, i32, i32]
        L.ocd_max_lipschitz.restype = f64
        L.ocd_psf_cut.argtypes = [P, i32, i32, P]
        L.ocd_max_sidelobe.argtypes = [P, i32, i32]
        L.ocd_max_sidelobe.restype = f32
        L.ocd_amap_scan.argtypes = [P, i32, i32, P]
        L.ocd_amap.argtypes = [P, i32, i32, i32, i32, i32, i32, i32, i32, P]
        L.ocd_padded_fourier_correlation.argtypes = [P, i32, i32, i32, i32, P]
        L.ocd_padded_convolve.argtypes = [P, i32, i32, i32, i32, P, i32, P]
        L.ocd_psf_squared.argtypes = [P, i32, i32, P]
        L.ocd_get_abs_max_diff.argtypes = [P, P, P, i32, f32, f32]
        L.ocd_get_abs_max_diff.restype = f32
        L.ocd_get_abs_max_pixel.argtypes = [P, P, P, i32, f32, f32, P, P]
        L.ocd_get_abs_max_pixel.restype = f32
        L.ocd_deconvolve.argtypes = [P, P, P, i32, P, i32, i32, f32, f32, i32, f32, P, P]
        L.ocd_major_cycle.argtypes = [P, P, i64, P, i32, i32, P, i32, P, P, i32, i32, f32, f32, i32, f32,
                                      P, P, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def params(consts: dict) -> Params:
    return Params(int(consts["vis_count"]), int(consts["grid_size"]), int(consts["subgrid_size"]),
                  int(consts["kernel_size"]), int(consts["max_timesteps"]), float(consts["scale_arcsec"]),
                  int(consts["wlayer_count"]), float(consts["wstep"]))


def _check(code, what):
    if code != OK:
        raise OracleError(code, what)


def partition(consts, uvw, freq):
    """Partitioner.CreatePartition -> structured array in reference order."""
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    pr = params(consts)
    out = ctypes.c_void_p()
    n = ctypes.c_int64()
    _check(lib().oc_partition(ctypes.byref(pr), _p(uvw), uvw.shape[0], uvw.shape[1], _p(freq), len(freq),
                              ctypes.byref(out), ctypes.byref(n)), "partition")
    res = np.zeros(n.value, SUBGRID_DTYPE)
    if n.value:
        ctypes.memmove(res.ctypes.data, out, n.value * SUBGRID_DTYPE.itemsize)
    lib().oc_free(out)
    return res


def fft1d(x, sign):
    x = _c128(x)
    out = np.empty_like(x)
    lib().oc_fft1d(_p(x), 1, _p(out), len(x), sign)
    return out


def fft2d(x, sign):
    x = _c128(x).copy()
    lib().oc_fft2d(_p(x), x.shape[0], x.shape[1], sign)
    return x


def gridder_forward(consts, subs, uvw, vis, freq, taper=None):
    S = consts["subgrid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    vis = _c128(vis)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    out = np.zeros((len(subs), S, S), np.complex128)
    tp = None if taper is None else np.ascontiguousarray(taper, np.float32)
    pr = params(consts)
    lib().oc_gridder_forward(ctypes.byref(pr), _p(subs), len(subs), _p(uvw), uvw.shape[1], _p(vis), _p(freq),
                             len(freq), _p(tp), _p(out))
    return out


def gridder_backward(consts, subs, data, uvw, freq, nbl=None, taper=None, vis_out=None):
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    data = _c128(data)
    uvw = np.ascontiguousarray(uvw, np.float64)
    freq = np.ascontiguousarray(freq, np.float64)
    if vis_out is None:
        vis_out = np.zeros((uvw.shape[0], uvw.shape[1], len(freq)), np.complex128)
    tp = None if taper is None else np.ascontiguousarray(taper, np.float32)
    pr = params(consts)
    lib().oc_gridder_backward(ctypes.byref(pr), _p(subs), len(subs), _p(data), _p(uvw), uvw.shape[1], _p(freq),
                              len(freq), _p(tp), _p(vis_out))
    return vis_out


def subgrid_fft_forward(consts, data):
    d = _c128(data).copy()
    pr = params(consts)
    lib().oc_subgrid_fft_forward(ctypes.byref(pr), d.shape[0], _p(d))
    return d


def subgrid_fft_backward(consts, data):
    d = _c128(data).copy()
    pr = params(consts)
    lib().oc_subgrid_fft_backward(ctypes.byref(pr), d.shape[0], _p(d))
    return d


def adder_add(consts, subs, data):
    N = consts["grid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    data = _c128(data)
    g = np.zeros((N, N), np.complex128)
    pr = params(consts)
    _check(lib().oc_adder_add(ctypes.byref(pr), _p(subs), len(subs), _p(data), _p(g)), "Adder.Add")
    return g


def adder_split(consts, subs, grid):
    S = consts["subgrid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    grid = _c128(grid)
    out = np.zeros((len(subs), S, S), np.complex128)
    pr = params(consts)
    lib().oc_adder_split(ctypes.byref(pr), _p(subs), len(subs), _p(grid), _p(out))
    return out


def adder_wstack_add(consts, subs, data):
    N, W = consts["grid_size"], consts["wlayer_count"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    data = _c128(data)
    g = np.zeros((W, N, N), np.complex128)
    pr = params(consts)
    _check(lib().oc_adder_wstack_add(ctypes.byref(pr), _p(subs), len(subs), _p(data), _p(g)), "AdderWStack.Add")
    return g


def adder_wstack_split(consts, subs, grid):
    S = consts["subgrid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    grid = _c128(grid)
    out = np.zeros((len(subs), S, S), np.complex128)
    pr = params(consts)
    lib().oc_adder_wstack_split(ctypes.byref(pr), _p(subs), len(subs), _p(grid), _p(out))
    return out


def shift(a):
    """FFT.Shift on a copy (complex, float64 or float32 square array)."""
    a = np.ascontiguousarray(a).copy()
    if a.dtype == np.complex128:
        lib().oc_shift_complex(_p(a), a.shape[0])
    elif a.dtype == np.float64:
        lib().oc_shift_double(_p(a), a.shape[0])
    elif a.dtype == np.float32:
        lib().oc_shift_float(_p(a), a.shape[0])
    else:
        raise TypeError(a.dtype)
    return a


def wstack_ifft_float(layers, vis_count):
    layers = _c128(layers)
    W, N, _ = layers.shape
    out = np.zeros((N, N), np.float32)
    lib().oc_wstack_ifft_float(_p(layers), W, N, int(vis_count), _p(out))
    return out


def fft_backward_real(grid, vis_count):
    grid = _c128(grid)
    N = grid.shape[0]
    out = np.zeros((N, N), np.float64)
    lib().oc_fft_backward_real(_p(grid), N, int(vis_count), _p(out))
    return out


def fft_forward_float(img, norm=1.0):
    img = np.ascontiguousarray(img, np.float32)
    N = img.shape[0]
    out = np.zeros((N, N), np.complex128)
    lib().oc_fft_forward_float(_p(img), N, float(norm), _p(out))
    return out


def idg_grid(consts, subs, vis, uvw, freq):
    N = consts["grid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    vis, uvw, freq = _c128(vis), np.ascontiguousarray(uvw, np.float64), np.ascontiguousarray(freq, np.float64)
    g = np.zeros((N, N), np.complex128)
    pr = params(consts)
    _check(lib().oc_idg_grid(ctypes.byref(pr), _p(subs), len(subs), _p(vis), _p(uvw), uvw.shape[1], _p(freq),
                             len(freq), _p(g)), "IDG.Grid")
    return g


def idg_grid_w(consts, subs, vis, uvw, freq):
    N, W = consts["grid_size"], consts["wlayer_count"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    vis, uvw, freq = _c128(vis), np.ascontiguousarray(uvw, np.float64), np.ascontiguousarray(freq, np.float64)
    g = np.zeros((W, N, N), np.complex128)
    pr = params(consts)
    _check(lib().oc_idg_grid_w(ctypes.byref(pr), _p(subs), len(subs), _p(vis), _p(uvw), uvw.shape[1], _p(freq),
                               len(freq), _p(g)), "IDG.GridW")
    return g


def idg_degrid(consts, subs, grid, uvw, freq, wstack=False):
    """IDG.DeGrid / DeGridW.  Returns (vis, shifted_grid) -- the reference shifts the caller's grid in place."""
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    g = _c128(grid).copy()
    uvw, freq = np.ascontiguousarray(uvw, np.float64), np.ascontiguousarray(freq, np.float64)
    nbl, nt = uvw.shape[0], uvw.shape[1]
    vis = np.zeros((nbl, nt, len(freq)), np.complex128)
    pr = params(consts)
    fn = lib().oc_idg_degrid_w if wstack else lib().oc_idg_degrid
    _check(fn(ctypes.byref(pr), _p(subs), len(subs), _p(g), _p(uvw), nbl, nt, _p(freq), len(freq), _p(vis)),
           "IDG.DeGrid")
    return vis, g


def unit_vis(flags):
    f = np.ascontiguousarray(flags, np.uint8)
    out = np.zeros(f.shape, np.complex128)
    lib().oc_unit_vis(_p(f), f.size, _p(out))
    return out


def vis_subtract(v0, v1, flags):
    v0, v1 = _c128(v0), _c128(v1)
    f = np.ascontiguousarray(flags, np.uint8)
    out = np.zeros_like(v0)
    lib().oc_vis_subtract(_p(v0), _p(v1), _p(f), f.size, _p(out))
    return out


def num_threads():
    return lib().oc_num_threads()


def set_num_threads(n):
    lib().oc_set_num_threads(int(n))


# ---------- deconvolution side of the serial major cycle (deconv_oracle.c) ----------

INDEX_OUT_OF_RANGE = 10

CYCLE_DTYPE = np.dtype([("max_dirty", "<f4"), ("max_b", "<f4"), ("current_lambda", "<f4"), ("abs_max", "<f4"),
                        ("deconvolved", "<i4"), ("converged", "<i4"), ("iterations", "<i4"), ("pad", "<i4"),
                        ("objective", "<f8")])


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def elastic_net_penalty(img, lam, alpha):
    img = _f32(img)
    return lib().ocd_elastic_net_penalty(_p(img), img.shape[0], img.shape[1], float(lam), float(alpha))


def get_max(img):
    img = _f32(img)
    return float(lib().ocd_get_max(_p(img), img.size))


def residual_penalty(img):
    img = _f32(img)
    return lib().ocd_residual_penalty(_p(img), img.size)


def max_lipschitz(psf):
    psf = _f32(psf)
    return lib().ocd_max_lipschitz(_p(psf), psf.shape[0], psf.shape[1])


def psf_cut(psf, factor):
    psf = _f32(psf)
    m = psf.shape[0] // factor
    out = np.zeros((m, m), np.float32)
    lib().ocd_psf_cut(_p(psf), psf.shape[0], int(factor), _p(out))
    return out


def max_sidelobe(psf, factor):
    psf = _f32(psf)
    return float(lib().ocd_max_sidelobe(_p(psf), psf.shape[0], int(factor)))


def amap_scan(psf):
    psf = _f32(psf)
    out = np.zeros(psf.shape, np.float64)
    lib().ocd_amap_scan(_p(psf), psf.shape[0], psf.shape[1], _p(out))
    return out


def amap(psf, total, section=None):
    """PSF.CalcAMap(psf, totalSize=(0,0,*total), imageSection=(y, x, yEnd, xEnd))."""
    psf = _f32(psf)
    sy, sx, sye, sxe = section if section is not None else (0, 0, total[0], total[1])
    out = np.zeros((sye - sy, sxe - sx), np.float32)
    lib().ocd_amap(_p(psf), psf.shape[0], psf.shape[1], int(total[0]), int(total[1]), sy, sx, sye, sxe, _p(out))
    return out


def padded_fourier_correlation(psf, pad):
    psf = _f32(psf)
    out = np.zeros((pad[0] + psf.shape[0], pad[1] + psf.shape[1]), np.complex128)
    _check(lib().ocd_padded_fourier_correlation(_p(psf), psf.shape[0], psf.shape[1], int(pad[0]), int(pad[1]),
                                                _p(out)), "PSF.CalcPaddedFourierCorrelation")
    return out


def padded_convolve(kernel, kernel_rect, img):
    kernel = _c128(kernel)
    img = _f32(img)
    out = np.zeros(img.shape, np.float32)
    _check(lib().ocd_padded_convolve(_p(kernel), kernel.shape[0], kernel.shape[1], int(kernel_rect[0]),
                                     int(kernel_rect[1]), _p(img), img.shape[0], _p(out)), "PaddedConvolver.Convolve")
    return out


def psf_squared(psf):
    psf = _f32(psf)
    out = np.zeros((2 * psf.shape[0], 2 * psf.shape[1]), np.float32)
    _check(lib().ocd_psf_squared(_p(psf), psf.shape[0], psf.shape[1], _p(out)), "PSF.CalcPSFSquared")
    return out


def get_abs_max_diff(x, g, a, lam, alpha):
    x, g, a = _f32(x), _f32(g), _f32(a)
    return float(lib().ocd_get_abs_max_diff(_p(x), _p(g), _p(a), x.shape[0], float(lam), float(alpha)))


def get_abs_max_pixel(x, g, a, lam, alpha):
    """FastSerialCD.GetAbsMax -> (y, x, diff, new value)."""
    x, g, a = _f32(x), _f32(g), _f32(a)
    yx = np.zeros(2, np.int32)
    xn = np.zeros(1, np.float32)
    d = lib().ocd_get_abs_max_pixel(_p(x), _p(g), _p(a), x.shape[0], float(lam), float(alpha), _p(yx), _p(xn))
    return int(yx[0]), int(yx[1]), float(d), float(xn[0])


def deconvolve(x, g, a, psf2, lam, alpha, iterations, epsilon):
    """FastSerialCD.Deconvolve on copies -> (x, g, converged, iterations)."""
    x, g = _f32(x).copy(), _f32(g).copy()
    a, psf2 = _f32(a), _f32(psf2)
    conv = np.zeros(1, np.int32)
    it = np.zeros(1, np.int32)
    _check(lib().ocd_deconvolve(_p(x), _p(g), _p(a), x.shape[0], _p(psf2), psf2.shape[0], psf2.shape[1], float(lam),
                                float(alpha), int(iterations), float(epsilon), _p(conv), _p(it)),
           "FastSerialCD.Deconvolve")
    return x, g, bool(conv[0]), int(it[0])


def major_cycle(consts, subs, uvw, freq, vis, flags, psf_cut_factor, max_major, lam, alpha, deconv_iterations,
                deconv_epsilon):
    """MajorCycle.ReconstructSerialCD with FastSerialCD -> dict(model, residual, psf, cycles)."""
    N = consts["grid_size"]
    subs = np.ascontiguousarray(subs, SUBGRID_DTYPE)
    uvw, freq = np.ascontiguousarray(uvw, np.float64), np.ascontiguousarray(freq, np.float64)
    vis = _c128(vis)
    flags = np.ascontiguousarray(flags, np.uint8)
    nbl, nt = uvw.shape[0], uvw.shape[1]
    model = np.zeros((N, N), np.float32)
    resid = np.zeros((N, N), np.float32)
    psf = np.zeros((N, N), np.float32)
    cycles = np.zeros(max(1, max_major), CYCLE_DTYPE)
    nc = np.zeros(1, np.int32)
    pr = params(consts)
    _check(lib().ocd_major_cycle(ctypes.byref(pr), _p(subs), len(subs), _p(uvw), nbl, nt, _p(freq), len(freq),
                                 _p(vis), _p(flags), int(psf_cut_factor), int(max_major), float(lam), float(alpha),
                                 int(deconv_iterations), float(deconv_epsilon), _p(model), _p(resid), _p(psf),
                                 _p(cycles), _p(nc)), "MajorCycle.ReconstructSerialCD")
    return dict(model=model, residual=resid, psf=psf, cycles=cycles[:nc[0]])
