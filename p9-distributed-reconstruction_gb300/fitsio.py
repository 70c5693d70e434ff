"""FitsIO (Core/FitsIO.cs) over the C ABI: the reference's FITS data layout, read and written
by the library's host code (big-endian decoding split over the host cores)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _native as nat
from .idg import P9IDGError, _check, _ptr


def _path(file) -> bytes:
    return os.fsencode(os.fspath(file))


def shape(file):
    """(BITPIX, FITS axes with NAXIS1 first) of the primary array."""
    bp, na = ctypes.c_int32(), ctypes.c_int32()
    axes = np.zeros(16, np.int64)
    _check(nat.lib().p9idg_fits_shape(_path(file), ctypes.byref(bp), ctypes.byref(na), _ptr(axes), 16))
    return bp.value, tuple(int(a) for a in axes[:na.value])


class FitsIO:
    @staticmethod
    def CountBaselines(file) -> int:
        return shape(file)[1][2]

    @staticmethod
    def ReadUVW(file, fromBl=None, toBl=None) -> np.ndarray:
        _, ax = shape(file)
        if len(ax) != 3:
            raise P9IDGError(nat.INVALID_ARGUMENT, f"{os.fspath(file)}: ReadUVW needs a [baseline][time][3] array")
        fromBl = 0 if fromBl is None else int(fromBl)
        toBl = ax[2] if toBl is None else int(toBl)
        out = np.zeros((toBl - fromBl, ax[1], 3), np.float64)
        _check(nat.lib().p9idg_fits_read_uvw(_path(file), fromBl, toBl, _ptr(out)))
        return out

    @staticmethod
    def ReadFrequencies(file) -> np.ndarray:
        _, ax = shape(file)
        if len(ax) != 1:
            raise P9IDGError(nat.INVALID_ARGUMENT, f"{os.fspath(file)}: ReadFrequencies needs a 1-D array")
        out = np.zeros(ax[0], np.float64)
        _check(nat.lib().p9idg_fits_read_frequencies(_path(file), _ptr(out), len(out)))
        return out

    @staticmethod
    def ReadVisibilities(file, baselinesCount, timessamplesCount, channelsCount, norm, fromBl=0) -> np.ndarray:
        """ReadVisibilities(file, nbl, nt, nch, norm), or with fromBl the (file, fromBl, toBl, ...) overload
        where baselinesCount is then toBl."""
        toBl = int(baselinesCount)
        out = np.zeros((toBl - fromBl, timessamplesCount, channelsCount), np.complex128)
        _check(nat.lib().p9idg_fits_read_visibilities(_path(file), int(fromBl), toBl, int(timessamplesCount),
                                                      int(channelsCount), float(norm), _ptr(out)))
        return out

    @staticmethod
    def ReadFlags(file, baselinesCount, timessamplesCount, channelsCount, fromBl=0) -> np.ndarray:
        toBl = int(baselinesCount)
        out = np.zeros((toBl - fromBl, timessamplesCount, channelsCount), np.uint8)
        _check(nat.lib().p9idg_fits_read_flags(_path(file), int(fromBl), toBl, int(timessamplesCount),
                                               int(channelsCount), _ptr(out)))
        return out.astype(bool)

    @staticmethod
    def _read_image(file, bitpix, dtype):
        _, ax = shape(file)
        if len(ax) != 2:
            raise P9IDGError(nat.INVALID_ARGUMENT, f"{os.fspath(file)}: not a 2-D image")
        out = np.zeros((ax[1], ax[0]), dtype)
        _check(nat.lib().p9idg_fits_read_image(_path(file), bitpix, _ptr(out), out.size))
        return out

    @staticmethod
    def ReadImage(file) -> np.ndarray:
        return FitsIO._read_image(file, -32, np.float32)

    @staticmethod
    def ReadImageDouble(file) -> np.ndarray:
        return FitsIO._read_image(file, -64, np.float64)

    @staticmethod
    def Write(img, file="Outputfile.fits"):
        """Write<T>(T[,] img): float32 images as BITPIX -32, anything else as float64 (-64)."""
        a = np.asarray(img)
        if np.iscomplexobj(a):  # Write(Complex[,]) keeps the real part
            a = a.real
        a = np.ascontiguousarray(a, np.float32 if a.dtype == np.float32 else np.float64)
        bitpix = -32 if a.dtype == np.float32 else -64
        _check(nat.lib().p9idg_fits_write_image(_path(file), bitpix, _ptr(a), a.shape[0], a.shape[1]))
