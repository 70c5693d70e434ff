"""GB300-native (sm_103a) image-domain gridder with w-stacking.

Drop-in for the gridding path of lord-blueberry/p9-distributed-reconstruction
(Core.ImageDomainGridder + the Core.FFT members it uses) and for the deconvolution side of
its serial major cycle (FastSerialCD, PaddedConvolver, the PSF helpers, MajorCycle).  The compute lives in
libp9idg.so (CUDA kernels + C ABI, include/p9idg.h); this package is the host-side
mirror of the reference API over that ABI.
"""
from . import _native
from ._native import (MODE_FP32, MODE_TC_BF16X3, MODE_TC_FP16X3, NativeLibraryMissing, STAGES, TC_MAX_W_TERM,
                      TC_MAX_W_TERM2)
from .idg import (FFT, IDG, Batch, GriddingConstants, P9IDGError, Partition, Partitioner, Plan, Subgrid, SUBGRID_DTYPE,
                  autotune, device_count, measure_sincos_peak, plan_from_subgrids, set_chunking)
from .deconv import PSF, DeconvolutionResult, FastSerialCD, MajorCycle, PaddedConvolver, Rectangle
from .fitsio import FitsIO

__all__ = ["FFT", "IDG", "Batch", "autotune", "set_chunking", "GriddingConstants", "P9IDGError", "Partition", "Partitioner", "Plan", "Subgrid",
           "SUBGRID_DTYPE", "MODE_FP32", "MODE_TC_BF16X3", "MODE_TC_FP16X3", "NativeLibraryMissing", "STAGES",
           "TC_MAX_W_TERM", "TC_MAX_W_TERM2",
           "device_count", "measure_sincos_peak", "plan_from_subgrids",
           "PSF", "DeconvolutionResult", "FastSerialCD", "MajorCycle", "PaddedConvolver", "Rectangle", "FitsIO"]
