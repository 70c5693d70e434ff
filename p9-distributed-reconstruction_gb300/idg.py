"""Host-side mirror of the reference's gridding API over the C ABI.

Names, argument order and meaning follow Distributed-Reconstruction/Core:
GriddingConstants (ImageDomainGridder/GriddingConstants.cs:33), Subgrid (Subgrid.cs:15),
Partitioner.CreatePartition (Partitioner.cs:20), IDG.Grid/DeGrid/GridW/DeGridW/GridPSF/
ToImage/CalculatePSF (IDG.cs:12-114) and FFT.WStackIFFTFloat/Shift/Forward/BackwardFloat
(FFT.cs).  Arrays are numpy: uvw float64[nbl, nt, 3], frequencies float64[nch],
visibilities complex128[nbl, nt, nch], flags bool[nbl, nt, nch], grids complex128[N, N].
The reference's exceptions become P9IDGError carrying the same message.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat

SUBGRID_DTYPE = np.dtype([("baseline_idx", "<i4"), ("time_sample_start", "<i4"), ("time_sample_count", "<i4"),
                          ("u_pixel", "<i4"), ("v_pixel", "<i4"), ("w_lambda", "<i4")])

_MESSAGES = {
    nat.CANNOT_PLACE: "could not place (all) visibilities on subgrid (too many channnels, kernel size too large)",
    nat.SUBGRID_OUT_OF_GRID: "subgrid falls not within grid",
    nat.INVALID_GRID: "invalid grid",
}


class P9IDGError(RuntimeError):
    """A failed library call; .code is the p9idg_status."""

    def __init__(self, code: int, detail: str):
        msg = _MESSAGES.get(code, detail) if not detail else detail
        super().__init__(msg)
        self.code = code


def _check(code: int):
    if code != nat.OK:
        raise P9IDGError(code, nat.last_error())


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _c128(a, name):
    a = np.asarray(a)
    if a.dtype != np.complex128 or not a.flags.c_contiguous:
        a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _out(out, shape):
    """A caller-supplied output array (checked) or a new one."""
    if out is None:
        return np.empty(shape, np.complex128)
    if not (isinstance(out, np.ndarray) and out.dtype == np.complex128 and out.shape == tuple(shape)
            and out.flags.c_contiguous and out.flags.writeable):
        raise ValueError(f"out must be a writeable C-contiguous complex128 array of shape {tuple(shape)}")
    return out


def _expect_shape(a, shape, name):
    """The C ABI sizes every array from the plan; a wrong shape would be read or written out of
    bounds, so it is refused here (the reference throws IndexOutOfRangeException)."""
    if a is not None and tuple(np.shape(a)) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(np.shape(a))}; the plan needs {tuple(shape)}")


def _check_inputs(p, c, vis=None, uvw=None, flags=None, grid=None):
    _expect_shape(vis, (p.nbl, p.nt, p.nch), "visibilities")
    _expect_shape(uvw, (p.nbl, p.nt, 3), "uvw")
    _expect_shape(flags, (p.nbl, p.nt, p.nch), "flags")
    _expect_shape(grid, (c.GridSize, c.GridSize), "grid")


class GriddingConstants:
    """Immutable gridding parameters (GriddingConstants.cs:11-52).

    scaleArcSec is the cell size in radians, held as float32 like the reference.
    WStepLambda is never assigned by the reference constructor and stays 0.
    """

    def __init__(self, visCount, gridSize, subgridSize, kernelSize, maxTimesteps, scaleArcSec, wLayerCount, wStep):
        self.VisibilitiesCount = int(visCount)
        self.GridSize = int(gridSize)
        self.SubgridSize = int(subgridSize)
        self.KernelSize = int(kernelSize)
        self.MaxTimestepsPerSubgrid = int(maxTimesteps)
        self.ScaleArcSec = float(np.float32(scaleArcSec))
        self.ImageSize = float(np.float32(scaleArcSec) * np.float32(gridSize))
        self.WLayerCount = int(wLayerCount)
        self.WStep = float(wStep)
        self.WStepLambda = 0.0
        self.SubgridSpheroidal = np.ones((self.SubgridSize, self.SubgridSize), np.float32)
        self.GridSpheroidal = None  # identity, not materialised

    @classmethod
    def from_dict(cls, d):
        return cls(d["vis_count"], d["grid_size"], d["subgrid_size"], d["kernel_size"], d["max_timesteps"],
                   d["scale_arcsec"], d["wlayer_count"], d["wstep"])

    def native(self) -> nat.Params:
        return nat.Params(self.VisibilitiesCount, self.GridSize, self.SubgridSize, self.KernelSize,
                          self.MaxTimestepsPerSubgrid, self.ScaleArcSec, self.WLayerCount, self.WStep)

    def key(self):
        return (self.VisibilitiesCount, self.GridSize, self.SubgridSize, self.KernelSize,
                self.MaxTimestepsPerSubgrid, self.ScaleArcSec, self.WLayerCount, self.WStep)


class Subgrid:
    """Subgrid.cs:15-24."""
    __slots__ = ("baselineIdx", "timeSampleStart", "timeSampleCount", "UPixel", "VPixel", "WLambda")

    def __init__(self, baselineIdx=0, timeSampleStart=0, timeSampleCount=0, UPixel=0, VPixel=0, WLambda=0):
        self.baselineIdx = int(baselineIdx)
        self.timeSampleStart = int(timeSampleStart)
        self.timeSampleCount = int(timeSampleCount)
        self.UPixel = int(UPixel)
        self.VPixel = int(VPixel)
        self.WLambda = int(WLambda)

    def __eq__(self, o):
        return all(getattr(self, k) == getattr(o, k) for k in self.__slots__)

    def __repr__(self):
        return "Subgrid(" + ", ".join(f"{k}={getattr(self, k)}" for k in self.__slots__) + ")"


class Plan:
    """Owns a native p9idg_plan (subgrid list, device buffers, stream)."""

    def __init__(self, handle, consts: GriddingConstants, nbl, nt, nch):
        self._h = handle
        self.constants = consts
        self.nbl, self.nt, self.nch = nbl, nt, nch

    @property
    def handle(self):
        if not self._h:
            raise ValueError("plan destroyed")
        return self._h

    def destroy(self):
        if getattr(self, "_h", None):
            nat.lib().p9idg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # ---- description ----
    def subgrids(self) -> np.ndarray:
        n = ctypes.c_int64()
        _check(nat.lib().p9idg_plan_num_subgrids(self.handle, ctypes.byref(n)))
        out = np.zeros(n.value, SUBGRID_DTYPE)
        _check(nat.lib().p9idg_plan_get_subgrids(self.handle, _ptr(out) if n.value else None, n.value))
        return out

    def info(self) -> dict:
        i = nat.PlanInfo()
        _check(nat.lib().p9idg_plan_get_info(self.handle, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in nat.PlanInfo._fields_}

    def set_mode(self, mode: int) -> int:
        """Selects the kernels; returns the mode the plan runs.  A tensor-core mode on a plan whose
        w term exceeds TC_MAX_W_TERM keeps the FP32 kernels (``info()["tc_w_term"]`` says by how
        much)."""
        _check(nat.lib().p9idg_plan_set_mode(self.handle, int(mode)))
        return self.info()["mode"]

    def set_tc_order(self, order: int):
        """Tensor-core form: 0 = automatic (first order where its bound holds), 2 = second order."""
        _check(nat.lib().p9idg_plan_set_tc_order(self.handle, int(order)))

    def set_taper(self, taper):
        t = None if taper is None else np.ascontiguousarray(taper, np.float32)
        _check(nat.lib().p9idg_plan_set_taper(self.handle, _ptr(t)))

    def set_host_access(self, in_place: bool):
        """Host-array calls use the caller's arrays in place (1, where the device reaches host
        memory) or stage them through device copies (0)."""
        _check(nat.lib().p9idg_plan_set_host_access(self.handle, int(bool(in_place))))

    def host_access(self) -> bool:
        v = ctypes.c_int32()
        _check(nat.lib().p9idg_plan_get_host_access(self.handle, ctypes.byref(v)))
        return bool(v.value)

    def set_stream(self, stream_handle: int):
        _check(nat.lib().p9idg_plan_set_stream(self.handle, ctypes.c_void_p(stream_handle or None)))

    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(nat.lib().p9idg_plan_get_stream(self.handle, ctypes.byref(s)))
        return s.value or 0

    # ---- device-resident entry points (raw device pointers, complex64) ----
    def grid_w_device(self, d_vis: int, d_layers: int):
        _check(nat.lib().p9idg_grid_w_device(self.handle, ctypes.c_void_p(d_vis), ctypes.c_void_p(d_layers)))

    def degrid_w_device(self, d_grid: int, d_vis: int):
        _check(nat.lib().p9idg_degrid_w_device(self.handle, ctypes.c_void_p(d_grid), ctypes.c_void_p(d_vis)))

    def grid_device(self, d_vis: int, d_grid: int):
        _check(nat.lib().p9idg_grid_device(self.handle, ctypes.c_void_p(d_vis), ctypes.c_void_p(d_grid)))

    def degrid_device(self, d_grid: int, d_vis: int):
        _check(nat.lib().p9idg_degrid_device(self.handle, ctypes.c_void_p(d_grid), ctypes.c_void_p(d_vis)))

    def wstack_image_device(self, d_layers: int, d_image: int, shift: bool = True):
        _check(nat.lib().p9idg_wstack_image_device(self.handle, ctypes.c_void_p(d_layers),
                                                   ctypes.c_void_p(d_image), int(bool(shift))))

    def synchronize(self):
        _check(nat.lib().p9idg_synchronize(self.handle))

    # ---- timing ----
    def enable_timing(self, on=True):
        _check(nat.lib().p9idg_plan_enable_timing(self.handle, int(bool(on))))

    def reset_timing(self):
        _check(nat.lib().p9idg_plan_reset_timing(self.handle))

    def stage_times(self) -> dict:
        ms = np.zeros(len(nat.STAGES), np.float64)
        n = np.zeros(len(nat.STAGES), np.int64)
        _check(nat.lib().p9idg_plan_stage_times(self.handle, _ptr(ms), _ptr(n)))
        return {s: (float(ms[i]), int(n[i])) for i, s in enumerate(nat.STAGES)}


class Partition(list):
    """List<List<Subgrid>> (one list per baseline) bound to the native plan that made it."""

    def __init__(self, lists, plan: Plan):
        super().__init__(lists)
        self.plan = plan

    @staticmethod
    def from_array(arr: np.ndarray, nbl: int, plan: Plan) -> "Partition":
        lists = [[] for _ in range(nbl)]
        for r in arr:
            lists[int(r["baseline_idx"])].append(Subgrid(*[int(r[k]) for k in SUBGRID_DTYPE.names]))
        return Partition(lists, plan)


def _flatten(metadata) -> np.ndarray:
    rows = []
    for bl, lst in enumerate(metadata):
        for s in lst:
            # the reference gridder indexes uvw/vis by list position (Gridder.cs:28,58)
            rows.append((bl, s.timeSampleStart, s.timeSampleCount, s.UPixel, s.VPixel, s.WLambda))
    return np.array(rows, SUBGRID_DTYPE) if rows else np.zeros(0, SUBGRID_DTYPE)


def plan_from_subgrids(c: GriddingConstants, subgrids: np.ndarray, uvw, frequencies) -> Plan:
    uvw = _f64(uvw)
    freq = _f64(frequencies)
    subgrids = np.ascontiguousarray(subgrids, SUBGRID_DTYPE)
    h = ctypes.c_void_p()
    pr = c.native()
    _check(nat.lib().p9idg_plan_create_from_subgrids(ctypes.byref(pr), _ptr(subgrids) if len(subgrids) else None,
                                                     len(subgrids), _ptr(uvw), uvw.shape[0], uvw.shape[1],
                                                     _ptr(freq), len(freq), ctypes.byref(h)))
    return Plan(h, c, uvw.shape[0], uvw.shape[1], len(freq))


def _plan_for(c: GriddingConstants, metadata, uvw, frequencies) -> Plan:
    if uvw is None:
        # the uvw the partition was made from, kept on the device by its plan (p9idg_* with uvw NULL)
        if not (isinstance(metadata, Partition) and metadata.plan is not None
                and metadata.plan.constants.key() == c.key() and metadata.plan.nch == len(frequencies)):
            raise ValueError("uvw=None needs the Partition (with its plan) that Partitioner.CreatePartition made")
        return metadata.plan
    uvw = np.asarray(uvw)
    if isinstance(metadata, Partition) and metadata.plan is not None:
        p = metadata.plan
        if p.constants.key() == c.key() and (p.nbl, p.nt, p.nch) == (uvw.shape[0], uvw.shape[1], len(frequencies)):
            return p
    return plan_from_subgrids(c, _flatten(metadata), uvw, frequencies)


class Partitioner:
    @staticmethod
    def CreatePartition(c: GriddingConstants, uvw, frequencies) -> Partition:
        """Partitioner.CreatePartition (Partitioner.cs:20-125)."""
        uvw = _f64(uvw)
        freq = _f64(frequencies)
        h = ctypes.c_void_p()
        pr = c.native()
        _check(nat.lib().p9idg_plan_create(ctypes.byref(pr), _ptr(uvw), uvw.shape[0], uvw.shape[1], _ptr(freq),
                                           len(freq), ctypes.byref(h)))
        plan = Plan(h, c, uvw.shape[0], uvw.shape[1], len(freq))
        return Partition.from_array(plan.subgrids(), uvw.shape[0], plan)

    @staticmethod
    def MetersToPixels(meters, imageSize, frequency):
        return meters * imageSize * (frequency / 299792458.0)

    @staticmethod
    def MetersToLambda(meters, frequency):
        return meters * (frequency / 299792458.0)


class IDG:
    """IDG.cs:10-115."""

    @staticmethod
    def Grid(c, metadata, visibilities, uvw, frequencies, out=None) -> np.ndarray:
        p = _plan_for(c, metadata, uvw, frequencies)
        vis, uvw = _c128(visibilities, "visibilities"), _f64(uvw)
        _check_inputs(p, c, vis=vis, uvw=uvw)
        out = _out(out, (c.GridSize, c.GridSize))
        _check(nat.lib().p9idg_grid(p.handle, _ptr(vis), _ptr(uvw), _ptr(out)))
        return out

    @staticmethod
    def DeGrid(c, metadata, grid, uvw, frequencies, out=None) -> np.ndarray:
        """Like the reference, FFT.Shift is applied to `grid` in place when it is a
        C-contiguous complex128 array."""
        return IDG._degrid(c, metadata, grid, uvw, frequencies, nat.lib().p9idg_degrid, out)

    @staticmethod
    def GridW(c, metadata, visibilities, uvw, frequencies, out=None) -> np.ndarray:
        """`out` (optional): a C-contiguous complex128 [W][N][N] array to write into, e.g. in
        page-locked memory; the reference returns a new List<Complex[,]>.  `uvw` None (here and in
        every IDG member): the uvw the partition was made from, which its plan keeps on the device,
        so a call uploads and compares none (the reference's callers pass the same uvw every
        cycle, MajorCycle.cs:46,88)."""
        p = _plan_for(c, metadata, uvw, frequencies)
        vis, uvw = _c128(visibilities, "visibilities"), _f64(uvw)
        _check_inputs(p, c, vis=vis, uvw=uvw)
        out = _out(out, (c.WLayerCount, c.GridSize, c.GridSize))
        _check(nat.lib().p9idg_grid_w(p.handle, _ptr(vis), _ptr(uvw), _ptr(out)))
        return out

    @staticmethod
    def DeGridW(c, metadata, grid, uvw, frequencies, out=None) -> np.ndarray:
        return IDG._degrid(c, metadata, grid, uvw, frequencies, nat.lib().p9idg_degrid_w, out)

    @staticmethod
    def _degrid(c, metadata, grid, uvw, frequencies, fn, out=None):
        p = _plan_for(c, metadata, uvw, frequencies)
        g = grid if (isinstance(grid, np.ndarray) and grid.dtype == np.complex128 and grid.flags.c_contiguous
                     and grid.flags.writeable) else _c128(grid, "grid").copy()
        uvw = _f64(uvw)
        _check_inputs(p, c, uvw=uvw, grid=g)
        vis = _out(out, (p.nbl, p.nt, p.nch))
        _check(fn(p.handle, _ptr(g), _ptr(uvw), _ptr(vis)))
        return vis

    @staticmethod
    def GridPSF(c, metadata, uvw, flags, frequencies) -> np.ndarray:
        p = _plan_for(c, metadata, uvw, frequencies)
        f = np.ascontiguousarray(flags, dtype=np.uint8)
        uvw = _f64(uvw)
        _check_inputs(p, c, uvw=uvw, flags=f)
        out = np.empty((c.GridSize, c.GridSize), np.complex128)
        _check(nat.lib().p9idg_grid_psf(p.handle, _ptr(uvw), _ptr(f), _ptr(out)))
        return out

    @staticmethod
    def ToImage(c, metadata, visibilities, uvw, frequencies) -> np.ndarray:
        p = _plan_for(c, metadata, uvw, frequencies)
        vis, uvw = _c128(visibilities, "visibilities"), _f64(uvw)
        _check_inputs(p, c, vis=vis, uvw=uvw)
        out = np.empty((c.GridSize, c.GridSize), np.float64)
        _check(nat.lib().p9idg_to_image(p.handle, _ptr(vis), _ptr(uvw), _ptr(out)))
        return out

    @staticmethod
    def CalculatePSF(c, metadata, uvw, flags, frequencies) -> np.ndarray:
        p = _plan_for(c, metadata, uvw, frequencies)
        f = np.ascontiguousarray(flags, dtype=np.uint8)
        uvw = _f64(uvw)
        _check_inputs(p, c, uvw=uvw, flags=f)
        out = np.empty((c.GridSize, c.GridSize), np.float64)
        _check(nat.lib().p9idg_calculate_psf(p.handle, _ptr(uvw), _ptr(f), _ptr(out)))
        return out


class FFT:
    """Core/FFT.cs static members on the path."""

    @staticmethod
    def WStackIFFTFloat(grid, visibilityCount) -> np.ndarray:
        layers = _c128(np.asarray(grid), "grid")
        if layers.ndim == 2:
            layers = layers[None]
        W, N, _ = layers.shape
        out = np.empty((N, N), np.float32)
        _check(nat.lib().p9idg_wstack_ifft_float(_ptr(layers), W, N, int(visibilityCount), _ptr(out)))
        return out

    @staticmethod
    def Shift(a):
        """In-place quadrant swap (FFT.cs:221-264) of a square array or a stack of them."""
        if not (isinstance(a, np.ndarray) and a.flags.c_contiguous and a.flags.writeable):
            raise TypeError("FFT.Shift needs a writeable C-contiguous numpy array")
        if a.ndim == 3:
            for layer in a:
                FFT.Shift(layer)
            return a
        if a.dtype.itemsize not in (4, 8, 16):
            raise TypeError(a.dtype)
        _check(nat.lib().p9idg_fft_shift(_ptr(a), a.shape[0], a.dtype.itemsize))
        return a

    @staticmethod
    def Forward(image, norm=1.0) -> np.ndarray:
        img = np.ascontiguousarray(image, np.float32)
        out = np.empty(img.shape, np.complex128)
        _check(nat.lib().p9idg_fft_forward_float(_ptr(img), img.shape[0], float(norm), _ptr(out)))
        return out

    @staticmethod
    def BackwardFloat(grid, norm) -> np.ndarray:
        g = _c128(grid, "grid")
        out = np.empty(g.shape, np.float32)
        _check(nat.lib().p9idg_fft_backward_float(_ptr(g), g.shape[0], float(norm), _ptr(out)))
        return out


class Tuning(ctypes.Structure):
    _fields_ = [("subgrid_size", ctypes.c_int32), ("kernel_size", ctypes.c_int32),
                ("gridder_max_vis", ctypes.c_int32), ("degridder_max_vis", ctypes.c_int32),
                ("seconds_per_gridded_vis", ctypes.c_double), ("gridded_fraction", ctypes.c_double)]


def autotune(c: GriddingConstants, uvw, frequencies, mode=nat.MODE_FP32, subgrid_sizes=None) -> dict:
    """p9idg_autotune: subgrid size and work-item sizes timed on a sample of the baselines."""
    uvw = _f64(uvw)
    freq = _f64(frequencies)
    sizes = None if subgrid_sizes is None else np.ascontiguousarray(subgrid_sizes, np.int32)
    out = Tuning()
    pr = c.native()
    _check(nat.lib().p9idg_autotune(ctypes.byref(pr), _ptr(uvw), uvw.shape[0], uvw.shape[1], _ptr(freq), len(freq),
                                    int(mode), _ptr(sizes), 0 if sizes is None else len(sizes), ctypes.byref(out)))
    return {k: getattr(out, k) for k, _ in Tuning._fields_}


class Batch:
    """p9idg_batch: many plans gridded/degridded with one launch per kernel stage.

    Device buffers (raw pointers, complex64) are fixed at creation: per plan its
    visibilities, w layers (output of grid_w), model grid (input of degrid_w) and
    degridded visibilities."""

    def __init__(self, plans, d_vis, d_layers, d_grids, d_vis_out):
        n = len(plans)
        arr = lambda xs: (ctypes.c_void_p * n)(*[ctypes.c_void_p(int(x)) for x in xs])  # noqa: E731
        self._plans = list(plans)  # keep the plans alive
        self._h = ctypes.c_void_p()
        _check(nat.lib().p9idg_batch_create((ctypes.c_void_p * n)(*[p.handle for p in plans]), n, arr(d_vis),
                                            arr(d_layers), arr(d_grids), arr(d_vis_out), ctypes.byref(self._h)))

    def grid_w(self):
        _check(nat.lib().p9idg_batch_grid_w(self._h))

    def degrid_w(self):
        _check(nat.lib().p9idg_batch_degrid_w(self._h))

    def capture_graph(self):
        _check(nat.lib().p9idg_batch_capture_graph(self._h))

    def run(self):
        _check(nat.lib().p9idg_batch_run(self._h))

    THROUGHPUT, SMALL_FIRST = 0, 1

    def set_schedule(self, schedule: int):
        """Work-item order: Batch.THROUGHPUT (default) or Batch.SMALL_FIRST; drops a captured graph."""
        _check(nat.lib().p9idg_batch_set_schedule(self._h, int(schedule)))

    def synchronize(self):
        _check(nat.lib().p9idg_batch_synchronize(self._h))

    def latencies_ms(self) -> np.ndarray:
        out = np.zeros(len(self._plans), np.float64)
        _check(nat.lib().p9idg_batch_latencies(self._h, _ptr(out)))
        return out

    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(nat.lib().p9idg_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def destroy(self):
        if getattr(self, "_h", None) and self._h.value:
            nat.lib().p9idg_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def set_chunking(plan: Plan, gridder_max_vis: int, degridder_max_vis: int):
    _check(nat.lib().p9idg_plan_set_chunking(plan.handle, int(gridder_max_vis), int(degridder_max_vis)))


def device_count() -> int:
    return int(nat.lib().p9idg_device_count())


def measure_sincos_peak():
    s = ctypes.c_double()
    f = ctypes.c_double()
    _check(nat.lib().p9idg_measure_sincos_peak(ctypes.byref(s), ctypes.byref(f)))
    return s.value, f.value
