"""p9idg_grid_w_device_noalloc: the w-stacked gridder for callers that cannot allocate
device memory (a pipeline with a fixed memory reservation, a framework that owns every
device byte, a process under a device-memory quota).

Its output is checked against the regular device entry point, p9idg_grid_w_device, on two
calls in a row with different visibilities, so the second call also shows that whatever the
first left in the shared scratch array does not leak into the result.  This file sorts last
so a run that stops at the first failure has run everything else first.
"""
import ctypes

import numpy as np
import pytest

from conftest import constants, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _compare_two_calls(cd_over, min_subgrids=0):
    torch = pytest.importorskip("torch")
    obs, cd = workload("meerkat_3072", n_ant=10, nt=300 if not min_subgrids else 1000, nch=16)
    c, cd = constants(cd, **cd_over)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    plan = part.plan
    stream = torch.cuda.current_stream()
    plan.set_stream(stream.cuda_stream)
    N, W = cd["grid_size"], cd["wlayer_count"]
    subs = plan.subgrids()
    assert len(subs) >= max(1, min_subgrids)
    d_subs = torch.from_numpy(subs.view(np.int32).reshape(-1, 6).copy()).cuda()
    d_uvw = torch.from_numpy(obs.uvw).cuda()
    freq = np.ascontiguousarray(obs.frequencies, np.float64)
    params = c.native()
    rng = np.random.default_rng(12)
    second = (rng.standard_normal(obs.vis.shape) + 1j * rng.standard_normal(obs.vis.shape)).astype(np.complex64)
    L = pkg._native.lib()
    for vis in (obs.vis.astype(np.complex64), second):
        d_vis = torch.from_numpy(vis).cuda()
        ref = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
        plan.grid_w_device(d_vis.data_ptr(), ref.data_ptr())
        plan.synchronize()
        out = torch.full((W, N, N), 7.0 + 7.0j, dtype=torch.complex64, device="cuda")  # stale output contents
        st = L.p9idg_grid_w_device_noalloc(ctypes.byref(params), ctypes.c_void_p(d_subs.data_ptr()), len(subs),
                                           ctypes.c_void_p(d_uvw.data_ptr()), obs.uvw.shape[0], obs.uvw.shape[1],
                                           freq.ctypes.data_as(ctypes.c_void_p), len(freq),
                                           ctypes.c_void_p(d_vis.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, pkg._native.last_error()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < TOL
    plan.set_stream(0)


@pytest.mark.parametrize("S,kernel", [(32, 8), (16, 4), (48, 8)])
def test_noalloc_matches_regular_entry_point(need_gpu, S, kernel):
    _compare_two_calls(dict(subgrid_size=S, kernel_size=kernel))


def test_noalloc_several_batches(need_gpu):
    """More subgrids than the scratch array holds at once (1,816 at S = 48): the call grids
    them in consecutive batches that reuse the same descriptors, partial subgrids and status
    word, and must still match the regular entry point."""
    _compare_two_calls(dict(subgrid_size=48, kernel_size=8, max_timesteps=8), min_subgrids=2 * 1816 + 1)


def test_noalloc_rejects_sizes_beyond_its_limits(need_gpu):
    obs, cd = workload("small_256", n_ant=4, nt=20, nch=4)
    c, cd = constants(cd, subgrid_size=64, kernel_size=16)
    params = c.native()
    freq = np.ascontiguousarray(obs.frequencies, np.float64)
    L = pkg._native.lib()
    st = L.p9idg_grid_w_device_noalloc(ctypes.byref(params), None, 0, None, 1, 1,
                                       freq.ctypes.data_as(ctypes.c_void_p), len(freq), None,
                                       ctypes.c_void_p(1), None)
    assert st == 8 and "subgrid size" in pkg._native.last_error()
    c, cd = constants(cd, subgrid_size=32, kernel_size=8)
    params = c.native()
    freq65 = np.linspace(1e9, 1.1e9, 65)
    st = L.p9idg_grid_w_device_noalloc(ctypes.byref(params), None, 0, None, 1, 1,
                                       freq65.ctypes.data_as(ctypes.c_void_p), 65, None, ctypes.c_void_p(1), None)
    assert st == 8 and "64 channels" in pkg._native.last_error()
