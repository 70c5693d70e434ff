"""Order independence of the adder, and the kernels' own bounds checks.

* Order independence.  Overlapping subgrids meet in FP32 atomics in the adder, so the order in
  which subgrids (and gridder work items) are processed changes only the rounding of the sums.
  The reference adds subgrids one after another (AdderWStack.cs:11-78); a plan built from the
  same subgrids in another order must give the same w layers within FP32 rounding, and the same
  degridded visibilities bit for bit (each visibility is evaluated once, by one thread).
* Bounds checks.  p9idg_grid_w_device_noalloc takes its subgrid list in device memory and so
  cannot check it on the host: the gridder kernel checks each subgrid's baseline and sample
  range before reading uvw/vis, the adder checks its w layer before writing; a failed check
  skips the access, sets the status word, and the call returns P9IDG_DEVICE_CHECK_FAILED.  A
  subgrid placed outside the grid is skipped without a status, as AdderWStack.Add skips it
  (AdderWStack.cs:47-48).  Every case here is caught by those checks before any access.
"""
import ctypes

import numpy as np
import pytest

from conftest import constants, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu
MODES = [pytest.param(pkg.MODE_FP32, id="fp32"), pytest.param(pkg.MODE_TC_BF16X3, id="tc_bf16x3")]
DEVICE_CHECK_FAILED = 9


@pytest.mark.parametrize("mode", MODES)
def test_subgrid_order_changes_only_rounding(need_gpu, mode):
    obs, cd = workload("meerkat_3072", n_ant=10, nt=300, nch=16)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    subs = part.plan.subgrids()
    rng = np.random.default_rng(3)
    orders = {"reversed": subs[::-1].copy(), "shuffled": subs[rng.permutation(len(subs))].copy()}
    part.plan.set_mode(mode)
    ref = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    N = cd["grid_size"]
    model = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)))
    vref = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    for name, arr in orders.items():
        plan = pkg.plan_from_subgrids(c, arr, obs.uvw, obs.frequencies)
        assert plan.set_mode(mode) == mode
        other = pkg.Partition.from_array(plan.subgrids(), obs.uvw.shape[0], plan)
        got = pkg.IDG.GridW(c, other, obs.vis, obs.uvw, obs.frequencies)
        err = rel_l2(got, ref)
        print(f"{name} order, mode {mode}: w layers differ by rel-L2 {err:.2e}")
        assert err < 1e-6
        vis = pkg.IDG.DeGridW(c, other, model.copy(), obs.uvw, obs.frequencies)
        assert np.array_equal(vis, vref)
        plan.destroy()


def _noalloc(c, d_subs, nsub, d_uvw, uvw_shape, freq, d_vis, out, stream):
    L = pkg._native.lib()
    params = c.native()
    return L.p9idg_grid_w_device_noalloc(ctypes.byref(params), ctypes.c_void_p(d_subs), nsub,
                                         ctypes.c_void_p(d_uvw), uvw_shape[0], uvw_shape[1],
                                         freq.ctypes.data_as(ctypes.c_void_p), len(freq), ctypes.c_void_p(d_vis),
                                         ctypes.c_void_p(out), ctypes.c_void_p(stream))


def test_noalloc_bounds_checks(need_gpu):
    torch = pytest.importorskip("torch")
    obs, cd = workload("small_256", n_ant=8, nt=200, nch=4)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    subs = part.plan.subgrids()
    nbl, nt = obs.uvw.shape[:2]
    N, W = cd["grid_size"], cd["wlayer_count"]
    stream = torch.cuda.current_stream()
    d_uvw = torch.from_numpy(obs.uvw).cuda()
    d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    freq = np.ascontiguousarray(obs.frequencies, np.float64)
    out = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")

    def call(arr):
        d = torch.from_numpy(np.ascontiguousarray(arr, pkg.SUBGRID_DTYPE).view(np.int32).reshape(-1, 6).copy()).cuda()
        st = _noalloc(c, d.data_ptr(), len(arr), d_uvw.data_ptr(), obs.uvw.shape, freq, d_vis.data_ptr(),
                      out.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        return st, out.cpu().numpy()

    st, good = call(subs)
    assert st == 0, pkg._native.last_error()
    bad_fields = {
        "baseline past the last": ("baseline_idx", nbl),
        "negative baseline": ("baseline_idx", -1),
        "samples past the track": ("time_sample_start", nt - 1),
        "negative sample count": ("time_sample_count", -5),
        "w layer past the stack": ("w_lambda", W),
        "negative w beyond the stack": ("w_lambda", -W - 1),
    }
    S = cd["subgrid_size"]
    # a subgrid whose mirrored position (negative w) is inside the grid too, so that the w check,
    # not the grid-range skip, is what stops it
    inner = (subs["u_pixel"] >= 2) & (subs["u_pixel"] <= N - S - 2) & (subs["v_pixel"] >= 2) & \
            (subs["v_pixel"] <= N - S - 2) & (subs["time_sample_count"] > 0)
    k = int(np.flatnonzero(inner)[0])
    for name, (field, value) in bad_fields.items():
        arr = subs.copy()
        arr[k][field] = value
        if field == "time_sample_start":
            arr[k]["time_sample_count"] = 2  # samples nt-1 and nt: one past the end
        st, _ = call(arr)
        assert st == DEVICE_CHECK_FAILED, (name, st)
        assert "outside" in pkg._native.last_error()
        # the next call on the same scratch array is right again
        st, again = call(subs)
        assert st == 0 and rel_l2(again, good) < 1e-6, name
    # off the grid: skipped without a status, as AdderWStack.Add skips it; the rest is gridded
    arr = subs.copy()
    arr[k]["u_pixel"] = N
    st, got = call(arr)
    assert st == 0
    keep = np.ones(len(subs), bool)
    keep[k] = False
    st, ref = call(subs[keep])
    assert st == 0 and rel_l2(got, ref) < 1e-6
