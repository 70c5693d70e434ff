"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Bar (FP32 kernels): relative L2 error <= 1e-5 against the oracle for grids, visibilities
and images; exact known answers to 1e-5; adjoint identities to FP32 rounding (1e-5).
"""
import numpy as np
import pytest

from conftest import C_LIGHT, constants, kat_constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu
TOL = 1e-5

CASES = [("small_256", dict(n_ant=10, nt=400, nch=8)),
         ("meerkat_3072", dict(n_ant=10, nt=300, nch=16))]


def _setup(name, kw, **over):
    obs, cd = workload(name, **kw)
    c, cd = constants(cd, **over)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    return obs, c, cd, part, subs


def _model_grid(obs):
    return oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))


@pytest.mark.parametrize("name,kw", CASES)
def test_grid_w(need_gpu, name, kw):
    obs, c, cd, part, subs = _setup(name, kw)
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert got.shape == ref.shape
    assert rel_l2(got, ref) < TOL


@pytest.mark.parametrize("name,kw", CASES)
def test_degrid_w_and_in_place_shift(need_gpu, name, kw):
    obs, c, cd, part, subs = _setup(name, kw)
    model = _model_grid(obs)
    grid_io = model.copy()
    got = pkg.IDG.DeGridW(c, part, grid_io, obs.uvw, obs.frequencies)
    ref, shifted = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(got, ref) < TOL
    # IDG.DeGridW shifts the caller's grid in place (IDG.cs:44)
    assert np.array_equal(grid_io, shifted)
    # samples the partitioner dropped stay exactly zero
    covered = np.zeros(obs.vis.shape[:2], bool)
    for s in subs:
        covered[s["baseline_idx"], s["time_sample_start"]:s["time_sample_start"] + s["time_sample_count"]] = True
    assert np.all(got[~covered] == 0)


def test_grid_and_degrid_non_w(need_gpu):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=10, nt=400, nch=8))
    got = pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL
    model = _model_grid(obs)
    got_v = pkg.IDG.DeGrid(c, part, model.copy(), obs.uvw, obs.frequencies)
    ref_v, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies)
    assert rel_l2(got_v, ref_v) < TOL


def test_psf_and_images(need_gpu):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=10, nt=400, nch=8))
    flags = np.random.default_rng(5).random(obs.vis.shape) < 0.1
    unit = oracle.unit_vis(flags)
    g_ref = oracle.idg_grid(cd, subs, unit, obs.uvw, obs.frequencies)
    assert rel_l2(pkg.IDG.GridPSF(c, part, obs.uvw, flags, obs.frequencies), g_ref) < TOL
    psf_ref = oracle.shift(oracle.fft_backward_real(g_ref, cd["vis_count"]))
    assert rel_l2(pkg.IDG.CalculatePSF(c, part, obs.uvw, flags, obs.frequencies), psf_ref) < TOL
    img_ref = oracle.shift(oracle.fft_backward_real(
        oracle.idg_grid(cd, subs, obs.vis, obs.uvw, obs.frequencies), cd["vis_count"]))
    assert rel_l2(pkg.IDG.ToImage(c, part, obs.vis, obs.uvw, obs.frequencies), img_ref) < TOL


def test_fft_members(need_gpu):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=10, nt=400, nch=8))
    layers = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(pkg.FFT.WStackIFFTFloat(layers, cd["vis_count"]),
                  oracle.wstack_ifft_float(layers, cd["vis_count"])) < TOL
    img = obs.model_image.astype(np.float32)
    assert rel_l2(pkg.FFT.Forward(img, 2.0), oracle.fft_forward_float(img, 2.0)) < TOL
    g = oracle.fft_forward_float(img)
    back = pkg.FFT.BackwardFloat(g, g.size)
    assert rel_l2(back, img) < TOL


@pytest.mark.parametrize("pu,pv", [(0, 0), (3, -5), (11, 9)])
def test_known_answer_unit_delta(need_gpu, pu, pv):
    cd = kat_constants()
    c = pkg.GriddingConstants.from_dict(cd)
    uvw = np.array([[[pu, pv, 0.0]]])
    freq = np.array([C_LIGHT])
    part = pkg.Partitioner.CreatePartition(c, uvw, freq)
    g = pkg.IDG.Grid(c, part, np.ones((1, 1, 1), np.complex128), uvw, freq)
    N = cd["grid_size"]
    expect = np.zeros((N, N), np.complex128)
    expect[pv % N, pu % N] = 1.0
    assert np.abs(g - expect).max() < 1e-5
    v = pkg.IDG.DeGrid(c, part, expect.copy(), uvw, freq)
    assert abs(v[0, 0, 0] - 1.0) < 1e-5


@pytest.mark.parametrize("S", [8, 16, 24, 48])
def test_subgrid_sizes(need_gpu, S):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=8, nt=200, nch=4), subgrid_size=S,
                                    kernel_size=max(2, S // 4))
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL
    model = _model_grid(obs)
    gv = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    rv, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(gv, rv) < TOL


def test_odd_grid_size(need_gpu):
    """FFT.Shift on odd N swaps only the leading 2*(N/2) square (FFT.cs:248-264)."""
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=8, nt=200, nch=4), grid_size=255)
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL
    model = oracle.fft_forward_float(obs.model_image[:255, :255].astype(np.float32))
    gv = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    rv, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(gv, rv) < TOL


def test_device_api_matches_host_api(need_gpu):
    torch = pytest.importorskip("torch")
    obs, c, cd, part, subs = _setup("meerkat_3072", dict(n_ant=10, nt=300, nch=16))
    plan = part.plan
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    N, W = cd["grid_size"], cd["wlayer_count"]
    d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    d_layers = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
    plan.grid_w_device(d_vis.data_ptr(), d_layers.data_ptr())
    plan.synchronize()
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(d_layers.cpu().numpy(), ref) < TOL
    model = _model_grid(obs)
    d_grid = torch.from_numpy(model.astype(np.complex64)).cuda()
    d_out = torch.empty_like(d_vis)
    plan.degrid_w_device(d_grid.data_ptr(), d_out.data_ptr())
    plan.synchronize()
    ref_v, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(d_out.cpu().numpy(), ref_v) < TOL
    # the device grid is not modified (the shift is folded into the splitter)
    assert torch.equal(d_grid.cpu(), torch.from_numpy(model.astype(np.complex64)))
    d_img = torch.empty((N, N), dtype=torch.float32, device="cuda")
    plan.wstack_image_device(d_layers.data_ptr(), d_img.data_ptr(), True)
    plan.synchronize()
    img_ref = oracle.shift(oracle.wstack_ifft_float(ref, cd["vis_count"]))
    assert rel_l2(d_img.cpu().numpy(), img_ref) < TOL
    plan.set_stream(0)


@pytest.mark.parametrize("mode,tol", [(pkg.MODE_FP32, TOL), (pkg.MODE_TC_BF16X3, 1e-4)], ids=["fp32", "tc_bf16x3"])
def test_device_outputs_fully_written(need_gpu, mode, tol):
    """The device entry points write every element of their outputs, which start as NaN here: the
    w layers are zero-filled beside the gridder, and the visibilities no subgrid covers (quirk P1
    drops 18 % of this observation's samples) beside the degridder, which writes all the others.
    The layers start 8 bytes past a 16-byte boundary and hold an odd number of elements (N = 3071),
    so the fill's single first and last words are exercised too."""
    torch = pytest.importorskip("torch")
    obs, c, cd, part, subs = _setup("meerkat_3072", dict(n_ant=10, nt=300, nch=16), grid_size=3071)
    plan = part.plan
    assert plan.set_mode(mode) == mode
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    N, W = cd["grid_size"], cd["wlayer_count"]
    nan = complex(float("nan"), float("nan"))
    d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    buf = torch.full((W * N * N + 1,), nan, dtype=torch.complex64, device="cuda")
    d_layers = buf[1:]
    assert d_layers.data_ptr() % 16 == 8
    plan.grid_w_device(d_vis.data_ptr(), d_layers.data_ptr())
    plan.synchronize()
    layers = d_layers.cpu().numpy().reshape(W, N, N)
    assert np.isfinite(layers).all() and np.isnan(buf[0].item().real)  # the word before is untouched
    assert rel_l2(layers, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < tol
    model = oracle.fft_forward_float(obs.model_image[:N, :N].astype(np.float32))
    d_grid = torch.from_numpy(model.astype(np.complex64)).cuda()
    d_out = torch.full_like(d_vis, nan)
    plan.degrid_w_device(d_grid.data_ptr(), d_out.data_ptr())
    plan.synchronize()
    out = d_out.cpu().numpy()
    covered = np.zeros(obs.vis.shape[:2], bool)
    for s in subs:
        covered[s["baseline_idx"], s["time_sample_start"]:s["time_sample_start"] + s["time_sample_count"]] = True
    assert (~covered).any() and np.isfinite(out).all()
    assert not out[~covered].any()
    ref_v, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(out, ref_v) < tol
    plan.set_stream(0)


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_uvw_kept_on_the_device(need_gpu, mode):
    """uvw=None (NULL in the C ABI): the uvw the partition was made from, which the plan keeps on
    the device.  The same results as passing it, also after a call with another uvw in between
    (that call's uvw replaces the device copy; the next None call puts the plan's back)."""
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=8, nt=300, nch=8))
    assert part.plan.set_mode(mode) == mode
    model = _model_grid(obs)
    lay = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    other = obs.uvw.copy()
    other[..., 2] *= 0.5
    tol = TOL if mode == pkg.MODE_FP32 else 1e-4
    for step in range(2):
        assert rel_l2(pkg.IDG.GridW(c, part, obs.vis, None, obs.frequencies), lay) < 1e-6
        assert np.array_equal(pkg.IDG.DeGridW(c, part, model.copy(), None, obs.frequencies), vis)
        lay_o = pkg.IDG.GridW(c, part, obs.vis, other, obs.frequencies)
        assert rel_l2(lay_o, oracle.idg_grid_w(cd, subs, obs.vis, other, obs.frequencies)) < tol
    assert rel_l2(lay, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < tol
    with pytest.raises(ValueError):
        pkg.IDG.GridW(c, [list(x) for x in part], obs.vis, None, obs.frequencies)


def test_adjoint_identity_gpu(need_gpu):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=10, nt=400, nch=8))
    rng = np.random.default_rng(4)
    N = cd["grid_size"]
    g = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    Gv = pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies)
    Dg = pkg.IDG.DeGrid(c, part, g.copy(), obs.uvw, obs.frequencies)
    lhs, rhs = np.vdot(Gv, g), np.vdot(obs.vis, Dg)
    assert abs(lhs - rhs) / abs(lhs) < TOL


def test_empty_plan_and_stage_timing(need_gpu):
    cd = kat_constants()
    c = pkg.GriddingConstants.from_dict(cd)
    uvw = np.zeros((2, 0, 3))
    freq = np.array([C_LIGHT])
    part = pkg.Partitioner.CreatePartition(c, uvw, freq)
    layers = pkg.IDG.GridW(c, part, np.zeros((2, 0, 1), np.complex128), uvw, freq)
    assert layers.shape == (1, 64, 64) and not layers.any()
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=6, nt=100, nch=4))
    part.plan.enable_timing(True)
    pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    t = part.plan.stage_times()
    # one gridder + adder pass; with host arrays used in place, one for the other w layers and one
    # per row band (up to 4) of the busiest layer
    n = t["gridder"][1]
    assert 1 <= n <= 5 and t["gridder"][0] > 0 and t["subgrid_ifft_add"][1] == n


def test_sincos_probe(need_gpu):
    s, f = pkg.measure_sincos_peak()
    assert s > 1e11 and f > 1e12
