"""Device-resident entry points and plan settings the other GPU tests reach only through the
host API: IDG.Grid / DeGrid on device buffers, the deconvolver and the padded convolver on
device images, and the taper (GriddingConstants' spheroidal, identity in the reference)."""
import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_grid_degrid_device_match_host(need_gpu, mode):
    torch = pytest.importorskip("torch")
    obs, cd = workload("small_256", n_ant=8, nt=300, nch=8)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    plan = part.plan
    plan.set_mode(mode)
    N = cd["grid_size"]
    host_grid = pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies)
    d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    d_grid = torch.empty((N, N), dtype=torch.complex64, device="cuda")
    plan.grid_device(d_vis.data_ptr(), d_grid.data_ptr())
    plan.synchronize()
    assert rel_l2(d_grid.cpu().numpy(), host_grid) < 1e-6
    rng = np.random.default_rng(3)
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    host_vis = pkg.IDG.DeGrid(c, part, model.copy(), obs.uvw, obs.frequencies)
    d_model = torch.from_numpy(model.astype(np.complex64)).cuda()
    d_out = torch.empty_like(d_vis)
    plan.degrid_device(d_model.data_ptr(), d_out.data_ptr())
    plan.synchronize()
    assert rel_l2(d_out.cpu().numpy(), host_vis) < 1e-6


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_taper_scales_grid_and_visibilities(need_gpu, mode):
    """A constant taper of 0.5 halves the gridded subgrids and the degridded visibilities
    exactly (a power of two in FP32 and in the BF16 split); None restores the identity."""
    obs, cd = workload("small_256", n_ant=8, nt=300, nch=8)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    S, N = cd["subgrid_size"], cd["grid_size"]
    ref = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    vref = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    part.plan.set_taper(np.full((S, S), 0.5, np.float32))
    half = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    vhalf = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    assert rel_l2(half, 0.5 * ref) < 1e-6
    assert rel_l2(vhalf, 0.5 * vref) < 1e-6
    part.plan.set_taper(None)
    assert rel_l2(pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies), ref) < 1e-6
    assert N == cd["grid_size"]


def test_deconvolve_and_convolve_device_match_host(need_gpu):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    n, p = 128, 32
    yy, xx = np.mgrid[:p, :p] - p // 2
    psf = (np.exp(-(yy ** 2 + xx ** 2) / 20.0) + 0.01 * rng.standard_normal((p, p))).astype(np.float32)
    g0 = (rng.standard_normal((n, n)) * 10).astype(np.float32)
    cd = pkg.FastSerialCD(pkg.Rectangle(0, 0, n, n), psf)
    xh, gh = np.zeros((n, n), np.float32), g0.copy()
    rh = cd.Deconvolve(xh, gh, 0.5, 0.2, 200, 1e-6)
    d_x = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    d_g = torch.from_numpy(g0.copy()).cuda()
    rd = cd.deconvolve_device(d_x.data_ptr(), d_g.data_ptr(), 0.5, 0.2, 200, 1e-6)
    torch.cuda.synchronize()
    assert rd.IterationCount == rh.IterationCount and rd.Converged == rh.Converged
    assert np.array_equal(d_x.cpu().numpy(), xh) and np.array_equal(d_g.cpu().numpy(), gh)
    conv = pkg.PaddedConvolver.correlation(psf, pkg.Rectangle(0, 0, n, n))
    img = rng.standard_normal((n, n)).astype(np.float32)
    host = conv.Convolve(img)
    d_img = torch.from_numpy(img).cuda()
    d_out = torch.empty((n, n), dtype=torch.float32, device="cuda")
    conv.convolve_device(d_img.data_ptr(), n, d_out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), host)


def test_psf_max_lipschitz_matches_the_deconvolver(need_gpu):
    """PSF.CalcMaxLipschitz on the host equals what FastSerialCD computes on the device."""
    rng = np.random.default_rng(5)
    psf = rng.standard_normal((24, 24)).astype(np.float32)
    cd = pkg.FastSerialCD(pkg.Rectangle(0, 0, 64, 64), psf)
    # the deconvolver keeps it as a float, as FastSerialCD's field is
    assert cd.MaxLipschitz == float(np.float32(pkg.PSF.CalcMaxLipschitz(psf)))
