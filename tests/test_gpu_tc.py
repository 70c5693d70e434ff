"""Tensor-core split-precision gridder/degridder (P9IDG_MODE_TC_BF16X3 / _FP16X3).

Bar: relative L2 error <= 1e-4 against the FP64 oracle (the bound stated for the
tensor-core form), for grids, degridded visibilities and the dirty image.  The GEMM
self-test pins the tcgen05 operand layout, descriptors and TMEM read-out with exactly
representable inputs (error at FP32 accumulation level).
"""
import ctypes

import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu
TOL_TC = 1e-4
MODES = [pytest.param(pkg.MODE_TC_BF16X3, id="bf16x3"), pytest.param(pkg.MODE_TC_FP16X3, id="fp16x3")]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n", [32, 64, 128])
def test_tcgen05_gemm_selftest(need_gpu, mode, n):
    err = ctypes.c_double(-1)
    st = pkg._native.lib().p9idg_tc_selftest(mode, n, ctypes.byref(err))
    assert st == 0, pkg._native.last_error()
    assert 0 <= err.value < 1e-6


def _setup(name, kw, mode):
    obs, cd = workload(name, **kw)
    c, cd = constants(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    return obs, c, cd, part, subs


CASES = [("meerkat_3072", dict(n_ant=10, nt=300, nch=16)), ("small_256", dict(n_ant=8, nt=300, nch=8))]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name,kw", CASES)
def test_tc_grid_w(need_gpu, mode, name, kw):
    obs, c, cd, part, subs = _setup(name, kw, mode)
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL_TC
    img = pkg.FFT.WStackIFFTFloat(got, cd["vis_count"])
    assert rel_l2(img, oracle.wstack_ifft_float(ref, cd["vis_count"])) < TOL_TC


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name,kw", CASES)
def test_tc_degrid_w(need_gpu, mode, name, kw):
    obs, c, cd, part, subs = _setup(name, kw, mode)
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    got = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    ref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(got, ref) < TOL_TC


def test_tc_non_w_and_psf(need_gpu):
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=8, nt=300, nch=8), pkg.MODE_TC_BF16X3)
    assert rel_l2(pkg.IDG.Grid(c, part, obs.vis, obs.uvw, obs.frequencies),
                  oracle.idg_grid(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < TOL_TC
    flags = np.zeros(obs.vis.shape, bool)
    g_ref = oracle.idg_grid(cd, subs, oracle.unit_vis(flags), obs.uvw, obs.frequencies)
    psf_ref = oracle.shift(oracle.fft_backward_real(g_ref, cd["vis_count"]))
    assert rel_l2(pkg.IDG.CalculatePSF(c, part, obs.uvw, flags, obs.frequencies), psf_ref) < TOL_TC


def test_tc_rejects_other_subgrid_sizes():
    obs, cd = workload("small_256", n_ant=4, nt=50, nch=4)
    c, cd = constants(cd, subgrid_size=48, kernel_size=8)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    with pytest.raises(pkg.P9IDGError) as e:
        part.plan.set_mode(pkg.MODE_TC_BF16X3)
    assert e.value.code == 8


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("S", [8, 16, 24])
def test_tc_smaller_subgrids(need_gpu, mode, S):
    """Subgrids of S < 32 pixels run padded to the kernels' 32 operand rows (the padding rows and
    columns are computed and never written, the padded pixels of the degridder's input are zero):
    the same bound as S = 32 for w layers, degridded visibilities and the dirty image."""
    obs, cd = workload("small_256", n_ant=8, nt=300, nch=8)
    c, cd = constants(cd, subgrid_size=S, kernel_size=max(2, S // 4))
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, ref) < TOL_TC
    img = pkg.FFT.WStackIFFTFloat(got, cd["vis_count"])
    assert rel_l2(img, oracle.wstack_ifft_float(ref, cd["vis_count"])) < TOL_TC
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    vref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(vis, vref) < TOL_TC


EDGE_SHAPES = [
    (1, 37, 256, None),       # one channel: work items far from a multiple of the 32 / 128 tiles
    (3, 301, 255, None),      # odd grid size, odd channel count
    (16, 120, 512, (2048, 2048)),  # small work items: several partial subgrids per subgrid
]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("nch,nt,N,chunks", EDGE_SHAPES)
def test_tc_edge_shapes(need_gpu, mode, nch, nt, N, chunks):
    obs, cd = workload("small_256", n_ant=9, nt=nt, nch=nch, seed=nch * 100 + nt)
    c, cd = constants(cd, grid_size=N)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    if chunks:
        pkg.set_chunking(part.plan, *chunks)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert len(subs) > 0
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < TOL_TC
    rng = np.random.default_rng(N)
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))  # the plan's grid size
    vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    ref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(vis, ref) < TOL_TC


SMALL_S_EDGE_SHAPES = [
    (16, 4, 1, 37, 255, None),        # odd grid size, one channel
    (24, 8, 3, 301, 256, (384, 384)),    # several partial subgrids per subgrid
    (8, 2, 5, 120, 129, None),        # odd grid size, subgrids of 8 pixels
]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("S,kernel,nch,nt,N,chunks", SMALL_S_EDGE_SHAPES)
def test_tc_smaller_subgrid_edge_shapes(need_gpu, mode, S, kernel, nch, nt, N, chunks):
    """The padded small-subgrid path on the edge shapes: odd grid sizes (the FFT.Shift keeps the
    last row and column), one channel, and work items split across a subgrid."""
    obs, cd = workload("small_256", n_ant=9, nt=nt, nch=nch, seed=nch * 100 + nt + S)
    c, cd = constants(cd, grid_size=N, subgrid_size=S, kernel_size=kernel)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    if chunks:
        pkg.set_chunking(part.plan, *chunks)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert len(subs) > 0
    got = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(got, oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)) < TOL_TC
    rng = np.random.default_rng(N + S)
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    ref, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(vis, ref) < TOL_TC


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("nch,nt,N,chunks", EDGE_SHAPES)
def test_tc_edge_shapes_device(need_gpu, mode, nch, nt, N, chunks):
    """The same shapes through the device API with complex64 visibilities, the single-plan path
    that stages inputs with TMA: a stage's visibility tile starts at the even index at or below
    its first sample, and the samples past a work item's end (the next item's) weigh nothing."""
    torch = pytest.importorskip("torch")
    obs, cd = workload("small_256", n_ant=9, nt=nt, nch=nch, seed=nch * 100 + nt)
    c, cd = constants(cd, grid_size=N)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    plan = part.plan
    plan.set_mode(mode)
    if chunks:
        pkg.set_chunking(plan, *chunks)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    W = cd["wlayer_count"]
    d_vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    d_layers = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
    plan.grid_w_device(d_vis.data_ptr(), d_layers.data_ptr())
    plan.synchronize()
    ref = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    assert rel_l2(d_layers.cpu().numpy(), ref) < TOL_TC
    rng = np.random.default_rng(N)
    model = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    d_grid = torch.from_numpy(model.astype(np.complex64)).cuda()
    d_out = torch.empty_like(d_vis)
    plan.degrid_w_device(d_grid.data_ptr(), d_out.data_ptr())
    plan.synchronize()
    ref_v, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    assert rel_l2(d_out.cpu().numpy(), ref_v) < TOL_TC


@pytest.mark.parametrize("mode", MODES)
def test_tc_unit_delta_known_answer(need_gpu, mode):
    """The hand-derived known answer of the FP32 path (a unit visibility at integer uv pixel p
    grids to 1 at grid[p]) holds for the tensor-core path to its stated bound."""
    from conftest import C_LIGHT, kat_constants
    for pu, pv in [(0, 0), (3, -5), (11, 9)]:
        cd = kat_constants(N=128, S=32, kernel=8)
        c, cd = constants(cd)
        uvw = np.array([[[pu, pv, 0.0]]], np.float64)
        freq = np.array([C_LIGHT])
        part = pkg.Partitioner.CreatePartition(c, uvw, freq)
        part.plan.set_mode(mode)
        g = pkg.IDG.Grid(c, part, np.ones((1, 1, 1), np.complex128), uvw, freq)
        expect = np.zeros_like(g)
        expect[pv % 128, pu % 128] = 1.0
        assert np.abs(g - expect).max() < 1e-4


def test_tc_coefficients_follow_uvw_between_calls(need_gpu):
    """Host calls upload uvw every time; the tensor-core coefficients are recomputed exactly when
    the upload differs from the one they were made from (compared on the device).  A changed uvw
    (same partition) must give the oracle's result for that uvw, and changing back the first."""
    obs, c, cd, part, subs = _setup("small_256", dict(n_ant=8, nt=300, nch=8), pkg.MODE_TC_BF16X3)
    uvw_b = obs.uvw * 1.0002
    ref_a = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    ref_b = oracle.idg_grid_w(cd, subs, obs.vis, uvw_b, obs.frequencies)
    assert rel_l2(ref_b, ref_a) > 1e-3  # the change is visible at the tolerance used below
    for uvw, ref in [(obs.uvw, ref_a), (obs.uvw.copy(), ref_a), (uvw_b, ref_b), (uvw_b.copy(), ref_b),
                     (obs.uvw, ref_a)]:
        got = pkg.IDG.GridW(c, part, obs.vis, uvw, obs.frequencies)
        assert rel_l2(got, ref) < TOL_TC
        model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
        vis = pkg.IDG.DeGridW(c, part, model.copy(), uvw, obs.frequencies)
        vref, _ = oracle.idg_degrid(cd, subs, model, uvw, obs.frequencies, wstack=True)
        assert rel_l2(vis, vref) < TOL_TC
