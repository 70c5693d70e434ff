"""The 3072^2 workload at full size (2016 baselines x 2000 times x 16 channels, 8 w layers).

The FP64 oracle cannot grid 42M visibilities in test time, so full size is checked by
(a) exact FP64 per-subgrid sums on a seeded subset of subgrids (>= 10k visibilities)
gridded from the full-size arrays, (b) linearity, and (c) the real-inner-product adjoint
identity of GridW/DeGridW over every interior subgrid.
"""
import functools

import numpy as np
import pytest

from conftest import oracle, pkg, rel_l2, synth

pytestmark = pytest.mark.gpu
TOL = 1e-5


@functools.lru_cache(maxsize=1)
def full():
    obs, cd = synth.build("meerkat_3072")
    c = pkg.GriddingConstants.from_dict(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    return obs, cd, c, part


def _subset(subs, n_vis_min, seed, nch):
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(subs))
    take, tot = [], 0
    for i in idx:
        take.append(i)
        tot += int(subs[i]["time_sample_count"]) * nch
        if tot >= n_vis_min:
            break
    return np.sort(np.array(take))


@pytest.mark.parametrize("mode,tol,n_vis", [(pkg.MODE_FP32, TOL, 10_000), (pkg.MODE_TC_BF16X3, 1e-4, 100_000),
                                            (pkg.MODE_TC_FP16X3, 1e-4, 100_000)], ids=["fp32", "tc_bf16x3", "tc_fp16x3"])
def test_fullsize_subset_against_fp64(need_gpu, mode, tol, n_vis):
    """Seeded subgrids of the full-size plan, gridded from the full-size arrays, against the FP64
    oracle: FP32 at 1e-5, the tensor-core forms at their 1e-4 bound on >= 100k visibilities."""
    obs, cd, c, part = full()
    subs = part.plan.subgrids()
    sel = subs[_subset(subs, n_vis, 1, obs.vis.shape[2])]
    sub_plan = pkg.plan_from_subgrids(c, sel, obs.uvw, obs.frequencies)
    assert sub_plan.set_mode(mode) == mode
    sub_part = pkg.Partition([[]], sub_plan)
    got = pkg.IDG.GridW(c, sub_part, obs.vis, obs.uvw, obs.frequencies)
    ref = oracle.idg_grid_w(cd, sel, obs.vis, obs.uvw, obs.frequencies)
    e_grid = rel_l2(got, ref)
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    gv = pkg.IDG.DeGridW(c, sub_part, model.copy(), obs.uvw, obs.frequencies)
    rv, _ = oracle.idg_degrid(cd, sel, model, obs.uvw, obs.frequencies, wstack=True)
    e_vis = rel_l2(gv, rv)
    print(f"3072^2 subset ({int(sel['time_sample_count'].sum()) * obs.vis.shape[2]} vis), mode {mode}: "
          f"GridW {e_grid:.2e}, DeGridW {e_vis:.2e}")
    assert e_grid < tol and e_vis < tol


def test_fullsize_linearity_and_adjoint(need_gpu):
    torch = pytest.importorskip("torch")
    obs, cd, c, part = full()
    N, S, W = cd["grid_size"], cd["subgrid_size"], cd["wlayer_count"]
    subs = part.plan.subgrids()
    # interior subgrids: Add and Split use different edge tests for negative w (AdderWStack.cs:47 vs :220)
    u, v = subs["u_pixel"], subs["v_pixel"]
    interior = (u >= 2) & (u < N - S - 1) & (v >= 2) & (v < N - S - 1)
    plan = pkg.plan_from_subgrids(c, subs[interior], obs.uvw, obs.frequencies)
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    vis = torch.from_numpy(obs.vis.astype(np.complex64)).cuda()
    L1 = torch.empty((W, N, N), dtype=torch.complex64, device="cuda")
    L2 = torch.empty_like(L1)
    plan.grid_w_device(vis.data_ptr(), L1.data_ptr())
    vis2 = vis * 2.0
    plan.grid_w_device(vis2.data_ptr(), L2.data_ptr())
    plan.synchronize()
    assert float(torch.linalg.vector_norm(L2 - 2 * L1) / torch.linalg.vector_norm(2 * L1)) < 1e-6
    g = torch.randn((N, N), dtype=torch.complex64, device="cuda", generator=torch.Generator("cuda").manual_seed(3))
    Dg = torch.empty_like(vis)
    plan.degrid_w_device(g.data_ptr(), Dg.data_ptr())
    plan.synchronize()
    # GridW shifts its output and DeGridW its input; FFT.Shift is a symmetric permutation, so
    # Re<Shift(A v), g> = Re<v, A^H Shift(g)> pairs the layer sum with the unshifted g
    Lsum = L1.sum(0).cpu().numpy().astype(np.complex128)
    lhs = np.vdot(Lsum, g.cpu().numpy().astype(np.complex128)).real
    rhs = np.vdot(obs.vis, Dg.cpu().numpy().astype(np.complex128)).real
    # Both inner products are accumulated in FP64 from the FP32 kernels' outputs, whose error
    # against FP64 is ~1e-6 relative (GridW 3.5e-7, DeGridW 1.0e-6 measured on this workload).
    # The operands' errors are uncorrelated with g and the visibilities, so each inner product
    # carries a relative error of the same order, not sqrt(#terms) more: 1e-5 leaves a 10x margin.
    err = abs(lhs - rhs) / abs(lhs)
    print(f"3072^2 adjoint identity: relative difference {err:.2e}")
    assert err < 1e-5
    plan.set_stream(0)


@pytest.mark.parametrize("mode,tol", [(pkg.MODE_FP32, TOL), (pkg.MODE_TC_BF16X3, 1e-4)], ids=["fp32", "tc_bf16x3"])
def test_config1_full_size_against_fp64(need_gpu, mode, tol):
    """The 256^2 workload (30 antennas, 1440 times, 8 channels: 5.0 M visibilities) at full size
    against the FP64 oracle: w-stacked grid, degridded visibilities and the dirty image."""
    obs, cd = synth.build("small_256")
    c = pkg.GriddingConstants.from_dict(cd)
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    subs = part.plan.subgrids()
    layers = pkg.IDG.GridW(c, part, obs.vis, obs.uvw, obs.frequencies)
    ref_layers = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    e_grid = rel_l2(layers, ref_layers)
    e_img = rel_l2(pkg.FFT.WStackIFFTFloat(layers, cd["vis_count"]),
                   oracle.wstack_ifft_float(ref_layers, cd["vis_count"]))
    model = oracle.fft_forward_float(oracle.shift(obs.model_image.astype(np.float32)))
    vis = pkg.IDG.DeGridW(c, part, model.copy(), obs.uvw, obs.frequencies)
    ref_vis, _ = oracle.idg_degrid(cd, subs, model, obs.uvw, obs.frequencies, wstack=True)
    e_vis = rel_l2(vis, ref_vis)
    print(f"config-1 full size, mode {mode}: GridW {e_grid:.2e}, dirty image {e_img:.2e}, DeGridW {e_vis:.2e}")
    assert e_grid < tol and e_img < tol and e_vis < tol
