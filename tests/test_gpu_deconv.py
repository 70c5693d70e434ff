"""GPU parity of the deconvolution side of the serial major cycle against the oracle.

FastSerialCD on the GPU must reproduce the oracle's coordinate descent bit for bit (pixel
sequence, values, gradients, iteration count) when both start from the same float32 inputs;
the PSF^2 map comes from FP64 FFTs on both sides (cuFFT vs the oracle's FFT) and agrees to
float rounding; the Lipschitz map is bit-identical (same double scan, same QueryScan sums).
The whole major cycle runs with the FP32 (and tensor-core) gridder on complex64 data, so it is
compared with the FP64 oracle within stated tolerances.
"""
import numpy as np
import pytest

from conftest import constants, oracle, pkg, rel_l2, workload

pytestmark = pytest.mark.gpu


def _problem(n, p, seed, nonneg=False):
    rng = np.random.default_rng(seed)
    psf = (rng.standard_normal((p, p)) * 0.05).astype(np.float32)
    psf[p // 2, p // 2] = 1.0
    x = np.zeros((n, n), np.float32)
    k = max(1, n // 16)
    x[rng.integers(0, n, k), rng.integers(0, n, k)] = rng.random(k).astype(np.float32)
    g = (rng.standard_normal((n, n)) * 2).astype(np.float32)
    return psf, x, g


def _cd(n, psf):
    return pkg.FastSerialCD(pkg.Rectangle(0, 0, n, n), psf)


@pytest.mark.parametrize("n,p", [(64, 8), (200, 24), (256, 64), (96, 96), (130, 10)])
def test_maps_match_oracle(need_gpu, n, p):
    psf, _, _ = _problem(n, p, seed=n + p)
    cd = _cd(n, psf)
    psf2, amap = cd.maps()
    opsf2 = oracle.psf_squared(psf)
    assert psf2.shape == (2 * p, 2 * p)
    assert np.abs(psf2 - opsf2).max() <= 2e-7 * np.abs(opsf2).max()
    assert np.array_equal(amap, oracle.amap(psf, (n, n)))
    assert cd.MaxLipschitz == pytest.approx(float(opsf2.max()), rel=1e-6)
    cd.destroy()


@pytest.mark.parametrize("n,p,lam,alpha,iters,eps", [
    (64, 8, 0.4, 0.2, 300, 1e-5),
    (200, 24, 1.0, 0.05, 500, 1e-5),     # image not a multiple of the 128-pixel tile width
    (256, 64, 0.5, 0.2, 400, 1e-6),      # window spans several tiles in both directions
    (96, 96, 0.5, 0.2, 300, 1e-5),       # full PSF: the window covers the whole image
    (512, 16, 0.2, 0.1, 1500, 1e-7),     # many graph replays
])
def test_deconvolve_bit_exact_vs_oracle(need_gpu, n, p, lam, alpha, iters, eps):
    psf, x0, g0 = _problem(n, p, seed=n * 7 + p)
    cd = _cd(n, psf)
    psf2, amap = cd.maps()
    ox, og, oconv, oit = oracle.deconvolve(x0, g0, amap, psf2, lam, alpha, iters, eps)
    x, g = x0.copy(), g0.copy()
    r = cd.Deconvolve(x, g, lam, alpha, iters, eps)
    assert (r.Converged, r.IterationCount) == (oconv, oit)
    assert oit > 0
    assert x.tobytes() == ox.tobytes()
    assert g.tobytes() == og.tobytes()
    cd.destroy()


def test_deconvolve_bit_exact_with_windows_inside_the_image(need_gpu):
    """A 1024^2 gradient map that peaks near the centre and a 160^2 PSF: the 320^2 update
    windows lie inside the image and span whole rows and columns of tiles, as on a real sky in
    the major cycle (the other cases mostly clip their windows at the image edges)."""
    n, p = 1024, 160
    psf, x0, g0 = _problem(n, p, seed=17)
    yy, xx = np.mgrid[:n, :n] - n // 2
    g0 = (g0 * np.exp(-(yy ** 2 + xx ** 2) / (2 * 120.0 ** 2))).astype(np.float32)
    cd = _cd(n, psf)
    psf2, amap = cd.maps()
    ox, og, oconv, oit = oracle.deconvolve(x0, g0, amap, psf2, 0.3, 0.1, 400, 1e-7)
    x, g = x0.copy(), g0.copy()
    r = cd.Deconvolve(x, g, 0.3, 0.1, 400, 1e-7)
    assert (r.Converged, r.IterationCount) == (oconv, oit) and oit > 100
    changed = np.argwhere(x != x0)
    assert len(changed) > 0 and np.all((changed >= p) & (changed < n - p))  # windows inside
    assert x.tobytes() == ox.tobytes()
    assert g.tobytes() == og.tobytes()
    cd.destroy()


def test_deconvolve_stops_at_iteration_cap_and_on_no_change(need_gpu):
    n, p = 64, 8
    psf, x0, g0 = _problem(n, p, seed=3)
    cd = _cd(n, psf)
    psf2, amap = cd.maps()
    x, g = x0.copy(), g0.copy()
    r = cd.Deconvolve(x, g, 0.1, 0.1, 5, 0.0)
    ox, og, oconv, oit = oracle.deconvolve(x0, g0, amap, psf2, 0.1, 0.1, 5, 0.0)
    assert (r.Converged, r.IterationCount) == (False, 5) == (oconv, oit)
    assert x.tobytes() == ox.tobytes() and g.tobytes() == og.tobytes()
    z = np.zeros((n, n), np.float32)
    r = cd.Deconvolve(z.copy(), z.copy(), 0.5, 0.2, 10, 1e-4)
    assert r.Converged and r.IterationCount == 0
    # epsilon 0 and no pixel changes: the reference would index pixel (-1, -1)
    with pytest.raises(pkg.P9IDGError) as e:
        cd.Deconvolve(z.copy(), z.copy(), 0.5, 0.2, 10, 0.0)
    assert e.value.code == 1
    # the deconvolver stays usable after the error
    r = cd.Deconvolve(x0.copy(), g0.copy(), 0.1, 0.1, 5, 0.0)
    assert r.IterationCount == 5
    cd.destroy()


@pytest.mark.parametrize("lam,alpha", [(0.5, 0.2), (0.0, 1.0), (2.0, 0.01)])
def test_get_abs_max_diff_vs_oracle(need_gpu, lam, alpha):
    n, p = 160, 16
    psf, x, g = _problem(n, p, seed=11)
    cd = _cd(n, psf)
    _, amap = cd.maps()
    assert cd.GetAbsMaxDiff(x, g, lam, alpha) == oracle.get_abs_max_diff(x, g, amap, lam, alpha)
    cd.destroy()


def test_deconvolve_path_vs_oracle(need_gpu):
    """FastSerialCD.DeconvolvePath (FastSerialCD.cs:49-74) restated over the oracle's pieces."""
    n, p = 96, 12
    psf, x0, g0 = _problem(n, p, seed=21)
    cd = _cd(n, psf)
    psf2, amap = cd.maps()
    lam_min, factor, alpha, paths, iters, eps = 0.3, 4.0, 0.2, 5, 200, 1e-5
    ox, og, total, conv = x0.copy(), g0.copy(), 0, False
    for _ in range(paths):
        mx = oracle.get_abs_max_diff(ox, og, amap, 0.0, 1.0)
        lam_cur = np.float32(np.float32(np.float32(1) / np.float32(alpha)) * np.float32(mx)) / np.float32(factor)
        lam_cur = lam_cur if lam_cur > np.float32(lam_min) else np.float32(lam_min)
        ox, og, c, it = oracle.deconvolve(ox, og, amap, psf2, lam_cur, alpha, iters, eps)
        conv = (np.float32(lam_min) == lam_cur) and c
        total += it
        if conv:
            break
    x, g = x0.copy(), g0.copy()
    r = cd.DeconvolvePath(x, g, lam_min, factor, alpha, paths, iters, eps)
    assert (r.Converged, r.IterationCount) == (conv, total)
    assert x.tobytes() == ox.tobytes() and g.tobytes() == og.tobytes()
    cd.destroy()


def test_reset_lipschitz_map(need_gpu):
    """FastSerialCD.ResetLipschitzMap (FastSerialCD.cs:116-127)."""
    n, p, pf = 128, 16, 64
    psf, _, _ = _problem(n, p, seed=5)
    full, _, _ = _problem(n, pf, seed=6)
    cd = _cd(n, psf)
    psf2_before, _ = cd.maps()
    cd.ResetLipschitzMap(full)
    psf2, amap = cd.maps()
    max_full = float(oracle.psf_squared(full).max())
    assert cd.MaxLipschitz == pytest.approx(max_full, rel=1e-6)
    assert np.array_equal(amap, oracle.amap(full, (n, n)))
    scale = np.float32(np.float32(cd.MaxLipschitz) / np.float32(psf2_before.max()))
    assert np.array_equal(psf2, (psf2_before * scale).astype(np.float32))
    cd.destroy()


@pytest.mark.parametrize("p,n", [(8, 64), (16, 128), (64, 256)])
def test_psf_helpers_and_convolver_vs_oracle(need_gpu, p, n):
    rng = np.random.default_rng(p + n)
    psf = rng.standard_normal((p, p)).astype(np.float32)
    k = pkg.PSF.CalcPaddedFourierCorrelation(psf, pkg.Rectangle(0, 0, n, n))
    ok = oracle.padded_fourier_correlation(psf, (n, n))
    assert rel_l2(k, ok) < 1e-12
    sq = pkg.PSF.CalcPSFSquared(psf)
    osq = oracle.psf_squared(psf)
    assert np.abs(sq - osq).max() <= 2e-7 * np.abs(osq).max()
    assert np.array_equal(pkg.PSF.CalcAMap(psf, pkg.Rectangle(0, 0, n, n)), oracle.amap(psf, (n, n)))
    img = rng.standard_normal((n, n)).astype(np.float32)
    ref = oracle.padded_convolve(ok, (p, p), img)
    conv = pkg.PaddedConvolver.correlation(psf, pkg.Rectangle(0, 0, n, n))
    out = conv.Convolve(img)
    assert np.abs(out - ref).max() <= 1e-6 * np.abs(ref).max()
    conv.destroy()
    conv2 = pkg.PaddedConvolver(ok, pkg.Rectangle(0, 0, p, p))
    assert np.abs(conv2.Convolve(img) - ref).max() <= 1e-6 * np.abs(ref).max()
    conv2.destroy()
    big = rng.standard_normal((2 * n, 2 * n)).astype(np.float32)
    assert np.array_equal(pkg.PSF.Cut(big, 4), oracle.psf_cut(big, 4))
    assert pkg.PSF.CalcMaxSidelobe(big, 4) == oracle.max_sidelobe(big, 4)


def _mc_inputs():
    obs, cd = workload("small_256", n_ant=8, nt=200, nch=4, seed=3)
    c, cd = constants(cd)
    return obs, c, cd


MC_ARGS = dict(psfCutFactor=8, maxMajorCycle=3, lambda_=0.5, alpha=0.05, deconvIterations=2000, deconvEpsilon=1e-5)


def _run_gpu_mc(obs, c, mode, flags=None):
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    part.plan.set_mode(mode)
    if flags is None:
        flags = np.zeros(obs.vis.shape, bool)
    return pkg.MajorCycle.ReconstructSerialCD(c, part, obs.vis, obs.uvw, obs.frequencies, flags, **MC_ARGS)


@pytest.mark.parametrize("flag_fraction", [0.0, 0.1], ids=["unflagged", "flagged"])
def test_major_cycle_vs_oracle(need_gpu, flag_fraction):
    """MajorCycle.ReconstructSerialCD with the FP32 gridder vs the FP64 oracle loop: the same
    number of cycles and decisions, PSF and first dirty image to FP32-gridder accuracy, and the
    final model and residual within 1e-3 relative L2 (the CD sequence depends on gradients that
    differ at ~1e-6 between the FP32 and FP64 gridders).  With flags, the PSF uses unit
    visibilities only where unflagged, the first cycle grids the raw visibilities (flagged ones
    included, as MajorCycle.cs:83,88 does) and later cycles the flag-zeroed residuals."""
    obs, c, cd = _mc_inputs()
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    flags = (np.random.default_rng(12).random(obs.vis.shape) < flag_fraction).astype(np.uint8)
    ref = oracle.major_cycle(cd, subs, obs.uvw, obs.frequencies, obs.vis, flags, MC_ARGS["psfCutFactor"],
                             MC_ARGS["maxMajorCycle"], MC_ARGS["lambda_"], MC_ARGS["alpha"],
                             MC_ARGS["deconvIterations"], MC_ARGS["deconvEpsilon"])
    got = _run_gpu_mc(obs, c, pkg.MODE_FP32, flags.astype(bool))
    cyc, rc = got["cycles"], ref["cycles"]
    assert len(cyc) == len(rc)
    assert [x["deconvolved"] for x in cyc] == list(rc["deconvolved"])
    assert rel_l2(got["psf"], ref["psf"]) < 1e-5
    assert cyc[0]["max_dirty"] == pytest.approx(float(rc["max_dirty"][0]), rel=1e-5)
    assert cyc[0]["max_b"] == pytest.approx(float(rc["max_b"][0]), rel=1e-5)
    assert cyc[0]["current_lambda"] == pytest.approx(float(rc["current_lambda"][0]), rel=1e-5)
    for a, b in zip(cyc, rc):
        assert abs(a["iterations"] - int(b["iterations"])) <= max(2, int(b["iterations"]) // 50)
        # the reference's per-cycle objective (MajorCycle.cs:102)
        assert a["objective"] == pytest.approx(float(b["objective"]), rel=1e-4)
    assert rel_l2(got["model"], ref["model"]) < 1e-3
    assert rel_l2(got["residual"], ref["residual"]) < 1e-3


def test_major_cycle_tensor_core_vs_fp32(need_gpu):
    """The split-precision gridder in the loop: the objective the reconstruction minimises
    (MajorCycle.cs:102) agrees with the FP32 loop's cycle by cycle to 1e-4; the images agree to
    the gridders' own difference.  The models are compared more loosely (1e-2): greedy coordinate
    descent picks the pixel with the largest proximal change, and gradients that differ at the
    1e-5 level reorder near-equal candidates, so the two loops place some flux on neighbouring
    pixels at an equal objective."""
    obs, c, _ = _mc_inputs()
    a = _run_gpu_mc(obs, c, pkg.MODE_FP32)
    b = _run_gpu_mc(obs, c, pkg.MODE_TC_BF16X3)
    assert len(a["cycles"]) == len(b["cycles"])
    for x, y in zip(b["cycles"], a["cycles"]):
        assert x["objective"] == pytest.approx(y["objective"], rel=1e-4)
    print("objective per cycle, tensor core / FP32:",
          [(round(x["objective"], 6), round(y["objective"], 6)) for x, y in zip(b["cycles"], a["cycles"])],
          f"model rel-L2 {rel_l2(b['model'], a['model']):.2e}")
    assert rel_l2(b["psf"], a["psf"]) < 1e-4
    assert rel_l2(b["model"], a["model"]) < 1e-2
    assert rel_l2(b["residual"], a["residual"]) < 1e-3


@pytest.mark.parametrize("mode", [pkg.MODE_FP32, pkg.MODE_TC_BF16X3], ids=["fp32", "tc_bf16x3"])
def test_config1_reconstruction_full_size(need_gpu, mode):
    """The 256^2 workload at full size (30 antennas, 1440 times, 8 channels; two point sources and
    noise) through PSF, dirty image and serial coordinate descent (lambda 0.5, alpha 0.05), two
    major cycles, against the FP64 oracle loop on the same inputs: the same decisions, the
    reference's objective per cycle, and the final model and residual."""
    obs, cd = workload("small_256")
    c, cd = constants(cd)
    args = dict(MC_ARGS, maxMajorCycle=2)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    flags = np.zeros(obs.vis.shape, np.uint8)
    ref = oracle.major_cycle(cd, subs, obs.uvw, obs.frequencies, obs.vis, flags, args["psfCutFactor"],
                             args["maxMajorCycle"], args["lambda_"], args["alpha"], args["deconvIterations"],
                             args["deconvEpsilon"])
    part = pkg.Partitioner.CreatePartition(c, obs.uvw, obs.frequencies)
    assert part.plan.set_mode(mode) == mode
    got = pkg.MajorCycle.ReconstructSerialCD(c, part, obs.vis, obs.uvw, obs.frequencies, flags.astype(bool), **args)
    cyc, rc = got["cycles"], ref["cycles"]
    tol = 1e-5 if mode == pkg.MODE_FP32 else 1e-4
    print(f"config-1 reconstruction, mode {mode}: objective GPU / oracle",
          [(round(x["objective"], 6), round(float(y["objective"]), 6)) for x, y in zip(cyc, rc)],
          f"model {rel_l2(got['model'], ref['model']):.2e} residual {rel_l2(got['residual'], ref['residual']):.2e}")
    assert len(cyc) == len(rc)
    assert [x["deconvolved"] for x in cyc] == list(rc["deconvolved"])
    assert rel_l2(got["psf"], ref["psf"]) < tol
    assert cyc[0]["max_dirty"] == pytest.approx(float(rc["max_dirty"][0]), rel=tol)
    for a, b in zip(cyc, rc):
        assert a["objective"] == pytest.approx(float(b["objective"]), rel=10 * tol)
    assert rel_l2(got["model"], ref["model"]) < 1e-2
    assert rel_l2(got["residual"], ref["residual"]) < 1e-3
