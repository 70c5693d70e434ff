"""Pins for the FP64 CPU oracle (oracle/idg_oracle.c).

The C# reference cannot run here and ships no golden vectors, so the oracle is pinned by
(1) hand-derived known answers of the whole gridding chain, (2) an independent numpy
restatement (oracle/idg_np.py), (3) numpy.fft for the FFTW conventions, and (4) the
adjoint identities the reference's operators satisfy.  tests/golden holds a small
regression fixture of oracle outputs (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

import idg_np
from conftest import C_LIGHT, kat_constants, oracle, rel_l2, workload

GOLDEN_NPZ = os.path.join(os.path.dirname(__file__), "golden", "idg_small.npz")


def _single_vis(pu, pv, w=0.0, N=64, S=16, W=1, wstep=0.0):
    cd = kat_constants(N=N, S=S, W=W, wstep=wstep)
    uvw = np.array([[[pu, pv, w]]], np.float64)
    freq = np.array([C_LIGHT])
    vis = np.ones((1, 1, 1), np.complex128)
    return cd, uvw, freq, vis


@pytest.mark.parametrize("pu,pv", [(0, 0), (3, -5), (-7, 2), (11, 9)])
def test_unit_visibility_grids_to_unit_delta(pu, pv):
    """A unit visibility at integer uv pixel p (w = 0) grids to exactly 1 at grid[p_v mod N, p_u mod N].

    By hand: the subgrid pixels are exp(2 pi i d (x - S/2 + 1/2)/S) with d = centre - p, the
    scaled IFFT turns them into exp(i pi d/S) at one Fourier pixel, and the adder phasor
    exp(i pi (x' - S/2)/S) at that pixel is exp(-i pi d/S) (IDG.cs:12-20, Gridder.cs,
    SubgridFFT.cs:11-52, Adder.cs:13-55, FFT.cs:248-264)."""
    cd, uvw, freq, vis = _single_vis(pu, pv)
    subs = oracle.partition(cd, uvw, freq)
    g = oracle.idg_grid(cd, subs, vis, uvw, freq)
    N = cd["grid_size"]
    expect = np.zeros((N, N), np.complex128)
    expect[pv % N, pu % N] = 1.0
    assert np.abs(g - expect).max() < 1e-12


def test_negative_w_mirrors_and_conjugates():
    """w index -1 (w slightly below 0) lands in layer 0 at the Hermitian mirror -p (AdderWStack.cs:37-70)."""
    cd, uvw, freq, vis = _single_vis(5, -3, w=-1e-12, W=2, wstep=1.0)
    vis = vis * (0.6 + 0.8j)
    subs = oracle.partition(cd, uvw, freq)
    assert subs["w_lambda"][0] == -1
    layers = oracle.idg_grid_w(cd, subs, vis, uvw, freq)
    N = cd["grid_size"]
    expect = np.zeros((2, N, N), np.complex128)
    expect[0, 3 % N, -5 % N] = 0.6 - 0.8j
    assert np.abs(layers - expect).max() < 1e-9


@pytest.mark.parametrize("q", [(0, 0), (4, -6)])
def test_degrid_of_unit_delta(q):
    """DeGrid is the adjoint of Grid, so a unit delta at grid[q] degrids to 1 at the visibility sitting
    on pixel q and to 0 at integer pixels elsewhere in the same subgrid."""
    qu, qv = q
    cd = kat_constants()
    N = cd["grid_size"]
    uvw = np.array([[[qu, qv, 0.0], [qu + 2, qv, 0.0], [qu, qv - 3, 0.0]]], np.float64)
    freq = np.array([C_LIGHT])
    subs = oracle.partition(cd, uvw, freq)
    grid = np.zeros((N, N), np.complex128)
    grid[qv % N, qu % N] = 1.0
    vis, shifted = oracle.idg_degrid(cd, subs, grid, uvw, freq)
    assert np.allclose(vis[0, :, 0], [1.0, 0.0, 0.0], atol=1e-12)
    assert np.array_equal(shifted, oracle.shift(grid))  # IDG.cs:24 shifts the caller's grid


def test_unit_visibility_image_is_flat():
    """ToImage of a unit visibility at the origin: Re(IFFT(delta)) / visCount everywhere (IDG.cs:68-83)."""
    cd, uvw, freq, vis = _single_vis(0, 0)
    subs = oracle.partition(cd, uvw, freq)
    g = oracle.idg_grid(cd, subs, vis, uvw, freq)
    img = oracle.shift(oracle.fft_backward_real(g, 4))
    assert np.allclose(img, 0.25, atol=1e-14)


def test_fft_conventions_match_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 5, 7, 8, 24, 32, 48, 96, 3 * 7):
        x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        assert rel_l2(oracle.fft1d(x, -1), np.fft.fft(x)) < 1e-13          # FFTW_FORWARD
        assert rel_l2(oracle.fft1d(x, +1), np.fft.ifft(x) * n) < 1e-13     # FFTW_BACKWARD
    X = rng.standard_normal((24, 40)) + 1j * rng.standard_normal((24, 40))
    assert rel_l2(oracle.fft2d(X, -1), np.fft.fft2(X)) < 1e-13
    assert rel_l2(oracle.fft2d(X, +1), np.fft.ifft2(X) * X.size) < 1e-13


@pytest.mark.parametrize("n", [6, 7, 8])
def test_shift_matches_restatement(n):
    a = np.arange(n * n, dtype=np.float64).reshape(n, n)
    assert np.array_equal(oracle.shift(a), idg_np.fft_shift(a))
    assert np.array_equal(oracle.shift(a.astype(np.float32)), idg_np.fft_shift(a.astype(np.float32)))
    if n % 2 == 0:
        assert np.array_equal(oracle.shift(a), np.fft.fftshift(a))


@pytest.mark.parametrize("name,kw", [("small_256", dict(n_ant=5, nt=150, nch=3)),
                                     ("meerkat_3072", dict(n_ant=5, nt=120, nch=4))])
def test_c_oracle_matches_numpy_restatement(name, kw):
    obs, cd = workload(name, **kw)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert len(subs) > 0 and (subs["w_lambda"] < 0).any()
    sg = oracle.gridder_forward(cd, subs, obs.uvw, obs.vis, obs.frequencies)
    assert rel_l2(sg, idg_np.gridder_forward(cd, subs, obs.uvw, obs.vis, obs.frequencies)) < 1e-13
    f = oracle.subgrid_fft_forward(cd, sg)
    assert rel_l2(f, idg_np.subgrid_fft_forward(cd, sg)) < 1e-13
    layers = oracle.adder_wstack_add(cd, subs, f)
    assert rel_l2(layers, idg_np.adder_wstack_add(cd, subs, f)) < 1e-13
    g = layers.sum(0)
    s = oracle.adder_wstack_split(cd, subs, g)
    assert rel_l2(s, idg_np.adder_wstack_split(cd, subs, g)) < 1e-13
    b = oracle.subgrid_fft_backward(cd, s)
    assert rel_l2(b, idg_np.subgrid_fft_backward(cd, s)) < 1e-13
    v = oracle.gridder_backward(cd, subs, b, obs.uvw, obs.frequencies)
    vn = idg_np.gridder_backward(cd, subs, b, obs.uvw, obs.frequencies, obs.uvw.shape[0], obs.uvw.shape[1])
    assert rel_l2(v, vn) < 1e-12
    img = oracle.wstack_ifft_float(layers, cd["vis_count"])
    assert rel_l2(img, idg_np.wstack_ifft_float(layers, cd["vis_count"])) < 1e-6


def test_adjoint_grid_degrid():
    """<Grid v, g> = <v, DeGrid g> (IDG.cs:12-30: Split = Add^H, FFT = IFFT^H, both 1/S^2)."""
    obs, cd = workload("small_256", n_ant=5, nt=100, nch=3)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    rng = np.random.default_rng(7)
    N = cd["grid_size"]
    g = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    Gv = oracle.idg_grid(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    Dg, _ = oracle.idg_degrid(cd, subs, g, obs.uvw, obs.frequencies)
    lhs = np.vdot(Gv, g)
    rhs = np.vdot(obs.vis, Dg)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_adjoint_wstack_real_inner_product():
    """GridW conjugates negative-w subgrids (antilinear), so the identity holds for the real inner
    product: Re<sum_k GridW(v)_k, g> = Re<v, DeGridW(g)> for subgrids away from the grid edge."""
    obs, cd = workload("meerkat_3072", n_ant=5, nt=120, nch=4)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    assert (subs["w_lambda"] < 0).any() and (subs["w_lambda"] >= 0).any()
    rng = np.random.default_rng(8)
    N = cd["grid_size"]
    g = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    L = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies).sum(0)
    Dg, _ = oracle.idg_degrid(cd, subs, g, obs.uvw, obs.frequencies, wstack=True)
    lhs = np.vdot(L, g).real
    rhs = np.vdot(obs.vis, Dg).real
    assert abs(lhs - rhs) / abs(lhs) < 1e-11


def test_wstack_ifft_is_linear_in_layers():
    """FFT.WStackIFFTFloat has no per-layer w correction, so it equals the transform of the layer sum."""
    obs, cd = workload("small_256", n_ant=5, nt=100, nch=3)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    L = oracle.idg_grid_w(cd, subs, obs.vis, obs.uvw, obs.frequencies)
    a = oracle.wstack_ifft_float(L, cd["vis_count"])
    b = oracle.wstack_ifft_float(L.sum(0, keepdims=True), cd["vis_count"])
    assert rel_l2(a, b) < 1e-6


def test_golden_fixture_regression():
    """Oracle outputs committed by tests/golden/make_golden.py: guards the restatement against drift."""
    z = np.load(GOLDEN_NPZ)
    cd = {k: z["consts"][k].item() for k in z["consts"].dtype.names}
    subs = oracle.partition(cd, z["uvw"], z["freq"])
    assert np.array_equal(subs.view(np.int32), z["subgrids"].view(np.int32))
    layers = oracle.idg_grid_w(cd, subs, z["vis"], z["uvw"], z["freq"])
    assert rel_l2(layers, z["layers"]) < 1e-13
    vis, _ = oracle.idg_degrid(cd, subs, z["model_grid"], z["uvw"], z["freq"], wstack=True)
    assert rel_l2(vis, z["degridded"]) < 1e-13
    img = oracle.wstack_ifft_float(layers, cd["vis_count"])
    assert rel_l2(img, z["image"]) < 1e-6
