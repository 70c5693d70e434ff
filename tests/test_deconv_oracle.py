"""Pins for the deconvolution oracle (oracle/deconv_oracle.c): FastSerialCD, the PSF helpers,
the padded Fourier correlation and the serial major cycle.

The C# reference cannot run here and ships no golden vectors, so the oracle is pinned by
(1) an independent pure-Python restatement of FastSerialCD.cs and PSF.CalcAMap/QueryScan in
numpy float32 scalar arithmetic (bit-exact comparisons), (2) numpy.fft for the FFT-based
helpers (FFTW conventions), and (3) hand-derived known answers: with a delta PSF every pixel
is set once to the proximal value of its gradient, in order of decreasing change.
"""
import numpy as np
import pytest

from conftest import constants, oracle, rel_l2, workload

f32 = np.float32


# ---------------- independent restatement (pure Python, float32 scalars) ----------------

def _maxf(a, b):
    """.NET Core 3.0 Math.Max(float, float)."""
    if a != b:
        if not np.isnan(a):
            return a if b < a else b
        return a
    return a if np.signbit(b) else b


def _prox(x, lip, lam, alpha):
    num = _maxf(f32(x - f32(lam * alpha)), f32(0.0))
    den = f32(lip + f32(lam * f32(f32(1.0) - alpha)))
    return f32(num / den)


def _abs_max(x, g, a, lam, alpha):
    """FastSerialCD.GetAbsMax: row winners by strict <, then rows by strict <."""
    n = x.shape[0]
    best = (-1, -1, f32(0), f32(0))
    for y in range(n):
        cur = (-1, -1, f32(0), f32(0))
        for xx in range(n):
            old = x[y, xx]
            xt = _prox(f32(f32(old * a[y, xx]) + g[y, xx]), a[y, xx], lam, alpha)
            d = abs(f32(old - xt))
            if cur[2] < d:
                cur = (y, xx, d, xt)
        if best[2] < cur[2]:
            best = cur
    return best


def _deconvolve(x, g, a, psf2, lam, alpha, iterations, eps):
    x, g = x.copy(), g.copy()
    n = x.shape[0]
    ph, pw = psf2.shape
    it, conv = 0, False
    lam, alpha, eps = f32(lam), f32(alpha), f32(eps)
    while not conv and it < iterations:
        y, xx, d, xn = _abs_max(x, g, a, lam, alpha)
        conv = d < eps
        if not conv:
            old = x[y, xx]
            x[y, xx] = xn
            xd = f32(old - xn)
            for i in range(max(y - ph // 2, 0), min(y - ph // 2 + ph, n)):
                for j in range(max(xx - pw // 2, 0), min(xx - pw // 2 + pw, n)):
                    g[i, j] = f32(g[i, j] + f32(psf2[i + ph // 2 - y, j + pw // 2 - xx] * xd))
            it += 1
    return x, g, conv, it


def _query_scan(scan, y, x, yl, xl):
    sh, sw = scan.shape
    yo = max(0, (y + (sh - sh // 2)) - yl)
    xo = max(0, (x + (sw - sw // 2)) - xl)
    yu = -(y - sh // 2)
    xu = -(x - sw // 2)
    yui, xui = max(1, yu) - 1, max(1, xu) - 1
    if yo <= 0 and xo <= 0 and yu <= 0 and xu <= 0:
        return scan[sh - 1, sw - 1]
    if yu > 0 and xu > 0:
        return scan[sh - 1, sw - 1] - scan[sh - 1, xui] - scan[yui, sw - 1] + scan[yui, xui]
    corr = 0.0
    if yu > 0:
        corr += scan[yui, sw - xo - 1]
    if xu > 0:
        corr += scan[sh - yo - 1, xui]
    return scan[sh - 1 - yo, sw - 1 - xo] - corr


def _scan(psf):
    h, w = psf.shape
    s = np.zeros((h, w), np.float64)
    for i in range(h):
        for j in range(w):
            iB = s[i - 1, j] if i > 0 else 0.0
            jB = s[i, j - 1] if j > 0 else 0.0
            ijB = s[i - 1, j - 1] if i > 0 and j > 0 else 0.0
            s[i, j] = float(f32(psf[i, j] * psf[i, j])) + iB + jB - ijB
    return s


def _np_shift(a):
    n2 = a.shape[0] // 2
    b = a.copy()
    m = 2 * n2
    b[:m, :m] = np.roll(np.roll(a[:m, :m], n2, 0), n2, 1)
    return b


def _np_correlation(psf, pad):
    h, w = psf.shape
    H, W = pad[0] + h, pad[1] + w
    p = np.zeros((H, W))
    for y in range(h):
        for x in range(w):
            if y + pad[0] // 2 + 1 < H and x + pad[1] // 2 + 1 < W:
                p[y + pad[0] // 2 + 1, x + pad[1] // 2 + 1] = psf[h - y - 1, w - x - 1]
    return np.fft.fft2(_np_shift(p))


def _np_convolve(kernel, ky, kx, img):
    H, W = kernel.shape
    n = img.shape[0]
    buf = np.zeros((H, W), np.complex128)
    buf[ky // 2:ky // 2 + n, kx // 2:kx // 2 + n] = img
    out = np.fft.ifft2(np.fft.fft2(buf) * kernel) * (H * W)
    return (out.real[ky // 2:ky // 2 + n, kx // 2:kx // 2 + n] / (H * W)).astype(np.float32)


def _rand_problem(n=12, p=4, seed=0):
    rng = np.random.default_rng(seed)
    psf = rng.standard_normal((p, p)).astype(np.float32) * 0.1
    psf[p // 2, p // 2] = 1.0
    x = np.zeros((n, n), np.float32)
    x[rng.integers(0, n, 3), rng.integers(0, n, 3)] = rng.random(3).astype(np.float32)
    g = rng.standard_normal((n, n)).astype(np.float32)
    psf2 = oracle.psf_squared(psf)
    a = oracle.amap(psf, (n, n))
    return x, g, a, psf2


# ---------------- tests ----------------

@pytest.mark.parametrize("seed", [0, 1, 2])
def test_get_abs_max_matches_restatement(seed):
    x, g, a, _ = _rand_problem(seed=seed)
    for lam, alpha in [(0.5, 0.2), (0.0, 1.0), (3.0, 0.05)]:
        y, xx, d, xn = oracle.get_abs_max_pixel(x, g, a, lam, alpha)
        ry, rx, rd, rxn = _abs_max(x, g, a, f32(lam), f32(alpha))
        assert (y, xx) == (ry, rx)
        assert np.float32(d).tobytes() == rd.tobytes() and np.float32(xn).tobytes() == rxn.tobytes()


@pytest.mark.parametrize("seed,iters", [(0, 25), (3, 7), (4, 60)])
def test_deconvolve_matches_restatement_bit_exact(seed, iters):
    x, g, a, psf2 = _rand_problem(seed=seed)
    ox, og, oc, oi = oracle.deconvolve(x, g, a, psf2, 0.4, 0.2, iters, 1e-5)
    rx, rg, rc, ri = _deconvolve(x, g, a, psf2, 0.4, 0.2, iters, 1e-5)
    assert (oc, oi) == (rc, ri)
    assert ox.tobytes() == rx.tobytes() and og.tobytes() == rg.tobytes()


def test_delta_psf_known_answer():
    """With a delta PSF (psf2 = delta, aMap = 1) each pixel with |change| > 0 is set once to
    max(b - lambda alpha, 0) / (1 + lambda (1 - alpha)); the next candidate at that pixel
    then has no change, so CD stops after exactly that many iterations, converged."""
    n, lam, alpha = 16, 0.5, 0.2
    rng = np.random.default_rng(5)
    b = rng.standard_normal((n, n)).astype(np.float32)
    psf = np.zeros((2, 2), np.float32)
    psf[1, 1] = 1.0
    psf2 = oracle.psf_squared(psf)
    assert np.allclose(psf2, np.pad([[1.0]], ((2, 1), (2, 1))), atol=1e-7)
    psf2 = np.zeros((4, 4), np.float32)
    psf2[2, 2] = 1.0
    a = np.ones((n, n), np.float32)
    x0 = np.zeros((n, n), np.float32)
    expect = np.maximum(b - f32(lam * alpha), 0) / f32(1 + f32(lam * f32(1 - alpha)))
    x, g, conv, it = oracle.deconvolve(x0, b, a, psf2, lam, alpha, 10_000, 1e-7)
    assert conv and it == int(np.count_nonzero(expect))
    assert np.allclose(x, expect, rtol=1e-6, atol=0)


def test_deconvolve_iteration_cap_and_no_candidate():
    x, g, a, psf2 = _rand_problem(seed=7)
    _, _, conv, it = oracle.deconvolve(x, g, a, psf2, 0.1, 0.1, 3, 0.0)
    assert not conv and it == 3
    z = np.zeros_like(x)
    _, _, conv, it = oracle.deconvolve(z, z, a, psf2, 0.5, 0.2, 10, 1e-4)
    assert conv and it == 0
    with pytest.raises(oracle.OracleError) as e:
        oracle.deconvolve(z, z, a, psf2, 0.5, 0.2, 10, 0.0)
    assert e.value.code == oracle.INDEX_OUT_OF_RANGE


@pytest.mark.parametrize("p,n", [(4, 12), (5, 9), (8, 8), (16, 16)])
def test_amap_matches_restatement(p, n):
    rng = np.random.default_rng(p * 31 + n)
    psf = rng.standard_normal((p, p)).astype(np.float32)
    s = _scan(psf)
    assert np.array_equal(oracle.amap_scan(psf), s)
    ref = np.array([[_query_scan(s, y, x, n, n) for x in range(n)] for y in range(n)], np.float64).astype(np.float32)
    assert np.array_equal(oracle.amap(psf, (n, n)), ref)


def test_psf_cut_sidelobe_lipschitz():
    rng = np.random.default_rng(9)
    psf = rng.standard_normal((32, 32)).astype(np.float32)
    cut = oracle.psf_cut(psf, 4)
    assert np.array_equal(cut, psf[12:20, 12:20])
    a = np.abs(psf).copy()
    a[12:20, 12:20] = 0
    assert oracle.max_sidelobe(psf, 4) == float(a.max())
    seq = 0.0
    for v in (cut * cut).ravel():  # float products summed in double, in order
        seq += float(v)
    assert oracle.max_lipschitz(cut) == seq
    img = rng.standard_normal((7, 7)).astype(np.float32)
    assert oracle.get_max(img) == float(max(0.0, img.max()))
    assert oracle.get_max(-np.abs(img)) == 0.0
    assert oracle.residual_penalty(img) == pytest.approx(0.5 * float(np.sum(img.astype(np.float64) ** 2)), rel=1e-6)


@pytest.mark.parametrize("p,n", [(4, 12), (6, 10), (8, 24)])
def test_padded_correlation_and_convolve_match_numpy(p, n):
    rng = np.random.default_rng(n)
    psf = rng.standard_normal((p, p)).astype(np.float32)
    k = oracle.padded_fourier_correlation(psf, (n, n))
    kr = _np_correlation(psf.astype(np.float64), (n, n))
    assert rel_l2(k, kr) < 1e-13
    img = rng.standard_normal((n, n)).astype(np.float32)
    out = oracle.padded_convolve(k, (p, p), img)
    assert rel_l2(out, _np_convolve(kr, p, p, img.astype(np.float64))) < 1e-6


def test_padded_convolve_is_correlation_with_the_psf():
    """Convolving an image with a single unit pixel by the correlation kernel of a PSF places the
    PSF mirrored around that pixel (out[y, x] = psf[8 - y + p/2, 7 - x + p/2]): b = PSF (*) image,
    the gradient of the residual.  Even sizes (the reference's FFT.Shift is a plain quadrant swap
    only for even sizes)."""
    p, n = 6, 16
    rng = np.random.default_rng(2)
    psf = rng.standard_normal((p, p)).astype(np.float32)
    img = np.zeros((n, n), np.float32)
    img[8, 7] = 1.0
    out = oracle.padded_convolve(oracle.padded_fourier_correlation(psf, (n, n)), (p, p), img)
    # out[y, x] = sum_k img[k] psf[k - (y, x) + centre] : a flipped copy of psf centred on (8, 7)
    ref = np.zeros((n, n))
    for y in range(n):
        for x in range(n):
            dy, dx = 8 - y + p // 2, 7 - x + p // 2
            if 0 <= dy < p and 0 <= dx < p:
                ref[y, x] = psf[dy, dx]
    assert np.abs(out - ref).max() < 1e-6


def test_psf_squared_is_autocorrelation():
    """CalcPSFSquared = the PSF correlated with itself, on a 2h x 2w grid centred at (h, w)."""
    p = 6
    rng = np.random.default_rng(4)
    psf = rng.standard_normal((p, p)).astype(np.float32)
    out = oracle.psf_squared(psf)
    full = np.zeros((2 * p, 2 * p))
    for dy in range(-p + 1, p):
        for dx in range(-p + 1, p):
            s = 0.0
            for y in range(p):
                for x in range(p):
                    if 0 <= y + dy < p and 0 <= x + dx < p:
                        s += float(psf[y, x]) * float(psf[y + dy, x + dx])
            full[p + dy, p + dx] = s
    assert np.abs(out - full).max() < 1e-5 * np.abs(full).max()


def test_major_cycle_small():
    """The serial major cycle on a small observation: the residual image falls cycle by cycle,
    and the model carries flux at the brightest dirty-image pixel."""
    obs, cd = workload("small_256", n_ant=8, nt=200, nch=4, seed=3)
    c, cd = constants(cd)
    subs = oracle.partition(cd, obs.uvw, obs.frequencies)
    flags = np.zeros(obs.vis.shape, np.uint8)
    r = oracle.major_cycle(cd, subs, obs.uvw, obs.frequencies, obs.vis, flags, 8, 3, 0.5, 0.05, 2000, 1e-5)
    cyc = r["cycles"]
    assert len(cyc) >= 2
    assert all(cyc["deconvolved"][:-1] == 1)
    assert cyc["max_dirty"][-1] < cyc["max_dirty"][0]
    assert float(r["model"].max()) > 0
    psf = r["psf"]
    assert np.unravel_index(np.argmax(psf), psf.shape) == (cd["grid_size"] // 2, cd["grid_size"] // 2)
