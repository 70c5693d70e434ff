"""Seeded synthetic interferometer observations for the IDG workloads.

The reference reads MeerKAT/LMC measurement sets from FITS files
(Core/FitsIO.cs:196-357, SingleReconstruction/MeasurementData.cs:34-64); those
files are not distributed with it.  This module produces observations with the
same array layout (``uvw[baseline][time][3]`` in metres, ``frequencies[ch]`` in
Hz, ``vis[baseline][time][ch]`` complex, ``flags[baseline][time][ch]`` bool) so
the gridder sees the same shapes, uv-track geometry and value distributions.

Geometry: antennas in a local east/north plane at latitude ``lat_deg``, rotated
to equatorial XYZ and tracked over an hour-angle range centred on transit
(standard Earth-rotation synthesis, u = sin H Lx + cos H Ly, ...).

Sky: point sources (and optional elliptical Gaussians) on the image grid.  Small
skies are evaluated exactly, ``V = sum S exp(-2 pi i (u l + v m + w (n - 1)))``;
large skies are sampled from a 2x-oversampled FFT of the model image with
bilinear interpolation (w-term ignored).  With this sign a source at image
pixel (x, y) appears at pixel (x, y) of the reference's dirty image
(IDG.GridW + FFT.WStackIFFTFloat + FFT.Shift).

Noise: complex Gaussian with standard deviation ``noise_sigma`` per real and
per imaginary component.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

SPEED_OF_LIGHT = 299792458.0  # Core/ImageDomainGridder/MathFunctions.cs:11


@dataclasses.dataclass
class Observation:
    uvw: np.ndarray            # float64 [nbl][nt][3], metres
    frequencies: np.ndarray    # float64 [nch], Hz
    vis: np.ndarray            # complex128 [nbl][nt][nch]
    flags: np.ndarray          # bool [nbl][nt][nch]
    model_image: Optional[np.ndarray]  # float64 [N][N] sky model on the image grid (Jy/pixel)
    meta: dict

    @property
    def vis_count(self) -> int:
        """Unflagged visibilities (SingleReconstruction/MeasurementData.cs:26-31)."""
        return int(np.count_nonzero(~self.flags))


def cell_rad(arcsec: float) -> float:
    return arcsec / 3600.0 * math.pi / 180.0


def antennas_uniform_disk(rng, n, diameter_m):
    r = 0.5 * diameter_m * np.sqrt(rng.random(n))
    t = 2 * np.pi * rng.random(n)
    return np.stack([r * np.cos(t), r * np.sin(t)], axis=1)


def antennas_log_radial(rng, n, diameter_m, r_min=25.0):
    r_max = 0.5 * diameter_m
    r = np.exp(rng.uniform(math.log(r_min), math.log(r_max), n))
    t = 2 * np.pi * rng.random(n)
    return np.stack([r * np.cos(t), r * np.sin(t)], axis=1)


def earth_rotation_uvw(enu_xy, lat_deg, dec_deg, nt, dump_s):
    """uvw[bl][t][3] for all antenna pairs i<j (ordered i-major)."""
    lat = math.radians(lat_deg)
    dec = math.radians(dec_deg)
    e = enu_xy[:, 0]
    nn = enu_xy[:, 1]
    up = np.zeros_like(e)
    X = -math.sin(lat) * nn + math.cos(lat) * up
    Y = e
    Z = math.cos(lat) * nn + math.sin(lat) * up
    ia, ib = np.triu_indices(len(e), k=1)
    Lx, Ly, Lz = X[ib] - X[ia], Y[ib] - Y[ia], Z[ib] - Z[ia]
    omega = 2 * math.pi / 86164.0905  # sidereal rate, rad/s
    t = (np.arange(nt) - (nt - 1) / 2.0) * dump_s
    H = omega * t
    sH, cH = np.sin(H)[None, :], np.cos(H)[None, :]
    Lx, Ly, Lz = Lx[:, None], Ly[:, None], Lz[:, None]
    u = sH * Lx + cH * Ly
    v = -math.sin(dec) * cH * Lx + math.sin(dec) * sH * Ly + math.cos(dec) * Lz
    w = math.cos(dec) * cH * Lx - math.cos(dec) * sH * Ly + math.sin(dec) * Lz
    return np.ascontiguousarray(np.stack([u, v, w], axis=-1))


def _vis_points_exact(uvw, freqs, lm, flux):
    nbl, nt, _ = uvw.shape
    out = np.zeros((nbl, nt, len(freqs)), np.complex128)
    for (l, m), s in zip(lm, flux):
        n1 = math.sqrt(1.0 - l * l - m * m) - 1.0
        arg = uvw[..., 0] * l + uvw[..., 1] * m + uvw[..., 2] * n1  # metres
        for c, f in enumerate(freqs):
            out[:, :, c] += s * np.exp(-2j * np.pi * arg * (f / SPEED_OF_LIGHT))
    return out


def _vis_from_image_fft(uvw, freqs, image, imagesize):
    """Bilinear samples of the 2x-oversampled image FFT at each uv point."""
    N = image.shape[0]
    M = 2 * N
    pad = np.zeros((M, M), np.complex64)
    idx = (np.arange(N) - N // 2) % M
    pad[np.ix_(idx, idx)] = image.astype(np.complex64)
    F = np.fft.fft2(pad).astype(np.complex64)
    nbl, nt, _ = uvw.shape
    out = np.empty((nbl, nt, len(freqs)), np.complex128)
    for c, f in enumerate(freqs):
        scale = imagesize * f / SPEED_OF_LIGHT * 2.0  # oversampled-grid index per metre
        qu = uvw[..., 0] * scale
        qv = uvw[..., 1] * scale
        u0 = np.floor(qu)
        v0 = np.floor(qv)
        fu = (qu - u0).astype(np.float32)
        fv = (qv - v0).astype(np.float32)
        iu0 = u0.astype(np.int64) % M
        iv0 = v0.astype(np.int64) % M
        iu1 = (iu0 + 1) % M
        iv1 = (iv0 + 1) % M
        val = (F[iv0, iu0] * (1 - fu) * (1 - fv) + F[iv0, iu1] * fu * (1 - fv)
               + F[iv1, iu0] * (1 - fu) * fv + F[iv1, iu1] * fu * fv)
        out[:, :, c] = val
    return out


def _power_law_fluxes(rng, n, index, s_min, s_max):
    # N(S) ~ S^index; inverse CDF for index != -1
    a = index + 1.0
    u = rng.random(n)
    return (s_min ** a + u * (s_max ** a - s_min ** a)) ** (1.0 / a)


def make_observation(*, seed, n_ant, array_diameter_m, layout, nt, dump_s, f_lo, f_hi, nch,
                     grid_size, cell_arcsec, lat_deg=-30.7215, dec_deg=-70.0,
                     point_fluxes=None, n_power_law=0, power_law=(-1.6, 1e-3, 1.0),
                     n_gauss=0, gauss_sigma_px=(3.0, 30.0), noise_sigma=0.0,
                     flag_fraction=0.0, exact_sky=None) -> Observation:
    rng = np.random.default_rng(seed)
    if layout == "uniform":
        ants = antennas_uniform_disk(rng, n_ant, array_diameter_m)
    elif layout == "log_radial":
        ants = antennas_log_radial(rng, n_ant, array_diameter_m)
    else:
        raise ValueError(layout)
    uvw = earth_rotation_uvw(ants, lat_deg, dec_deg, nt, dump_s)
    freqs = np.linspace(f_lo, f_hi, nch)
    N = grid_size
    cell = cell_rad(cell_arcsec)
    imagesize = float(np.float32(cell)) * N

    image = np.zeros((N, N))
    pts_xy, pts_flux = [], []
    if point_fluxes is not None:
        for s in point_fluxes:
            x, y = rng.integers(N // 4, 3 * N // 4, size=2)
            image[y, x] += s
            pts_xy.append((int(x), int(y)))
            pts_flux.append(float(s))
    if n_power_law:
        fl = _power_law_fluxes(rng, n_power_law, *power_law)
        xs = rng.integers(N // 10, N - N // 10, size=n_power_law)
        ys = rng.integers(N // 10, N - N // 10, size=n_power_law)
        np.add.at(image, (ys, xs), fl)
        pts_xy += list(zip(xs.tolist(), ys.tolist()))
        pts_flux += fl.tolist()
    if n_gauss:
        yy, xx = np.mgrid[0:N, 0:N]
        for _ in range(n_gauss):
            cx, cy = rng.uniform(N * 0.15, N * 0.85, size=2)
            sa, sb = rng.uniform(*gauss_sigma_px, size=2)
            th = rng.uniform(0, np.pi)
            peak = rng.uniform(1e-4, 1e-2)
            r = int(4 * max(sa, sb)) + 1
            x0, x1 = max(0, int(cx) - r), min(N, int(cx) + r)
            y0, y1 = max(0, int(cy) - r), min(N, int(cy) + r)
            dx = xx[y0:y1, x0:x1] - cx
            dy = yy[y0:y1, x0:x1] - cy
            a = (dx * math.cos(th) + dy * math.sin(th)) / sa
            b = (-dx * math.sin(th) + dy * math.cos(th)) / sb
            image[y0:y1, x0:x1] += peak * np.exp(-0.5 * (a * a + b * b))

    if exact_sky is None:
        exact_sky = (n_gauss == 0 and len(pts_flux) <= 16)
    if exact_sky:
        lm = [((x - N // 2) * cell, (y - N // 2) * cell) for x, y in pts_xy]
        vis = _vis_points_exact(uvw, freqs, lm, pts_flux)
    else:
        vis = _vis_from_image_fft(uvw, freqs, image, imagesize)
    if noise_sigma > 0:
        vis += noise_sigma * (rng.standard_normal(vis.shape) + 1j * rng.standard_normal(vis.shape))
    flags = np.zeros(vis.shape, bool)
    if flag_fraction > 0:
        flags = rng.random(vis.shape) < flag_fraction
    meta = dict(seed=seed, n_ant=n_ant, n_baselines=uvw.shape[0], nt=nt, nch=nch, dump_s=dump_s,
                lat_deg=lat_deg, dec_deg=dec_deg, array_diameter_m=array_diameter_m, layout=layout,
                f_lo=f_lo, f_hi=f_hi, grid_size=N, cell_arcsec=cell_arcsec,
                noise_sigma_per_component=noise_sigma, exact_sky=bool(exact_sky),
                n_sources=len(pts_flux), n_gauss=n_gauss, flag_fraction=flag_fraction)
    return Observation(uvw=uvw, frequencies=freqs, vis=vis, flags=flags, model_image=image, meta=meta)


def wstep_for(uvw, frequencies, w_layers):
    """w step in wavelengths: max |w| at the highest frequency / layer count.

    Follows SingleReconstruction/RunningMethod.cs:48-53.
    """
    max_w = float(np.max(np.abs(uvw[..., 2]))) if uvw.size else 0.0
    max_w = max_w * (float(frequencies[-1]) / SPEED_OF_LIGHT)
    return max_w / w_layers


# Workloads.  Each entry gives the observation and the gridding constants.
WORKLOADS = {
    # 256^2, 30 antennas in a 2 km (diameter) disk, 4 h at dec -70, 10 s dumps, 8 ch 1.00-1.10 GHz.
    "small_256": dict(obs=dict(seed=1, n_ant=30, array_diameter_m=2000.0, layout="uniform", nt=1440,
                               dump_s=10.0, f_lo=1.00e9, f_hi=1.10e9, nch=8, grid_size=256,
                               cell_arcsec=5.0, point_fluxes=[1.0, 0.5], noise_sigma=0.1),
                      grid=dict(subgrid_size=32, kernel_size=8, max_timesteps=1024, w_layers=4)),
    # 3072^2, 64 antennas log-radial within an 8 km (diameter) array, 2000 x 10 s, 16 ch 1.2-1.5 GHz.
    "meerkat_3072": dict(obs=dict(seed=2, n_ant=64, array_diameter_m=8000.0, layout="log_radial", nt=2000,
                                  dump_s=10.0, f_lo=1.2e9, f_hi=1.5e9, nch=16, grid_size=3072,
                                  cell_arcsec=1.5, n_power_law=2000, n_gauss=20, noise_sigma=1e-3),
                         grid=dict(subgrid_size=32, kernel_size=8, max_timesteps=1024, w_layers=8)),
}


def batched_workloads(n=64, seed=4, subgrid_size=32, w_layers=8, mix="config"):
    """Independent imaging problems of mixed sizes, 1.5 arcsec cells, the sky of the 3072^2
    workload (power-law points + Gaussians), antennas log-radial within 8 km.
    mix "config": images 512^2..2048^2, 200-2000 times, 4-32 channels, 16-64 antennas.
    mix "small": images 512^2..1024^2, 200-500 times, 4-16 channels, 16-32 antennas (problems
    too small to fill the GPU on their own)."""
    rng = np.random.default_rng(seed)
    lim = dict(config=((256, 1025), (16, 65), (200, 2001), (4, 33)),
               small=((256, 513), (16, 33), (200, 501), (4, 17)))[mix]
    out = []
    for i in range(n):
        N = 2 * int(rng.integers(*lim[0]))
        obs = dict(seed=seed * 1000 + i, n_ant=int(rng.integers(*lim[1])), array_diameter_m=8000.0,
                   layout="log_radial", nt=int(rng.integers(*lim[2])), dump_s=10.0, f_lo=1.2e9, f_hi=1.5e9,
                   nch=int(rng.integers(*lim[3])), grid_size=N, cell_arcsec=1.5, n_power_law=2000, n_gauss=20,
                   noise_sigma=1e-3)
        out.append(dict(obs=obs, grid=dict(subgrid_size=subgrid_size, kernel_size=8, max_timesteps=1024,
                                           w_layers=w_layers)))
    return out


def build_geometry(workload):
    """uvw, frequencies and gridding constants of a workload without its sky (cheap)."""
    o, g = workload["obs"], workload["grid"]
    rng = np.random.default_rng(o["seed"])
    if o["layout"] == "uniform":
        ants = antennas_uniform_disk(rng, o["n_ant"], o["array_diameter_m"])
    else:
        ants = antennas_log_radial(rng, o["n_ant"], o["array_diameter_m"])
    uvw = earth_rotation_uvw(ants, o.get("lat_deg", -30.7215), o.get("dec_deg", -70.0), o["nt"], o["dump_s"])
    freqs = np.linspace(o["f_lo"], o["f_hi"], o["nch"])
    cell = cell_rad(o["cell_arcsec"])
    consts = dict(vis_count=int(uvw.shape[0] * uvw.shape[1] * o["nch"]), grid_size=o["grid_size"],
                  subgrid_size=g["subgrid_size"], kernel_size=g["kernel_size"], max_timesteps=g["max_timesteps"],
                  scale_arcsec=float(np.float32(cell)), wlayer_count=g["w_layers"],
                  wstep=wstep_for(uvw, freqs, g["w_layers"]))
    return uvw, freqs, consts


def scaled_workload(name, *, n_ant=None, nt=None, nch=None, seed=None):
    """A copy of a workload with fewer antennas/times/channels (parity-test sizes)."""
    w = WORKLOADS[name]
    obs = dict(w["obs"])
    if n_ant is not None:
        obs["n_ant"] = n_ant
    if nt is not None:
        obs["nt"] = nt
    if nch is not None:
        obs["nch"] = nch
    if seed is not None:
        obs["seed"] = seed
    return dict(obs=obs, grid=dict(w["grid"]))


def build(workload) -> tuple[Observation, dict]:
    """Observation plus the GriddingConstants arguments for a workload dict."""
    if isinstance(workload, str):
        workload = WORKLOADS[workload]
    obs = make_observation(**workload["obs"])
    g = workload["grid"]
    cell = cell_rad(workload["obs"]["cell_arcsec"])
    consts = dict(vis_count=obs.vis_count, grid_size=workload["obs"]["grid_size"],
                  subgrid_size=g["subgrid_size"], kernel_size=g["kernel_size"],
                  max_timesteps=g["max_timesteps"], scale_arcsec=float(np.float32(cell)),
                  wlayer_count=g["w_layers"], wstep=wstep_for(obs.uvw, obs.frequencies, g["w_layers"]))
    return obs, consts
