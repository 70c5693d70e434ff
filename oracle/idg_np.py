"""Vectorised numpy restatement of the reference IDG path (second oracle).

TEST INFRASTRUCTURE ONLY.  Written independently of idg_oracle.c in array
form, so the two restatements cross-check each other's indexing, shifts,
mirroring and conventions.  Only small cases (a few subgrids) are practical.
Parity with the C# reference itself is unpinned (see idg_oracle.c).

FFTs use numpy.fft: numpy's fft2 is FFTW_FORWARD's convention (exp(-i),
unnormalised) and ifft2 * n is FFTW_BACKWARD's (exp(+i), unnormalised).
"""
from __future__ import annotations

import math

import numpy as np

SPEED_OF_LIGHT = 299792458.0


def image_size(c):
    return np.float32(c["scale_arcsec"]) * np.float32(c["grid_size"])


def lmn(c):
    """Gridder.ComputeL / ComputeN tables in float32 (Gridder.cs:163-174)."""
    S = c["subgrid_size"]
    img = image_size(c)
    x = np.arange(S)
    l = ((x - S // 2).astype(np.float32) + np.float32(0.5)) * img / np.float32(S)
    L = np.broadcast_to(l[None, :], (S, S)).astype(np.float32)
    M = np.broadcast_to(l[:, None], (S, S)).astype(np.float32)
    tmp = L * L + M * M
    den = (tmp.astype(np.float64) + np.sqrt(1.0 - tmp.astype(np.float64))).astype(np.float32)
    return l.astype(np.float32), (tmp / den).astype(np.float32)


def wavenumbers(freq):
    return 2.0 * math.pi * np.asarray(freq, np.float64) / SPEED_OF_LIGHT


def _offsets(c, sg):
    S, N = c["subgrid_size"], c["grid_size"]
    img = float(image_size(c))
    uoff = (int(sg["u_pixel"]) + S // 2 - N // 2) * (2 * math.pi / img)
    voff = (int(sg["v_pixel"]) + S // 2 - N // 2) * (2 * math.pi / img)
    return uoff, voff, 0.0  # wOffset = 2 pi WStepLambda (...) = 0


def gridder_forward(c, subs, uvw, vis, freq):
    S = c["subgrid_size"]
    l, n = lmn(c)
    L = np.broadcast_to(l[None, :], (S, S)).astype(np.float64)
    M = np.broadcast_to(l[:, None], (S, S)).astype(np.float64)
    Nn = n.astype(np.float64)
    k = wavenumbers(freq)
    out = np.zeros((len(subs), S, S), np.complex128)
    for i, sg in enumerate(subs):
        bl, t0, nt = int(sg["baseline_idx"]), int(sg["time_sample_start"]), int(sg["time_sample_count"])
        uoff, voff, woff = _offsets(c, sg)
        u = uvw[bl, t0:t0 + nt, 0][:, None, None]
        v = uvw[bl, t0:t0 + nt, 1][:, None, None]
        w = uvw[bl, t0:t0 + nt, 2][:, None, None]
        pidx = u * L + v * M + w * Nn                               # [t][y][x]
        poff = uoff * L + voff * M + woff * Nn                      # [y][x]
        phase = poff[None, None] - pidx[:, None] * k[None, :, None, None]   # [t][ch][y][x]
        vv = vis[bl, t0:t0 + nt, :][:, :, None, None]
        pix = np.sum(vv * np.exp(1j * phase), axis=(0, 1))
        out[i] = np.roll(pix, (S // 2, S // 2), axis=(0, 1))        # dest (y+S/2)%S
    return out


def gridder_backward(c, subs, data, uvw, freq, nbl, nt_all):
    S = c["subgrid_size"]
    l, n = lmn(c)
    L = np.broadcast_to(l[None, :], (S, S)).astype(np.float64)
    M = np.broadcast_to(l[:, None], (S, S)).astype(np.float64)
    Nn = n.astype(np.float64)
    k = wavenumbers(freq)
    out = np.zeros((nbl, nt_all, len(freq)), np.complex128)
    scale = float(np.float32(1.0) / np.float32(S * S))
    for i, sg in enumerate(subs):
        bl, t0, nt = int(sg["baseline_idx"]), int(sg["time_sample_start"]), int(sg["time_sample_count"])
        pix = np.roll(data[i], (-(S // 2), -(S // 2)), axis=(0, 1))  # src (y+S/2)%S
        uoff, voff, woff = _offsets(c, sg)
        u = uvw[bl, t0:t0 + nt, 0][:, None, None]
        v = uvw[bl, t0:t0 + nt, 1][:, None, None]
        w = uvw[bl, t0:t0 + nt, 2][:, None, None]
        pidx = u * L + v * M + w * Nn
        poff = uoff * L + voff * M + woff * Nn
        phase = pidx[:, None] * k[None, :, None, None] - poff[None, None]
        out[bl, t0:t0 + nt, :] = np.sum(pix[None, None] * np.exp(1j * phase), axis=(2, 3)) * scale
    return out


def subgrid_fft_forward(c, data):
    S = c["subgrid_size"]
    return np.fft.ifft2(data, axes=(-2, -1)) * (S * S) * (1.0 / (S * S))


def subgrid_fft_backward(c, data):
    return np.fft.fft2(data, axes=(-2, -1))


def _add_phasor(S, sign):
    x = np.arange(S)
    ph = sign * math.pi * (x[None, :] + x[:, None] - S) / S
    return np.exp(1j * ph)


def adder_wstack_add(c, subs, data):
    S, N, W = c["subgrid_size"], c["grid_size"], c["wlayer_count"]
    layers = np.zeros((W, N, N), np.complex128)
    ph = _add_phasor(S, +1.0)
    for i, sg in enumerate(subs):
        x0, y0, w = int(sg["u_pixel"]), int(sg["v_pixel"]), int(sg["w_lambda"])
        blk = ph * np.roll(data[i], (-(S // 2), -(S // 2)), axis=(0, 1))   # value at sub pixel (y_, x_)
        if w < 0:
            x0, y0, w = N - x0 - S + 1, N - y0 - S + 1, -w - 1
            blk = np.conj(blk[::-1, ::-1])
        if not (1 <= x0 < N - S and 1 <= y0 < N - S):
            continue
        layers[w, y0:y0 + S, x0:x0 + S] += blk
    return layers


def adder_wstack_split(c, subs, grid):
    S, N = c["subgrid_size"], c["grid_size"]
    out = np.zeros((len(subs), S, S), np.complex128)
    ph = _add_phasor(S, -1.0)
    for i, sg in enumerate(subs):
        x0, y0, w = int(sg["u_pixel"]), int(sg["v_pixel"]), int(sg["w_lambda"])
        if not (1 <= x0 < N - S and 1 <= y0 < N - S):
            continue
        if w < 0:
            ys = N - y0 - np.arange(S)
            xs = N - x0 - np.arange(S)
            blk = np.conj(grid[np.ix_(ys, xs)])
        else:
            blk = grid[y0:y0 + S, x0:x0 + S]
        out[i] = np.roll(ph * blk, (S // 2, S // 2), axis=(0, 1))
    return out


def fft_shift(a):
    n = a.shape[0]
    n2 = n // 2
    b = a.copy()
    b[:n2, :n2], b[n2:2 * n2, n2:2 * n2] = a[n2:2 * n2, n2:2 * n2], a[:n2, :n2]
    b[n2:2 * n2, :n2], b[:n2, n2:2 * n2] = a[:n2, n2:2 * n2], a[n2:2 * n2, :n2]
    return b


def wstack_ifft_float(layers, vis_count):
    N = layers.shape[-1]
    out = np.zeros((N, N), np.float32)
    for L in layers:
        out += (np.fft.ifft2(L) * (N * N)).real.astype(np.float64).__truediv__(vis_count).astype(np.float32)
    return out
