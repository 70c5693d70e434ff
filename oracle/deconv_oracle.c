/*
 * deconv_oracle.c -- CPU restatement of the deconvolution side of the reference's
 * serial major cycle (lord-blueberry/p9-distributed-reconstruction, C# project
 * "Core" and "SingleReconstruction"): the PSF helpers (Core/Common.cs PSF.*),
 * Residuals and ElasticNet, the padded Fourier correlation (Core/PaddedConvolver.cs),
 * the serial coordinate descent FastSerialCD (Core/Deconvolution/FastSerialCD.cs)
 * and the major-cycle loop MajorCycle.ReconstructSerialCD
 * (SingleReconstruction/MajorCycle.cs:33-134), which calls the gridder oracle in
 * idg_oracle.c.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it.  The product never
 * links or calls it.
 *
 * PARITY UNPINNED against the reference itself: the C# reference cannot be built
 * or run in this environment and ships no golden vectors.  The restatement keeps
 * the C# arithmetic types and evaluation order: images and the coordinate descent
 * in float (no FMA contraction; RyuJIT emits none), the prefix-sum scan of
 * PSF.CalcAMap and the FFT correlations in double, .NET Core 3.0 Math.Max(float)
 * (IEEE 754:2019 maximum), System.Numerics.Complex multiplication
 * (re = ac - bd, im = bc + ad), FFTW's sign and normalisation conventions.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* from idg_oracle.c */
typedef struct {
    int64_t vis_count;
    int32_t grid_size, subgrid_size, kernel_size, max_timesteps;
    float scale_arcsec;
    int32_t wlayer_count;
    double wstep;
} ocd_gparams;
typedef struct {
    int32_t baseline_idx, time_sample_start, time_sample_count, u_pixel, v_pixel, w_lambda;
} ocd_gsubgrid;
void oc_fft2d(double *data, int ny, int nx, int sign);
void oc_shift_float(float *img, int n);
void oc_shift_double(double *img, int n);
void oc_fft_forward_float(const float *img, int N, double norm, double *out);
void oc_wstack_ifft_float(const double *layers, int W, int N, int64_t vis_count, float *out);
int oc_idg_grid_w(const ocd_gparams *c, const ocd_gsubgrid *subs, int64_t nsub, const double *vis,
                  const double *uvw, int32_t nt, const double *freq, int32_t nch, double *layers_out);
int oc_idg_degrid_w(const ocd_gparams *c, const ocd_gsubgrid *subs, int64_t nsub, double *grid,
                    const double *uvw, int32_t nbl, int32_t nt, const double *freq, int32_t nch, double *vis_out);
void oc_unit_vis(const uint8_t *flags, int64_t n, double *vis);
void oc_vis_subtract(const double *v0, const double *v1, const uint8_t *flags, int64_t n, double *out);

#define OCD_OK 0
#define OCD_INVALID_ARGUMENT 1
#define OCD_OUT_OF_MEMORY 5
#define OCD_INDEX_OUT_OF_RANGE 10 /* the C# code would throw IndexOutOfRangeException */

/* .NET Core 3.0 Math.Max(float, float): IEEE 754:2019 maximum (NaN wins, +0 > -0). */
static float cs_maxf(float a, float b) {
    if (a != b) {
        if (!isnan(a)) return b < a ? a : b;
        return a;
    }
    return signbit(b) ? a : b;
}

/* ElasticNet.ProximalOperator (Common.cs:28-29). */
static float prox(float x, float lipschitz, float lambda, float alpha) {
    float t = lambda * alpha;
    float num = cs_maxf(x - t, 0.0f);
    float den = lipschitz + lambda * (1.0f - alpha);
    return num / den;
}

/* Common.ElasticNetPenalty (Common.cs:22-23): a float expression widened to double on return. */
static double elastic_penalty(float value, float alpha) {
    float q = (1.0f / 2.0f) * (1 - alpha) * (value * value);
    float r = alpha * fabsf(value);
    return (double)(q + r);
}

/* ElasticNet.CalcPenalty (Common.cs:31-41). */
double ocd_elastic_net_penalty(const float *img, int h, int w, float lambda, float alpha) {
    double out = 0;
    for (int64_t i = 0; i < (int64_t)h * w; i++) out += lambda * elastic_penalty(img[i], alpha);
    return out;
}

/* Residuals.GetMax (Common.cs:244-251): max(0, max pixel), .NET Math.Max. */
float ocd_get_max(const float *img, int64_t n) {
    float m = 0.0f;
    for (int64_t i = 0; i < n; i++) m = cs_maxf(m, img[i]);
    return m;
}

/* Residuals.CalcPenalty (Common.cs:253-260). */
double ocd_residual_penalty(const float *img, int64_t n) {
    double out = 0;
    for (int64_t i = 0; i < n; i++) out += img[i] * img[i];
    return 0.5 * out;
}

/* PSF.CalcMaxLipschitz (Common.cs:107-114): float products summed in double. */
double ocd_max_lipschitz(const float *psf, int h, int w) {
    double s = 0.0;
    for (int64_t i = 0; i < (int64_t)h * w; i++) s += psf[i] * psf[i];
    return s;
}

/* PSF.Cut (Common.cs:216-226) of a square n x n PSF. */
void ocd_psf_cut(const float *psf, int n, int factor, float *out) {
    int m = n / factor;
    int off = n / 2 - m / 2;
    for (int y = 0; y < m; y++)
        for (int x = 0; x < m; x++) out[(int64_t)y * m + x] = psf[(int64_t)(off + y) * n + off + x];
}

/* PSF.CalcMaxSidelobe (Common.cs:203-214) of a square n x n PSF. */
float ocd_max_sidelobe(const float *psf, int n, int factor) {
    int m = n / factor;
    int off = n / 2 - m / 2;
    float out = 0.0f;
    for (int y = 0; y < n; y++)
        for (int x = 0; x < n; x++)
            if (!(y >= off && y < off + m) || !(x >= off && x < off + m))
                out = cs_maxf(out, fabsf(psf[(int64_t)y * n + x]));
    return out;
}

/* The double prefix-sum scan of psf^2 in PSF.CalcAMap (Common.cs:84-93). */
void ocd_amap_scan(const float *psf, int h, int w, double *scan) {
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            double iBefore = i > 0 ? scan[(int64_t)(i - 1) * w + j] : 0.0;
            double jBefore = j > 0 ? scan[(int64_t)i * w + j - 1] : 0.0;
            double ijBefore = (i > 0 && j > 0) ? scan[(int64_t)(i - 1) * w + j - 1] : 0.0;
            float current = psf[(int64_t)i * w + j] * psf[(int64_t)i * w + j];
            scan[(int64_t)i * w + j] = (double)current + iBefore + jBefore - ijBefore;
        }
}

/* PSF.QueryScan (Common.cs:46-74). */
static double query_scan(const double *scan, int sh, int sw, int yPixel, int xPixel, int yLength, int xLength) {
#define S(a, b) scan[(int64_t)(a) * sw + (b)]
    int yOver = (yPixel + (sh - sh / 2)) - yLength;
    int xOver = (xPixel + (sw - sw / 2)) - xLength;
    yOver = yOver > 0 ? yOver : 0;
    xOver = xOver > 0 ? xOver : 0;
    int yUnder = (-1) * (yPixel - sh / 2);
    int xUnder = (-1) * (xPixel - sw / 2);
    int yUnderIdx = (yUnder > 1 ? yUnder : 1) - 1;
    int xUnderIdx = (xUnder > 1 ? xUnder : 1) - 1;
    if (yOver <= 0 && xOver <= 0 && yUnder <= 0 && xUnder <= 0) return S(sh - 1, sw - 1);
    if (yUnder > 0 && xUnder > 0)
        return S(sh - 1, sw - 1) - S(sh - 1, xUnderIdx) - S(yUnderIdx, sw - 1) + S(yUnderIdx, xUnderIdx);
    double correction = 0.0;
    if (yUnder > 0) correction += S(yUnderIdx, sw - xOver - 1);
    if (xUnder > 0) correction += S(sh - yOver - 1, xUnderIdx);
    return S(sh - 1 - yOver, sw - 1 - xOver) - correction;
#undef S
}

/* PSF.CalcAMap(psf, totalSize, imageSection) (Common.cs:81-105) with totalSize = (0,0,ty_end,tx_end)
 * and imageSection = (sy, sx, sy_end, sx_end); out is [sy_end-sy][sx_end-sx]. */
void ocd_amap(const float *psf, int h, int w, int ty_end, int tx_end, int sy, int sx, int sy_end, int sx_end,
              float *out) {
    double *scan = (double *)malloc(sizeof(double) * (size_t)h * w);
    ocd_amap_scan(psf, h, w, scan);
    int ow = sx_end - sx;
#pragma omp parallel for schedule(static)
    for (int y = sy; y < sy_end; y++)
        for (int x = sx; x < sx_end; x++)
            out[(int64_t)(y - sy) * ow + (x - sx)] = (float)query_scan(scan, h, w, y, x, ty_end, tx_end);
    free(scan);
}

/* FFT.Shift<T>(T[,]) (FFT.cs:248-264) on a square n x n array of 16-byte complex. */
static void shift_complex(double *a, int n) {
    int n2 = n / 2;
    for (int i = 0; i < n2; i++)
        for (int j = 0; j < n2; j++) {
            double t[2];
            double *p = a + 2 * ((int64_t)i * n + j), *q = a + 2 * ((int64_t)(i + n2) * n + j + n2);
            memcpy(t, p, 16); memcpy(p, q, 16); memcpy(q, t, 16);
            p = a + 2 * ((int64_t)(i + n2) * n + j);
            q = a + 2 * ((int64_t)i * n + j + n2);
            memcpy(t, p, 16); memcpy(p, q, 16); memcpy(q, t, 16);
        }
}

/* PSF.CalcPaddedFourierCorrelation (Common.cs:123-139): out complex [(pad_y + h)][(pad_x + w)].
 * The reference's FFT.Shift(double[,]) uses the row count for both axes, so the padded array
 * must be square (it is for every caller: square PSF, square padding). */
int ocd_padded_fourier_correlation(const float *psf, int h, int w, int pad_y, int pad_x, double *out) {
    int H = pad_y + h, W = pad_x + w;
    if (H != W) return OCD_INVALID_ARGUMENT;
    double *padded = (double *)calloc((size_t)H * W, sizeof(double));
    if (!padded) return OCD_OUT_OF_MEMORY;
    int yh = pad_y / 2, xh = pad_x / 2;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            if (y + yh + 1 < H && x + xh + 1 < W)
                padded[(int64_t)(y + yh + 1) * W + x + xh + 1] = psf[(int64_t)(h - y - 1) * w + (w - x - 1)];
    oc_shift_double(padded, H);
    for (int64_t i = 0; i < (int64_t)H * W; i++) { out[2 * i] = padded[i]; out[2 * i + 1] = 0.0; }
    free(padded);
    oc_fft2d(out, H, W, -1); /* FFT.Forward(double[,], 1.0): FFTW forward, / 1.0 is exact */
    return OCD_OK;
}

/* System.Numerics.Complex multiplication. */
static void cmul(const double *a, const double *b, double *o) {
    double re = a[0] * b[0] - a[1] * b[1];
    double im = a[1] * b[0] + a[0] * b[1];
    o[0] = re;
    o[1] = im;
}

/* PaddedConvolver(kernel, kernelSize).Convolve(image) (PaddedConvolver.cs:36-65, 87-107):
 * kernel complex [H][W]; kernel rectangle ky x kx; image and out float [n][n]. */
int ocd_padded_convolve(const double *kernel, int H, int W, int ky, int kx, const float *img, int n, float *out) {
    double *buf = (double *)calloc((size_t)H * W * 2, sizeof(double));
    if (!buf) return OCD_OUT_OF_MEMORY;
    int yh = ky / 2, xh = kx / 2;
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++)
            if (i >= yh && i < n + yh && j >= xh && j < n + xh) buf[2 * ((int64_t)i * W + j)] = img[(int64_t)(i - yh) * n + j - xh];
    oc_fft2d(buf, H, W, -1);
    for (int64_t i = 0; i < (int64_t)H * W; i++) cmul(buf + 2 * i, kernel + 2 * i, buf + 2 * i);
    oc_fft2d(buf, H, W, +1);
    const int32_t len = H * W; /* kernel.Length */
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            out[(int64_t)i * n + j] = (float)(buf[2 * ((int64_t)(i + yh) * W + j + xh)] / len);
    free(buf);
    return OCD_OK;
}

/* PSF.CalcPSFSquared (Common.cs:162-174) of an h x w PSF: out float [2h][2w]. */
int ocd_psf_squared(const float *psf, int h, int w, float *out) {
    int H = 2 * h, W = 2 * w;
    double *corr = (double *)malloc(sizeof(double) * 2 * (size_t)H * W);
    float *padded = (float *)calloc((size_t)H * W, sizeof(float));
    double *spec = (double *)malloc(sizeof(double) * 2 * (size_t)H * W);
    if (!corr || !padded || !spec) { free(corr); free(padded); free(spec); return OCD_OUT_OF_MEMORY; }
    int st = ocd_padded_fourier_correlation(psf, h, w, h, w, corr);
    if (st) { free(corr); free(padded); free(spec); return st; }
    /* SetPsfInWindow(psfPadded, psf, fullWindow, h, w) (Common.cs:176-195): every target is in the window */
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) padded[(int64_t)(i + h / 2) * W + j + w / 2] = psf[(int64_t)i * w + j];
    /* FFT.Forward(float[,]) (FFT.cs:99-117); square by construction */
    if (H == W) {
        oc_fft_forward_float(padded, H, 1.0, spec);
    } else {
        for (int64_t i = 0; i < (int64_t)H * W; i++) { spec[2 * i] = padded[i]; spec[2 * i + 1] = 0; }
        oc_fft2d(spec, H, W, -1);
    }
    for (int64_t i = 0; i < (int64_t)H * W; i++) cmul(spec + 2 * i, corr + 2 * i, spec + 2 * i);
    /* FFT.Backward(PSF2, (long)psfCorrelated.Length) (FFT.cs:159-185): Re(IFFT) / count */
    oc_fft2d(spec, H, W, +1);
    const int64_t count = (int64_t)H * W;
    for (int64_t i = 0; i < count; i++) out[i] = (float)(spec[2 * i] / (double)count);
    free(corr); free(padded); free(spec);
    return OCD_OK;
}

typedef struct {
    int32_t y, x;
    float diff, xnew;
} ocd_pixel;

/* FastSerialCD.GetAbsMax (FastSerialCD.cs:135-170) over the whole n x n image (patch = subpatch =
 * total size, offsets 0).  Rows are independent; the row winners are merged in row order. */
static ocd_pixel get_abs_max(const float *x, const float *g, const float *a, int n, float lambda, float alpha) {
    ocd_pixel *rows = (ocd_pixel *)malloc(sizeof(ocd_pixel) * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < n; y++) {
        ocd_pixel cur = {-1, -1, 0.0f, 0.0f};
        for (int xx = 0; xx < n; xx++) {
            int64_t i = (int64_t)y * n + xx;
            float currentA = a[i];
            float old = x[i];
            float xTmp = prox(old * currentA + g[i], currentA, lambda, alpha);
            float xDiff = old - xTmp;
            if (cur.diff < fabsf(xDiff)) {
                cur.y = y;
                cur.x = xx;
                cur.diff = fabsf(xDiff);
                cur.xnew = xTmp;
            }
        }
        rows[y] = cur;
    }
    ocd_pixel best = {-1, -1, 0.0f, 0.0f};
    for (int y = 0; y < n; y++)
        if (best.diff < rows[y].diff) best = rows[y];
    free(rows);
    return best;
}

/* FastSerialCD.UpdateGradients (FastSerialCD.cs:227-245). */
static void update_gradients(float *g, int n, const float *psf2, int ph, int pw, int yPixel, int xPixel, float xDiff) {
    int yh = ph / 2, xh = pw / 2;
    int yMin = yPixel - yh > 0 ? yPixel - yh : 0;
    int xMin = xPixel - xh > 0 ? xPixel - xh : 0;
    int yMax = yPixel - yh + ph < n ? yPixel - yh + ph : n;
    int xMax = xPixel - xh + pw < n ? xPixel - xh + pw : n;
#pragma omp parallel for schedule(static)
    for (int i = yMin; i < yMax; i++)
        for (int j = xMin; j < xMax; j++) {
            int yb = i + yh - yPixel, xb = j + xh - xPixel;
            float p = psf2[(int64_t)yb * pw + xb] * xDiff;
            g[(int64_t)i * n + j] += p;
        }
}

/* FastSerialCD.GetAbsMaxDiff (FastSerialCD.cs:129-132). */
float ocd_get_abs_max_diff(const float *x, const float *g, const float *a, int n, float lambda, float alpha) {
    return get_abs_max(x, g, a, n, lambda, alpha).diff;
}

/* The selected pixel of one GetAbsMax (for tests): out = {y, x}, returns diff, *xnew. */
float ocd_get_abs_max_pixel(const float *x, const float *g, const float *a, int n, float lambda, float alpha,
                            int32_t *yx, float *xnew) {
    ocd_pixel p = get_abs_max(x, g, a, n, lambda, alpha);
    yx[0] = p.y;
    yx[1] = p.x;
    *xnew = p.xnew;
    return p.diff;
}

/* FastSerialCD.Deconvolve (FastSerialCD.cs:76-102) on the whole image.  x and g (the bMap) are
 * updated in place.  Returns OCD_OK and *converged / *iterations, or OCD_INDEX_OUT_OF_RANGE where
 * the reference would index pixel (-1, -1) (no pixel changes while epsilon <= 0). */
int ocd_deconvolve(float *x, float *g, const float *a, int n, const float *psf2, int ph, int pw, float lambda,
                   float alpha, int32_t iterations, float epsilon, int32_t *converged_out, int32_t *iterations_out) {
    int converged = 0;
    int32_t iter = 0;
    while (!converged && iter < iterations) {
        ocd_pixel mp = get_abs_max(x, g, a, n, lambda, alpha);
        converged = mp.diff < epsilon;
        if (!converged) {
            if (mp.y < 0) {
                *converged_out = 0;
                *iterations_out = iter;
                return OCD_INDEX_OUT_OF_RANGE;
            }
            int64_t i = (int64_t)mp.y * n + mp.x;
            float old = x[i];
            x[i] = mp.xnew;
            update_gradients(g, n, psf2, ph, pw, mp.y, mp.x, old - mp.xnew);
            iter++;
        }
    }
    *converged_out = converged;
    *iterations_out = iter;
    return OCD_OK;
}

/* Per-cycle record of the major cycle (for the tests). */
typedef struct {
    float max_dirty, max_b, current_lambda, abs_max;
    int32_t deconvolved, converged, iterations, pad;
    double objective; /* MajorCycle.cs:102, before this cycle's Deconvolve */
} ocd_cycle;

/* MajorCycle.ReconstructSerialCD (MajorCycle.cs:33-134) with the CPU deconvolver (FastSerialCD,
 * MajorCycle.cs:65-70), without the FITS writes.  vis complex [nbl][nt][nch]; flags 1 byte each.
 * Outputs: model (xImage) and the last cycle's dirty (residual) image, float [N][N]; psf_out
 * (float [N][N], may be NULL); cycles[max_major]; *ncycles = cycles run. */
int ocd_major_cycle(const ocd_gparams *c, const ocd_gsubgrid *subs, int64_t nsub, const double *uvw, int32_t nbl,
                    int32_t nt, const double *freq, int32_t nch, const double *vis, const uint8_t *flags,
                    int32_t psf_cut_factor, int32_t max_major, float lambda, float alpha, int32_t deconv_iterations,
                    float deconv_epsilon, float *model, float *residual, float *psf_out, ocd_cycle *cycles,
                    int32_t *ncycles) {
    const float MAJOR_EPSILON = 1e-4f;
    const int N = c->grid_size, W = c->wlayer_count;
    const int64_t nn = (int64_t)N * N, nvis = (int64_t)nbl * nt * nch;
    int st = OCD_OK;
    double *layers = (double *)malloc(sizeof(double) * 2 * (size_t)nn * W);
    double *vbuf = (double *)malloc(sizeof(double) * 2 * (size_t)(nvis > 0 ? nvis : 1));
    double *resid = (double *)malloc(sizeof(double) * 2 * (size_t)(nvis > 0 ? nvis : 1));
    float *psf = (float *)malloc(sizeof(float) * (size_t)nn);
    double *xgrid = (double *)malloc(sizeof(double) * 2 * (size_t)nn);
    if (!layers || !vbuf || !resid || !psf || !xgrid) { st = OCD_OUT_OF_MEMORY; goto done; }
    *ncycles = 0;

    oc_unit_vis(flags, nvis, vbuf);
    if ((st = oc_idg_grid_w(c, subs, nsub, vbuf, uvw, nt, freq, nch, layers))) goto done;
    oc_wstack_ifft_float(layers, W, N, c->vis_count, psf);
    oc_shift_float(psf, N);
    if (psf_out) memcpy(psf_out, psf, sizeof(float) * (size_t)nn);

    const int P = N / psf_cut_factor;
    float *psf_cut = (float *)malloc(sizeof(float) * (size_t)P * P);
    float *psf2 = (float *)malloc(sizeof(float) * (size_t)4 * P * P);
    float *amap = (float *)malloc(sizeof(float) * (size_t)nn);
    double *kern = (double *)malloc(sizeof(double) * 2 * (size_t)(N + P) * (N + P));
    float *grad = (float *)malloc(sizeof(float) * (size_t)nn);
    if (!psf_cut || !psf2 || !amap || !kern || !grad) {
        free(psf_cut); free(psf2); free(amap); free(kern); free(grad);
        st = OCD_OUT_OF_MEMORY;
        goto done;
    }
    ocd_psf_cut(psf, N, psf_cut_factor, psf_cut);
    float max_sidelobe = ocd_max_sidelobe(psf, N, psf_cut_factor);
    /* new FastSerialCD(totalSize, psfCut) (FastSerialCD.cs:31-46) */
    if ((st = ocd_psf_squared(psf_cut, P, P, psf2))) goto inner_done;
    ocd_amap(psf_cut, P, P, N, N, 0, 0, N, N, amap);
    /* gCalculator = PaddedConvolver(CalcPaddedFourierCorrelation(psfCut, totalSize), psfCut rectangle) */
    if ((st = ocd_padded_fourier_correlation(psf_cut, P, P, N, N, kern))) goto inner_done;
    double max_lipschitz = ocd_max_lipschitz(psf_cut, P, P);
    float lambda_lipschitz = (float)(lambda * max_lipschitz);
    float lambda_true = (float)(lambda * ocd_max_lipschitz(psf, N, N));
    int switched = 0;

    memset(model, 0, sizeof(float) * (size_t)nn);
    memcpy(resid, vis, sizeof(double) * 2 * (size_t)nvis);
    for (int cycle = 0; cycle < max_major; cycle++) {
        ocd_cycle *rec = &cycles[cycle];
        memset(rec, 0, sizeof(*rec));
        if ((st = oc_idg_grid_w(c, subs, nsub, resid, uvw, nt, freq, nch, layers))) goto inner_done;
        oc_wstack_ifft_float(layers, W, N, c->vis_count, residual);
        oc_shift_float(residual, N);

        float max_dirty = ocd_get_max(residual, nn);
        if ((st = ocd_padded_convolve(kern, N + P, N + P, P, P, residual, N, grad))) goto inner_done;
        float max_b = ocd_get_max(grad, nn);
        double cf = (double)max_b / ((double)max_dirty * max_lipschitz);
        double correction = cf > 1.0 ? cf : (isnan(cf) ? cf : 1.0); /* Math.Max(double, 1.0f) */
        double side = (double)(max_b * max_sidelobe) * correction;
        double l1 = side / alpha;
        double l2 = (double)lambda_lipschitz;
        double lm = (l1 != l2) ? (!isnan(l1) ? (l2 < l1 ? l1 : l2) : l1) : (signbit(l2) ? l1 : l2);
        float current_lambda = (float)lm;
        float abs_max = ocd_get_abs_max_diff(model, grad, amap, N, lambda_true, alpha);
        /* objective = Residuals.CalcPenalty(dirtyImage) + ElasticNet.CalcPenalty(xImage, lambdaTrue, alpha) */
        rec->objective = ocd_residual_penalty(residual, nn) + ocd_elastic_net_penalty(model, N, N, lambda_true, alpha);
        rec->max_dirty = max_dirty;
        rec->max_b = max_b;
        rec->current_lambda = current_lambda;
        rec->abs_max = abs_max;
        if (abs_max >= MAJOR_EPSILON) {
            int32_t conv = 0, iters = 0;
            if ((st = ocd_deconvolve(model, grad, amap, N, psf2, 2 * P, 2 * P, current_lambda, alpha,
                                     deconv_iterations, deconv_epsilon, &conv, &iters)))
                goto inner_done;
            rec->deconvolved = 1;
            rec->converged = conv;
            rec->iterations = iters;
        }
        if (lambda == current_lambda && !switched) {
            /* MajorCycle.cs:109-115: only maxLipschitz changes what follows (the other
             * convolver is assigned but never used) */
            lambda = lambda_true;
            max_lipschitz = ocd_max_lipschitz(psf, N, N);
            switched = 1;
        }
        *ncycles = cycle + 1;
        if (abs_max < MAJOR_EPSILON) break;
        oc_shift_float(model, N);
        oc_fft_forward_float(model, N, 1.0, xgrid);
        oc_shift_float(model, N);
        if ((st = oc_idg_degrid_w(c, subs, nsub, xgrid, uvw, nbl, nt, freq, nch, vbuf))) goto inner_done;
        oc_vis_subtract(vis, vbuf, flags, nvis, resid);
    }
inner_done:
    free(psf_cut); free(psf2); free(amap); free(kern); free(grad);
done:
    free(layers); free(vbuf); free(resid); free(psf); free(xgrid);
    return st;
}
