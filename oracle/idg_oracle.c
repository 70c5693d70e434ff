/*
 * idg_oracle.c -- FP64 CPU restatement of the reference's image-domain gridder
 * (lord-blueberry/p9-distributed-reconstruction, C# project "Core").
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it.  The product
 * (the CUDA library) never links or calls it.
 *
 * PARITY UNPINNED against the reference itself: the reference is C# on
 * .NET Core 3.0, which cannot be built or run in this environment, and it
 * ships no tests, golden vectors or fixtures for this path.  The restatement
 * follows the C# source line by line (citations below), including its
 * arithmetic types (FP32 l/m/n, FP64 phase and accumulation), its evaluation
 * order, banker's rounding of Math.Round, NaN-propagating Math.Min/Max, the
 * .NET Core 3.0 x64 double->int conversion, and the quirks of the partitioner.
 * The FFTs follow FFTW's documented convention (FFTW_FORWARD = exp(-i),
 * FFTW_BACKWARD = exp(+i), both unnormalised), which is what the reference's
 * FFTW.NET 1.0.1 wrapper calls; the tests pin this FFT against numpy.fft.
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).  FMA
 * contraction must stay off so FP64/FP32 expressions round as the C# code does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OC_OK 0
#define OC_INVALID_ARGUMENT 1
#define OC_CANNOT_PLACE 2        /* Partitioner.cs:86,91 */
#define OC_SUBGRID_OUT_OF_GRID 3 /* Partitioner.cs:118 */
#define OC_INVALID_GRID 4        /* Adder.cs:49 */
#define OC_OUT_OF_MEMORY 5

static const double SPEED_OF_LIGHT = 299792458.0; /* MathFunctions.cs:11 */
static const double PI = 3.14159265358979323846;  /* System.Math.PI */

/* GriddingConstants (GriddingConstants.cs:11-52).  WStepLambda is never
 * assigned in the constructor and therefore 0.0f (GriddingConstants.cs:25). */
typedef struct {
    int64_t vis_count;
    int32_t grid_size;
    int32_t subgrid_size;
    int32_t kernel_size;
    int32_t max_timesteps;
    float scale_arcsec; /* cell size in radians, stored as float */
    int32_t wlayer_count;
    double wstep;
} oc_params;

/* Subgrid (Subgrid.cs:15-24). */
typedef struct {
    int32_t baseline_idx;
    int32_t time_sample_start;
    int32_t time_sample_count;
    int32_t u_pixel;
    int32_t v_pixel;
    int32_t w_lambda;
} oc_subgrid;

typedef struct { double re, im; } cplx;

/* ---------- .NET semantics helpers ---------- */

/* (int)x for double x as .NET Core 3.0 on x64 does it: truncation, and
 * 0x80000000 for NaN or values outside the int range. */
static int32_t cs_to_int(double x) {
    if (isnan(x) || x >= 2147483648.0 || x <= -2147483649.0) return INT32_MIN;
    return (int32_t)x;
}

/* Math.Min / Math.Max (double) of .NET Core 3.0: NaN-propagating, -0 < +0. */
static double cs_min(double a, double b) {
    if (a < b || isnan(a)) return a;
    if (a == b) return signbit(a) ? a : b;
    return b;
}
static double cs_max(double a, double b) {
    if (a > b || isnan(a)) return a;
    if (a == b) return signbit(a) ? b : a;
    return b;
}

/* Math.Round(double): round half to even (the default rounding mode). */
static double cs_round(double x) { return nearbyint(x); }

/* unchecked int32 arithmetic */
static int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

/* ---------- MathFunctions / GriddingConstants ---------- */

/* ImageSize = ScaleArcSec * GridSize, a float product (GriddingConstants.cs:42). */
static float image_size(const oc_params *c) { return c->scale_arcsec * (float)c->grid_size; }

/* FrequencyToWavenumber (MathFunctions.cs:107-113): 2.0f * Math.PI * f / c. */
static double wavenumber(double f) { return 2.0 * PI * f / SPEED_OF_LIGHT; }

/* Gridder.ComputeL (Gridder.cs:163-166), float arithmetic. */
static float compute_l(int x, int s, float imagesize) {
    float a = (float)(x - (s / 2)) + 0.5f;
    float b = a * imagesize;
    return b / (float)s;
}

/* Gridder.ComputeN (Gridder.cs:168-174): tmp / (float)(tmp/1.0f + Sqrt(1.0 - tmp)). */
static float compute_n(float l, float m) {
    float tmp = (l * l) + (m * m);
    double d = (double)(tmp / 1.0f) + sqrt(1.0 - (double)tmp);
    return tmp / (float)d;
}

/* ---------- Partitioner (Partitioner.cs:20-255) ---------- */

typedef struct { double u, v, w; } datapoint;

typedef struct {
    const oc_params *c;
    double umin, umax, vmin, vmax, uvwidth;
    int32_t upixel, vpixel, windex;
} part_subgrid;

static void ps_reset(part_subgrid *s) { /* Partitioner.cs:173-184 */
    s->umin = INFINITY; s->umax = -INFINITY; s->vmin = INFINITY; s->vmax = -INFINITY;
    s->uvwidth = 0; s->windex = 0; s->upixel = 0; s->vpixel = 0;
}

static int ps_add(part_subgrid *s, const datapoint *dp) { /* Partitioner.cs:186-221 */
    if (isinf(dp->u) || isinf(dp->v)) return 0;
    int32_t widx = 0;
    if (s->c->wstep != 0.0) widx = cs_to_int(floor(dp->w / s->c->wstep));
    if (!isinf(s->umin) && s->windex != widx) return 0;
    double umin_ = cs_min(s->umin, dp->u);
    double umax_ = cs_max(s->umax, dp->u);
    double vmin_ = cs_min(s->vmin, dp->v);
    double vmax_ = cs_max(s->vmax, dp->v);
    double w_ = cs_max(umax_ - umin_, vmax_ - vmin_);
    if ((w_ + (double)s->c->kernel_size) >= (double)s->c->subgrid_size) return 0;
    s->umin = umin_; s->umax = umax_; s->vmin = vmin_; s->vmax = vmax_;
    s->uvwidth = w_; s->windex = widx;
    return 1;
}

static void ps_finish(part_subgrid *s) { /* ComputeCoordinates, Partitioner.cs:236-248 */
    const oc_params *c = s->c;
    s->upixel = cs_to_int(cs_round((s->umax + s->umin) / 2));
    s->vpixel = cs_to_int(cs_round((s->vmax + s->vmin) / 2));
    s->upixel = wrap_add(s->upixel, c->grid_size / 2);
    s->vpixel = wrap_add(s->vpixel, c->grid_size / 2);
    s->upixel = wrap_add(s->upixel, -(c->subgrid_size / 2));
    s->vpixel = wrap_add(s->vpixel, -(c->subgrid_size / 2));
}

static int ps_in_range(const part_subgrid *s) { /* Partitioner.cs:223-234 */
    const oc_params *c = s->c;
    int32_t mx = s->upixel > s->vpixel ? s->upixel : s->vpixel;
    int32_t mn = s->upixel < s->vpixel ? s->upixel : s->vpixel;
    return mn >= 1 && mx <= (c->grid_size - c->subgrid_size) &&
           s->windex >= -c->wlayer_count && s->windex < c->wlayer_count;
}

/* MetersToPixels / MetersToLambda (Partitioner.cs:127-129). */
static double meters_to_pixels(double m, double imgsize, double f) { return m * imgsize * (f / SPEED_OF_LIGHT); }
static double meters_to_lambda(double m, double f) { return m * (f / SPEED_OF_LIGHT); }

/* Partitioner.CreatePartition.  Returns a malloc'd array in reference order
 * (baseline-major, then time) through *out; free with oc_free. */
int oc_partition(const oc_params *c, const double *uvw, int32_t nbl, int32_t nt,
                 const double *freq, int32_t nch, oc_subgrid **out, int64_t *n_out) {
    *out = NULL;
    *n_out = 0;
    if (nbl < 0 || nt < 0 || nch < 0) return OC_INVALID_ARGUMENT;
    if (nbl > 0 && nt > 0 && nch == 0) return OC_INVALID_ARGUMENT; /* datapoints[t, -1] throws */
    int64_t cap = 1024, n = 0;
    oc_subgrid *res = (oc_subgrid *)malloc(sizeof(oc_subgrid) * cap);
    if (!res) return OC_OUT_OF_MEMORY;
    const double imgsize = (double)image_size(c); /* Partitioner.cs:22, float */
    datapoint *dp0 = (datapoint *)malloc(sizeof(datapoint) * (size_t)(nt > 0 ? nt : 1));
    datapoint *dpm = (datapoint *)malloc(sizeof(datapoint) * (size_t)(nt > 0 ? nt : 1));
    if (!dp0 || !dpm) { free(res); free(dp0); free(dpm); return OC_OUT_OF_MEMORY; }
    int status = OC_OK;
    for (int32_t bl = 0; bl < nbl && status == OC_OK; bl++) {
        /* Partitioner.cs:30-47; only channel 0 and the last channel are used. */
        for (int32_t t = 0; t < nt; t++) {
            const double *p = uvw + ((int64_t)bl * nt + t) * 3;
            dp0[t].u = meters_to_pixels(p[0], imgsize, freq[0]);
            dp0[t].v = meters_to_pixels(p[1], imgsize, freq[0]);
            dp0[t].w = meters_to_lambda(p[2], freq[0]);
            dpm[t].u = meters_to_pixels(p[0], imgsize, freq[nch - 1]);
            dpm[t].v = meters_to_pixels(p[1], imgsize, freq[nch - 1]);
            /* "hack": the last channel carries channel 0's w (Partitioner.cs:61-62) */
            dpm[t].w = dp0[t].w;
        }
        part_subgrid sg;
        sg.c = c;
        ps_reset(&sg);
        int32_t time = 0;
        while (time < nt) { /* Partitioner.cs:51-121 */
            ps_reset(&sg);
            int32_t tsp = 0;
            for (; time < nt; time++) {
                if (ps_add(&sg, &dp0[time]) && ps_add(&sg, &dpm[time])) {
                    tsp++;
                    if (tsp == c->max_timesteps) { time++; break; }
                } else {
                    break;
                }
            }
            if (tsp == 0) { /* Partitioner.cs:80-99 */
                if (isinf(dp0[time].u) || isinf(dp0[time].v)) { status = OC_CANNOT_PLACE; break; }
                time++;
                continue;
            }
            ps_finish(&sg);
            if (!ps_in_range(&sg)) { status = OC_SUBGRID_OUT_OF_GRID; break; }
            if (n == cap) {
                cap *= 2;
                oc_subgrid *r2 = (oc_subgrid *)realloc(res, sizeof(oc_subgrid) * cap);
                if (!r2) { status = OC_OUT_OF_MEMORY; break; }
                res = r2;
            }
            res[n].baseline_idx = bl;
            res[n].time_sample_start = time - tsp;
            res[n].time_sample_count = tsp;
            res[n].u_pixel = sg.upixel;
            res[n].v_pixel = sg.vpixel;
            res[n].w_lambda = sg.windex;
            n++;
        }
    }
    free(dp0);
    free(dpm);
    if (status != OC_OK) { free(res); return status; }
    *out = res;
    *n_out = n;
    return OC_OK;
}

void oc_free(void *p) { free(p); }

/* ---------- FFT with FFTW's convention (sign -1: FFTW_FORWARD, +1: FFTW_BACKWARD) ---------- */

static void fft_rec(const cplx *in, int64_t is, cplx *out, int n, int N, const cplx *tw, cplx *scratch) {
    if (n == 1) { out[0] = in[0]; return; }
    int p;
    if (n % 4 == 0) p = 4;
    else if (n % 2 == 0) p = 2;
    else if (n % 3 == 0) p = 3;
    else if (n % 5 == 0) p = 5;
    else {
        p = n; /* prime length: direct DFT */
    }
    int m = n / p;
    for (int r = 0; r < p; r++) fft_rec(in + r * is, is * p, out + r * m, m, N, tw, scratch);
    /* X[k + q m] = sum_r W_n^{r (k + q m)} Y_r[k] */
    int64_t step = N / n;
    for (int k = 0; k < m; k++) {
        for (int q = 0; q < p; q++) {
            double re = 0, im = 0;
            for (int r = 0; r < p; r++) {
                int64_t e = ((int64_t)r * (k + (int64_t)q * m)) % n;
                cplx w = tw[e * step];
                cplx y = out[r * m + k];
                re += y.re * w.re - y.im * w.im;
                im += y.re * w.im + y.im * w.re;
            }
            scratch[q].re = re;
            scratch[q].im = im;
        }
        for (int q = 0; q < p; q++) out[k + q * m] = scratch[q];
    }
}

static cplx *make_twiddles(int n, int sign) {
    cplx *tw = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (int j = 0; j < n; j++) {
        double a = 2.0 * PI * (double)j / (double)n;
        tw[j].re = cos(a);
        tw[j].im = sign * sin(a);
    }
    return tw;
}

/* 1D transform of n points with input stride is; out contiguous. */
void oc_fft1d(const double *in, int64_t is, double *out, int n, int sign) {
    cplx *tw = make_twiddles(n, sign);
    cplx *scratch = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    fft_rec((const cplx *)in, is, (cplx *)out, n, n, tw, scratch);
    free(tw);
    free(scratch);
}

/* In-place 2D transform of a row-major [ny][nx] complex array. */
void oc_fft2d(double *data, int ny, int nx, int sign) {
    cplx *a = (cplx *)data;
    cplx *twx = make_twiddles(nx, sign);
    cplx *twy = make_twiddles(ny, sign);
    int nmax = nx > ny ? nx : ny;
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * (size_t)nmax);
        cplx *col = (cplx *)malloc(sizeof(cplx) * (size_t)nmax);
        cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)nmax);
#pragma omp for schedule(static)
        for (int y = 0; y < ny; y++) {
            fft_rec(a + (int64_t)y * nx, 1, buf, nx, nx, twx, scr);
            memcpy(a + (int64_t)y * nx, buf, sizeof(cplx) * nx);
        }
#pragma omp for schedule(static)
        for (int x = 0; x < nx; x++) {
            for (int y = 0; y < ny; y++) col[y] = a[(int64_t)y * nx + x];
            fft_rec(col, 1, buf, ny, ny, twy, scr);
            for (int y = 0; y < ny; y++) a[(int64_t)y * nx + x] = buf[y];
        }
        free(buf);
        free(col);
        free(scr);
    }
    free(twx);
    free(twy);
}

/* ---------- Gridder (Gridder.cs) ---------- */

/* Gridder.Forward (Gridder.cs:15-87) for the listed subgrids.  vis is
 * Complex[nbl][nt][nch] (re,im interleaved), uvw double[nbl][nt][3].
 * out: [nsub][S][S] complex, fftshifted as the reference writes it.
 * The baseline used for indexing is the subgrid's list position, stored in
 * baseline_idx (Gridder.cs:28,58). taper: float[S][S] or NULL (identity). */
void oc_gridder_forward(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *uvw,
                        int32_t nt, const double *vis, const double *freq, int32_t nch,
                        const float *taper, double *out) {
    const int S = c->subgrid_size, N = c->grid_size;
    const float imgsize = image_size(c);
    double *wn = (double *)malloc(sizeof(double) * (size_t)(nch > 0 ? nch : 1));
    for (int i = 0; i < nch; i++) wn[i] = wavenumber(freq[i]);
    const float wstep_lambda = 0.0f; /* GriddingConstants.WStepLambda, never assigned */
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t s = 0; s < nsub; s++) {
        const oc_subgrid *meta = &subs[s];
        const int bl = meta->baseline_idx;
        const double uoff = (double)(meta->u_pixel + S / 2 - N / 2) * (2 * PI / (double)imgsize);
        const double voff = (double)(meta->v_pixel + S / 2 - N / 2) * (2 * PI / (double)imgsize);
        const double tmpw = (double)wstep_lambda * ((double)meta->w_lambda + 0.5);
        const double woff = 2 * PI * tmpw;
        cplx *o = (cplx *)(out + (size_t)s * S * S * 2);
        for (int y = 0; y < S; y++) {
            for (int x = 0; x < S; x++) {
                double pre = 0, pim = 0;
                const float l = compute_l(x, S, imgsize);
                const float m = compute_l(y, S, imgsize);
                const float n = compute_n(l, m);
                const int end = meta->time_sample_start + meta->time_sample_count;
                for (int t = meta->time_sample_start; t < end; t++) {
                    const double *p = uvw + ((int64_t)bl * nt + t) * 3;
                    const double pidx = p[0] * (double)l + p[1] * (double)m + p[2] * (double)n;
                    const double poff = uoff * (double)l + voff * (double)m + woff * (double)n;
                    const double *vv = vis + (((int64_t)bl * nt + t) * nch) * 2;
                    for (int ch = 0; ch < nch; ch++) {
                        const double ph = poff - (pidx * wn[ch]);
                        const double cr = cos(ph), si = sin(ph);
                        const double vr = vv[2 * ch], vi = vv[2 * ch + 1];
                        pre += vr * cr - vi * si;
                        pim += vi * cr + vr * si;
                    }
                }
                const double sph = taper ? (double)taper[y * S + x] : 1.0;
                const int xd = (x + S / 2) % S, yd = (y + S / 2) % S;
                o[yd * S + xd].re = pre * sph;
                o[yd * S + xd].im = pim * sph;
            }
        }
    }
    free(wn);
}

/* Gridder.Backwards (Gridder.cs:91-160) for the listed subgrids.  data:
 * [nsub][S][S] (after SubgridFFT.Backward).  Writes vis_out[bl][t][ch] for
 * the samples each subgrid covers; other entries are left untouched (the
 * caller zero-initialises, as `new Complex[...]` does). */
void oc_gridder_backward(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *data,
                         const double *uvw, int32_t nt, const double *freq, int32_t nch,
                         const float *taper, double *vis_out) {
    const int S = c->subgrid_size, N = c->grid_size;
    const float imgsize = image_size(c);
    double *wn = (double *)malloc(sizeof(double) * (size_t)(nch > 0 ? nch : 1));
    for (int i = 0; i < nch; i++) wn[i] = wavenumber(freq[i]);
    const float wstep_lambda = 0.0f;
    /* l, m, n tables (same values ComputeL/ComputeN give inside the loop) */
    float *lt = (float *)malloc(sizeof(float) * S);
    float *nt_ = (float *)malloc(sizeof(float) * S * S);
    for (int x = 0; x < S; x++) lt[x] = compute_l(x, S, imgsize);
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) nt_[y * S + x] = compute_n(lt[x], lt[y]);
    const double scale = (double)(1.0f / (float)(S * S)); /* Gridder.cs:151 */
#pragma omp parallel
    {
        cplx *pix = (cplx *)malloc(sizeof(cplx) * S * S);
#pragma omp for schedule(dynamic, 1)
        for (int64_t s = 0; s < nsub; s++) {
            const oc_subgrid *meta = &subs[s];
            const int bl = meta->baseline_idx;
            const cplx *d = (const cplx *)(data + (size_t)s * S * S * 2);
            for (int y = 0; y < S; y++)
                for (int x = 0; x < S; x++) {
                    const double sph = taper ? (double)taper[y * S + x] : 1.0;
                    const int xs = (x + S / 2) % S, ys = (y + S / 2) % S;
                    pix[y * S + x].re = sph * d[ys * S + xs].re;
                    pix[y * S + x].im = sph * d[ys * S + xs].im;
                }
            const double uoff = (double)(meta->u_pixel + S / 2 - N / 2) * (2 * PI / (double)imgsize);
            const double voff = (double)(meta->v_pixel + S / 2 - N / 2) * (2 * PI / (double)imgsize);
            const double tmpw = (double)wstep_lambda * ((double)meta->w_lambda + 0.5);
            const double woff = 2 * PI * tmpw;
            const int end = meta->time_sample_start + meta->time_sample_count;
            for (int t = meta->time_sample_start; t < end; t++) {
                const double *p = uvw + ((int64_t)bl * nt + t) * 3;
                double *vo = vis_out + (((int64_t)bl * nt + t) * nch) * 2;
                for (int ch = 0; ch < nch; ch++) {
                    double vr = 0, vi = 0;
                    for (int y = 0; y < S; y++) {
                        for (int x = 0; x < S; x++) {
                            const float l = lt[x], m = lt[y], n = nt_[y * S + x];
                            const double pidx = p[0] * (double)l + p[1] * (double)m + p[2] * (double)n;
                            const double poff = uoff * (double)l + voff * (double)m + woff * (double)n;
                            const double ph = (pidx * wn[ch]) - poff;
                            const double cr = cos(ph), si = sin(ph);
                            const cplx q = pix[y * S + x];
                            vr += q.re * cr - q.im * si;
                            vi += q.im * cr + q.re * si;
                        }
                    }
                    vo[2 * ch] = vr * scale;
                    vo[2 * ch + 1] = vi * scale;
                }
            }
        }
        free(pix);
    }
    free(lt);
    free(nt_);
    free(wn);
}

/* ---------- SubgridFFT (SubgridFFT.cs) ---------- */

/* SubgridFFT.Forward (SubgridFFT.cs:11-52): FFTW backward, times 1/S^2. */
void oc_subgrid_fft_forward(const oc_params *c, int64_t nsub, double *data) {
    const int S = c->subgrid_size;
    const double norm = 1.0 / (double)(S * S);
    cplx *tw = make_twiddles(S, +1);
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * S), *col = (cplx *)malloc(sizeof(cplx) * S);
        cplx *scr = (cplx *)malloc(sizeof(cplx) * S);
#pragma omp for schedule(static)
        for (int64_t s = 0; s < nsub; s++) {
            cplx *a = (cplx *)(data + (size_t)s * S * S * 2);
            for (int y = 0; y < S; y++) {
                fft_rec(a + y * S, 1, buf, S, S, tw, scr);
                memcpy(a + y * S, buf, sizeof(cplx) * S);
            }
            for (int x = 0; x < S; x++) {
                for (int y = 0; y < S; y++) col[y] = a[y * S + x];
                fft_rec(col, 1, buf, S, S, tw, scr);
                for (int y = 0; y < S; y++) a[y * S + x] = buf[y];
            }
            for (int i = 0; i < S * S; i++) { a[i].re *= norm; a[i].im *= norm; }
        }
        free(buf); free(col); free(scr);
    }
    free(tw);
}

/* SubgridFFT.Backward (SubgridFFT.cs:54-90): FFTW forward, unnormalised. */
void oc_subgrid_fft_backward(const oc_params *c, int64_t nsub, double *data) {
    const int S = c->subgrid_size;
    cplx *tw = make_twiddles(S, -1);
#pragma omp parallel
    {
        cplx *buf = (cplx *)malloc(sizeof(cplx) * S), *col = (cplx *)malloc(sizeof(cplx) * S);
        cplx *scr = (cplx *)malloc(sizeof(cplx) * S);
#pragma omp for schedule(static)
        for (int64_t s = 0; s < nsub; s++) {
            cplx *a = (cplx *)(data + (size_t)s * S * S * 2);
            for (int y = 0; y < S; y++) {
                fft_rec(a + y * S, 1, buf, S, S, tw, scr);
                memcpy(a + y * S, buf, sizeof(cplx) * S);
            }
            for (int x = 0; x < S; x++) {
                for (int y = 0; y < S; y++) col[y] = a[y * S + x];
                fft_rec(col, 1, buf, S, S, tw, scr);
                for (int y = 0; y < S; y++) a[y * S + x] = buf[y];
            }
        }
        free(buf); free(col); free(scr);
    }
    free(tw);
}

/* ---------- Adder / AdderWStack ---------- */

/* Adder.Add (Adder.cs:13-55).  grid [N][N] complex, zero-initialised by the caller. */
int oc_adder_add(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *data, double *grid) {
    const int S = c->subgrid_size, N = c->grid_size;
    cplx *g = (cplx *)grid;
    for (int64_t s = 0; s < nsub; s++) {
        const int gx = subs[s].u_pixel, gy = subs[s].v_pixel;
        if (!(gx >= 0 && gx < N - S && gy >= 0 && gy < N - S)) return OC_INVALID_GRID;
        const cplx *d = (const cplx *)(data + (size_t)s * S * S * 2);
        for (int y = 0; y < S; y++)
            for (int x = 0; x < S; x++) {
                const int xs = (x + S / 2) % S, ys = (y + S / 2) % S;
                const double ph = PI * (double)(x + y - S) / (double)S;
                const double pr = cos(ph), pi_ = sin(ph);
                const cplx v = d[ys * S + xs];
                cplx *o = &g[(int64_t)(gy + y) * N + gx + x];
                o->re += v.re * pr - v.im * pi_;
                o->im += v.im * pr + v.re * pi_;
            }
    }
    return OC_OK;
}

/* Adder.Split (Adder.cs:57-95).  out [nsub][S][S], zeroed here. */
void oc_adder_split(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *grid, double *out) {
    const int S = c->subgrid_size, N = c->grid_size;
    const cplx *g = (const cplx *)grid;
    memset(out, 0, sizeof(double) * 2 * (size_t)nsub * S * S);
    for (int64_t s = 0; s < nsub; s++) {
        const int gx = subs[s].u_pixel, gy = subs[s].v_pixel;
        cplx *d = (cplx *)(out + (size_t)s * S * S * 2);
        if (!(gx >= 0 && gx < N - S && gy >= 0 && gy < N - S)) continue;
        for (int y = 0; y < S; y++)
            for (int x = 0; x < S; x++) {
                const int xd = (x + S / 2) % S, yd = (y + S / 2) % S;
                const double ph = -PI * (double)(x + y - S) / (double)S;
                const double pr = cos(ph), pi_ = sin(ph);
                const cplx v = g[(int64_t)(gy + y) * N + gx + x];
                d[yd * S + xd].re = v.re * pr - v.im * pi_;
                d[yd * S + xd].im = v.im * pr + v.re * pi_;
            }
    }
}

/* AdderWStack.Add (AdderWStack.cs:11-78).  layers [W][N][N] complex, zero-initialised. */
int oc_adder_wstack_add(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *data, double *layers) {
    const int S = c->subgrid_size, N = c->grid_size, W = c->wlayer_count;
    cplx *ph = (cplx *)malloc(sizeof(cplx) * S * S);
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) {
            const double a = PI * (double)(x + y - S) / (double)S;
            ph[y * S + x].re = cos(a);
            ph[y * S + x].im = sin(a);
        }
    int status = OC_OK;
    for (int64_t s = 0; s < nsub; s++) {
        int sx = subs[s].u_pixel, sy = subs[s].v_pixel, sw = subs[s].w_lambda;
        const int neg = sw < 0;
        if (neg) { sx = N - sx - S + 1; sy = N - sy - S + 1; sw = -sw - 1; }
        if (!(sx >= 1 && sx < N - S && sy >= 1 && sy < N - S)) continue;
        if (sw >= W) { status = OC_INVALID_ARGUMENT; break; } /* grid[subgridW] out of range */
        const cplx *d = (const cplx *)(data + (size_t)s * S * S * 2);
        cplx *g = (cplx *)(layers + (size_t)sw * N * N * 2);
        for (int y = 0; y < S; y++) {
            const int y_ = neg ? S - 1 - y : y;
            for (int x = 0; x < S; x++) {
                const int x_ = neg ? S - 1 - x : x;
                const int xs = (x_ + S / 2) % S, ys = (y_ + S / 2) % S;
                const cplx p = ph[y_ * S + x_];
                const cplx v = d[ys * S + xs];
                double re = p.re * v.re - p.im * v.im;
                double im = p.im * v.re + p.re * v.im;
                if (neg) im = -im;
                cplx *o = &g[(int64_t)(sy + y) * N + sx + x];
                o->re += re;
                o->im += im;
            }
        }
    }
    free(ph);
    return status;
}

/* AdderWStack.Split (AdderWStack.cs:81-139).  Reads ONE grid; out [nsub][S][S], zeroed here. */
void oc_adder_wstack_split(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *grid, double *out) {
    const int S = c->subgrid_size, N = c->grid_size;
    const cplx *g = (const cplx *)grid;
    cplx *ph = (cplx *)malloc(sizeof(cplx) * S * S);
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) {
            const double a = -PI * (double)(x + y - S) / (double)S;
            ph[y * S + x].re = cos(a);
            ph[y * S + x].im = sin(a);
        }
    memset(out, 0, sizeof(double) * 2 * (size_t)nsub * S * S);
    for (int64_t s = 0; s < nsub; s++) {
        const int sx = subs[s].u_pixel, sy = subs[s].v_pixel, sw = subs[s].w_lambda;
        const int neg = sw < 0;
        cplx *d = (cplx *)(out + (size_t)s * S * S * 2);
        if (!(sx >= 1 && sx < N - S && sy >= 1 && sy < N - S)) continue;
        for (int y = 0; y < S; y++)
            for (int x = 0; x < S; x++) {
                const int xd = (x + S / 2) % S, yd = (y + S / 2) % S;
                const int xs = neg ? N - sx - x : sx + x;
                const int ys = neg ? N - sy - y : sy + y;
                const cplx p = ph[y * S + x];
                cplx v = g[(int64_t)ys * N + xs];
                if (neg) v.im = -v.im;
                d[yd * S + xd].re = p.re * v.re - p.im * v.im;
                d[yd * S + xd].im = p.im * v.re + p.re * v.im;
            }
    }
    free(ph);
}

/* ---------- FFT.cs helpers ---------- */

/* FFT.Shift (FFT.cs:221-264): quadrant swap with n2 = n/2 (square arrays).
 * elem_doubles: 2 for Complex, 1 for double; works on a [n][n] array. */
static void shift_generic(void *a, int n, size_t esz) {
    char *p = (char *)a;
    const int n2 = n / 2;
    char tmp[16];
    for (int i = 0; i < n2; i++)
        for (int j = 0; j < n2; j++) {
            char *a13 = p + ((size_t)i * n + j) * esz, *b13 = p + ((size_t)(i + n2) * n + j + n2) * esz;
            memcpy(tmp, a13, esz); memcpy(a13, b13, esz); memcpy(b13, tmp, esz);
            char *a24 = p + ((size_t)(i + n2) * n + j) * esz, *b24 = p + ((size_t)i * n + j + n2) * esz;
            memcpy(tmp, a24, esz); memcpy(a24, b24, esz); memcpy(b24, tmp, esz);
        }
}
void oc_shift_complex(double *grid, int n) { shift_generic(grid, n, 16); }
void oc_shift_double(double *img, int n) { shift_generic(img, n, 8); }
void oc_shift_float(float *img, int n) { shift_generic(img, n, 4); }

/* FFT.WStackIFFTFloat (FFT.cs:188-215): for each layer FFTW backward, out += (float)(Re / visCount).
 * layers [W][N][N] complex (not modified). out float [N][N]. */
void oc_wstack_ifft_float(const double *layers, int W, int N, int64_t vis_count, float *out) {
    double *buf = (double *)malloc(sizeof(double) * 2 * (size_t)N * N);
    memset(out, 0, sizeof(float) * (size_t)N * N);
    for (int k = 0; k < W; k++) {
        memcpy(buf, layers + (size_t)k * N * N * 2, sizeof(double) * 2 * (size_t)N * N);
        oc_fft2d(buf, N, N, +1);
        for (int64_t i = 0; i < (int64_t)N * N; i++) out[i] += (float)(buf[2 * i] / (double)vis_count);
    }
    free(buf);
}

/* FFT.Backward(Complex[,] grid, long visibilityCount) (FFT.cs:159-185): Re(IFFT)/visCount, double. */
void oc_fft_backward_real(const double *grid, int N, int64_t vis_count, double *out) {
    double *buf = (double *)malloc(sizeof(double) * 2 * (size_t)N * N);
    memcpy(buf, grid, sizeof(double) * 2 * (size_t)N * N);
    oc_fft2d(buf, N, N, +1);
    for (int64_t i = 0; i < (int64_t)N * N; i++) out[i] = buf[2 * i] / (double)vis_count;
    free(buf);
}

/* FFT.Forward(float[,] image, double norm = 1.0) (FFT.cs:99-117): FFTW forward / norm. */
void oc_fft_forward_float(const float *img, int N, double norm, double *out) {
    for (int64_t i = 0; i < (int64_t)N * N; i++) { out[2 * i] = (double)img[i]; out[2 * i + 1] = 0.0; }
    oc_fft2d(out, N, N, -1);
    for (int64_t i = 0; i < 2 * (int64_t)N * N; i++) out[i] = out[i] / norm;
}

/* ---------- IDG facade (IDG.cs) ---------- */

static double *alloc_sub(const oc_params *c, int64_t nsub) {
    size_t n = (size_t)(nsub > 0 ? nsub : 1) * c->subgrid_size * c->subgrid_size * 2;
    return (double *)calloc(n, sizeof(double));
}

/* IDG.Grid (IDG.cs:12-20): grid_out [N][N] complex. */
int oc_idg_grid(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *vis, const double *uvw,
                int32_t nt, const double *freq, int32_t nch, double *grid_out) {
    double *sub = alloc_sub(c, nsub);
    if (!sub) return OC_OUT_OF_MEMORY;
    oc_gridder_forward(c, subs, nsub, uvw, nt, vis, freq, nch, NULL, sub);
    oc_subgrid_fft_forward(c, nsub, sub);
    memset(grid_out, 0, sizeof(double) * 2 * (size_t)c->grid_size * c->grid_size);
    int st = oc_adder_add(c, subs, nsub, sub, grid_out);
    free(sub);
    if (st) return st;
    oc_shift_complex(grid_out, c->grid_size);
    return OC_OK;
}

/* IDG.GridW (IDG.cs:32-40): layers_out [W][N][N] complex. */
int oc_idg_grid_w(const oc_params *c, const oc_subgrid *subs, int64_t nsub, const double *vis, const double *uvw,
                  int32_t nt, const double *freq, int32_t nch, double *layers_out) {
    double *sub = alloc_sub(c, nsub);
    if (!sub) return OC_OUT_OF_MEMORY;
    oc_gridder_forward(c, subs, nsub, uvw, nt, vis, freq, nch, NULL, sub);
    oc_subgrid_fft_forward(c, nsub, sub);
    const size_t nn = (size_t)c->grid_size * c->grid_size;
    memset(layers_out, 0, sizeof(double) * 2 * nn * c->wlayer_count);
    int st = oc_adder_wstack_add(c, subs, nsub, sub, layers_out);
    free(sub);
    if (st) return st;
    for (int k = 0; k < c->wlayer_count; k++) oc_shift_complex(layers_out + 2 * nn * k, c->grid_size);
    return OC_OK;
}

/* IDG.DeGrid (IDG.cs:22-30): shifts grid in place (as the reference does), vis_out [nbl][nt][nch]. */
int oc_idg_degrid(const oc_params *c, const oc_subgrid *subs, int64_t nsub, double *grid, const double *uvw,
                  int32_t nbl, int32_t nt, const double *freq, int32_t nch, double *vis_out) {
    oc_shift_complex(grid, c->grid_size);
    double *sub = alloc_sub(c, nsub);
    if (!sub) return OC_OUT_OF_MEMORY;
    oc_adder_split(c, subs, nsub, grid, sub);
    oc_subgrid_fft_backward(c, nsub, sub);
    memset(vis_out, 0, sizeof(double) * 2 * (size_t)nbl * nt * nch);
    oc_gridder_backward(c, subs, nsub, sub, uvw, nt, freq, nch, NULL, vis_out);
    free(sub);
    return OC_OK;
}

/* IDG.DeGridW (IDG.cs:42-50). */
int oc_idg_degrid_w(const oc_params *c, const oc_subgrid *subs, int64_t nsub, double *grid, const double *uvw,
                    int32_t nbl, int32_t nt, const double *freq, int32_t nch, double *vis_out) {
    oc_shift_complex(grid, c->grid_size);
    double *sub = alloc_sub(c, nsub);
    if (!sub) return OC_OUT_OF_MEMORY;
    oc_adder_wstack_split(c, subs, nsub, grid, sub);
    oc_subgrid_fft_backward(c, nsub, sub);
    memset(vis_out, 0, sizeof(double) * 2 * (size_t)nbl * nt * nch);
    oc_gridder_backward(c, subs, nsub, sub, uvw, nt, freq, nch, NULL, vis_out);
    free(sub);
    return OC_OK;
}

/* Unit visibilities where unflagged (IDG.cs:52-66, 85-98). flags: 1 byte per sample. */
void oc_unit_vis(const uint8_t *flags, int64_t n, double *vis) {
    for (int64_t i = 0; i < n; i++) { vis[2 * i] = flags[i] ? 0.0 : 1.0; vis[2 * i + 1] = 0.0; }
}

/* Visibilities.Substract (Common.cs:305-317). */
void oc_vis_subtract(const double *v0, const double *v1, const uint8_t *flags, int64_t n, double *out) {
    for (int64_t i = 0; i < n; i++) {
        if (!flags[i]) { out[2 * i] = v0[2 * i] - v1[2 * i]; out[2 * i + 1] = v0[2 * i + 1] - v1[2 * i + 1]; }
        else { out[2 * i] = 0; out[2 * i + 1] = 0; }
    }
}

int oc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
