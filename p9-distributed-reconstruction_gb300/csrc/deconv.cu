// Deconvolution side of the serial major cycle on the GPU:
//   * serial coordinate descent, Core/Deconvolution/FastSerialCD.cs (Deconvolve, DeconvolvePath,
//     GetAbsMaxDiff, ResetLipschitzMap), bit-identical to the C# arithmetic: float values, no
//     FMA contraction, the same pixel choice (largest |change|, first in row-major order);
//   * the PSF preparation of Core/Common.cs (PSF.CalcPaddedFourierCorrelation, CalcPSFSquared,
//     CalcAMap, Cut, CalcMaxSidelobe, CalcMaxLipschitz, Residuals.GetMax) and the padded FFT
//     correlation of Core/PaddedConvolver.cs, in FP64 with cuFFT as the reference does with FFTW;
//   * MajorCycle.ReconstructSerialCD (SingleReconstruction/MajorCycle.cs:33-134) with the
//     visibilities, grids and images resident in HBM.
//
// Coordinate descent.  One iteration of FastSerialCD picks the pixel whose proximal update
// changes it most (a scan of the whole image), sets it, and adds the scaled PSF^2 to the
// gradient map in a window around it.  Only pixels in that window change, so the GPU keeps
// the best candidate of every 40 x 128 tile and, per iteration, re-evaluates only the tiles
// the window touches: one launch reduces the tile candidates the previous launch left to the
// selected pixel (every CTA does this itself), updates the window's gradients and writes those
// tiles' new candidates into the other of two state buffers.  A candidate is one 64-bit key,
// (|change| bits << 32) | (0xFFFFFFFF - pixel index), so the largest key is the largest change
// and, among equal changes, the first pixel, which is the order in which GetAbsMax
// (FastSerialCD.cs:135-170) keeps its winner.  Iterations are launched from a captured CUDA
// graph, 256 at a time, each chained to the previous by programmatic dependent launch; a launch
// after the stopping iteration does nothing, so the iteration count and result equal the
// reference's loop.

#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.cuh"

using namespace p9idg;

namespace {

p9idg_status fail(p9idg_status st, const std::string &msg) {
    record_last_error(msg);
    return st;
}

p9idg_status cuda_fail(cudaError_t e, const char *what) {
    const p9idg_status st = (e == cudaErrorMemoryAllocation) ? P9IDG_OUT_OF_MEMORY
                            : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? P9IDG_NO_DEVICE
                                                                                             : P9IDG_CUDA_ERROR;
    return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(x)                                                \
    do {                                                     \
        cudaError_t e_ = (x);                                \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);     \
    } while (0)

#define TRY(x)                         \
    do {                               \
        p9idg_status s_ = (x);         \
        if (s_ != P9IDG_OK) return s_; \
    } while (0)

#define CUFFT(x)                                                                              \
    do {                                                                                      \
        cufftResult r_ = (x);                                                                 \
        if (r_ != CUFFT_SUCCESS) return fail(P9IDG_CUDA_ERROR, std::string(#x) + " failed"); \
    } while (0)

struct Buf {  // device buffer, freed when it goes out of scope (every early return included)
    void *p = nullptr;
    size_t bytes = 0;
    Buf() = default;
    Buf(const Buf &) = delete;
    Buf &operator=(const Buf &) = delete;
    ~Buf() { release(); }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = device_alloc(&p, std::max<size_t>(n, 256));
        if (e == cudaSuccess) bytes = std::max<size_t>(n, 256);
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T *as() const { return static_cast<T *>(p); }
};

p9idg_status have_device() {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(P9IDG_NO_DEVICE, "no CUDA device available");
    return P9IDG_OK;
}

// ------------------------------------------------------------------------------------------
// device arithmetic in the reference's float semantics

// .NET Core 3.0 Math.Max(float, float): IEEE 754:2019 maximum (NaN wins, +0 above -0).
__device__ __forceinline__ float cs_maxf(float a, float b) {
    if (a != b) {
        if (!isnan(a)) return b < a ? a : b;
        return a;
    }
    return signbit(b) ? a : b;
}

// ElasticNet.ProximalOperator (Common.cs:28-29), un-fused.
__device__ __forceinline__ float prox(float x, float lipschitz, float lambda, float alpha) {
    const float num = cs_maxf(__fsub_rn(x, __fmul_rn(lambda, alpha)), 0.0f);
    const float den = __fadd_rn(lipschitz, __fmul_rn(lambda, __fsub_rn(1.0f, alpha)));
    return __fdiv_rn(num, den);
}

constexpr int kNT = 512, kWarps = kNT / 32;  // image reductions
// Coordinate descent: tiles of kTY x kTX pixels, one CTA of kCdNT threads per tile (8 pixels a
// thread).  A 768^2 update window (a 384^2 PSF) spans 21 x 7 = 147 such tiles, one CTA per SM of
// the 152, each evaluating 5,120 pixels; 32 x 128 tiles of 512 threads need 175 CTAs, two on some
// SMs, and the 3072^2 major cycle's coordinate descent ran 19 % slower with them.
constexpr int kTY = 40, kTX = 128, kCdNT = 640, kCdWarps = kCdNT / 32, kCdBlocksPerSM = 1;
constexpr int kGraphIters = 256;  // even: every replay ends on state buffer 0

struct CdCtl {  // the state one launch hands to the next
    int32_t iter, done, converged, error;
};

struct CdParams {  // device-resident, read by every launch (so one captured graph serves all calls)
    float *x, *g;
    const float *a, *psf2;
    unsigned long long *tile_key;  // [2][ntiles]: best key of each tile (double-buffered by launch parity)
    float2 *tile_val;              // [2][ntiles]: (new value, current value) of each tile's best pixel
    CdCtl *ctl;                    // [2]
    int32_t n, ph, pw, tiles_x, tiles_y, max_iter;
    float lambda, alpha, eps;
    int32_t pad;
};

// Max of a 64-bit key over the warp as two 32-bit hardware reductions: the high words, then the
// low words of the lanes holding the highest one (the same lexicographic maximum).
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v) {
    const unsigned hi = static_cast<unsigned>(v >> 32);
    const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
    const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? static_cast<unsigned>(v) : 0u);
    return (static_cast<unsigned long long>(mh) << 32) | ml;
}

// Block-wide max with one barrier: every warp reduces the per-warp results itself.  sm[kCdWarps]
// must not be reused by the same CTA afterwards (each call site has its own array).
__device__ unsigned long long block_max(unsigned long long v, unsigned long long *sm) {
    static_assert(kCdWarps <= 32, "one warp reduces the per-warp results");
    v = warp_max(v);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31;
    return warp_max(lane < kCdWarps ? sm[lane] : 0ull);
}

// The best key over all tiles of one buffer (8 loads in flight per thread: one round up to
// 4096 tiles, e.g. a 4096^2 image).
__device__ unsigned long long reduce_tiles(const unsigned long long *keys, int ntiles, unsigned long long *sm) {
    unsigned long long best = 0;
    for (int base = 0; base < ntiles; base += 8 * kCdNT) {
        unsigned long long v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int t = base + j * kCdNT + static_cast<int>(threadIdx.x);
            v[j] = t < ntiles ? __ldcg(keys + t) : 0ull;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) best = v[j] > best ? v[j] : best;
    }
    return block_max(best, sm);
}

struct Window {
    uint32_t sel;  // selected pixel index
    int py, px, y0, y1, x0, x1, yh, xh;
};

// Evaluates (and with UPDATE first updates) one tile; writes its best key and values.  All of a
// thread's loads are issued before any is used (predicated, no early exits), so a tile costs one
// memory latency rather than one per pixel.
template <bool UPDATE>
__device__ void eval_tile(const CdParams &P, float lambda, float alpha, int ty, int tx, const Window &w,
                          const float2 *sel_val, unsigned long long *key_out, float2 *val_out,
                          unsigned long long *sm) {
    constexpr int R = kTY / kCdWarps, K = kTX / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int yb = ty * kTY + warp * R, xb = tx * kTX + lane;
    // the selected pixel's (new, current) values: every thread loads them beside its pixels (one
    // request per warp), so no block barrier is needed to share them
    float2 sv = make_float2(0.0f, 0.0f);
    if (UPDATE) sv = __ldcg(sel_val);
    float gv[R][K], xv[R][K], av[R][K], pv[R][K];
#pragma unroll
    for (int r = 0; r < R; r++) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int y = yb + r, xc = xb + 32 * k;
            const bool in = y < P.n && xc < P.n;
            const uint32_t i = static_cast<uint32_t>(y) * static_cast<uint32_t>(P.n) + static_cast<uint32_t>(xc);
            gv[r][k] = 0.0f;
            xv[r][k] = 0.0f;
            av[r][k] = 1.0f;
            pv[r][k] = 0.0f;
            if (in) {
                gv[r][k] = P.g[i];
                xv[r][k] = P.x[i];
                av[r][k] = __ldg(P.a + i);
            }
            if (UPDATE && in && y >= w.y0 && y < w.y1 && xc >= w.x0 && xc < w.x1)
                pv[r][k] = __ldg(P.psf2 + static_cast<int64_t>(y + w.yh - w.py) * P.pw + (xc + w.xh - w.px));
        }
    }
    float xnew = 0.0f, xdiff = 0.0f;
    if (UPDATE) {
        xnew = sv.x;
        xdiff = __fsub_rn(sv.y, sv.x);  // pixelOld - maxPixel.PixelNew
    }
    unsigned long long best = 0;
    float bnew = 0.0f, bold = 0.0f;
#pragma unroll
    for (int r = 0; r < R; r++) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int y = yb + r, xc = xb + 32 * k;
            if (y >= P.n || xc >= P.n) continue;
            const uint32_t i = static_cast<uint32_t>(y) * static_cast<uint32_t>(P.n) + static_cast<uint32_t>(xc);
            float g = gv[r][k], old = xv[r][k];
            if (UPDATE) {
                if (y >= w.y0 && y < w.y1 && xc >= w.x0 && xc < w.x1) {
                    g = __fadd_rn(g, __fmul_rn(pv[r][k], xdiff));  // gradients[i, j] += psf2 * xDiff
                    P.g[i] = g;
                }
                if (i == w.sel) {
                    old = xnew;
                    P.x[i] = xnew;
                }
            }
            const float a = av[r][k];
            const float xt = prox(__fadd_rn(__fmul_rn(old, a), g), a, lambda, alpha);
            const float d = fabsf(__fsub_rn(old, xt));
            const unsigned long long key =
                (0.0f < d) ? ((static_cast<unsigned long long>(__float_as_uint(d)) << 32) | (0xFFFFFFFFu - i)) : 0ull;
            if (key > best) {
                best = key;
                bnew = xt;
                bold = old;
            }
        }
    }
    const unsigned long long m = block_max(best, sm);
    const int t = ty * P.tiles_x + tx;
    if (threadIdx.x == 0) key_out[t] = m;
    if (m != 0ull && best == m) val_out[t] = make_float2(bnew, bold);
}

// Full scan into state buffer 0: the candidate of every tile (GetAbsMax over the whole image).
__global__ void __launch_bounds__(kCdNT) cd_scan_kernel(const CdParams *pp, float lambda, float alpha) {
    __shared__ unsigned long long sm[kCdWarps];
    const CdParams P = *pp;
    Window w{};
    eval_tile<false>(P, lambda, alpha, blockIdx.y, blockIdx.x, w, nullptr, P.tile_key, P.tile_val, sm);
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) P.ctl[0] = CdCtl{0, 0, 0, 0};
}

// The selected pixel's key and values of state buffer 0 (GetAbsMax's result), for the host.
__global__ void __launch_bounds__(kCdNT) cd_pick_kernel(const CdParams *pp, unsigned long long *out_key, float2 *out_val) {
    __shared__ unsigned long long sm[kCdWarps];
    const CdParams P = *pp;
    const unsigned long long best = reduce_tiles(P.tile_key, P.tiles_x * P.tiles_y, sm);
    if (threadIdx.x == 0) {
        *out_key = best;
        float2 v = make_float2(0.0f, 0.0f);
        if (best) {
            const uint32_t idx = 0xFFFFFFFFu - static_cast<uint32_t>(best);
            v = P.tile_val[static_cast<int>((idx / P.n) / kTY) * P.tiles_x + static_cast<int>((idx % P.n) / kTX)];
        }
        *out_val = v;
    }
}

// One coordinate-descent iteration (FastSerialCD.cs:83-98).  Launch k reads state buffer k % 2
// (tile candidates and control) and writes buffer (k + 1) % 2: the window's tiles re-evaluated,
// every other tile's candidate copied.  Each CTA finds the selected pixel itself from the input
// buffer, so a launch needs no grid-wide synchronisation.
//
// The fixed fields (state buffers, maps, sizes) are a kernel parameter captured with the graph,
// so the first loads of a launch (the tile keys) need no pointer loaded from memory first; the
// per-call fields (images, lambda, alpha, eps, iteration cap) come from pp, which only the host
// writes before the graph is launched.
__global__ void __launch_bounds__(kCdNT, kCdBlocksPerSM)
    cd_iter_kernel(const __grid_constant__ CdParams F, const CdParams *pp, int parity) {
    __shared__ unsigned long long sm_in[kCdWarps], sm_out[kCdWarps];
    __shared__ CdCtl c;
    CdParams P = F;
    P.x = pp->x;
    P.g = pp->g;
    P.lambda = pp->lambda;
    P.alpha = pp->alpha;
    P.eps = pp->eps;
    P.max_iter = pp->max_iter;
    // Programmatic dependent launch: this grid is launched while the previous iteration finishes
    // (each CTA of that grid releases it as its last step) and waits here until that grid has
    // completed and its candidates and control are visible.  Nothing the previous grid writes is
    // read before the wait.  Releasing at the end rather than the start measured faster: early
    // waiting CTAs cost ~2 us per iteration when most of the window lies outside the image.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const int ntiles = P.tiles_x * P.tiles_y;
    const unsigned long long *kin = P.tile_key + static_cast<int64_t>(parity) * ntiles;
    const float2 *vin = P.tile_val + static_cast<int64_t>(parity) * ntiles;
    unsigned long long *kout = P.tile_key + static_cast<int64_t>(1 - parity) * ntiles;
    float2 *vout = P.tile_val + static_cast<int64_t>(1 - parity) * ntiles;
    const CdCtl *cin = P.ctl + parity;
    CdCtl *cout = P.ctl + (1 - parity);
    if (threadIdx.x == 0) c = *cin;
    const unsigned long long key = reduce_tiles(kin, ntiles, sm_in);  // its barrier publishes c
    const bool lead = blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0;
    if (c.done) {
        if (lead) *cout = c;
        return;
    }
    if (c.iter >= P.max_iter) {  // while (!converged & iter < iterations)
        if (lead) *cout = CdCtl{c.iter, 1, 0, 0};
        return;
    }
    const float diff = __uint_as_float(static_cast<uint32_t>(key >> 32));
    if (diff < P.eps) {  // converged = maxPixel.PixelMaxDiff < epsilon
        if (lead) *cout = CdCtl{c.iter, 1, 1, 0};
        return;
    }
    if (key == 0ull) {  // the reference would index pixel (-1, -1)
        if (lead) *cout = CdCtl{c.iter, 1, 0, 1};
        return;
    }
    Window w;
    w.sel = 0xFFFFFFFFu - static_cast<uint32_t>(key);
    w.py = static_cast<int>(w.sel / P.n);
    w.px = static_cast<int>(w.sel % P.n);
    w.yh = P.ph / 2;
    w.xh = P.pw / 2;
    w.y0 = max(w.py - w.yh, 0);
    w.x0 = max(w.px - w.xh, 0);
    w.y1 = min(w.py - w.yh + P.ph, P.n);
    w.x1 = min(w.px - w.xh + P.pw, P.n);
    const int ty0 = w.y0 / kTY, ty1 = (w.y1 - 1) / kTY, tx0 = w.x0 / kTX, tx1 = (w.x1 - 1) / kTX;
    // candidates of the tiles outside the window carry over unchanged
    const int nb = gridDim.x * gridDim.y, b = blockIdx.y * gridDim.x + blockIdx.x;
    for (int t = b + nb * static_cast<int>(threadIdx.x); t < ntiles; t += nb * kCdNT) {
        const int tty = t / P.tiles_x, ttx = t % P.tiles_x;
        if (tty < ty0 || tty > ty1 || ttx < tx0 || ttx > tx1) {
            kout[t] = __ldcg(kin + t);
            vout[t] = __ldcg(vin + t);
        }
    }
    const float2 *sel_val = vin + static_cast<int>(w.py / kTY) * P.tiles_x + static_cast<int>(w.px / kTX);
    const int ty = ty0 + static_cast<int>(blockIdx.y), tx = tx0 + static_cast<int>(blockIdx.x);
    if (ty <= ty1 && tx <= tx1) eval_tile<true>(P, P.lambda, P.alpha, ty, tx, w, sel_val, kout, vout, sm_out);
    if (lead) *cout = CdCtl{c.iter + 1, 0, 0, 0};
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");  // the next iteration may launch
}

// ------------------------------------------------------------------------------------------
// PSF preparation and the padded correlation (FP64, as the reference)

// psfPadded of PSF.CalcPaddedFourierCorrelation (Common.cs:128-135), FFT.Shift-ed, as complex.
__global__ void corr_pad_kernel(const float *psf, int h, int w, int H, int yh, int xh, double2 *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(H) * H) return;
    int r = static_cast<int>(i / H), c = static_cast<int>(i % H);
    shift_index(H, r, c);  // out[i] = padded[shifted position]
    const int y = r - yh - 1, x = c - xh - 1;
    double v = 0.0;
    if (y >= 0 && x >= 0 && y < h && x < w) v = psf[static_cast<int64_t>(h - y - 1) * w + (w - x - 1)];
    out[i] = make_double2(v, 0.0);
}

// PaddedConvolver.InsertImage (PaddedConvolver.cs:87-107): image at (yh, xh) of an H x W buffer.
__global__ void conv_pad_kernel(const float *img, int n, int H, int W, int yh, int xh, double2 *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(H) * W) return;
    const int r = static_cast<int>(i / W) - yh, c = static_cast<int>(i % W) - xh;
    const double v = (r >= 0 && c >= 0 && r < n && c < n) ? static_cast<double>(img[static_cast<int64_t>(r) * n + c]) : 0.0;
    out[i] = make_double2(v, 0.0);
}

// psfPadded of PSF.CalcPSFSquared (Common.cs:165-167): psf at (h/2, w/2) of a 2h x 2w buffer.
__global__ void sq_pad_kernel(const float *psf, int h, int w, double2 *out) {
    const int W = 2 * w;
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(2 * h) * W) return;
    const int r = static_cast<int>(i / W) - h / 2, c = static_cast<int>(i % W) - w / 2;
    const double v = (r >= 0 && c >= 0 && r < h && c < w) ? static_cast<double>(psf[static_cast<int64_t>(r) * w + c]) : 0.0;
    out[i] = make_double2(v, 0.0);
}

// a *= b, System.Numerics.Complex multiplication (re = ac - bd, im = bc + ad), un-fused.
__global__ void cmul_kernel(double2 *a, const double2 *b, int64_t count) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= count) return;
    const double2 x = a[i], y = b[i];
    a[i] = make_double2(__dsub_rn(__dmul_rn(x.x, y.x), __dmul_rn(x.y, y.y)),
                        __dadd_rn(__dmul_rn(x.y, y.x), __dmul_rn(x.x, y.y)));
}

// out[i][j] = (float)(buf[i + yh][j + xh].Real / len)   (PaddedConvolver.cs:55-62)
__global__ void conv_extract_kernel(const double2 *buf, int W, int yh, int xh, int n, double len, float *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(n) * n) return;
    const int r = static_cast<int>(i / n), c = static_cast<int>(i % n);
    out[i] = static_cast<float>(buf[static_cast<int64_t>(r + yh) * W + c + xh].x / len);
}

// PSF.QueryScan (Common.cs:46-74) per pixel of the image section, from the host-built scan.
__global__ void amap_kernel(const double *scan, int sh, int sw, int ty_end, int tx_end, int sy, int sx, int oh,
                            int ow, float *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(oh) * ow) return;
    const int yPixel = sy + static_cast<int>(i / ow), xPixel = sx + static_cast<int>(i % ow);
#define S(a, b) scan[static_cast<int64_t>(a) * sw + (b)]
    int yOver = max(0, (yPixel + (sh - sh / 2)) - ty_end);
    int xOver = max(0, (xPixel + (sw - sw / 2)) - tx_end);
    const int yUnder = -(yPixel - sh / 2), xUnder = -(xPixel - sw / 2);
    const int yUi = max(1, yUnder) - 1, xUi = max(1, xUnder) - 1;
    double v;
    if (yOver <= 0 && xOver <= 0 && yUnder <= 0 && xUnder <= 0) {
        v = S(sh - 1, sw - 1);
    } else if (yUnder > 0 && xUnder > 0) {
        v = __dadd_rn(__dsub_rn(__dsub_rn(S(sh - 1, sw - 1), S(sh - 1, xUi)), S(yUi, sw - 1)), S(yUi, xUi));
    } else {
        double corr = 0.0;
        if (yUnder > 0) corr = __dadd_rn(corr, S(yUi, sw - xOver - 1));
        if (xUnder > 0) corr = __dadd_rn(corr, S(sh - yOver - 1, xUi));
        v = __dsub_rn(S(sh - 1 - yOver, sw - 1 - xOver), corr);
    }
#undef S
    out[i] = static_cast<float>(v);
}

// Residuals.GetMax (Common.cs:244-251) and PSF.CalcMaxSidelobe (Common.cs:203-214): max over
// non-negative values starting at 0 (NaN propagates), as uint bits with atomicMax.
__global__ void max_kernel(const float *img, int n, int cut_off, int cut_len, bool sidelobe, unsigned int *out) {
    __shared__ float sm[kWarps];
    float m = 0.0f;
    const int64_t total = static_cast<int64_t>(n) * n;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        float v = img[i];
        if (sidelobe) {
            const int y = static_cast<int>(i / n), x = static_cast<int>(i % n);
            if ((y >= cut_off && y < cut_off + cut_len) && (x >= cut_off && x < cut_off + cut_len)) continue;
            v = fabsf(v);
        }
        m = cs_maxf(m, v);
    }
    for (int o = 16; o; o >>= 1) m = cs_maxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kWarps; k++) m = cs_maxf(m, sm[k]);
        atomicMax(out, __float_as_uint(m));  // m is +0, positive or NaN: its bits order as uint
    }
}

// Partial sums of squares (PSF.CalcMaxLipschitz, Common.cs:107-114) per block, fixed assignment.
__global__ void sumsq_kernel(const float *psf, int64_t count, double *partial) {
    __shared__ double sm[kWarps];
    double s = 0.0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float v = __fmul_rn(psf[i], psf[i]);
        s = __dadd_rn(s, static_cast<double>(v));
    }
    for (int o = 16; o; o >>= 1) s = __dadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kWarps; k++) s = __dadd_rn(s, sm[k]);
        partial[blockIdx.x] = s;
    }
}

// The two sums of the major cycle's objective (MajorCycle.cs:102) in the reference's types:
// Residuals.CalcPenalty's float squares (Common.cs:253-260) and ElasticNet.CalcPenalty's
// lambda * ElasticNetPenalty (Common.cs:22-23, 31-41; a float expression widened to double),
// each summed in double: per-block partials, summed in block order on the host.
__global__ void objective_kernel(const float *dirty, const float *x, int64_t count, float lambda, float alpha,
                                 double *partial) {
    __shared__ double sm[2][kWarps];
    double sr = 0.0, sx = 0.0;
    const float half_1ma = __fmul_rn(1.0f / 2.0f, __fsub_rn(1.0f, alpha));
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float r = dirty[i], v = x[i];
        sr = __dadd_rn(sr, static_cast<double>(__fmul_rn(r, r)));
        const float pen = __fadd_rn(__fmul_rn(half_1ma, __fmul_rn(v, v)), __fmul_rn(alpha, fabsf(v)));
        sx = __dadd_rn(sx, __dmul_rn(static_cast<double>(lambda), static_cast<double>(pen)));
    }
    for (int o = 16; o; o >>= 1) {
        sr = __dadd_rn(sr, __shfl_xor_sync(0xffffffffu, sr, o));
        sx = __dadd_rn(sx, __shfl_xor_sync(0xffffffffu, sx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sm[0][threadIdx.x >> 5] = sr;
        sm[1][threadIdx.x >> 5] = sx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kWarps; k++) {
            sr = __dadd_rn(sr, sm[0][k]);
            sx = __dadd_rn(sx, sm[1][k]);
        }
        partial[2 * blockIdx.x] = sr;
        partial[2 * blockIdx.x + 1] = sx;
    }
}

// PSF.Cut (Common.cs:216-226) of a square n x n image.
__global__ void cut_kernel(const float *psf, int n, int m, int off, float *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(m) * m) return;
    const int y = static_cast<int>(i / m), x = static_cast<int>(i % m);
    out[i] = psf[static_cast<int64_t>(off + y) * n + off + x];
}

// psf2[i, j] *= (maxFull / maxCut)  (FastSerialCD.ResetLipschitzMap, FastSerialCD.cs:123-126)
__global__ void scale_kernel(float *a, int64_t count, float f) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < count) a[i] = __fmul_rn(a[i], f);
}

// Visibilities.Substract (Common.cs:305-317) on complex64.
__global__ void vis_subtract_kernel(const float2 *v0, const float2 *v1, const uint8_t *flags, int64_t count,
                                    float2 *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= count) return;
    const float2 a = v0[i], b = v1[i];
    out[i] = flags[i] ? make_float2(0.0f, 0.0f) : make_float2(a.x - b.x, a.y - b.y);
}

// FFT.Shift(xImage) then the complex input of FFT.Forward (MajorCycle.cs:125-126).
__global__ void shifted_real_to_c64_kernel(const float *img, int n, float2 *out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<int64_t>(n) * n) return;
    int r = static_cast<int>(i / n), c = static_cast<int>(i % n);
    shift_index(n, r, c);
    out[i] = make_float2(img[static_cast<int64_t>(r) * n + c], 0.0f);
}

inline unsigned grid_for(int64_t count, int threads = 256) {
    return static_cast<unsigned>((count + threads - 1) / threads);
}

// ------------------------------------------------------------------------------------------
// host helpers

// The double prefix-sum scan of psf^2 in PSF.CalcAMap (Common.cs:84-93), in the reference's
// order (host: its dependencies make it sequential and it is psf-sized).
void amap_scan(const float *psf, int h, int w, std::vector<double> &scan) {
    scan.assign(static_cast<size_t>(h) * w, 0.0);
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            const double iB = i > 0 ? scan[static_cast<size_t>(i - 1) * w + j] : 0.0;
            const double jB = j > 0 ? scan[static_cast<size_t>(i) * w + j - 1] : 0.0;
            const double ijB = (i > 0 && j > 0) ? scan[static_cast<size_t>(i - 1) * w + j - 1] : 0.0;
            const float cur = psf[static_cast<size_t>(i) * w + j] * psf[static_cast<size_t>(i) * w + j];
            scan[static_cast<size_t>(i) * w + j] = static_cast<double>(cur) + iB + jB - ijB;
        }
}

struct Z2Z {
    cufftHandle h = 0;
    int ny = 0, nx = 0;
    p9idg_status get(int y, int x, cudaStream_t st) {
        if (h && (y != ny || x != nx)) {
            cufftDestroy(h);
            h = 0;
        }
        if (!h) {
            if (cufftPlan2d(&h, y, x, CUFFT_Z2Z) != CUFFT_SUCCESS) {
                h = 0;
                return fail(P9IDG_CUDA_ERROR, "cufftPlan2d (Z2Z) failed");
            }
            ny = y;
            nx = x;
        }
        CUFFT(cufftSetStream(h, st));
        return P9IDG_OK;
    }
    void release() {
        if (h) cufftDestroy(h);
        h = 0;
    }
};

// PSF.CalcPaddedFourierCorrelation on the device: psf (device h x w) -> out (device H x H complex).
p9idg_status dev_padded_correlation(const float *d_psf, int h, int w, int pad_y, int pad_x, double2 *d_out, Z2Z &fft,
                                    cudaStream_t st) {
    const int H = pad_y + h, W = pad_x + w;
    if (H != W) return fail(P9IDG_INVALID_ARGUMENT, "padded PSF must be square (FFT.Shift uses the row count)");
    corr_pad_kernel<<<grid_for(static_cast<int64_t>(H) * H), 256, 0, st>>>(d_psf, h, w, H, pad_y / 2, pad_x / 2, d_out);
    CK(cudaGetLastError());
    TRY(fft.get(H, W, st));
    CUFFT(cufftExecZ2Z(fft.h, reinterpret_cast<cufftDoubleComplex *>(d_out), reinterpret_cast<cufftDoubleComplex *>(d_out),
                       CUFFT_FORWARD));
    return P9IDG_OK;
}

// PSF.CalcPSFSquared on the device: psf (device h x w) -> out (device 2h x 2w float).
p9idg_status dev_psf_squared(const float *d_psf, int h, int w, float *d_out, Buf &b0, Buf &b1, Z2Z &fft,
                             cudaStream_t st) {
    const int64_t count = static_cast<int64_t>(2 * h) * (2 * w);
    CK(b0.ensure(sizeof(double2) * count));
    CK(b1.ensure(sizeof(double2) * count));
    TRY(dev_padded_correlation(d_psf, h, w, h, w, b0.as<double2>(), fft, st));
    sq_pad_kernel<<<grid_for(count), 256, 0, st>>>(d_psf, h, w, b1.as<double2>());
    CK(cudaGetLastError());
    auto *s = reinterpret_cast<cufftDoubleComplex *>(b1.p);
    CUFFT(cufftExecZ2Z(fft.h, s, s, CUFFT_FORWARD));
    cmul_kernel<<<grid_for(count), 256, 0, st>>>(b1.as<double2>(), b0.as<double2>(), count);
    CK(cudaGetLastError());
    CUFFT(cufftExecZ2Z(fft.h, s, s, CUFFT_INVERSE));
    // FFT.Backward(PSF2, (long)psfCorrelated.Length): Re / count
    conv_extract_kernel<<<grid_for(count), 256, 0, st>>>(b1.as<double2>(), 2 * w, 0, 0, 2 * w,
                                                         static_cast<double>(count), d_out);
    CK(cudaGetLastError());
    return P9IDG_OK;
}

// Residuals.GetMax / PSF.CalcMaxSidelobe on a device n x n image (synchronises the stream).
p9idg_status dev_max(const float *d_img, int n, int cut_factor, unsigned int *d_word, float *out, cudaStream_t st) {
    CK(cudaMemsetAsync(d_word, 0, sizeof(unsigned int), st));
    const int m = cut_factor > 0 ? n / cut_factor : 0;
    const int off = cut_factor > 0 ? n / 2 - m / 2 : 0;
    max_kernel<<<std::min<unsigned>(grid_for(static_cast<int64_t>(n) * n), 1024), kNT, 0, st>>>(d_img, n, off, m,
                                                                                                 cut_factor > 0, d_word);
    CK(cudaGetLastError());
    unsigned int bits = 0;
    CK(cudaMemcpyAsync(&bits, d_word, sizeof(bits), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    std::memcpy(out, &bits, sizeof(float));
    return P9IDG_OK;
}

// Residuals.CalcPenalty(dirty) + ElasticNet.CalcPenalty(x, lambda, alpha) (MajorCycle.cs:102).
p9idg_status dev_objective(const float *d_dirty, const float *d_x, int64_t count, float lambda, float alpha,
                           Buf &partial, double *out, cudaStream_t st) {
    constexpr int kBlocks = 256;
    CK(partial.ensure(sizeof(double) * 2 * kBlocks));
    objective_kernel<<<kBlocks, kNT, 0, st>>>(d_dirty, d_x, count, lambda, alpha, partial.as<double>());
    CK(cudaGetLastError());
    double h[2 * kBlocks];
    CK(cudaMemcpyAsync(h, partial.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double r = 0.0, x = 0.0;
    for (int b = 0; b < kBlocks; b++) {
        r += h[2 * b];
        x += h[2 * b + 1];
    }
    *out = 0.5 * r + x;
    return P9IDG_OK;
}

// PSF.CalcMaxLipschitz of a device image (deterministic: fixed partials summed in order).
p9idg_status dev_sumsq(const float *d_img, int64_t count, Buf &partial, double *out, cudaStream_t st) {
    constexpr int kBlocks = 256;
    CK(partial.ensure(sizeof(double) * kBlocks));
    sumsq_kernel<<<kBlocks, kNT, 0, st>>>(d_img, count, partial.as<double>());
    CK(cudaGetLastError());
    double h[kBlocks];
    CK(cudaMemcpyAsync(h, partial.p, sizeof(h), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double s = 0.0;
    for (double v : h) s += v;
    *out = s;
    return P9IDG_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// PaddedConvolver

struct p9idg_convolver {
    int device = -1;
    cudaStream_t stream = nullptr, own = nullptr;
    int H = 0, W = 0, ky = 0, kx = 0;
    Buf kernel, buf;
    Z2Z fft;
};

namespace {

p9idg_status conv_init(p9idg_convolver *c, int H, int W, int ky, int kx) {
    CK(cudaGetDevice(&c->device));
    CK(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
    c->stream = c->own;
    c->H = H;
    c->W = W;
    c->ky = ky;
    c->kx = kx;
    CK(c->kernel.ensure(sizeof(double2) * static_cast<size_t>(H) * W));
    CK(c->buf.ensure(sizeof(double2) * static_cast<size_t>(H) * W));
    TRY(c->fft.get(H, W, c->stream));
    return P9IDG_OK;
}

void conv_release(p9idg_convolver *c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->kernel.release();
    c->buf.release();
    c->fft.release();
    if (c->own) cudaStreamDestroy(c->own);
}

// PaddedConvolver.Convolve (PaddedConvolver.cs:43-65) of a device n x n image.
p9idg_status conv_run(p9idg_convolver *c, const float *d_img, int n, float *d_out) {
    if (n + c->ky / 2 > c->H || n + c->kx / 2 > c->W)
        return fail(P9IDG_INVALID_ARGUMENT, "image larger than the convolver's padded buffer");
    const int64_t count = static_cast<int64_t>(c->H) * c->W;
    conv_pad_kernel<<<grid_for(count), 256, 0, c->stream>>>(d_img, n, c->H, c->W, c->ky / 2, c->kx / 2,
                                                            c->buf.as<double2>());
    CK(cudaGetLastError());
    TRY(c->fft.get(c->H, c->W, c->stream));
    auto *s = reinterpret_cast<cufftDoubleComplex *>(c->buf.p);
    CUFFT(cufftExecZ2Z(c->fft.h, s, s, CUFFT_FORWARD));
    cmul_kernel<<<grid_for(count), 256, 0, c->stream>>>(c->buf.as<double2>(), c->kernel.as<double2>(), count);
    CK(cudaGetLastError());
    CUFFT(cufftExecZ2Z(c->fft.h, s, s, CUFFT_INVERSE));
    conv_extract_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, c->stream>>>(
        c->buf.as<double2>(), c->W, c->ky / 2, c->kx / 2, n, static_cast<double>(static_cast<int32_t>(count)), d_out);
    CK(cudaGetLastError());
    return P9IDG_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// FastSerialCD

struct p9idg_cd {
    int device = -1;
    cudaStream_t stream = nullptr, own = nullptr;
    int n = 0, ph = 0, pw = 0;  // image size, psf2 size
    int tiles_x = 0, tiles_y = 0;
    float max_lipschitz = 0.0f;
    Buf x, g, amap, psf2, tile_key, tile_val, params, ctl, pick, word, partial, sq0, sq1, psf_tmp;
    Z2Z fft;
    CdParams hp{};
    CdParams captured{};                   // hp as the iteration graph was captured with
    CdCtl *h_ctl = nullptr;                // pinned
    unsigned long long *h_pick = nullptr;  // pinned: selected key
    cudaEvent_t ev_ctl = nullptr;          // the control word of a replay has reached h_ctl
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

p9idg_status cd_set_maps(p9idg_cd *cd, const float *h_psf, int h, int w) {
    // psf2 = PSF.CalcPSFSquared(psf); aMap = PSF.CalcAMap(psf, totalSize); MaxLipschitz = GetMax(psf2)
    const int n = cd->n;
    CK(cd->psf_tmp.ensure(sizeof(float) * static_cast<size_t>(h) * w));
    CK(cudaMemcpyAsync(cd->psf_tmp.p, h_psf, sizeof(float) * static_cast<size_t>(h) * w, cudaMemcpyHostToDevice,
                       cd->stream));
    CK(cd->psf2.ensure(sizeof(float) * static_cast<size_t>(4) * h * w));
    TRY(dev_psf_squared(cd->psf_tmp.as<float>(), h, w, cd->psf2.as<float>(), cd->sq0, cd->sq1, cd->fft, cd->stream));
    cd->ph = 2 * h;
    cd->pw = 2 * w;
    std::vector<double> scan;
    amap_scan(h_psf, h, w, scan);
    Buf d_scan;
    CK(d_scan.ensure(sizeof(double) * scan.size()));
    cudaError_t e = cudaMemcpyAsync(d_scan.p, scan.data(), sizeof(double) * scan.size(), cudaMemcpyHostToDevice,
                                    cd->stream);
    if (e == cudaSuccess) {
        amap_kernel<<<grid_for(static_cast<int64_t>(n) * n), 256, 0, cd->stream>>>(d_scan.as<double>(), h, w, n, n, 0,
                                                                                   0, n, n, cd->amap.as<float>());
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(cd->stream);
    d_scan.release();
    if (e != cudaSuccess) return cuda_fail(e, "aMap");
    // psf2 is square (2h x 2w with h == w for every caller); GetMax over it
    float m = 0.0f;
    if (cd->ph == cd->pw) {
        TRY(dev_max(cd->psf2.as<float>(), cd->ph, 0, cd->word.as<unsigned int>(), &m, cd->stream));
    } else {
        std::vector<float> host(static_cast<size_t>(cd->ph) * cd->pw);
        CK(cudaMemcpy(host.data(), cd->psf2.p, sizeof(float) * host.size(), cudaMemcpyDeviceToHost));
        for (float v : host) m = v > m ? v : m;
    }
    cd->max_lipschitz = m;
    return P9IDG_OK;
}

p9idg_status cd_upload_params(p9idg_cd *cd) {
    CK(cudaMemcpyAsync(cd->params.p, &cd->hp, sizeof(CdParams), cudaMemcpyHostToDevice, cd->stream));
    return P9IDG_OK;
}

dim3 cd_window_grid(const p9idg_cd *cd) {
    const int wy = std::min(cd->tiles_y, (cd->ph + kTY - 1) / kTY + 1);
    const int wx = std::min(cd->tiles_x, (cd->pw + kTX - 1) / kTX + 1);
    return dim3(static_cast<unsigned>(wx), static_cast<unsigned>(wy));
}

// The fields the iteration kernels take from their captured parameter (the rest come from the
// device copy of the parameters on every launch).
bool same_fixed_params(const CdParams &a, const CdParams &b) {
    return a.a == b.a && a.psf2 == b.psf2 && a.tile_key == b.tile_key && a.tile_val == b.tile_val && a.ctl == b.ctl &&
           a.n == b.n && a.ph == b.ph && a.pw == b.pw && a.tiles_x == b.tiles_x && a.tiles_y == b.tiles_y;
}

p9idg_status cd_capture(p9idg_cd *cd) {
    if (cd->exec) {
        if (same_fixed_params(cd->captured, cd->hp)) return P9IDG_OK;
        cudaGraphExecDestroy(cd->exec);
        cudaGraphDestroy(cd->graph);
        cd->exec = nullptr;
        cd->graph = nullptr;
    }
    // captured on the deconvolver's own stream (never the legacy stream); replayed on cd->stream
    const dim3 grid = cd_window_grid(cd);
    // every launch allows programmatic serialisation with the one before it (the kernel waits on
    // it with griddepcontrol.wait before reading its results)
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kCdNT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = cd->own;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CK(cudaStreamBeginCapture(cd->own, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < kGraphIters && le == cudaSuccess; k++)
        le = cudaLaunchKernelEx(&cfg, cd_iter_kernel, cd->hp, static_cast<const CdParams *>(cd->params.as<CdParams>()),
                                k & 1);
    cudaGraph_t gph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(cd->own, &gph);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (gph) cudaGraphDestroy(gph);
        return cuda_fail(le != cudaSuccess ? le : ce, "capturing the coordinate-descent graph");
    }
    cd->graph = gph;
    CK(cudaGraphInstantiate(&cd->exec, cd->graph, 0));
    cd->captured = cd->hp;
    return P9IDG_OK;
}

// Candidates of every tile with (lambda, alpha) into state buffer 0, control reset.
p9idg_status cd_scan(p9idg_cd *cd, float lambda, float alpha) {
    cd_scan_kernel<<<dim3(cd->tiles_x, cd->tiles_y), kCdNT, 0, cd->stream>>>(cd->params.as<CdParams>(), lambda, alpha);
    CK(cudaGetLastError());
    return P9IDG_OK;
}

// FastSerialCD.Deconvolve on device buffers x, g (n x n float), in place.
p9idg_status cd_run(p9idg_cd *cd, float *d_x, float *d_g, float lambda, float alpha, int32_t max_iter, float eps,
                    p9idg_cd_result *res) {
    const auto t0 = std::chrono::steady_clock::now();
    cd->hp.x = d_x;
    cd->hp.g = d_g;
    cd->hp.lambda = lambda;
    cd->hp.alpha = alpha;
    cd->hp.eps = eps;
    cd->hp.max_iter = max_iter;
    TRY(cd_upload_params(cd));
    TRY(cd_scan(cd, lambda, alpha));
    TRY(cd_capture(cd));
    // One replay stays in flight while the host reads the control word the previous one left: the
    // copy after replay r is enqueued before replay r + 1, so the GPU never waits on the host.  A
    // replay launched after the stopping one does nothing (every launch sees the done flag).
    const int64_t max_replays = static_cast<int64_t>(std::max(max_iter, 0)) / kGraphIters + 2;
    CK(cudaGraphLaunch(cd->exec, cd->stream));
    for (int64_t r = 0; r < max_replays; r++) {
        CK(cudaMemcpyAsync(cd->h_ctl, cd->ctl.p, sizeof(CdCtl), cudaMemcpyDeviceToHost, cd->stream));
        CK(cudaEventRecord(cd->ev_ctl, cd->stream));
        if (r + 1 < max_replays) CK(cudaGraphLaunch(cd->exec, cd->stream));
        CK(cudaEventSynchronize(cd->ev_ctl));
        if (cd->h_ctl->done) break;
    }
    CK(cudaStreamSynchronize(cd->stream));  // the replay in flight, if any
    if (!cd->h_ctl->done) return fail(P9IDG_DEVICE_CHECK_FAILED, "coordinate descent did not stop");
    if (cd->h_ctl->error)
        return fail(P9IDG_INVALID_ARGUMENT,
                    "no pixel changes and epsilon <= 0: the reference would index pixel (-1, -1)");
    if (res) {
        res->converged = cd->h_ctl->converged;
        res->iterations = cd->h_ctl->iter;
        res->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return P9IDG_OK;
}

p9idg_status cd_abs_max(p9idg_cd *cd, const float *d_x, const float *d_g, float lambda, float alpha, float *out) {
    cd->hp.x = const_cast<float *>(d_x);
    cd->hp.g = const_cast<float *>(d_g);
    TRY(cd_upload_params(cd));
    TRY(cd_scan(cd, lambda, alpha));
    cd_pick_kernel<<<1, kCdNT, 0, cd->stream>>>(cd->params.as<CdParams>(), cd->pick.as<unsigned long long>(),
                                             reinterpret_cast<float2 *>(cd->pick.as<unsigned long long>() + 1));
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cd->h_pick, cd->pick.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, cd->stream));
    CK(cudaStreamSynchronize(cd->stream));
    const uint32_t bits = static_cast<uint32_t>(*cd->h_pick >> 32);
    std::memcpy(out, &bits, sizeof(float));
    return P9IDG_OK;
}

void cd_release(p9idg_cd *cd) {
    if (cd->stream) cudaStreamSynchronize(cd->stream);
    if (cd->ev_ctl) cudaEventDestroy(cd->ev_ctl);
    if (cd->exec) cudaGraphExecDestroy(cd->exec);
    if (cd->graph) cudaGraphDestroy(cd->graph);
    Buf *bufs[] = {&cd->x, &cd->g, &cd->amap, &cd->psf2, &cd->tile_key, &cd->tile_val, &cd->params, &cd->ctl,
                   &cd->pick, &cd->word, &cd->partial, &cd->sq0, &cd->sq1, &cd->psf_tmp};
    for (Buf *b : bufs) b->release();
    cd->fft.release();
    if (cd->h_ctl) cudaFreeHost(cd->h_ctl);
    if (cd->h_pick) cudaFreeHost(cd->h_pick);
    if (cd->own) cudaStreamDestroy(cd->own);
}

p9idg_status cd_init(p9idg_cd *cd, int n, const float *psf, int h, int w) {
    CK(cudaGetDevice(&cd->device));
    CK(cudaStreamCreateWithFlags(&cd->own, cudaStreamNonBlocking));
    cd->stream = cd->own;
    CK(cudaMallocHost(reinterpret_cast<void **>(&cd->h_ctl), sizeof(CdCtl)));
    CK(cudaMallocHost(reinterpret_cast<void **>(&cd->h_pick), sizeof(unsigned long long)));
    CK(cudaEventCreateWithFlags(&cd->ev_ctl, cudaEventDisableTiming));
    cd->n = n;
    cd->tiles_x = (n + kTX - 1) / kTX;
    cd->tiles_y = (n + kTY - 1) / kTY;
    const size_t nn = static_cast<size_t>(n) * n, nt = static_cast<size_t>(cd->tiles_x) * cd->tiles_y;
    CK(cd->amap.ensure(sizeof(float) * nn));
    CK(cd->tile_key.ensure(sizeof(unsigned long long) * 2 * nt));
    CK(cd->tile_val.ensure(sizeof(float2) * 2 * nt));
    CK(cd->params.ensure(sizeof(CdParams)));
    CK(cd->ctl.ensure(sizeof(CdCtl) * 2));
    CK(cd->pick.ensure(sizeof(unsigned long long) + sizeof(float2)));
    CK(cd->word.ensure(sizeof(unsigned int)));
    TRY(cd_set_maps(cd, psf, h, w));
    cd->hp = CdParams{};
    cd->hp.a = cd->amap.as<float>();
    cd->hp.psf2 = cd->psf2.as<float>();
    cd->hp.tile_key = cd->tile_key.as<unsigned long long>();
    cd->hp.tile_val = cd->tile_val.as<float2>();
    cd->hp.ctl = cd->ctl.as<CdCtl>();
    cd->hp.n = n;
    cd->hp.ph = cd->ph;
    cd->hp.pw = cd->pw;
    cd->hp.tiles_x = cd->tiles_x;
    cd->hp.tiles_y = cd->tiles_y;
    return P9IDG_OK;
}

p9idg_status check_cd_args(int32_t n, const float *psf, int32_t h, int32_t w) {
    if (n <= 0 || n > 65535 || !psf || h <= 0 || w <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    if (h != w) return fail(P9IDG_INVALID_ARGUMENT, "the PSF must be square (FFT.Shift uses the row count)");
    return P9IDG_OK;
}

}  // namespace

extern "C" {

p9idg_status p9idg_cd_create(int32_t n, const float *psf, int32_t psf_h, int32_t psf_w, p9idg_cd **out) {
    if (!out) return fail(P9IDG_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    TRY(check_cd_args(n, psf, psf_h, psf_w));
    TRY(have_device());
    auto *cd = new (std::nothrow) p9idg_cd();
    if (!cd) return fail(P9IDG_OUT_OF_MEMORY, "deconvolver allocation");
    p9idg_status st = cd_init(cd, n, psf, psf_h, psf_w);
    if (st != P9IDG_OK) {
        cd_release(cd);
        delete cd;
        return st;
    }
    *out = cd;
    return P9IDG_OK;
}

p9idg_status p9idg_cd_max_lipschitz(const p9idg_cd *cd, float *out) {
    if (!cd || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *out = cd->max_lipschitz;
    return P9IDG_OK;
}

p9idg_status p9idg_cd_get_maps(p9idg_cd *cd, float *psf2_out, float *amap_out) {
    if (!cd) return fail(P9IDG_INVALID_ARGUMENT, "null deconvolver");
    CK(cudaSetDevice(cd->device));
    CK(cudaStreamSynchronize(cd->stream));
    if (psf2_out) CK(cudaMemcpy(psf2_out, cd->psf2.p, sizeof(float) * static_cast<size_t>(cd->ph) * cd->pw,
                                cudaMemcpyDeviceToHost));
    if (amap_out) CK(cudaMemcpy(amap_out, cd->amap.p, sizeof(float) * static_cast<size_t>(cd->n) * cd->n,
                                cudaMemcpyDeviceToHost));
    return P9IDG_OK;
}

p9idg_status p9idg_cd_psf2_size(const p9idg_cd *cd, int32_t *h, int32_t *w) {
    if (!cd || !h || !w) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *h = cd->ph;
    *w = cd->pw;
    return P9IDG_OK;
}

p9idg_status p9idg_cd_set_stream(p9idg_cd *cd, void *cuda_stream) {
    if (!cd) return fail(P9IDG_INVALID_ARGUMENT, "null deconvolver");
    cudaStream_t s = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : cd->own;
    if (s != cd->stream) {
        CK(cudaStreamSynchronize(cd->stream));
        cd->stream = s;
    }
    return P9IDG_OK;
}

p9idg_status p9idg_cd_deconvolve_device(p9idg_cd *cd, float *d_x, float *d_bmap, float lambda, float alpha,
                                        int32_t max_iter, float epsilon, p9idg_cd_result *res) {
    if (!cd || !d_x || !d_bmap) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(cd->device));
    return cd_run(cd, d_x, d_bmap, lambda, alpha, max_iter, epsilon, res);
}

p9idg_status p9idg_cd_deconvolve(p9idg_cd *cd, float *x, float *bmap, float lambda, float alpha, int32_t max_iter,
                                 float epsilon, p9idg_cd_result *res) {
    if (!cd || !x || !bmap) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(cd->device));
    const size_t bytes = sizeof(float) * static_cast<size_t>(cd->n) * cd->n;
    CK(cd->x.ensure(bytes));
    CK(cd->g.ensure(bytes));
    CK(cudaMemcpyAsync(cd->x.p, x, bytes, cudaMemcpyHostToDevice, cd->stream));
    CK(cudaMemcpyAsync(cd->g.p, bmap, bytes, cudaMemcpyHostToDevice, cd->stream));
    TRY(cd_run(cd, cd->x.as<float>(), cd->g.as<float>(), lambda, alpha, max_iter, epsilon, res));
    // the reference updates reconstruction and bMap in place
    CK(cudaMemcpyAsync(x, cd->x.p, bytes, cudaMemcpyDeviceToHost, cd->stream));
    CK(cudaMemcpyAsync(bmap, cd->g.p, bytes, cudaMemcpyDeviceToHost, cd->stream));
    CK(cudaStreamSynchronize(cd->stream));
    return P9IDG_OK;
}

p9idg_status p9idg_cd_get_abs_max_diff_device(p9idg_cd *cd, const float *d_x, const float *d_bmap, float lambda,
                                              float alpha, float *out) {
    if (!cd || !d_x || !d_bmap || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(cd->device));
    return cd_abs_max(cd, d_x, d_bmap, lambda, alpha, out);
}

p9idg_status p9idg_cd_get_abs_max_diff(p9idg_cd *cd, const float *x, const float *bmap, float lambda, float alpha,
                                       float *out) {
    if (!cd || !x || !bmap || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(cd->device));
    const size_t bytes = sizeof(float) * static_cast<size_t>(cd->n) * cd->n;
    CK(cd->x.ensure(bytes));
    CK(cd->g.ensure(bytes));
    CK(cudaMemcpyAsync(cd->x.p, x, bytes, cudaMemcpyHostToDevice, cd->stream));
    CK(cudaMemcpyAsync(cd->g.p, bmap, bytes, cudaMemcpyHostToDevice, cd->stream));
    return cd_abs_max(cd, cd->x.as<float>(), cd->g.as<float>(), lambda, alpha, out);
}

p9idg_status p9idg_cd_deconvolve_path(p9idg_cd *cd, float *x, float *bmap, float lambda_min, float lambda_factor,
                                      float alpha, int32_t max_path_iter, int32_t max_iter, float epsilon,
                                      p9idg_cd_result *res) {
    // FastSerialCD.DeconvolvePath (FastSerialCD.cs:49-74)
    if (!cd || !x || !bmap) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(cd->device));
    const auto t0 = std::chrono::steady_clock::now();
    const size_t bytes = sizeof(float) * static_cast<size_t>(cd->n) * cd->n;
    CK(cd->x.ensure(bytes));
    CK(cd->g.ensure(bytes));
    CK(cudaMemcpyAsync(cd->x.p, x, bytes, cudaMemcpyHostToDevice, cd->stream));
    CK(cudaMemcpyAsync(cd->g.p, bmap, bytes, cudaMemcpyHostToDevice, cd->stream));
    bool converged = false;
    int32_t total = 0;
    for (int32_t p = 0; p < max_path_iter; p++) {
        float mx = 0.0f;
        TRY(cd_abs_max(cd, cd->x.as<float>(), cd->g.as<float>(), 0.0f, 1.0f, &mx));
        const float lambda_max = 1 / alpha * mx;
        float lambda_cur = lambda_max / lambda_factor;
        lambda_cur = lambda_cur > lambda_min ? lambda_cur : lambda_min;
        p9idg_cd_result r{};
        TRY(cd_run(cd, cd->x.as<float>(), cd->g.as<float>(), lambda_cur, alpha, max_iter, epsilon, &r));
        converged = (lambda_min == lambda_cur) && r.converged;
        total += r.iterations;
        if (converged) break;
    }
    CK(cudaMemcpyAsync(x, cd->x.p, bytes, cudaMemcpyDeviceToHost, cd->stream));
    CK(cudaMemcpyAsync(bmap, cd->g.p, bytes, cudaMemcpyDeviceToHost, cd->stream));
    CK(cudaStreamSynchronize(cd->stream));
    if (res) {
        res->converged = converged;
        res->iterations = total;
        res->elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return P9IDG_OK;
}

p9idg_status p9idg_cd_reset_lipschitz_map(p9idg_cd *cd, const float *psf, int32_t h, int32_t w) {
    // FastSerialCD.ResetLipschitzMap (FastSerialCD.cs:116-127); aMap over the patch (= total size)
    if (!cd || !psf || h <= 0 || w <= 0 || h != w) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    CK(cudaSetDevice(cd->device));
    // maxCut = GetMax(psf2) of the current map
    float max_cut = 0.0f;
    if (cd->ph != cd->pw) return fail(P9IDG_UNSUPPORTED, "non-square PSF^2");
    TRY(dev_max(cd->psf2.as<float>(), cd->ph, 0, cd->word.as<unsigned int>(), &max_cut, cd->stream));
    // psf2Local = CalcPSFSquared(psf); maxFull = GetMax(psf2Local)
    Buf local;
    CK(local.ensure(sizeof(float) * static_cast<size_t>(4) * h * w));
    CK(cd->psf_tmp.ensure(sizeof(float) * static_cast<size_t>(h) * w));
    CK(cudaMemcpyAsync(cd->psf_tmp.p, psf, sizeof(float) * static_cast<size_t>(h) * w, cudaMemcpyHostToDevice,
                       cd->stream));
    p9idg_status st = dev_psf_squared(cd->psf_tmp.as<float>(), h, w, local.as<float>(), cd->sq0, cd->sq1, cd->fft,
                                      cd->stream);
    float max_full = 0.0f;
    if (st == P9IDG_OK) st = dev_max(local.as<float>(), 2 * h, 0, cd->word.as<unsigned int>(), &max_full, cd->stream);
    local.release();
    if (st != P9IDG_OK) return st;
    cd->max_lipschitz = max_full;
    std::vector<double> scan;
    amap_scan(psf, h, w, scan);
    Buf d_scan;
    CK(d_scan.ensure(sizeof(double) * scan.size()));
    CK(cudaMemcpyAsync(d_scan.p, scan.data(), sizeof(double) * scan.size(), cudaMemcpyHostToDevice, cd->stream));
    amap_kernel<<<grid_for(static_cast<int64_t>(cd->n) * cd->n), 256, 0, cd->stream>>>(
        d_scan.as<double>(), h, w, cd->n, cd->n, 0, 0, cd->n, cd->n, cd->amap.as<float>());
    CK(cudaGetLastError());
    const float f = max_full / max_cut;
    scale_kernel<<<grid_for(static_cast<int64_t>(cd->ph) * cd->pw), 256, 0, cd->stream>>>(
        cd->psf2.as<float>(), static_cast<int64_t>(cd->ph) * cd->pw, f);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(cd->stream));
    d_scan.release();
    return P9IDG_OK;
}

void p9idg_cd_destroy(p9idg_cd *cd) {
    if (!cd) return;
    cudaSetDevice(cd->device);
    cd_release(cd);
    delete cd;
}

// ---- PaddedConvolver ----

p9idg_status p9idg_convolver_create(const double *kernel, int32_t h, int32_t w, int32_t kernel_h, int32_t kernel_w,
                                    p9idg_convolver **out) {
    if (!out) return fail(P9IDG_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (!kernel || h <= 0 || w <= 0 || kernel_h <= 0 || kernel_w <= 0)
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    TRY(have_device());
    auto *c = new (std::nothrow) p9idg_convolver();
    if (!c) return fail(P9IDG_OUT_OF_MEMORY, "convolver allocation");
    p9idg_status st = conv_init(c, h, w, kernel_h, kernel_w);
    if (st == P9IDG_OK) {
        cudaError_t e = cudaMemcpyAsync(c->kernel.p, kernel, sizeof(double2) * static_cast<size_t>(h) * w,
                                        cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "convolver kernel upload");
    }
    if (st != P9IDG_OK) {
        conv_release(c);
        delete c;
        return st;
    }
    *out = c;
    return P9IDG_OK;
}

p9idg_status p9idg_convolver_create_correlation(const float *psf, int32_t psf_h, int32_t psf_w, int32_t n,
                                                p9idg_convolver **out) {
    if (!out) return fail(P9IDG_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    if (!psf || psf_h <= 0 || psf_w <= 0 || n <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    if (n + psf_h != n + psf_w) return fail(P9IDG_INVALID_ARGUMENT, "padded PSF must be square");
    TRY(have_device());
    auto *c = new (std::nothrow) p9idg_convolver();
    if (!c) return fail(P9IDG_OUT_OF_MEMORY, "convolver allocation");
    p9idg_status st = conv_init(c, n + psf_h, n + psf_w, psf_h, psf_w);
    Buf d_psf;
    if (st == P9IDG_OK) {
        cudaError_t e = d_psf.ensure(sizeof(float) * static_cast<size_t>(psf_h) * psf_w);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_psf.p, psf, sizeof(float) * static_cast<size_t>(psf_h) * psf_w,
                                cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "psf upload");
    }
    if (st == P9IDG_OK)
        st = dev_padded_correlation(d_psf.as<float>(), psf_h, psf_w, n, n, c->kernel.as<double2>(), c->fft, c->stream);
    if (st == P9IDG_OK) {
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "correlation kernel");
    }
    d_psf.release();
    if (st != P9IDG_OK) {
        conv_release(c);
        delete c;
        return st;
    }
    *out = c;
    return P9IDG_OK;
}

p9idg_status p9idg_convolver_convolve_device(p9idg_convolver *c, const float *d_image, int32_t n, float *d_out) {
    if (!c || !d_image || !d_out || n <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    CK(cudaSetDevice(c->device));
    return conv_run(c, d_image, n, d_out);
}

p9idg_status p9idg_convolver_convolve(p9idg_convolver *c, const float *image, int32_t n, float *out) {
    if (!c || !image || !out || n <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    CK(cudaSetDevice(c->device));
    const size_t bytes = sizeof(float) * static_cast<size_t>(n) * n;
    Buf in, res;
    CK(in.ensure(bytes));
    CK(res.ensure(bytes));
    CK(cudaMemcpyAsync(in.p, image, bytes, cudaMemcpyHostToDevice, c->stream));
    p9idg_status st = conv_run(c, in.as<float>(), n, res.as<float>());
    if (st == P9IDG_OK) {
        cudaError_t e = cudaMemcpyAsync(out, res.p, bytes, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) st = cuda_fail(e, "convolve");
    }
    in.release();
    res.release();
    return st;
}

void p9idg_convolver_destroy(p9idg_convolver *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    conv_release(c);
    delete c;
}

// ---- PSF helpers on host arrays ----

p9idg_status p9idg_psf_padded_fourier_correlation(const float *psf, int32_t h, int32_t w, int32_t pad_y,
                                                  int32_t pad_x, double *out) {
    if (!psf || !out || h <= 0 || w <= 0 || pad_y < 0 || pad_x < 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    TRY(have_device());
    const int H = pad_y + h, W = pad_x + w;
    if (H != W) return fail(P9IDG_INVALID_ARGUMENT, "padded PSF must be square (FFT.Shift uses the row count)");
    cudaStream_t st = nullptr;
    Buf d_psf, d_out;
    Z2Z fft;
    CK(d_psf.ensure(sizeof(float) * static_cast<size_t>(h) * w));
    CK(d_out.ensure(sizeof(double2) * static_cast<size_t>(H) * W));
    CK(cudaMemcpy(d_psf.p, psf, sizeof(float) * static_cast<size_t>(h) * w, cudaMemcpyHostToDevice));
    p9idg_status s = dev_padded_correlation(d_psf.as<float>(), h, w, pad_y, pad_x, d_out.as<double2>(), fft, st);
    if (s == P9IDG_OK) {
        cudaError_t e = cudaMemcpy(out, d_out.p, sizeof(double2) * static_cast<size_t>(H) * W, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = cuda_fail(e, "correlation");
    }
    fft.release();
    d_psf.release();
    d_out.release();
    return s;
}

p9idg_status p9idg_psf_squared(const float *psf, int32_t h, int32_t w, float *out) {
    if (!psf || !out || h <= 0 || w <= 0 || h != w) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    TRY(have_device());
    Buf d_psf, d_out, b0, b1;
    Z2Z fft;
    CK(d_psf.ensure(sizeof(float) * static_cast<size_t>(h) * w));
    CK(d_out.ensure(sizeof(float) * static_cast<size_t>(4) * h * w));
    CK(cudaMemcpy(d_psf.p, psf, sizeof(float) * static_cast<size_t>(h) * w, cudaMemcpyHostToDevice));
    p9idg_status s = dev_psf_squared(d_psf.as<float>(), h, w, d_out.as<float>(), b0, b1, fft, nullptr);
    if (s == P9IDG_OK) {
        cudaError_t e = cudaMemcpy(out, d_out.p, sizeof(float) * static_cast<size_t>(4) * h * w, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = cuda_fail(e, "psf squared");
    }
    fft.release();
    Buf *bufs[] = {&d_psf, &d_out, &b0, &b1};
    for (Buf *b : bufs) b->release();
    return s;
}

p9idg_status p9idg_psf_amap(const float *psf, int32_t h, int32_t w, int32_t total_h, int32_t total_w, float *out) {
    if (!psf || !out || h <= 0 || w <= 0 || total_h <= 0 || total_w <= 0)
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    TRY(have_device());
    std::vector<double> scan;
    amap_scan(psf, h, w, scan);
    Buf d_scan, d_out;
    CK(d_scan.ensure(sizeof(double) * scan.size()));
    CK(d_out.ensure(sizeof(float) * static_cast<size_t>(total_h) * total_w));
    CK(cudaMemcpy(d_scan.p, scan.data(), sizeof(double) * scan.size(), cudaMemcpyHostToDevice));
    amap_kernel<<<grid_for(static_cast<int64_t>(total_h) * total_w), 256>>>(d_scan.as<double>(), h, w, total_h, total_w,
                                                                            0, 0, total_h, total_w, d_out.as<float>());
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, d_out.p, sizeof(float) * static_cast<size_t>(total_h) * total_w, cudaMemcpyDeviceToHost));
    d_scan.release();
    d_out.release();
    return P9IDG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// MajorCycle.ReconstructSerialCD on device buffers

namespace {

struct McState {
    Buf layers, resid, model_vis, xgrid, grad, psf_cut, word, partial, own_model, own_resid, own_psf;
    cufftHandle c2c = 0;
    ~McState() {
        Buf *bufs[] = {&layers, &resid, &model_vis, &xgrid, &grad, &psf_cut, &word, &partial, &own_model, &own_resid,
                       &own_psf};
        for (Buf *b : bufs) b->release();
        if (c2c) cufftDestroy(c2c);
    }
};

double elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

p9idg_status major_cycle(p9idg_plan *plan, const p9idg_mc_params *mp, const float2 *d_vis, const uint8_t *d_flags,
                         float *d_model, float *d_residual, float *d_psf, p9idg_mc_cycle *cycles, int32_t *ncycles) {
    p9idg_plan_info info{};
    TRY(p9idg_plan_get_info(plan, &info));
    p9idg_params c{};
    TRY(p9idg_plan_get_params(plan, &c));
    TRY(p9idg_plan_init_device(plan));
    void *sv = nullptr;
    TRY(p9idg_plan_get_stream(plan, &sv));
    cudaStream_t st = static_cast<cudaStream_t>(sv);
    const int N = c.grid_size;
    const int64_t nn = static_cast<int64_t>(N) * N;
    const int64_t nvis = static_cast<int64_t>(info.nbl) * info.nt * info.nch;
    if (mp->psf_cut_factor <= 0 || N / mp->psf_cut_factor <= 0)
        return fail(P9IDG_INVALID_ARGUMENT, "psf cut factor must leave a PSF");
    const int P = N / mp->psf_cut_factor;
    if (mp->max_major_cycles < 0) return fail(P9IDG_INVALID_ARGUMENT, "negative cycle count");
    McState s;
    CK(s.layers.ensure(sizeof(float2) * nn * c.wlayer_count));
    CK(s.resid.ensure(sizeof(float2) * std::max<int64_t>(1, nvis)));
    CK(s.model_vis.ensure(sizeof(float2) * std::max<int64_t>(1, nvis)));
    CK(s.xgrid.ensure(sizeof(float2) * nn));
    CK(s.grad.ensure(sizeof(float) * nn));
    CK(s.psf_cut.ensure(sizeof(float) * static_cast<size_t>(P) * P));
    CK(s.word.ensure(sizeof(unsigned int)));
    if (!d_psf) {
        CK(s.own_psf.ensure(sizeof(float) * nn));
        d_psf = s.own_psf.as<float>();
    }
    cudaEvent_t ev[5];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    struct EvGuard {
        cudaEvent_t *e;
        ~EvGuard() {
            for (int i = 0; i < 5; i++) cudaEventDestroy(e[i]);
        }
    } evg{ev};

    // PSF: unit visibilities where unflagged, GridW, WStackIFFTFloat, Shift (MajorCycle.cs:35-48)
    CK(launch_unit_vis(d_flags, nvis, s.resid.as<float2>(), st));
    TRY(p9idg_grid_w_device(plan, s.resid.p, s.layers.p));
    TRY(p9idg_wstack_image_device(plan, s.layers.p, d_psf, 1));
    // psfCut, maxSidelobe (MajorCycle.cs:54-55)
    cut_kernel<<<grid_for(static_cast<int64_t>(P) * P), 256, 0, st>>>(d_psf, N, P, N / 2 - P / 2, s.psf_cut.as<float>());
    CK(cudaGetLastError());
    float max_sidelobe = 0.0f;
    TRY(dev_max(d_psf, N, mp->psf_cut_factor, s.word.as<unsigned int>(), &max_sidelobe, st));
    TRY(p9idg_synchronize(plan));
    std::vector<float> h_cut(static_cast<size_t>(P) * P);
    CK(cudaMemcpy(h_cut.data(), s.psf_cut.p, sizeof(float) * h_cut.size(), cudaMemcpyDeviceToHost));

    // deconvolver = new FastSerialCD(totalSize, psfCut); gCalculator (MajorCycle.cs:57-73)
    p9idg_cd *cd = nullptr;
    TRY(p9idg_cd_create(N, h_cut.data(), P, P, &cd));
    struct CdGuard {
        p9idg_cd *cd;
        ~CdGuard() { p9idg_cd_destroy(cd); }
    } cdg{cd};
    TRY(p9idg_cd_set_stream(cd, st));
    p9idg_convolver *conv = nullptr;
    TRY(p9idg_convolver_create_correlation(h_cut.data(), P, P, N, &conv));
    struct ConvGuard {
        p9idg_convolver *c;
        ~ConvGuard() { p9idg_convolver_destroy(c); }
    } convg{conv};
    conv->stream = st;

    // maxLipschitz = CalcMaxLipschitz(psfCut): float squares summed in double in the reference's order
    double max_lipschitz = 0.0;
    for (float v : h_cut) {
        const float q = v * v;
        max_lipschitz += q;
    }
    const float lambda_lipschitz = static_cast<float>(mp->lambda * max_lipschitz);
    double lip_full = 0.0;
    TRY(dev_sumsq(d_psf, nn, s.partial, &lip_full, st));
    const float lambda_true = static_cast<float>(mp->lambda * lip_full);
    float lambda = mp->lambda;
    bool switched = false;

    CK(cudaMemsetAsync(d_model, 0, sizeof(float) * nn, st));
    const float2 *resid_src = d_vis;  // residualVis = data.Visibilities
    cufftHandle &c2c = s.c2c;
    CUFFT(cufftPlan2d(&c2c, N, N, CUFFT_C2C));
    CUFFT(cufftSetStream(c2c, st));
    *ncycles = 0;
    for (int cycle = 0; cycle < mp->max_major_cycles; cycle++) {
        p9idg_mc_cycle rec{};
        CK(cudaEventRecord(ev[0], st));
        TRY(p9idg_grid_w_device(plan, resid_src, s.layers.p));
        CK(cudaEventRecord(ev[1], st));
        TRY(p9idg_wstack_image_device(plan, s.layers.p, d_residual, 1));
        TRY(p9idg_synchronize(plan));
        float max_dirty = 0.0f, max_b = 0.0f;
        TRY(dev_max(d_residual, N, 0, s.word.as<unsigned int>(), &max_dirty, st));
        TRY(conv_run(conv, d_residual, N, s.grad.as<float>()));
        TRY(dev_max(s.grad.as<float>(), N, 0, s.word.as<unsigned int>(), &max_b, st));
        CK(cudaEventRecord(ev[2], st));
        // MajorCycle.cs:98-100 in the reference's types
        const double cf = static_cast<double>(max_b) / (static_cast<double>(max_dirty) * max_lipschitz);
        const double correction = cf > 1.0 ? cf : (std::isnan(cf) ? cf : 1.0);
        const double side = static_cast<double>(max_b * max_sidelobe) * correction;
        const double l1 = side / mp->alpha, l2 = lambda_lipschitz;
        const double lm = (l1 != l2) ? (!std::isnan(l1) ? (l2 < l1 ? l1 : l2) : l1) : (std::signbit(l2) ? l1 : l2);
        const float current_lambda = static_cast<float>(lm);
        float abs_max = 0.0f;
        TRY(p9idg_cd_get_abs_max_diff_device(cd, d_model, s.grad.as<float>(), lambda_true, mp->alpha, &abs_max));
        TRY(dev_objective(d_residual, d_model, nn, lambda_true, mp->alpha, s.partial, &rec.objective, st));
        rec.max_dirty = max_dirty;
        rec.max_b = max_b;
        rec.current_lambda = current_lambda;
        rec.abs_max = abs_max;
        if (abs_max >= mp->major_epsilon) {
            p9idg_cd_result r{};
            TRY(p9idg_cd_deconvolve_device(cd, d_model, s.grad.as<float>(), current_lambda, mp->alpha,
                                           mp->deconv_iterations, mp->deconv_epsilon, &r));
            rec.deconvolved = 1;
            rec.converged = r.converged;
            rec.iterations = r.iterations;
        }
        CK(cudaEventRecord(ev[3], st));
        if (lambda == current_lambda && !switched) {  // MajorCycle.cs:109-115
            lambda = lambda_true;
            max_lipschitz = lip_full;
            switched = true;
        }
        const bool stop = abs_max < mp->major_epsilon;
        if (!stop) {
            shifted_real_to_c64_kernel<<<grid_for(nn), 256, 0, st>>>(d_model, N, s.xgrid.as<float2>());
            CK(cudaGetLastError());
            CUFFT(cufftExecC2C(c2c, s.xgrid.as<cufftComplex>(), s.xgrid.as<cufftComplex>(), CUFFT_FORWARD));
            TRY(p9idg_degrid_w_device(plan, s.xgrid.p, s.model_vis.p));
            vis_subtract_kernel<<<grid_for(nvis), 256, 0, st>>>(d_vis, s.model_vis.as<float2>(), d_flags, nvis,
                                                                 s.resid.as<float2>());
            CK(cudaGetLastError());
            resid_src = s.resid.as<float2>();
        }
        CK(cudaEventRecord(ev[4], st));
        TRY(p9idg_synchronize(plan));
        rec.grid_ms = elapsed_ms(ev[0], ev[1]);
        rec.image_ms = elapsed_ms(ev[1], ev[2]);
        rec.deconv_ms = elapsed_ms(ev[2], ev[3]);
        rec.degrid_ms = elapsed_ms(ev[3], ev[4]);
        if (cycles) cycles[cycle] = rec;
        *ncycles = cycle + 1;
        if (stop) break;
    }
    return P9IDG_OK;
}

}  // namespace

extern "C" {

p9idg_status p9idg_major_cycle_serial_cd_device(p9idg_plan *plan, const p9idg_mc_params *params, const void *d_vis,
                                                const uint8_t *d_flags, float *d_model, float *d_residual,
                                                float *d_psf, p9idg_mc_cycle *cycles, int32_t *ncycles) {
    if (!plan || !params || !d_vis || !d_flags || !d_model || !d_residual || !ncycles)
        return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    return major_cycle(plan, params, static_cast<const float2 *>(d_vis), d_flags, d_model, d_residual, d_psf, cycles,
                       ncycles);
}

p9idg_status p9idg_major_cycle_serial_cd(p9idg_plan *plan, const p9idg_mc_params *params, const double *vis,
                                         const uint8_t *flags, float *model_out, float *residual_out, float *psf_out,
                                         p9idg_mc_cycle *cycles, int32_t *ncycles) {
    if (!plan || !params || !vis || !flags || !model_out || !residual_out || !ncycles)
        return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(have_device());
    p9idg_plan_info info{};
    TRY(p9idg_plan_get_info(plan, &info));
    p9idg_params c{};
    TRY(p9idg_plan_get_params(plan, &c));
    TRY(p9idg_plan_init_device(plan));
    const int64_t nvis = static_cast<int64_t>(info.nbl) * info.nt * info.nch;
    const int64_t nn = static_cast<int64_t>(c.grid_size) * c.grid_size;
    Buf v128, v64, fl, model, resid, psf;
    CK(v128.ensure(sizeof(double2) * std::max<int64_t>(1, nvis)));
    CK(v64.ensure(sizeof(float2) * std::max<int64_t>(1, nvis)));
    CK(fl.ensure(std::max<int64_t>(1, nvis)));
    CK(model.ensure(sizeof(float) * nn));
    CK(resid.ensure(sizeof(float) * nn));
    CK(psf.ensure(sizeof(float) * nn));
    void *sv = nullptr;
    TRY(p9idg_plan_get_stream(plan, &sv));
    cudaStream_t st = static_cast<cudaStream_t>(sv);
    CK(cudaMemcpyAsync(v128.p, vis, sizeof(double2) * nvis, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(fl.p, flags, nvis, cudaMemcpyHostToDevice, st));
    CK(launch_c128_to_c64(v128.as<double2>(), nvis, v64.as<float2>(), st));
    CK(cudaStreamSynchronize(st));
    v128.release();
    TRY(major_cycle(plan, params, v64.as<float2>(), fl.as<uint8_t>(), model.as<float>(), resid.as<float>(),
                    psf.as<float>(), cycles, ncycles));
    CK(cudaMemcpy(model_out, model.p, sizeof(float) * nn, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(residual_out, resid.p, sizeof(float) * nn, cudaMemcpyDeviceToHost));
    if (psf_out) CK(cudaMemcpy(psf_out, psf.p, sizeof(float) * nn, cudaMemcpyDeviceToHost));
    Buf *bufs[] = {&v64, &fl, &model, &resid, &psf};
    for (Buf *b : bufs) b->release();
    return P9IDG_OK;
}

}  // extern "C"
