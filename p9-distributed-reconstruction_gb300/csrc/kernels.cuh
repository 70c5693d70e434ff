// Device-side helpers and kernel launchers shared by the .cu files.
#pragma once

#include <cuda_runtime.h>

#include "p9idg_internal.h"

namespace p9idg {

// Device status word bits set by kernels whose own checks trip (the access is skipped).
// kStatusWTerm: a tensor-core call's uvw put |dw r| above P9IDG_TC_MAX_W_TERM (the plan's own
// uvw was checked when the mode was selected; this catches a different uvw passed to a call)
enum : int32_t { kStatusIndex = 1, kStatusWait = 2, kStatusWTerm = 4 };

// cudaMalloc for every device buffer the library keeps (plans, deconvolvers, tensor-core state),
// failing with cudaErrorMemoryAllocation once p9idg_debug_fail_device_allocations has armed it
// (api.cu).  The allocation-free entry point's fixed scratch array does not come through here.
cudaError_t device_alloc(void **p, size_t bytes);

// FFT.Shift (FFT.cs:221-264) as an index map on a square [n][n] array: the quadrant swap
// of the leading 2*(n/2) rows/columns; for odd n the last row and column stay in place.
__host__ __device__ inline void shift_index(int n, int &r, int &c) {
    const int n2 = n / 2, m = 2 * n2;
    if (r < m && c < m) {
        r = r + n2 < m ? r + n2 : r - n2;
        c = c + n2 < m ? c + n2 : c - n2;
    }
}

__device__ inline float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.y * b.x + a.x * b.y);
}

__device__ inline float2 load_vis(const float2 *v, int64_t i) { return v[i]; }
__device__ inline float2 load_vis(const double2 *v, int64_t i) {
    const double2 d = v[i];
    return make_float2(static_cast<float>(d.x), static_cast<float>(d.y));
}
__device__ inline void store_vis(float2 *v, int64_t i, float2 x) { v[i] = x; }
__device__ inline void store_vis(double2 *v, int64_t i, float2 x) { v[i] = make_double2(x.x, x.y); }

// ---- launchers (gridder_fp32.cu) ----
struct GridderArgs {
    Geometry g;
    const WorkItem *items;
    int32_t nitems;
    const DevSubgrid *subs;
    const double *uvw;         // [nbl][nt][3]
    const void *vis;           // complex64 or complex128 [nbl][nt][nch]
    bool vis_c128;
    const double *wavenumbers; // [nch]
    const float *lmn;          // l[S], n[S*S]
    const float *taper;        // [S*S]
    float2 *partials;          // gridder: [slots][S][S] (fftshifted, as Gridder.Forward writes)
    const float2 *subgrids;    // degridder: [nsub][S][S] after SubgridFFT.Backward
    void *vis_out;             // degridder output (complex64 or complex128)
    bool out_c128;
    int32_t nsub;              // subgrids in `subs`
    int32_t *status;           // device status word
    // batched launches: work items left in this problem; the CTA finishing the last one
    // records the GPU time (ns) in *finish_ns.  Null when not tracked.
    int32_t *done;
    unsigned long long *finish_ns;
};

// Batched launches pass `probs` (device array of per-problem arguments, indexed by
// WorkItem::problem); `a` then only supplies the launch-wide item list and sizes.
cudaError_t launch_gridder_fp32(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs = nullptr);
cudaError_t launch_degridder_fp32(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs = nullptr);
bool fp32_subgrid_size_supported(int S);

__device__ inline unsigned long long device_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Called by thread 0 after the block's last global store for an item: counts the item down
// and stamps the problem's completion time when it was the last one.
__device__ inline void note_item_done(int32_t *done, unsigned long long *finish_ns) {
    if (!done) return;
    __threadfence();
    if (atomicSub(done, 1) == 1) *finish_ns = device_ns();
}

// ---- launchers (subgrid_ops.cu) ----
struct SubgridOpArgs {
    Geometry g;
    const DevSubgrid *subs;
    int32_t nsub;
    const float2 *add_phasor;  // exp(+i pi (x+y-S)/S), [S][S]
    const float2 *partials;    // ifft_add input
    float2 *layers;            // ifft_add output [W][N][N] (or one grid)
    const float2 *grid;        // split input [N][N]
    bool grid_shifted;         // split: grid already FFT.Shift-ed (else the shift is applied on read)
    bool out_shifted;          // ifft_add: apply FFT.Shift to the destination index
    float2 *subgrids;          // split output [nsub][S][S]
    bool wstack;               // AdderWStack (mirror/conjugate negative w) vs Adder
    int32_t *status;
    const int2 *refs;          // batched launches: (problem, subgrid) per block; nsub = count
    const int32_t *sub_list;   // own launches: subgrid index per block (null: the block index)
    const float2 *twiddles;    // exp(+2 pi i j / S), j < S, made in FP64 (null: the kernels make them)
};
cudaError_t launch_subgrid_ifft_add(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs = nullptr);
cudaError_t launch_split_subgrid_fft(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs = nullptr);

// ---- launchers (grid_ops.cu) ----
// c128 (unshifted, host layout) -> c64 shifted copy and, when out128 != null, c128 shifted copy.
cudaError_t launch_shift_convert(const double2 *in, int n, float2 *out64, double2 *out128, cudaStream_t st);
cudaError_t launch_c64_to_c128(const float2 *in, int64_t count, double2 *out, cudaStream_t st);
// zeroes the (start, count) index ranges of a complex64 or complex128 array
cudaError_t launch_zero_ranges(void *out, bool c128, const int64_t *ranges, int64_t nranges, cudaStream_t st);
// zero-fills to run beside a tensor-core gridder or degridder: CTAs of 128 threads, at most one per SM
cudaError_t launch_zero_ranges_beside(void *out, bool c128, const int64_t *ranges, int64_t nranges, cudaStream_t st);
cudaError_t launch_zero_c64_beside(float2 *out, int64_t count, cudaStream_t st);
cudaError_t launch_zero_c128(double2 *out, int64_t count, cudaStream_t st);
// *flag (int32, device) = whether two device arrays of nwords 64-bit words differ anywhere
cudaError_t launch_words_differ(const void *a, const void *b, int64_t nwords, int32_t *flag, cudaStream_t st);
cudaError_t launch_c128_to_c64(const double2 *in, int64_t count, float2 *out, cudaStream_t st);
cudaError_t launch_unit_vis(const uint8_t *flags, int64_t count, float2 *out, cudaStream_t st);
// sum over layers (c64 or c128 input) -> c64 grid
cudaError_t launch_layer_sum(const void *layers, bool c128, int nlayers, int64_t nn, float2 *out, cudaStream_t st);
// real part / norm, optional FFT.Shift, to float or double
cudaError_t launch_real_part(const float2 *in, int n, double norm, bool shift, float *outf, double *outd,
                             cudaStream_t st);
cudaError_t launch_real_to_c64(const float *in, int64_t count, float2 *out, cudaStream_t st);
cudaError_t launch_scale_c64_to_c128(const float2 *in, int64_t count, double inv_norm, double2 *out, cudaStream_t st);
cudaError_t launch_shift_inplace(void *a, int n, int elem_bytes, cudaStream_t st);
cudaError_t measure_sincos(double *sincos_per_s, double *fma_per_s);

}  // namespace p9idg
