// W-stacked gridding that allocates no memory: p9idg_grid_w_device_noalloc.
//
// Who needs it: callers that cannot call cudaMalloc -- a pipeline that reserves all
// of its device memory at start-up and forbids allocation afterwards, a host
// framework whose own allocator owns every device byte, or code running on a GPU
// share with a hard memory quota.  The regular entry points keep per-plan device
// buffers that they allocate on first use; this one keeps its working memory (the
// partial subgrids, their descriptors, the adder's phasor table and a status word)
// in one file-scope __device__ array of fixed size instead.
//
// Limits and sharing:
//  * kNoAllocScratchBytes (32 MiB) is held on every GPU that loads this library's device
//    code, for the life of the process.  Under CUDA's lazy module loading (the default) that
//    happens at the first call on a device (the cudaGetSymbolAddress below), not when the
//    library is loaded: a caller with a fixed start-up reservation makes one warm-up call
//    (nsub = 0) at start-up.  The subgrids are processed in batches that fit the array
//    (4,077 subgrids at S = 32, 1,816 at S = 48); subgrid sizes above 48 and more than 64
//    channels are rejected.
//  * All calls share the array and it keeps the previous call's contents.  Every
//    scratch word a batch reads is written earlier in the same batch, and the status
//    word is cleared at the start of each call.  Calls whose GPU work overlaps (on
//    different streams, or from different host threads) race on the array: order them
//    on one stream or synchronise between them.
//  * The first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it; make that first
//    call before any stream capture begins.

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "kernels.cuh"

namespace p9idg {

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kNoAllocMaxChannels = 64;
constexpr int kNoAllocMaxDevices = 64;
constexpr size_t kStatusBytes = 256;
constexpr size_t kPhasorBytes = 48 * 48 * sizeof(float2);  // largest supported S

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device (the host-side name is only a stand-in).
void *g_scratch_ptr[kNoAllocMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

struct NoAllocArgs {
    Geometry g;
    float imagesize;
    double wn[kNoAllocMaxChannels];
    const p9idg_subgrid *subs;  // caller's device array (this batch starts at subs[0])
    int32_t count;
    const double *uvw;
    const float2 *vis;
    float2 *partials;           // scratch: [count][S][S]
    DevSubgrid *dsubs;          // scratch: [count]
    int32_t *status;            // scratch
};

__host__ __device__ constexpr int noalloc_ppt(int S) {
    for (int d = 1; d <= S; d++)
        if (S % d == 0 && S * S / d <= 256) return d;
    return S;
}

// Gridder.ComputeL / ComputeN (Gridder.cs:163-174) with explicitly rounded operations,
// so the values equal the host planner's FP32 tables.
__device__ float noalloc_l(int x, int S, float imagesize) {
    return __fdiv_rn(__fmul_rn(__fadd_rn(static_cast<float>(x - S / 2), 0.5f), imagesize), static_cast<float>(S));
}
__device__ float noalloc_n(float l, float m) {
    const float tmp = __fadd_rn(__fmul_rn(l, l), __fmul_rn(m, m));
    const double d = __dadd_rn(static_cast<double>(__fdiv_rn(tmp, 1.0f)),
                               __dsqrt_rn(__dsub_rn(1.0, static_cast<double>(tmp))));
    return __fdiv_rn(tmp, static_cast<float>(d));
}

// exp(+i pi (x+y-S)/S) for the adder (Adder.cs:39), into scratch
__global__ void noalloc_phasor_kernel(float2 *ph, int S) {
    for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < S * S; i += blockDim.x * gridDim.x) {
        const int y = i / S, x = i - (i / S) * S;
        double s, c;
        sincospi(static_cast<double>(x + y - S) / S, &s, &c);
        ph[i] = make_float2(static_cast<float>(c), static_cast<float>(s));
    }
}

// One CTA per subgrid of the batch: the FP32 gridder over all of the subgrid's samples
// into one partial subgrid, plus the descriptor the subgrid IFFT + adder kernel reads.
template <int S>
__global__ void __launch_bounds__(S * S / noalloc_ppt(S)) noalloc_gridder_kernel(const NoAllocArgs a) {
    constexpr int PPT = noalloc_ppt(S);
    constexpr int NT = S * S / PPT;
    __shared__ float4 s_d[NT];
    __shared__ float2 s_v[NT];
    const Geometry &g = a.g;
    const p9idg_subgrid sg = a.subs[blockIdx.x];
    const bool valid = sg.baseline_idx >= 0 && sg.baseline_idx < g.nbl && sg.time_sample_start >= 0 &&
                       sg.time_sample_count >= 0 &&
                       static_cast<int64_t>(sg.time_sample_start) + sg.time_sample_count <= g.nt_all;
    const int tid = threadIdx.x;
    if (tid == 0) {
        a.dsubs[blockIdx.x] = {sg.baseline_idx, sg.time_sample_start, sg.time_sample_count, sg.u_pixel,
                               sg.v_pixel, sg.w_lambda, static_cast<int32_t>(blockIdx.x), valid ? 1 : 0};
        if (!valid) atomicOr(a.status, kStatusIndex);
    }
    if (!valid) return;  // block-uniform
    const int p0 = tid * PPT;
    const int y = p0 / S, x0 = p0 % S;
    const float m = noalloc_l(y, S, a.imagesize);
    float l[PPT], n[PPT], ar[PPT], ai[PPT];
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        l[k] = noalloc_l(x0 + k, S, a.imagesize);
        n[k] = noalloc_n(l[k], m);
        ar[k] = ai[k] = 0.f;
    }
    const double uoff = static_cast<double>(sg.u_pixel + S / 2 - g.N / 2) * g.uv_scale;
    const double voff = static_cast<double>(sg.v_pixel + S / 2 - g.N / 2) * g.uv_scale;
    const double woff = 2 * kPi * (static_cast<double>(g.wstep_lambda) * (static_cast<double>(sg.w_lambda) + 0.5));
    const int nvis = sg.time_sample_count * g.nch;
    for (int b = 0; b < nvis; b += NT) {
        const int j = b + tid;
        if (j < nvis) {
            const int t = sg.time_sample_start + j / g.nch, ch = j - (j / g.nch) * g.nch;
            const int64_t row = static_cast<int64_t>(sg.baseline_idx) * g.nt_all + t;
            const double *q = a.uvw + row * 3;
            const double k = a.wn[ch];
            s_d[tid] = make_float4(static_cast<float>(uoff - k * q[0]), static_cast<float>(voff - k * q[1]),
                                   static_cast<float>(woff - k * q[2]), 0.f);
            s_v[tid] = a.vis[row * g.nch + ch];
        }
        __syncthreads();
        const int cnt = min(NT, nvis - b);
#pragma unroll 4
        for (int q = 0; q < cnt; q++) {
            const float4 d = s_d[q];
            const float2 v = s_v[q];
            const float base = d.y * m;
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                const float ph = fmaf(d.x, l[k], fmaf(d.z, n[k], base));
                float sn, cs;
                __sincosf(ph, &sn, &cs);
                ar[k] = fmaf(v.x, cs, fmaf(-v.y, sn, ar[k]));
                ai[k] = fmaf(v.y, cs, fmaf(v.x, sn, ai[k]));
            }
        }
        __syncthreads();
    }
    float2 *out = a.partials + static_cast<int64_t>(blockIdx.x) * S * S;
    const int yd = (y + S / 2) % S;
#pragma unroll
    for (int k = 0; k < PPT; k++) out[yd * S + (x0 + k + S / 2) % S] = make_float2(ar[k], ai[k]);
}

template <int S>
cudaError_t launch_noalloc_gridder(const NoAllocArgs &a, cudaStream_t st) {
    noalloc_gridder_kernel<S><<<a.count, S * S / noalloc_ppt(S), 0, st>>>(a);
    return cudaGetLastError();
}

p9idg_status noalloc_fail(p9idg_status st, const std::string &msg) {
    record_last_error(msg);
    return st;
}

// Set-up, once per device, with that device current.
p9idg_status scratch_address(unsigned char **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(P9IDG_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return noalloc_fail(P9IDG_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return noalloc_fail(P9IDG_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_scratch_ptr[dev]);
    return P9IDG_OK;
}

}  // namespace

}  // namespace p9idg

using namespace p9idg;

extern "C" p9idg_status p9idg_grid_w_device_noalloc(const p9idg_params *c, const p9idg_subgrid *d_subgrids,
                                                    int64_t nsub, const double *d_uvw, int32_t nbl, int32_t nt,
                                                    const double *frequencies, int32_t nch, const void *d_vis,
                                                    void *d_layers, void *cuda_stream) {
    if (!c || !d_layers || (nsub > 0 && (!d_subgrids || !d_uvw || !d_vis)) || (nch > 0 && !frequencies))
        return noalloc_fail(P9IDG_INVALID_ARGUMENT, "null argument");
    if (nsub < 0 || nbl < 0 || nt < 0 || nch < 0 || c->grid_size <= 0 || c->wlayer_count < 0)
        return noalloc_fail(P9IDG_INVALID_ARGUMENT, "negative size");
    const int S = c->subgrid_size, N = c->grid_size;
    if (!(S == 8 || S == 16 || S == 24 || S == 32 || S == 48) || S > N)
        return noalloc_fail(P9IDG_UNSUPPORTED, "subgrid size must be 8, 16, 24, 32 or 48 (and at most the grid size)");
    if (nch > kNoAllocMaxChannels)
        return noalloc_fail(P9IDG_UNSUPPORTED, "more than 64 channels: the allocation-free gridder keeps the "
                                               "wavenumbers in its kernel parameters");
    unsigned char *scratch = nullptr;
    p9idg_status stt = scratch_address(&scratch);
    if (stt != P9IDG_OK) return stt;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    int32_t *d_status = reinterpret_cast<int32_t *>(scratch);
    float2 *d_phasor = reinterpret_cast<float2 *>(scratch + kStatusBytes);
    unsigned char *batch_base = scratch + kStatusBytes + kPhasorBytes;
    const size_t per_subgrid = sizeof(float2) * S * S + sizeof(DevSubgrid);
    // 256 bytes of slack for aligning the partial-subgrid block after the descriptors
    const int64_t batch =
        static_cast<int64_t>((kNoAllocScratchBytes - kStatusBytes - kPhasorBytes - 256) / per_subgrid);
    DevSubgrid *d_dsubs = reinterpret_cast<DevSubgrid *>(batch_base);
    float2 *d_partials = reinterpret_cast<float2 *>(batch_base + ((sizeof(DevSubgrid) * batch + 255) / 256) * 256);

    NoAllocArgs a{};
    a.g.N = N;
    a.g.S = S;
    a.g.W = c->wlayer_count;
    a.g.nch = nch;
    a.g.nt_all = nt;
    a.g.nbl = nbl;
    a.imagesize = image_size(*c);
    a.g.uv_scale = 2 * kPi / static_cast<double>(a.imagesize);
    a.g.wstep_lambda = 0.0f;
    a.g.inv_s2 = 1.0f / static_cast<float>(S * S);
    for (int i = 0; i < nch; i++) a.wn[i] = wavenumber(frequencies[i]);
    a.uvw = d_uvw;
    a.vis = static_cast<const float2 *>(d_vis);
    a.partials = d_partials;
    a.dsubs = d_dsubs;
    a.status = d_status;

    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(int32_t), st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_layers, 0, sizeof(float2) * static_cast<size_t>(c->wlayer_count) * N * N, st);
    if (e == cudaSuccess) {
        noalloc_phasor_kernel<<<(S * S + 255) / 256, 256, 0, st>>>(d_phasor, S);
        e = cudaGetLastError();
    }
    for (int64_t first = 0; first < nsub && e == cudaSuccess; first += batch) {
        a.subs = d_subgrids + first;
        a.count = static_cast<int32_t>(nsub - first < batch ? nsub - first : batch);
        switch (S) {
            case 8: e = launch_noalloc_gridder<8>(a, st); break;
            case 16: e = launch_noalloc_gridder<16>(a, st); break;
            case 24: e = launch_noalloc_gridder<24>(a, st); break;
            case 32: e = launch_noalloc_gridder<32>(a, st); break;
            default: e = launch_noalloc_gridder<48>(a, st); break;
        }
        if (e != cudaSuccess) break;
        SubgridOpArgs o{};
        o.g = a.g;
        o.subs = d_dsubs;
        o.nsub = a.count;
        o.add_phasor = d_phasor;
        o.partials = d_partials;
        o.layers = static_cast<float2 *>(d_layers);
        o.out_shifted = true;
        o.wstack = true;
        o.status = d_status;
        e = launch_subgrid_ifft_add(o, st);
    }
    if (e != cudaSuccess) return noalloc_fail(P9IDG_CUDA_ERROR, std::string("launch: ") + cudaGetErrorString(e));
    int32_t status = 0;
    e = cudaMemcpyAsync(&status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(P9IDG_CUDA_ERROR, std::string("sync: ") + cudaGetErrorString(e));
    if (status != 0)
        return noalloc_fail(P9IDG_DEVICE_CHECK_FAILED, "a subgrid indexes samples outside uvw/vis or a w layer "
                                                       "outside the stack (status " + std::to_string(status) + ")");
    return P9IDG_OK;
}
