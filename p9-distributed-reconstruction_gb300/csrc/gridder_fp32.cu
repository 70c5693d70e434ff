// FP32 gridder and degridder kernels (the plain sincos + FMA form).
//
// Gridder.Forward (Distributed-Reconstruction/Core/ImageDomainGridder/Gridder.cs:15-87) and
// Gridder.Backwards (Gridder.cs:91-160) compute, per subgrid pixel (x, y) and visibility
// (t, ch), the phase
//     phi = (uOff - k_ch u_t) l_x + (vOff - k_ch v_t) m_y + (wOff - k_ch w_t) n_xy
// (the reference writes it as phaseOffset - phaseIndex * k_ch).  Here the three
// coefficients are formed per visibility in FP64 relative to the subgrid centre and
// rounded once to FP32; the per-pixel work is two FP32 FMAs, one hardware sincos and a
// complex multiply-accumulate.  l, m, n are the reference's own FP32 values
// (ComputeL/ComputeN, Gridder.cs:163-174), computed on the host.
//
// Work is split into (subgrid, time chunk) items ordered largest first.  The gridder
// writes one partial subgrid per item (summed, in a fixed order, by the subgrid IFFT
// kernel), so results do not depend on scheduling.  Batched launches cover the items of
// many problems (plans); each item then reads its problem's arguments from a table.

#include "kernels.cuh"

namespace p9idg {

namespace {

// Pixels per thread: the smallest divisor of S that keeps the block at <= 256 threads,
// so every thread's pixels lie in one row and share m_y.
__host__ __device__ constexpr int ppt_for(int S) {
    for (int d = 1; d <= S; d++)
        if (S % d == 0 && S * S / d <= 256) return d;
    return S;
}

constexpr int kDegridThreads = 128;
constexpr int kDegridVpt = 4;  // visibilities per degridder thread

template <int S, typename VisT, bool BATCH>
__global__ void __launch_bounds__(S * S / ppt_for(S))
    gridder_fp32_kernel(const GridderArgs L, const GridderArgs *__restrict__ probs) {
    constexpr int PPT = ppt_for(S);
    constexpr int NT = S * S / PPT;
    __shared__ float4 s_d[NT];  // per-visibility phase coefficients (du, dv, dw)
    __shared__ float2 s_v[NT];  // visibilities

    const WorkItem it = L.items[blockIdx.x];
    const GridderArgs &a = BATCH ? probs[it.problem] : L;
    const Geometry g = a.g;
    const DevSubgrid sg = a.subs[it.subgrid];
    const int tid = threadIdx.x;
    const int p0 = tid * PPT;
    const int y = p0 / S, x0 = p0 % S;
    const float m = a.lmn[y];
    float l[PPT], n[PPT], ar[PPT], ai[PPT];
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        l[k] = a.lmn[x0 + k];
        n[k] = a.lmn[S + y * S + x0 + k];
        ar[k] = 0.f;
        ai[k] = 0.f;
    }
    // Gridder.cs:38-41 (WStepLambda is 0 in the reference, so wOff is 0)
    const double uoff = static_cast<double>(sg.u + S / 2 - g.N / 2) * g.uv_scale;
    const double voff = static_cast<double>(sg.v + S / 2 - g.N / 2) * g.uv_scale;
    const double woff = 2 * kPi * (static_cast<double>(g.wstep_lambda) * (static_cast<double>(sg.w) + 0.5));

    const VisT *vis = static_cast<const VisT *>(a.vis);
    const double *uvw = a.uvw;
    const double *wn = a.wavenumbers;
    const int nvis = it.nt * g.nch;
    for (int b = 0; b < nvis; b += NT) {
        const int j = b + tid;
        if (j < nvis) {
            const int t = it.t0 + j / g.nch, ch = j - (j / g.nch) * g.nch;
            const int64_t row = static_cast<int64_t>(sg.bl) * g.nt_all + t;
            const double *q = uvw + row * 3;
            const double k = wn[ch];
            const double du = uoff - k * q[0];
            const double dv = voff - k * q[1];
            const double dw = woff - k * q[2];
            s_d[tid] = make_float4(static_cast<float>(du), static_cast<float>(dv), static_cast<float>(dw), 0.f);
            s_v[tid] = load_vis(vis, row * g.nch + ch);
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
    // taper and fftshifted destination (Gridder.cs:76-79)
    float2 *out = a.partials + static_cast<int64_t>(it.slot) * S * S;
    const int yd = (y + S / 2) % S;
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        const int x = x0 + k;
        const float tap = a.taper[y * S + x];
        out[yd * S + (x + S / 2) % S] = make_float2(ar[k] * tap, ai[k] * tap);
    }
}

// One pass of the FP32 degridder over visibility slots k < NK of this thread (b + k * 128 + tid):
// the phases in FP32 from FP64 coefficients, one sincos per pixel and visibility (Gridder.cs:97-157).
template <int S, typename OutT, int NK>
__device__ __forceinline__ void degrid_pass(const GridderArgs &a, const Geometry &g, const DevSubgrid &sg,
                                            const WorkItem &it, const float4 *s_pix, const float *s_m, double uoff,
                                            double voff, double woff, int b, int nvis) {
    const int tid = threadIdx.x;
    OutT *out = static_cast<OutT *>(a.vis_out);
    const double *uvw = a.uvw;
    const double *wn = a.wavenumbers;
    float du[NK], dv[NK], dw[NK], ar[NK], ai[NK];
    int64_t idx[NK];
#pragma unroll
    for (int k = 0; k < NK; k++) {
        const int j = b + k * kDegridThreads + tid;
        ar[k] = ai[k] = 0.f;
        du[k] = dv[k] = dw[k] = 0.f;
        idx[k] = -1;
        if (j < nvis) {
            const int t = it.t0 + j / g.nch, ch = j - (j / g.nch) * g.nch;
            const int64_t row = static_cast<int64_t>(sg.bl) * g.nt_all + t;
            const double *q = uvw + row * 3;
            const double kw = wn[ch];
            du[k] = static_cast<float>(uoff - kw * q[0]);
            dv[k] = static_cast<float>(voff - kw * q[1]);
            dw[k] = static_cast<float>(woff - kw * q[2]);
            idx[k] = row * g.nch + ch;
        }
    }
    for (int y = 0; y < S; y++) {
        const float m = s_m[y];
        float base[NK];
#pragma unroll
        for (int k = 0; k < NK; k++) base[k] = dv[k] * m;
        const float4 *row = s_pix + y * S;
#pragma unroll 4
        for (int x = 0; x < S; x++) {
            const float4 p = row[x];
#pragma unroll
            for (int k = 0; k < NK; k++) {
                const float ph = fmaf(du[k], p.z, fmaf(dw[k], p.w, base[k]));
                float sn, cs;
                __sincosf(ph, &sn, &cs);
                // pixel * exp(-i ph)   (Gridder.cs:145-147)
                ar[k] = fmaf(p.x, cs, fmaf(p.y, sn, ar[k]));
                ai[k] = fmaf(p.y, cs, fmaf(-p.x, sn, ai[k]));
            }
        }
    }
#pragma unroll
    for (int k = 0; k < NK; k++)
        if (idx[k] >= 0) store_vis(out, idx[k], make_float2(ar[k] * g.inv_s2, ai[k] * g.inv_s2));
}

template <int S, typename OutT, bool BATCH>
__global__ void __launch_bounds__(kDegridThreads)
    degridder_fp32_kernel(const GridderArgs L, const GridderArgs *__restrict__ probs) {
    extern __shared__ float4 s_pix[];  // [S*S] {re, im, l_x, n_xy}, tapered and un-shifted
    __shared__ float s_m[S];

    const WorkItem it = L.items[blockIdx.x];
    const GridderArgs &a = BATCH ? probs[it.problem] : L;
    const Geometry g = a.g;
    const DevSubgrid sg = a.subs[it.subgrid];
    const int tid = threadIdx.x;
    const float2 *data = a.subgrids + static_cast<int64_t>(it.subgrid) * S * S;
    // Gridder.cs:106-117: pixels_copy[y, x] = sph * data[(y+S/2)%S, (x+S/2)%S]
    for (int i = tid; i < S * S; i += kDegridThreads) {
        const int y = i / S, x = i - (i / S) * S;
        const float2 d = data[((y + S / 2) % S) * S + (x + S / 2) % S];
        const float tap = a.taper[i];
        s_pix[i] = make_float4(tap * d.x, tap * d.y, a.lmn[x], a.lmn[S + i]);
    }
    if (tid < S) s_m[tid] = a.lmn[tid];
    __syncthreads();

    const double uoff = static_cast<double>(sg.u + S / 2 - g.N / 2) * g.uv_scale;
    const double voff = static_cast<double>(sg.v + S / 2 - g.N / 2) * g.uv_scale;
    const double woff = 2 * kPi * (static_cast<double>(g.wstep_lambda) * (static_cast<double>(sg.w) + 0.5));
    const int nvis = it.nt * g.nch;
    for (int b = 0; b < nvis; b += kDegridThreads * kDegridVpt) {
        // visibility slots k hold b + k * 128 + tid: only the slots with some visibility left are
        // evaluated (a block-uniform count; the item's last pass is often short)
        const int nk = min(kDegridVpt, (nvis - b + kDegridThreads - 1) / kDegridThreads);
        switch (nk) {
            case 1: degrid_pass<S, OutT, 1>(a, g, sg, it, s_pix, s_m, uoff, voff, woff, b, nvis); break;
            case 2: degrid_pass<S, OutT, 2>(a, g, sg, it, s_pix, s_m, uoff, voff, woff, b, nvis); break;
            case 3: degrid_pass<S, OutT, 3>(a, g, sg, it, s_pix, s_m, uoff, voff, woff, b, nvis); break;
            default: degrid_pass<S, OutT, kDegridVpt>(a, g, sg, it, s_pix, s_m, uoff, voff, woff, b, nvis); break;
        }
    }
    if (BATCH) {
        __syncthreads();
        if (tid == 0) note_item_done(a.done, a.finish_ns);
    }
}

template <int S, bool BATCH>
cudaError_t gridder_dispatch(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    constexpr int NT = S * S / ppt_for(S);
    if (a.nitems == 0) return cudaSuccess;
    if (a.vis_c128)
        gridder_fp32_kernel<S, double2, BATCH><<<a.nitems, NT, 0, st>>>(a, probs);
    else
        gridder_fp32_kernel<S, float2, BATCH><<<a.nitems, NT, 0, st>>>(a, probs);
    return cudaGetLastError();
}

template <int S, bool BATCH>
cudaError_t degridder_dispatch(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    if (a.nitems == 0) return cudaSuccess;
    const size_t smem = sizeof(float4) * S * S;
    if (a.out_c128) {
        cudaError_t e = cudaFuncSetAttribute(degridder_fp32_kernel<S, double2, BATCH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        degridder_fp32_kernel<S, double2, BATCH><<<a.nitems, kDegridThreads, smem, st>>>(a, probs);
    } else {
        cudaError_t e = cudaFuncSetAttribute(degridder_fp32_kernel<S, float2, BATCH>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        degridder_fp32_kernel<S, float2, BATCH><<<a.nitems, kDegridThreads, smem, st>>>(a, probs);
    }
    return cudaGetLastError();
}

template <bool BATCH>
cudaError_t gridder_by_size(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    switch (a.g.S) {
        case 8: return gridder_dispatch<8, BATCH>(a, st, probs);
        case 16: return gridder_dispatch<16, BATCH>(a, st, probs);
        case 24: return gridder_dispatch<24, BATCH>(a, st, probs);
        case 32: return gridder_dispatch<32, BATCH>(a, st, probs);
        case 48: return gridder_dispatch<48, BATCH>(a, st, probs);
        default: return cudaErrorInvalidValue;
    }
}

template <bool BATCH>
cudaError_t degridder_by_size(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    switch (a.g.S) {
        case 8: return degridder_dispatch<8, BATCH>(a, st, probs);
        case 16: return degridder_dispatch<16, BATCH>(a, st, probs);
        case 24: return degridder_dispatch<24, BATCH>(a, st, probs);
        case 32: return degridder_dispatch<32, BATCH>(a, st, probs);
        case 48: return degridder_dispatch<48, BATCH>(a, st, probs);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool fp32_subgrid_size_supported(int S) { return S == 8 || S == 16 || S == 24 || S == 32 || S == 48; }

cudaError_t launch_gridder_fp32(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    return probs ? gridder_by_size<true>(a, st, probs) : gridder_by_size<false>(a, st, nullptr);
}

cudaError_t launch_degridder_fp32(const GridderArgs &a, cudaStream_t st, const GridderArgs *probs) {
    return probs ? degridder_by_size<true>(a, st, probs) : degridder_by_size<false>(a, st, nullptr);
}

}  // namespace p9idg
