// Subgrid FFTs fused with the adder and the splitter.
//
//  * subgrid_ifft_add: sums a subgrid's partial buffers (one per gridder work item),
//    applies SubgridFFT.Forward (FFTW backward, times 1/S^2; SubgridFFT.cs:11-52) and
//    adds the result into the grid as Adder.Add (Adder.cs:13-55) or AdderWStack.Add
//    (AdderWStack.cs:11-78) does: phasor exp(+i pi (x+y-S)/S), fftshifted source index,
//    and for negative w the mirrored origin, flipped pixel order and conjugated value in
//    layer -w-1.  FFT.Shift of the destination (IDG.cs:17,37) is folded into the index.
//    Overlapping subgrids meet in global FP32 vector atomics.
//  * split_subgrid_fft: Adder.Split (Adder.cs:57-95) / AdderWStack.Split
//    (AdderWStack.cs:81-139) followed by SubgridFFT.Backward (FFTW forward, unnormalised;
//    SubgridFFT.cs:54-90).  FFT.Shift of the input grid (IDG.cs:24,44) can be folded
//    into the read index.
//
// One CTA per subgrid.  The S x S transform is two passes of S-point DFTs against a
// twiddle table in shared memory (S is 8..48, so the O(S^3) form stays in the noise
// next to the gridder's O(vis * S^2) work).

#include "kernels.cuh"

namespace p9idg {

namespace {

constexpr int kThreads = 256;

template <int S>
__device__ void dft_2d(float2 (*buf)[S + 1], float2 (*tmp)[S + 1], const float2 *tw, float scale) {
    // rows: tmp[y][k] = sum_x buf[y][x] tw[(x k) mod S]
    for (int i = threadIdx.x; i < S * S; i += kThreads) {
        const int y = i / S, k = i - (i / S) * S;
        float re = 0.f, im = 0.f;
        int e = 0;
#pragma unroll 8
        for (int x = 0; x < S; x++) {
            const float2 a = buf[y][x], w = tw[e];
            re = fmaf(a.x, w.x, fmaf(-a.y, w.y, re));
            im = fmaf(a.x, w.y, fmaf(a.y, w.x, im));
            e += k;
            if (e >= S) e -= S;
        }
        tmp[y][k] = make_float2(re, im);
    }
    __syncthreads();
    // columns: buf[k][x] = scale * sum_y tmp[y][x] tw[(y k) mod S]
    for (int i = threadIdx.x; i < S * S; i += kThreads) {
        const int k = i / S, x = i - (i / S) * S;
        float re = 0.f, im = 0.f;
        int e = 0;
#pragma unroll 8
        for (int y = 0; y < S; y++) {
            const float2 a = tmp[y][x], w = tw[e];
            re = fmaf(a.x, w.x, fmaf(-a.y, w.y, re));
            im = fmaf(a.x, w.y, fmaf(a.y, w.x, im));
            e += k;
            if (e >= S) e -= S;
        }
        buf[k][x] = make_float2(re * scale, im * scale);
    }
    __syncthreads();
}

// exp(sign * 2 pi i j / S), evaluated in FP64
template <int S>
__device__ void load_twiddles(float2 *tw, int sign) {
    for (int j = threadIdx.x; j < S; j += kThreads) {
        double s, c;
        sincospi(2.0 * j / S, &s, &c);
        tw[j] = make_float2(static_cast<float>(c), static_cast<float>(sign * s));
    }
}

// Block -> (arguments, subgrid index): its own launch (all subgrids, or those of a subgrid list),
// or the (problem, subgrid) pair of a batch.
template <bool BATCH>
__device__ __forceinline__ const SubgridOpArgs &block_args(const SubgridOpArgs &L, const SubgridOpArgs *probs,
                                                          int &sidx) {
    if (BATCH) {
        const int2 r = L.refs[blockIdx.x];
        sidx = r.y;
        return probs[r.x];
    }
    sidx = L.sub_list ? L.sub_list[blockIdx.x] : static_cast<int>(blockIdx.x);
    return L;
}

template <int S, bool WSTACK, bool BATCH>
__global__ void __launch_bounds__(kThreads)
    subgrid_ifft_add_kernel(const SubgridOpArgs L, const SubgridOpArgs *__restrict__ probs) {
    __shared__ float2 buf[S][S + 1];
    __shared__ float2 tmp[S][S + 1];
    __shared__ float2 tw[S];
    int sidx;
    const SubgridOpArgs &a = block_args<BATCH>(L, probs, sidx);
    const Geometry g = a.g;
    const int N = g.N;
    const DevSubgrid sg = a.subs[sidx];
    int sx = sg.u, sy = sg.v, sw = sg.w;
    bool neg = false;
    if (WSTACK) {
        neg = sw < 0;
        if (neg) {  // AdderWStack.cs:38-44
            sx = N - sx - S + 1;
            sy = N - sy - S + 1;
            sw = -sw - 1;
        }
        if (!(sx >= 1 && sx < N - S && sy >= 1 && sy < N - S)) return;  // AdderWStack.cs:47-48
        if (sw >= g.W) {
            if (threadIdx.x == 0) atomicOr(a.status, kStatusIndex);
            return;
        }
    } else {
        if (!(sx >= 0 && sx < N - S && sy >= 0 && sy < N - S)) {  // checked on the host (Adder.cs:30-50)
            if (threadIdx.x == 0) atomicOr(a.status, kStatusIndex);
            return;
        }
        sw = 0;
    }
    load_twiddles<S>(tw, +1);
    // sum of the partial subgrids, in slot order
    const float2 *part = a.partials + static_cast<int64_t>(sg.item_begin) * S * S;
    for (int i = threadIdx.x; i < S * S; i += kThreads) {
        float re = 0.f, im = 0.f;
        for (int k = 0; k < sg.item_count; k++) {
            const float2 v = part[static_cast<int64_t>(k) * S * S + i];
            re += v.x;
            im += v.y;
        }
        buf[i / S][i % S] = make_float2(re, im);
    }
    __syncthreads();
    dft_2d<S>(buf, tmp, tw, static_cast<float>(1.0 / (S * S)));

    float2 *layer = a.layers + static_cast<int64_t>(sw) * N * N;
    for (int i = threadIdx.x; i < S * S; i += kThreads) {
        const int y = i / S, x = i - (i / S) * S;
        const int y_ = neg ? S - 1 - y : y, x_ = neg ? S - 1 - x : x;
        const float2 d = buf[(y_ + S / 2) % S][(x_ + S / 2) % S];
        float2 v = cmul(a.add_phasor[y_ * S + x_], d);
        if (neg) v.y = -v.y;
        int r = sy + y, c = sx + x;
        if (a.out_shifted) shift_index(N, r, c);
        if (r < 0 || r >= N || c < 0 || c >= N) {
            atomicOr(a.status, kStatusIndex);
            continue;
        }
        atomicAdd(layer + static_cast<int64_t>(r) * N + c, v);
    }
}

template <int S, bool WSTACK, bool BATCH>
__global__ void __launch_bounds__(kThreads)
    split_subgrid_fft_kernel(const SubgridOpArgs L, const SubgridOpArgs *__restrict__ probs) {
    __shared__ float2 buf[S][S + 1];
    __shared__ float2 tmp[S][S + 1];
    __shared__ float2 tw[S];
    int sidx;
    const SubgridOpArgs &a = block_args<BATCH>(L, probs, sidx);
    const Geometry g = a.g;
    const int N = g.N;
    const DevSubgrid sg = a.subs[sidx];
    const int sx = sg.u, sy = sg.v;
    const bool neg = WSTACK && sg.w < 0;
    const bool in_range = WSTACK ? (sx >= 1 && sx < N - S && sy >= 1 && sy < N - S)
                                 : (sx >= 0 && sx < N - S && sy >= 0 && sy < N - S);
    load_twiddles<S>(tw, -1);
    for (int i = threadIdx.x; i < S * S; i += kThreads) {
        const int y = i / S, x = i - (i / S) * S;
        float2 v = make_float2(0.f, 0.f);
        if (in_range) {
            int r = neg ? N - sy - y : sy + y;  // AdderWStack.cs:117-118
            int c = neg ? N - sx - x : sx + x;
            if (!a.grid_shifted) shift_index(N, r, c);
            if (r >= 0 && r < N && c >= 0 && c < N) {
                float2 gv = a.grid[static_cast<int64_t>(r) * N + c];
                if (neg) gv.y = -gv.y;
                const float2 ap = a.add_phasor[y * S + x];
                v = cmul(make_float2(ap.x, -ap.y), gv);  // exp(-i pi (x+y-S)/S) * value
            } else {
                atomicOr(a.status, kStatusIndex);
            }
        }
        buf[(y + S / 2) % S][(x + S / 2) % S] = v;
    }
    __syncthreads();
    dft_2d<S>(buf, tmp, tw, 1.0f);
    float2 *out = a.subgrids + static_cast<int64_t>(sidx) * S * S;
    for (int i = threadIdx.x; i < S * S; i += kThreads) out[i] = buf[i / S][i % S];
}

template <int S, bool BATCH>
cudaError_t ifft_add_dispatch(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    if (a.nsub == 0) return cudaSuccess;
    if (a.wstack)
        subgrid_ifft_add_kernel<S, true, BATCH><<<a.nsub, kThreads, 0, st>>>(a, probs);
    else
        subgrid_ifft_add_kernel<S, false, BATCH><<<a.nsub, kThreads, 0, st>>>(a, probs);
    return cudaGetLastError();
}

template <int S, bool BATCH>
cudaError_t split_dispatch(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    if (a.nsub == 0) return cudaSuccess;
    if (a.wstack)
        split_subgrid_fft_kernel<S, true, BATCH><<<a.nsub, kThreads, 0, st>>>(a, probs);
    else
        split_subgrid_fft_kernel<S, false, BATCH><<<a.nsub, kThreads, 0, st>>>(a, probs);
    return cudaGetLastError();
}

template <bool BATCH>
cudaError_t ifft_add_by_size(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    switch (a.g.S) {
        case 8: return ifft_add_dispatch<8, BATCH>(a, st, probs);
        case 16: return ifft_add_dispatch<16, BATCH>(a, st, probs);
        case 24: return ifft_add_dispatch<24, BATCH>(a, st, probs);
        case 32: return ifft_add_dispatch<32, BATCH>(a, st, probs);
        case 48: return ifft_add_dispatch<48, BATCH>(a, st, probs);
        default: return cudaErrorInvalidValue;
    }
}

template <bool BATCH>
cudaError_t split_by_size(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    switch (a.g.S) {
        case 8: return split_dispatch<8, BATCH>(a, st, probs);
        case 16: return split_dispatch<16, BATCH>(a, st, probs);
        case 24: return split_dispatch<24, BATCH>(a, st, probs);
        case 32: return split_dispatch<32, BATCH>(a, st, probs);
        case 48: return split_dispatch<48, BATCH>(a, st, probs);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

cudaError_t launch_subgrid_ifft_add(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    return probs ? ifft_add_by_size<true>(a, st, probs) : ifft_add_by_size<false>(a, st, nullptr);
}

cudaError_t launch_split_subgrid_fft(const SubgridOpArgs &a, cudaStream_t st, const SubgridOpArgs *probs) {
    return probs ? split_by_size<true>(a, st, probs) : split_by_size<false>(a, st, nullptr);
}

}  // namespace p9idg
