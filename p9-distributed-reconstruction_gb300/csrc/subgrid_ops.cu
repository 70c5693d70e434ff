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
// twiddle table in shared memory, each split radix-4 and then in two (S is 8..48, all
// multiples of 8: an eighth of the O(S^3) multiply-adds, against the gridder's O(vis * S^2)
// work).

#include "kernels.cuh"

namespace p9idg {

namespace {

constexpr int kThreads = 256;

// One pass of the 2-D transform over S lines (ROWS: dst[y][k] = sum_x src[y][x] w^(x k); else
// dst[k][x] = sum_y src[y][x] w^(y k)), times scale, with w = tw[1] = exp(sign 2 pi i / S).
// Radix-4 split: with Q = S / 4 the outputs k + Q j (j < 4) of a line come from the four sums
// P_r(k) = sum over x = 4 m + r of a_x w^(x k) = w^(r k) sum_m a_(4m+r) w^(4 m k) through a
// 4-point DFT with root w^Q = sign i.  A thread keeps its Q twiddles w^(4 m k) in registers and
// applies w^(r k) once per sum; and as w^(4 m (k + Q/2)) = (-1)^m w^(4 m k), the even-m and
// odd-m halves of its sums give the outputs of k and of k + Q/2 together.  A pass thus reads S
// inputs and Q + 6 twiddles from shared memory per eight outputs (the pass is bound by the
// shared-memory pipe) for S complex multiply-adds.
template <int S, bool ROWS>
__device__ __forceinline__ void dft_pass(float2 (*src)[S + 1], float2 (*dst)[S + 1], const float2 *tw, float sign,
                                         float scale) {
    static_assert(S % 8 == 0, "the split needs S divisible by 8");
    constexpr int Q = S / 4, H = Q / 2;
    for (int t = threadIdx.x; t < S * H; t += kThreads) {
        const int line = t / H, k = t - (t / H) * H;
        float2 v[Q];  // w^(4 m k)
        {
            int e = 0, step = (4 * k) % S;
#pragma unroll
            for (int m = 0; m < Q; m++) {
                v[m] = tw[e];
                e += step;
                if (e >= S) e -= S;
            }
        }
        float2 Ev[4], Od[4];
#pragma unroll
        for (int r = 0; r < 4; r++) Ev[r] = Od[r] = make_float2(0.f, 0.f);
#pragma unroll
        for (int m = 0; m < Q; m++) {
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int x = 4 * m + r;
                const float2 a = ROWS ? src[line][x] : src[x][line], w = v[m];
                float2 &acc = (m & 1) ? Od[r] : Ev[r];
                acc.x = fmaf(a.x, w.x, fmaf(-a.y, w.y, acc.x));
                acc.y = fmaf(a.x, w.y, fmaf(a.y, w.x, acc.y));
            }
        }
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int kk = k + half * H;
            float2 P[4];
#pragma unroll
            for (int r = 0; r < 4; r++)
                P[r] = half ? make_float2(Ev[r].x - Od[r].x, Ev[r].y - Od[r].y)
                            : make_float2(Ev[r].x + Od[r].x, Ev[r].y + Od[r].y);
#pragma unroll
            for (int r = 1; r < 4; r++) {  // times w^(r kk)
                const float2 w = tw[(r * kk) % S];
                P[r] = make_float2(fmaf(P[r].x, w.x, -P[r].y * w.y), fmaf(P[r].x, w.y, P[r].y * w.x));
            }
            const float2 A = make_float2(P[0].x + P[2].x, P[0].y + P[2].y),
                         B = make_float2(P[0].x - P[2].x, P[0].y - P[2].y);
            const float2 C = make_float2(P[1].x + P[3].x, P[1].y + P[3].y);
            const float2 D = make_float2(-sign * (P[1].y - P[3].y), sign * (P[1].x - P[3].x));  // sign i (P1 - P3)
            const float2 X[4] = {make_float2(A.x + C.x, A.y + C.y), make_float2(B.x + D.x, B.y + D.y),
                                 make_float2(A.x - C.x, A.y - C.y), make_float2(B.x - D.x, B.y - D.y)};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 val = make_float2(X[j].x * scale, X[j].y * scale);
                if (ROWS)
                    dst[line][kk + Q * j] = val;
                else
                    dst[kk + Q * j][line] = val;
            }
        }
    }
    __syncthreads();
}

// S x S transform of buf in place (tmp: scratch), the sign of the twiddles given
template <int S>
__device__ void dft_2d(float2 (*buf)[S + 1], float2 (*tmp)[S + 1], const float2 *tw, float sign, float scale) {
    dft_pass<S, true>(buf, tmp, tw, sign, 1.f);
    dft_pass<S, false>(tmp, buf, tw, sign, scale);
}

// exp(sign * 2 pi i j / S): the plan's FP64-made table, or evaluated here in FP64
template <int S>
__device__ void load_twiddles(float2 *tw, int sign, const float2 *table) {
    for (int j = threadIdx.x; j < S; j += kThreads) {
        if (table) {
            const float2 t = table[j];
            tw[j] = make_float2(t.x, sign * t.y);
        } else {
            double s, c;
            sincospi(2.0 * j / S, &s, &c);
            tw[j] = make_float2(static_cast<float>(c), static_cast<float>(sign * s));
        }
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

// 8 CTAs per SM (32 registers) up to S = 32: 0.164 ms at 3072^2 against 0.170 ms at 6 CTAs per
// SM (its partial-subgrid loads need the resident CTAs more than registers); S = 48 fits 6 CTAs
// by shared memory (40 registers)
template <int S, bool WSTACK, bool BATCH>
__global__ void __launch_bounds__(kThreads, S <= 32 ? 8 : 6)
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
    load_twiddles<S>(tw, +1, a.twiddles);
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
    dft_2d<S>(buf, tmp, tw, 1.f, static_cast<float>(1.0 / (S * S)));

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
    load_twiddles<S>(tw, -1, a.twiddles);
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
    dft_2d<S>(buf, tmp, tw, -1.f, 1.0f);
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
