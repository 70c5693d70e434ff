// Grid-wide element kernels: FFT.Shift folded into conversions, complex128 <-> complex64
// boundary conversions, unit (PSF) visibilities, the w-layer sum and the real-part
// extraction that follows the full-grid inverse FFT (FFT.WStackIFFTFloat, FFT.cs:188-215;
// FFT.Backward, FFT.cs:159-185), plus the sincos throughput probe used as the FP32/SFU
// roofline denominator.  All are grid-stride loops sized to the SM count.

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "kernels.cuh"

namespace p9idg {

namespace {

int sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 132;
    }
    return sms;
}

int grid_blocks(int64_t n, int threads) {
    const int sms = sm_count();
    const int64_t want = (n + threads - 1) / threads;
    return static_cast<int>(want < static_cast<int64_t>(sms) * 8 ? (want > 0 ? want : 1) : sms * 8);
}

__global__ void shift_convert_kernel(const double2 *__restrict__ in, int n, float2 *__restrict__ out64,
                                     double2 *__restrict__ out128) {
    const int64_t nn = static_cast<int64_t>(n) * n;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nn;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int r = static_cast<int>(i / n), c = static_cast<int>(i - (i / n) * n);
        shift_index(n, r, c);
        const double2 v = in[static_cast<int64_t>(r) * n + c];
        out64[i] = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
        if (out128) out128[i] = v;
    }
}

__global__ void c64_to_c128_kernel(const float2 *__restrict__ in, int64_t count, double2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2(v.x, v.y);
    }
}

__global__ void c128_to_c64_kernel(const double2 *__restrict__ in, int64_t count, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
}

__global__ void unit_vis_kernel(const uint8_t *__restrict__ flags, int64_t count, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = make_float2(flags[i] ? 0.f : 1.f, 0.f);  // IDG.cs:59-62
}

template <typename T>
__global__ void layer_sum_kernel(const T *__restrict__ layers, int nlayers, int64_t nn, float2 *__restrict__ out) {
    // complex128 layers sum in FP64; complex64 layers in FP32 (the single-precision transform
    // that follows dominates the rounding, and FP64 arithmetic is slow on this GPU)
    using Acc = typename std::conditional<sizeof(T) == 16, double, float>::type;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nn;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        Acc re = 0, im = 0;
        for (int k = 0; k < nlayers; k++) {
            const T v = layers[static_cast<int64_t>(k) * nn + i];
            re += v.x;
            im += v.y;
        }
        out[i] = make_float2(static_cast<float>(re), static_cast<float>(im));
    }
}

// inv_norm = 1 / norm, made on the host: a multiply instead of an FP64 division per pixel
__global__ void real_part_kernel(const float2 *__restrict__ in, int n, double inv_norm, bool shift,
                                 float *__restrict__ outf, double *__restrict__ outd) {
    const int64_t nn = static_cast<int64_t>(n) * n;
    const bool small = nn < (int64_t(1) << 31);  // 32-bit index arithmetic
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nn;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int r, c;
        if (small) {
            const uint32_t u = static_cast<uint32_t>(i), q = u / static_cast<uint32_t>(n);
            r = static_cast<int>(q);
            c = static_cast<int>(u - q * static_cast<uint32_t>(n));
        } else {
            r = static_cast<int>(i / n);
            c = static_cast<int>(i - static_cast<int64_t>(r) * n);
        }
        if (shift) shift_index(n, r, c);
        const double v = static_cast<double>(in[static_cast<int64_t>(r) * n + c].x) * inv_norm;
        if (outf) outf[i] = static_cast<float>(v);
        if (outd) outd[i] = v;
    }
}

__global__ void real_to_c64_kernel(const float *__restrict__ in, int64_t count, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = make_float2(in[i], 0.f);
}

// inv_norm = 1 / norm, made on the host (the values come from a single-precision transform)
__global__ void scale_c64_to_c128_kernel(const float2 *__restrict__ in, int64_t count, double inv_norm,
                                         double2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2(static_cast<double>(v.x) * inv_norm, static_cast<double>(v.y) * inv_norm);
    }
}

template <typename T>
__global__ void shift_inplace_kernel(T *a, int n) {
    const int n2 = n / 2;
    const int64_t cnt = static_cast<int64_t>(n2) * n2;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < cnt;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int i = static_cast<int>(k / n2), j = static_cast<int>(k - (k / n2) * n2);
        const int64_t a13 = static_cast<int64_t>(i) * n + j, b13 = static_cast<int64_t>(i + n2) * n + j + n2;
        const int64_t a24 = static_cast<int64_t>(i + n2) * n + j, b24 = static_cast<int64_t>(i) * n + j + n2;
        T t = a[a13];
        a[a13] = a[b13];
        a[b13] = t;
        t = a[a24];
        a[a24] = a[b24];
        a[b24] = t;
    }
}

// Throughput probe: independent chains of the FP32 hardware sincos the kernels use.
constexpr int kProbeChains = 8;
__global__ void sincos_probe_kernel(int iters, float seed, float *sink) {
    float x[kProbeChains], acc = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) x[c] = seed + 0.001f * (threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kProbeChains; c++) {
            float s, co;
            __sincosf(x[c], &s, &co);
            x[c] = fmaf(s, 0.5f, co);
        }
    }
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) acc += x[c];
    if (acc == 12345.678f) sink[0] = acc;
}

__global__ void fma_probe_kernel(int iters, float seed, float *sink) {
    float x[kProbeChains], acc = 0.f;
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) x[c] = seed + 0.001f * (threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kProbeChains; c++) x[c] = fmaf(x[c], 0.9999f, 0.0001f);
    }
#pragma unroll
    for (int c = 0; c < kProbeChains; c++) acc += x[c];
    if (acc == 12345.678f) sink[0] = acc;
}

}  // namespace

cudaError_t launch_shift_convert(const double2 *in, int n, float2 *out64, double2 *out128, cudaStream_t st) {
    shift_convert_kernel<<<grid_blocks(static_cast<int64_t>(n) * n, 256), 256, 0, st>>>(in, n, out64, out128);
    return cudaGetLastError();
}

// Zeroes the listed index ranges (pairs start, count) of a complex64 or complex128 array.
template <typename T>
__global__ void zero_ranges_kernel(T *__restrict__ out, const int64_t *__restrict__ ranges, int64_t nranges) {
    T z;
    z.x = 0;
    z.y = 0;
    for (int64_t r = blockIdx.x; r < nranges; r += gridDim.x) {
        const int64_t start = ranges[2 * r], count = ranges[2 * r + 1];
        for (int64_t j = threadIdx.x; j < count; j += blockDim.x) out[start + j] = z;
    }
}

// Zeroes n8 8-byte words from an 8-byte aligned address, in 16-byte stores from the first 16-byte
// boundary on (the word before it, if any, and an odd last word by single stores).
__global__ void zero_words_kernel(uint2 *__restrict__ out, int64_t n8) {
    const int64_t head = (reinterpret_cast<uintptr_t>(out) & 15) != 0 && n8 > 0 ? 1 : 0;
    const int64_t n16 = (n8 - head) / 2;
    uint4 *body = reinterpret_cast<uint4 *>(out + head);
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n16;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        body[i] = make_uint4(0u, 0u, 0u, 0u);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (head) out[0] = make_uint2(0u, 0u);
        if ((n8 - head) & 1) out[n8 - 1] = make_uint2(0u, 0u);
    }
}

__global__ void zero_c128_kernel(double2 *__restrict__ out, int64_t count) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        out[i] = make_double2(0.0, 0.0);
}

// *flag = 1 when the two arrays of n 64-bit words differ anywhere (bitwise); *flag must be 0 before.
__global__ void words_differ_kernel(const uint64_t *__restrict__ a, const uint64_t *__restrict__ b, int64_t n,
                                    int32_t *flag) {
    bool diff = false;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        diff |= a[i] != b[i];
    if (__syncthreads_or(diff) && threadIdx.x == 0) *flag = 1;
}

cudaError_t launch_words_differ(const void *a, const void *b, int64_t nwords, int32_t *flag, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
    if (e != cudaSuccess || nwords == 0) return e;
    words_differ_kernel<<<grid_blocks(nwords, 256), 256, 0, st>>>(static_cast<const uint64_t *>(a),
                                                                  static_cast<const uint64_t *>(b), nwords, flag);
    return cudaGetLastError();
}

// Few CTAs: this zero-fill of host memory is bound by the link and runs beside the gridder, which
// should keep the SMs.
cudaError_t launch_zero_c128(double2 *out, int64_t count, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    zero_c128_kernel<<<32, 512, 0, st>>>(out, count);
    return cudaGetLastError();
}

cudaError_t launch_zero_ranges(void *out, bool c128, const int64_t *ranges, int64_t nranges, cudaStream_t st) {
    if (nranges == 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>(nranges, 8192));
    if (c128)
        zero_ranges_kernel<double2><<<blocks, 256, 0, st>>>(static_cast<double2 *>(out), ranges, nranges);
    else
        zero_ranges_kernel<float2><<<blocks, 256, 0, st>>>(static_cast<float2 *>(out), ranges, nranges);
    return cudaGetLastError();
}

// The two zero-fills that run beside the gridder or degridder (on a high-priority stream): CTAs of
// 128 threads, which fit in the registers, threads and shared memory that two tensor-core gridder
// or degridder CTAs leave free on an SM, so they neither wait for those kernels' items nor take an
// SM from them.  Measured on the 3072^2 workload: the 604 MB layer fill slowed the gridder by
// 0.023 ms with one CTA per four SMs, 0.032 ms with one per SM, and 0.070 ms as a cudaMemsetAsync
// on the same stream, ending well before the gridder does; the 180 MB fill of the uncovered
// visibilities, over 823 ranges, cost splitter + degridder 0.010 ms less with one CTA per SM than
// with one per four SMs.
cudaError_t launch_zero_ranges_beside(void *out, bool c128, const int64_t *ranges, int64_t nranges, cudaStream_t st) {
    if (nranges == 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>(std::min<int64_t>(nranges, sm_count()));
    if (c128)
        zero_ranges_kernel<double2><<<blocks, 128, 0, st>>>(static_cast<double2 *>(out), ranges, nranges);
    else
        zero_ranges_kernel<float2><<<blocks, 128, 0, st>>>(static_cast<float2 *>(out), ranges, nranges);
    return cudaGetLastError();
}

cudaError_t launch_zero_c64_beside(float2 *out, int64_t count, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    zero_words_kernel<<<std::max(1, sm_count() / 4), 128, 0, st>>>(reinterpret_cast<uint2 *>(out), count);
    return cudaGetLastError();
}

cudaError_t launch_c64_to_c128(const float2 *in, int64_t count, double2 *out, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    c64_to_c128_kernel<<<grid_blocks(count, 256), 256, 0, st>>>(in, count, out);
    return cudaGetLastError();
}

cudaError_t launch_c128_to_c64(const double2 *in, int64_t count, float2 *out, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    c128_to_c64_kernel<<<grid_blocks(count, 256), 256, 0, st>>>(in, count, out);
    return cudaGetLastError();
}

cudaError_t launch_unit_vis(const uint8_t *flags, int64_t count, float2 *out, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    unit_vis_kernel<<<grid_blocks(count, 256), 256, 0, st>>>(flags, count, out);
    return cudaGetLastError();
}

cudaError_t launch_layer_sum(const void *layers, bool c128, int nlayers, int64_t nn, float2 *out, cudaStream_t st) {
    if (c128)
        layer_sum_kernel<double2><<<grid_blocks(nn, 256), 256, 0, st>>>(static_cast<const double2 *>(layers),
                                                                         nlayers, nn, out);
    else
        layer_sum_kernel<float2><<<grid_blocks(nn, 256), 256, 0, st>>>(static_cast<const float2 *>(layers),
                                                                        nlayers, nn, out);
    return cudaGetLastError();
}

cudaError_t launch_real_part(const float2 *in, int n, double norm, bool shift, float *outf, double *outd,
                             cudaStream_t st) {
    real_part_kernel<<<grid_blocks(static_cast<int64_t>(n) * n, 256), 256, 0, st>>>(in, n, 1.0 / norm, shift, outf,
                                                                                 outd);
    return cudaGetLastError();
}

cudaError_t launch_real_to_c64(const float *in, int64_t count, float2 *out, cudaStream_t st) {
    real_to_c64_kernel<<<grid_blocks(count, 256), 256, 0, st>>>(in, count, out);
    return cudaGetLastError();
}

cudaError_t launch_scale_c64_to_c128(const float2 *in, int64_t count, double norm, double2 *out, cudaStream_t st) {
    scale_c64_to_c128_kernel<<<grid_blocks(count, 256), 256, 0, st>>>(in, count, 1.0 / norm, out);
    return cudaGetLastError();
}

cudaError_t launch_shift_inplace(void *a, int n, int elem_bytes, cudaStream_t st) {
    const int64_t cnt = static_cast<int64_t>(n / 2) * (n / 2);
    if (cnt == 0) return cudaSuccess;
    const int b = grid_blocks(cnt, 256);
    switch (elem_bytes) {
        case 4: shift_inplace_kernel<float><<<b, 256, 0, st>>>(static_cast<float *>(a), n); break;
        case 8: shift_inplace_kernel<double><<<b, 256, 0, st>>>(static_cast<double *>(a), n); break;
        case 16: shift_inplace_kernel<double2><<<b, 256, 0, st>>>(static_cast<double2 *>(a), n); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t measure_sincos(double *sincos_per_s, double *fma_per_s) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *sink = nullptr;
    if ((e = cudaMalloc(&sink, sizeof(float))) != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    sincos_probe_kernel<<<blocks, threads>>>(64, 0.1f, sink);  // warm-up
    cudaEventRecord(a);
    sincos_probe_kernel<<<blocks, threads>>>(iters, 0.1f, sink);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    *sincos_per_s = static_cast<double>(blocks) * threads * iters * kProbeChains / (ms * 1e-3);
    fma_probe_kernel<<<blocks, threads>>>(64, 0.1f, sink);
    cudaEventRecord(a);
    fma_probe_kernel<<<blocks, threads>>>(iters * 4, 0.1f, sink);
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    *fma_per_s = static_cast<double>(blocks) * threads * iters * 4 * kProbeChains / (ms * 1e-3);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    return cudaGetLastError();
}

}  // namespace p9idg
