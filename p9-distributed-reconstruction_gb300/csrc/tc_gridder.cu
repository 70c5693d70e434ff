// Tensor-core (tcgen05) gridder and degridder, 32 operand rows per subgrid axis (S = 32, or a
// smaller S padded to 32), split precision.
//
// The per-subgrid phase of the reference (Gridder.cs:61-67, 143-145) is
//     phi_k(x, y) = du_k l_x + dv_k m_y + dw_k n(x, y)
// with n the reference's FP32 ComputeN table.  Writing n = f(x) + g(y) + r(x, y), with
// f(x) = n(l_x, 0) + c/2, g(y) = n(0, m_y) + c/2 (the same table) and r the small remainder
// (~ l^2 m^2 / 4) less the constant c that centres its range on zero (halving max |r|), the
// phasor factorises as A_k(x) B_k(y) exp(i dw_k r(x, y)) with
// A_k(x) = exp(i(du_k l_x + dw_k f_x)), B_k(y) = exp(i(dv_k m_y + dw_k g_y)).  To first
// order in dw r (|dw r| <= P9IDG_TC_MAX_W_TERM = 0.01 is enforced, so the term left out is
// <= 5e-5 of each visibility's contribution; ~5e-4 at the 3072^2 workload, ~1e-7 left out):
//   gridder:   P[y][x] = sum_k vis_k A B (1 + i dw_k r) = P0 + i r (.) P1,
//              P0 = B diag(vis) A^T,  P1 = B diag(vis dw) A^T          (rank-K updates)
//   degridder: vis_k = 1/S^2 sum_y conj(B_k(y)) [T0_k(y) - i dw_k T1_k(y)],
//              T_j = sum_x Q_j[y][x] conj(A_k(x)),  Q0 = pix, Q1 = r (.) pix   (GEMM, M = visibilities)
// Only 2*S sincos per visibility remain (vs S^2 in the FP32 kernels); the contractions
// run on tcgen05 with BF16 (or FP16) hi+lo operands: x ~ hi + lo, products hi*hi + hi*lo +
// lo*hi (the gridder also forms lo*lo) accumulated in FP32 in tensor memory.  The first-order
// rows B1 = dw B are hi only.
//
// Gridder MMA layout (per stage of 64 visibilities = K64, k = visibility; real and imaginary
// parts in separate rows; both operands MN-major, so two rows of one visibility pack into one
// BF16 pair and a lane, owning one visibility, writes 16-byte lines of 8 rows):
//   A rows (128, x = row % 32):  [Wh_re ; Wh_im ; Wl_re ; Wl_im],  W = vis_k A_k(x) = Wh + Wl
//   B rows (192, y = row % 32):  [Bh_re ; Bh_im ; B1_re ; B1_im ; Bl_re ; Bl_im]
//       B = B_k(y) = Bh + Bl,  B1 = dw_k B_k(y) (hi only); second order: + [B2_re ; B2_im]
//   one MMA per K16: M128 N192 (N256) -> TMEM lanes = the W rows, columns = the y rows
//   A warp reads its lane quarter (one W part: hi or lo, re or im; lane = x) against the re or
//   im y columns, and writes plane [y][x] of (Bh + Bl), of B1 (and of B2); the pixel step sums
//   the W hi and lo planes: P0 = (re.re - im.im, re.im + im.re) of the (Bh + Bl) planes, P1 of
//   the B1 planes.
// Degridder (per tile of 128 visibilities = rows; k = 2x + re/im):
//   A rows: [cos, sin](phase_A);  static B rows (192):  [B0_lo ; B0_hi ; B1_hi], each block of 64
//       rows in groups of four (re y, re y+1, im y, im y+1), y even, so that the epilogue reads
//       rows y and y + 1 as packed FP32 pairs
//   MMA1: A_hi x B rows 64-191 (N128) -> cols 0..127 = [T0 | T1];  MMA2: A_hi x B0_lo (N64),
//   MMA3: A_lo x B0_hi (N64) -> cols 0..63.  Two accumulators alternate (256 columns).

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>

#include "tc_gridder.cuh"
#include "tc_ptx.cuh"

namespace p9idg {

namespace {

using namespace tc;

constexpr int kS = 32;  // operand rows per subgrid axis: a subgrid of S < 32 pixels is padded to 32
// plan tables (device floats), each padded with zeros past the plan's S: the separable part g[32],
// the remainder r[32][32], and l[32] (the reference's FP32 ComputeL values)
constexpr int kTabR = kS, kTabL = kS + kS * kS, kTabs = kTabL + kS;
constexpr uint64_t kWaitNs = 2000000000ull;  // 2 s per wait before a kernel gives up

// Tensor maps for TMA staging (single-plan launches with complex64 visibilities in device
// memory): coefficients as a [ncoef][4] float32 tensor, visibilities as a [nvis] 64-bit tensor
// read 66 at a time from an even index (the TMA x coordinate must be 16-byte aligned).
struct TmaMaps {
    CUtensorMap coef;
    CUtensorMap vis;
};
constexpr int kVisBox = 66;

// (i + S / 2) mod S for 0 <= i < S: the fftshifted index of a subgrid pixel, without a division
__device__ __forceinline__ int shift_half(int i, int S) {
    const int j = i + (S >> 1);
    return j >= S ? j - S : j;
}

// The dynamic shared memory rounded up to a 1 KB boundary by pointer arithmetic on the
// __shared__ array itself, so that every pointer derived from it stays in the shared state
// space and its loads and stores compile to shared-memory instructions (an integer round trip
// would leave generic pointers behind).
__device__ __forceinline__ unsigned char *smem_1k(unsigned char *raw) {
    return raw + ((1024u - (smem_u32(raw) & 1023u)) & 1023u);
}

// ---------------- bf16 / fp16 splitting ----------------

template <bool BF16>
struct Half16;

template <>
struct Half16<true> {
    static __device__ __forceinline__ uint32_t pack(float a, float b) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    static __device__ __forceinline__ float lo_of(uint32_t w) { return __uint_as_float(w << 16); }
    static __device__ __forceinline__ float hi_of(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }
    static __device__ __forceinline__ uint32_t mul2(uint32_t x, uint32_t y) {
        __nv_bfloat162 r = __hmul2(*reinterpret_cast<__nv_bfloat162 *>(&x), *reinterpret_cast<__nv_bfloat162 *>(&y));
        return *reinterpret_cast<uint32_t *>(&r);
    }
};

template <>
struct Half16<false> {
    static __device__ __forceinline__ uint32_t pack(float a, float b) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
    static __device__ __forceinline__ float lo_of(uint32_t w) {
        return __half2float(__ushort_as_half(static_cast<unsigned short>(w & 0xFFFFu)));
    }
    static __device__ __forceinline__ float hi_of(uint32_t w) {
        return __half2float(__ushort_as_half(static_cast<unsigned short>(w >> 16)));
    }
    static __device__ __forceinline__ uint32_t mul2(uint32_t x, uint32_t y) {
        __half2 r = __hmul2(*reinterpret_cast<__half2 *>(&x), *reinterpret_cast<__half2 *>(&y));
        return *reinterpret_cast<uint32_t *>(&r);
    }
};

// (a, b) -> packed hi pair and packed lo pair (residuals).  MIXED: the residual x - hi is one
// mixed-precision FMA per value (16-bit hi times -1 plus the FP32 x; exact, as hi is x rounded);
// otherwise hi is widened back to FP32 and subtracted.  Both give the same bits; which is faster
// was measured per kernel and type (the gridder: mixed for both types, 1.5 % on BF16; the
// degridder: mixed for FP16, 2.4 % faster, the widening form for BF16, 7 % faster).
template <bool BF16, bool MIXED = true>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t &hi, uint32_t &lo) {
    hi = Half16<BF16>::pack(a, b);
    if (!MIXED) {
        lo = Half16<BF16>::pack(a - Half16<BF16>::lo_of(hi), b - Half16<BF16>::hi_of(hi));
        return;
    }
    float ra, rb;
    if (BF16)
        asm("{.reg .b16 h0, h1, m1;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m1, 0xBF80;\n\t"
            "fma.rn.f32.bf16 %0, h0, m1, %3;\n\tfma.rn.f32.bf16 %1, h1, m1, %4;\n\t}"
            : "=f"(ra), "=f"(rb) : "r"(hi), "f"(a), "f"(b));
    else
        asm("{.reg .b16 h0, h1, m1;\n\tmov.b32 {h0, h1}, %2;\n\tmov.b16 m1, 0xBC00;\n\t"
            "fma.rn.f32.f16 %0, h0, m1, %3;\n\tfma.rn.f32.f16 %1, h1, m1, %4;\n\t}"
            : "=f"(ra), "=f"(rb) : "r"(hi), "f"(a), "f"(b));
    lo = Half16<BF16>::pack(ra, rb);
}

// The "memory" clobber keeps global loads from moving across these stores, so the kernels
// prefetch the next stage's inputs into registers explicitly before storing this one.
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

__device__ __forceinline__ void named_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// 2^-e with m * 2^-e in [0.5, 1) (1 for m == 0): exact power-of-two scale
__device__ __forceinline__ float pow2_scale(float m) {
    if (!(m > 0.f) || isinf(m)) return 1.f;
    int e;
    frexpf(m, &e);
    return ldexpf(1.f, -e);
}

// max over the 256 threads of warps 0-7 (named barrier 2); red: 9 floats of shared memory
__device__ __forceinline__ float block256_max(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    named_bar(2, 256);
    if (threadIdx.x == 0) {
        float m = red[0];
        for (int i = 1; i < 8; i++) m = fmaxf(m, red[i]);
        red[8] = m;
    }
    named_bar(2, 256);
    return red[8];
}

// ---------------- per-visibility coefficients (FP64 -> FP32) ----------------

// dw_limit = P9IDG_TC_MAX_W_TERM / max |r|: a visibility with a larger |dw| (possible only when a
// call passes a uvw other than the plan's, which was checked on the host) sets kStatusWTerm.
__global__ void tc_coef_kernel(const DevSubgrid *subs, const int64_t *coef_off, const double *uvw, const double *wn,
                               Geometry g, float4 *coef, const int32_t *recompute, double dw_limit,
                               int32_t *status) {
    if (recompute && *recompute == 0) return;  // uvw bit-identical to the one coef was made from
    const DevSubgrid sg = subs[blockIdx.x];
    const double uoff = static_cast<double>(sg.u + g.S / 2 - g.N / 2) * g.uv_scale;
    const double voff = static_cast<double>(sg.v + g.S / 2 - g.N / 2) * g.uv_scale;
    const double woff = 2 * kPi * (static_cast<double>(g.wstep_lambda) * (static_cast<double>(sg.w) + 0.5));
    const int nvis = sg.nt * g.nch;
    float4 *out = coef + coef_off[blockIdx.x];
    bool over = false;
    for (int j = threadIdx.x; j < nvis; j += blockDim.x) {
        const int t = sg.t0 + j / g.nch, ch = j - (j / g.nch) * g.nch;
        const double *q = uvw + (static_cast<int64_t>(sg.bl) * g.nt_all + t) * 3;
        const double k = wn[ch];
        const double dw = woff - k * q[2];
        over |= !(fabs(dw) <= dw_limit);
        out[j] = make_float4(static_cast<float>(uoff - k * q[0]), static_cast<float>(voff - k * q[1]),
                             static_cast<float>(dw), 0.f);
    }
    if (over) atomicOr(status, kStatusWTerm);
}

// ---------------- gridder ----------------
//
// Warps 0-7 produce the MMA operands (a lane: 8 visibilities of a stage for one row, y on the A
// side and x on the B side), warp 8 issues the MMAs, warp 9 streams each stage's
// 64 coefficients and visibilities into a shared-memory ring (TMA or cp.async) so the
// producers never wait on global memory.

constexpr int kGVps = 64;      // visibilities per pipeline stage (K = 64)
constexpr int kGStages = 2;
constexpr int kGProducerWarps = 8;
constexpr int kGMmaWarp = 8;
constexpr int kGLoaderWarp = 9;
constexpr int kGThreads = 10 * 32;
constexpr int kGRing = 4;                                // input ring depth (stages)
constexpr uint32_t kGRingVis = kGVps * 16;               // visibilities after the coefficients
constexpr uint32_t kGRingSlot = kGRingVis + kGVps * 16;  // coefficients + visibilities (complex128 at most)
constexpr uint32_t kGSbo = kGVps / 8 * 128;              // bytes between 8-row groups of an operand
constexpr uint32_t kGRows32 = 4 * kGSbo;                 // bytes of 32 operand rows
constexpr uint32_t kGStageA = 128 * kGVps * 2;  // the MMA's A operand: the 128 W rows
// its B operand: the 192 y rows (256 in the second-order form)
__host__ __device__ constexpr uint32_t g_stage_bytes(bool o2) { return kGStageA + (o2 ? 256 : 192) * kGVps * 2; }
// epilogue planes (32 x 33 floats each, [y][x]): 16 (24 in the second-order form), over the
// operand stages and, in the second-order form, the input ring behind them
constexpr uint32_t kGPlane = 32 * 33 * 4;
static_assert(16 * kGPlane <= kGStages * g_stage_bytes(false), "first-order planes must fit in the stages");
static_assert(24 * kGPlane <= kGStages * g_stage_bytes(true) + kGRing * kGRingSlot,
              "second-order planes must fit in the stages and the ring");
__host__ __device__ constexpr uint32_t g_smem(bool o2) {
    return kGStages * g_stage_bytes(o2) + kGRing * kGRingSlot + 512 + 1024;
}
constexpr uint32_t kGTmemCols = 256;  // the 192 (256) columns of the y rows

// The gridder epilogue's last step for the 4 pixels a producer thread finishes: P = P0 + i r P1
// (- (r^2 / 2) P2) from the planes E, times the taper, into the work item's partial subgrid
// (fftshifted as Gridder.Forward writes it).  Rows and columns past the plan's S are padding:
// computed, never written.  SC: the subgrid size when it is the full 32 (compile-time indexing),
// else 0 and s_rt.
template <int SC, bool O2>
__device__ __forceinline__ void gridder_finish(const TcArgs &a, const float *E, int s_rt, int slot, float sv,
                                               float sw) {
    const int S = SC ? SC : s_rt;
    float ep_r[4], ep_t[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int p = threadIdx.x + k * kGProducerWarps * 32;
        const int y = p >> 5, x = p & 31;
        ep_r[k] = a.tabs[kTabR + p];
        ep_t[k] = (y < S && x < S) ? a.taper[y * S + x] : 0.f;
    }
    float2 *out = a.partials + static_cast<int64_t>(slot) * S * S;
    const float i0 = 1.f / sv, i1 = 1.f / (sv * sw), i2 = 0.5f / (sv * sw * sw);  // exact: powers of two
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int p = threadIdx.x + k * kGProducerWarps * 32;
        const int y = p >> 5, x = p & 31;
        const int e = y * 33 + x;
        // plane (kind, W part t, y part u), the W hi and lo quarters summed
        auto pl = [&](int kind, int t, int u) {
            return E[(kind * 8 + 2 * t + u) * 1056 + e] + E[(kind * 8 + 4 + 2 * t + u) * 1056 + e];
        };
        const float p0re = (pl(0, 0, 0) - pl(0, 1, 1)) * i0;
        const float p0im = (pl(0, 0, 1) + pl(0, 1, 0)) * i0;
        const float p1re = (pl(1, 0, 0) - pl(1, 1, 1)) * i1;
        const float p1im = (pl(1, 0, 1) + pl(1, 1, 0)) * i1;
        const float rr = ep_r[k], tap = ep_t[k];
        float re = fmaf(-rr, p1im, p0re), im = fmaf(rr, p1re, p0im);
        if (O2) {  // - (r^2 / 2) P2
            const float h2 = rr * rr * i2;
            re = fmaf(-h2, pl(2, 0, 0) - pl(2, 1, 1), re);
            im = fmaf(-h2, pl(2, 0, 1) + pl(2, 1, 0), im);
        }
        if (y < S && x < S) out[shift_half(y, S) * S + shift_half(x, S)] = make_float2(re * tap, im * tap);
    }
}

// O2: the second-order form (|dw r| up to P9IDG_TC_MAX_W_TERM2): y rows 192-255 carry
// B2 = dw^2 Bh (N = 256), so P = P0 + i r (.) P1 - (r^2 / 2) (.) P2 with P2 = B diag(vis dw^2) A^T.
template <bool BF16, typename VisT, bool BATCH, bool TMA, bool O2>
__global__ void __launch_bounds__(kGThreads, 2)
    tc_gridder_kernel(const TcArgs L, const TcArgs *__restrict__ probs, const __grid_constant__ TmaMaps maps) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_1k(smem_raw);
    constexpr uint32_t kGStageBytes = g_stage_bytes(O2);
    unsigned char *ring = smem + kGStages * kGStageBytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + kGRing * kGRingSlot);
    uint64_t *empty = full + kGStages;
    uint64_t *accb = empty + kGStages;
    uint64_t *in_full = accb + 1;
    uint64_t *in_empty = in_full + kGRing;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(in_empty + kGRing);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    float *red = reinterpret_cast<float *>(tmem_slot + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const WorkItem it = L.items[blockIdx.x];
    const TcArgs &a = BATCH ? probs[it.problem] : L;
    const Geometry g = a.g;
    const DevSubgrid sg = a.subs[it.subgrid];
    const int nvis = it.nt * g.nch;
    const int nstages = (nvis + kGVps - 1) / kGVps;
    // an item is a run of whole time samples: its visibilities and coefficients are contiguous
    const int64_t v0 = (static_cast<int64_t>(sg.bl) * g.nt_all + it.t0) * g.nch;  // first visibility
    const int64_t c0 = a.coef_off[it.subgrid] + static_cast<int64_t>(it.t0 - sg.t0) * g.nch;
    const VisT *vrow = static_cast<const VisT *>(a.vis) + v0;
    const float4 *crow = a.coef + c0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGStages; s++) {
            mbar_init(&full[s], kGProducerWarps);
            mbar_init(&empty[s], 1);
        }
        for (int s = 0; s < kGRing; s++) {
            mbar_init(&in_full[s], TMA ? 1 : 32);  // one expect_tx arrival, or one cp.async arrival per lane
            mbar_init(&in_empty[s], kGProducerWarps);
        }
        mbar_init(accb, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == kGMmaWarp) {
        tmem_alloc(tmem_slot, kGTmemCols);
        tmem_relinquish();
    }
    const uint32_t sbase = smem_u32(smem), rbase = smem_u32(ring);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == kGMmaWarp) {
        // ---- MMA issuer ----
        if (lane == 0) {
            constexpr uint32_t idn = idesc_f16(128, O2 ? 256 : 192, BF16, true);
            for (int i = 0; i < nstages; i++) {
                const int s = i % kGStages;
                const uint32_t ph = (i / kGStages) & 1;
                if (!mbar_wait(&full[s], ph, abort_flag, a.wait_ns)) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                    break;
                }
                tc_fence_after();
                const uint32_t A = sbase + s * kGStageBytes, B = A + kGStageA;
#pragma unroll
                for (int kc = 0; kc < kGVps / 16; kc++)
                    mma_f16(tmem, smem_desc(A + kc * 256, 128, kGSbo), smem_desc(B + kc * 256, 128, kGSbo), idn,
                            (i > 0 || kc > 0) ? 1u : 0u);
                mma_commit(&empty[s]);
            }
            mma_commit(accb);
            // the MMAs must be finished before the TMEM is released: this wait does not stop early
            // when another warp has aborted (only at its time limit)
            volatile int never = 0;
            if (!mbar_wait(accb, 0, &never, a.wait_ns)) atomicOr(a.status, kStatusWait);
        }
        __syncwarp();
    } else if (warp == kGLoaderWarp && TMA) {
        // ---- loader (TMA): stage i's 64 coefficients (one 2-D tile) and 66 visibilities from the
        // even index at or below the stage's first (one 1-D tile) -> ring slot i % kGRing
        // The last stage of an item, when it ends inside the stage, gets its visibilities from plain
        // loads with the samples past the item's end written as zeros (a TMA tile would bring the
        // next item's samples), so the producers never mask.
        int issued = 0;
        for (int i = 0; i < nstages; i++) {
            const int slot = i % kGRing;
            const uint32_t ph = (i / kGRing) & 1;
            if (!warp_wait(&in_empty[slot], ph ^ 1, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            if (i == a.debug_skip_stage) {  // fault injection: this stage never arrives
                issued = i + 1;
                continue;
            }
            const uint32_t dst = rbase + slot * kGRingSlot;
            const int valid = nvis - i * kGVps;
            if (valid < kGVps) {
                const int off = static_cast<int>((v0 + i * kGVps) & 1);
                float2 *rvw = reinterpret_cast<float2 *>(ring + slot * kGRingSlot + kGRingVis) + off;
                const float2 *src = reinterpret_cast<const float2 *>(vrow) + i * kGVps;
#pragma unroll
                for (int h = 0; h < kGVps / 32; h++) {
                    const int q = lane + 32 * h;
                    rvw[q] = q < valid ? src[q] : make_float2(0.f, 0.f);
                }
                fence_proxy_async();  // later TMA copies into this slot are ordered after these stores
                __syncwarp();
            }
            if (lane == 0) {
                mbar_expect_tx(&in_full[slot], kGVps * 16 + (valid < kGVps ? 0 : kVisBox * 8));
                tma_load_2d(dst, &maps.coef, 0, static_cast<int32_t>(c0 + i * kGVps), &in_full[slot]);
                if (valid >= kGVps)
                    tma_load_1d(dst + kGRingVis, &maps.vis, static_cast<int32_t>((v0 + i * kGVps) & ~int64_t(1)),
                                &in_full[slot]);
            }
            issued = i + 1;
        }
        // tiles still in flight land before the CTA can exit (consumed ones have completed)
        if (lane == 0) {
            volatile int never = 0;
            for (int i = issued > kGRing ? issued - kGRing : 0; i < issued; i++)
                if (!mbar_wait(&in_full[i % kGRing], (i / kGRing) & 1, &never, a.wait_ns)) atomicOr(a.status, kStatusWait);
        }
        __syncwarp();
    } else if (warp == kGLoaderWarp) {
        // ---- loader: stage i's 64 coefficients and visibilities -> ring slot i % kGRing
        for (int i = 0; i < nstages; i++) {
            const int slot = i % kGRing;
            const uint32_t ph = (i / kGRing) & 1;
            if (!warp_wait(&in_empty[slot], ph ^ 1, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            if (i == a.debug_skip_stage) continue;  // fault injection: this stage never arrives
            const uint32_t dst = rbase + slot * kGRingSlot;
#pragma unroll
            for (int h = 0; h < kGVps / 32; h++) {
                const int q = lane + 32 * h, j = i * kGVps + q;
                const bool in = j < nvis;
                cp_async_16(dst + q * 16, in ? crow + j : crow, in ? 16u : 0u);
                if (sizeof(VisT) == 16)
                    cp_async_16(dst + kGRingVis + q * 16, in ? vrow + j : vrow, in ? 16u : 0u);
                else
                    cp_async_8(dst + kGRingVis + q * 8, in ? vrow + j : vrow, in ? 8u : 0u);
            }
            cp_async_arrive(&in_full[slot]);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else {
        // ---- producers
        // Lane = visibility: warp w covers visibilities 32 (w & 1) + lane of each stage and the 8
        // rows 8 (w >> 1) .. +7 (y on the B side, x on the W side).  A lane loads its own
        // visibility's coefficients and sample (coalesced: a few shared-memory wavefronts per
        // warp instead of several per visibility for broadcasts), evaluates the 8 rows, and
        // stores each operand row group as one 16-byte line of an MN-major core matrix
        // (8 rows of one k): a warp writes 512 contiguous bytes per row group.
        const int half = warp & 1, rg = warp >> 1, kl = 32 * half + lane;
        float2 mt[4], gt[4];  // m_y and g_y of the 8 rows in pairs (l_x and f_x are the same values)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            mt[j] = make_float2(a.tabs[kTabL + 8 * rg + 2 * j], a.tabs[kTabL + 8 * rg + 2 * j + 1]);
            gt[j] = make_float2(a.tabs[8 * rg + 2 * j], a.tabs[8 * rg + 2 * j + 1]);
        }
        float sv = 1.f;  // FP16: power-of-two scale of this item's visibilities
        if (!BF16) {
            float mx = 0.f;
            for (int j = threadIdx.x; j < nvis; j += kGProducerWarps * 32) {
                const float2 v = load_vis(vrow, j);
                mx = fmaxf(mx, fmaxf(fabsf(v.x), fabsf(v.y)));
            }
            sv = pow2_scale(block256_max(mx, red));
        }
        const float sw = BF16 ? 1.f : a.dw_scale;
        for (int i = 0; i < nstages; i++) {
            const int s = i % kGStages, slot = i % kGRing;
            const uint32_t ph = (i / kGStages) & 1, iph = (i / kGRing) & 1;
            if (!warp_wait(&in_full[slot], iph, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            // the lane's own coefficients and visibility (zeros past the item's end: the loader
            // writes them so)
            const float4 c = reinterpret_cast<const float4 *>(ring + slot * kGRingSlot)[kl];
            const int off = TMA ? static_cast<int>((v0 + i * kGVps) & 1) : 0;
            const float2 vv = load_vis(reinterpret_cast<const VisT *>(ring + slot * kGRingSlot + kGRingVis) + off, kl);
            // the ring slot is released only after the values read from it have been used (below)
            if (!warp_wait(&empty[s], ph ^ 1, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            const float dws = c.z * sw;
            // both halves of a packed pair are rows of this lane's visibility: one dw for the pair,
            // and the first-order rows dw * Bh are one packed 16-bit multiply of the hi pair (relative
            // error 2^-8 of a term <= |dw r| <= P9IDG_TC_MAX_W_TERM of the sum: <= 4e-5 at the limit,
            // 7.8e-6 total error measured there against 7.7e-6 with FP32 products; 2.9 % faster)
            const uint32_t dw2 = Half16<BF16>::pack(dws, dws);
            const float vre = vv.x * sv, vim = vv.y * sv;
            const float2 cx2 = make_float2(c.x, c.x), cy2 = make_float2(c.y, c.y), cz2 = make_float2(c.z, c.z);
            const float2 vre2 = make_float2(vre, vre), vim2 = make_float2(vim, vim), nvim2 = make_float2(-vim, -vim);
            const float2 dws2 = make_float2(dws, dws);
            // words: [row pair][type] with type = Bh_re, Bh_im, B1_re, B1_im, Bl_re, Bl_im, Wh_re, Wh_im,
            // Wl_re, Wl_im; a pair packs rows (2p, 2p+1) of the warp's eight
            uint32_t wd[4][O2 ? 12 : 10];
#pragma unroll
            for (int pr = 0; pr < 4; pr++) {
                // the two rows of a pair side by side in packed FP32x2 arithmetic
                const float2 zg = __fmul2_rn(cz2, gt[pr]);
                const float2 pb = __ffma2_rn(cy2, mt[pr], zg), pa = __ffma2_rn(cx2, mt[pr], zg);
                float2 cb, sb, ca, sa;
                __sincosf(pb.x, &sb.x, &cb.x);  // B_k(y)
                __sincosf(pb.y, &sb.y, &cb.y);
                __sincosf(pa.x, &sa.x, &ca.x);  // A_k(x)
                __sincosf(pa.y, &sa.y, &ca.y);
                const float2 wre = __ffma2_rn(vre2, ca, __fmul2_rn(nvim2, sa));
                const float2 wim = __ffma2_rn(vre2, sa, __fmul2_rn(vim2, ca));
                split_pair<BF16>(cb.x, cb.y, wd[pr][0], wd[pr][4]);
                split_pair<BF16>(sb.x, sb.y, wd[pr][1], wd[pr][5]);
                if (O2) {  // dw * B rounded once from FP32: the first-order term reaches 0.03 here
                    const float2 dcb = __fmul2_rn(dws2, cb), dsb = __fmul2_rn(dws2, sb);
                    wd[pr][2] = Half16<BF16>::pack(dcb.x, dcb.y);
                    wd[pr][3] = Half16<BF16>::pack(dsb.x, dsb.y);
                } else {
                    wd[pr][2] = Half16<BF16>::mul2(wd[pr][0], dw2);  // dw * Bh (hi only)
                    wd[pr][3] = Half16<BF16>::mul2(wd[pr][1], dw2);
                }
                if (O2) {
                    wd[pr][O2 ? 10 : 0] = Half16<BF16>::mul2(wd[pr][2], dw2);  // dw^2 * Bh
                    wd[pr][O2 ? 11 : 1] = Half16<BF16>::mul2(wd[pr][3], dw2);
                }
                split_pair<BF16>(wre.x, wre.y, wd[pr][6], wd[pr][8]);
                split_pair<BF16>(wim.x, wim.y, wd[pr][7], wd[pr][9]);
            }
            // MN-major: row group G (8 rows) of an operand at G * 1024 bytes, k at 16 k
            const uint32_t A = sbase + s * kGStageBytes, B = A + kGStageA;
            const uint32_t ko = static_cast<uint32_t>(rg * kGSbo + kl * 16);
#define P9_ST(addr, r) st_shared_v4((addr), wd[0][r], wd[1][r], wd[2][r], wd[3][r])
            P9_ST(B + ko, 0);                   // Bh_re: B rows 0-31
            P9_ST(B + kGRows32 + ko, 1);        // Bh_im: 32-63
            P9_ST(B + 2 * kGRows32 + ko, 2);    // B1_re: 64-95
            P9_ST(B + 3 * kGRows32 + ko, 3);    // B1_im: 96-127
            P9_ST(B + 4 * kGRows32 + ko, 4);    // Bl_re: 128-159
            P9_ST(B + 5 * kGRows32 + ko, 5);    // Bl_im: 160-191
            if (O2) {
                P9_ST(B + 6 * kGRows32 + ko, O2 ? 10 : 0);  // B2_re: 192-223
                P9_ST(B + 7 * kGRows32 + ko, O2 ? 11 : 0);  // B2_im: 224-255
            }
            P9_ST(A + ko, 6);                   // Wh_re: A rows 0-31
            P9_ST(A + kGRows32 + ko, 7);        // Wh_im: 32-63
            P9_ST(A + 2 * kGRows32 + ko, 8);    // Wl_re: 64-95
            P9_ST(A + 3 * kGRows32 + ko, 9);    // Wl_im: 96-127
#undef P9_ST
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&full[s]);
                mbar_arrive(&in_empty[slot]);
            }
        }
        // ---- epilogue: TMEM -> smem planes -> partial subgrid
        const bool ok = warp_wait(accb, 0, abort_flag, a.wait_ns);
        tc_fence_after();
        float *E = reinterpret_cast<float *>(smem);  // the stages are free once accb completed
        // warp: TMEM lane quarter q (the W rows Wh_re, Wh_im, Wl_re, Wl_im; lane = x) against the real
        // (u = 0) or imaginary (u = 1) y rows: plane kind * 8 + 2 q + u holds [y][x] of
        // kind 0: (Bh + Bl) columns, 1: B1, 2: B2
        const int q = warp & 3, u = warp >> 2;
        if (ok) {
            uint32_t r[32];
            const uint32_t t = tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>(32 * u);
            float *e0 = E + (2 * q + u) * 1056 + lane;
            tmem_ld32(t, r);  // Bh_u
            tmem_ld_wait(r);
#pragma unroll
            for (int j = 0; j < 32; j++) e0[j * 33] = __uint_as_float(r[j]);
            tmem_ld32(t + 128, r);  // Bl_u
            tmem_ld_wait(r);
#pragma unroll
            for (int j = 0; j < 32; j++) e0[j * 33] += __uint_as_float(r[j]);
            float *e1 = E + (8 + 2 * q + u) * 1056 + lane;
            tmem_ld32(t + 64, r);  // B1_u
            tmem_ld_wait(r);
#pragma unroll
            for (int j = 0; j < 32; j++) e1[j * 33] = __uint_as_float(r[j]);
            if (O2) {
                float *e2 = E + (16 + 2 * q + u) * 1056 + lane;
                tmem_ld32(t + 192, r);  // B2_u
                tmem_ld_wait(r);
#pragma unroll
                for (int j = 0; j < 32; j++) e2[j * 33] = __uint_as_float(r[j]);
            }
        }
        tc_fence_before();
        named_bar(1, kGProducerWarps * 32);
        if (ok && !*abort_flag) {
            if (g.S == kS)  // the full size with compile-time indexing, smaller subgrids padded
                gridder_finish<kS, O2>(a, E, g.S, it.slot, sv, sw);
            else
                gridder_finish<0, O2>(a, E, g.S, it.slot, sv, sw);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kGMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem, kGTmemCols);
    }
}

// ---------------- degridder ----------------
//
// Warps 0-3 produce the A tile (128 visibilities x 32 x phasors), warps 4-7 turn the
// accumulators into visibilities, warp 8 issues the MMAs, warp 9 streams each tile's 128
// coefficients into a shared-memory ring with cp.async.

constexpr int kDTile = 128;
constexpr int kDMmaWarp = 8;
constexpr int kDLoaderWarp = 9;
constexpr int kDThreads = 10 * 32;
constexpr int kDRing = 4;
constexpr uint32_t kDRingSlot = kDTile * 16;
constexpr uint32_t kDStatic = 192 * 64 * 2;   // static B operand: [B0_lo; B0_hi; B1_hi]
constexpr uint32_t kDStatic2 = 256 * 64 * 2;  // second order: [B0_lo; B0_hi; B1_hi; B2_hi]
constexpr uint32_t kDTileHalf = 128 * 64 * 2;  // hi (or lo) operand of one tile
constexpr uint32_t kDTileBytes = 2 * kDTileHalf;
constexpr uint32_t kDSmem = kDStatic + 2 * kDTileBytes + kDRing * kDRingSlot + 256 + 512 + 1024;
constexpr uint32_t kDSmem2 = kDStatic2 + 2 * kDTileBytes + kDRing * kDRingSlot + 256 + 512 + 1024;
constexpr uint32_t kDTmemCols = 256;

// O2: the second-order form: vis = S^-2 sum_y conj(B(y)) [T0 - i dw T1 - (dw^2 / 2) T2] with
// T2 = (r^2 (.) pix) conj(A); MMA1 covers [T0 | T1 | T2] (N = 192) in one accumulator of 192
// columns (the two accumulators of the first-order form would need 384), so the MMA of tile i + 1
// waits for the epilogue of tile i.
template <bool BF16, typename OutT, bool BATCH, bool TMA, bool O2>
__global__ void __launch_bounds__(kDThreads, 2)
    tc_degridder_kernel(const TcArgs L, const TcArgs *__restrict__ probs, const __grid_constant__ TmaMaps maps) {
    constexpr int NB = O2 ? 1 : 2;  // accumulator buffers
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_1k(smem_raw);
    unsigned char *bstat = smem;
    unsigned char *tiles = smem + (O2 ? kDStatic2 : kDStatic);
    unsigned char *ring = tiles + 2 * kDTileBytes;
    float *tab_m = reinterpret_cast<float *>(ring + kDRing * kDRingSlot);  // m[32], g[32]
    float *tab_g = tab_m + kS;
    uint64_t *a_full = reinterpret_cast<uint64_t *>(tab_m + 2 * kS);
    uint64_t *a_empty = a_full + 2;
    uint64_t *acc_full = a_empty + 2;
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *in_full = acc_empty + 2;
    uint64_t *in_empty = in_full + kDRing;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(in_empty + kDRing);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    float *red = reinterpret_cast<float *>(tmem_slot + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const WorkItem it = L.items[blockIdx.x];
    const TcArgs &a = BATCH ? probs[it.problem] : L;
    const Geometry g = a.g;
    const DevSubgrid sg = a.subs[it.subgrid];
    const int nvis = it.nt * g.nch;
    const int ntiles = (nvis + kDTile - 1) / kDTile;
    const int64_t c0 = a.coef_off[it.subgrid] + static_cast<int64_t>(it.t0 - sg.t0) * g.nch;
    const float4 *crow = a.coef + c0;

    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; b++) {
            mbar_init(&a_full[b], 4);
            mbar_init(&a_empty[b], 1);
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 4);
        }
        for (int s = 0; s < kDRing; s++) {
            mbar_init(&in_full[s], TMA ? 1 : 32);  // one expect_tx arrival, or one cp.async arrival per lane
            mbar_init(&in_empty[s], 8);  // 4 producer + 4 epilogue warps read each slot
        }
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (threadIdx.x < kS) {
        tab_m[threadIdx.x] = a.tabs[kTabL + threadIdx.x];
        tab_g[threadIdx.x] = a.tabs[threadIdx.x];
    }
    if (warp == kDMmaWarp) {
        tmem_alloc(tmem_slot, kDTmemCols);
        tmem_relinquish();
    }
    // static B operand from the subgrid: row (block, 4 (y / 2) + 2 p + y % 2), k = 2x + q; pixels
    // past the plan's S (a subgrid of S < 32 padded to 32) are zero
    float sq = 1.f;  // FP16: power-of-two scale of this subgrid's pixels
    if (warp < 8) {
        const int S = g.S;
        const float2 *data = a.subgrids + static_cast<int64_t>(it.subgrid) * S * S;
        if (!BF16) {
            float mx = 0.f;
            for (int pi = threadIdx.x; pi < kS * kS; pi += 256) {
                const int y = pi >> 5, x = pi & 31;
                if (y < S && x < S) {
                    const float2 d = data[shift_half(y, S) * S + shift_half(x, S)];
                    const float tap = fabsf(a.taper[y * S + x]);
                    mx = fmaxf(mx, fmaxf(fabsf(d.x), fabsf(d.y)) * tap);
                }
            }
            sq = pow2_scale(block256_max(mx, red));
        }
        const float sr = BF16 ? 1.f : a.r_scale;
        const uint32_t bs = smem_u32(bstat);
        for (int cc = threadIdx.x; cc < (O2 ? 256 : 192) * 8; cc += 256) {
            const int cm = cc >> 3, r8 = cc & 7;
            const int row = (cm >> 3) * 8 + r8, kg = cm & 7;
            const int blk = row >> 6, rr = row & 63, y = ((rr >> 2) << 1) | (rr & 1), p = (rr >> 1) & 1;
            // the four x of this chunk: S is a multiple of 4, so they are wholly inside or outside the
            // subgrid and on one side of the fftshift wrap (consecutive source pixels)
            const int x0 = kg * 4;
            float2 dv[4];
            float tv[4];
            if (y < S && x0 < S) {
                const float2 *src = data + shift_half(y, S) * S + shift_half(x0, S);
                const float *tsrc = a.taper + y * S + x0;
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    dv[u] = src[u];
                    tv[u] = tsrc[u] * sq;
                }
            } else {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    dv[u] = make_float2(0.f, 0.f);
                    tv[u] = 0.f;
                }
            }
            uint32_t w[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int x = x0 + u;
                const float2 d = dv[u];
                const float tap = tv[u];
                float qre = tap * d.x, qim = tap * d.y;
                if (blk >= 2) {  // r (.) pix, and r^2 (.) pix for block 3
                    const float rr2 = a.tabs[kTabR + y * kS + x] * sr;
                    qre *= rr2;
                    qim *= rr2;
                    if (blk == 3) {
                        qre *= rr2;
                        qim *= rr2;
                    }
                }
                // p = re: (Q_re, Q_im);  p = im: (Q_im, -Q_re)
                const float e0 = p == 0 ? qre : qim, e1 = p == 0 ? qim : -qre;
                uint32_t hi, lo;
                split_pair<BF16>(e0, e1, hi, lo);
                w[u] = blk == 0 ? lo : hi;
            }
            st_shared_v4(bs + cc * 16, w[0], w[1], w[2], w[3]);
        }
        fence_proxy_async();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t bs = smem_u32(bstat), ts = smem_u32(tiles), rbase = smem_u32(ring);

    int drain_phase = 0;  // MMA warp: commits to a_empty[0] before the drain commit
    if (warp == kDMmaWarp) {
        // ---- MMA issuer
        if (lane == 0) {
            constexpr uint32_t id1 = idesc_f16(128, O2 ? 192 : 128, BF16), id64 = idesc_f16(128, 64, BF16);
            for (int i = 0; i < ntiles; i++) {
                const int b = i & 1, cb = i % NB;
                const uint32_t ph = (i >> 1) & 1, cph = (i / NB) & 1;
                if (!mbar_wait(&a_full[b], ph, abort_flag, a.wait_ns) ||
                    !mbar_wait(&acc_empty[cb], cph ^ 1, abort_flag, a.wait_ns)) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                    break;
                }
                tc_fence_after();
                const uint32_t ahi = ts + b * kDTileBytes, alo = ahi + kDTileHalf;
                const uint32_t acc = tmem + static_cast<uint32_t>(cb * 128);
#pragma unroll
                for (int kc = 0; kc < 4; kc++) {
                    const uint64_t dahi = smem_desc(ahi + kc * 256, 128, 1024);
                    mma_f16(acc, dahi, smem_desc(bs + 8 * 1024 + kc * 256, 128, 1024), id1, kc > 0 ? 1u : 0u);
                    mma_f16(acc, dahi, smem_desc(bs + kc * 256, 128, 1024), id64, 1u);
                    mma_f16(acc, smem_desc(alo + kc * 256, 128, 1024), smem_desc(bs + 8 * 1024 + kc * 256, 128, 1024),
                            id64, 1u);
                }
                mma_commit(&a_empty[b]);
                mma_commit(&acc_full[cb]);
                if (b == 0) drain_phase++;
            }
            // drain: every issued MMA finished before the TMEM is released
            mma_commit(&a_empty[0]);
        }
        __syncwarp();
    } else if (warp == kDLoaderWarp && TMA) {
        // ---- loader (TMA): tile i's 128 coefficients as one 2-D tile -> ring slot i % kDRing; rows
        // past the item's end belong to the next item and only feed visibilities never stored
        if (lane == 0) {
            int issued = 0;
            for (int i = 0; i < ntiles; i++) {
                const int slot = i % kDRing;
                const uint32_t ph = (i / kDRing) & 1;
                if (!mbar_wait(&in_empty[slot], ph ^ 1, abort_flag, a.wait_ns)) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                    break;
                }
                if (i == a.debug_skip_stage) {  // fault injection: this tile never arrives
                    issued = i + 1;
                    continue;
                }
                mbar_expect_tx(&in_full[slot], kDTile * 16);
                tma_load_2d(rbase + slot * kDRingSlot, &maps.coef, 0, static_cast<int32_t>(c0 + i * kDTile),
                            &in_full[slot]);
                issued = i + 1;
            }
            volatile int never = 0;
            for (int i = issued > kDRing ? issued - kDRing : 0; i < issued; i++)
                if (!mbar_wait(&in_full[i % kDRing], (i / kDRing) & 1, &never, a.wait_ns)) atomicOr(a.status, kStatusWait);
        }
        __syncwarp();
    } else if (warp == kDLoaderWarp) {
        // ---- loader: tile i's 128 coefficients -> ring slot i % kDRing
        for (int i = 0; i < ntiles; i++) {
            const int slot = i % kDRing;
            const uint32_t ph = (i / kDRing) & 1;
            if (!warp_wait(&in_empty[slot], ph ^ 1, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            if (i == a.debug_skip_stage) continue;  // fault injection: this tile never arrives
            const uint32_t dst = rbase + slot * kDRingSlot;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int row = lane + 32 * u, j = i * kDTile + row;
                const bool in = j < nvis;
                cp_async_16(dst + row * 16, in ? crow + j : crow, in ? 16u : 0u);
            }
            cp_async_arrive(&in_full[slot]);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else if (warp < 4) {
        // ---- producers: A tile, hi and lo.  Thread t writes the 16-byte chunks cc = t + 128 u
        // (u < 8): rows 8 (2u + t/64) + t%8 = row0 + 16 u, one fixed group of 4 x values.
        const int kg = (threadIdx.x >> 3) & 7;
        const int row0 = (threadIdx.x >> 6) * 8 + (threadIdx.x & 7);
        float2 lx[2], fx[2];  // l_x and f_x of the thread's 4 x values, in pairs
#pragma unroll
        for (int v = 0; v < 2; v++) {
            lx[v] = make_float2(tab_m[kg * 4 + 2 * v], tab_m[kg * 4 + 2 * v + 1]);
            fx[v] = make_float2(tab_g[kg * 4 + 2 * v], tab_g[kg * 4 + 2 * v + 1]);
        }
        for (int i = 0; i < ntiles; i++) {
            const int b = i & 1, slot = i % kDRing;
            const uint32_t ph = (i >> 1) & 1, iph = (i / kDRing) & 1;
            if (!warp_wait(&in_full[slot], iph, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            float2 cu[8];  // (du, dw) of this thread's 8 rows
            {
                const float4 *rc = reinterpret_cast<const float4 *>(ring + slot * kDRingSlot);
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const float4 c = rc[row0 + 16 * u];
                    cu[u] = make_float2(c.x, c.z);
                }
            }
            // the slot is released once cu has been used (below), not right after the loads
            if (!warp_wait(&a_empty[b], ph ^ 1, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            const uint32_t ahi = ts + b * kDTileBytes, alo = ahi + kDTileHalf;
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int cc = threadIdx.x + 128 * u;
                uint32_t whi[4], wlo[4];
                const float2 cx = make_float2(cu[u].x, cu[u].x), cz = make_float2(cu[u].y, cu[u].y);
#pragma unroll
                for (int v = 0; v < 2; v++) {
                    const float2 ph = __ffma2_rn(cx, lx[v], __fmul2_rn(cz, fx[v]));
                    float sa, ca;
                    __sincosf(ph.x, &sa, &ca);
                    split_pair<BF16, !BF16>(ca, sa, whi[2 * v], wlo[2 * v]);
                    __sincosf(ph.y, &sa, &ca);
                    split_pair<BF16, !BF16>(ca, sa, whi[2 * v + 1], wlo[2 * v + 1]);
                }
                st_shared_v4(ahi + cc * 16, whi[0], whi[1], whi[2], whi[3]);
                st_shared_v4(alo + cc * 16, wlo[0], wlo[1], wlo[2], wlo[3]);
            }
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&a_full[b]);
                mbar_arrive(&in_empty[slot]);
            }
        }
    } else {
        // ---- epilogue: one visibility per thread
        const int q = warp & 3;
        OutT *out = static_cast<OutT *>(a.vis_out) + (static_cast<int64_t>(sg.bl) * g.nt_all + it.t0) * g.nch;
        for (int i = 0; i < ntiles; i++) {
            const int b = i % NB, slot = i % kDRing;
            const uint32_t ph = (i / NB) & 1, iph = (i / kDRing) & 1;
            const int row = q * 32 + lane, j = i * kDTile + row;
            if (!warp_wait(&in_full[slot], iph, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            const float4 c = reinterpret_cast<const float4 *>(ring + slot * kDRingSlot)[row];
            // the slot is released once c has been used (below), not right after the load
            if (!warp_wait(&acc_full[b], ph, abort_flag, a.wait_ns)) {
                if (lane == 0) {
                    *abort_flag = 1;
                    atomicOr(a.status, kStatusWait);
                }
                break;
            }
            tc_fence_after();
            const float dwe = BF16 ? c.z : c.z / a.r_scale;  // T1 was formed from r * r_scale
            const uint32_t acc = tmem + (static_cast<uint32_t>(32 * q) << 16) + static_cast<uint32_t>(b * 128);
            // accumulator columns come in groups of four: (re y, re y+1, im y, im y+1), so rows y and
            // y + 1 are handled side by side in packed FP32x2 arithmetic; vis = sum over y of
            // conj(B) z = (a1 + a2) + i (a3 - a4), both halves of each pair summed at the end
            const float2 cy = make_float2(c.y, c.y), cz = make_float2(c.z, c.z);
            const float2 dw = make_float2(dwe, dwe), ndw = make_float2(-dwe, -dwe);
            float2 a1 = make_float2(0.f, 0.f), a2 = a1, a3 = a1, a4 = a1;
            auto row_pair = [&](int y0, float2 zre, float2 zim) {
                const float2 my = BATCH ? make_float2(tab_m[y0], tab_m[y0 + 1]) : make_float2(L.m_tab[y0], L.m_tab[y0 + 1]);
                const float2 gy = BATCH ? make_float2(tab_g[y0], tab_g[y0 + 1]) : make_float2(L.g_tab[y0], L.g_tab[y0 + 1]);
                const float2 ph = __ffma2_rn(cy, my, __fmul2_rn(cz, gy));
                float2 sb, cb;
                __sincosf(ph.x, &sb.x, &cb.x);
                __sincosf(ph.y, &sb.y, &cb.y);
                a1 = __ffma2_rn(cb, zre, a1);
                a2 = __ffma2_rn(sb, zim, a2);
                a3 = __ffma2_rn(cb, zim, a3);
                a4 = __ffma2_rn(sb, zre, a4);
            };
            auto pair = [](const uint32_t *t, int i) { return make_float2(__uint_as_float(t[i]), __uint_as_float(t[i + 1])); };
            if (O2) {
                // z = T0 - i dw T1 - (dw^2 / 2) T2, 8 rows (16 columns) of each block at a time
                const float hd2 = 0.5f * dwe * dwe;  // T2 was formed from r^2 * r_scale^2
                const float2 nhd2 = make_float2(-hd2, -hd2);
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    uint32_t t0[16], t1[16], t2[16];
                    tmem_ld16(acc + h * 16, t0);
                    tmem_ld16(acc + 64 + h * 16, t1);
                    tmem_ld16(acc + 128 + h * 16, t2);
                    tmem_ld_wait(t0);
                    tmem_ld_wait(t1);
                    tmem_ld_wait(t2);
#pragma unroll
                    for (int yq = 0; yq < 4; yq++) {
                        const float2 zre = __ffma2_rn(nhd2, pair(t2, 4 * yq), __ffma2_rn(dw, pair(t1, 4 * yq + 2), pair(t0, 4 * yq)));
                        const float2 zim = __ffma2_rn(nhd2, pair(t2, 4 * yq + 2), __ffma2_rn(ndw, pair(t1, 4 * yq), pair(t0, 4 * yq + 2)));
                        row_pair(h * 8 + 2 * yq, zre, zim);
                    }
                }
            }
#pragma unroll
            for (int h = 0; h < (O2 ? 0 : 4); h++) {
                uint32_t t0[16], t1[16];
                tmem_ld16(acc + h * 16, t0);
                tmem_ld16(acc + 64 + h * 16, t1);
                tmem_ld_wait(t0);
                tmem_ld_wait(t1);
#pragma unroll
                for (int yq = 0; yq < 4; yq++) {
                    // z = T0 - i dw T1 (single-plan launches: the tables are kernel parameters)
                    const float2 zre = __ffma2_rn(dw, pair(t1, 4 * yq + 2), pair(t0, 4 * yq));
                    const float2 zim = __ffma2_rn(ndw, pair(t1, 4 * yq), pair(t0, 4 * yq + 2));
                    row_pair(h * 8 + 2 * yq, zre, zim);
                }
            }
            const float vre_s = (a1.x + a1.y) + (a2.x + a2.y), vim_s = (a3.x + a3.y) - (a4.x + a4.y);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&acc_empty[b]);
                mbar_arrive(&in_empty[slot]);
            }
            if (j < nvis) {
                const float sc = g.inv_s2 / sq;  // exact: sq is a power of two
                store_vis(out, j, make_float2(vre_s * sc, vim_s * sc));
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == kDMmaWarp) {
        // wait (bounded) for the drain commit: all MMAs of this CTA are complete.  The phase count
        // is what was issued (fewer tiles after an abort), and the wait does not stop early on an
        // abort: the TMEM may only be released once no MMA is in flight.
        if (lane == 0) {
            volatile int never = 0;
            if (!mbar_wait(&a_empty[0], static_cast<uint32_t>(drain_phase & 1), &never, a.wait_ns))
                atomicOr(a.status, kStatusWait);
        }
        __syncwarp();
        tc_fence_after();
        tmem_dealloc(tmem, kDTmemCols);
    }
    if (BATCH && threadIdx.x == 0) note_item_done(a.done, a.finish_ns);  // every visibility store is done
}

// ---------------- self-test GEMM: C[128][N] = A[128][64] . B[N][64]^T ----------------

template <bool BF16, bool MN>
__global__ void __launch_bounds__(128) tc_selftest_kernel(const float *A, const float *B, int N, float *C,
                                                          int32_t *status) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *smem = smem_1k(smem_raw);
    unsigned char *sa = smem, *sb = smem + 128 * 128;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sb + 128 * 128);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_slot, 128);
        tmem_relinquish();
    }
    // operands: K-major, each 16-byte chunk (row, kg) holds 8 consecutive k of one row; MN-major,
    // each 16-byte chunk (row group g, k) at g * 1024 + 16 k holds 8 consecutive rows of one k
    for (int cc = threadIdx.x; cc < 128 * 8; cc += 128) {
        uint32_t w[4];
        if (MN) {
            const int g = cc >> 6, k = cc & 63;
            for (int u = 0; u < 4; u++)
                w[u] = Half16<BF16>::pack(A[(8 * g + 2 * u) * 64 + k], A[(8 * g + 2 * u + 1) * 64 + k]);
            st_shared_v4(smem_u32(sa) + cc * 16, w[0], w[1], w[2], w[3]);
            if (8 * g < N) {
                for (int u = 0; u < 4; u++)
                    w[u] = Half16<BF16>::pack(B[(8 * g + 2 * u) * 64 + k], B[(8 * g + 2 * u + 1) * 64 + k]);
                st_shared_v4(smem_u32(sb) + cc * 16, w[0], w[1], w[2], w[3]);
            }
            continue;
        }
        const int row = (cc >> 6) * 8 + (cc & 7), kg = (cc >> 3) & 7;
        for (int u = 0; u < 4; u++)
            w[u] = Half16<BF16>::pack(A[row * 64 + kg * 8 + 2 * u], A[row * 64 + kg * 8 + 2 * u + 1]);
        st_shared_v4(smem_u32(sa) + cc * 16, w[0], w[1], w[2], w[3]);
        if (row < N) {
            for (int u = 0; u < 4; u++)
                w[u] = Half16<BF16>::pack(B[row * 64 + kg * 8 + 2 * u], B[row * 64 + kg * 8 + 2 * u + 1]);
            st_shared_v4(smem_u32(sb) + cc * 16, w[0], w[1], w[2], w[3]);
        }
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (threadIdx.x == 0) {
        const uint32_t idesc = idesc_f16(128, N, BF16, MN);
        for (int kc = 0; kc < 4; kc++)
            mma_f16(tmem, smem_desc(smem_u32(sa) + kc * 256, 128, 1024), smem_desc(smem_u32(sb) + kc * 256, 128, 1024),
                    idesc, kc > 0 ? 1u : 0u);
        mma_commit(bar);
    }
    __syncwarp();
    const bool ok = warp_wait(bar, 0, abort_flag, kWaitNs);
    if (!ok && lane == 0) atomicOr(status, kStatusWait);
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 32) {
            uint32_t r[32];
            tmem_ld32(tmem + (static_cast<uint32_t>(32 * warp) << 16) + c0, r);
            tmem_ld_wait(r);
            for (int j = 0; j < 32; j++) C[(32 * warp + lane) * N + c0 + j] = __uint_as_float(r[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
}

template <typename K>
cudaError_t set_smem(K kernel, uint32_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

std::atomic<uint64_t> g_wait_ns{kWaitNs};
std::atomic<int32_t> g_skip_stage{-1};

void fill_args(TcArgs &t, const GridderArgs &a, const TcPlanState &st) {
    t.wait_ns = g_wait_ns.load();
    t.debug_skip_stage = g_skip_stage.load();
    t.g = a.g;
    t.subs = a.subs;
    t.coef_off = static_cast<const int64_t *>(st.coef_off);
    t.coef = static_cast<const float4 *>(st.coef);
    t.lmn = a.lmn;
    t.tabs = static_cast<const float *>(st.tables);
    t.taper = a.taper;
    t.dw_scale = st.dw_scale;
    t.r_scale = st.r_scale;
    for (int i = 0; i < kS; i++) {
        t.m_tab[i] = st.m_tab[i];
        t.g_tab[i] = st.g_tab[i];
    }
}

}  // namespace

// S < 32 runs padded to 32 operand rows (the per-visibility cost of S = 32)
bool tc_subgrid_size_supported(int S) { return S == 8 || S == 16 || S == 24 || S == 32; }

int tc_order_for(double w_term, int want_order) {
    if (want_order != 2 && w_term <= P9IDG_TC_MAX_W_TERM) return 1;
    if (w_term <= P9IDG_TC_MAX_W_TERM2) return 2;
    return 0;
}

void tc_set_order(TcPlanState &st, int want_order) {
    st.want_order = want_order;
    st.order = tc_order_for(st.max_w_r, want_order);
    const double limit = st.order == 1 ? P9IDG_TC_MAX_W_TERM : P9IDG_TC_MAX_W_TERM2;
    st.dw_limit = st.r_max > 0 ? limit / st.r_max : INFINITY;
}

void tc_debug_set(uint64_t wait_ns, int32_t skip_stage) {
    g_wait_ns.store(wait_ns > 0 ? wait_ns : kWaitNs);
    g_skip_stage.store(skip_stage);
}

namespace {

// The separable part f (serving as f(x) and g(y)) and the remainder r of the reference's FP32 n
// table (Gridder.cs:168-174 values in lmn[S..]): f(x) = n(l_x, 0) + c/2 and r = n - f(x) - f(y),
// where the constant c centres the range of r on zero; with l (lmn[0..S)) they make the kTabs-float
// table the kernels read, padded with zeros past S.  Returns max |r| over the S x S pixels.
double separable_tables(const std::vector<float> &lmn, int S, std::vector<float> &tabs) {
    tabs.assign(kTabs, 0.f);
    std::vector<double> f0(S);
    for (int x = 0; x < S; x++) {
        const double l = lmn[x], t = l * l;
        f0[x] = t / (t + std::sqrt(1.0 - t));
        tabs[kTabL + x] = lmn[x];
    }
    double rlo = INFINITY, rhi = -INFINITY;
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) {
            const double r = static_cast<double>(lmn[S + y * S + x]) - static_cast<float>(f0[x]) -
                             static_cast<float>(f0[y]);
            rlo = std::min(rlo, r);
            rhi = std::max(rhi, r);
        }
    const double c = 0.5 * (rlo + rhi);
    for (int x = 0; x < S; x++) tabs[x] = static_cast<float>(f0[x] + 0.5 * c);
    double rmax = 0;
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) {
            const double r = static_cast<double>(lmn[S + y * S + x]) - tabs[x] - tabs[y];
            tabs[kTabR + y * kS + x] = static_cast<float>(r);
            rmax = std::max(rmax, std::fabs(r));
        }
    return rmax;
}

// max |w| over the gridded samples and max |k| over the channels
void w_k_max(const std::vector<p9idg_subgrid> &subs, const std::vector<double> &wn, const double *uvw_host,
             int nt_all, double &wmax, double &kmax) {
    wmax = 0;
    kmax = 0;
    for (double k : wn) kmax = std::max(kmax, std::fabs(k));
    for (const auto &sg : subs)
        for (int t = 0; t < sg.time_sample_count; t++) {
            const double w = uvw_host[(static_cast<int64_t>(sg.baseline_idx) * nt_all + sg.time_sample_start + t) * 3 + 2];
            wmax = std::max(wmax, std::fabs(w));
        }
}

}  // namespace

double tc_w_term(const std::vector<p9idg_subgrid> &subs, const std::vector<float> &lmn, int S,
                 const std::vector<double> &wn, const double *uvw_host, int nt_all) {
    if (!tc_subgrid_size_supported(S)) return INFINITY;
    std::vector<float> tabs;
    const double rmax = separable_tables(lmn, S, tabs);
    double wmax, kmax;
    w_k_max(subs, wn, uvw_host, nt_all, wmax, kmax);
    return wmax * kmax * rmax;
}

p9idg_status tc_prepare(TcPlanState &st, const std::vector<p9idg_subgrid> &subs, const std::vector<float> &lmn,
                        int S, int nch, const std::vector<double> &wn, const double *uvw_host, int nt_all,
                        cudaStream_t stream, std::string &err) {
    if (st.ready) return P9IDG_OK;
    if (!tc_subgrid_size_supported(S)) {
        err = "tensor-core kernels support subgrid sizes 8, 16, 24 and 32";
        return P9IDG_UNSUPPORTED;
    }
    std::vector<float> tabs;
    const double rmax = separable_tables(lmn, S, tabs);
    // coefficient offsets per subgrid and the largest |dw|
    std::vector<int64_t> off(subs.size() + 1, 0);
    for (size_t i = 0; i < subs.size(); i++)
        off[i + 1] = off[i] + static_cast<int64_t>(subs[i].time_sample_count) * nch;
    double wmax, kmax;
    w_k_max(subs, wn, uvw_host, nt_all, wmax, kmax);
    st.max_w_r = wmax * kmax * rmax;
    st.r_max = rmax;
    tc_set_order(st, st.want_order);
    for (int i = 0; i < kS; i++) {
        st.m_tab[i] = tabs[kTabL + i];
        st.g_tab[i] = tabs[i];
    }
    // powers of two keeping dw * B and r * pix inside the FP16 range (|woff| = 0, so |dw| <= k |w|)
    auto pow2_below = [](double m) {
        if (!(m > 0) || !std::isfinite(m)) return 1.f;
        int e;
        std::frexp(m, &e);
        return static_cast<float>(std::ldexp(1.0, -e));
    };
    st.dw_scale = pow2_below(wmax * kmax * 1.0001);
    st.r_scale = pow2_below(rmax);
    if (st.order == 0) {
        err = "w term too large for the separable tensor-core forms (|dw r| = " + std::to_string(st.max_w_r) +
              " > " + std::to_string(P9IDG_TC_MAX_W_TERM2) + ")";
        return P9IDG_UNSUPPORTED;
    }
    // degridder work items: whole time samples, up to degrid_chunk visibilities each
    std::vector<DevSubgrid> dtmp;
    std::vector<WorkItem> ditems;
    build_work_items(subs, nch, st.degrid_chunk, dtmp, ditems);
    st.ncoef = off.back();
    cudaError_t e;
    if ((e = device_alloc(&st.coef, sizeof(float4) * std::max<int64_t>(1, st.ncoef))) != cudaSuccess ||
        (e = device_alloc(&st.coef_off, sizeof(int64_t) * off.size())) != cudaSuccess ||
        (e = device_alloc(&st.tables, sizeof(float) * tabs.size())) != cudaSuccess ||
        (e = device_alloc(&st.ditems, sizeof(WorkItem) * std::max<size_t>(1, ditems.size()))) != cudaSuccess) {
        err = std::string("tensor-core buffers: ") + cudaGetErrorString(e);
        tc_release(st);
        return e == cudaErrorMemoryAllocation ? P9IDG_OUT_OF_MEMORY : P9IDG_CUDA_ERROR;
    }
    cudaMemcpyAsync(st.coef_off, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, stream);
    cudaMemcpyAsync(st.tables, tabs.data(), sizeof(float) * tabs.size(), cudaMemcpyHostToDevice, stream);
    if (!ditems.empty())
        cudaMemcpyAsync(st.ditems, ditems.data(), sizeof(WorkItem) * ditems.size(), cudaMemcpyHostToDevice, stream);
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) {
        err = std::string("tensor-core tables: ") + cudaGetErrorString(e);
        return P9IDG_CUDA_ERROR;
    }
    st.nditems = static_cast<int32_t>(ditems.size());
    st.ditems_host = ditems;
    st.S = S;
    st.ready = true;
    return P9IDG_OK;
}

// Per-visibility phase coefficients depend only on the plan and uvw: computed once and kept
// until uvw is uploaded again (the plan clears coef_valid then; when it compared the new upload
// with the previous one on the device, the kernel recomputes only if they differ).
static p9idg_status launch_coef(TcPlanState &st, const GridderArgs &a, int32_t nsub, cudaStream_t stream,
                                std::string &err) {
    if (nsub == 0 || st.coef_valid) return P9IDG_OK;
    tc_coef_kernel<<<nsub, 256, 0, stream>>>(a.subs, static_cast<const int64_t *>(st.coef_off), a.uvw, a.wavenumbers,
                                             a.g, static_cast<float4 *>(st.coef), st.coef_recompute_flag,
                                             st.dw_limit, a.status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("coefficient kernel: ") + cudaGetErrorString(e);
        return P9IDG_CUDA_ERROR;
    }
    st.coef_valid = true;
    st.coef_recompute_flag = nullptr;
    return P9IDG_OK;
}

namespace {

template <bool BF16, typename VisT, bool BATCH, bool TMA, bool O2>
cudaError_t run_gridder(const TcArgs &t, const TcArgs *probs, int32_t nitems, const TmaMaps &maps,
                        cudaStream_t stream) {
    cudaError_t e = set_smem(tc_gridder_kernel<BF16, VisT, BATCH, TMA, O2>, g_smem(O2));
    if (e == cudaSuccess)
        tc_gridder_kernel<BF16, VisT, BATCH, TMA, O2><<<nitems, kGThreads, g_smem(O2), stream>>>(t, probs, maps);
    return e;
}

template <bool BF16, typename OutT, bool BATCH, bool TMA, bool O2>
cudaError_t run_degridder(const TcArgs &t, const TcArgs *probs, int32_t nitems, const TmaMaps &maps,
                          cudaStream_t stream) {
    constexpr uint32_t smem = O2 ? kDSmem2 : kDSmem;
    cudaError_t e = set_smem(tc_degridder_kernel<BF16, OutT, BATCH, TMA, O2>, smem);
    if (e == cudaSuccess)
        tc_degridder_kernel<BF16, OutT, BATCH, TMA, O2><<<nitems, kDThreads, smem, stream>>>(t, probs, maps);
    return e;
}

// maps: TMA staging for a single-plan launch (nullptr: cp.async staging).  Batched launches read
// per-problem buffers and always use cp.async.
template <bool BATCH, bool O2>
p9idg_status launch_tc_gridder(const TcArgs &t, const TcArgs *probs, int32_t nitems, bool c128, int mode,
                               const TmaMaps *maps, cudaStream_t stream, std::string &err) {
    if (nitems == 0) return P9IDG_OK;
    static const TmaMaps kNoMaps{};
    const bool bf16 = mode == P9IDG_MODE_TC_BF16X3;
    const TmaMaps &m = maps ? *maps : kNoMaps;
    cudaError_t e = cudaSuccess;
    bool done = false;
    if constexpr (!BATCH) {
        if (maps && !c128) {
            e = bf16 ? run_gridder<true, float2, false, true, O2>(t, probs, nitems, m, stream)
                     : run_gridder<false, float2, false, true, O2>(t, probs, nitems, m, stream);
            done = true;
        }
    }
    if (!done) {
        if (bf16 && c128)
            e = run_gridder<true, double2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else if (bf16)
            e = run_gridder<true, float2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else if (c128)
            e = run_gridder<false, double2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else
            e = run_gridder<false, float2, BATCH, false, O2>(t, probs, nitems, m, stream);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("tensor-core gridder: ") + cudaGetErrorString(e);
        return P9IDG_CUDA_ERROR;
    }
    return P9IDG_OK;
}

template <bool BATCH, bool O2>
p9idg_status launch_tc_degridder(const TcArgs &t, const TcArgs *probs, int32_t nitems, bool c128, int mode,
                                 const TmaMaps *maps, cudaStream_t stream, std::string &err) {
    if (nitems == 0) return P9IDG_OK;
    static const TmaMaps kNoMaps{};
    const bool bf16 = mode == P9IDG_MODE_TC_BF16X3;
    const TmaMaps &m = maps ? *maps : kNoMaps;
    cudaError_t e = cudaSuccess;
    bool done = false;
    if constexpr (!BATCH) {
        if (maps) {
            if (bf16 && c128)
                e = run_degridder<true, double2, false, true, O2>(t, probs, nitems, m, stream);
            else if (bf16)
                e = run_degridder<true, float2, false, true, O2>(t, probs, nitems, m, stream);
            else if (c128)
                e = run_degridder<false, double2, false, true, O2>(t, probs, nitems, m, stream);
            else
                e = run_degridder<false, float2, false, true, O2>(t, probs, nitems, m, stream);
            done = true;
        }
    }
    if (!done) {
        if (bf16 && c128)
            e = run_degridder<true, double2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else if (bf16)
            e = run_degridder<true, float2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else if (c128)
            e = run_degridder<false, double2, BATCH, false, O2>(t, probs, nitems, m, stream);
        else
            e = run_degridder<false, float2, BATCH, false, O2>(t, probs, nitems, m, stream);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("tensor-core degridder: ") + cudaGetErrorString(e);
        return P9IDG_CUDA_ERROR;
    }
    return P9IDG_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to the driver library).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return static_cast<EncodeTiledFn>(nullptr);
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// Tensor maps over the coefficients (tiles of box_rows float4 rows) and, when vis is given,
// over nvis complex64 visibilities; false (use cp.async) when a map cannot be made.
bool make_maps(TmaMaps &m, const float4 *coef, int64_t ncoef, int box_rows, const void *vis, int64_t nvis) {
    const EncodeTiledFn fn = encode_tiled();
    constexpr int64_t kMaxCoord = (int64_t(1) << 31) - 1024;  // TMA coordinates are signed 32-bit
    if (!fn || !coef || ncoef <= 0 || ncoef > kMaxCoord || (reinterpret_cast<uintptr_t>(coef) & 15)) return false;
    const cuuint64_t cdim[2] = {4, static_cast<cuuint64_t>(ncoef)};
    const cuuint64_t cstride[1] = {16};
    const cuuint32_t cbox[2] = {4, static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t ones[2] = {1, 1};
    if (fn(&m.coef, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float4 *>(coef), cdim, cstride, cbox, ones,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    if (vis) {
        if (nvis <= 0 || nvis > kMaxCoord || (reinterpret_cast<uintptr_t>(vis) & 15)) return false;
        const cuuint64_t vdim[1] = {static_cast<cuuint64_t>(nvis)};
        const cuuint64_t vstride[1] = {8};
        const cuuint32_t vbox[1] = {kVisBox};
        if (fn(&m.vis, CU_TENSOR_MAP_DATA_TYPE_UINT64, 1, const_cast<void *>(vis), vdim, vstride, vbox, ones,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

}  // namespace

void tc_fill_args(const TcPlanState &st, const GridderArgs &a, TcArgs &t) {
    fill_args(t, a, st);
    t.items = a.items;
    t.vis = a.vis;
    t.partials = a.partials;
    t.subgrids = a.subgrids;
    t.vis_out = a.vis_out;
    t.status = a.status;
    t.done = a.done;
    t.finish_ns = a.finish_ns;
}

p9idg_status tc_coefs(TcPlanState &st, const GridderArgs &a, cudaStream_t stream, std::string &err) {
    if (!st.ready) {
        err = "tensor-core state not prepared";
        return P9IDG_INVALID_ARGUMENT;
    }
    return launch_coef(st, a, a.nsub, stream, err);
}

p9idg_status tc_grid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err) {
    p9idg_status s = tc_coefs(st, a, stream, err);
    if (s != P9IDG_OK) return s;
    TcArgs t{};
    tc_fill_args(st, a, t);
    TmaMaps maps;
    const int64_t nvis = static_cast<int64_t>(a.g.nbl) * a.g.nt_all * a.g.nch;
    const bool tma =
        !a.vis_c128 && make_maps(maps, static_cast<const float4 *>(st.coef), st.ncoef, kGVps, a.vis, nvis);
    return st.order == 2 ? launch_tc_gridder<false, true>(t, nullptr, a.nitems, a.vis_c128, mode, tma ? &maps : nullptr,
                                                          stream, err)
                         : launch_tc_gridder<false, false>(t, nullptr, a.nitems, a.vis_c128, mode,
                                                           tma ? &maps : nullptr, stream, err);
}

p9idg_status tc_degrid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err) {
    p9idg_status s = tc_coefs(st, a, stream, err);
    if (s != P9IDG_OK) return s;
    TcArgs t{};
    tc_fill_args(st, a, t);
    t.items = static_cast<const WorkItem *>(st.ditems);
    TmaMaps maps;
    const bool tma = make_maps(maps, static_cast<const float4 *>(st.coef), st.ncoef, kDTile, nullptr, 0);
    return st.order == 2 ? launch_tc_degridder<false, true>(t, nullptr, st.nditems, a.out_c128, mode,
                                                            tma ? &maps : nullptr, stream, err)
                         : launch_tc_degridder<false, false>(t, nullptr, st.nditems, a.out_c128, mode,
                                                             tma ? &maps : nullptr, stream, err);
}

p9idg_status tc_grid_batch(const TcArgs *probs, const WorkItem *items, int32_t nitems, int mode, int order,
                           cudaStream_t stream, std::string &err) {
    TcArgs t{};
    t.items = items;
    return order == 2 ? launch_tc_gridder<true, true>(t, probs, nitems, false, mode, nullptr, stream, err)
                      : launch_tc_gridder<true, false>(t, probs, nitems, false, mode, nullptr, stream, err);
}

p9idg_status tc_degrid_batch(const TcArgs *probs, const WorkItem *items, int32_t nitems, int mode, int order,
                             cudaStream_t stream, std::string &err) {
    TcArgs t{};
    t.items = items;
    return order == 2 ? launch_tc_degridder<true, true>(t, probs, nitems, false, mode, nullptr, stream, err)
                      : launch_tc_degridder<true, false>(t, probs, nitems, false, mode, nullptr, stream, err);
}

void tc_release(TcPlanState &st) {
    if (st.coef) cudaFree(st.coef);
    if (st.coef_off) cudaFree(st.coef_off);
    if (st.tables) cudaFree(st.tables);
    if (st.ditems) cudaFree(st.ditems);
    st = TcPlanState();
}

p9idg_status tc_selftest(int mode, int N, double *max_rel_err, std::string &err) {
    if (N != 32 && N != 64 && N != 128) {
        err = "self-test N must be 32, 64 or 128";
        return P9IDG_INVALID_ARGUMENT;
    }
    std::vector<float> A(128 * 64), B(128 * 64);
    uint32_t seed = 12345;
    auto rnd = [&]() {
        seed = seed * 1664525u + 1013904223u;
        return static_cast<float>((seed >> 8) & 0xFFFF) / 65536.0f - 0.5f;
    };
    for (auto &v : A) v = rnd();
    for (auto &v : B) v = rnd();
    // operands exactly representable in 16 bits so the product is exact up to FP32 accumulation
    const bool bf16 = mode == P9IDG_MODE_TC_BF16X3;
    for (auto *v : {&A, &B})
        for (auto &x : *v) {
            uint32_t u;
            std::memcpy(&u, &x, 4);
            u &= bf16 ? 0xFFFF0000u : 0xFFFFE000u;
            std::memcpy(&x, &u, 4);
        }
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int32_t *dS = nullptr;
    cudaError_t e = cudaMalloc(&dA, A.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dB, B.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dC, 128 * N * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dS, 4);
    if (e == cudaSuccess) e = cudaMemcpy(dA, A.data(), A.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B.data(), B.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dS, 0, 4);
    const uint32_t smem = 2 * 128 * 128 + 64 + 1024;
    std::vector<float> C(128 * N), C2(128 * N);
    for (int layout = 0; layout < 2 && e == cudaSuccess; layout++) {  // K-major, then MN-major operands
        auto run = [&](auto kernel) {
            cudaError_t r = set_smem(kernel, smem);
            if (r == cudaSuccess) kernel<<<1, 128, smem>>>(dA, dB, N, dC, dS);
            return r;
        };
        if (bf16)
            e = layout ? run(tc_selftest_kernel<true, true>) : run(tc_selftest_kernel<true, false>);
        else
            e = layout ? run(tc_selftest_kernel<false, true>) : run(tc_selftest_kernel<false, false>);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(layout ? C2.data() : C.data(), dC, C.size() * 4, cudaMemcpyDeviceToHost);
    }
    int32_t status = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&status, dS, 4, cudaMemcpyDeviceToHost);
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    cudaFree(dS);
    if (e != cudaSuccess) {
        err = std::string("self-test: ") + cudaGetErrorString(e);
        return P9IDG_CUDA_ERROR;
    }
    if (status != 0) {
        err = "self-test: a wait timed out";
        return P9IDG_DEVICE_CHECK_FAILED;
    }
    double maxerr = 0, maxref = 0;
    for (int i = 0; i < 128; i++)
        for (int j = 0; j < N; j++) {
            double ref = 0;
            for (int k = 0; k < 64; k++) ref += static_cast<double>(A[i * 64 + k]) * B[j * 64 + k];
            maxerr = std::max(maxerr, std::max(std::fabs(ref - C[i * N + j]), std::fabs(ref - C2[i * N + j])));
            maxref = std::max(maxref, std::fabs(ref));
        }
    *max_rel_err = maxerr / std::max(maxref, 1e-30);
    return P9IDG_OK;
}

}  // namespace p9idg
