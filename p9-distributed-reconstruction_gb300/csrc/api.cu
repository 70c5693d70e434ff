// C ABI of the GB300 gridder (include/p9idg.h): plans, device buffers, streams, cuFFT
// plans, stage timing, and the IDG / FFT entry points that replace
// Distributed-Reconstruction/Core/ImageDomainGridder/IDG.cs and Core/FFT.cs.
//
// A plan is created on the host only (partitioning needs no GPU); device state is
// created on the first call that needs it, on the device current at that time.

#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "tc_gridder.cuh"

using namespace p9idg;

namespace {

thread_local std::string g_last_error;

p9idg_status fail(p9idg_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

p9idg_status cuda_fail(cudaError_t e, const char *what) {
    const p9idg_status st = (e == cudaErrorMemoryAllocation) ? P9IDG_OUT_OF_MEMORY
                            : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? P9IDG_NO_DEVICE
                                                                                             : P9IDG_CUDA_ERROR;
    return fail(st, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(x)                                                   \
    do {                                                        \
        cudaError_t e_ = (x);                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #x);        \
    } while (0)

#define TRY(x)                                \
    do {                                      \
        p9idg_status s_ = (x);                \
        if (s_ != P9IDG_OK) return s_;        \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
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

struct FftCache {
    cufftHandle h = 0;
    int n = 0;
    cudaStream_t st = nullptr;
    p9idg_status get(int size, cudaStream_t stream, cufftHandle *out) {
        if (h && n != size) {
            cufftDestroy(h);
            h = 0;
        }
        if (!h) {
            if (cufftPlan2d(&h, size, size, CUFFT_C2C) != CUFFT_SUCCESS) {
                h = 0;
                return fail(P9IDG_CUDA_ERROR, "cufftPlan2d failed");
            }
            n = size;
            st = nullptr;
        }
        if (st != stream) {
            cufftSetStream(h, stream);
            st = stream;
        }
        *out = h;
        return P9IDG_OK;
    }
    void release() {
        if (h) cufftDestroy(h);
        h = 0;
        n = 0;
    }
};

struct PendingTiming {
    int stage;
    cudaEvent_t a, b;
};

}  // namespace

void p9idg::record_last_error(const std::string &msg) { g_last_error = msg; }

namespace {
// successful device allocations left before device_alloc fails (-1: never)
std::atomic<int64_t> g_alloc_budget{-1};
}  // namespace

cudaError_t p9idg::device_alloc(void **p, size_t bytes) {
    int64_t b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
    }
    return cudaMalloc(p, bytes);
}

extern "C" p9idg_status p9idg_debug_tc_wait(int64_t wait_ns, int32_t skip_stage) {
    if (wait_ns < 0) return fail(P9IDG_INVALID_ARGUMENT, "negative wait limit");
    tc_debug_set(static_cast<uint64_t>(wait_ns), skip_stage);
    return P9IDG_OK;
}

extern "C" p9idg_status p9idg_debug_fail_device_allocations(int64_t after) {
    g_alloc_budget.store(after < 0 ? -1 : after);
    return P9IDG_OK;
}

struct p9idg_plan {
    p9idg_params c{};
    int32_t nbl = 0, nt = 0, nch = 0;
    int32_t mode = P9IDG_MODE_FP32;
    int32_t requested_mode = P9IDG_MODE_FP32;
    double tc_w_term = -1;  // max |dw| * max |r| of the plan's samples, once a tensor-core mode was asked for
    std::vector<double> freq, wn, uvw;
    std::vector<p9idg_subgrid> subs;
    std::vector<DevSubgrid> dsub;
    std::vector<WorkItem> gitems, ditems;
    int32_t nslots = 0;
    bool items_dirty = true;  // gridder items / subgrid list not yet on the device
    int32_t gchunk = 0;       // gridder visibilities per work item (0 = per-mode default)
    int32_t dchunk = 0;       // degridder visibilities per work item (0 = per-mode default)
    int64_t gridded_vis = 0;
    std::vector<float> lmn, taper;
    std::vector<float> add_phasor;  // interleaved float2: [S][S] adder phasors, then S FFT twiddles
    bool taper_dirty = true;

    // device state
    bool dev_ready = false;
    int device = -1;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    bool uvw_uploaded = false;
    DevBuf d_uvw, d_wn, d_sub, d_gitems, d_ditems, d_lmn, d_taper, d_phasor, d_status;
    DevBuf d_partials, d_subgrids, d_vis_in, d_vis_out, d_layers, d_out128, d_grid128, d_grid128b, d_grid64,
        d_flags, d_image;
    TcPlanState tc;
    FftCache fft;
    // Host arrays used in place by the kernels (device reads/writes host memory through the host's
    // page tables, e.g. NVLink-C2C on Grace systems) instead of staged through device copies.
    bool host_direct = false;   // the device can access any host address
    int32_t host_access = 1;    // caller's choice: 1 = in place where possible, 0 = staged copies
    std::vector<int64_t> gaps;  // (start, count) ranges of visibilities no subgrid covers
    std::vector<char> layer_used;  // w layers some subgrid adds into
    bool gaps_ready = false;
    DevBuf d_gaps;
    cudaStream_t side = nullptr;  // the D2H copy of DeGrid's shifted grid runs here, beside the degridder
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_mid = nullptr;
    // Zero-fills beside the gridder and degridder (ZeroSide): a high-priority stream, so that its few
    // CTAs take the room the kernels leave on each SM instead of queueing behind their work items.
    cudaStream_t zside = nullptr;
    cudaEvent_t ev_zfork = nullptr, ev_zjoin = nullptr;
    // In-place GridW: the gridder items and the subgrids regrouped so that every w layer but the
    // busiest one is gridded and added first; those layers then cross the link while the busiest
    // one grids.  Items keep their partial-subgrid slots; built with the gridder items.
    std::vector<WorkItem> gitems_lyr;  // items of the other layers, then of the busiest layer
    std::vector<int32_t> sub_lyr;      // subgrid indices in the same grouping
    int32_t lyr_minor_items = 0, lyr_minor_subs = 0, lyr_major = -1;
    // The busiest layer's part in row bands (the rows the adder writes, before the output's
    // FFT.Shift), so that each band's rows cross the link while the next band grids: band b is
    // items [lyr_band_items[b], lyr_band_items[b + 1]) and subgrids [lyr_band_subs[b], ...) of
    // that part, and once it is added, rows [lyr_band_rows[b], lyr_band_rows[b + 1]) are final.
    std::vector<int32_t> lyr_band_items, lyr_band_subs, lyr_band_rows;
    bool lyr_ready = false;
    DevBuf d_gitems_lyr, d_sub_lyr, d_zero128;
    DevBuf d_uvw_prev, d_uvw_flag;  // the previous uvw upload and the "uvw differs" flag

    bool timing = false;
    std::vector<PendingTiming> pending;
    std::vector<cudaEvent_t> event_pool;
    double stage_ms[P9IDG_NUM_STAGES] = {0};
    int64_t stage_launches[P9IDG_NUM_STAGES] = {0};

    Geometry geom() const {
        Geometry g;
        g.N = c.grid_size;
        g.S = c.subgrid_size;
        g.W = c.wlayer_count;
        g.nch = nch;
        g.nt_all = nt;
        g.nbl = nbl;
        g.uv_scale = 2 * kPi / static_cast<double>(image_size(c));
        g.wstep_lambda = 0.0f;  // GriddingConstants.WStepLambda is never assigned
        g.inv_s2 = 1.0f / static_cast<float>(c.subgrid_size * c.subgrid_size);
        return g;
    }
};

namespace {

// ---------- timing ----------

cudaEvent_t take_event(p9idg_plan *p) {
    if (!p->event_pool.empty()) {
        cudaEvent_t e = p->event_pool.back();
        p->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

struct StageScope {
    p9idg_plan *p;
    int stage;
    cudaEvent_t a = nullptr;
    StageScope(p9idg_plan *plan, int s) : p(plan), stage(s) {
        if (p->timing) {
            a = take_event(p);
            cudaEventRecord(a, p->stream);
        }
    }
    ~StageScope() {
        if (p->timing && a) {
            cudaEvent_t b = take_event(p);
            cudaEventRecord(b, p->stream);
            p->pending.push_back({stage, a, b});
        }
    }
};

void collect_timing(p9idg_plan *p) {
    for (auto &pt : p->pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(pt.b) == cudaSuccess && cudaEventElapsedTime(&ms, pt.a, pt.b) == cudaSuccess) {
            p->stage_ms[pt.stage] += ms;
            p->stage_launches[pt.stage] += 1;
        }
        p->event_pool.push_back(pt.a);
        p->event_pool.push_back(pt.b);
    }
    p->pending.clear();
}

// ---------- plan construction ----------

p9idg_status check_params(const p9idg_params *c) {
    if (!c) return fail(P9IDG_INVALID_ARGUMENT, "null params");
    if (c->grid_size <= 0 || c->subgrid_size <= 0 || c->subgrid_size > c->grid_size || c->wlayer_count < 0)
        return fail(P9IDG_INVALID_ARGUMENT, "invalid grid/subgrid/w-layer sizes");
    return P9IDG_OK;
}

// Gridder work items keep whole time samples: up to 1024 visibilities for the FP32 kernel,
// 4096 for the tensor-core kernel.  The tensor-core item is one FP32 accumulation in tensor
// memory, so its length sets the rounding error: 8192 measured 1 % faster at 3072² but raised
// the rel-L2 error against FP64 from 1.1e-5 to 2.6e-5.  The subgrid list records each
// subgrid's item slots for the subgrid IFFT + adder.
void build_gridder_items(p9idg_plan *p) {
    const int64_t chunk = p->gchunk > 0 ? p->gchunk : (p->mode == P9IDG_MODE_FP32 ? 1024 : 4096);
    build_work_items(p->subs, p->nch, chunk, p->dsub, p->gitems);
    // FP32 degridder items: 512 visibilities by default (4 per thread of a 128-thread block)
    std::vector<DevSubgrid> tmp;
    build_work_items(p->subs, p->nch, p->dchunk > 0 ? p->dchunk : 512, tmp, p->ditems);
    p->nslots = 0;
    for (const auto &d : p->dsub) p->nslots += d.item_count;
    p->items_dirty = true;
    p->lyr_ready = false;
}

void finish_plan(p9idg_plan *p) {
    const int S = p->c.subgrid_size;
    build_gridder_items(p);
    p->gridded_vis = 0;
    for (const auto &s : p->subs) p->gridded_vis += static_cast<int64_t>(s.time_sample_count) * p->nch;
    const float img = image_size(p->c);
    p->lmn.assign(S + S * S, 0.f);
    for (int x = 0; x < S; x++) p->lmn[x] = compute_l(x, S, img);
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) p->lmn[S + y * S + x] = compute_n(p->lmn[x], p->lmn[y]);
    p->taper.assign(S * S, 1.0f);  // CalcIdentitySpheroidal (MathFunctions.cs:69-78)
    p->add_phasor.assign(2 * S * S + 2 * S, 0.f);
    for (int y = 0; y < S; y++)
        for (int x = 0; x < S; x++) {
            const double ph = kPi * static_cast<double>(x + y - S) / static_cast<double>(S);  // Adder.cs:39
            p->add_phasor[2 * (y * S + x)] = static_cast<float>(std::cos(ph));
            p->add_phasor[2 * (y * S + x) + 1] = static_cast<float>(std::sin(ph));
        }
    for (int j = 0; j < S; j++) {  // subgrid FFT twiddles exp(+2 pi i j / S)
        const double ph = 2 * kPi * static_cast<double>(j) / static_cast<double>(S);
        p->add_phasor[2 * (S * S + j)] = static_cast<float>(std::cos(ph));
        p->add_phasor[2 * (S * S + j) + 1] = static_cast<float>(std::sin(ph));
    }
    p->wn.resize(p->nch);
    for (int i = 0; i < p->nch; i++) p->wn[i] = wavenumber(p->freq[i]);
}

// ---------- device state ----------

p9idg_status ensure_device(p9idg_plan *p) {
    if (p->dev_ready) {
        CK(cudaSetDevice(p->device));
        return P9IDG_OK;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(P9IDG_NO_DEVICE, "no CUDA device available");
    CK(cudaGetDevice(&p->device));
    // each object is made once: a call that failed part-way (e.g. out of memory) and is retried
    // continues from what exists
    if (!p->own_stream) CK(cudaStreamCreateWithFlags(&p->own_stream, cudaStreamNonBlocking));
    if (!p->stream) p->stream = p->own_stream;
    if (!p->side) CK(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
    if (!p->ev_fork) CK(cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming));
    if (!p->ev_join) CK(cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming));
    if (!p->ev_mid) CK(cudaEventCreateWithFlags(&p->ev_mid, cudaEventDisableTiming));
    if (!p->zside) {
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CK(cudaStreamCreateWithPriority(&p->zside, cudaStreamNonBlocking, greatest));
    }
    if (!p->ev_zfork) CK(cudaEventCreateWithFlags(&p->ev_zfork, cudaEventDisableTiming));
    if (!p->ev_zjoin) CK(cudaEventCreateWithFlags(&p->ev_zjoin, cudaEventDisableTiming));
    {
        int pageable = 0, host_tables = 0;
        CK(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, p->device));
        CK(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, p->device));
        p->host_direct = pageable != 0 && host_tables != 0;
    }
    const int S = p->c.subgrid_size;
    CK(p->d_wn.ensure(sizeof(double) * std::max(1, p->nch)));
    CK(p->d_lmn.ensure(sizeof(float) * p->lmn.size()));
    CK(p->d_taper.ensure(sizeof(float) * S * S));
    CK(p->d_phasor.ensure(sizeof(float) * p->add_phasor.size()));
    CK(p->d_status.ensure(sizeof(int32_t)));
    cudaStream_t st = p->stream;
    CK(cudaMemcpyAsync(p->d_wn.p, p->wn.data(), sizeof(double) * p->nch, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p->d_lmn.p, p->lmn.data(), sizeof(float) * p->lmn.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(p->d_phasor.p, p->add_phasor.data(), sizeof(float) * p->add_phasor.size(),
                       cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(p->d_status.p, 0, sizeof(int32_t), st));
    CK(cudaStreamSynchronize(st));
    p->taper_dirty = true;
    p->dev_ready = true;
    return P9IDG_OK;
}

p9idg_status upload_uvw(p9idg_plan *p, const double *uvw) {
    const size_t bytes = sizeof(double) * 3 * static_cast<size_t>(p->nbl) * p->nt;
    CK(p->d_uvw.ensure(bytes));
    if (uvw) {
        StageScope t(p, P9IDG_STAGE_H2D);
        if (p->tc.coef_valid) {
            // the tensor-core coefficients exist for the uvw now in d_uvw: the new upload goes to
            // the other buffer and is compared with it on the device, and the coefficient kernel
            // recomputes only if some word differs (no host synchronisation either way)
            std::swap(p->d_uvw, p->d_uvw_prev);
            CK(p->d_uvw.ensure(bytes));
            CK(p->d_uvw_flag.ensure(sizeof(int32_t)));
            CK(cudaMemcpyAsync(p->d_uvw.p, uvw, bytes, cudaMemcpyHostToDevice, p->stream));
            CK(launch_words_differ(p->d_uvw.p, p->d_uvw_prev.p, static_cast<int64_t>(bytes / 8),
                                   p->d_uvw_flag.as<int32_t>(), p->stream));
            p->tc.coef_recompute_flag = p->d_uvw_flag.as<int32_t>();
        } else {
            CK(cudaMemcpyAsync(p->d_uvw.p, uvw, bytes, cudaMemcpyHostToDevice, p->stream));
            p->tc.coef_recompute_flag = nullptr;
        }
        p->uvw_uploaded = (uvw == p->uvw.data());
        p->tc.coef_valid = false;
    } else if (!p->uvw_uploaded) {
        StageScope t(p, P9IDG_STAGE_H2D);
        CK(cudaMemcpyAsync(p->d_uvw.p, p->uvw.data(), bytes, cudaMemcpyHostToDevice, p->stream));
        p->uvw_uploaded = true;
        p->tc.coef_valid = false;
        p->tc.coef_recompute_flag = nullptr;
    }
    return P9IDG_OK;
}

p9idg_status upload_items(p9idg_plan *p) {
    CK(p->d_sub.ensure(sizeof(DevSubgrid) * std::max<size_t>(1, p->dsub.size())));
    CK(p->d_gitems.ensure(sizeof(WorkItem) * std::max<size_t>(1, p->gitems.size())));
    CK(p->d_ditems.ensure(sizeof(WorkItem) * std::max<size_t>(1, p->ditems.size())));
    if (!p->ditems.empty())
        CK(cudaMemcpyAsync(p->d_ditems.p, p->ditems.data(), sizeof(WorkItem) * p->ditems.size(),
                           cudaMemcpyHostToDevice, p->stream));
    if (!p->dsub.empty())
        CK(cudaMemcpyAsync(p->d_sub.p, p->dsub.data(), sizeof(DevSubgrid) * p->dsub.size(), cudaMemcpyHostToDevice,
                           p->stream));
    if (!p->gitems.empty())
        CK(cudaMemcpyAsync(p->d_gitems.p, p->gitems.data(), sizeof(WorkItem) * p->gitems.size(),
                           cudaMemcpyHostToDevice, p->stream));
    CK(cudaStreamSynchronize(p->stream));  // the host vectors may be rebuilt by a later set_mode
    p->items_dirty = false;
    return P9IDG_OK;
}

// Device state for a call, without the uvw upload (in-place host calls start their transfers in
// the other direction first and upload uvw beside them).
p9idg_status prepare_state(p9idg_plan *p) {
    TRY(ensure_device(p));
    if (p->items_dirty) TRY(upload_items(p));
    if (p->taper_dirty) {
        CK(cudaMemcpyAsync(p->d_taper.p, p->taper.data(), sizeof(float) * p->taper.size(), cudaMemcpyHostToDevice,
                           p->stream));
        p->taper_dirty = false;
    }
    CK(cudaMemsetAsync(p->d_status.p, 0, sizeof(int32_t), p->stream));
    return P9IDG_OK;
}

p9idg_status prepare(p9idg_plan *p, const double *uvw) {
    TRY(prepare_state(p));
    return upload_uvw(p, uvw);
}

p9idg_status finish_call(p9idg_plan *p) {
    int32_t status = 0;
    CK(cudaMemcpyAsync(&status, p->d_status.p, sizeof(int32_t), cudaMemcpyDeviceToHost, p->stream));
    CK(cudaStreamSynchronize(p->stream));
    if (p->timing) collect_timing(p);
    if (status == kStatusWTerm)
        return fail(P9IDG_UNSUPPORTED, "this call's uvw puts |dw r| above the bound of the plan's tensor-core "
                                       "form: use P9IDG_MODE_FP32 or a plan made from this uvw");
    if (status != 0)
        return fail(P9IDG_DEVICE_CHECK_FAILED, "a kernel bounds check tripped (status " + std::to_string(status) + ")");
    return P9IDG_OK;
}

GridderArgs gridder_args(p9idg_plan *p) {
    GridderArgs a{};
    a.g = p->geom();
    a.subs = p->d_sub.as<DevSubgrid>();
    a.uvw = p->d_uvw.as<double>();
    a.wavenumbers = p->d_wn.as<double>();
    a.lmn = p->d_lmn.as<float>();
    a.taper = p->d_taper.as<float>();
    a.nsub = static_cast<int32_t>(p->dsub.size());
    a.status = p->d_status.as<int32_t>();
    return a;
}

p9idg_status ensure_tc(p9idg_plan *p) {
    if (p->tc.ready) return P9IDG_OK;
    // degridder items do not accumulate across visibilities: 16384 measured 1.6 % faster than 8192
    // (32768 the same as 16384), 8192 3.5 % faster than 4096
    p->tc.degrid_chunk = p->dchunk > 0 ? p->dchunk : 16384;
    return tc_prepare(p->tc, p->subs, p->lmn, p->c.subgrid_size, p->nch, p->wn, p->uvw.data(), p->nt, p->stream,
                      g_last_error);
}

SubgridOpArgs subgrid_args(p9idg_plan *p) {
    SubgridOpArgs a{};
    a.g = p->geom();
    a.subs = p->d_sub.as<DevSubgrid>();
    a.nsub = static_cast<int32_t>(p->dsub.size());
    a.add_phasor = p->d_phasor.as<float2>();
    a.twiddles = p->d_phasor.as<float2>() + static_cast<size_t>(p->c.subgrid_size) * p->c.subgrid_size;
    a.status = p->d_status.as<int32_t>();
    return a;
}

bool use_tc(const p9idg_plan *p) { return p->mode != P9IDG_MODE_FP32; }

// Adder.Add throws "invalid grid" for subgrids outside [0, N-S) (Adder.cs:30-50).
p9idg_status check_adder_range(const p9idg_plan *p) {
    const int N = p->c.grid_size, S = p->c.subgrid_size;
    for (const auto &s : p->subs)
        if (!(s.u_pixel >= 0 && s.u_pixel < N - S && s.v_pixel >= 0 && s.v_pixel < N - S))
            return fail(P9IDG_INVALID_GRID, "invalid grid");
    return P9IDG_OK;
}

// AdderWStack.Add indexes grid[subgridW] after its range check (AdderWStack.cs:47-67).
p9idg_status check_wstack_layers(const p9idg_plan *p) {
    const int N = p->c.grid_size, S = p->c.subgrid_size, W = p->c.wlayer_count;
    for (const auto &s : p->subs) {
        int sx = s.u_pixel, sy = s.v_pixel, sw = s.w_lambda;
        if (sw < 0) {
            sx = N - sx - S + 1;
            sy = N - sy - S + 1;
            sw = -sw - 1;
        }
        if (!(sx >= 1 && sx < N - S && sy >= 1 && sy < N - S)) continue;
        if (sw >= W) return fail(P9IDG_INVALID_ARGUMENT, "subgrid w layer index outside the w stack");
    }
    return P9IDG_OK;
}

// vis (device, complex64 or complex128) -> layers (device complex64, W or 1 grids)
size_t vis_count_of(const p9idg_plan *p) { return static_cast<size_t>(p->nbl) * p->nt * p->nch; }
size_t nn_of(const p9idg_plan *p) { return static_cast<size_t>(p->c.grid_size) * p->c.grid_size; }

// A zero-fill of output memory that the kernels queued meanwhile on the plan's stream do not touch
// (the w layers while the gridder writes its partial subgrids; the visibilities no subgrid covers
// while the splitter and degridder write the others), run on the zeroing stream: fork() before those
// kernels, the fill launched after them (so that their first CTAs are placed first), join() before
// the first kernel that needs it.  A call that returns early with an error waits for the fill on
// the host, so none outlives the call.
struct ZeroSide {
    p9idg_plan *p;
    bool forked = false, joined = false;
    p9idg_status fork() {
        CK(cudaEventRecord(p->ev_zfork, p->stream));
        CK(cudaStreamWaitEvent(p->zside, p->ev_zfork, 0));
        forked = true;
        return P9IDG_OK;
    }
    p9idg_status join() {
        CK(cudaEventRecord(p->ev_zjoin, p->zside));
        CK(cudaStreamWaitEvent(p->stream, p->ev_zjoin, 0));
        joined = true;
        return P9IDG_OK;
    }
    ~ZeroSide() {
        if (forked && !joined) (void)cudaStreamSynchronize(p->zside);
    }
};

// Gridder over nitems work items (all of the plan's, or a group of them) into their partial slots.
p9idg_status grid_items(p9idg_plan *p, const void *d_vis, bool vis_c128, const WorkItem *d_items, int32_t nitems) {
    const int S = p->c.subgrid_size;
    CK(p->d_partials.ensure(sizeof(float2) * S * S * std::max<size_t>(1, p->nslots)));
    StageScope t(p, P9IDG_STAGE_GRIDDER);
    GridderArgs a = gridder_args(p);
    a.items = d_items;
    a.nitems = nitems;
    a.vis = d_vis;
    a.vis_c128 = vis_c128;
    a.partials = p->d_partials.as<float2>();
    if (use_tc(p)) {
        TRY(ensure_tc(p));
        TRY(tc_grid(p->tc, a, p->mode, p->stream, g_last_error));
    } else {
        CK(launch_gridder_fp32(a, p->stream));
    }
    return P9IDG_OK;
}

// Subgrid IFFT + adder of nsub subgrids (all, or the subgrid list d_list) into the layers.
p9idg_status add_subgrids(p9idg_plan *p, float2 *d_layers, bool wstack, const int32_t *d_list, int32_t nsub) {
    StageScope t(p, P9IDG_STAGE_SUBGRID_IFFT_ADD);
    SubgridOpArgs a = subgrid_args(p);
    a.partials = p->d_partials.as<float2>();
    a.layers = d_layers;
    a.out_shifted = true;  // IDG.cs:17,37
    a.wstack = wstack;
    if (d_list) {
        a.sub_list = d_list;
        a.nsub = nsub;
    }
    CK(launch_subgrid_ifft_add(a, p->stream));
    return P9IDG_OK;
}

// The layers are zeroed beside the gridder (a 604 MB fill at 3072^2 with 8 layers, 0.09 ms of the
// adder's stage when it ran there).
p9idg_status run_grid(p9idg_plan *p, const void *d_vis, bool vis_c128, float2 *d_layers, bool wstack) {
    const int nl = wstack ? p->c.wlayer_count : 1;
    ZeroSide z{p};
    TRY(z.fork());
    TRY(grid_items(p, d_vis, vis_c128, p->d_gitems.as<WorkItem>(), static_cast<int32_t>(p->gitems.size())));
    CK(launch_zero_c64_beside(d_layers, static_cast<int64_t>(nl) * static_cast<int64_t>(nn_of(p)), p->zside));
    TRY(z.join());
    return add_subgrids(p, d_layers, wstack, nullptr, 0);
}

// grid (device complex64) -> vis (device, complex64 or complex128); uncovered samples are 0
p9idg_status ensure_gaps(p9idg_plan *p);

// The degridder writes every visibility some subgrid covers; only the others (quirk P1's drops,
// baselines without subgrids) are zeroed apart.  Output in host memory (out_in_host): before the
// degridder, on the plan's stream.  Output in device memory: beside the splitter and degridder, on
// the zeroing stream, as the two write disjoint visibilities (the whole output, 516 MB at 3072^2,
// was zeroed before the degridder, 0.08 ms of its stage).
p9idg_status run_degrid(p9idg_plan *p, const float2 *d_grid, bool grid_shifted, void *d_vis, bool out_c128,
                        bool wstack, bool out_in_host = false) {
    const int S = p->c.subgrid_size;
    CK(p->d_subgrids.ensure(sizeof(float2) * S * S * std::max<size_t>(1, p->dsub.size())));
    TRY(ensure_gaps(p));
    const int64_t ngaps = static_cast<int64_t>(p->gaps.size() / 2);
    ZeroSide z{p};
    if (!out_in_host) TRY(z.fork());
    {
        StageScope t(p, P9IDG_STAGE_SPLIT_SUBGRID_FFT);
        SubgridOpArgs a = subgrid_args(p);
        a.grid = d_grid;
        a.grid_shifted = grid_shifted;
        a.subgrids = p->d_subgrids.as<float2>();
        a.wstack = wstack;
        CK(launch_split_subgrid_fft(a, p->stream));
    }
    if (!out_in_host) CK(launch_zero_ranges_beside(d_vis, out_c128, p->d_gaps.as<int64_t>(), ngaps, p->zside));
    {
        StageScope t(p, P9IDG_STAGE_DEGRIDDER);
        if (out_in_host) CK(launch_zero_ranges(d_vis, out_c128, p->d_gaps.as<int64_t>(), ngaps, p->stream));
        GridderArgs a = gridder_args(p);
        a.items = p->d_ditems.as<WorkItem>();
        a.nitems = static_cast<int32_t>(p->ditems.size());
        a.subgrids = p->d_subgrids.as<float2>();
        a.vis_out = d_vis;
        a.out_c128 = out_c128;
        if (use_tc(p)) {
            TRY(ensure_tc(p));
            TRY(tc_degrid(p->tc, a, p->mode, p->stream, g_last_error));
        } else {
            CK(launch_degridder_fp32(a, p->stream));
        }
    }
    if (!out_in_host) TRY(z.join());
    return P9IDG_OK;
}

p9idg_status h2d(p9idg_plan *p, void *dst, const void *src, size_t bytes) {
    StageScope t(p, P9IDG_STAGE_H2D);
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, p->stream));
    return P9IDG_OK;
}

p9idg_status d2h(p9idg_plan *p, void *dst, const void *src, size_t bytes) {
    StageScope t(p, P9IDG_STAGE_D2H);
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, p->stream));
    return P9IDG_OK;
}

// device layers complex64 -> host Complex (double) array
p9idg_status layers_to_host(p9idg_plan *p, const float2 *d_layers, size_t count, double *out) {
    CK(p->d_out128.ensure(sizeof(double2) * count));
    {
        StageScope t(p, P9IDG_STAGE_CONVERT);
        CK(launch_c64_to_c128(d_layers, static_cast<int64_t>(count), p->d_out128.as<double2>(), p->stream));
    }
    return d2h(p, out, p->d_out128.p, sizeof(double2) * count);
}

// Uncovered visibility ranges (quirk P1 drops, baselines without subgrids), built once.
p9idg_status ensure_gaps(p9idg_plan *p) {
    if (p->gaps_ready) return P9IDG_OK;
    p->gaps.clear();
    std::vector<std::vector<std::pair<int32_t, int32_t>>> cov(std::max(0, p->nbl));
    for (const auto &sg : p->subs)
        if (sg.baseline_idx >= 0 && sg.baseline_idx < p->nbl)
            cov[sg.baseline_idx].emplace_back(sg.time_sample_start, sg.time_sample_start + sg.time_sample_count);
    const int64_t nch = p->nch;
    for (int b = 0; b < p->nbl; b++) {
        auto &v = cov[b];
        std::sort(v.begin(), v.end());
        int32_t t = 0;
        for (const auto &r : v) {
            const int32_t a = std::max(0, std::min(r.first, p->nt)), e = std::max(0, std::min(r.second, p->nt));
            if (a > t) {
                p->gaps.push_back((static_cast<int64_t>(b) * p->nt + t) * nch);
                p->gaps.push_back(static_cast<int64_t>(a - t) * nch);
            }
            t = std::max(t, e);
        }
        if (t < p->nt) {
            p->gaps.push_back((static_cast<int64_t>(b) * p->nt + t) * nch);
            p->gaps.push_back(static_cast<int64_t>(p->nt - t) * nch);
        }
    }
    // AdderWStack.Add's target layer of each subgrid it does not skip (AdderWStack.cs:41-51)
    const int N = p->c.grid_size, S = p->c.subgrid_size, W = p->c.wlayer_count;
    p->layer_used.assign(std::max(W, 1), 0);
    for (const auto &sg : p->subs) {
        int sx = sg.u_pixel, sy = sg.v_pixel, sw = sg.w_lambda;
        if (sw < 0) {
            sx = N - sx - S + 1;
            sy = N - sy - S + 1;
            sw = -sw - 1;
        }
        if (sx >= 1 && sx < N - S && sy >= 1 && sy < N - S && sw >= 0 && sw < W) p->layer_used[sw] = 1;
    }
    CK(p->d_gaps.ensure(sizeof(int64_t) * std::max<size_t>(2, p->gaps.size())));
    if (!p->gaps.empty())
        CK(cudaMemcpyAsync(p->d_gaps.p, p->gaps.data(), sizeof(int64_t) * p->gaps.size(), cudaMemcpyHostToDevice,
                           p->stream));
    CK(cudaStreamSynchronize(p->stream));
    p->gaps_ready = true;
    return P9IDG_OK;
}

bool host_in_place(const p9idg_plan *p) { return p->host_direct && p->host_access != 0; }

// Work forked onto the side stream writes the caller's arrays: a call that returns early with an
// error must not leave it running, so this waits for the side stream when it goes out of scope
// (on success the main stream has already joined it).
struct SideJoin {
    p9idg_plan *p;
    ~SideJoin() { (void)cudaStreamSynchronize(p->side); }
};

// Target w layer and first destination row of each subgrid as AdderWStack.Add places it
// (AdderWStack.cs:38-51; layer -1: skipped), the busiest layer by gridded time samples, and the
// gridder items and subgrids regrouped as [every other layer | the busiest layer in row bands].
// A subgrid at row y0 adds into rows y0 .. y0 + S - 1, so once the bands up to b are added, every
// row below the first row of band b + 1 is final.  A band holds about kBandItems gridder items
// (about four waves of the tensor-core gridder's two CTAs per SM), at most kMaxBands bands: on the
// 3072^2 workload (13,951 items in the busiest layer) 2, 4, 8, 12, 16 and 24 bands gave GridW in
// 8.13, 7.80, 7.56, 7.39, 7.52 and 7.82 ms, against 8.03 ms writing the layer back after all of it.
constexpr int kBandItems = 1152, kMaxBands = 16;

p9idg_status ensure_layer_split(p9idg_plan *p) {
    if (p->lyr_ready) return P9IDG_OK;
    const int N = p->c.grid_size, S = p->c.subgrid_size, W = p->c.wlayer_count;
    std::vector<int32_t> layer(p->subs.size(), -1), row(p->subs.size(), 0);
    std::vector<int64_t> work(std::max(W, 1), 0);
    for (size_t i = 0; i < p->subs.size(); i++) {
        const auto &sg = p->subs[i];
        int sx = sg.u_pixel, sy = sg.v_pixel, sw = sg.w_lambda;
        if (sw < 0) {
            sx = N - sx - S + 1;
            sy = N - sy - S + 1;
            sw = -sw - 1;
        }
        if (sx >= 1 && sx < N - S && sy >= 1 && sy < N - S && sw >= 0 && sw < W) {
            layer[i] = sw;
            row[i] = sy;
            work[sw] += sg.time_sample_count;
        }
    }
    p->lyr_major = -1;
    int64_t best = 0;
    for (int k = 0; k < W; k++)
        if (work[k] > best) {
            best = work[k];
            p->lyr_major = k;
        }
    p->gitems_lyr.clear();
    p->sub_lyr.clear();
    p->lyr_band_items.clear();
    p->lyr_band_subs.clear();
    p->lyr_band_rows.clear();
    p->lyr_minor_items = p->lyr_minor_subs = 0;
    if (p->lyr_major >= 0) {
        const int32_t major = p->lyr_major;
        for (const auto &it : p->gitems)
            if (layer[it.subgrid] != major) p->gitems_lyr.push_back(it);
        for (size_t i = 0; i < layer.size(); i++)
            if (layer[i] != major) p->sub_lyr.push_back(static_cast<int32_t>(i));
        p->lyr_minor_items = static_cast<int32_t>(p->gitems_lyr.size());
        p->lyr_minor_subs = static_cast<int32_t>(p->sub_lyr.size());
        // the busiest layer's subgrids by first row, cut into bands of about equal work
        std::vector<int32_t> msubs;
        for (size_t i = 0; i < layer.size(); i++)
            if (layer[i] == major) msubs.push_back(static_cast<int32_t>(i));
        std::stable_sort(msubs.begin(), msubs.end(), [&](int32_t a, int32_t b) { return row[a] < row[b]; });
        int64_t mitems = 0;
        for (const auto &it : p->gitems) mitems += layer[it.subgrid] == major;
        const int nb = static_cast<int>(std::min<int64_t>(
            std::min<int64_t>(kMaxBands, std::max<int64_t>(1, (mitems + kBandItems / 2) / kBandItems)),
            static_cast<int64_t>(msubs.size())));
        std::vector<int32_t> band(p->subs.size(), -1);
        int64_t acc = 0;
        int b = 0;
        for (int32_t i : msubs) {
            band[i] = b;
            acc += p->subs[i].time_sample_count;
            if (b + 1 < nb && acc * nb >= best * (b + 1)) b++;
        }
        p->lyr_band_rows.assign(nb + 1, N);
        p->lyr_band_rows[0] = 0;
        for (int32_t i : msubs)  // first row of each band (the bands are in row order)
            if (band[i] > 0) p->lyr_band_rows[band[i]] = std::min(p->lyr_band_rows[band[i]], row[i]);
        for (int k = nb - 1; k >= 1; k--)  // a band that received no subgrid ends where the next starts
            p->lyr_band_rows[k] = std::min(p->lyr_band_rows[k], p->lyr_band_rows[k + 1]);
        p->lyr_band_items.push_back(0);
        p->lyr_band_subs.push_back(0);
        for (int k = 0; k < nb; k++) {
            for (const auto &it : p->gitems)  // largest first within the band, as gitems is
                if (layer[it.subgrid] == major && band[it.subgrid] == k) p->gitems_lyr.push_back(it);
            for (int32_t i : msubs)
                if (band[i] == k) p->sub_lyr.push_back(i);
            p->lyr_band_items.push_back(static_cast<int32_t>(p->gitems_lyr.size()) - p->lyr_minor_items);
            p->lyr_band_subs.push_back(static_cast<int32_t>(p->sub_lyr.size()) - p->lyr_minor_subs);
        }
        CK(p->d_gitems_lyr.ensure(sizeof(WorkItem) * std::max<size_t>(1, p->gitems_lyr.size())));
        CK(p->d_sub_lyr.ensure(sizeof(int32_t) * std::max<size_t>(1, p->sub_lyr.size())));
        if (!p->gitems_lyr.empty())
            CK(cudaMemcpyAsync(p->d_gitems_lyr.p, p->gitems_lyr.data(), sizeof(WorkItem) * p->gitems_lyr.size(),
                               cudaMemcpyHostToDevice, p->stream));
        if (!p->sub_lyr.empty())
            CK(cudaMemcpyAsync(p->d_sub_lyr.p, p->sub_lyr.data(), sizeof(int32_t) * p->sub_lyr.size(),
                               cudaMemcpyHostToDevice, p->stream));
        CK(cudaStreamSynchronize(p->stream));
    }
    p->lyr_ready = true;
    return P9IDG_OK;
}

// Page-locked host memory (first and last byte): written by the copy engines, which reach the
// link's full device-to-host rate; pageable memory reached through the host page tables is
// written by kernels instead.
bool host_pinned(const void *ptr, size_t bytes) {
    for (const char *q : {static_cast<const char *>(ptr), static_cast<const char *>(ptr) + bytes - 1}) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
            (void)cudaGetLastError();
            return false;
        }
        if (at.type != cudaMemoryTypeHost) return false;
    }
    return true;
}

// One complex64 layer -> the caller's complex128 layer in host memory: widened on the device into
// the staging slot and copied by a copy engine (pinned), or widened straight into host memory.
p9idg_status layer_to_host(const float2 *d_layer, size_t nn, double2 *h_out, double2 *d_stage, bool pinned,
                           cudaStream_t st) {
    if (pinned) {
        CK(launch_c64_to_c128(d_layer, static_cast<int64_t>(nn), d_stage, st));
        CK(cudaMemcpyAsync(h_out, d_stage, sizeof(double2) * nn, cudaMemcpyDeviceToHost, st));
    } else {
        CK(launch_c64_to_c128(d_layer, static_cast<int64_t>(nn), h_out, st));
    }
    return P9IDG_OK;
}

// Rows [r0, r1) of one complex64 layer, as the adder numbers them (before the FFT.Shift the layer
// is stored with), -> the same rows of the caller's complex128 layer: the shifted rows of the range
// form at most two contiguous runs (three for an odd N), each widened and copied on its own.
p9idg_status layer_rows_to_host(const float2 *d_layer, int N, int r0, int r1, double2 *h_out, double2 *d_stage,
                                bool pinned, cudaStream_t st) {
    const int n2 = N / 2, m = 2 * n2;
    auto stored = [&](int r) { return r < m ? (r + n2 < m ? r + n2 : r - n2) : r; };  // shift_index's row map
    for (int r = r0; r < r1;) {
        const int a = stored(r);
        int len = 1;
        while (r + len < r1 && stored(r + len) == a + len) len++;
        const size_t off = static_cast<size_t>(a) * N, count = static_cast<size_t>(len) * N;
        TRY(layer_to_host(d_layer + off, count, h_out + off, pinned ? d_stage + off : nullptr, pinned, st));
        r += len;
    }
    return P9IDG_OK;
}

// Zeros one complex128 layer of the caller's output in host memory.
p9idg_status zero_host_layer(p9idg_plan *p, double2 *h_out, size_t nn, bool pinned, cudaStream_t st) {
    if (pinned) {
        if (p->d_zero128.bytes < sizeof(double2) * nn) {
            CK(p->d_zero128.ensure(sizeof(double2) * nn));
            CK(cudaMemsetAsync(p->d_zero128.p, 0, sizeof(double2) * nn, st));
        }
        CK(cudaMemcpyAsync(h_out, p->d_zero128.p, sizeof(double2) * nn, cudaMemcpyDeviceToHost, st));
    } else {
        CK(launch_zero_c128(h_out, static_cast<int64_t>(nn), st));
    }
    return P9IDG_OK;
}


p9idg_status host_grid_common(p9idg_plan *p, const double *vis, const double *uvw, double *out, bool wstack) {
    if (!p || !vis || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(wstack ? check_wstack_layers(p) : check_adder_range(p));
    TRY(prepare_state(p));
    const size_t nvis = vis_count_of(p), nl = wstack ? p->c.wlayer_count : 1;
    if (host_in_place(p)) {
        // The gridder reads the caller's complex128 visibilities in host memory, once each, while
        // the layers no subgrid adds into are zeroed in the output beside it (those writes use the
        // device-to-host direction of the link, the gridder's reads the other).  With w stacking
        // the layers other than the busiest are gridded and added first and written back while the
        // busiest one grids, so only the busiest layer's writeback follows the gridder.
        const size_t nn = nn_of(p);
        CK(p->d_layers.ensure(sizeof(float2) * nl * nn));
        std::vector<char> used(nl, 1);
        bool banded = false;
        if (wstack) {
            TRY(ensure_gaps(p));
            used.assign(p->layer_used.begin(), p->layer_used.begin() + nl);
            TRY(ensure_layer_split(p));
            banded = p->lyr_major >= 0 && !p->lyr_band_rows.empty();
        }
        auto *out128 = reinterpret_cast<double2 *>(out);
        const bool pinned = host_pinned(out, sizeof(double2) * nl * nn);
        std::vector<size_t> stage_slot(nl, 0);  // staging layer of each used layer (pinned output)
        size_t nused = 0;
        for (size_t k = 0; k < nl; k++)
            if (used[k]) stage_slot[k] = nused++;
        if (pinned) CK(p->d_out128.ensure(sizeof(double2) * std::max<size_t>(1, nused) * nn));
        auto stage = [&](size_t k) { return pinned ? p->d_out128.as<double2>() + stage_slot[k] * nn : nullptr; };
        SideJoin join{p};
        CK(cudaEventRecord(p->ev_fork, p->stream));
        CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
        for (size_t k = 0; k < nl; k++)
            if (!used[k]) TRY(zero_host_layer(p, out128 + k * nn, nn, pinned, p->side));
        TRY(upload_uvw(p, uvw));  // host-to-device, beside the zero-fill
        float2 *layers = p->d_layers.as<float2>();
        if (!banded) {
            TRY(run_grid(p, vis, true, layers, wstack));
            StageScope t(p, P9IDG_STAGE_D2H);
            for (size_t k = 0; k < nl; k++)
                if (used[k])
                    TRY(layer_to_host(layers + k * nn, nn, out128 + k * nn, stage(k), pinned,
                                      p->stream));
        } else {
            const WorkItem *items = p->d_gitems_lyr.as<WorkItem>();
            const int32_t *subl = p->d_sub_lyr.as<int32_t>();
            const int32_t nmi = p->lyr_minor_items, nms = p->lyr_minor_subs;
            const size_t major = static_cast<size_t>(p->lyr_major);
            // every layer is zeroed beside the first gridder launch, before the first add
            ZeroSide z{p};
            TRY(z.fork());
            auto zero_layers = [&]() -> p9idg_status {
                if (z.joined) return P9IDG_OK;
                CK(launch_zero_c64_beside(layers, static_cast<int64_t>(nl * nn), p->zside));
                return z.join();
            };
            if (nmi > 0 || nms > 0) {
                TRY(grid_items(p, vis, true, items, nmi));
                TRY(zero_layers());
                TRY(add_subgrids(p, layers, true, subl, nms));
                CK(cudaEventRecord(p->ev_mid, p->stream));
                CK(cudaStreamWaitEvent(p->side, p->ev_mid, 0));
                for (size_t k = 0; k < nl; k++)
                    if (used[k] && k != major)
                        TRY(layer_to_host(layers + k * nn, nn, out128 + k * nn, stage(k), pinned,
                                          p->side));
            }
            const auto &bi = p->lyr_band_items, &bs = p->lyr_band_subs, &br = p->lyr_band_rows;
            const int N = p->c.grid_size;
            for (size_t b = 0; b + 1 < br.size(); b++) {
                TRY(grid_items(p, vis, true, items + nmi + bi[b], bi[b + 1] - bi[b]));
                TRY(zero_layers());
                TRY(add_subgrids(p, layers, true, subl + nms + bs[b], bs[b + 1] - bs[b]));
                // the band's final rows cross the link while the next band grids
                CK(cudaEventRecord(p->ev_mid, p->stream));
                CK(cudaStreamWaitEvent(p->side, p->ev_mid, 0));
                TRY(layer_rows_to_host(layers + major * nn, N, br[b], br[b + 1], out128 + major * nn,
                                       stage(major), pinned, p->side));
            }
            TRY(zero_layers());  // (done by then: the busiest layer has at least one band)
        }
        CK(cudaEventRecord(p->ev_join, p->side));
        CK(cudaStreamWaitEvent(p->stream, p->ev_join, 0));
        return finish_call(p);
    }
    TRY(upload_uvw(p, uvw));
    CK(p->d_vis_in.ensure(sizeof(double2) * std::max<size_t>(1, nvis)));
    CK(p->d_layers.ensure(sizeof(float2) * nl * nn_of(p)));
    TRY(h2d(p, p->d_vis_in.p, vis, sizeof(double2) * nvis));
    TRY(run_grid(p, p->d_vis_in.p, true, p->d_layers.as<float2>(), wstack));
    TRY(layers_to_host(p, p->d_layers.as<float2>(), nl * nn_of(p), out));
    return finish_call(p);
}

p9idg_status host_degrid_common(p9idg_plan *p, double *grid_io, const double *uvw, double *vis_out, bool wstack) {
    if (!p || !grid_io || !vis_out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(prepare_state(p));
    const size_t nn = nn_of(p), nvis = vis_count_of(p);
    if (host_in_place(p)) {
        CK(p->d_grid128b.ensure(sizeof(double2) * nn));
        CK(p->d_grid64.ensure(sizeof(float2) * nn));
        {
            StageScope t(p, P9IDG_STAGE_H2D);  // reads the caller's grid in host memory
            CK(launch_shift_convert(reinterpret_cast<const double2 *>(grid_io), p->c.grid_size,
                                    p->d_grid64.as<float2>(), p->d_grid128b.as<double2>(), p->stream));
        }
        // FFT.Shift(grid) mutates the caller's array (IDG.cs:24,44): copied back beside the degridder
        SideJoin join{p};
        CK(cudaEventRecord(p->ev_fork, p->stream));
        CK(cudaStreamWaitEvent(p->side, p->ev_fork, 0));
        CK(cudaMemcpyAsync(grid_io, p->d_grid128b.p, sizeof(double2) * nn, cudaMemcpyDeviceToHost, p->side));
        CK(cudaEventRecord(p->ev_join, p->side));
        TRY(upload_uvw(p, uvw));  // host-to-device, beside the copy-back of the shifted grid
        // the degridder writes the caller's complex128 output in place; uncovered samples are zeroed
        TRY(run_degrid(p, p->d_grid64.as<float2>(), true, vis_out, true, wstack, true));
        CK(cudaStreamWaitEvent(p->stream, p->ev_join, 0));
        return finish_call(p);
    }
    CK(p->d_grid128.ensure(sizeof(double2) * nn));
    CK(p->d_grid128b.ensure(sizeof(double2) * nn));
    CK(p->d_grid64.ensure(sizeof(float2) * nn));
    CK(p->d_vis_out.ensure(sizeof(double2) * std::max<size_t>(1, nvis)));
    TRY(upload_uvw(p, uvw));
    TRY(h2d(p, p->d_grid128.p, grid_io, sizeof(double2) * nn));
    {
        StageScope t(p, P9IDG_STAGE_CONVERT);
        CK(launch_shift_convert(p->d_grid128.as<double2>(), p->c.grid_size, p->d_grid64.as<float2>(),
                                p->d_grid128b.as<double2>(), p->stream));
    }
    // FFT.Shift(grid) mutates the caller's array (IDG.cs:24,44)
    TRY(d2h(p, grid_io, p->d_grid128b.p, sizeof(double2) * nn));
    TRY(run_degrid(p, p->d_grid64.as<float2>(), true, p->d_vis_out.p, true, wstack));
    TRY(d2h(p, vis_out, p->d_vis_out.p, sizeof(double2) * nvis));
    return finish_call(p);
}

// unit visibilities (IDG.cs:52-66) into a device complex64 buffer
p9idg_status unit_vis_device(p9idg_plan *p, const uint8_t *flags, float2 **d_vis) {
    const size_t nvis = vis_count_of(p);
    CK(p->d_flags.ensure(std::max<size_t>(1, nvis)));
    CK(p->d_vis_in.ensure(sizeof(double2) * std::max<size_t>(1, nvis)));
    TRY(h2d(p, p->d_flags.p, flags, nvis));
    {
        StageScope t(p, P9IDG_STAGE_CONVERT);
        CK(launch_unit_vis(p->d_flags.as<uint8_t>(), static_cast<int64_t>(nvis), p->d_vis_in.as<float2>(),
                           p->stream));
    }
    *d_vis = p->d_vis_in.as<float2>();
    return P9IDG_OK;
}

// grid (device complex64, in place) -> Re(IFFT)/norm, optionally shifted, into d_image (float or double)
p9idg_status image_from_grid(p9idg_plan *p, float2 *d_grid, double norm, bool shift, float *outf, double *outd) {
    StageScope t(p, P9IDG_STAGE_LAYER_FFT);
    cufftHandle h;
    TRY(p->fft.get(p->c.grid_size, p->stream, &h));
    if (cufftExecC2C(h, reinterpret_cast<cufftComplex *>(d_grid), reinterpret_cast<cufftComplex *>(d_grid),
                     CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail(P9IDG_CUDA_ERROR, "cufftExecC2C failed");
    CK(launch_real_part(d_grid, p->c.grid_size, norm, shift, outf, outd, p->stream));
    return P9IDG_OK;
}

// ---------- plan-less FFT helpers (FFT.cs entry points) ----------

struct Standalone {
    std::mutex mu;
    bool ready = false;
    int device = -1;
    cudaStream_t st = nullptr;
    DevBuf a, b, c;
    FftCache fft;
    p9idg_status init() {
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
            return fail(P9IDG_NO_DEVICE, "no CUDA device available");
        if (!ready) {
            CK(cudaGetDevice(&device));
            CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
            ready = true;
        }
        CK(cudaSetDevice(device));
        return P9IDG_OK;
    }
};

Standalone &standalone() {
    static Standalone s;
    return s;
}

}  // namespace

// ---------- batches: many plans, one launch per kernel stage ----------

struct p9idg_batch {
    std::vector<p9idg_plan *> plans;
    int device = -1;
    int32_t mode = P9IDG_MODE_FP32;
    cudaStream_t stream = nullptr;
    DevBuf d_gargs, d_dargs, d_aargs, d_sargs, d_tg, d_td;  // per-problem argument tables
    DevBuf d_gitems, d_ditems, d_refs, d_done_init, d_done, d_finish, d_start;
    int32_t ngitems = 0, nditems = 0, nrefs = 0;
    std::vector<WorkItem> h_gitems, h_ditems;  // merged work items of all problems, in launch order
    // problems may mix subgrid sizes: the items and subgrid references are grouped by size,
    // one launch per kernel stage and size (group k: items [g0, g0 + gn), [d0, d0 + dn), refs [r0, r0 + rn))
    struct Group {
        int32_t S, g0, gn, d0, dn, r0, rn;
    };
    std::vector<Group> groups;
    int tc_order = 1;  // tensor-core batches: 2 when any plan needs the second-order form
    std::vector<int64_t> prob_vis;             // visibilities per problem (for the schedules)
    int32_t schedule = P9IDG_SCHEDULE_THROUGHPUT;
    std::vector<void *> layers, vis_out;
    std::vector<size_t> layer_bytes, vis_bytes;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

__global__ void stamp_kernel(unsigned long long *t) { *t = device_ns(); }

p9idg_status batch_grid(p9idg_batch *b) {
    for (size_t i = 0; i < b->plans.size(); i++)
        CK(cudaMemsetAsync(b->layers[i], 0, b->layer_bytes[i], b->stream));
    for (const auto &g : b->groups) {
        GridderArgs L{};
        L.g.S = g.S;
        L.items = b->d_gitems.as<WorkItem>() + g.g0;
        L.nitems = g.gn;
        if (b->mode == P9IDG_MODE_FP32) {
            if (g.gn > 0) CK(launch_gridder_fp32(L, b->stream, b->d_gargs.as<GridderArgs>()));
        } else {
            TRY(tc_grid_batch(b->d_tg.as<TcArgs>(), L.items, g.gn, b->mode, b->tc_order, b->stream, g_last_error));
        }
    }
    for (const auto &g : b->groups) {
        SubgridOpArgs A{};
        A.g.S = g.S;
        A.refs = b->d_refs.as<int2>() + g.r0;
        A.nsub = g.rn;
        A.wstack = true;
        if (g.rn > 0) CK(launch_subgrid_ifft_add(A, b->stream, b->d_aargs.as<SubgridOpArgs>()));
    }
    return P9IDG_OK;
}

p9idg_status batch_degrid(p9idg_batch *b) {
    const size_t n = b->plans.size();
    stamp_kernel<<<1, 1, 0, b->stream>>>(b->d_start.as<unsigned long long>());
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(b->d_done.p, b->d_done_init.p, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, b->stream));
    CK(cudaMemsetAsync(b->d_finish.p, 0, sizeof(unsigned long long) * n, b->stream));
    for (const auto &g : b->groups) {
        SubgridOpArgs A{};
        A.g.S = g.S;
        A.refs = b->d_refs.as<int2>() + g.r0;
        A.nsub = g.rn;
        A.wstack = true;
        if (g.rn > 0) CK(launch_split_subgrid_fft(A, b->stream, b->d_sargs.as<SubgridOpArgs>()));
    }
    for (size_t i = 0; i < n; i++) CK(cudaMemsetAsync(b->vis_out[i], 0, b->vis_bytes[i], b->stream));
    for (const auto &g : b->groups) {
        GridderArgs L{};
        L.g.S = g.S;
        L.items = b->d_ditems.as<WorkItem>() + g.d0;
        L.nitems = g.dn;
        if (b->mode == P9IDG_MODE_FP32) {
            if (g.dn > 0) CK(launch_degridder_fp32(L, b->stream, b->d_dargs.as<GridderArgs>()));
        } else {
            TRY(tc_degrid_batch(b->d_td.as<TcArgs>(), L.items, g.dn, b->mode, b->tc_order, b->stream,
                                g_last_error));
        }
    }
    return P9IDG_OK;
}

template <typename T>
p9idg_status upload(DevBuf &buf, const std::vector<T> &v) {
    CK(buf.ensure(sizeof(T) * std::max<size_t>(1, v.size())));
    if (!v.empty()) CK(cudaMemcpy(buf.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
    return P9IDG_OK;
}

// Launch order of the merged work items.  THROUGHPUT: largest item first across all problems
// (the tail is short).  SMALL_FIRST: problems in order of size, each problem's items largest
// first, so small problems finish early in each phase.
p9idg_status batch_order(p9idg_batch *b, int32_t schedule) {
    const auto &pv = b->prob_vis;
    auto item_vis = [&](const WorkItem &w) { return static_cast<int64_t>(w.nt) * b->plans[w.problem]->nch; };
    auto throughput = [&](const WorkItem &x, const WorkItem &y) { return item_vis(x) > item_vis(y); };
    auto small_first = [&](const WorkItem &x, const WorkItem &y) {
        if (x.problem != y.problem)
            return pv[x.problem] != pv[y.problem] ? pv[x.problem] < pv[y.problem] : x.problem < y.problem;
        return item_vis(x) > item_vis(y);
    };
    auto size_of = [&](const WorkItem &w) { return b->plans[w.problem]->c.subgrid_size; };
    for (auto *v : {&b->h_gitems, &b->h_ditems}) {
        if (schedule == P9IDG_SCHEDULE_SMALL_FIRST)
            std::stable_sort(v->begin(), v->end(), small_first);
        else
            std::stable_sort(v->begin(), v->end(), throughput);
        // one launch per subgrid size: the items of each size contiguous, in size order
        std::stable_sort(v->begin(), v->end(),
                         [&](const WorkItem &x, const WorkItem &y) { return size_of(x) < size_of(y); });
    }
    for (auto &g : b->groups) {
        g.g0 = g.gn = g.d0 = g.dn = 0;
        bool gs = false, ds = false;
        for (size_t k = 0; k < b->h_gitems.size(); k++)
            if (size_of(b->h_gitems[k]) == g.S) {
                if (!gs) g.g0 = static_cast<int32_t>(k), gs = true;
                g.gn++;
            }
        for (size_t k = 0; k < b->h_ditems.size(); k++)
            if (size_of(b->h_ditems[k]) == g.S) {
                if (!ds) g.d0 = static_cast<int32_t>(k), ds = true;
                g.dn++;
            }
    }
    TRY(upload(b->d_gitems, b->h_gitems));
    TRY(upload(b->d_ditems, b->h_ditems));
    b->schedule = schedule;
    return P9IDG_OK;
}

void batch_release(p9idg_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    DevBuf *bufs[] = {&b->d_gargs, &b->d_dargs, &b->d_aargs, &b->d_sargs, &b->d_tg, &b->d_td, &b->d_gitems,
                      &b->d_ditems, &b->d_refs, &b->d_done_init, &b->d_done, &b->d_finish, &b->d_start};
    for (DevBuf *x : bufs) x->release();
    if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

// ====================================================================================
extern "C" {

p9idg_status p9idg_plan_create(const p9idg_params *c, const double *uvw, int32_t nbl, int32_t nt,
                               const double *frequencies, int32_t nch, p9idg_plan **out) {
    if (!out) return fail(P9IDG_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    TRY(check_params(c));
    if (nbl < 0 || nt < 0 || nch < 0) return fail(P9IDG_INVALID_ARGUMENT, "negative dimension");
    if ((static_cast<int64_t>(nbl) * nt > 0 && !uvw) || (nch > 0 && !frequencies))
        return fail(P9IDG_INVALID_ARGUMENT, "null uvw or frequencies");
    auto *p = new (std::nothrow) p9idg_plan();
    if (!p) return fail(P9IDG_OUT_OF_MEMORY, "plan allocation");
    p->c = *c;
    p->nbl = nbl;
    p->nt = nt;
    p->nch = nch;
    std::string err;
    p9idg_status st = partition(*c, uvw, nbl, nt, frequencies, nch, p->subs, err);
    if (st != P9IDG_OK) {
        delete p;
        return fail(st, err);
    }
    p->freq.assign(frequencies, frequencies + nch);
    p->uvw.assign(uvw, uvw + static_cast<size_t>(nbl) * nt * 3);
    finish_plan(p);
    *out = p;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_create_from_subgrids(const p9idg_params *c, const p9idg_subgrid *subgrids, int64_t nsub,
                                             const double *uvw, int32_t nbl, int32_t nt,
                                             const double *frequencies, int32_t nch, p9idg_plan **out) {
    if (!out) return fail(P9IDG_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    TRY(check_params(c));
    if (nbl < 0 || nt < 0 || nch < 0 || nsub < 0 || (nsub > 0 && !subgrids))
        return fail(P9IDG_INVALID_ARGUMENT, "invalid dimensions");
    if ((static_cast<int64_t>(nbl) * nt > 0 && !uvw) || (nch > 0 && !frequencies))
        return fail(P9IDG_INVALID_ARGUMENT, "null uvw or frequencies");
    std::string err;
    TRY(validate_subgrids(*c, subgrids, nsub, nbl, nt, err) == P9IDG_OK ? P9IDG_OK : fail(P9IDG_INVALID_ARGUMENT, err));
    auto *p = new (std::nothrow) p9idg_plan();
    if (!p) return fail(P9IDG_OUT_OF_MEMORY, "plan allocation");
    p->c = *c;
    p->nbl = nbl;
    p->nt = nt;
    p->nch = nch;
    p->subs.assign(subgrids, subgrids + nsub);
    p->freq.assign(frequencies, frequencies + nch);
    p->uvw.assign(uvw, uvw + static_cast<size_t>(nbl) * nt * 3);
    finish_plan(p);
    *out = p;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_num_subgrids(const p9idg_plan *plan, int64_t *n) {
    if (!plan || !n) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *n = static_cast<int64_t>(plan->subs.size());
    return P9IDG_OK;
}

p9idg_status p9idg_plan_get_subgrids(const p9idg_plan *plan, p9idg_subgrid *out, int64_t capacity) {
    if (!plan || (!out && !plan->subs.empty())) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    if (capacity < static_cast<int64_t>(plan->subs.size())) return fail(P9IDG_INVALID_ARGUMENT, "capacity too small");
    if (!plan->subs.empty()) std::memcpy(out, plan->subs.data(), sizeof(p9idg_subgrid) * plan->subs.size());
    return P9IDG_OK;
}

p9idg_status p9idg_plan_get_info(const p9idg_plan *plan, p9idg_plan_info *out) {
    if (!plan || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    out->num_subgrids = static_cast<int64_t>(plan->subs.size());
    out->input_visibilities = static_cast<int64_t>(plan->nbl) * plan->nt * plan->nch;
    out->gridded_visibilities = plan->gridded_vis;
    out->work_items = static_cast<int64_t>(plan->gitems.size());
    out->nbl = plan->nbl;
    out->nt = plan->nt;
    out->nch = plan->nch;
    out->mode = plan->mode;
    out->requested_mode = plan->requested_mode;
    out->tc_w_term = plan->tc_w_term;
    out->tc_order = plan->mode == P9IDG_MODE_FP32 ? 0 : tc_order_for(plan->tc_w_term, plan->tc.want_order);
    return P9IDG_OK;
}

p9idg_status p9idg_plan_set_mode(p9idg_plan *plan, int32_t mode) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    if (mode != P9IDG_MODE_FP32 && mode != P9IDG_MODE_TC_BF16X3 && mode != P9IDG_MODE_TC_FP16X3)
        return fail(P9IDG_INVALID_ARGUMENT, "unknown mode");
    if (mode == P9IDG_MODE_FP32 && !fp32_subgrid_size_supported(plan->c.subgrid_size))
        return fail(P9IDG_UNSUPPORTED, "subgrid size not supported by the FP32 kernels");
    if (mode != P9IDG_MODE_FP32 && !tc_subgrid_size_supported(plan->c.subgrid_size))
        return fail(P9IDG_UNSUPPORTED, "subgrid size not supported by the tensor-core kernels");
    plan->requested_mode = mode;
    if (mode != P9IDG_MODE_FP32) {
        if (plan->tc_w_term < 0)
            plan->tc_w_term = tc_w_term(plan->subs, plan->lmn, plan->c.subgrid_size, plan->wn, plan->uvw.data(),
                                        plan->nt);
        if (tc_order_for(plan->tc_w_term, plan->tc.want_order) == 0) {
            // outside both tensor-core forms' error bounds: the FP32 kernels grid this plan
            g_last_error = "tensor-core mode not used: |dw r| = " + std::to_string(plan->tc_w_term) + " > " +
                           std::to_string(P9IDG_TC_MAX_W_TERM2) + " for this plan; it runs the FP32 kernels";
            mode = P9IDG_MODE_FP32;
        }
    }
    const bool regroup = (plan->mode == P9IDG_MODE_FP32) != (mode == P9IDG_MODE_FP32);
    plan->mode = mode;
    if (regroup) build_gridder_items(plan);
    return P9IDG_OK;
}

p9idg_status p9idg_plan_set_tc_order(p9idg_plan *plan, int32_t order) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    if (order != 0 && order != 2) return fail(P9IDG_INVALID_ARGUMENT, "order must be 0 (automatic) or 2");
    if (plan->tc.ready) {
        TRY(ensure_device(plan));
        CK(cudaStreamSynchronize(plan->stream));  // launches in flight use the previous form's limit
    }
    tc_set_order(plan->tc, order);
    return P9IDG_OK;
}

p9idg_status p9idg_plan_set_taper(p9idg_plan *plan, const float *taper) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    const int S = plan->c.subgrid_size;
    if (taper)
        plan->taper.assign(taper, taper + S * S);
    else
        plan->taper.assign(S * S, 1.0f);
    plan->taper_dirty = true;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_set_stream(p9idg_plan *plan, void *cuda_stream) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    plan->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : plan->own_stream;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_get_stream(const p9idg_plan *plan, void **cuda_stream) {
    if (!plan || !cuda_stream) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *cuda_stream = plan->stream;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_get_params(const p9idg_plan *plan, p9idg_params *out) {
    if (!plan || !out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *out = plan->c;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_set_host_access(p9idg_plan *plan, int32_t in_place) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    plan->host_access = in_place != 0;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_get_host_access(p9idg_plan *plan, int32_t *in_place) {
    if (!plan || !in_place) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(ensure_device(plan));
    *in_place = host_in_place(plan) ? 1 : 0;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_init_device(p9idg_plan *plan) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    return ensure_device(plan);
}

void p9idg_plan_destroy(p9idg_plan *plan) {
    if (!plan) return;
    if (plan->device >= 0) {  // device state exists (complete, or left part-way by a failed call)
        cudaSetDevice(plan->device);
        if (plan->stream) cudaStreamSynchronize(plan->stream);
        for (auto &pt : plan->pending) {
            cudaEventDestroy(pt.a);
            cudaEventDestroy(pt.b);
        }
        for (auto e : plan->event_pool) cudaEventDestroy(e);
        DevBuf *bufs[] = {&plan->d_uvw, &plan->d_wn, &plan->d_sub, &plan->d_gitems, &plan->d_ditems, &plan->d_lmn,
                          &plan->d_taper, &plan->d_phasor, &plan->d_status, &plan->d_partials, &plan->d_subgrids,
                          &plan->d_vis_in, &plan->d_vis_out, &plan->d_layers, &plan->d_out128, &plan->d_grid128,
                          &plan->d_grid128b, &plan->d_grid64, &plan->d_flags, &plan->d_image};
        for (DevBuf *b : bufs) b->release();
        tc_release(plan->tc);
        plan->fft.release();
        plan->d_gaps.release();
        plan->d_gitems_lyr.release();
        plan->d_sub_lyr.release();
        plan->d_zero128.release();
        plan->d_uvw_prev.release();
        plan->d_uvw_flag.release();
        if (plan->side) cudaStreamDestroy(plan->side);
        if (plan->ev_fork) cudaEventDestroy(plan->ev_fork);
        if (plan->ev_join) cudaEventDestroy(plan->ev_join);
        if (plan->ev_mid) cudaEventDestroy(plan->ev_mid);
        if (plan->zside) cudaStreamDestroy(plan->zside);
        if (plan->ev_zfork) cudaEventDestroy(plan->ev_zfork);
        if (plan->ev_zjoin) cudaEventDestroy(plan->ev_zjoin);
        if (plan->own_stream) cudaStreamDestroy(plan->own_stream);
    }
    delete plan;
}

// ---- IDG facade, host arrays ----

p9idg_status p9idg_grid(p9idg_plan *plan, const double *vis, const double *uvw, double *grid_out) {
    return host_grid_common(plan, vis, uvw, grid_out, false);
}

p9idg_status p9idg_grid_w(p9idg_plan *plan, const double *vis, const double *uvw, double *layers_out) {
    return host_grid_common(plan, vis, uvw, layers_out, true);
}

p9idg_status p9idg_degrid(p9idg_plan *plan, double *grid_io, const double *uvw, double *vis_out) {
    return host_degrid_common(plan, grid_io, uvw, vis_out, false);
}

p9idg_status p9idg_degrid_w(p9idg_plan *plan, double *grid_io, const double *uvw, double *vis_out) {
    return host_degrid_common(plan, grid_io, uvw, vis_out, true);
}

p9idg_status p9idg_grid_psf(p9idg_plan *plan, const double *uvw, const uint8_t *flags, double *grid_out) {
    if (!plan || !flags || !grid_out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(check_adder_range(plan));
    TRY(prepare(plan, uvw));
    float2 *d_vis = nullptr;
    TRY(unit_vis_device(plan, flags, &d_vis));
    CK(plan->d_layers.ensure(sizeof(float2) * nn_of(plan)));
    TRY(run_grid(plan, d_vis, false, plan->d_layers.as<float2>(), false));
    TRY(layers_to_host(plan, plan->d_layers.as<float2>(), nn_of(plan), grid_out));
    return finish_call(plan);
}

static p9idg_status to_image_common(p9idg_plan *plan, const void *d_vis, bool c128, double *image_out) {
    CK(plan->d_layers.ensure(sizeof(float2) * nn_of(plan)));
    CK(plan->d_image.ensure(sizeof(double) * nn_of(plan)));
    TRY(run_grid(plan, d_vis, c128, plan->d_layers.as<float2>(), false));
    // FFT.Backward(grid, VisibilitiesCount) then FFT.Shift (IDG.cs:74-75)
    TRY(image_from_grid(plan, plan->d_layers.as<float2>(), static_cast<double>(plan->c.vis_count), true, nullptr,
                        plan->d_image.as<double>()));
    TRY(d2h(plan, image_out, plan->d_image.p, sizeof(double) * nn_of(plan)));
    return finish_call(plan);
}

p9idg_status p9idg_to_image(p9idg_plan *plan, const double *vis, const double *uvw, double *image_out) {
    if (!plan || !vis || !image_out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(check_adder_range(plan));
    TRY(prepare(plan, uvw));
    const size_t nvis = vis_count_of(plan);
    CK(plan->d_vis_in.ensure(sizeof(double2) * std::max<size_t>(1, nvis)));
    TRY(h2d(plan, plan->d_vis_in.p, vis, sizeof(double2) * nvis));
    return to_image_common(plan, plan->d_vis_in.p, true, image_out);
}

p9idg_status p9idg_calculate_psf(p9idg_plan *plan, const double *uvw, const uint8_t *flags, double *psf_out) {
    if (!plan || !flags || !psf_out) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(check_adder_range(plan));
    TRY(prepare(plan, uvw));
    float2 *d_vis = nullptr;
    TRY(unit_vis_device(plan, flags, &d_vis));
    return to_image_common(plan, d_vis, false, psf_out);
}

// ---- FFT.cs ----

p9idg_status p9idg_wstack_ifft_float(const double *layers, int32_t nlayers, int32_t n, int64_t vis_count,
                                     float *image_out) {
    if (!image_out || n <= 0 || nlayers < 0 || (nlayers > 0 && !layers))
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    Standalone &s = standalone();
    std::lock_guard<std::mutex> lk(s.mu);
    TRY(s.init());
    const size_t nn = static_cast<size_t>(n) * n;
    if (nlayers == 0) {
        std::memset(image_out, 0, sizeof(float) * nn);
        return P9IDG_OK;
    }
    CK(s.a.ensure(sizeof(double2) * nn * nlayers));
    CK(s.b.ensure(sizeof(float2) * nn));
    CK(s.c.ensure(sizeof(float) * nn));
    CK(cudaMemcpyAsync(s.a.p, layers, sizeof(double2) * nn * nlayers, cudaMemcpyHostToDevice, s.st));
    CK(launch_layer_sum(s.a.p, true, nlayers, static_cast<int64_t>(nn), s.b.as<float2>(), s.st));
    cufftHandle h;
    TRY(s.fft.get(n, s.st, &h));
    if (cufftExecC2C(h, s.b.as<cufftComplex>(), s.b.as<cufftComplex>(), CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail(P9IDG_CUDA_ERROR, "cufftExecC2C failed");
    CK(launch_real_part(s.b.as<float2>(), n, static_cast<double>(vis_count), false, s.c.as<float>(), nullptr, s.st));
    CK(cudaMemcpyAsync(image_out, s.c.p, sizeof(float) * nn, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return P9IDG_OK;
}

p9idg_status p9idg_fft_forward_float(const float *image, int32_t n, double norm, double *grid_out) {
    if (!image || !grid_out || n <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    Standalone &s = standalone();
    std::lock_guard<std::mutex> lk(s.mu);
    TRY(s.init());
    const size_t nn = static_cast<size_t>(n) * n;
    CK(s.a.ensure(sizeof(double2) * nn));
    CK(s.b.ensure(sizeof(float2) * nn));
    CK(s.c.ensure(sizeof(float) * nn));
    CK(cudaMemcpyAsync(s.c.p, image, sizeof(float) * nn, cudaMemcpyHostToDevice, s.st));
    CK(launch_real_to_c64(s.c.as<float>(), static_cast<int64_t>(nn), s.b.as<float2>(), s.st));
    cufftHandle h;
    TRY(s.fft.get(n, s.st, &h));
    if (cufftExecC2C(h, s.b.as<cufftComplex>(), s.b.as<cufftComplex>(), CUFFT_FORWARD) != CUFFT_SUCCESS)
        return fail(P9IDG_CUDA_ERROR, "cufftExecC2C failed");
    CK(launch_scale_c64_to_c128(s.b.as<float2>(), static_cast<int64_t>(nn), norm, s.a.as<double2>(), s.st));
    CK(cudaMemcpyAsync(grid_out, s.a.p, sizeof(double2) * nn, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return P9IDG_OK;
}

p9idg_status p9idg_fft_backward_float(const double *grid, int32_t n, double norm, float *image_out) {
    if (!grid || !image_out || n <= 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    Standalone &s = standalone();
    std::lock_guard<std::mutex> lk(s.mu);
    TRY(s.init());
    const size_t nn = static_cast<size_t>(n) * n;
    CK(s.a.ensure(sizeof(double2) * nn));
    CK(s.b.ensure(sizeof(float2) * nn));
    CK(s.c.ensure(sizeof(float) * nn));
    CK(cudaMemcpyAsync(s.a.p, grid, sizeof(double2) * nn, cudaMemcpyHostToDevice, s.st));
    CK(launch_c128_to_c64(s.a.as<double2>(), static_cast<int64_t>(nn), s.b.as<float2>(), s.st));
    cufftHandle h;
    TRY(s.fft.get(n, s.st, &h));
    if (cufftExecC2C(h, s.b.as<cufftComplex>(), s.b.as<cufftComplex>(), CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail(P9IDG_CUDA_ERROR, "cufftExecC2C failed");
    CK(launch_real_part(s.b.as<float2>(), n, norm, false, s.c.as<float>(), nullptr, s.st));
    CK(cudaMemcpyAsync(image_out, s.c.p, sizeof(float) * nn, cudaMemcpyDeviceToHost, s.st));
    CK(cudaStreamSynchronize(s.st));
    return P9IDG_OK;
}

p9idg_status p9idg_fft_shift(void *array, int32_t n, int32_t elem_bytes) {
    if (!array || n < 0 || (elem_bytes != 4 && elem_bytes != 8 && elem_bytes != 16))
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    fft_shift_host(array, n, elem_bytes);
    return P9IDG_OK;
}

// ---- device-resident interface ----

p9idg_status p9idg_grid_w_device(p9idg_plan *plan, const void *d_vis, void *d_layers) {
    if (!plan || !d_vis || !d_layers) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(check_wstack_layers(plan));
    TRY(prepare(plan, nullptr));
    return run_grid(plan, d_vis, false, static_cast<float2 *>(d_layers), true);
}

p9idg_status p9idg_degrid_w_device(p9idg_plan *plan, const void *d_grid, void *d_vis) {
    if (!plan || !d_grid || !d_vis) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(prepare(plan, nullptr));
    return run_degrid(plan, static_cast<const float2 *>(d_grid), false, d_vis, false, true);
}

p9idg_status p9idg_grid_device(p9idg_plan *plan, const void *d_vis, void *d_grid) {
    if (!plan || !d_vis || !d_grid) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(check_adder_range(plan));
    TRY(prepare(plan, nullptr));
    return run_grid(plan, d_vis, false, static_cast<float2 *>(d_grid), false);
}

p9idg_status p9idg_degrid_device(p9idg_plan *plan, const void *d_grid, void *d_vis) {
    if (!plan || !d_grid || !d_vis) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(prepare(plan, nullptr));
    return run_degrid(plan, static_cast<const float2 *>(d_grid), false, d_vis, false, false);
}

p9idg_status p9idg_wstack_image_device(p9idg_plan *plan, const void *d_layers, float *d_image, int32_t shift) {
    if (!plan || !d_layers || !d_image) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    TRY(ensure_device(plan));
    CK(plan->d_grid64.ensure(sizeof(float2) * nn_of(plan)));
    {
        StageScope t(plan, P9IDG_STAGE_LAYER_FFT);
        CK(launch_layer_sum(d_layers, false, plan->c.wlayer_count, static_cast<int64_t>(nn_of(plan)),
                            plan->d_grid64.as<float2>(), plan->stream));
    }
    return image_from_grid(plan, plan->d_grid64.as<float2>(), static_cast<double>(plan->c.vis_count), shift != 0,
                           d_image, nullptr);
}

p9idg_status p9idg_synchronize(p9idg_plan *plan) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    if (!plan->dev_ready) return P9IDG_OK;
    CK(cudaSetDevice(plan->device));
    return finish_call(plan);
}

// ---- timing ----

p9idg_status p9idg_plan_enable_timing(p9idg_plan *plan, int32_t on) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    plan->timing = on != 0;
    return P9IDG_OK;
}

p9idg_status p9idg_plan_stage_times(p9idg_plan *plan, double *ms, int64_t *launches) {
    if (!plan || !ms) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    if (plan->dev_ready) {
        CK(cudaSetDevice(plan->device));
        CK(cudaStreamSynchronize(plan->stream));
        collect_timing(plan);
    }
    for (int i = 0; i < P9IDG_NUM_STAGES; i++) {
        ms[i] = plan->stage_ms[i];
        if (launches) launches[i] = plan->stage_launches[i];
    }
    return P9IDG_OK;
}

p9idg_status p9idg_plan_reset_timing(p9idg_plan *plan) {
    if (!plan) return fail(P9IDG_INVALID_ARGUMENT, "null plan");
    if (plan->dev_ready) {
        CK(cudaSetDevice(plan->device));
        CK(cudaStreamSynchronize(plan->stream));
        collect_timing(plan);
    }
    for (int i = 0; i < P9IDG_NUM_STAGES; i++) {
        plan->stage_ms[i] = 0;
        plan->stage_launches[i] = 0;
    }
    return P9IDG_OK;
}

// ---- misc ----

const char *p9idg_last_error(void) { return g_last_error.c_str(); }

const char *p9idg_version(void) { return "p9idg-gb300 0.1 (sm_103a)"; }

int32_t p9idg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

p9idg_status p9idg_tc_selftest(int32_t mode, int32_t n, double *max_rel_err) {
    if (!max_rel_err || (mode != P9IDG_MODE_TC_BF16X3 && mode != P9IDG_MODE_TC_FP16X3))
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    if (p9idg_device_count() == 0) return fail(P9IDG_NO_DEVICE, "no CUDA device available");
    return tc_selftest(mode, n, max_rel_err, g_last_error);
}

p9idg_status p9idg_measure_sincos_peak(double *sincos_per_s, double *fma_per_s) {
    if (!sincos_per_s || !fma_per_s) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    if (p9idg_device_count() == 0) return fail(P9IDG_NO_DEVICE, "no CUDA device available");
    CK(measure_sincos(sincos_per_s, fma_per_s));
    return P9IDG_OK;
}

// ---- work-item sizes and batches ----

p9idg_status p9idg_plan_set_chunking(p9idg_plan *plan, int32_t gridder_max_vis, int32_t degridder_max_vis) {
    if (!plan || gridder_max_vis < 0 || degridder_max_vis < 0) return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    plan->gchunk = gridder_max_vis;
    plan->dchunk = degridder_max_vis;
    build_gridder_items(plan);
    if (plan->tc.ready) {
        if (plan->dev_ready) {
            CK(cudaSetDevice(plan->device));
            CK(cudaStreamSynchronize(plan->stream));
        }
        tc_release(plan->tc);  // rebuilt (with the new degridder items) on the next tensor-core call
    }
    return P9IDG_OK;
}

p9idg_status p9idg_batch_create(p9idg_plan *const *plans, int32_t nplans, const void *const *d_vis,
                                void *const *d_layers, const void *const *d_grids, void *const *d_vis_out,
                                p9idg_batch **out) {
    if (!out || !plans || nplans <= 0 || !d_vis || !d_layers || !d_grids || !d_vis_out)
        return fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    *out = nullptr;
    for (int i = 0; i < nplans; i++) {
        if (!plans[i] || !d_vis[i] || !d_layers[i] || !d_grids[i] || !d_vis_out[i])
            return fail(P9IDG_INVALID_ARGUMENT, "null plan or buffer");
        if (plans[i]->mode != plans[0]->mode)
            return fail(P9IDG_UNSUPPORTED, "a batch needs one precision mode");
    }
    auto *b = new (std::nothrow) p9idg_batch();
    if (!b) return fail(P9IDG_OUT_OF_MEMORY, "batch allocation");
    auto bail = [&](p9idg_status st) {
        batch_release(b);
        delete b;
        return st;
    };
    b->plans.assign(plans, plans + nplans);
    b->mode = plans[0]->mode;
    std::vector<GridderArgs> ga(nplans), da(nplans);
    std::vector<SubgridOpArgs> aa(nplans), sa(nplans);
    std::vector<TcArgs> tg(nplans), td(nplans);
    std::vector<WorkItem> gitems, ditems;
    std::vector<int2> refs;
    std::vector<int32_t> done(nplans, 0);
    // device-side completion tracking first: the argument tables point into it
    p9idg_status st;
    for (int i = 0; i < nplans; i++) {
        p9idg_plan *p = plans[i];
        if ((st = check_wstack_layers(p)) != P9IDG_OK) return bail(st);
        if ((st = prepare(p, nullptr)) != P9IDG_OK) return bail(st);
        if (i == 0) b->device = p->device;
        if (p->device != b->device) return bail(fail(P9IDG_UNSUPPORTED, "a batch runs on one device"));
    }
    {
        cudaError_t e = cudaSetDevice(b->device);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = b->d_done.ensure(sizeof(int32_t) * nplans);
        if (e == cudaSuccess) e = b->d_done_init.ensure(sizeof(int32_t) * nplans);
        if (e == cudaSuccess) e = b->d_finish.ensure(sizeof(unsigned long long) * nplans);
        if (e == cudaSuccess) e = b->d_start.ensure(sizeof(unsigned long long));
        if (e != cudaSuccess) return bail(cuda_fail(e, "batch buffers"));
    }
    for (int i = 0; i < nplans; i++) {
        p9idg_plan *p = plans[i];
        const int S = p->c.subgrid_size;
        cudaError_t e = p->d_partials.ensure(sizeof(float2) * S * S * std::max<size_t>(1, p->nslots));
        if (e == cudaSuccess) e = p->d_subgrids.ensure(sizeof(float2) * S * S * std::max<size_t>(1, p->dsub.size()));
        if (e != cudaSuccess) return bail(cuda_fail(e, "plan buffers"));
        ga[i] = gridder_args(p);
        ga[i].vis = d_vis[i];
        ga[i].vis_c128 = false;
        ga[i].partials = p->d_partials.as<float2>();
        da[i] = gridder_args(p);
        da[i].subgrids = p->d_subgrids.as<float2>();
        da[i].vis_out = d_vis_out[i];
        da[i].out_c128 = false;
        da[i].done = b->d_done.as<int32_t>() + i;
        da[i].finish_ns = b->d_finish.as<unsigned long long>() + i;
        aa[i] = subgrid_args(p);
        aa[i].partials = p->d_partials.as<float2>();
        aa[i].layers = static_cast<float2 *>(d_layers[i]);
        aa[i].out_shifted = true;
        aa[i].wstack = true;
        sa[i] = subgrid_args(p);
        sa[i].grid = static_cast<const float2 *>(d_grids[i]);
        sa[i].grid_shifted = false;
        sa[i].subgrids = p->d_subgrids.as<float2>();
        sa[i].wstack = true;
        const std::vector<WorkItem> *dsrc = &p->ditems;
        if (b->mode != P9IDG_MODE_FP32) {
            if ((st = ensure_tc(p)) != P9IDG_OK) return bail(st);
            b->tc_order = std::max(b->tc_order, p->tc.order);
            if ((st = tc_coefs(p->tc, ga[i], p->stream, g_last_error)) != P9IDG_OK) return bail(st);
            tc_fill_args(p->tc, ga[i], tg[i]);
            tc_fill_args(p->tc, da[i], td[i]);
            dsrc = &p->tc.ditems_host;
        }
        for (WorkItem w : p->gitems) {
            w.problem = i;
            gitems.push_back(w);
        }
        for (WorkItem w : *dsrc) {
            w.problem = i;
            ditems.push_back(w);
        }
        done[i] = static_cast<int32_t>(dsrc->size());
        for (size_t s = 0; s < p->dsub.size(); s++) refs.push_back(make_int2(i, static_cast<int>(s)));
        bool known = false;
        for (const auto &g : b->groups) known |= g.S == S;
        if (!known) b->groups.push_back({S, 0, 0, 0, 0, 0, 0});
        b->layers.push_back(d_layers[i]);
        b->layer_bytes.push_back(sizeof(float2) * static_cast<size_t>(p->c.wlayer_count) * nn_of(p));
        b->vis_out.push_back(d_vis_out[i]);
        b->vis_bytes.push_back(sizeof(float2) * vis_count_of(p));
        cudaError_t e2 = cudaStreamSynchronize(p->stream);
        if (e2 != cudaSuccess) return bail(cuda_fail(e2, "plan preparation"));
    }
    std::sort(b->groups.begin(), b->groups.end(),
              [](const p9idg_batch::Group &x, const p9idg_batch::Group &y) { return x.S < y.S; });
    // subgrid references grouped by size (plan order inside a group)
    std::stable_sort(refs.begin(), refs.end(), [&](const int2 &x, const int2 &y) {
        return plans[x.x]->c.subgrid_size < plans[y.x]->c.subgrid_size;
    });
    for (auto &g : b->groups) {
        g.r0 = g.rn = 0;
        bool rs = false;
        for (size_t k = 0; k < refs.size(); k++)
            if (plans[refs[k].x]->c.subgrid_size == g.S) {
                if (!rs) g.r0 = static_cast<int32_t>(k), rs = true;
                g.rn++;
            }
    }
    b->prob_vis.assign(nplans, 0);
    for (const WorkItem &w : gitems) b->prob_vis[w.problem] += static_cast<int64_t>(w.nt) * plans[w.problem]->nch;
    b->h_gitems = std::move(gitems);
    b->h_ditems = std::move(ditems);
    b->ngitems = static_cast<int32_t>(b->h_gitems.size());
    b->nditems = static_cast<int32_t>(b->h_ditems.size());
    b->nrefs = static_cast<int32_t>(refs.size());
    if ((st = upload(b->d_gargs, ga)) != P9IDG_OK || (st = upload(b->d_dargs, da)) != P9IDG_OK ||
        (st = upload(b->d_aargs, aa)) != P9IDG_OK || (st = upload(b->d_sargs, sa)) != P9IDG_OK ||
        (st = upload(b->d_tg, tg)) != P9IDG_OK || (st = upload(b->d_td, td)) != P9IDG_OK ||
        (st = upload(b->d_refs, refs)) != P9IDG_OK || (st = upload(b->d_done_init, done)) != P9IDG_OK ||
        (st = batch_order(b, P9IDG_SCHEDULE_THROUGHPUT)) != P9IDG_OK)
        return bail(st);
    *out = b;
    return P9IDG_OK;
}

p9idg_status p9idg_batch_set_schedule(p9idg_batch *b, int32_t schedule) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    if (schedule != P9IDG_SCHEDULE_THROUGHPUT && schedule != P9IDG_SCHEDULE_SMALL_FIRST)
        return fail(P9IDG_INVALID_ARGUMENT, "unknown schedule");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    if (b->exec) {  // the captured graph launches the old order's item count; capture again
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return batch_order(b, schedule);
}

p9idg_status p9idg_batch_grid_w(p9idg_batch *b) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    return batch_grid(b);
}

p9idg_status p9idg_batch_degrid_w(p9idg_batch *b) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    return batch_degrid(b);
}

p9idg_status p9idg_batch_run(p9idg_batch *b) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    if (b->exec) {
        CK(cudaGraphLaunch(b->exec, b->stream));
        return P9IDG_OK;
    }
    TRY(batch_grid(b));
    return batch_degrid(b);
}

p9idg_status p9idg_batch_capture_graph(p9idg_batch *b) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    if (b->exec) return P9IDG_OK;
    // one eager pass first: module loading and kernel attributes happen outside the capture
    TRY(batch_grid(b));
    TRY(batch_degrid(b));
    CK(cudaStreamSynchronize(b->stream));
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    p9idg_status st = batch_grid(b);
    if (st == P9IDG_OK) st = batch_degrid(b);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st != P9IDG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    b->graph = g;
    CK(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return P9IDG_OK;
}

p9idg_status p9idg_batch_synchronize(p9idg_batch *b) {
    if (!b) return fail(P9IDG_INVALID_ARGUMENT, "null batch");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    for (p9idg_plan *p : b->plans) TRY(finish_call(p));
    return P9IDG_OK;
}

p9idg_status p9idg_batch_latencies(p9idg_batch *b, double *ms) {
    if (!b || !ms) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->stream));
    const size_t n = b->plans.size();
    std::vector<unsigned long long> fin(n);
    unsigned long long start = 0;
    CK(cudaMemcpy(fin.data(), b->d_finish.p, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&start, b->d_start.p, sizeof(start), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) ms[i] = fin[i] >= start ? static_cast<double>(fin[i] - start) * 1e-6 : -1.0;
    return P9IDG_OK;
}

p9idg_status p9idg_batch_get_stream(const p9idg_batch *b, void **cuda_stream) {
    if (!b || !cuda_stream) return fail(P9IDG_INVALID_ARGUMENT, "null argument");
    *cuda_stream = b->stream;
    return P9IDG_OK;
}

void p9idg_batch_destroy(p9idg_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_release(b);
    delete b;
}

}  // extern "C"
