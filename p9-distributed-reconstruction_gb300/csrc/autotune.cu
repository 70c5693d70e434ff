// Autotuner: chooses the subgrid size and the work-item sizes (the time-chunk length of a
// gridder / degridder work item) by timing grid + degrid on a sample of the observation.
//
// The sample is every k-th baseline (up to 256 of them), with all their time samples and
// channels, and pseudo-random visibilities and model grid.  Each candidate subgrid size
// gets its own plan (its own partition); for each work-item size pair the plan runs one
// warm-up and three timed grid + degrid passes through the device entry points, timed with
// CUDA events on the plan's stream.  The subgrid size changes which visibilities the
// partitioner keeps (a channel span must fit in S - KernelSize pixels), so only
// candidates that keep at least 99.9 % of the best candidate's gridded visibilities compete;
// among those the fastest per gridded visibility wins.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "p9idg_internal.h"

using namespace p9idg;

namespace {

struct Candidate {
    int S;
    int gchunk, dchunk;
    double sec_per_vis;
    int64_t gridded, input;
};

p9idg_status tune_fail(p9idg_status st, const std::string &msg) {
    record_last_error(msg);
    return st;
}

uint32_t lcg(uint32_t &s) {
    s = s * 1664525u + 1013904223u;
    return s;
}

}  // namespace

extern "C" p9idg_status p9idg_autotune(const p9idg_params *c, const double *uvw, int32_t nbl, int32_t nt,
                                       const double *frequencies, int32_t nch, int32_t mode,
                                       const int32_t *subgrid_sizes, int32_t nsizes, p9idg_tuning *out) {
    if (!c || !uvw || !frequencies || !out || nbl <= 0 || nt <= 0 || nch <= 0 || nsizes < 0)
        return tune_fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    if (p9idg_device_count() == 0) return tune_fail(P9IDG_NO_DEVICE, "no CUDA device available");
    std::vector<int> sizes;
    if (subgrid_sizes && nsizes > 0)
        sizes.assign(subgrid_sizes, subgrid_sizes + nsizes);
    else
        sizes = {24, 32, 48};
    // sample: every k-th baseline, up to 256 baselines
    const int stride = std::max(1, nbl / 256);
    std::vector<double> su;
    int nbs = 0;
    for (int b = 0; b < nbl; b += stride, nbs++)
        su.insert(su.end(), uvw + static_cast<size_t>(b) * nt * 3, uvw + static_cast<size_t>(b + 1) * nt * 3);
    const size_t nvis = static_cast<size_t>(nbs) * nt * nch;
    const size_t nn = static_cast<size_t>(c->grid_size) * c->grid_size;
    std::vector<float> hv(2 * nvis), hg(2 * nn);
    uint32_t seed = 7;
    for (auto &v : hv) v = static_cast<float>(lcg(seed) >> 8) / 16777216.0f - 0.5f;
    for (auto &v : hg) v = static_cast<float>(lcg(seed) >> 8) / 16777216.0f - 0.5f;
    void *d_vis = nullptr, *d_out = nullptr, *d_grid = nullptr, *d_layers = nullptr;
    cudaError_t e = cudaMalloc(&d_vis, sizeof(float) * 2 * std::max<size_t>(1, nvis));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(float) * 2 * std::max<size_t>(1, nvis));
    if (e == cudaSuccess) e = cudaMalloc(&d_grid, sizeof(float) * 2 * nn);
    if (e == cudaSuccess) e = cudaMalloc(&d_layers, sizeof(float) * 2 * nn * std::max(1, c->wlayer_count));
    if (e == cudaSuccess) e = cudaMemcpy(d_vis, hv.data(), sizeof(float) * hv.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_grid, hg.data(), sizeof(float) * hg.size(), cudaMemcpyHostToDevice);
    auto cleanup = [&]() {
        cudaFree(d_vis);
        cudaFree(d_out);
        cudaFree(d_grid);
        cudaFree(d_layers);
    };
    if (e != cudaSuccess) {
        cleanup();
        return tune_fail(e == cudaErrorMemoryAllocation ? P9IDG_OUT_OF_MEMORY : P9IDG_CUDA_ERROR,
                         std::string("autotune buffers: ") + cudaGetErrorString(e));
    }
    const bool fp32 = mode == P9IDG_MODE_FP32;
    const std::vector<int> gchunks = fp32 ? std::vector<int>{512, 1024, 2048} : std::vector<int>{2048, 4096, 8192};
    const std::vector<int> dchunks = fp32 ? std::vector<int>{256, 512, 1024} : std::vector<int>{8192, 16384, 32768};
    std::vector<Candidate> results;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int S : sizes) {
        if (S <= c->kernel_size + 1 || S > c->grid_size) continue;
        p9idg_params p = *c;
        p.subgrid_size = S;
        p9idg_plan *plan = nullptr;
        if (p9idg_plan_create(&p, su.data(), nbs, nt, frequencies, nch, &plan) != P9IDG_OK) continue;
        if (p9idg_plan_set_mode(plan, mode) != P9IDG_OK) {
            p9idg_plan_destroy(plan);
            continue;
        }
        p9idg_plan_info info{};
        p9idg_plan_get_info(plan, &info);
        if (info.mode != mode) {  // a tensor-core mode this sample's w term rules out
            p9idg_plan_destroy(plan);
            continue;
        }
        void *stream = nullptr;
        for (int gc : gchunks)
            for (int dc : dchunks) {
                if (p9idg_plan_set_chunking(plan, gc, dc) != P9IDG_OK) continue;
                if (p9idg_grid_w_device(plan, d_vis, d_layers) != P9IDG_OK ||
                    p9idg_degrid_w_device(plan, d_grid, d_out) != P9IDG_OK || p9idg_synchronize(plan) != P9IDG_OK)
                    continue;
                p9idg_plan_get_stream(plan, &stream);
                cudaStream_t st = static_cast<cudaStream_t>(stream);
                cudaEventRecord(e0, st);
                bool ok = true;
                for (int r = 0; r < 3 && ok; r++)
                    ok = p9idg_grid_w_device(plan, d_vis, d_layers) == P9IDG_OK &&
                         p9idg_degrid_w_device(plan, d_grid, d_out) == P9IDG_OK;
                cudaEventRecord(e1, st);
                if (!ok || p9idg_synchronize(plan) != P9IDG_OK) continue;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double per = info.gridded_visibilities > 0
                                       ? ms * 1e-3 / 3.0 / static_cast<double>(info.gridded_visibilities)
                                       : 1e30;
                results.push_back({S, gc, dc, per, info.gridded_visibilities, info.input_visibilities});
            }
        p9idg_plan_destroy(plan);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cleanup();
    if (results.empty()) return tune_fail(P9IDG_UNSUPPORTED, "no candidate configuration could run");
    int64_t best_gridded = 0;
    for (const auto &r : results) best_gridded = std::max(best_gridded, r.gridded);
    const Candidate *best = nullptr;
    for (const auto &r : results)
        if (static_cast<double>(r.gridded) >= 0.999 * static_cast<double>(best_gridded) &&
            (!best || r.sec_per_vis < best->sec_per_vis))
            best = &r;
    out->subgrid_size = best->S;
    out->kernel_size = c->kernel_size;
    out->gridder_max_vis = best->gchunk;
    out->degridder_max_vis = best->dchunk;
    out->seconds_per_gridded_vis = best->sec_per_vis;
    out->gridded_fraction = best->input > 0 ? static_cast<double>(best->gridded) / best->input : 0.0;
    return P9IDG_OK;
}
