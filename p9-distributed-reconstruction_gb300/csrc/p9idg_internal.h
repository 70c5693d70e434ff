// Internal declarations shared by the host runtime (api.cu, planner.cpp) and the kernels.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/p9idg.h"

namespace p9idg {

constexpr double kPi = 3.14159265358979323846;
constexpr double kSpeedOfLight = 299792458.0;  // Core/ImageDomainGridder/MathFunctions.cs:11

// One subgrid as the kernels see it (32 bytes).
struct DevSubgrid {
    int32_t bl, t0, nt;      // baseline list index, first time sample, time samples
    int32_t u, v, w;         // UPixel, VPixel, WLambda (w layer index)
    int32_t item_begin;      // first gridder work item (slot) of this subgrid
    int32_t item_count;      // number of gridder work items
};

// A (subgrid, time chunk) unit of gridder or degridder work (24 bytes).
struct WorkItem {
    int32_t subgrid;
    int32_t t0;      // first time sample of the chunk
    int32_t nt;      // time samples in the chunk
    int32_t slot;    // gridder: index of this item's partial subgrid buffer
    int32_t problem; // batched launches: index of the imaging problem (plan) it belongs to
    int32_t pad;
};

// Scalars every kernel needs.
struct Geometry {
    int32_t N, S, W, nch, nt_all, nbl;
    double uv_scale;     // 2*pi / ImageSize (radians per pixel offset per unit l)
    float wstep_lambda;  // GriddingConstants.WStepLambda (never assigned: 0)
    float inv_s2;        // 1.0f / (S*S), Gridder.cs:151
};

// ---- planner (planner.cpp; host only, no CUDA) ----
float image_size(const p9idg_params &c);
float compute_l(int x, int s, float imagesize);
float compute_n(float l, float m);
double wavenumber(double f);
p9idg_status partition(const p9idg_params &c, const double *uvw, int32_t nbl, int32_t nt, const double *freq,
                       int32_t nch, std::vector<p9idg_subgrid> &out, std::string &err);
p9idg_status validate_subgrids(const p9idg_params &c, const p9idg_subgrid *subs, int64_t n, int32_t nbl, int32_t nt,
                               std::string &err);
// Splits subgrids into work items of at most max_vis visibilities (whole time samples, at
// least one), numbering slots per subgrid, and orders the launch list by descending size.
void build_work_items(const std::vector<p9idg_subgrid> &subs, int32_t nch, int64_t max_vis,
                      std::vector<DevSubgrid> &dsub, std::vector<WorkItem> &items);
void fft_shift_host(void *a, int32_t n, int32_t elem_bytes);

// Sets the thread-local message p9idg_last_error() returns (api.cu).
void record_last_error(const std::string &msg);

}  // namespace p9idg
