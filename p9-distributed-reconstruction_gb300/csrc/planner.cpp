// Host subgrid planner: Partitioner.CreatePartition of the reference
// (Distributed-Reconstruction/Core/ImageDomainGridder/Partitioner.cs:20-255).
//
// The subgrid list must be bit-identical to the reference's, because it decides
// which visibilities are gridded at all.  The arithmetic therefore follows the C#
// expression by expression in the same types (the ImageSize product is float,
// pixel coordinates double), with .NET Core 3.0 semantics for Math.Round (ties to
// even), Math.Min/Max (NaN-propagating) and the double->int conversion (0x80000000
// for NaN and out-of-range values).  Compile without FMA contraction.
//
// Baselines are independent, so they are partitioned on all host threads; the
// result is concatenated in baseline order and, on failure, the error of the
// lowest failing baseline is returned -- what the sequential reference throws.

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <thread>

#include "p9idg_internal.h"

namespace p9idg {

namespace {

int32_t dotnet_to_int(double x) {
    if (std::isnan(x) || x >= 2147483648.0 || x <= -2147483649.0) return INT32_MIN;
    return static_cast<int32_t>(x);
}

double dotnet_min(double a, double b) {
    if (a < b || std::isnan(a)) return a;
    if (a == b) return std::signbit(a) ? a : b;
    return b;
}

double dotnet_max(double a, double b) {
    if (a > b || std::isnan(a)) return a;
    if (a == b) return std::signbit(a) ? b : a;
    return b;
}

int32_t add_wrap(int32_t a, int32_t b) { return static_cast<int32_t>(static_cast<uint32_t>(a) + static_cast<uint32_t>(b)); }

struct UvPoint {
    double u, v, w;  // pixels, pixels, wavelengths
};

// The private Subgrid class of Partitioner.cs:154-254: a growing uv box.
class UvBox {
   public:
    explicit UvBox(const p9idg_params &c) : c_(c) { reset(); }

    void reset() {
        umin_ = INFINITY;
        umax_ = -INFINITY;
        vmin_ = INFINITY;
        vmax_ = -INFINITY;
        windex_ = 0;
        upix_ = vpix_ = 0;
    }

    // AddVisibility (Partitioner.cs:186-221)
    bool add(const UvPoint &p) {
        if (std::isinf(p.u) || std::isinf(p.v)) return false;
        int32_t widx = 0;
        if (c_.wstep != 0.0) widx = dotnet_to_int(std::floor(p.w / c_.wstep));
        if (!std::isinf(umin_) && windex_ != widx) return false;
        const double umin = dotnet_min(umin_, p.u), umax = dotnet_max(umax_, p.u);
        const double vmin = dotnet_min(vmin_, p.v), vmax = dotnet_max(vmax_, p.v);
        const double width = dotnet_max(umax - umin, vmax - vmin);
        if ((width + static_cast<double>(c_.kernel_size)) >= static_cast<double>(c_.subgrid_size)) return false;
        umin_ = umin;
        umax_ = umax;
        vmin_ = vmin;
        vmax_ = vmax;
        windex_ = widx;
        return true;
    }

    // Finish / ComputeCoordinates (Partitioner.cs:236-253)
    void finish() {
        upix_ = dotnet_to_int(std::nearbyint((umax_ + umin_) / 2));
        vpix_ = dotnet_to_int(std::nearbyint((vmax_ + vmin_) / 2));
        upix_ = add_wrap(add_wrap(upix_, c_.grid_size / 2), -(c_.subgrid_size / 2));
        vpix_ = add_wrap(add_wrap(vpix_, c_.grid_size / 2), -(c_.subgrid_size / 2));
    }

    // InRange (Partitioner.cs:223-234)
    bool in_range() const {
        const int32_t hi = std::max(upix_, vpix_), lo = std::min(upix_, vpix_);
        return lo >= 1 && hi <= (c_.grid_size - c_.subgrid_size) && windex_ >= -c_.wlayer_count &&
               windex_ < c_.wlayer_count;
    }

    int32_t upix() const { return upix_; }
    int32_t vpix() const { return vpix_; }
    int32_t windex() const { return windex_; }

   private:
    const p9idg_params &c_;
    double umin_, umax_, vmin_, vmax_;
    int32_t windex_, upix_, vpix_;
};

struct BaselineResult {
    std::vector<p9idg_subgrid> subs;
    p9idg_status status = P9IDG_OK;
};

void partition_baseline(const p9idg_params &c, const double *uvw, int32_t bl, int32_t nt, const double *freq,
                        int32_t nch, std::vector<UvPoint> &p0, std::vector<UvPoint> &pm, BaselineResult &res) {
    // MetersToPixels / MetersToLambda (Partitioner.cs:127-129) for channel 0 and the last
    // channel; the last channel carries channel 0's w (the "hack", Partitioner.cs:61-62).
    const double imgsize = static_cast<double>(image_size(c));
    const double f0 = freq[0] / kSpeedOfLight, fm = freq[nch - 1] / kSpeedOfLight;
    for (int32_t t = 0; t < nt; t++) {
        const double *q = uvw + (static_cast<int64_t>(bl) * nt + t) * 3;
        p0[t] = {q[0] * imgsize * f0, q[1] * imgsize * f0, q[2] * f0};
        pm[t] = {q[0] * imgsize * fm, q[1] * imgsize * fm, p0[t].w};
    }
    UvBox box(c);
    int32_t time = 0;
    while (time < nt) {  // Partitioner.cs:51-121
        box.reset();
        int32_t count = 0;
        for (; time < nt; time++) {
            if (box.add(p0[time]) && box.add(pm[time])) {
                count++;
                if (count == c.max_timesteps) {
                    time++;
                    break;
                }
            } else {
                break;
            }
        }
        if (count == 0) {  // nothing fits: skip the sample, or fail on infinite coordinates
            if (std::isinf(p0[time].u) || std::isinf(p0[time].v)) {
                res.status = P9IDG_CANNOT_PLACE;
                return;
            }
            time++;
            continue;
        }
        box.finish();
        if (!box.in_range()) {
            res.status = P9IDG_SUBGRID_OUT_OF_GRID;
            return;
        }
        res.subs.push_back({bl, time - count, count, box.upix(), box.vpix(), box.windex()});
    }
}

}  // namespace

float image_size(const p9idg_params &c) { return c.scale_arcsec * static_cast<float>(c.grid_size); }

float compute_l(int x, int s, float imagesize) {  // Gridder.cs:163-166
    const float a = static_cast<float>(x - (s / 2)) + 0.5f;
    const float b = a * imagesize;
    return b / static_cast<float>(s);
}

float compute_n(float l, float m) {  // Gridder.cs:168-174
    const float tmp = (l * l) + (m * m);
    const double d = static_cast<double>(tmp / 1.0f) + std::sqrt(1.0 - static_cast<double>(tmp));
    return tmp / static_cast<float>(d);
}

double wavenumber(double f) { return 2.0 * kPi * f / kSpeedOfLight; }  // MathFunctions.cs:107-113

p9idg_status partition(const p9idg_params &c, const double *uvw, int32_t nbl, int32_t nt, const double *freq,
                       int32_t nch, std::vector<p9idg_subgrid> &out, std::string &err) {
    out.clear();
    if (nbl < 0 || nt < 0 || nch < 0) {
        err = "negative dimension";
        return P9IDG_INVALID_ARGUMENT;
    }
    if (nbl == 0 || nt == 0) return P9IDG_OK;
    if (nch == 0) {
        err = "no channels (the reference indexes datapoints[time, -1])";
        return P9IDG_INVALID_ARGUMENT;
    }
    if (!uvw || !freq) {
        err = "null uvw or frequencies";
        return P9IDG_INVALID_ARGUMENT;
    }
    std::vector<BaselineResult> results(nbl);
    unsigned nthreads = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64u));
    nthreads = std::min<unsigned>(nthreads, static_cast<unsigned>(nbl));
    auto worker = [&](unsigned tid) {
        std::vector<UvPoint> p0(nt), pm(nt);
        for (int32_t bl = static_cast<int32_t>(tid); bl < nbl; bl += static_cast<int32_t>(nthreads))
            partition_baseline(c, uvw, bl, nt, freq, nch, p0, pm, results[bl]);
    };
    if (nthreads == 1) {
        worker(0);
    } else {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nthreads; t++) pool.emplace_back(worker, t);
        for (auto &th : pool) th.join();
    }
    size_t total = 0;
    for (int32_t bl = 0; bl < nbl; bl++) {
        if (results[bl].status != P9IDG_OK) {
            err = results[bl].status == P9IDG_CANNOT_PLACE
                      ? "could not place (all) visibilities on subgrid (too many channnels, kernel size too large)"
                      : "subgrid falls not within grid";
            err += " (baseline " + std::to_string(bl) + ")";
            return results[bl].status;
        }
        total += results[bl].subs.size();
    }
    out.reserve(total);
    for (auto &r : results) out.insert(out.end(), r.subs.begin(), r.subs.end());
    return P9IDG_OK;
}

p9idg_status validate_subgrids(const p9idg_params &c, const p9idg_subgrid *subs, int64_t n, int32_t nbl, int32_t nt,
                               std::string &err) {
    for (int64_t i = 0; i < n; i++) {
        const p9idg_subgrid &s = subs[i];
        if (s.baseline_idx < 0 || s.baseline_idx >= nbl || s.time_sample_start < 0 || s.time_sample_count < 0 ||
            static_cast<int64_t>(s.time_sample_start) + s.time_sample_count > nt) {
            err = "subgrid " + std::to_string(i) + " indexes samples outside uvw/vis";
            return P9IDG_INVALID_ARGUMENT;
        }
    }
    (void)c;
    return P9IDG_OK;
}

void build_work_items(const std::vector<p9idg_subgrid> &subs, int32_t nch, int64_t max_vis,
                      std::vector<DevSubgrid> &dsub, std::vector<WorkItem> &items) {
    dsub.resize(subs.size());
    items.clear();
    const int32_t chunk = static_cast<int32_t>(std::max<int64_t>(1, max_vis / std::max<int32_t>(1, nch)));
    int32_t slot = 0;
    for (size_t i = 0; i < subs.size(); i++) {
        const p9idg_subgrid &s = subs[i];
        DevSubgrid &d = dsub[i];
        d = {s.baseline_idx, s.time_sample_start, s.time_sample_count, s.u_pixel, s.v_pixel, s.w_lambda, slot, 0};
        for (int32_t t = 0; t < s.time_sample_count; t += chunk) {
            const int32_t len = std::min(chunk, s.time_sample_count - t);
            items.push_back({static_cast<int32_t>(i), s.time_sample_start + t, len, slot++, 0, 0});
            d.item_count++;
        }
    }
    // Largest first: blocks are scheduled roughly in launch order, so this is an LPT schedule.
    std::stable_sort(items.begin(), items.end(), [](const WorkItem &a, const WorkItem &b) { return a.nt > b.nt; });
}

void fft_shift_host(void *a, int32_t n, int32_t esz) {  // FFT.Shift (FFT.cs:221-264)
    char *p = static_cast<char *>(a);
    const int32_t n2 = n / 2;
    char tmp[16];
    for (int32_t i = 0; i < n2; i++)
        for (int32_t j = 0; j < n2; j++) {
            char *a13 = p + (static_cast<size_t>(i) * n + j) * esz;
            char *b13 = p + (static_cast<size_t>(i + n2) * n + j + n2) * esz;
            std::memcpy(tmp, a13, esz);
            std::memcpy(a13, b13, esz);
            std::memcpy(b13, tmp, esz);
            char *a24 = p + (static_cast<size_t>(i + n2) * n + j) * esz;
            char *b24 = p + (static_cast<size_t>(i) * n + j + n2) * esz;
            std::memcpy(tmp, a24, esz);
            std::memcpy(a24, b24, esz);
            std::memcpy(b24, tmp, esz);
        }
}

}  // namespace p9idg
