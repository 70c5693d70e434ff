// Tensor-core (tcgen05) gridder and degridder: split-precision complex GEMM form.
#pragma once

#include <string>
#include <vector>

#include "kernels.cuh"

namespace p9idg {

// Per-plan state of the tensor-core kernels (device buffers and host-built tables).
struct TcPlanState {
    bool ready = false;
    bool coef_valid = false;      // coefficients match the uvw now on the device
    // Set when a new uvw upload was compared on the device with the one the coefficients were
    // computed from: the coefficient kernel then recomputes only if this int32 flag is nonzero.
    const int32_t *coef_recompute_flag = nullptr;
    int S = 0;
    int64_t ncoef = 0;
    void *coef = nullptr;         // float4 {du, dv, dw, 0} per gridded visibility, subgrid order
    void *coef_off = nullptr;     // int64 per subgrid: first coefficient of the subgrid
    void *tables = nullptr;       // float: g[32] (separable part of n), r[32][32] (remainder), l[32],
                                  // zero past the plan's S
    void *ditems = nullptr;       // degridder work items (<= degrid_chunk visibilities)
    int32_t nditems = 0;
    std::vector<WorkItem> ditems_host;  // the same list on the host (batches merge them)
    int64_t degrid_chunk = 16384;       // visibilities per degridder work item (set before tc_prepare)
    double max_w_r = 0;           // max |dw| * max |r|: bound on the phase the form expands
    double r_max = 0;             // max |r| of the centred remainder table
    int want_order = 0;           // 0: the lowest order whose bound holds; 2: always the second-order form
    int order = 1;                // the form the kernels run: 1 (first order) or 2 (second order)
    double dw_limit = 0;          // limit of the form / max |r|: the largest |dw| a visibility may have
    float dw_scale = 1.f;         // FP16 mode: power of two with max |dw| * dw_scale < 1
    float r_scale = 1.f;          // FP16 mode: power of two with max |r| * r_scale < 1
    float m_tab[32] = {}, g_tab[32] = {};  // m_y and g_y (the same values serve l_x and f_x)
};

// Arguments of one problem for the tensor-core kernels.
struct TcArgs {
    Geometry g;
    const WorkItem *items;
    const DevSubgrid *subs;
    const int64_t *coef_off;
    const float4 *coef;
    const void *vis;
    const float *lmn;   // l[S], n[S*S]
    const float *tabs;  // f[S], r[S*S]
    const float *taper;
    float2 *partials;
    const float2 *subgrids;
    void *vis_out;
    int32_t *status;
    float dw_scale;  // FP16 operands: power of two bringing max |dw| below 1 (1 for BF16)
    float r_scale;   // FP16 operands: power of two bringing max |r| below 1 (1 for BF16)
    // m_y and g_y by value: a single-plan launch reads them from the parameter bank, where the
    // degridder's unrolled per-row loop uses them as instruction operands
    float m_tab[32], g_tab[32];
    int32_t *done;   // batched launches: completion count / time (see GridderArgs)
    unsigned long long *finish_ns;
    uint64_t wait_ns;          // limit of every pipeline wait before the kernel gives up (2 s)
    int32_t debug_skip_stage;  // fault injection: the loader never delivers this stage (-1: off)
};

bool tc_subgrid_size_supported(int S);
// Fault injection for the bounded-wait path (p9idg_debug_tc_wait): later launches use this wait
// limit and have their loader skip input stage `skip_stage` of every work item (-1: off).
void tc_debug_set(uint64_t wait_ns, int32_t skip_stage);
// max |dw| * max |r| over the gridded samples of a plan: the largest phase dw * r(x, y) the
// tensor-core form expands to first order (|dw| <= max |k| * max |w|, as WStepLambda is 0).
// Host only; compared with P9IDG_TC_MAX_W_TERM before a plan selects a tensor-core mode.
double tc_w_term(const std::vector<p9idg_subgrid> &subs, const std::vector<float> &lmn, int S,
                 const std::vector<double> &wn, const double *uvw_host, int nt_all);
// Per-problem arguments of a prepared plan (host side; device pointers inside).
void tc_fill_args(const TcPlanState &st, const GridderArgs &a, TcArgs &t);
// Coefficients for the plan's current uvw (no-op when still valid).
p9idg_status tc_coefs(TcPlanState &st, const GridderArgs &a, cudaStream_t stream, std::string &err);
// One launch over the work items of many problems; `probs` is a device array of TcArgs
// indexed by WorkItem::problem.
// order: 2 when any problem of the batch needs the second-order form (it serves first-order
// problems as well, a little more accurately).
p9idg_status tc_grid_batch(const TcArgs *probs, const WorkItem *items, int32_t nitems, int mode, int order,
                           cudaStream_t stream, std::string &err);
p9idg_status tc_degrid_batch(const TcArgs *probs, const WorkItem *items, int32_t nitems, int mode, int order,
                             cudaStream_t stream, std::string &err);
// The form (1 or 2) a plan with this w term runs for a requested order (0 = automatic), or 0 when
// neither bound holds (the plan then keeps the FP32 kernels).
int tc_order_for(double w_term, int want_order);
// Re-selects the form of a prepared state after p9idg_plan_set_tc_order (no device work).
void tc_set_order(TcPlanState &st, int want_order);
// Builds the tables and uploads them (once per plan).
p9idg_status tc_prepare(TcPlanState &st, const std::vector<p9idg_subgrid> &subs, const std::vector<float> &lmn,
                        int S, int nch, const std::vector<double> &wn, const double *uvw_host, int nt_all,
                        cudaStream_t stream, std::string &err);
p9idg_status tc_grid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err);
p9idg_status tc_degrid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err);
void tc_release(TcPlanState &st);
// Known GEMM C[128][n] = A[128][64] B[n][64]^T through the tcgen05 operand layout and
// descriptors; reports the largest error relative to max |C|.
p9idg_status tc_selftest(int mode, int n, double *max_rel_err, std::string &err);

}  // namespace p9idg
