// Tensor-core gridder/degridder (tcgen05).  Not yet available: every call reports
// P9IDG_UNSUPPORTED and p9idg_plan_set_mode refuses the tensor-core modes.
#include "tc_gridder.cuh"

namespace p9idg {

bool tc_subgrid_size_supported(int) { return false; }

p9idg_status tc_grid(TcPlanState &, const GridderArgs &, int, cudaStream_t, std::string &err) {
    err = "tensor-core gridder not available";
    return P9IDG_UNSUPPORTED;
}

p9idg_status tc_degrid(TcPlanState &, const GridderArgs &, int, cudaStream_t, std::string &err) {
    err = "tensor-core degridder not available";
    return P9IDG_UNSUPPORTED;
}

void tc_release(TcPlanState &st) {
    if (st.scratch) cudaFree(st.scratch);
    st.scratch = nullptr;
    st.scratch_bytes = 0;
}

}  // namespace p9idg
