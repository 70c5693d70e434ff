// Tensor-core (tcgen05) gridder and degridder: split-precision complex GEMM form.
#pragma once

#include <string>

#include "kernels.cuh"

namespace p9idg {

// Device buffers owned by a plan for the tensor-core kernels.
struct TcPlanState {
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
};

bool tc_subgrid_size_supported(int S);
p9idg_status tc_grid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err);
p9idg_status tc_degrid(TcPlanState &st, const GridderArgs &a, int mode, cudaStream_t stream, std::string &err);
void tc_release(TcPlanState &st);

}  // namespace p9idg
