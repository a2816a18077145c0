// Tensor-core path of the split-precision executors (see tc_gemm.h).
#include "tc_gemm.h"

namespace qxg {

bool tc_plan_step(const StepArgs&, size_t, size_t, size_t, bool, TcStep*) { return false; }

cudaError_t tc_run_step(const TcStep&, const StepArgs&, int*, void*, cudaStream_t, int) {
    return cudaErrorNotSupported;
}

}  // namespace qxg
