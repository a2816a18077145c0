// Tensor-core (tcgen05) path of the split-precision executors: a contraction step whose
// summed and free extents are large enough is run as a complex GEMM on 3xBF16 or 3xTF32
// operand splits with FP32 accumulation in tensor memory.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

#include "qxgpu_internal.h"

namespace qxg {

struct TcStep {
    int64_t M = 0, N = 0, K = 0, batch = 0;   // GEMM extents of the step
    size_t scratch_bytes = 0;                 // split operands staged in device scratch
    bool tf32 = false;
};

// Decide whether a step goes to the tensor cores; fills `tc` when it does.
bool tc_plan_step(const StepArgs& s, size_t a_bits, size_t b_bits, size_t c_bits, bool tf32, TcStep* tc);

// Run a planned tensor-core step (scratch: at least tc.scratch_bytes of device memory).
cudaError_t tc_run_step(const TcStep& tc, const StepArgs& s, int* exps, void* scratch, cudaStream_t st,
                        int sm_count);

}  // namespace qxg
