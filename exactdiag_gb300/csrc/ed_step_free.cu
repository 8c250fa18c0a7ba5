// ed_step_free.cu -- fused step kernel for rows of blocks with a trivial stabiliser (the bulk of
// every doped sector), in two register budgets: 3 or 4 resident CTAs per SM.
#include "ed_step.cuh"

namespace ed {

int step_hv_free(int dtype, int minb, const StepArgs& a, cudaStream_t st) {
    return minb == 4 ? step_kind_dtype<4, kRowsFree>(dtype, a, st) : step_kind_dtype<3, kRowsFree>(dtype, a, st);
}

int step_free_occupancy(int minb, size_t smem) {
    return minb == 4 ? step_kind_occupancy<4, kRowsFree>(smem) : step_kind_occupancy<3, kRowsFree>(smem);
}

}  // namespace ed
