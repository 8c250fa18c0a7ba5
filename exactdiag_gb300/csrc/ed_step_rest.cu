// ed_step_rest.cu -- fused step kernels for rows of blocks with a non-trivial stabiliser
// (coset candidates + bitmap lookups) and for rows that take the orbit walk.
#include "ed_step.cuh"

namespace ed {

// Real FP32 rows fit a 4-CTA register budget without spilling; the wider types keep 3.
int step_hv_cand(int dtype, const StepArgs& a, cudaStream_t st) {
    return dtype == ED_F32 ? launch_step_kind<float, false, 4, kRowsCand>(a, st) : step_kind_dtype<3, kRowsCand>(dtype, a, st);
}

int step_hv_generic(int dtype, const StepArgs& a, cudaStream_t st) {
    return step_kind_dtype<3, kRowsGeneric>(dtype, a, st);
}

int step_expand(int dtype, const StepArgs& a, cudaStream_t st) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    switch (dtype) {
    case ED_F64: return launch_expand<double, false>(a, st, sms);
    case ED_C128: return launch_expand<double, true>(a, st, sms);
    case ED_F32: return launch_expand<float, false>(a, st, sms);
    default: return launch_expand<float, true>(a, st, sms);
    }
}

int step_rest_occupancy(size_t smem, bool f32) {
    return f32 ? step_kind_occupancy<4, kRowsCand>(smem) : step_kind_occupancy<3, kRowsCand>(smem);
}

}  // namespace ed
